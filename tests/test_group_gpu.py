"""Grouped launch (hb_group_*): several engines' sweeps with different models, node counts, delays,
sweep values and step counts in one launch of the streamed-history work-queue kernel, replayed from a
CUDA graph.
Each member's results must equal the oracle's run of that member alone (same tolerances as the
other parity tests), on the first and on a repeated execution."""
import numpy as np
import pytest

from hyburn_gb300 import BatchHybridEngine, GroupedSweep, SweepParam
from hyburn_gb300._abi import HB_RUN_STREAM_NPT, HB_SEM_BOLD_PER_POINT, HB_SEM_DELAY_RING
from hyburn_gb300.config import MonitorConfig, Unsupported
from oracle.hb_oracle import OracleEngine

from cases import noise_for, single_model
from test_parity_gpu import BOLD_ATOL, close

pytestmark = pytest.mark.gpu


def _check(members, sem, results):
    for (cfg, n_pts, param, vals, n_steps, noise), r in zip(members, results):
        o = OracleEngine.from_config(cfg, n_pts, semantics=sem).run_sweep(param, vals, n_steps, noise=noise)
        close(r.final_states[0], o.final_states[0], what=f"final ({cfg.network.subnetworks[0].nnodes} nodes)")
        close(r.tavg[0], o.tavg[0], what=f"tavg ({cfg.network.subnetworks[0].nnodes} nodes)")
        if o.bold is not None:
            for m in range(len(o.bold)):
                close(r.bold[m], o.bold[m], atol=BOLD_ATOL, what="bold")


@pytest.mark.parametrize("sem,run_flags", [(HB_SEM_DELAY_RING, 0), (HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT, 0),
                                           (HB_SEM_DELAY_RING, HB_RUN_STREAM_NPT(4))])
def test_group_uneven_sizes_steps_and_bold(sem, run_flags):
    """run_flags HB_RUN_STREAM_NPT(4): the 768-thread form, four nodes per consumer thread."""
    mons = [MonitorConfig("Bold", tr=0.004, bold_period=10)]
    spec = [(20, 3, 260, "rk4"), (45, 2, 180, "rk4"), (70, 4, 330, "heun"), (33, 1, 90, "rk4")]
    members, cfgs = [], []
    for i, (n, pts, steps, integ) in enumerate(spec):
        cfg = single_model("MontbrioPazoRoxin", n, integ, "Linear", (0.3,), weights="csr", delays="per_edge_long",
                           monitors=mons, dt=0.05, seed=i)
        vals = np.linspace(-1.0, 0.5, pts).astype(np.float32).tolist()
        members.append((cfg, pts, SweepParam(0, 4), vals, steps, None))
    engines = [BatchHybridEngine.from_config(c, p, semantics=sem) for c, p, *_ in members]
    g = GroupedSweep([(e, m[2], m[3], m[4], m[5]) for e, m in zip(engines, members)], run_flags=run_flags)
    for _ in range(2):
        g.execute()
        _check(members, sem, g.results())
        assert g.last_kernel_time() > 0
    g.close()


def test_group_stochastic_members():
    members = []
    for i, (n, steps) in enumerate([(24, 200), (40, 120)]):
        cfg = single_model("Generic2dOscillator", n, "heun_stochastic", "Linear", (0.2,), weights="csr",
                           delays="per_edge_long", nsig=1e-3, seed=i)
        members.append((cfg, 3, SweepParam(-1, 0), [0.0, 0.1, 0.2], steps, noise_for(cfg, steps, 3, False, 5 + i)))
    engines = [BatchHybridEngine.from_config(c, p, semantics=HB_SEM_DELAY_RING) for c, p, *_ in members]
    g = GroupedSweep([(e, m[2], m[3], m[4], m[5]) for e, m in zip(engines, members)])
    g.execute()
    _check(members, HB_SEM_DELAY_RING, g.results())


@pytest.mark.parametrize("npt", [0, 4])
def test_group_mixed_models_one_launch(npt):
    """Generic2dOscillator, MontbrioPazoRoxin, JansenRit and Kuramoto (the [sin, cos] coupling form)
    networks with different sizes, step counts, integrators and parameter tables in one launch of the
    work-queue kernel; each member equals the oracle's run of it alone, on two executions."""
    sem = HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT
    mons = [MonitorConfig("Bold", tr=0.004, bold_period=10)]
    members = []
    g2 = single_model("Generic2dOscillator", 30, "heun_stochastic", "Linear", (0.2,), weights="csr", delays="per_edge_long",
                      nsig=1e-3, seed=1, monitors=mons)
    members.append((g2, 3, SweepParam(-1, 0), [0.0, 0.1, 0.2], 240, noise_for(g2, 240, 3, False, 7)))
    mpr = single_model("MontbrioPazoRoxin", 52, "rk4", "Linear", (0.3,), weights="csr", delays="per_edge_long", dt=0.05,
                       seed=2, monitors=mons)
    p = np.asarray(mpr.network.subnetworks[0].params, np.float32)
    rows = np.tile(p, (2, 52, 1))
    rows[1, :, 2] = -4.0
    mpr.network.subnetworks[0].node_params = rows
    members.append((mpr, 2, SweepParam(-1, 0), [0.2, 0.6], 300, None))
    jr = single_model("JansenRit", 24, "heun", "Sigmoidal", (0.0, 0.1, 0.0, 1.0, 0.05), weights="csr",
                      delays="per_edge_long", seed=3)
    members.append((jr, 2, SweepParam(-1, 3), [0.5, 1.5], 160, None))
    ku = single_model("Kuramoto", 40, "heun", "Kuramoto", (1.5,), weights="csr", delays="per_edge_long", seed=4)
    ku.network.subnetworks[0].node_params = np.random.default_rng(4).standard_normal((40, 1)).astype(np.float32)
    members.append((ku, 3, SweepParam(-1, 0), [0.5, 1.0, 2.0], 200, None))
    engines = [BatchHybridEngine.from_config(c, n, semantics=sem) for c, n, *_ in members]
    g = GroupedSweep([(e, m[2], m[3], m[4], m[5]) for e, m in zip(engines, members)],
                     run_flags=HB_RUN_STREAM_NPT(npt) if npt else 0)
    for _ in range(2):
        g.execute()
        _check(members, sem, g.results())
    assert engines[0].last_kernel_time()[2] == 5
    g.close()


def test_group_rejects_short_delays():
    c = single_model("Generic2dOscillator", 20, "heun", "Linear", (0.3,), weights="csr", delays="per_edge")
    ec = BatchHybridEngine.from_config(c, 2, semantics=HB_SEM_DELAY_RING)
    with pytest.raises(Unsupported, match="streamed-history"):
        GroupedSweep([(ec, SweepParam(0, 1), [0.0, 0.1], 50, None)])


@pytest.mark.parametrize("big", [False, True])
def test_group_many_points_per_cta(big):
    """More work items than resident CTAs (about 150 on the device): each CTA of the persistent
    work-queue kernel runs several points one after another and must leave its barriers and shared
    memory as it found them. big: a 150-node member moves the launch to two nodes per consumer thread."""
    members = []
    sizes = [(20, 200, 240), (28, 200, 300)] + ([(150, 40, 160)] if big else [])
    for i, (n, pts, steps) in enumerate(sizes):
        cfg = single_model("MontbrioPazoRoxin", n, "rk4", "Linear", (0.3,), weights="csr", delays="per_edge_long",
                           dt=0.05, seed=10 + i)
        vals = np.linspace(-1.0, 0.5, pts).astype(np.float32).tolist()
        members.append((cfg, pts, SweepParam(0, 4), vals, steps, None))
    engines = [BatchHybridEngine.from_config(c, p, semantics=HB_SEM_DELAY_RING) for c, p, *_ in members]
    g = GroupedSweep([(e, m[2], m[3], m[4], m[5]) for e, m in zip(engines, members)])
    for _ in range(2):
        g.execute()
        _check(members, HB_SEM_DELAY_RING, g.results())
    g.close()


@pytest.mark.parametrize("sem", [HB_SEM_DELAY_RING, HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT])
@pytest.mark.parametrize("exact", [True, False])
def test_group_large_member_split_over_a_cluster(sem, exact):
    """Clusters of 4 CTAs (the launch's choice for a 400-node member): its 6 points run split over a
    cluster (100 nodes per CTA), while the 30- and 70-node members run 4 points per cluster, one per CTA;
    the MPR grid's (G, eta) tables,
    different step counts, a first and a repeated execution.
    exact (HB_RUN_EXACT_SUMS, the reference's summation order): every member's states equal the FP32
    oracle's bit for bit (no transcendental functions in MPR; BOLD to the usual tolerance).
    Default (regrouped, fused sums): this grid's last point amplifies the reordering of its 80-term
    sums to about 3e-5 relative over the 160 RK4 steps (the one-CTA form of the same run reaches
    1.2e-5), so the default form is held to 5e-5."""
    from hyburn_gb300 import inputs
    from hyburn_gb300._abi import HB_RUN_EXACT_SUMS, HB_RUN_STREAM_CLUSTER
    mons = [MonitorConfig("Bold", tr=0.004, bold_period=10)]
    members = []
    cfg, meta = inputs.mpr_grid(400, 6, 160, seed=7, bold=False)
    if sem & HB_SEM_BOLD_PER_POINT:
        cfg.monitors = mons
    members.append((cfg, 6, SweepParam(-1, 0), meta["values"], 160, None))
    for i, (n, pts, steps) in enumerate([(30, 5, 200), (70, 7, 120)]):
        c = single_model("MontbrioPazoRoxin", n, "rk4", "Linear", (0.3,), weights="csr", delays="per_edge_long",
                         monitors=mons if sem & HB_SEM_BOLD_PER_POINT else [], dt=0.05, seed=20 + i)
        vals = np.linspace(-1.0, 0.5, pts).astype(np.float32).tolist()
        members.append((c, pts, SweepParam(0, 4), vals, steps, None))
    engines = [BatchHybridEngine.from_config(c, p, semantics=sem) for c, p, *_ in members]
    g = GroupedSweep([(e, m[2], m[3], m[4], m[5]) for e, m in zip(engines, members)],
                     run_flags=(HB_RUN_EXACT_SUMS if exact else 0) | HB_RUN_STREAM_CLUSTER(4))
    for _ in range(2):
        g.execute()
        for (cfg_m, n_pts, param, vals, n_steps, noise), r in zip(members, g.results()):
            o = OracleEngine.from_config(cfg_m, n_pts, semantics=sem).run_sweep(param, vals, n_steps, noise=noise)
            what = f"{cfg_m.network.subnetworks[0].nnodes} nodes"
            if exact:
                assert np.array_equal(r.final_states[0], o.final_states[0]), what
                assert np.array_equal(r.tavg[0], o.tavg[0]), what
            else:
                close(r.final_states[0], o.final_states[0], rtol=5e-5, what=f"final ({what})")
                close(r.tavg[0], o.tavg[0], rtol=5e-5, what=f"tavg ({what})")
            if o.bold is not None:
                for m in range(len(o.bold)):
                    close(r.bold[m], o.bold[m], atol=BOLD_ATOL, what="bold")
    g.close()
