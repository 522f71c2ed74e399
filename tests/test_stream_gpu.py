"""Parity of the streamed-history kernel (delay history in HBM, [node][time][channel] layout)
with the CPU oracle. Small networks force it with HB_RUN_STREAM; large ones select it because
their history ring does not fit shared memory. Same tolerances as the other parity tests."""
import numpy as np
import pytest

from hyburn_gb300 import BatchHybridEngine, SweepParam
from hyburn_gb300._abi import (HB_RUN_STREAM, HB_RUN_STREAM_NPT, HB_RUN_STREAM_PREFETCH, HB_SEM_BOLD_PER_POINT,
                               HB_SEM_DELAY_RING, HB_SEM_NOISE_PER_POINT)
from hyburn_gb300.config import MonitorConfig, Unsupported
from oracle.hb_oracle import OracleEngine

from cases import NATIVE_SWEEP, noise_for, single_model, sweep_values
from test_parity_gpu import BOLD_ATOL, INTEGRATORS, close, compare

pytestmark = pytest.mark.gpu
STREAM_KIND = 4


def kind(eng):
    return eng.last_kernel_time()[2]


@pytest.mark.parametrize("model,coupling,cparams", [
    ("Generic2dOscillator", "Linear", (0.1,)),
    ("Kuramoto", "Kuramoto", (2.0,)),
    ("MontbrioPazoRoxin", "Linear", (0.5,)),
    ("WilsonCowan", "Sigmoidal", (1.0, 0.0, 2.0)),
    ("ReducedWongWang", "ScaledLinear", (0.3, 0.1)),
    ("JansenRit", "Linear", (0.01,)),
    ("Generic2dOscillator", "Difference", (0.1,)),
])
def test_stream_per_edge_delays(model, coupling, cparams):
    """runtime.rs:125-211 semantics (zero rows for d > s, current state at step 0) through the
    streamed history, with trajectories."""
    cfg = single_model(model, 24, "heun", coupling, cparams, weights="csr", delays="per_edge_long", density=0.3)
    eng, _, _, _ = compare(cfg, 3, SweepParam(0, NATIVE_SWEEP[model]), sweep_values(model, 3), 400,
                           semantics=HB_SEM_DELAY_RING, traj=True, run_flags=HB_RUN_STREAM)
    assert kind(eng) == STREAM_KIND


@pytest.mark.parametrize("integrator", INTEGRATORS)
def test_stream_integrators_bold_and_chunked_runs(integrator):
    """Every integrator, per-point BOLD, and runs split across calls (the HBM history and the
    running sums carry over between launches)."""
    mons = [MonitorConfig("Bold", tr=0.003, bold_period=10)]
    cfg = single_model("Generic2dOscillator", 40, integrator, "Linear", (0.2,), weights="csr",
                       delays="per_edge_long", nsig=1e-3, monitors=mons)
    sem = HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT
    eng = BatchHybridEngine.from_config(cfg, 3, semantics=sem)
    ora = OracleEngine.from_config(cfg, 3, semantics=sem)
    for n in (333, 201, 9):
        nz = noise_for(cfg, n, 3, False, n)
        g = eng.run_sweep(SweepParam(-1, 0), [0.0, 0.1, 0.2], n, noise=nz, run_flags=HB_RUN_STREAM)
        o = ora.run_sweep(SweepParam(-1, 0), [0.0, 0.1, 0.2], n, noise=nz)
        close(g.final_states[0], o.final_states[0], what=f"final after {n}")
        close(g.tavg[0], o.tavg[0], what=f"tavg after {n}")
        close(g.bold[0], o.bold[0], atol=BOLD_ATOL, what=f"bold after {n}")
        assert kind(eng) == STREAM_KIND


def test_stream_batch_mean_bold_and_noise_per_point():
    mons = [MonitorConfig("Bold", tr=0.004, bold_period=7)]
    cfg = single_model("MontbrioPazoRoxin", 30, "rk4_stochastic", "Linear", (0.3,), weights="csr",
                       delays="per_edge_long", nsig=1e-4, monitors=mons, dt=0.05)
    sem = HB_SEM_DELAY_RING | HB_SEM_NOISE_PER_POINT
    nz = noise_for(cfg, 300, 4, True, 11)
    eng, _, _, _ = compare(cfg, 4, SweepParam(0, 4), [-1.0, -0.5, 0.0, 0.5], 300, semantics=sem, noise=nz,
                           run_flags=HB_RUN_STREAM)
    assert kind(eng) == STREAM_KIND


def test_stream_coupling_sweep_batched_workload_small():
    """The batched-sweep workload (per-edge delays 37-666, Heun-stochastic) with its history in HBM."""
    from hyburn_gb300 import inputs
    cfg, meta = inputs.batched_sweep(n_steps=900, n_points=16)
    nz = inputs.standard_normal((900, 74 * 2), 4)
    eng, _, _, _ = compare(cfg, 16, SweepParam(-1, 0), meta["values"], 900, semantics=HB_SEM_DELAY_RING, noise=nz,
                           run_flags=HB_RUN_STREAM, traj=True)
    assert kind(eng) == STREAM_KIND


@pytest.mark.parametrize("flags", [0, HB_RUN_STREAM_NPT(4), HB_RUN_STREAM_PREFETCH, HB_RUN_STREAM_NPT(4) | HB_RUN_STREAM_PREFETCH])
def test_stream_selected_when_history_exceeds_shared_memory(flags):
    """MPR, 500 nodes, delays up to ~1330 steps: the ring (5.3 MB per point) only fits HBM; two or
    four nodes per consumer thread, with and without L2 prefetch of upcoming edges."""
    from hyburn_gb300 import inputs
    cfg, meta = inputs.mpr_grid(500, 3, 150, seed=3)
    eng, _, _, _ = compare(cfg, 3, SweepParam(-1, 0), [0.0, 0.5, 1.0], 150, semantics=HB_SEM_DELAY_RING,
                           run_flags=flags)
    assert kind(eng) == STREAM_KIND


def test_stream_kuramoto_1000_nodes():
    from hyburn_gb300 import inputs
    cfg, meta = inputs.kuramoto_scale(n=1000, n_points=3, n_steps=80, bold=True)
    eng, _, _, _ = compare(cfg, 3, SweepParam(-1, 0), [0.0, 1.0, 2.0], 80, semantics=HB_SEM_DELAY_RING, rtol=2e-5)
    assert kind(eng) == STREAM_KIND


def test_history_layout_cannot_change_mid_simulation():
    from hyburn_gb300.config import Unsupported
    cfg = single_model("Generic2dOscillator", 24, "heun", "Linear", (0.1,), weights="csr", delays="per_edge_long")
    eng = BatchHybridEngine.from_config(cfg, 2, semantics=HB_SEM_DELAY_RING)
    eng.run_sweep(SweepParam(0, 1), [0.0, 0.1], 50, run_flags=HB_RUN_STREAM)
    with pytest.raises(Unsupported, match="history layout"):
        eng.run_sweep(SweepParam(0, 1), [0.0, 0.1], 50)
    eng.reset()
    eng.run_sweep(SweepParam(0, 1), [0.0, 0.1], 50)
    assert np.isfinite(eng.states[0]).all()


@pytest.mark.parametrize("C,npt", [(2, 2), (3, 2), (4, 1), (4, 2), (5, 2), (6, 2), (8, 1), (8, 2)])
def test_stream_cluster_split_kuramoto(C, npt):
    """One point's 1000 nodes split over a cluster of C CTAs (HB_RUN_STREAM_CLUSTER): the CTAs read
    each other's history through global memory after each block's cluster-scope signal; per-node
    omega, per-point BOLD, with one (where a slice fits 512 threads) and two nodes per consumer thread."""
    from hyburn_gb300 import inputs
    from hyburn_gb300._abi import HB_RUN_STREAM_CLUSTER
    cfg, meta = inputs.kuramoto_scale(n=1000, n_points=3, n_steps=200, bold=True)
    cfg.monitors[0].tr = 0.005
    eng, _, _, _ = compare(cfg, 3, SweepParam(-1, 0), [0.0, 1.0, 2.0], 200, rtol=2e-5,
                           semantics=HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT,
                           run_flags=HB_RUN_STREAM | HB_RUN_STREAM_CLUSTER(C) | HB_RUN_STREAM_NPT(npt))
    assert kind(eng) == STREAM_KIND


@pytest.mark.parametrize("C", [2, 6, 8])
def test_stream_cluster_split_stochastic_chunked(C):
    """Uneven slices (74 nodes over C CTAs), shared noise staged per slice, trajectories, runs split
    across calls: the same results as the oracle."""
    from hyburn_gb300 import inputs
    from hyburn_gb300._abi import HB_RUN_STREAM_CLUSTER
    cfg, meta = inputs.batched_sweep(n_steps=500, n_points=6)
    eng = BatchHybridEngine.from_config(cfg, 6, semantics=HB_SEM_DELAY_RING)
    ora = OracleEngine.from_config(cfg, 6, semantics=HB_SEM_DELAY_RING)
    for n in (300, 77):
        nz = inputs.standard_normal((n, 148), n)
        flags = HB_RUN_STREAM | HB_RUN_STREAM_CLUSTER(C)
        g = eng.run_sweep_with_trajectory(SweepParam(-1, 0), meta["values"], n, noise=nz, run_flags=flags)
        o = ora.run_sweep_with_trajectory(SweepParam(-1, 0), meta["values"], n, noise=nz)
        close(g.final_states[0], o.final_states[0], what=f"final after {n}")
        close(g.tavg[0], o.tavg[0], what=f"tavg after {n}")
        close(g.trajectories[0], o.trajectories[0], what=f"trajectory after {n}")
        assert kind(eng) == STREAM_KIND


def test_stream_cluster_split_mpr_500_nodes():
    from hyburn_gb300 import inputs
    from hyburn_gb300._abi import HB_RUN_STREAM_CLUSTER
    cfg, meta = inputs.mpr_grid(500, 3, 150, seed=3)
    eng, _, _, _ = compare(cfg, 3, SweepParam(-1, 0), [0.0, 0.5, 1.0], 150, semantics=HB_SEM_DELAY_RING,
                           run_flags=HB_RUN_STREAM_CLUSTER(4))
    assert kind(eng) == STREAM_KIND


@pytest.mark.parametrize("C", [4, 6])
def test_stream_bulk_staged_gather_kuramoto(C):
    """HB_RUN_STREAM_BULK: the warp-cooperative gather with every edge window staged into shared memory
    by the bulk-copy engine (per-warp mbarrier, bounded waits), 4 and 6 CTAs per point (a slice's edge
    lists must sit in shared memory); the [sin, cos] channels (80-byte slots), per-node omega, per-point
    BOLD, against the oracle. One CTA per point is refused: its edge lists do not fit."""
    from hyburn_gb300 import inputs
    from hyburn_gb300._abi import HB_RUN_STREAM_BULK, HB_RUN_STREAM_CLUSTER
    cfg, meta = inputs.kuramoto_scale(n=1000, n_points=3, n_steps=200, bold=True)
    cfg.monitors[0].tr = 0.005
    eng, _, _, _ = compare(cfg, 3, SweepParam(-1, 0), [0.0, 1.0, 2.0], 200, rtol=2e-5,
                           semantics=HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT,
                           run_flags=HB_RUN_STREAM | HB_RUN_STREAM_CLUSTER(C) | HB_RUN_STREAM_BULK)
    assert kind(eng) == STREAM_KIND
    with pytest.raises(Unsupported):
        eng.run_sweep(SweepParam(-1, 0), [0.0, 1.0, 2.0], 20, run_flags=HB_RUN_STREAM | HB_RUN_STREAM_CLUSTER(1) | HB_RUN_STREAM_BULK)


def test_stream_bulk_staged_gather_one_channel():
    """HB_RUN_STREAM_BULK with one coupling channel (48-byte slots, windows starting at any 4-byte entry):
    a 300-node Generic2dOscillator network with 20 % CSR coupling, split over 2 CTAs, against the oracle."""
    from hyburn_gb300._abi import HB_RUN_STREAM_BULK, HB_RUN_STREAM_CLUSTER
    cfg = single_model("Generic2dOscillator", 300, "heun", "Linear", (0.02,), weights="csr", delays="per_edge_long", seed=4)
    eng, _, _, _ = compare(cfg, 2, SweepParam(-1, 0), [0.0, 0.5], 120, semantics=HB_SEM_DELAY_RING,
                           run_flags=HB_RUN_STREAM | HB_RUN_STREAM_CLUSTER(2) | HB_RUN_STREAM_BULK)
    assert kind(eng) == STREAM_KIND
