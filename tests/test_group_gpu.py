"""Grouped launch (hb_group_*): several engines' sweeps with different node counts, delays, sweep
values and step counts in one launch of the streamed-history kernel, replayed from a CUDA graph.
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


def test_group_rejects_mixed_models_and_short_delays():
    a = single_model("MontbrioPazoRoxin", 20, "rk4", "Linear", (0.3,), weights="csr", delays="per_edge_long", dt=0.05)
    b = single_model("Generic2dOscillator", 20, "heun", "Linear", (0.3,), weights="csr", delays="per_edge_long")
    ea = BatchHybridEngine.from_config(a, 2, semantics=HB_SEM_DELAY_RING)
    eb = BatchHybridEngine.from_config(b, 2, semantics=HB_SEM_DELAY_RING)
    with pytest.raises(Unsupported, match="share the model"):
        GroupedSweep([(ea, SweepParam(0, 4), [0.0, 0.1], 50, None), (eb, SweepParam(0, 1), [0.0, 0.1], 50, None)])
    c = single_model("Generic2dOscillator", 20, "heun", "Linear", (0.3,), weights="csr", delays="per_edge")
    ec = BatchHybridEngine.from_config(c, 2, semantics=HB_SEM_DELAY_RING)
    with pytest.raises(Unsupported, match="streamed-history"):
        GroupedSweep([(ec, SweepParam(0, 1), [0.0, 0.1], 50, None)])
