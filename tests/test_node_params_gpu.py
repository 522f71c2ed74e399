"""Per-node model parameters on the GPU: every kernel form against the oracle (rel 1e-5, abs 1e-6), and
the order-parameter adjoint's per-node omega gradient against central differences of the FP64
restatement."""
import copy

import numpy as np
import pytest

from hyburn_gb300 import BatchHybridEngine, GroupedSweep, SweepParam, inputs
from hyburn_gb300._abi import (HB_RUN_GENERIC, HB_RUN_NO_PIPE, HB_RUN_STREAM, HB_RUN_STREAM_NPT,
                               HB_SEM_BOLD_PER_POINT, HB_SEM_DELAY_RING)
from hyburn_gb300.config import InvalidConfig, Unsupported
from oracle.hb_oracle import OracleEngine

import kuramoto_adjoint_ref as kr
from cases import single_model
from test_parity_gpu import close, compare

pytestmark = pytest.mark.gpu

# kernel forms (hb_engine_last_kernel_time kind): generic 1, specialised 2, pipeline 3, streamed 4
FORMS = [(0, 3), (HB_RUN_NO_PIPE, 2), (HB_RUN_GENERIC, 1), (HB_RUN_STREAM | HB_RUN_STREAM_NPT(1), 4),
         (HB_RUN_STREAM | HB_RUN_STREAM_NPT(2), 4), (HB_RUN_STREAM | HB_RUN_STREAM_NPT(4), 4)]


def with_rows(cfg, rows):
    c = copy.deepcopy(cfg)
    c.network.subnetworks[0].node_params = np.asarray(rows, np.float32)
    return c


@pytest.mark.parametrize("flags,kind", FORMS)
def test_g2do_node_rows_every_kernel_form(flags, kind):
    cfg, meta = inputs.batched_sweep(n_steps=400, n_points=6)
    p = np.asarray(cfg.network.subnetworks[0].params, np.float32)
    rng = np.random.default_rng(9)
    rows = np.tile(p, (74, 1))
    rows[:, 1] = rng.uniform(-0.3, 0.3, 74)
    rows[:, 2] = rng.uniform(-2.5, -1.5, 74)
    noise = inputs.standard_normal((400, 148), 5)
    eng, _, _, _ = compare(with_rows(cfg, rows), 6, SweepParam(-1, 0), meta["values"][:6], 400,
                           semantics=HB_SEM_DELAY_RING, noise=noise, run_flags=flags)
    assert eng.last_kernel_time()[2] == kind


@pytest.mark.parametrize("flags,kind", FORMS)
def test_kuramoto_omega_per_node_every_kernel_form(flags, kind):
    """Phases are compared on the circle; tavg of wrapped phases at rel 2e-5 as the other Kuramoto tests."""
    cfg = single_model("Kuramoto", 60, "heun", "Kuramoto", (2.0,), weights="csr", delays="per_edge_long", density=0.2)
    omega = np.random.default_rng(3).standard_normal((60, 1)).astype(np.float32)
    c = with_rows(cfg, omega)
    eng = BatchHybridEngine.from_config(c, 4, semantics=HB_SEM_DELAY_RING)
    ora = OracleEngine.from_config(c, 4, semantics=HB_SEM_DELAY_RING)
    vals = [0.5, 1.0, 1.5, 2.5]
    g = eng.run_sweep(SweepParam(-1, 0), vals, 300, run_flags=flags)
    o = ora.run_sweep(SweepParam(-1, 0), vals, 300)
    assert eng.last_kernel_time()[2] == kind
    d = (np.asarray(g.final_states[0], np.float64) - o.final_states[0] + np.pi) % (2 * np.pi) - np.pi
    assert np.abs(d).max() <= 2e-5 * 2 * np.pi
    close(g.tavg[0], o.tavg[0], 2e-5, 1e-6, "tavg")


def test_native_sweep_overrides_node_rows_on_gpu():
    cfg, meta = inputs.batched_sweep(n_steps=300, n_points=4, nsig=0.0, integrator="heun")
    p = np.asarray(cfg.network.subnetworks[0].params, np.float32)
    rows = np.tile(p, (74, 1))
    rows[:, 1] = np.linspace(-0.2, 0.2, 74)
    rows[:, 5] = np.linspace(0.015, 0.025, 74)  # d, not swept: stays per node
    compare(with_rows(cfg, rows), 4, SweepParam(0, 1), [0.0, 0.1, 0.2, 0.3], 300, semantics=HB_SEM_DELAY_RING)


def test_mpr_eta_per_point_grouped_launch():
    """The uneven-batching grid in small: per-point eta tables with the coupling scale swept, two
    network sizes in one grouped launch with BOLD, each member against the oracle."""
    members, refs = [], []
    T = 400
    for n, seed in ((20, 3), (36, 4)):
        cfg, meta = inputs.mpr_grid(n, 6, T, seed=seed, bold=True, eta_per_point=False)
        G = np.linspace(0.0, 1.0, 3).astype(np.float32)
        eta = np.asarray([-6.0, -3.0], np.float32)
        p = np.asarray(cfg.network.subnetworks[0].params, np.float32)
        rows = np.tile(p, (6, n, 1))
        rows[:, :, 2] = np.repeat(np.tile(eta, 3), n).reshape(6, n)
        c = with_rows(cfg, rows)
        c.monitors[0].tr = 0.005  # a BOLD sample every 100 steps
        vals = np.repeat(G, 2)
        eng = BatchHybridEngine.from_config(c, 6, semantics=HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT)
        members.append((eng, SweepParam(-1, 0), vals, T, None))
        refs.append(OracleEngine.from_config(c, 6, semantics=HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT).run_sweep(
            SweepParam(-1, 0), vals, T))
    g = GroupedSweep(members)
    g.execute()
    res = g.results()
    for i, o in enumerate(refs):
        r = res[i]
        close(r.final_states[0], o.final_states[0], what=f"final[{i}]")
        close(r.tavg[0], o.tavg[0], what=f"tavg[{i}]")
        close(r.bold[0], o.bold[0], 1e-5, 2e-5, f"bold[{i}]")
    g.close()


def test_node_rows_validation_and_fc_adjoint_refusal():
    cfg = single_model("Kuramoto", 8, "heun", "Kuramoto", (1.0,), weights="csr", delays="per_edge_long")
    with pytest.raises(InvalidConfig):
        BatchHybridEngine.from_config(with_rows(cfg, np.zeros(5, np.float32)), 2, semantics=HB_SEM_DELAY_RING)
    jr, meta = inputs.jr_fc_adjoint(100, 2, 12)
    p = np.asarray(jr.network.subnetworks[0].params, np.float32)
    eng = BatchHybridEngine.from_config(with_rows(jr, np.tile(p, (12, 1))), 2, semantics=HB_SEM_DELAY_RING)
    with pytest.raises(Unsupported):
        eng.adjoint_fc(meta["gains"][:2], 100, np.eye(12, dtype=np.float32))


@pytest.mark.parametrize("flags,kind", [(0, 3), (HB_RUN_STREAM, 4), (HB_RUN_GENERIC, 1)])
def test_order_adjoint_per_node_omega_matches_central_differences(flags, kind):
    """dL/domega_i for omega ~ N(0, 1) per node, against central differences (h = 1e-6) of the FP64
    forward, within 1e-4 |fd| + 2e-6 as the shared-omega test; the per-point d_omega is their sum."""
    n, T, h = 16, 300, 1e-6
    cfg = single_model("Kuramoto", n, "heun", "Kuramoto", (1.0,), weights="csr", delays="per_edge_long", density=0.3,
                       seed=3)
    omega = np.random.default_rng(11).standard_normal(n).astype(np.float32)
    c = with_rows(cfg, omega.reshape(n, 1))
    pr = cfg.network.projections[0]
    net = (np.asarray(pr.weights["indptr"]), np.asarray(pr.weights["indices"]),
           np.asarray(pr.weights["data"], np.float64), np.asarray(pr.delays, np.int64))
    th0 = np.asarray(cfg.network.subnetworks[0].initial_state, np.float64)
    gains = [0.6, 1.9]
    eng = BatchHybridEngine.from_config(c, 2, semantics=HB_SEM_DELAY_RING)
    r = eng.adjoint_order(gains, T, run_flags=flags)
    assert eng.last_kernel_time()[2] == kind
    eng.close()
    om64 = omega.astype(np.float64)
    for b, a in enumerate(gains):
        L = lambda o: kr.order_loss(kr.forward(th0, o, a, *net, cfg.dt, T)[0])
        fd = np.array([(L(om64 + h * np.eye(n)[i]) - L(om64 - h * np.eye(n)[i])) / (2 * h) for i in range(n)])
        _, _, g64 = kr.adjoint(th0, om64, a, *net, cfg.dt, T)
        assert np.abs(g64 - fd).max() <= 1e-8
        err = np.abs(r.d_omega_node[b] - fd)
        assert (err <= 1e-4 * np.abs(fd) + 2e-6).all(), (b, err.max(), np.abs(fd).max())
        assert abs(r.d_omega[b] - r.d_omega_node[b].sum()) <= 1e-9 * max(1.0, abs(r.d_omega[b]))
