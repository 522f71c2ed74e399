"""The FP64 NumPy restatement of the Kuramoto order-parameter adjoint (tests/kuramoto_adjoint_ref.py):
its forward against the FP64 oracle, and its gradients against central differences."""
import numpy as np
import pytest

from hyburn_gb300 import SweepParam
from hyburn_gb300._abi import HB_SEM_DELAY_RING
from oracle.hb_oracle import OracleEngine

import kuramoto_adjoint_ref as kr
from cases import single_model


def kura_case(n=16, a=1.0, seed=0, dt=0.1):
    return single_model("Kuramoto", n, "heun", "Kuramoto", (a,), weights="csr", delays="per_edge_long",
                        density=0.3, seed=seed, dt=dt)


def arrays(cfg):
    pr = cfg.network.projections[0]
    w = pr.weights
    indptr, indices, data = (np.asarray(w[k]) for k in ("indptr", "indices", "data"))
    return indptr, indices, data.astype(np.float64), np.asarray(pr.delays, np.int64)


def test_numpy_forward_matches_fp64_oracle():
    n, T = 16, 300
    for a in (0.5, 2.0):
        cfg = kura_case(n, 1.0)
        sub = cfg.network.subnetworks[0]
        th0 = np.asarray(sub.initial_state, np.float64)
        th, _, _ = kr.forward(th0, float(sub.params[0]), a, *arrays(cfg), cfg.dt, T)
        o = OracleEngine.from_config(cfg, 1, semantics=HB_SEM_DELAY_RING, precision="f64").run_sweep_with_trajectory(
            SweepParam(-1, 0), [a], T)
        traj = np.asarray(o.trajectories[0], np.float64).reshape(T, n)
        d = np.abs(np.angle(np.exp(1j * (th[1:] - traj))))   # phases compared modulo 2 pi
        assert d.max() <= 1e-6, d.max()


def test_fp64_adjoint_matches_central_differences():
    n, T = 12, 200
    cfg = kura_case(n, 1.0, seed=2)
    sub = cfg.network.subnetworks[0]
    th0 = np.asarray(sub.initial_state, np.float64)
    net = arrays(cfg)
    omega, a, h = float(sub.params[0]), 1.7, 1e-6
    loss, g_a, g_w = kr.adjoint(th0, omega, a, *net, cfg.dt, T)

    def L(om=omega, aa=a):
        return kr.order_loss(kr.forward(th0, om, aa, *net, cfg.dt, T)[0])

    assert abs(loss - L()) <= 1e-14
    fd_a = (L(aa=a + h) - L(aa=a - h)) / (2 * h)
    fd_w = (L(om=omega + h) - L(om=omega - h)) / (2 * h)
    assert abs(g_a - fd_a) <= 1e-6 * abs(fd_a), (g_a, fd_a)
    assert abs(g_w - fd_w) <= 1e-6 * max(abs(fd_w), 1e-3), (g_w, fd_w)


@pytest.mark.gpu
@pytest.mark.parametrize("n,T,dt,form", [(16, 300, 0.1, "pipe"), (40, 500, 0.05, "pipe"), (16, 300, 0.1, "stream"),
                                        (40, 500, 0.05, "stream"), (16, 300, 0.1, "generic"),
                                        (128, 300, 0.1, "stream")])
def test_gpu_order_adjoint_matches_central_differences(n, T, dt, form):
    """hb_engine_adjoint_order against central differences (h = 1e-6) of the FP64 forward. With 128
    nodes and two points the streamed forward and the reverse sweep both split each point over a
    2-CTA cluster (64 nodes per CTA). The GPU differentiates its FP32 trajectory, whose phases drift
    from the FP64 ones by ~1e-6 over these runs: the loss agrees within 1e-4 (relative; measured 1e-5), each gradient within
    1e-4 |fd| + 2e-6 — the absolute floor covers gradients that nearly cancel (measured: dL/domega
    = -2.7e-4 off by 7.7e-7 on the 40-node case; elsewhere 3e-7 to 4e-5 relative)."""
    from hyburn_gb300 import BatchHybridEngine
    cfg = kura_case(n, 1.0, seed=3, dt=dt)
    sub = cfg.network.subnetworks[0]
    th0 = np.asarray(sub.initial_state, np.float64)
    net = arrays(cfg)
    omega, h = float(sub.params[0]), 1e-6
    gains = [0.6, 1.9]
    eng = BatchHybridEngine.from_config(cfg, len(gains), semantics=HB_SEM_DELAY_RING)
    from hyburn_gb300._abi import HB_RUN_GENERIC, HB_RUN_STREAM
    flags = {"pipe": 0, "stream": HB_RUN_STREAM, "generic": HB_RUN_GENERIC}[form]
    r = eng.adjoint_order(gains, T, run_flags=flags)
    kind = eng.last_kernel_time()[2]
    eng.close()
    print(f"forward kernel kind {kind}")
    # pipeline (3) and streamed-history (4) forms hand their coupling sums to the reverse sweep; the
    # generic resident form (1) does not, and the reverse gathers them again
    assert kind == {"pipe": 3, "stream": 4, "generic": 1}[form]

    def L(om, aa):
        return kr.order_loss(kr.forward(th0, om, aa, *net, cfg.dt, T)[0])

    for b, a in enumerate(gains):
        l64 = L(omega, a)
        fd_a = (L(omega, a + h) - L(omega, a - h)) / (2 * h)
        fd_w = (L(omega + h, a) - L(omega - h, a)) / (2 * h)
        ea, ew = abs(r.d_gain[b] - fd_a), abs(r.d_omega[b] - fd_w)
        print(f"point {b}: loss {r.loss[b]:.6g} vs {l64:.6g}; dL/da {r.d_gain[b]:.6g} vs {fd_a:.6g} ({ea:.2e}); "
              f"dL/domega {r.d_omega[b]:.6g} vs {fd_w:.6g} ({ew:.2e})")
        assert abs(r.loss[b] - l64) <= 1e-4 * abs(l64)
        assert ea <= 1e-4 * abs(fd_a) + 2e-6 and ew <= 1e-4 * abs(fd_w) + 2e-6
    assert r.forward_ms > 0 and r.reverse_ms > 0
