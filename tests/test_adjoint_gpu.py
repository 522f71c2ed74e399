"""FC-loss adjoint (hb_engine_adjoint_fc), for deterministic Heun and RK4, against central finite
differences of the FP64 NumPy forward, and against the engine's own forward run. Relative errors are 2-norms over each gradient
vector (the gain, and the per-node A, B, a of one sweep point); the bounds are given below.

Step of the differences: h = 1e-6. With h = 1e-3 the central difference has not converged for the
JansenRit rate constant a (0.1 ms^-1): at node 0 of this case it gives -0.112 where h = 1e-4, 1e-5,
1e-6 give -0.05732, -0.056786, -0.0567804 — the loss curves strongly on the scale of 1 % of a. In
FP64 the h = 1e-6 differences agree with h = 1e-5 to five digits for every parameter here.

Precision: the kernels differentiate the FP32 forward trajectory (the run the engine computes); the
differences follow the FP64 one. Gradients that are well conditioned (the coupling gain, the
per-node A and B) agree within 1e-4 (measured 4e-6 - 5.7e-5 here). The per-node rate constant a is
ill conditioned for some nodes: the same FP64 adjoint algorithm (tests/adjoint_ref.py) run along an
FP32 NumPy forward moves node 0's a-gradient by 6 % in a 200-step case while along the FP64 forward
it matches the differences to 1e-8 (tests/test_adjoint_ref.py). The a block is therefore held to
5e-4 (measured 7.6e-5 and 1.14e-4 on the two points of this case).
"""
import numpy as np
import pytest

from hyburn_gb300 import BatchHybridEngine, SweepParam
from hyburn_gb300._abi import HB_SEM_DELAY_RING

import adjoint_ref as ar
from test_adjoint_ref import arrays, jr_case

pytestmark = pytest.mark.gpu
N, T, H_FD = 12, 300, 1e-6
GAINS = [0.8, 1.25]
CP = lambda g: (0.0, 0.1, 0.0, g, 0.05)


def ref_setup(integrator="heun"):
    cfg = jr_case(N, 1.0, integrator=integrator)
    sub = cfg.network.subnetworks[0]
    x0 = np.asarray(sub.initial_state, np.float64).reshape(N, 6)
    indptr, indices, data, delays = arrays(cfg)
    tgt_ys = ar.forward(ar.params_dict(sub.params, N), x0, indptr, indices, data, delays, "Sigmoidal", CP(0.4),
                        cfg.dt, T, integrator)
    target = np.corrcoef(tgt_ys.T)
    return cfg, sub, x0, (indptr, indices, data, delays), target


def loss_at(sub, x0, net, cfg, target, gain, A=None, B=None, a=None):
    p = ar.params_dict(sub.params, N, A, B, a)
    ys = ar.forward(p, x0, *net, "Sigmoidal", CP(gain), cfg.dt, T, cfg.integrator)
    return ar.fc_loss(ys, target)[0]


def rel(g, fd):
    return float(np.linalg.norm(g - fd) / max(np.linalg.norm(fd), 1e-30))


@pytest.mark.parametrize("integrator", ["heun", "rk4"])
def test_adjoint_forward_and_loss_match_engine_and_fp64(integrator):
    cfg, sub, x0, net, target = ref_setup(integrator)
    eng = BatchHybridEngine.from_config(cfg, len(GAINS), semantics=HB_SEM_DELAY_RING)
    r = eng.adjoint_fc(GAINS, T, target, checkpoint_every=64, return_y=True)
    g = eng.run_sweep_with_trajectory(SweepParam(-1, 3), GAINS, T)
    traj = np.asarray(g.trajectories[0]).reshape(T, len(GAINS), N, 6)
    ys = traj[..., 1] - traj[..., 2]
    np.testing.assert_allclose(r.y, ys, rtol=1e-5, atol=1e-6)
    for b, gain in enumerate(GAINS):
        l64 = loss_at(sub, x0, net, cfg, target, gain)
        assert abs(r.loss[b] - l64) <= 1e-4 * abs(l64), (r.loss[b], l64)


@pytest.mark.parametrize("integrator,checkpoint_every", [("heun", 64), ("heun", 0), ("rk4", 64), ("rk4", 0)])
def test_adjoint_gradients_match_central_differences(integrator, checkpoint_every):
    """checkpoint_every 64: segments re-computed from checkpoints (two-phase forward); 0: every
    step kept (pipelined forward and reverse)."""
    cfg, sub, x0, net, target = ref_setup(integrator)
    eng = BatchHybridEngine.from_config(cfg, len(GAINS), semantics=HB_SEM_DELAY_RING)
    r = eng.adjoint_fc(GAINS, T, target, checkpoint_every=checkpoint_every)
    A0, B0, a0 = (float(sub.params[k]) for k in range(3))
    for b, gain in enumerate(GAINS):
        fd_g = (loss_at(sub, x0, net, cfg, target, gain + H_FD) - loss_at(sub, x0, net, cfg, target, gain - H_FD)) / (2 * H_FD)
        errs = {"gain": abs(r.d_gain[b] - fd_g) / abs(fd_g)}
        full_g, full_fd = [np.array([r.d_gain[b]])], [np.array([fd_g])]
        for name, base, got in (("A", A0, r.d_A[b]), ("B", B0, r.d_B[b]), ("a", a0, r.d_a[b])):
            fd = np.zeros(N)
            for i in range(N):
                vp, vm = np.full(N, base), np.full(N, base)
                vp[i] += H_FD
                vm[i] -= H_FD
                kw_p, kw_m = {name: vp}, {name: vm}
                fd[i] = (loss_at(sub, x0, net, cfg, target, gain, **kw_p) -
                         loss_at(sub, x0, net, cfg, target, gain, **kw_m)) / (2 * H_FD)
            errs[name] = rel(got, fd)
            full_g.append(got)
            full_fd.append(fd)
        errs["all"] = rel(np.concatenate(full_g), np.concatenate(full_fd))
        print(f"point {b}: relative errors {errs}")
        for k in ("gain", "A", "B"):
            assert errs[k] <= 1e-4, (b, k, errs)
        assert errs["a"] <= 5e-4, (b, errs)


@pytest.mark.parametrize("integrator", ["heun", "rk4"])
def test_adjoint_checkpoint_interval_changes_only_summation_rounding(integrator):
    cfg, sub, x0, net, target = ref_setup(integrator)
    eng = BatchHybridEngine.from_config(cfg, len(GAINS), semantics=HB_SEM_DELAY_RING)
    r1 = eng.adjoint_fc(GAINS, T, target, checkpoint_every=64)
    r2 = eng.adjoint_fc(GAINS, T, target, checkpoint_every=T)
    r3 = eng.adjoint_fc(GAINS, T, target, checkpoint_every=0)  # every step kept, no re-computation
    for f in ("loss", "d_gain", "d_A", "d_B", "d_a"):
        assert np.array_equal(getattr(r2, f), getattr(r3, f)), f
    # the re-computed trajectory is bitwise the same; the gradient sums regroup per segment (FP32
    # within a segment, FP64 across segments), so they agree to summation rounding
    assert np.array_equal(r1.loss, r2.loss)
    for f in ("d_gain", "d_A", "d_B", "d_a"):
        np.testing.assert_allclose(getattr(r1, f), getattr(r2, f), rtol=1e-5, atol=1e-9 * np.abs(getattr(r2, f)).max())


def test_adjoint_at_fc_workload_scale_with_checkpoints_every_500_steps():
    """The FC-adjoint workload's own network (JansenRit, 74 nodes, 20 % CSR, delays 37-666 steps,
    Sigmoidal coupling) for 2 000 steps with checkpoints every 500 steps, against a target FC of a
    seeded forward run. The FP64 restatement of the adjoint is pinned to central differences
    (h = 1e-6) on the gain and on six nodes' A, B, a; the GPU gradients are then compared with it on
    all 74 nodes: gain, A and B within 1e-4 (2-norm relative), a within 5e-4 (its conditioning, as
    above)."""
    from hyburn_gb300 import inputs
    n, T, K, h = 74, 2000, 500, 1e-6
    gains = [0.8, 1.2]
    cfg, meta = inputs.jr_fc_adjoint(T, len(gains), n)
    sub, pr = cfg.network.subnetworks[0], cfg.network.projections[0]
    w = pr.weights
    net = (np.asarray(w["indptr"]), np.asarray(w["indices"]), np.asarray(w["data"], np.float64),
           np.asarray(pr.delays, np.int64))
    x0 = np.asarray(sub.initial_state, np.float64).reshape(n, 6)
    rng = np.random.default_rng(40)
    ranges = [(-0.5, 0.5), (0.0, 20.0), (0.0, 20.0), (-1.0, 1.0), (-1.0, 1.0), (-1.0, 1.0)]
    x_t = np.stack([rng.uniform(lo, hi, n) for lo, hi in ranges], 1)
    cp = lambda g: (0.0, 0.1, 0.0, g, 0.05)
    target = np.corrcoef(ar.forward(ar.params_dict(sub.params, n), x_t, *net, "Sigmoidal", cp(1.0), cfg.dt, T).T)
    eng = BatchHybridEngine.from_config(cfg, len(gains), semantics=HB_SEM_DELAY_RING)
    r = eng.adjoint_fc(gains, T, target.astype(np.float32), checkpoint_every=K)
    base = {k: float(sub.params[i]) for i, k in enumerate(("A", "B", "a"))}
    nodes = [0, 13, 27, 41, 55, 73]

    def L(gain, **kw):
        return ar.fc_loss(ar.forward(ar.params_dict(sub.params, n, **kw), x0, *net, "Sigmoidal", cp(gain), cfg.dt, T),
                          target)[0]

    for b, gain in enumerate(gains):
        l64, gG, gA, gB, ga = ar.adjoint(ar.params_dict(sub.params, n), x0, *net, cp(gain), cfg.dt, T, target)
        fd_g = (L(gain + h) - L(gain - h)) / (2 * h)
        assert abs(gG - fd_g) <= 1e-6 * abs(fd_g), (gG, fd_g)
        for name, g64 in (("A", gA), ("B", gB), ("a", ga)):
            for i in nodes:
                vp, vm = np.full(n, base[name]), np.full(n, base[name])
                vp[i] += h
                vm[i] -= h
                fd = (L(gain, **{name: vp}) - L(gain, **{name: vm})) / (2 * h)
                assert abs(g64[i] - fd) <= 1e-5 * abs(fd) + 1e-9, (name, i, g64[i], fd)
        assert abs(r.loss[b] - l64) <= 1e-4 * abs(l64)
        errs = {"gain": abs(r.d_gain[b] - gG) / abs(gG), "A": rel(r.d_A[b], gA), "B": rel(r.d_B[b], gB),
                "a": rel(r.d_a[b], ga)}
        print(f"point {b}: relative errors against the FP64 adjoint {errs}")
        assert errs["gain"] <= 1e-4 and errs["A"] <= 1e-4 and errs["B"] <= 1e-4 and errs["a"] <= 5e-4, errs
