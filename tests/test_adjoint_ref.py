"""The FP64 NumPy forward used for the adjoint's finite differences equals the FP64 oracle."""
import numpy as np
import pytest

from hyburn_gb300 import SweepParam
from hyburn_gb300._abi import HB_SEM_DELAY_RING
from oracle.hb_oracle import OracleEngine

import adjoint_ref as ar
from cases import single_model


def jr_case(n=12, gain=1.0, seed=0, integrator="heun"):
    return single_model("JansenRit", n, integrator, "Sigmoidal", (0.0, 0.1, 0.0, gain, 0.05), weights="csr",
                        delays="per_edge_long", density=0.3, seed=seed)


def arrays(cfg):
    pr = cfg.network.projections[0]
    w = pr.weights
    indptr, indices, data = (np.asarray(w[k]) for k in ("indptr", "indices", "data"))
    return indptr, indices, data.astype(np.float64), np.asarray(pr.delays, np.int64)


@pytest.mark.parametrize("integrator", ["heun", "rk4"])
def test_numpy_forward_matches_fp64_oracle(integrator):
    n, T = 12, 300
    for gain in (0.7, 1.3):
        cfg = jr_case(n, gain, integrator=integrator)
        sub = cfg.network.subnetworks[0]
        x0 = np.asarray(sub.initial_state, np.float64).reshape(n, 6)
        indptr, indices, data, delays = arrays(cfg)
        ys = ar.forward(ar.params_dict(sub.params, n), x0, indptr, indices, data, delays, "Sigmoidal",
                        (0.0, 0.1, 0.0, gain, 0.05), cfg.dt, T, integrator)
        o = OracleEngine.from_config(cfg, 1, semantics=HB_SEM_DELAY_RING, precision="f64").run_sweep_with_trajectory(
            SweepParam(-1, 3), [gain], T)
        traj = np.asarray(o.trajectories[0], np.float64).reshape(T, 1, n, 6)[:, 0]
        ref = traj[:, :, 1] - traj[:, :, 2]
        assert np.max(np.abs(ys - ref)) <= 1e-6 * max(1.0, np.max(np.abs(ref))), np.max(np.abs(ys - ref))


@pytest.mark.parametrize("integrator", ["heun", "rk4"])
def test_fp64_adjoint_restatement_matches_central_differences(integrator):
    """The discrete-adjoint algorithm of the GPU kernels (restated in FP64 NumPy) against central
    differences (h = 1e-6) of the FP64 forward: the algorithm itself is exact to ~1e-8."""
    n, T = 8, 120
    cfg = jr_case(n, 1.0, seed=1)
    sub = cfg.network.subnetworks[0]
    x0 = np.asarray(sub.initial_state, np.float64).reshape(n, 6)
    net = arrays(cfg)
    cp = lambda g: (0.0, 0.1, 0.0, g, 0.05)
    target = np.corrcoef(ar.forward(ar.params_dict(sub.params, n), x0, *net, "Sigmoidal", cp(0.4), cfg.dt, T,
                                    integrator).T)
    gain, h = 1.1, 1e-6
    p = ar.params_dict(sub.params, n)
    loss, gG, gA, gB, ga = ar.adjoint(p, x0, *net, cp(gain), cfg.dt, T, target, integrator=integrator)

    def L(g=gain, **kw):
        return ar.fc_loss(ar.forward(ar.params_dict(sub.params, n, **kw), x0, *net, "Sigmoidal", cp(g), cfg.dt, T,
                                     integrator), target)[0]

    assert abs(loss - L()) <= 1e-12
    assert abs(gG - (L(gain + h) - L(gain - h)) / (2 * h)) <= 1e-6 * abs(gG)
    for name, got, base in (("A", gA, sub.params[0]), ("B", gB, sub.params[1]), ("a", ga, sub.params[2])):
        fd = np.zeros(n)
        for i in range(n):
            vp, vm = np.full(n, float(base)), np.full(n, float(base))
            vp[i] += h
            vm[i] -= h
            fd[i] = (L(**{name: vp}) - L(**{name: vm})) / (2 * h)
        assert np.linalg.norm(got - fd) <= 1e-6 * np.linalg.norm(fd), (name, got, fd)
