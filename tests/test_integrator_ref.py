"""The reference's integrator and uncoupled-run tests (src/engine/integrator.rs:336-469,
src/engine/mod.rs:49-87), restated as whole runs: on the CPU through the oracle, on the GPU through the
CUDA engine (against the oracle at rel 1e-5 / abs 1e-6, and for the properties themselves).

The reference draws its noise inside the step; this engine takes the N(0, 1) draws from the caller and
scales them by sqrt(2 nsig) sqrt(dt) per state variable, so "two runs draw different noise" becomes "two
draw arrays give different results, the same array gives the same result"."""
import numpy as np
import pytest

from hyburn_gb300.config import DEFAULT_PARAMS, NetworkConfig, ProjectionConfig, SimConfig, SubnetworkConfig
from hyburn_gb300.engine import SweepParam

G2DO = list(DEFAULT_PARAMS["Generic2dOscillator"])
NATIVE = SweepParam(0, 1)  # G2DO's I, the batch-native sweep index (dfun.rs:49-72)


def g2do(n, x0, integrator="heun", nsig=0.0, coupled=False):
    """n G2DO nodes; uncoupled (no projection, as the reference tests), or with a projection of weight
    0, which must give the same numbers."""
    projs = [ProjectionConfig(0, 0, 0.0, coupling_fn="Linear", coupling_params=[1.0, 0.0])] if coupled else []
    return SimConfig(sim_length=0.1, dt=0.1, integrator=integrator, nsig=nsig,
                     network=NetworkConfig([SubnetworkConfig("Generic2dOscillator", n, list(x0), list(G2DO))], projs))


def run(engine_cls, cfg, n_steps, noise=None, traj=False):
    eng = engine_cls.from_config(cfg, 1)
    return eng.run_sweep(NATIVE, [G2DO[1]], n_steps, noise=noise, run_flags=1 if traj else 0)


def oracle():
    from oracle.hb_oracle import OracleEngine
    return OracleEngine


X2 = [0.1, 0.5, 0.2, 0.4]                      # integrator.rs:339-342, [2 nodes][V, W]
X4 = [0.1, 0.5, 0.2, 0.4, 0.3, 0.1, 0.0, 0.2]  # integrator.rs:373-376


# ---- CPU: the oracle ----

def test_rk4_differs_from_euler_and_heun():  # integrator.rs:337-364
    out = {k: run(oracle(), g2do(2, X2, k), 1).final_states[0] for k in ("euler", "heun", "rk4")}
    for v in out.values():
        assert np.isfinite(v).all()
    assert np.abs(out["euler"] - out["rk4"]).sum() > 1e-8
    assert np.abs(out["heun"] - out["rk4"]).sum() > 1e-8


@pytest.mark.parametrize("kind", ["euler_stochastic", "heun_stochastic", "rk4_stochastic"])
def test_stochastic_runs_differ_with_the_draws(kind):  # integrator.rs:367-387
    cfg = g2do(4, X4, kind, nsig=[0.1, 0.2])
    a = np.random.default_rng(1).standard_normal((1, 8), dtype=np.float32)
    b = np.random.default_rng(2).standard_normal((1, 8), dtype=np.float32)
    ra, rb, ra2 = (run(oracle(), cfg, 1, z).final_states[0] for z in (a, b, a))
    assert np.isfinite(ra).all() and np.isfinite(rb).all()
    assert np.abs(ra - rb).sum() > 1e-6
    assert np.array_equal(ra, ra2)


@pytest.mark.parametrize("kind,det", [("euler_stochastic", "euler"), ("rk4_stochastic", "rk4")])
def test_per_variable_noise_zero_scale(kind, det):  # integrator.rs:390-410, 462-469
    """nsig = [0, 0.1]: Euler-Maruyama and the stochastic RK4 add the noise once, after the deterministic
    update, so after one step the first variable is the deterministic step's, bit for bit; the second is
    not. (Heun's predictor carries the noise of the second variable into the corrector's derivative of
    the first, so there only nsig = 0 for every variable gives the deterministic step.)"""
    z = np.random.default_rng(3).standard_normal((1, 4), dtype=np.float32)
    s = run(oracle(), g2do(2, X2, kind, nsig=[0.0, 0.1]), 1, z).final_states[0].reshape(2, 2)
    d = run(oracle(), g2do(2, X2, det), 1).final_states[0].reshape(2, 2)
    assert np.array_equal(s[:, 0], d[:, 0])
    assert not np.array_equal(s[:, 1], d[:, 1])


@pytest.mark.parametrize("kind,det", [("euler_stochastic", "euler"), ("heun_stochastic", "heun"),
                                      ("rk4_stochastic", "rk4")])
def test_zero_noise_scale_is_the_deterministic_step(kind, det):  # integrator.rs:390-410
    z = np.random.default_rng(4).standard_normal((50, 4), dtype=np.float32)
    s = run(oracle(), g2do(2, X2, kind, nsig=[0.0, 0.0]), 50, z).final_states[0]
    d = run(oracle(), g2do(2, X2, det), 50).final_states[0]
    assert np.array_equal(s, d)


def test_g2do_no_coupling_1000_steps():  # engine/mod.rs:49-87
    r = run(oracle(), g2do(2, [0.0] * 4), 1000, traj=True)
    assert np.isfinite(r.final_states[0]).all() and np.isfinite(r.trajectories[0]).all()
    # a projection of weight 0 is the same network
    r0 = run(oracle(), g2do(2, [0.0] * 4, coupled=True), 1000, traj=True)
    assert np.array_equal(r.final_states[0], r0.final_states[0])
    assert np.array_equal(r.trajectories[0], r0.trajectories[0])


# ---- GPU: the CUDA engine (networks with a projection of weight 0) ----

@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["euler", "heun", "rk4"])
def test_engine_deterministic_steps(kind):
    from test_parity_gpu import compare
    compare(g2do(2, X2, kind, coupled=True), 1, NATIVE, [G2DO[1]], 1)
    compare(g2do(2, [0.0] * 4, kind, coupled=True), 1, NATIVE, [G2DO[1]], 1000)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,det", [("euler_stochastic", "euler"), ("heun_stochastic", "heun"),
                                      ("rk4_stochastic", "rk4")])
def test_engine_noise_properties(kind, det):
    from hyburn_gb300 import BatchHybridEngine
    from test_parity_gpu import compare
    a = np.random.default_rng(1).standard_normal((1, 8), dtype=np.float32)
    b = np.random.default_rng(2).standard_normal((1, 8), dtype=np.float32)
    cfg = g2do(4, X4, kind, nsig=[0.1, 0.2], coupled=True)
    compare(cfg, 1, NATIVE, [G2DO[1]], 1, noise=a)
    ra, rb, ra2 = (run(BatchHybridEngine, cfg, 1, z).final_states[0] for z in (a, b, a))
    assert np.abs(ra - rb).sum() > 1e-6 and np.array_equal(ra, ra2)
    # zero noise scale: the deterministic step (within the FP32 tolerance: the stochastic and deterministic
    # kernels are separate instantiations)
    z = np.random.default_rng(3).standard_normal((1, 4), dtype=np.float32)
    d = run(BatchHybridEngine, g2do(2, X2, det, coupled=True), 1).final_states[0].reshape(2, 2)
    s0 = run(BatchHybridEngine, g2do(2, X2, kind, nsig=[0.0, 0.0], coupled=True), 1, z).final_states[0].reshape(2, 2)
    assert np.allclose(s0, d, rtol=1e-6, atol=1e-7)
    if kind != "heun_stochastic":
        s = run(BatchHybridEngine, g2do(2, X2, kind, nsig=[0.0, 0.1], coupled=True), 1, z).final_states[0].reshape(2, 2)
        assert np.allclose(s[:, 0], d[:, 0], rtol=1e-6, atol=1e-7)
        assert np.abs(s[:, 1] - d[:, 1]).max() > 1e-4
