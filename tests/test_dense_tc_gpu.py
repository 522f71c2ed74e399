"""Undelayed dense coupling on the tensor cores (HB_RUN_DENSE_TC, hb_dense_tc.cu) against the oracle.

The coupling sums are the batched matrix product of the batch engine (engine.rs:609-620), formed by
tcgen05.mma in three TF32 products with FP32 accumulation; each product term carries a relative error
below 2^-21 and the tensor core sums in its own order, so the comparison uses the parity tolerance of
the other GPU tests (rel 1e-5, abs 1e-6). Tiles of 128 points: the cases include partial tiles.
"""
import numpy as np
import pytest

from hyburn_gb300 import BatchHybridEngine, SweepParam
from hyburn_gb300._abi import HB_RUN_DENSE_TC
from hyburn_gb300.config import NetworkConfig, ProjectionConfig, SimConfig, Unsupported

from cases import NATIVE_SWEEP, noise_for, single_model, sub, sweep_values
from test_parity_gpu import compare

pytestmark = pytest.mark.gpu
TC_KIND = 8


def dense_case(model, n, integrator, coupling, cparams, seed=0, nsig=0.0, scale=1.0, delays=()):
    rng = np.random.default_rng(seed + 100)
    w = (rng.uniform(0.0, 1.0, (n, n)) * scale / n).astype(np.float32)
    np.fill_diagonal(w, 0.0)
    return SimConfig(sim_length=100.0, dt=0.1, integrator=integrator, nsig=nsig,
                     network=NetworkConfig([sub(model, n, seed)],
                                           [ProjectionConfig(0, 0, w.tolist(), coupling_fn=coupling,
                                                             coupling_params=list(cparams), delays=list(delays))]))


@pytest.mark.parametrize("model,n,B,integrator,coupling,cparams", [
    ("Generic2dOscillator", 74, 200, "heun", "Linear", (0.2,)),
    ("Generic2dOscillator", 74, 128, "rk4", "Linear", (0.1, 0.01)),
    ("WilsonCowan", 48, 130, "heun", "Sigmoidal", (1.0, 0.0, 2.0)),
    ("ReducedWongWang", 16, 40, "euler", "ScaledLinear", (0.3, 0.1)),
    ("JansenRit", 24, 129, "heun", "Linear", (0.05,)),
    ("Generic2dOscillator", 96, 256, "heun", "Sigmoidal", (-1.0, 1.0, 0.0, 1.0, 1.0)),
])
def test_dense_tensor_core_matches_oracle(model, n, B, integrator, coupling, cparams):
    cfg = dense_case(model, n, integrator, coupling, cparams)
    eng, _, _, _ = compare(cfg, B, SweepParam(0, NATIVE_SWEEP[model]), sweep_values(model, B), 200,
                           run_flags=HB_RUN_DENSE_TC)
    assert eng.last_kernel_time()[2] == TC_KIND


def test_dense_tensor_core_stochastic_coupling_sweep_and_chunked_runs():
    """Heun-stochastic with the shared draws, the coupling scale swept per point, and a run split over
    two calls (state and running sums carried over)."""
    cfg = dense_case("Generic2dOscillator", 74, "heun_stochastic", "Linear", (0.1,), nsig=1e-3, seed=3)
    B = 300
    vals = np.linspace(0.0, 0.3, B).astype(np.float32)
    from oracle.hb_oracle import OracleEngine
    from test_parity_gpu import close
    eng = BatchHybridEngine.from_config(cfg, B)
    ora = OracleEngine.from_config(cfg, B)
    for T in (150, 61):
        nz = noise_for(cfg, T, B, False, T)
        g = eng.run_sweep(SweepParam(-1, 0), vals, T, noise=nz, run_flags=HB_RUN_DENSE_TC)
        o = ora.run_sweep(SweepParam(-1, 0), vals, T, noise=nz)
        close(g.final_states[0], o.final_states[0], what=f"final after {T}")
        close(g.tavg[0], o.tavg[0], what=f"tavg after {T}")
        assert eng.last_kernel_time()[2] == TC_KIND


def test_dense_tensor_core_refuses_what_it_does_not_cover():
    delayed = dense_case("Generic2dOscillator", 20, "heun", "Linear", (0.1,), delays=[3])
    with pytest.raises(Unsupported, match="delay"):
        BatchHybridEngine.from_config(delayed, 4).run_sweep(SweepParam(0, 1), [0.0] * 4, 10, run_flags=HB_RUN_DENSE_TC)
    kura = single_model("Kuramoto", 20, "heun", "Kuramoto", (1.0,), weights="dense")
    with pytest.raises(Unsupported):
        BatchHybridEngine.from_config(kura, 4).run_sweep(SweepParam(0, 0), [1.0] * 4, 10, run_flags=HB_RUN_DENSE_TC)
    big = dense_case("Generic2dOscillator", 120, "heun", "Linear", (0.1,))
    with pytest.raises(Unsupported, match="112"):
        BatchHybridEngine.from_config(big, 4).run_sweep(SweepParam(0, 1), [0.0] * 4, 10, run_flags=HB_RUN_DENSE_TC)
