"""Pipeline kernel paths not covered elsewhere: noise rows that are not a multiple of 16 bytes (no
bulk copy), the 1024-thread form with eight producer lanes, and deterministic Heun through the
straight-line consumer loop with two coupling variables."""
import pytest

from hyburn_gb300 import SweepParam
from hyburn_gb300._abi import HB_RUN_PIPE_LANES, HB_RUN_PIPE_WIDE, HB_SEM_DELAY_RING

from cases import NATIVE_SWEEP, noise_for, single_model, sweep_values
from test_parity_gpu import compare

pytestmark = pytest.mark.gpu
PIPE_KIND = 3


def test_noise_rows_not_multiple_of_16_bytes():
    # 25 nodes x 2 variables = 50 floats per row: staged by the producers' own loads
    cfg = single_model("Generic2dOscillator", 25, "heun_stochastic", "Linear", (0.2,), weights="csr",
                       delays="per_edge_long", nsig=1e-3)
    nz = noise_for(cfg, 300, 3, False, 4)
    eng, _, _, _ = compare(cfg, 3, SweepParam(-1, 0), [0.0, 0.1, 0.2], 300, semantics=HB_SEM_DELAY_RING, noise=nz)
    assert eng.last_kernel_time()[2] == PIPE_KIND


def test_wide_form_eight_producer_lanes():
    from hyburn_gb300 import inputs
    cfg, meta = inputs.batched_sweep(n_steps=900, n_points=16)
    nz = inputs.standard_normal((900, 148), 6)
    eng, _, _, _ = compare(cfg, 16, SweepParam(-1, 0), meta["values"], 900, semantics=HB_SEM_DELAY_RING, noise=nz,
                           run_flags=HB_RUN_PIPE_WIDE | HB_RUN_PIPE_LANES(8))
    assert eng.last_kernel_time()[2] == PIPE_KIND


@pytest.mark.parametrize("integrator", ["heun", "heun_stochastic"])
def test_straight_consumer_two_coupling_variables(integrator):
    cfg = single_model("MontbrioPazoRoxin", 30, integrator, "Linear", (0.4, 0.01), weights="csr",
                       delays="per_edge_long", nsig=1e-4, dt=0.05)
    nz = noise_for(cfg, 400, 3, False, 2) if "stochastic" in integrator else None
    eng, _, _, _ = compare(cfg, 3, SweepParam(0, NATIVE_SWEEP["MontbrioPazoRoxin"]),
                           sweep_values("MontbrioPazoRoxin", 3), 400, semantics=HB_SEM_DELAY_RING, noise=nz, traj=False)
    assert eng.last_kernel_time()[2] == PIPE_KIND


@pytest.mark.parametrize("model,integrator,n_cv", [("JansenRit", "heun", 1), ("JansenRit", "heun_stochastic", 1),
                                                   ("MontbrioPazoRoxin", "heun", 2)])
def test_straight_consumer_sigmoidal(model, integrator, n_cv):
    """Sigmoidal coupling through the straight-line consumer, with and without a trajectory, and a
    coupling-parameter sweep (per-point coupling rows)."""
    dt = 0.05 if model == "MontbrioPazoRoxin" else 0.1
    cfg = single_model(model, 24, integrator, "Sigmoidal", (0.0, 0.1, 0.0, 1.0, 0.05), weights="csr",
                       delays="per_edge_long", nsig=1e-4, dt=dt, seed=6)
    nz = noise_for(cfg, 300, 3, False, 3) if "stochastic" in integrator else None
    for traj in (False, True):
        eng, _, _, _ = compare(cfg, 3, SweepParam(0, NATIVE_SWEEP[model]), sweep_values(model, 3), 300,
                               semantics=HB_SEM_DELAY_RING, noise=nz, traj=traj)
        assert eng.last_kernel_time()[2] == PIPE_KIND
    eng, _, _, _ = compare(cfg, 3, SweepParam(-1, 3), [0.5, 1.0, 1.5], 300, semantics=HB_SEM_DELAY_RING, noise=nz)
    assert eng.last_kernel_time()[2] == PIPE_KIND
