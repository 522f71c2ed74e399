"""One-warp-per-point kernel (Scalar coupling onto itself without delay): parity with the oracle for
the plain single simulation and for sweeps, in mean-field and diagonal form."""
import pytest

from hyburn_gb300 import SweepParam
from hyburn_gb300._abi import HB_SEM_NOISE_PER_POINT, HB_SEM_SCALAR_DIAGONAL

from cases import NATIVE_SWEEP, noise_for, single_model, sweep_values
from test_parity_gpu import compare

pytestmark = pytest.mark.gpu
SINGLE_KIND = 7


def test_plain_single_simulation():
    from hyburn_gb300 import inputs
    cfg, meta = inputs.plain_single_sim(3000)
    eng, _, _, _ = compare(cfg, 1, SweepParam(0, 1), [cfg.network.subnetworks[0].params[1]], 3000, traj=False)
    assert eng.last_kernel_time()[2] == SINGLE_KIND


@pytest.mark.parametrize("model,n", [("Generic2dOscillator", 74), ("JansenRit", 128), ("MontbrioPazoRoxin", 33),
                                     ("Kuramoto", 100), ("WilsonCowan", 64), ("ReducedWongWang", 5)])
@pytest.mark.parametrize("semantics", [0, HB_SEM_SCALAR_DIAGONAL, HB_SEM_NOISE_PER_POINT])
def test_sweeps_one_warp_per_point(model, n, semantics):
    integ = "heun_stochastic" if semantics == HB_SEM_NOISE_PER_POINT else "rk4"
    cfg = single_model(model, n, integ, "Linear", (0.05, 0.01), nsig=1e-4, dt=0.05)
    nz = noise_for(cfg, 400, 40, semantics == HB_SEM_NOISE_PER_POINT, 8) if "stochastic" in integ else None
    eng, _, _, _ = compare(cfg, 40, SweepParam(0, NATIVE_SWEEP[model]), sweep_values(model, 40), 400,
                           semantics=semantics, noise=nz)
    assert eng.last_kernel_time()[2] == SINGLE_KIND
