"""Failure detection on the device, exercised without faulting the GPU (src/error.rs:6-25 kinds).

- Non-finite states: a NaN planted in the initial state on the host propagates through the run;
  with HB_RUN_CHECK_FINITE every kernel form records it and the run fails with HB_ERR_NONFINITE
  (NonFinite), without the flag it returns normally. The engine stays usable afterwards.
- Bounded waits: with HB_RUN_TEST_UNSET_WAIT the pipeline kernel waits once on an mbarrier phase that
  nothing completes; the wait gives up after its poll limit, the kernel finishes its loop, the run
  returns HB_ERR_TIMEOUT (DeviceTimeout) and the CUDA context stays usable: the next run of the same
  engine matches a run that never timed out.
"""
import numpy as np
import pytest

from hyburn_gb300 import BatchHybridEngine, DeviceTimeout, NonFinite, SweepParam, inputs
from hyburn_gb300._abi import (HB_RUN_CHECK_FINITE, HB_RUN_GENERIC, HB_RUN_NO_PIPE, HB_RUN_STREAM,
                               HB_RUN_TEST_UNSET_WAIT, HB_SEM_DELAY_RING)

from cases import single_model

pytestmark = pytest.mark.gpu

# kernel forms of the engine (hb_engine_last_kernel_time kind): generic 1, specialised 2, pipeline 3,
# streamed history 4, one warp per point 7
FORMS = [("pipeline", 0, 3), ("streamed", HB_RUN_STREAM, 4), ("specialised", HB_RUN_NO_PIPE, 2), ("generic", HB_RUN_GENERIC, 1)]


def _sweep_with_nan(node=5):
    cfg, meta = inputs.batched_sweep(n_steps=200, n_points=4, nsig=0.0, integrator="heun")
    x0 = list(cfg.network.subnetworks[0].initial_state)
    x0[2 * node] = float("nan")
    cfg.network.subnetworks[0].initial_state = x0
    return cfg, meta


@pytest.mark.parametrize("form,flags,kind", FORMS)
def test_nonfinite_state_is_reported(form, flags, kind):
    cfg, meta = _sweep_with_nan()
    eng = BatchHybridEngine.from_config(cfg, 4, semantics=HB_SEM_DELAY_RING)
    with pytest.raises(NonFinite):
        eng.run_sweep(SweepParam(-1, 0), meta["values"], 200, run_flags=flags | HB_RUN_CHECK_FINITE)
    assert eng.last_kernel_time()[2] == kind
    eng.reset()
    r = eng.run_sweep(SweepParam(-1, 0), meta["values"], 200, run_flags=flags)  # unchecked: returns the NaNs
    assert np.isnan(r.final_states[0]).any()


def test_nonfinite_state_is_reported_one_warp_per_point():
    cfg = single_model("Generic2dOscillator", 40, "heun", "Linear", (0.05,))
    x0 = list(cfg.network.subnetworks[0].initial_state)
    x0[7] = float("inf")
    cfg.network.subnetworks[0].initial_state = x0
    eng = BatchHybridEngine.from_config(cfg, 3)
    with pytest.raises(NonFinite):
        eng.run_sweep(SweepParam(0, 1), [0.0, 0.1, 0.2], 100, run_flags=HB_RUN_CHECK_FINITE)
    assert eng.last_kernel_time()[2] == 7


def test_finite_run_passes_the_check():
    cfg, meta = inputs.batched_sweep(n_steps=200, n_points=4, nsig=0.0, integrator="heun")
    eng = BatchHybridEngine.from_config(cfg, 4, semantics=HB_SEM_DELAY_RING)
    r = eng.run_sweep(SweepParam(-1, 0), meta["values"], 200, run_flags=HB_RUN_CHECK_FINITE)
    assert np.isfinite(r.final_states[0]).all()


@pytest.mark.parametrize("stochastic", [False, True])
def test_bounded_wait_gives_up_and_reports_timeout(stochastic):
    n_steps = 300
    cfg, meta = inputs.batched_sweep(n_steps=n_steps, n_points=4, nsig=1e-3 if stochastic else 0.0,
                                     integrator="heun_stochastic" if stochastic else "heun")
    noise = inputs.standard_normal((n_steps, 148), 3) if stochastic else None
    eng = BatchHybridEngine.from_config(cfg, 4, semantics=HB_SEM_DELAY_RING)
    with pytest.raises(DeviceTimeout):
        eng.run_sweep(SweepParam(-1, 0), meta["values"], n_steps, noise=noise, run_flags=HB_RUN_TEST_UNSET_WAIT)
    assert eng.last_kernel_time()[2] == 3
    eng.reset()
    after = eng.run_sweep(SweepParam(-1, 0), meta["values"], n_steps, noise=noise)
    fresh = BatchHybridEngine.from_config(cfg, 4, semantics=HB_SEM_DELAY_RING).run_sweep(
        SweepParam(-1, 0), meta["values"], n_steps, noise=noise)
    assert np.array_equal(after.final_states[0], fresh.final_states[0])
    assert np.array_equal(after.tavg[0], fresh.tavg[0])
