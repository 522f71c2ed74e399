"""The plain per-operation comparator of bench.py (PlainTorchSweep) computes the same run as the
engine: final states agree within the FP32 differences of a regrouped coupling sum."""
import importlib.util
import os

import numpy as np
import pytest

from hyburn_gb300 import BatchHybridEngine, SweepParam, inputs
from hyburn_gb300._abi import HB_SEM_DELAY_RING

pytestmark = pytest.mark.gpu


def _bench():
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bench.py")
    spec = importlib.util.spec_from_file_location("bench_module", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_plain_comparator_matches_engine():
    bench = _bench()
    T = 500
    cfg, meta = inputs.batched_sweep(n_steps=T, n_points=8)
    noise = inputs.standard_normal((T, 148), 3)
    plain = bench.PlainTorchSweep(cfg, meta["values"], noise)
    x = plain.run(T).cpu().numpy().reshape(-1)
    eng = BatchHybridEngine.from_config(cfg, 8, semantics=HB_SEM_DELAY_RING)
    ref = eng.run_sweep(SweepParam(-1, 0), meta["values"], T, noise=noise).final_states[0]
    np.testing.assert_allclose(x, ref, rtol=1e-4, atol=1e-5)
