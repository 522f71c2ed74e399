"""Autotuner host logic on CPU (fake timings) and on the GPU (the chosen form matches the oracle)."""
import pytest

from hyburn_gb300 import SweepParam, autotune
from hyburn_gb300._abi import HB_RUN_STREAM, HB_SEM_DELAY_RING
from hyburn_gb300.config import Unsupported

from cases import single_model


def test_tune_picks_the_fastest_candidate_and_caches_it(tune_cache):
    cfg = single_model("Generic2dOscillator", 24, "heun", "Linear", (0.1,), weights="csr", delays="per_edge_long")
    names = [n for n, _ in autotune.candidates(cfg, HB_SEM_DELAY_RING)]
    assert names[0] == "engine" and any("pipeline" in n for n in names) and any("streamed" in n for n in names)
    cost = {flags: 10.0 + i for i, (_, flags) in enumerate(autotune.candidates(cfg, HB_SEM_DELAY_RING))}
    target = dict(autotune.candidates(cfg, HB_SEM_DELAY_RING))["streamed history 2 node(s) per thread"]
    cost[target] = 1.0

    def fake(config, n_sweep, semantics, param, values, n_steps, flags, noise, repeats):
        if flags == dict(autotune.candidates(cfg, HB_SEM_DELAY_RING))["per-step lanes 8"]:
            raise Unsupported("not for this shape")
        return cost[flags]

    flags, times = autotune.tune(cfg, 3, SweepParam(0, 1), [0.0, 0.1, 0.2], HB_SEM_DELAY_RING, measure=fake)
    assert flags == target and flags & HB_RUN_STREAM
    assert "per-step lanes 8" not in times
    autotune._MEMO.clear()
    assert autotune.best_run_flags(cfg, 3, HB_SEM_DELAY_RING) == target  # read back from the file
    assert autotune.best_run_flags(cfg, 4, HB_SEM_DELAY_RING) is None    # another shape


@pytest.fixture
def tune_cache(tmp_path, monkeypatch):
    """A private tuning cache; the in-process memo is cleared before and after so no tuned choice
    leaks into other tests."""
    monkeypatch.setenv("HYBURN_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    autotune._MEMO.clear()
    yield tmp_path / "tune.json"
    autotune._MEMO.clear()


@pytest.mark.gpu
def test_tuned_flags_run_and_match_the_oracle(tune_cache):
    from test_parity_gpu import compare
    from hyburn_gb300 import inputs
    cfg, meta = inputs.batched_sweep(n_steps=600, n_points=16)
    flags, times = autotune.tune(cfg, 16, SweepParam(-1, 0), meta["values"], HB_SEM_DELAY_RING, probe_steps=400)
    assert len(times) >= 8 and all(t > 0 for t in times.values())
    nz = inputs.standard_normal((600, 148), 5)
    compare(cfg, 16, SweepParam(-1, 0), meta["values"], 600, semantics=HB_SEM_DELAY_RING, noise=nz, run_flags=flags)


@pytest.mark.gpu
def test_engine_uses_the_tuned_choice_by_default(tune_cache):
    """A cached choice (here made to pick the per-step kernel with two lanes, kind 2) is what a default
    run uses; tune="off" and an explicit kernel choice bypass it; tune="auto" tunes an untuned shape."""
    from hyburn_gb300 import BatchHybridEngine, inputs
    cfg, meta = inputs.batched_sweep(n_steps=300, n_points=5, nsig=0.0, integrator="heun")
    want = dict(autotune.candidates(cfg, HB_SEM_DELAY_RING))["per-step lanes 2"]

    def fake(config, n_sweep, semantics, param, values, n_steps, flags, noise, repeats):
        return 1.0 if flags == want else 2.0

    autotune.tune(cfg, 5, SweepParam(-1, 0), meta["values"], HB_SEM_DELAY_RING, measure=fake)
    eng = BatchHybridEngine.from_config(cfg, 5, semantics=HB_SEM_DELAY_RING)
    a = eng.run_sweep(SweepParam(-1, 0), meta["values"], 300)
    assert eng.tuned_flags == want and eng.last_kernel_time()[2] == 2
    off = BatchHybridEngine.from_config(cfg, 5, semantics=HB_SEM_DELAY_RING, tune="off")
    b = off.run_sweep(SweepParam(-1, 0), meta["values"], 300)
    assert off.tuned_flags is None and off.last_kernel_time()[2] == 3
    eng.reset()
    eng.run_sweep(SweepParam(-1, 0), meta["values"], 300, run_flags=HB_RUN_STREAM)
    assert eng.tuned_flags is None and eng.last_kernel_time()[2] == 4
    import numpy as np
    assert np.allclose(a.final_states[0], b.final_states[0], rtol=1e-5, atol=1e-6)
    # an untuned shape with tune="auto": measured on its first run, then cached
    cfg6, meta6 = inputs.batched_sweep(n_steps=300, n_points=6, nsig=0.0, integrator="heun")
    assert autotune.best_run_flags(cfg6, 6, HB_SEM_DELAY_RING) is None
    auto = BatchHybridEngine.from_config(cfg6, 6, semantics=HB_SEM_DELAY_RING, tune="auto")
    auto.run_sweep(SweepParam(-1, 0), meta6["values"], 300)
    assert auto.tuned_flags is not None and autotune.best_run_flags(cfg6, 6, HB_SEM_DELAY_RING) == auto.tuned_flags


def test_a_refused_cached_choice_falls_back_to_the_fixed_rules(monkeypatch):
    """The cache key does not see every run option: when the engine refuses the cached kernel form for a
    run (HB_ERR_UNSUPPORTED), the run is made again with the caller's flags; a refusal of a form the
    caller chose is raised. (Host logic only: the library entry point is a fake.)"""
    from hyburn_gb300 import BatchHybridEngine, _abi
    eng = BatchHybridEngine.__new__(BatchHybridEngine)
    eng.tune, eng.config, eng.n_sweep, eng.semantics, eng.tuned_flags = "cache", None, 4, 0, None

    class Lib:
        @staticmethod
        def hb_last_error():
            return b"refused"

    eng._lib = Lib()
    monkeypatch.setattr(autotune, "best_run_flags", lambda *a: HB_RUN_STREAM)
    seen = []

    def refuses_stream(f):
        seen.append(f)
        return _abi.HB_ERR_UNSUPPORTED if f & HB_RUN_STREAM else _abi.HB_OK

    assert eng._run_tuned(refuses_stream, _abi.HB_RUN_TRAJECTORY) == _abi.HB_RUN_TRAJECTORY
    assert seen == [HB_RUN_STREAM | _abi.HB_RUN_TRAJECTORY, _abi.HB_RUN_TRAJECTORY] and eng.tuned_flags is None
    seen.clear()
    with pytest.raises(Unsupported):
        eng._run_tuned(refuses_stream, HB_RUN_STREAM)  # the caller's own choice: no cache, no second call
    assert seen == [HB_RUN_STREAM]
    assert eng._run_tuned(lambda f: _abi.HB_OK, 0) == HB_RUN_STREAM and eng.tuned_flags == HB_RUN_STREAM
    eng.tune = "off"
    assert eng._run_tuned(lambda f: _abi.HB_OK, 0) == 0 and eng.tuned_flags is None
