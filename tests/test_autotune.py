"""Autotuner host logic on CPU (fake timings) and on the GPU (the chosen form matches the oracle)."""
import pytest

from hyburn_gb300 import SweepParam, autotune
from hyburn_gb300._abi import HB_RUN_STREAM, HB_SEM_DELAY_RING
from hyburn_gb300.config import Unsupported

from cases import single_model


def test_tune_picks_the_fastest_candidate_and_caches_it(tmp_path, monkeypatch):
    monkeypatch.setenv("HYBURN_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    autotune._MEMO.clear()
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


@pytest.mark.gpu
def test_tuned_flags_run_and_match_the_oracle(tmp_path, monkeypatch):
    from test_parity_gpu import compare
    from hyburn_gb300 import inputs
    monkeypatch.setenv("HYBURN_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    autotune._MEMO.clear()
    cfg, meta = inputs.batched_sweep(n_steps=600, n_points=16)
    flags, times = autotune.tune(cfg, 16, SweepParam(-1, 0), meta["values"], HB_SEM_DELAY_RING, probe_steps=400)
    assert len(times) >= 8 and all(t > 0 for t in times.values())
    nz = inputs.standard_normal((600, 148), 5)
    compare(cfg, 16, SweepParam(-1, 0), meta["values"], 600, semantics=HB_SEM_DELAY_RING, noise=nz, run_flags=flags)
