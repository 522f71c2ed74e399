"""Measured choice of kernel form and lane counts for a network shape, cached on disk.

The engine picks its kernel by fixed rules (the warp-specialised pipeline when every delay is at
least 15 steps and the history fits shared memory, the streamed-history kernel when it does not,
the generic resident kernel otherwise) with fixed lane counts. `tune` instead runs each applicable
form for a short probe on a scratch engine built from the same configuration, keeps the fastest,
and caches the run flags under a key of the network's shape:
(model, nodes, edges, smallest and largest delay, sweep points, integrator, semantics, monitors).
Later runs of the same shape read the cache (`best_run_flags`): BatchHybridEngine does so by default
for every run that forces no kernel form (its `tune` option: "cache", "auto" to tune an untuned
shape on its first run, "off"), and GroupedSweep takes the tuned streamed-history form when its
members agree on one. Results are those of the chosen kernel form, which all agree with the CPU
oracle within the parity tolerance; only the time differs. A cached form that the engine refuses for a
particular run (one with options the key does not see, such as trajectories or per-node parameter
tables) gives way to the fixed rules for that run.

Cache file: $HYBURN_GB300_TUNE_CACHE, else ~/.cache/hyburn_gb300/tune.json.
"""
from __future__ import annotations

import json
import os
import statistics
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _abi
from .config import SimConfig, SimulationError
from .engine import BatchHybridEngine, SweepParam, noise_shape

_MEMO: Dict[str, int] = {}


def cache_path() -> str:
    p = os.environ.get("HYBURN_GB300_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "hyburn_gb300", "tune.json")


def shape_key(config: SimConfig, n_sweep: int, semantics: int) -> str:
    subs = config.network.subnetworks
    parts = [f"{s.model}x{s.nnodes}x{s.nmodes}" for s in subs]
    for p in config.network.projections:
        w = p.weights
        if isinstance(w, dict):
            nnz = len(w["data"])
        elif isinstance(w, (int, float)):
            nnz = -1
        else:
            nnz = int(np.count_nonzero(np.asarray(w)))
        d = list(p.delays) if p.delays else [0]
        parts.append(f"{p.src}>{p.tgt}:{p.coupling_fn}:nnz{nnz}:d{min(d)}-{max(d)}:n{len(d)}")
    mons = ",".join(m.monitor_type for m in config.monitors)
    return "|".join(parts) + f"|B{n_sweep}|{config.integrator}|sem{semantics}|{mons}"


def candidates(config: SimConfig, semantics: int) -> List[Tuple[str, int]]:
    """Run-flag sets worth measuring for this network (the engine's own choice is the first)."""
    out = [("engine", 0)]
    projs = config.network.projections
    single_sparse = (len(config.network.subnetworks) == 1 and len(projs) == 1 and
                     not isinstance(projs[0].weights, (int, float)))
    per_edge = bool(single_sparse and (semantics & _abi.HB_SEM_DELAY_RING) and projs[0].delays and
                    len(projs[0].delays) > 1)
    dmin = min(projs[0].delays) if per_edge else 0
    if single_sparse:
        for lanes in (1, 2, 4, 8):
            out.append((f"per-step lanes {lanes}", _abi.HB_RUN_NO_PIPE | _abi.HB_RUN_NO_STREAM | _abi.HB_RUN_LANES(lanes)))
        out.append(("two-phase", _abi.HB_RUN_TWO_PHASE | _abi.HB_RUN_NO_STREAM))
        if dmin >= 15:
            for pl in (1, 2, 4, 8):
                out.append((f"pipeline producer lanes {pl}", _abi.HB_RUN_NO_STREAM | _abi.HB_RUN_PIPE_LANES(pl)))
            for pl in (2, 4):
                out.append((f"pipeline (1024-thread form) producer lanes {pl}",
                            _abi.HB_RUN_NO_STREAM | _abi.HB_RUN_PIPE_WIDE | _abi.HB_RUN_PIPE_LANES(pl)))
            for npt in (1, 2, 4):
                out.append((f"streamed history {npt} node(s) per thread", _abi.HB_RUN_STREAM | _abi.HB_RUN_STREAM_NPT(npt)))
            # CTAs per point: a point's nodes split over a cluster (fewer points in flight, histories in L2)
            nodes = config.network.subnetworks[0].nnodes
            for c in (2, 3, 4, 5, 6, 8):
                if nodes >= 16 * c:
                    out.append((f"streamed history, {c} CTAs per point", _abi.HB_RUN_STREAM | _abi.HB_RUN_STREAM_CLUSTER(c)))
            # the warp gather's windows staged by the bulk-copy engine (the engine refuses it where the
            # warp gather does not apply; such candidates are skipped)
            out.append(("streamed history, bulk-staged windows", _abi.HB_RUN_STREAM | _abi.HB_RUN_STREAM_BULK))
        undelayed = not projs[0].delays or max(projs[0].delays) == 0
        if undelayed and projs[0].coupling_fn in ("Linear", "Sigmoidal", "ScaledLinear"):
            # 128 points per CTA: the coupling as a tensor-core matrix product
            out.append(("tensor-core dense coupling, 128 points per CTA", _abi.HB_RUN_DENSE_TC))
    else:
        for lanes in (1, 2, 4, 8):
            out.append((f"generic lanes {lanes}", _abi.HB_RUN_GENERIC | _abi.HB_RUN_LANES(lanes)))
    return out


def _measure(config: SimConfig, n_sweep: int, semantics: int, param: SweepParam, values, n_steps: int,
             run_flags: int, noise, repeats: int) -> float:
    eng = BatchHybridEngine.from_config(config, n_sweep, semantics=semantics, tune="off")
    try:
        eng.prepare(param, values, n_steps, noise=noise, run_flags=run_flags)
        eng.execute_prepared()
        times = []
        for _ in range(repeats):
            eng.execute_prepared()
            times.append(eng.last_kernel_time()[0])
        return statistics.median(times)
    finally:
        eng.close()


def _load() -> Dict[str, dict]:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(table: Dict[str, dict]) -> None:
    path = cache_path()
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tune(config: SimConfig, n_sweep: int, param: SweepParam, values: Sequence[float], semantics: int = 0,
         probe_steps: int = 2000, repeats: int = 3,
         measure: Optional[Callable[..., float]] = None) -> Tuple[int, Dict[str, float]]:
    """Measure every candidate on a probe of `probe_steps` steps; returns (best run flags, times in ms).
    Candidates the network cannot run (HB_ERR_UNSUPPORTED and the like) are skipped."""
    measure = measure or _measure
    # the pipelines take a slower start-up path for the first longest-delay steps: probe well past it
    longest = max((max(p.delays) for p in config.network.projections if p.delays), default=0)
    probe_steps = max(probe_steps, 3 * longest)
    noise = None
    if config.integrator.endswith("stochastic"):
        noise = np.random.default_rng(0).standard_normal(noise_shape(config, probe_steps, n_sweep, semantics),
                                                         dtype=np.float32)
    times: Dict[str, float] = {}
    best = None
    for name, flags in candidates(config, semantics):
        try:
            ms = measure(config, n_sweep, semantics, param, values, probe_steps, flags, noise, repeats)
        except SimulationError:
            continue
        times[name] = ms
        if best is None or ms < best[1]:
            best = (flags, ms)
    if best is None:
        raise SimulationError("no kernel form could run this network")
    key = shape_key(config, n_sweep, semantics)
    _MEMO[key] = best[0]
    table = _load()
    table[key] = {"run_flags": best[0], "times_ms": times, "probe_steps": probe_steps}
    _store(table)
    return best[0], times


def best_run_flags(config: SimConfig, n_sweep: int, semantics: int = 0) -> Optional[int]:
    """Cached run flags for this network shape, or None when it has not been tuned."""
    key = shape_key(config, n_sweep, semantics)
    if key in _MEMO:
        return _MEMO[key]
    entry = _load().get(key)
    if entry is None:
        return None
    _MEMO[key] = int(entry["run_flags"])
    return _MEMO[key]
