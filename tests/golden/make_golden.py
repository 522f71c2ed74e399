"""Golden input/output fixtures of the batched sweep, and the script that writes them.

Each fixture is one ``.npz`` file holding a whole run: the configuration (scalar fields as JSON,
connectivity, delays, initial states and per-node parameter rows as arrays), the sweep, the noise
draws, and the oracle's outputs (final states, temporal averages, BOLD) in FP32 and in the FP64
twin. Nothing has to be regenerated to use a fixture, so the CUDA engine can be held to it on a
machine where neither the oracle nor the input generators run the same way.

The cases are the workloads' own shapes, cut to a few hundred steps:

- ``bench_sweep_det``: the batched G2DO sweep (74 nodes, 20 % CSR, per-edge delays 37 to 667
  steps, the Linear coupling scale swept over 16 points), Heun, nsig 0, 900 steps;
- ``bench_sweep_stochastic``: the same network, 8 points, Heun-stochastic with the shared seeded
  draws, 200 steps;
- ``single_sim``: the single G2DO simulation (74 nodes, mean-field coupling), 3000 steps;
- ``kuramoto_1000n``: Kuramoto, 1000 nodes, 5 % CSR, delays up to 500 steps, per-node natural
  frequencies omega ~ N(0, 1), 3 coupling scales, BOLD on, 80 steps;
- ``meanfield_<model>_<integrator>``: each of the six models under Heun-stochastic and RK4, 20
  nodes, all-to-all scalar coupling, the model's native parameter swept over 4 points, 120 steps;
- ``refbench_3subnet_*``: the generic-engine workload of the reference's CUDA benchmark (a
  G2DO -> JansenRit -> WilsonCowan ring of 76 or 164 nodes per population, 1000 steps with the hybrid
  integrator), over 32 or 8 of its I values;
- ``refbench_single_*``: the single-model part of the same benchmark (76 uncoupled nodes, 1000 Euler
  steps) for G2DO, JansenRit, WilsonCowan and MPR, 16 points;
- ``example_*``: the reference's own example configurations (``examples/*.toml`` with their
  ``examples/init_*_74.npy`` initial states), loaded through this package's TOML reader, run for
  their full ``sim_length`` the way its batch-sweep command runs them (``hyburn run -c <config>
  --sweep <sweep>``, cli.rs:961-998): the G2DO and MPR sweep configurations over all 128 values of
  their sweep files, and the other single-population and multi-population examples over the first
  values of ``examples/sweep.toml`` or as one point. Their initial states are stored resolved, so the
  fixtures do not need the reference tree.

Short runs are compared element-wise (``bound`` "elementwise": rel/abs tolerances). The example runs
are 10 000 to 100 000 steps, where two FP32 roundings of the same run drift apart by more than rel
1e-5 in a few elements; they carry ``bound`` "fp32": the engine may be no farther from the FP32
oracle than twice the FP32 oracle's largest distance from the FP64 twin (stored per output as
``drift``), with the rel/abs tolerance as the floor.

The engine's semantics follow the reference's ``BatchHybridEngine::run_sweep``
(src/engine/batch_engine/engine.rs:477-842); the oracle restates it (oracle/hb_oracle.c).

Run ``python tests/golden/make_golden.py`` from the repository root to rewrite every fixture (the
``example_*`` cases read the reference tree, ``HYBURN_REFERENCE_TREE``, default /root/reference).
"""
from __future__ import annotations

import json
import os
import sys
from dataclasses import dataclass
from typing import Callable, Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
ROOT = os.path.dirname(TESTS)
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

from hyburn_gb300._abi import HB_SEM_DELAY_RING  # noqa: E402
from hyburn_gb300.config import (Memory, MonitorConfig, NetworkConfig, ProjectionConfig, SimConfig,  # noqa: E402
                                 SubnetworkConfig)
from hyburn_gb300.engine import SweepParam  # noqa: E402


@dataclass
class GoldenCase:
    """One run: what goes in, and what the oracle returned (``expected``)."""

    name: str
    cfg: SimConfig
    n_sweep: int
    param: SweepParam
    values: np.ndarray
    n_steps: int
    semantics: int
    noise: Optional[np.ndarray]
    rtol: float
    atol: float
    # True where the run has no transcendental function: the engine with the reference's summation
    # order (HB_RUN_EXACT_SUMS) must then reproduce the FP32 outputs bit for bit
    bitwise: bool
    # "elementwise" (rtol/atol per element) or "fp32" (within twice the FP32 oracle's own distance
    # from the FP64 twin, largest absolute difference per output)
    bound: str
    # largest |FP32 - FP64| of the oracle per output (final_i, tavg_i, bold_m)
    drift: Dict[str, float]
    source: str
    expected: Dict[str, np.ndarray]


# ---------------------------------------------------------------------------------------------
# configuration <-> arrays
# ---------------------------------------------------------------------------------------------

def _compact(a) -> np.ndarray:
    """float32 where that holds every value exactly, float64 otherwise."""
    a = np.asarray(a, np.float64)
    f = a.astype(np.float32)
    return f if np.array_equal(f.astype(np.float64), a) else a


def _index(a) -> np.ndarray:
    """Non-negative integers in uint16 where they fit, uint32 otherwise."""
    a = np.asarray(a, np.int64)
    if a.size and (a.min() < 0 or a.max() >= 2 ** 32):
        raise ValueError("index array out of the uint32 range")
    return a.astype(np.uint16 if not a.size or a.max() < 2 ** 16 else np.uint32)


def pack_config(cfg: SimConfig):
    """Split a SimConfig into a JSON description and the arrays it refers to by key."""
    arrays: Dict[str, np.ndarray] = {}
    subs = []
    for i, s in enumerate(cfg.network.subnetworks):
        d = {"model": s.model, "nnodes": s.nnodes, "nmodes": s.nmodes, "params": [float(v) for v in s.params]}
        init = s.initial_state
        if isinstance(init, Memory):
            arrays[f"sub{i}_x0"] = _compact(init.data)
            d["initial_state"] = {"memory_shape": list(init.shape), "key": f"sub{i}_x0"}
        elif isinstance(init, str):
            d["initial_state"] = init
        else:
            arrays[f"sub{i}_x0"] = _compact(init)
            d["initial_state"] = {"key": f"sub{i}_x0"}
        if s.node_params is not None:
            arrays[f"sub{i}_node_params"] = np.asarray(s.node_params)
            d["node_params"] = f"sub{i}_node_params"
        subs.append(d)
    projs = []
    for i, p in enumerate(cfg.network.projections):
        d = {"src": p.src, "tgt": p.tgt, "conn_type": p.conn_type, "coupling_fn": p.coupling_fn,
             "coupling_params": [float(v) for v in p.coupling_params], "cvar_map": p.cvar_map}
        w = p.weights
        if isinstance(w, dict):
            arrays[f"proj{i}_data"] = _compact(w["data"])
            arrays[f"proj{i}_indices"] = _index(w["indices"])
            arrays[f"proj{i}_indptr"] = _index(w["indptr"])
            d["weights"] = "csr"
        elif isinstance(w, (int, float)):
            d["weights"] = float(w)
        else:
            arrays[f"proj{i}_dense"] = _compact(w)
            d["weights"] = "dense"
        if p.delays:
            arrays[f"proj{i}_delays"] = _index(p.delays)
        if p.tract_lengths:
            arrays[f"proj{i}_lengths"] = _compact(p.tract_lengths)
        projs.append(d)
    desc = {"sim_length": cfg.sim_length, "dt": cfg.dt, "integrator": cfg.integrator, "noise_mode": cfg.noise_mode,
            "nsig": cfg.nsig if isinstance(cfg.nsig, (int, float)) else [float(v) for v in cfg.nsig],
            "speed": cfg.speed, "backend": cfg.backend, "stimuli": cfg.stimuli,
            "monitors": [vars(m) for m in cfg.monitors], "subnetworks": subs, "projections": projs}
    return json.dumps(desc), arrays


def unpack_config(text: str, arrays) -> SimConfig:
    d = json.loads(text)
    subs = []
    for s in d["subnetworks"]:
        init = s["initial_state"]
        if isinstance(init, dict):
            data = np.asarray(arrays[init["key"]], np.float64).tolist()
            init = Memory(data, list(init["memory_shape"])) if "memory_shape" in init else data
        sub = SubnetworkConfig(s["model"], int(s["nnodes"]), init, list(s["params"]), nmodes=int(s["nmodes"]))
        if "node_params" in s:
            sub.node_params = np.asarray(arrays[s["node_params"]])
        subs.append(sub)
    projs = []
    for i, p in enumerate(d["projections"]):
        w = p["weights"]
        if w == "csr":
            w = {"data": np.asarray(arrays[f"proj{i}_data"], np.float64).tolist(),
                 "indices": arrays[f"proj{i}_indices"].astype(np.int64).tolist(),
                 "indptr": arrays[f"proj{i}_indptr"].astype(np.int64).tolist()}
        elif w == "dense":
            w = np.asarray(arrays[f"proj{i}_dense"], np.float64).tolist()
        delays = arrays[f"proj{i}_delays"].astype(np.int64).tolist() if f"proj{i}_delays" in arrays else []
        lengths = np.asarray(arrays[f"proj{i}_lengths"], np.float64).tolist() if f"proj{i}_lengths" in arrays else []
        projs.append(ProjectionConfig(int(p["src"]), int(p["tgt"]), w, conn_type=p["conn_type"], delays=delays,
                                      tract_lengths=lengths, coupling_fn=p["coupling_fn"],
                                      coupling_params=list(p["coupling_params"]), cvar_map=p["cvar_map"]))
    return SimConfig(sim_length=d["sim_length"], dt=d["dt"], network=NetworkConfig(subs, projs),
                     integrator=d["integrator"], noise_mode=d["noise_mode"],
                     monitors=[MonitorConfig(**m) for m in d["monitors"]], stimuli=d["stimuli"], nsig=d["nsig"],
                     speed=d["speed"], backend=d["backend"])


def difference(key: str, a, b, cfg: SimConfig) -> np.ndarray:
    """|a - b| element-wise in float64; Kuramoto final phases (kept in [0, 2 pi)) on the circle, where a
    phase that wraps at a different step on the two sides is still the same phase."""
    d = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    kind, _, idx = key.partition("_")
    if kind == "final" and cfg.network.subnetworks[int(idx)].model == "Kuramoto":
        d = np.minimum(d, np.abs(2.0 * np.pi - d))
    return d


def path_of(name: str) -> str:
    return os.path.join(HERE, f"{name}.npz")


def load_case(name: str) -> GoldenCase:
    with np.load(path_of(name), allow_pickle=False) as z:
        arrays = {k: z[k] for k in z.files}
    meta = json.loads(str(arrays.pop("meta")))
    cfg = unpack_config(str(arrays.pop("config")), arrays)
    expected = {k[4:]: v for k, v in arrays.items() if k.startswith("out_")}
    noise = arrays.get("noise")
    return GoldenCase(name=name, cfg=cfg, n_sweep=meta["n_sweep"], param=SweepParam(*meta["param"]),
                      values=arrays["values"], n_steps=meta["n_steps"], semantics=meta["semantics"], noise=noise,
                      rtol=meta["rtol"], atol=meta["atol"], bitwise=meta["bitwise"], bound=meta["bound"],
                      drift=meta["drift"], source=meta["source"], expected=expected)


# ---------------------------------------------------------------------------------------------
# the cases
# ---------------------------------------------------------------------------------------------

def _bench_det():
    from hyburn_gb300 import inputs
    cfg, meta = inputs.batched_sweep(n_steps=900, n_points=16, nsig=0.0, integrator="heun")
    return dict(cfg=cfg, n_sweep=16, param=SweepParam(-1, 0), values=meta["values"], n_steps=900,
                semantics=HB_SEM_DELAY_RING, noise=None, rtol=1e-5, atol=1e-6, bitwise=True)


def _bench_stoch():
    from hyburn_gb300 import inputs
    cfg, meta = inputs.batched_sweep(n_steps=200, n_points=8)
    return dict(cfg=cfg, n_sweep=8, param=SweepParam(-1, 0), values=meta["values"], n_steps=200,
                semantics=HB_SEM_DELAY_RING, noise=inputs.standard_normal((200, 148), 2), rtol=1e-5, atol=1e-6,
                bitwise=True)


def _single():
    from hyburn_gb300 import inputs
    cfg, _ = inputs.plain_single_sim(3000)
    return dict(cfg=cfg, n_sweep=1, param=SweepParam(0, 1), values=[cfg.network.subnetworks[0].params[1]],
                n_steps=3000, semantics=0, noise=None, rtol=1e-5, atol=1e-6, bitwise=False)


def _kuramoto():
    from hyburn_gb300 import inputs
    cfg, _ = inputs.kuramoto_scale(n=1000, n_points=3, n_steps=80, bold=True)
    # sin/cos of 1000-node phase sums: the C library and CUDA differ by an ulp or two per call
    return dict(cfg=cfg, n_sweep=3, param=SweepParam(-1, 0), values=[0.0, 1.0, 2.0], n_steps=80,
                semantics=HB_SEM_DELAY_RING, noise=None, rtol=2e-5, atol=1e-6, bitwise=False)


def _meanfield(model: str, integrator: str):
    def make():
        from cases import NATIVE_SWEEP, noise_for, single_model, sweep_values
        cfg = single_model(model, 20, integrator, "Linear", (0.05,), nsig=1e-4)
        nz = noise_for(cfg, 120, 4, False, 3) if "stochastic" in integrator else None
        return dict(cfg=cfg, n_sweep=4, param=SweepParam(0, NATIVE_SWEEP[model]), values=sweep_values(model, 4),
                    n_steps=120, semantics=0, noise=nz, rtol=1e-5, atol=1e-6, bitwise=False)
    return make


MODELS = ["Generic2dOscillator", "MontbrioPazoRoxin", "ReducedWongWang", "Kuramoto", "JansenRit", "WilsonCowan"]
SHORT = {"Generic2dOscillator": "g2do", "MontbrioPazoRoxin": "mpr", "ReducedWongWang": "rww", "Kuramoto": "kuramoto",
         "JansenRit": "jr", "WilsonCowan": "wc"}

CASES: Dict[str, Callable[[], dict]] = {
    "bench_sweep_det": _bench_det,
    "bench_sweep_stochastic": _bench_stoch,
    "single_sim": _single,
    "kuramoto_1000n": _kuramoto,
}
for _m in MODELS:
    for _i in ("heun_stochastic", "rk4"):
        CASES[f"meanfield_{SHORT[_m]}_{_i}"] = _meanfield(_m, _i)


REFERENCE_TREE = os.environ.get("HYBURN_REFERENCE_TREE", "/root/reference")


def _example(config: str, sweep: Optional[str], n_points: int):
    """One of the reference's example configurations, run for its full sim_length: over the first
    n_points values of its sweep file, or (sweep None) as one point whose swept value is the model's
    own native parameter."""
    def make():
        from cases import NATIVE_SWEEP
        from hyburn_gb300.config import SweepConfig, parse_sweep_param, resolve_initial_state
        cwd = os.getcwd()
        os.chdir(REFERENCE_TREE)  # the examples name their initial-state files relative to the tree
        try:
            cfg = SimConfig.from_file(os.path.join("examples", config))
            for s in cfg.network.subnetworks:
                s.initial_state = np.asarray(resolve_initial_state(s), np.float64).tolist()
            if sweep:
                sw = SweepConfig.from_file(os.path.join("examples", sweep))
                param = SweepParam(*parse_sweep_param(sw.parameter_name, cfg))
                values = sw.generate_values()[:n_points]
            else:
                s0 = cfg.network.subnetworks[0]
                param = SweepParam(0, NATIVE_SWEEP[s0.model])
                values = [s0.params[param.param_idx]]
        finally:
            os.chdir(cwd)
        n_steps = int(round(cfg.sim_length / cfg.dt))
        src = f"examples/{config}" + (f" with examples/{sweep}" if sweep else "")
        return dict(cfg=cfg, n_sweep=len(values), param=param, values=values, n_steps=n_steps, semantics=0,
                    noise=None, rtol=1e-5, atol=1e-6, bitwise=False, bound="fp32", source=src)
    return make


def _refbench(nnodes: int, n_points: int):
    """The generic-engine workload of the reference's CUDA benchmark, the one its published 3-population
    times are for (examples/bench/hyburn_bench_generic_cuda.rs:21-56, 116-131): a G2DO -> JansenRit ->
    WilsonCowan ring, each population `nnodes` nodes from a zero state with its default parameters,
    all-to-all Scalar weights 0.01 with Linear(1.0) coupling and no delay, Heun at dt 0.1 for 1000 steps
    with the hybrid integrator (Heun for G2DO, Euler for the others; HB_SEM_HYBRID_INTEGRATOR), G2DO's I
    swept as -0.5 + i / (n - 1) in f32 (the benchmark runs 256 to 1024 points; fewer here)."""
    def make():
        from hyburn_gb300._abi import HB_SEM_HYBRID_INTEGRATOR
        from hyburn_gb300.config import DEFAULT_PARAMS
        n_steps, dt, w = 1000, 0.1, 0.01
        subs = [SubnetworkConfig(m, nnodes, [0.0] * (nv * nnodes), list(DEFAULT_PARAMS[m]))
                for m, nv in (("Generic2dOscillator", 2), ("JansenRit", 6), ("WilsonCowan", 2))]
        projs = [ProjectionConfig(s, t, w, coupling_fn="Linear", coupling_params=[1.0], delays=[0])
                 for s, t in ((0, 1), (1, 2), (2, 0))]
        cfg = SimConfig(sim_length=n_steps * dt, dt=dt, integrator="heun", network=NetworkConfig(subs, projs))
        f = np.float32
        values = [float(f(-0.5) + f(i) / f(max(n_points - 1, 1))) for i in range(n_points)]
        return dict(cfg=cfg, n_sweep=n_points, param=SweepParam(0, 1), values=values, n_steps=n_steps,
                    semantics=HB_SEM_HYBRID_INTEGRATOR, noise=None, rtol=1e-5, atol=1e-6, bitwise=False, bound="fp32",
                    source="examples/bench/hyburn_bench_generic_cuda.rs (generic BatchHybridEngine, hybrid integrator)")
    return make


CASES["refbench_3subnet_76n"] = _refbench(76, 32)
CASES["refbench_3subnet_164n"] = _refbench(164, 8)


def _refbench_single(model: str, nvar: int, n_points: int):
    """The single-model part of the reference's CUDA benchmark (examples/bench/hyburn_bench_generic_cuda.rs:
    60-107): 76 uncoupled nodes (no projection) from a zero state, default parameters (MPR: [1, 1, -5, 15,
    0, 1, 0]), Euler at dt 0.1 for 1000 steps, parameter 1 (MPR: 2) swept as -0.5 + i / (n - 1) in f32;
    only G2DO's index is batch-native, so the other models' points all run the same network."""
    def make():
        from hyburn_gb300.config import DEFAULT_PARAMS
        params = [1.0, 1.0, -5.0, 15.0, 0.0, 1.0, 0.0] if model == "MontbrioPazoRoxin" else list(DEFAULT_PARAMS[model])
        cfg = SimConfig(sim_length=10.0, dt=0.1, integrator="euler",
                        network=NetworkConfig([SubnetworkConfig(model, 76, [0.0] * (nvar * 76), params)], []))
        f = np.float32
        values = [float(f(-0.5) + f(i) / f(max(n_points - 1, 1))) for i in range(n_points)]
        return dict(cfg=cfg, n_sweep=n_points, param=SweepParam(0, 2 if model == "MontbrioPazoRoxin" else 1),
                    values=values, n_steps=1000, semantics=0, noise=None, rtol=1e-5, atol=1e-6, bitwise=False,
                    bound="fp32", source="examples/bench/hyburn_bench_generic_cuda.rs (single-model loop)")
    return make


for _short, (_m, _nv) in {"g2do": ("Generic2dOscillator", 2), "jr": ("JansenRit", 6), "wc": ("WilsonCowan", 2),
                          "mpr": ("MontbrioPazoRoxin", 2)}.items():
    CASES[f"refbench_single_{_short}"] = _refbench_single(_m, _nv, 16)

EXAMPLES = {
    "example_g2do_sweep": ("g2do_sweep.toml", "sweep.toml", 128),
    "example_mpr_sweep": ("mpr_sweep.toml", "sweep_mpr.toml", 128),
    "example_demo_sweep": ("demo.toml", "sweep.toml", 16),
    "example_g2do_bold": ("g2do_bold.toml", "sweep.toml", 8),
    "example_two_population_coupled": ("two_population_coupled.toml", "sweep.toml", 8),
    "example_whole_brain_multi_model": ("whole_brain_multi_model.toml", "sweep.toml", 8),
    "example_wilson_cowan_ring": ("wilson_cowan_ring.toml", None, 1),
    "example_g2do_simple": ("g2do_simple.toml", None, 1),
    "example_jansen_rit_evoked": ("jansen_rit_evoked.toml", None, 1),
}
for _n, (_c, _s, _p) in EXAMPLES.items():
    CASES[_n] = _example(_c, _s, _p)


def build_case(name: str) -> dict:
    """The case's inputs from the seeded generators (used to write fixtures, and by a CPU test that the
    generators still give the stored inputs)."""
    return CASES[name]()


def write_case(name: str) -> None:
    from oracle.hb_oracle import OracleEngine
    c = build_case(name)
    vals = np.asarray(c["values"], np.float32)
    text, arrays = pack_config(c["cfg"])
    bound = c.get("bound", "elementwise")
    runs = {}
    for prec in ("f32", "f64"):
        r = OracleEngine.from_config(c["cfg"], c["n_sweep"], semantics=c["semantics"], precision=prec,
                                     n_threads=os.cpu_count()).run_sweep(c["param"], vals, c["n_steps"],
                                                                         noise=c["noise"])
        # the FP64 twin integrates in double and returns its outputs rounded to float
        got = {}
        for i in range(len(r.final_states)):
            got[f"final_{i}"] = np.asarray(r.final_states[i], np.float32)
            got[f"tavg_{i}"] = np.asarray(r.tavg[i], np.float32)
        for m in range(len(r.bold or [])):
            got[f"bold_{m}"] = np.asarray(r.bold[m], np.float32)
        runs[prec] = got
    drift = {k: float(np.max(difference(k, v, runs["f64"][k], c["cfg"])) if v.size else 0.0)
             for k, v in runs["f32"].items()}
    out = {f"out_{k}": v for k, v in runs["f32"].items()}
    if bound == "elementwise":  # the long runs keep only the FP64 twin's drift, not its outputs
        out.update({f"out_{k.replace('_', '64_', 1)}": v for k, v in runs["f64"].items()})
    meta = {"n_sweep": c["n_sweep"], "param": [c["param"].sub_idx, c["param"].param_idx], "n_steps": c["n_steps"],
            "semantics": c["semantics"], "rtol": c["rtol"], "atol": c["atol"], "bitwise": c["bitwise"],
            "bound": bound, "drift": drift, "source": c.get("source", "seeded generators (hyburn_gb300.inputs, "
                                                               "tests/cases.py)")}
    extra = {} if c["noise"] is None else {"noise": np.asarray(c["noise"], np.float32)}
    np.savez_compressed(path_of(name), meta=np.asarray(json.dumps(meta)), config=np.asarray(text), values=vals,
                        **arrays, **extra, **out)


if __name__ == "__main__":
    for n in (sys.argv[1:] or list(CASES)):
        write_case(n)
        print(f"{n}: {os.path.getsize(path_of(n)) / 1024:.1f} KiB")
