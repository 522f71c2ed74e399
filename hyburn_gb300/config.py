"""TOML configuration surface, mirroring hyburn's ``src/config.rs`` (SimConfig and friends).

Field names, defaults and validation messages follow the reference so that an existing
``hyburn run -c cfg.toml --sweep sweep.toml`` configuration loads unchanged.
"""
from __future__ import annotations

import math
import tomllib
from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional, Sequence, Union

import numpy as np


class SimulationError(Exception):
    """src/error.rs:6-25 (SimulationError)."""


class InvalidConfig(SimulationError):
    pass


class InvalidState(SimulationError):
    pass


class BackendError(SimulationError):
    pass


class IOError_(SimulationError):
    pass


class NonFinite(SimulationError):
    pass


class DeviceTimeout(BackendError):
    """A bounded device-side wait gave up (HB_ERR_TIMEOUT)."""


class Unsupported(SimulationError):
    pass


# MODEL_REGISTRY (src/config.rs:43-72): name -> (nvar, ncvar, nparams)
MODEL_REGISTRY = {
    "Generic2dOscillator": (2, 1, 12),
    "MontbrioPazoRoxin": (2, 2, 7),
    "ReducedWongWang": (1, 1, 8),
    "Kuramoto": (1, 1, 1),
    "JansenRit": (6, 1, 13),
    "WilsonCowan": (2, 1, 22),
    "Linear": (1, 1, 1),
    "SupHopf": (2, 2, 2),
    "Hopfield": (2, 2, 3),
    "CoombesByrne2D": (2, 2, 4),
    "CoombesByrne": (4, 4, 5),
    "GastSchmidtKnoscheSD": (4, 4, 9),
    "GastSchmidtKnoscheSF": (4, 4, 9),
    "LarterBreakspear": (3, 1, 32),
    "Epileptor2D": (2, 1, 12),
    "Epileptor": (6, 2, 17),
    "ReducedWongWangExcInh": (2, 1, 19),
    "DecoBalancedExcInh": (2, 1, 20),
    "EpileptorCodim3": (3, 1, 13),
    "EpileptorCodim3SlowMod": (5, 1, 27),
    "EpileptorRestingState": (8, 3, 28),
    "ZetterbergJansen": (12, 1, 18),
    "ReducedSetFitzHughNagumo": (4, 2, 8),
    "ReducedSetHindmarshRose": (6, 2, 12),
    "DumontGutkin": (8, 4, 14),
    "ZerlautAdaptationFirstOrder": (5, 1, 50),
    "ZerlautAdaptationSecondOrder": (8, 1, 50),
    "KIonEx": (5, 1, 14),
}

# default parameters of the six hot-path models (src/model/*.rs *_default_params)
DEFAULT_PARAMS = {
    "Generic2dOscillator": [1.0, 0.0, -2.0, -10.0, 0.0, 0.02, 3.0, 1.0, 0.0, 1.0, 1.0, 1.0],
    "MontbrioPazoRoxin": [1.0, 1.0, -5.0, 15.0, 0.0, 1.0, 0.0],
    "ReducedWongWang": [0.270, 0.108, 154.0, 0.641, 100.0, 0.6, 0.2609, 0.33],
    "Kuramoto": [1.0],
    "JansenRit": [3.25, 22.0, 0.1, 0.05, 5.52, 0.0025, 0.56, 135.0, 1.0, 0.8, 0.25, 0.25, 0.22],
    "WilsonCowan": [12.0, 4.0, 13.0, 11.0, 10.0, 10.0, 1.2, 2.8, 1.0, 0.0, 1.0, 4.0, 1.0, 0.0,
                    1.0, 1.0, 1.0, 1.0, 0.0, 0.0, 1.0, 1.0],
}


def lookup_model(name: str):
    return MODEL_REGISTRY.get(name)


@dataclass
class Memory:
    """InitialStateConfig::Memory (config.rs:150-152)."""

    data: List[float]
    shape: List[int]


InitialState = Union[List[float], str, Memory]


@dataclass
class SubnetworkConfig:
    model: str
    nnodes: int
    initial_state: InitialState
    params: List[float]
    nmodes: int = 1
    # Extension of this engine (not in the reference's SubnetworkConfig): parameter rows per node,
    # [nnodes*nmodes, n_params] shared by all sweep points or [n_sweep, nnodes*nmodes, n_params];
    # they replace `params` node by node, and a swept model parameter still takes its sweep value.
    node_params: Optional[Any] = None


@dataclass
class ProjectionConfig:
    src: int
    tgt: int
    weights: Any  # float (Scalar) | list of rows (Dense) | {"data","indices","indptr"} (Csr)
    conn_type: str = "all_to_all"
    delays: List[int] = field(default_factory=list)
    tract_lengths: List[float] = field(default_factory=list)
    coupling_fn: str = "Linear"
    coupling_params: List[float] = field(default_factory=list)
    cvar_map: str = "0:0"


@dataclass
class NetworkConfig:
    subnetworks: List[SubnetworkConfig]
    projections: List[ProjectionConfig] = field(default_factory=list)


@dataclass
class MonitorConfig:
    monitor_type: str
    period: Optional[float] = None
    tr: Optional[float] = 2.0
    bold_period: Optional[int] = 10
    gain: Optional[List[List[float]]] = None
    gain_path: Optional[str] = None
    voi: Optional[List[int]] = None
    spatial_mask: Optional[List[float]] = None


@dataclass
class SimConfig:
    sim_length: float
    dt: float
    network: NetworkConfig
    integrator: str = "heun"
    noise_mode: str = "reproducible"
    monitors: List[MonitorConfig] = field(default_factory=list)
    stimuli: List[Dict[str, Any]] = field(default_factory=list)
    nsig: Union[float, List[float]] = 0.0
    speed: float = 3.0
    backend: str = "ndarray"

    # --- loading (config.rs:259-283) ---
    @staticmethod
    def from_toml_str(s: str) -> "SimConfig":
        try:
            raw = tomllib.loads(s)
        except tomllib.TOMLDecodeError as e:
            raise InvalidConfig(f"TOML parse error: {e}") from None
        return SimConfig.from_dict(raw)

    @staticmethod
    def from_file(path: str) -> "SimConfig":
        try:
            with open(path, "r") as f:
                text = f.read()
        except OSError as e:
            raise IOError_(str(e)) from None
        return SimConfig.from_toml_str(text)

    @staticmethod
    def from_dict(raw: Dict[str, Any]) -> "SimConfig":
        try:
            net = raw["network"]
            subs = []
            for s in net["subnetworks"]:
                init = s["initial_state"]
                if isinstance(init, list):
                    init = [float(v) for v in init]
                subs.append(SubnetworkConfig(model=s["model"], nnodes=int(s["nnodes"]),
                                             nmodes=int(s.get("nmodes", 1)), initial_state=init,
                                             params=[float(v) for v in s["params"]]))
            projs = []
            for p in net.get("projections", []):
                w = p["weights"]
                if isinstance(w, dict):
                    w = {"data": list(w["data"]), "indices": list(w["indices"]), "indptr": list(w["indptr"])}
                elif isinstance(w, (int, float)):
                    w = float(w)
                projs.append(ProjectionConfig(
                    src=int(p["src"]), tgt=int(p["tgt"]), weights=w,
                    conn_type=p.get("conn_type", "all_to_all"),
                    delays=[int(d) for d in p.get("delays", [])],
                    tract_lengths=[float(t) for t in p.get("tract_lengths", [])],
                    coupling_fn=p.get("coupling_fn", "Linear"),
                    coupling_params=[float(c) for c in p.get("coupling_params", [])],
                    cvar_map=p.get("cvar_map", "0:0")))
            mons = []
            for m in raw.get("monitors", []):
                mons.append(MonitorConfig(monitor_type=m["monitor_type"], period=m.get("period"),
                                          tr=m.get("tr", 2.0), bold_period=m.get("bold_period", 10),
                                          gain=m.get("gain"), gain_path=m.get("gain_path"),
                                          voi=m.get("voi"), spatial_mask=m.get("spatial_mask")))
            integ = raw.get("integrator", "heun")
            if integ not in ("heun", "euler", "euler_stochastic", "heun_stochastic", "rk4", "rk4_stochastic"):
                raise InvalidConfig(f"TOML parse error: unknown integrator kind: {integ}")
            # NoiseMode deserialises from these two names only (integrator.rs:57-63); this engine takes its
            # draws from the caller, so the mode names where they come from but changes no arithmetic
            noise_mode = raw.get("noise_mode", "reproducible")
            if noise_mode not in ("reproducible", "fast"):
                raise InvalidConfig(f"TOML parse error: unknown noise mode: {noise_mode}")
            return SimConfig(sim_length=float(raw["sim_length"]), dt=float(raw["dt"]),
                             network=NetworkConfig(subs, projs), integrator=integ,
                             noise_mode=noise_mode, monitors=mons,
                             stimuli=raw.get("stimuli", []), nsig=raw.get("nsig", 0.0),
                             speed=float(raw.get("speed", 3.0)), backend=raw.get("backend", "ndarray"))
        except KeyError as e:
            raise InvalidConfig(f"TOML parse error: missing field {e}") from None

    # --- NsigConfig::to_vec (config.rs:16-24) ---
    def nsig_vec(self, nvar: int) -> List[float]:
        if isinstance(self.nsig, (int, float)):
            return [float(self.nsig)] * nvar
        v = [float(x) for x in self.nsig]
        if len(v) != nvar:
            raise InvalidConfig(f"nsig per-variable length must match nvar (got {len(v)}, expected {nvar})")
        return v

    # --- SimConfig::validate (config.rs:286-429) ---
    def validate(self) -> None:
        if self.dt <= 0.0:
            raise InvalidConfig("dt must be positive")
        if self.sim_length <= 0.0:
            raise InvalidConfig("sim_length must be positive")
        subs = self.network.subnetworks
        if not subs:
            raise InvalidConfig("At least one subnetwork required")
        for i, sub in enumerate(subs):
            info = lookup_model(sub.model)
            if info is None:
                raise InvalidConfig(f"Unknown model '{sub.model}' in subnetwork {i}. Known models: "
                                    + ", ".join(MODEL_REGISTRY))
            nvar, _, nparams = info
            if sub.nmodes < 1:
                raise InvalidConfig(f"Subnetwork {i}: nmodes must be >= 1")
            if len(sub.params) != nparams:
                raise InvalidConfig(f"Subnetwork {i}: model '{sub.model}' expects {nparams} params, got {len(sub.params)}")
            if isinstance(sub.initial_state, list):
                exp = nvar * sub.nnodes * sub.nmodes
                if len(sub.initial_state) != exp:
                    raise InvalidConfig(
                        f"Subnetwork {i}: initial_state has {len(sub.initial_state)} values, expected {exp} "
                        f"(nvar={nvar} * nnodes={sub.nnodes} * nmodes={sub.nmodes})")
            elif isinstance(sub.initial_state, Memory):
                exp = nvar * sub.nnodes * sub.nmodes
                if len(sub.initial_state.data) != exp:
                    raise InvalidConfig(f"Subnetwork {i}: Memory initial_state has {len(sub.initial_state.data)} values, expected {exp}")
                if len(sub.initial_state.shape) != 3:
                    raise InvalidConfig(f"Subnetwork {i}: Memory initial_state shape has {len(sub.initial_state.shape)} dims, expected 3")
        if not isinstance(self.nsig, (int, float)):
            first = lookup_model(subs[0].model)
            if first is not None and len(self.nsig) != first[0]:
                raise InvalidConfig(f"nsig per-variable length {len(self.nsig)} does not match first subnetwork nvar {first[0]}")
        n_subs = len(subs)
        for i, p in enumerate(self.network.projections):
            if p.src >= n_subs:
                raise InvalidConfig(f"Projection {i}: src {p.src} >= number of subnetworks {n_subs}")
            if p.tgt >= n_subs:
                raise InvalidConfig(f"Projection {i}: tgt {p.tgt} >= number of subnetworks {n_subs}")
            sn, tn = subs[p.src].nnodes, subs[p.tgt].nnodes
            w = p.weights
            if isinstance(w, dict):
                if len(w["indptr"]) != tn + 1:
                    raise InvalidConfig(f"Projection {i}: CSR indptr length {len(w['indptr'])} != tgt_nnodes + 1 = {tn + 1}")
                if len(w["data"]) != len(w["indices"]):
                    raise InvalidConfig(f"Projection {i}: CSR data.len() {len(w['data'])} != indices.len() {len(w['indices'])}")
            elif isinstance(w, (int, float)):
                if sn != tn:
                    raise InvalidConfig(f"Projection {i}: scalar weights require src and tgt nnodes to match ({sn} != {tn})")
            else:
                if len(w) != tn:
                    raise InvalidConfig(f"Projection {i}: weights has {len(w)} rows, expected {tn} (tgt nnodes)")
                for r, row in enumerate(w):
                    if len(row) != sn:
                        raise InvalidConfig(f"Projection {i}: weights row {r} has {len(row)} cols, expected {sn} (src nnodes)")
            max_delay = max(p.delays) if p.delays else 0
            n_steps = int(self.sim_length / self.dt)
            if max_delay + 1 > n_steps + 1:
                raise InvalidConfig(f"Projection {i}: max delay {max_delay} requires horizon >= {max_delay + 1}, "
                                    f"but sim only runs {n_steps} steps")

    # --- SimConfig::resolve_delays (config.rs:436-452) ---
    def resolve_delays(self) -> None:
        if self.speed <= 0.0 and any(p.tract_lengths for p in self.network.projections):
            raise InvalidConfig("speed must be positive when tract_lengths are provided")
        for p in self.network.projections:
            if not p.delays and p.tract_lengths:
                p.delays = tract_lengths_to_delays(p.tract_lengths, self.speed, self.dt)


def tract_lengths_to_delays(lengths: Sequence[float], speed: float, dt: float) -> List[int]:
    """idelays = ceil(tract_length / speed / dt) in f32 arithmetic (config.rs:445-448)."""
    l = np.asarray(lengths, dtype=np.float32)
    q = (l / np.float32(speed)) / np.float32(dt)
    return [int(v) for v in np.maximum(np.ceil(q), np.float32(0)).astype(np.uint32)]


@dataclass
class SweepConfig:
    """SweepConfig (config.rs:457-503)."""

    parameter_name: str
    values: Optional[List[float]] = None
    range: Optional[Dict[str, float]] = None

    @staticmethod
    def from_file(path: str) -> "SweepConfig":
        with open(path, "rb") as f:
            raw = tomllib.load(f)
        return SweepConfig(parameter_name=raw["parameter_name"], values=raw.get("values"), range=raw.get("range"))

    def generate_values(self) -> List[float]:
        if self.values is not None:
            return [float(v) for v in self.values]
        if self.range is not None:
            start = np.float32(self.range["start"])
            step = np.float32(self.range["step"])
            end = np.float32(self.range["end"])
            if step <= 0:
                return []
            n = int(math.ceil(np.float32((end - start) / step))) + 1
            return [float(start + np.float32(i) * step) for i in range(n)]
        return []


def parse_sweep_param(name: str, cfg: SimConfig):
    """cli.rs:976-998: 'subnetworks[N].params[M]' -> (N, M)."""
    if name in ("dt", "nsig"):
        raise InvalidConfig(f"Batch sweep does not support sweeping {name} (model parameter sweeps only)")
    if name.startswith("subnetworks[") and "].params[" in name:
        try:
            sub_idx = int(name[name.index("[") + 1:name.index("]")])
        except ValueError as e:
            raise InvalidConfig(f"invalid subnetwork index: {e}") from None
        try:
            param_idx = int(name[name.rindex("[") + 1:name.rindex("]")])
        except ValueError as e:
            raise InvalidConfig(f"invalid param index: {e}") from None
        if sub_idx >= len(cfg.network.subnetworks):
            raise InvalidConfig(f"subnetwork index {sub_idx} out of range")
        return sub_idx, param_idx
    raise InvalidConfig(f"unsupported sweep parameter_name: {name}. Use format: subnetworks[N].params[M]")


def resolve_initial_state(sub: SubnetworkConfig) -> np.ndarray:
    """Single-point initial state in the batch layout [nnodes*nmodes, nvar], engine.rs:161-237.

    The 3-D NPY branch keeps the reference's index expression (engine.rs:207)."""
    info = lookup_model(sub.model)
    nvar = info[0] if info else 1
    init = sub.initial_state
    if isinstance(init, list):
        return np.asarray(init, dtype=np.float32)
    if isinstance(init, Memory):
        return np.asarray(init.data, dtype=np.float32)
    try:
        data = np.load(init)
    except (OSError, ValueError) as e:
        raise IOError_(str(e)) from None
    if data.dtype not in (np.float32, np.float64):
        raise IOError_(f"unsupported NPY dtype {data.dtype}")
    data = data.astype(np.float32)
    if data.ndim == 2:
        single = np.ascontiguousarray(data.T).ravel()
        if sub.nmodes > 1:
            single = np.tile(single, sub.nmodes)
        return single
    if data.ndim == 3:
        nv, nn, nm = data.shape
        flat = data.ravel()
        out = np.zeros(nn * nm * nv, dtype=np.float32)
        for m in range(nm):
            for n in range(nn):
                for v in range(nv):
                    src = (v * nn * n) * nm + m
                    if src >= flat.size:
                        # the reference indexes out of bounds here and panics
                        raise InvalidState(f"3-D initial state NPY: index {src} out of bounds for {flat.size} values")
                    out[(n * nm + m) * nv + v] = flat[src]
        return out
    raise InvalidConfig(f"Initial state NPY has {data.ndim} dims, expected 2 or 3")
