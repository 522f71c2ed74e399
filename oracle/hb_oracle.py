"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline / reference legs import this
module, as the checker of the CUDA engine. It exposes the same ``from_config`` / ``run_sweep`` /
``run_sweep_multi`` surface as :class:`hyburn_gb300.engine.BatchHybridEngine`, plus the unit entry
points used by the reference's known-answer tests.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

from hyburn_gb300 import _abi
from hyburn_gb300.config import SimConfig, resolve_initial_state
from hyburn_gb300.engine import BatchSweepResult, SweepParam, SweepSpec, raise_for

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {}


def build() -> None:
    """Compile the oracle (FP32 and FP64 twin) with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def load(precision: str = "f32"):
    if precision in _LIBS:
        return _LIBS[precision]
    name = "libhb_oracle.so" if precision == "f32" else "libhb_oracle64.so"
    path = os.path.join(HERE, "_build", name)
    src = os.path.join(HERE, "hb_oracle.c")
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        build()
    lib = C.CDLL(path)
    pre = "hbo_" if precision == "f32" else "hbo64_"
    P, I32, I64, U32, D = C.c_void_p, C.c_int32, C.c_int64, C.c_uint32, C.c_double
    FP = C.POINTER(C.c_float)
    sig = {
        "last_error": (C.c_char_p, []),
        "engine_create": (P, [C.POINTER(_abi.hb_sim_desc), I32, C.POINTER(I32)]),
        "engine_destroy": (None, [P]),
        "engine_reset": (None, [P]),
        "engine_run_sweep": (I32, [P, I32, I32, FP, I32, I64, U32, FP, I64, I32]),
        "engine_run_sweep_multi": (I32, [P, C.POINTER(_abi.hb_sweep_point), I32, I64, U32, FP, I64, I32]),
        "engine_step": (I64, [P]),
        "engine_n_bold": (I32, [P]),
        "result_tavg": (FP, [P, I32, C.POINTER(I64)]),
        "result_final": (FP, [P, I32, C.POINTER(I64)]),
        "result_traj": (FP, [P, I32, C.POINTER(I64)]),
        "result_bold": (FP, [P, I32, C.POINTER(I64)]),
        "result_params": (FP, [P, C.POINTER(I64)]),
        "dfun": (I32, [C.c_char_p, FP, I32, I32, FP, FP, I32, FP]),
        "clamp": (I32, [C.c_char_p, FP, I32]),
        "coupling_pre": (I32, [C.c_char_p, FP, I32, I32, FP, I32, I32, FP, C.POINTER(I32)]),
        "coupling_post": (I32, [C.c_char_p, FP, I32, I32, FP, I32, I32, FP, I32, FP, FP, C.POINTER(I32)]),
        "bold_model_run": (None, [I32, FP, D, I32, FP]),
        "bold_monitor_run": (FP, [I32, I32, D, D, FP, I32, I32, C.POINTER(I64), C.POINTER(I64)]),
        "free": (None, [P]),
    }
    funcs = {}
    for k, (res, args) in sig.items():
        fn = getattr(lib, pre + k)
        fn.restype, fn.argtypes = res, args
        funcs[k] = fn
    _LIBS[precision] = (lib, funcs)
    return _LIBS[precision]


def _fp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class OracleEngine:
    """CPU restatement of BatchHybridEngine with the engine's Python surface."""

    def __init__(self, config: SimConfig, n_sweep: int, semantics: int = 0, precision: str = "f32",
                 n_threads: Optional[int] = None):
        _, self._f = load(precision)
        self.config = config
        self.n_sweep = int(n_sweep)
        self.semantics = int(semantics)
        self.n_threads = int(n_threads or 1)
        states = [resolve_initial_state(s) for s in config.network.subnetworks]
        self._sd = _abi.build_sim_desc(config, states, semantics)
        st = C.c_int32()
        self._h = self._f["engine_create"](C.byref(self._sd.desc), self.n_sweep, C.byref(st))
        raise_for(st.value, self._f["last_error"]().decode())

    @classmethod
    def from_config(cls, config: SimConfig, n_sweep: int, semantics: int = 0, **kw) -> "OracleEngine":
        return cls(config, n_sweep, semantics, **kw)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._f["engine_destroy"](h)
            self._h = None

    def _collect(self, record_traj: bool, n_dims: int = 1) -> BatchSweepResult:
        f, n = self._f, C.c_int64()
        nsub = len(self.config.network.subnetworks)
        pv = _abi.copy_out(f["result_params"](self._h, C.byref(n)), n.value)
        tavg = [_abi.copy_out(f["result_tavg"](self._h, i, C.byref(n)), n.value) for i in range(nsub)]
        fin = [_abi.copy_out(f["result_final"](self._h, i, C.byref(n)), n.value) for i in range(nsub)]
        traj = None
        if record_traj:
            traj = [_abi.copy_out(f["result_traj"](self._h, i, C.byref(n)), n.value) for i in range(nsub)]
        nb = f["engine_n_bold"](self._h)
        bold = None
        if nb > 0:
            bold = []
            for m in range(nb):
                p = f["result_bold"](self._h, m, C.byref(n))
                bold.append(_abi.copy_out(p, n.value) if n.value > 0 else np.zeros(0, np.float32))
        return BatchSweepResult(param_values=pv, tavg=tavg, final_states=fin, trajectories=traj, bold=bold,
                                elapsed_ms=0.0, n_sweep=self.n_sweep)

    def run_sweep(self, param: SweepParam, param_values: Sequence[float], n_steps: int, noise=None,
                  run_flags: int = 0) -> BatchSweepResult:
        vals = np.ascontiguousarray(np.asarray(param_values, dtype=np.float32))
        nz = None if noise is None else np.ascontiguousarray(np.asarray(noise, dtype=np.float32))
        st = self._f["engine_run_sweep"](self._h, int(param.sub_idx), int(param.param_idx), _fp(vals), vals.size,
                                         int(n_steps), int(run_flags), _fp(nz) if nz is not None else None,
                                         0 if nz is None else nz.size, self.n_threads)
        raise_for(st, self._f["last_error"]().decode())
        return self._collect(bool(run_flags & _abi.HB_RUN_TRAJECTORY))

    def run_sweep_with_trajectory(self, param, values, n_steps, noise=None, run_flags: int = 0):
        return self.run_sweep(param, values, n_steps, noise, run_flags | _abi.HB_RUN_TRAJECTORY)

    def run_sweep_multi(self, spec: SweepSpec, n_steps: int, noise=None, run_flags: int = 0) -> BatchSweepResult:
        arr, keep = _abi.sweep_points(spec.points)
        nz = None if noise is None else np.ascontiguousarray(np.asarray(noise, dtype=np.float32))
        st = self._f["engine_run_sweep_multi"](self._h, arr, len(spec.points), int(n_steps), int(run_flags),
                                               _fp(nz) if nz is not None else None, 0 if nz is None else nz.size,
                                               self.n_threads)
        raise_for(st, self._f["last_error"]().decode())
        return self._collect(bool(run_flags & _abi.HB_RUN_TRAJECTORY), len(spec.points))

    def run_sweep_multi_with_trajectory(self, spec, n_steps, noise=None, run_flags: int = 0):
        return self.run_sweep_multi(spec, n_steps, noise, run_flags | _abi.HB_RUN_TRAJECTORY)

    @property
    def step(self) -> int:
        return int(self._f["engine_step"](self._h))

    def reset(self) -> None:
        self._f["engine_reset"](self._h)


# ---- unit entry points (known-answer tests) ----

def dfun(model: str, params, state, coupling, sweep_form: bool = False, precision: str = "f32") -> np.ndarray:
    _, f = load(precision)
    p = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(np.atleast_2d(state), dtype=np.float32)
    c = np.ascontiguousarray(np.atleast_2d(coupling), dtype=np.float32)
    out = np.zeros_like(x)
    raise_for(f["dfun"](model.encode(), _fp(p), p.size, int(sweep_form), _fp(x), _fp(c), x.shape[0], _fp(out)),
              f["last_error"]().decode())
    return out


def clamp(model: str, state, precision: str = "f32") -> np.ndarray:
    _, f = load(precision)
    x = np.ascontiguousarray(np.atleast_2d(state), dtype=np.float32).copy()
    raise_for(f["clamp"](model.encode(), _fp(x), x.shape[0]), f["last_error"]().decode())
    return x


def coupling_pre(name: str, params, x, cpu_form: bool = False) -> np.ndarray:
    _, f = load()
    p = np.ascontiguousarray(params, dtype=np.float32)
    xa = np.ascontiguousarray(np.atleast_2d(x), dtype=np.float32)
    out = np.zeros((xa.shape[0], max(2 * xa.shape[1], 1)), np.float32)
    pc = C.c_int32()
    raise_for(f["coupling_pre"](name.encode(), _fp(p) if p.size else None, p.size, int(cpu_form), _fp(xa),
                                xa.shape[0], xa.shape[1], _fp(out), C.byref(pc)), f["last_error"]().decode())
    return np.ascontiguousarray(out.ravel()[: xa.shape[0] * pc.value]).reshape(xa.shape[0], pc.value)


def coupling_post(name: str, params, gx, x_i=None, n_src: int = 1, rowsums=None) -> np.ndarray:
    _, f = load()
    p = np.ascontiguousarray(params, dtype=np.float32)
    g = np.ascontiguousarray(np.atleast_2d(gx), dtype=np.float32)
    xi = None if x_i is None else np.ascontiguousarray(np.atleast_2d(x_i), dtype=np.float32)
    rs = None if rowsums is None else np.ascontiguousarray(rowsums, dtype=np.float32)
    tgt_ncv = xi.shape[1] if xi is not None else g.shape[1]
    out = np.zeros((g.shape[0], max(g.shape[1], tgt_ncv)), np.float32)
    oc = C.c_int32()
    raise_for(f["coupling_post"](name.encode(), _fp(p) if p.size else None, p.size, int(n_src), _fp(g), g.shape[0],
                                 g.shape[1], _fp(xi) if xi is not None else None, tgt_ncv,
                                 _fp(rs) if rs is not None else None, _fp(out), C.byref(oc)), f["last_error"]().decode())
    return np.ascontiguousarray(out.ravel()[: g.shape[0] * oc.value]).reshape(g.shape[0], oc.value)


def bold_model_run(input_, dt: float, n_steps: int) -> np.ndarray:
    _, f = load()
    inp = np.ascontiguousarray(input_, dtype=np.float32)
    out = np.zeros((n_steps, inp.size), np.float32)
    f["bold_model_run"](inp.size, _fp(inp), float(dt), int(n_steps), _fp(out))
    return out


def bold_monitor_run(inputs, bold_period: int, tr: float, dt_neural: float, flush: bool = True):
    _, f = load()
    a = np.ascontiguousarray(np.atleast_2d(inputs), dtype=np.float32)
    rows, ns = C.c_int64(), C.c_int64()
    p = f["bold_monitor_run"](a.shape[1], int(bold_period), float(tr), float(dt_neural), _fp(a), a.shape[0],
                              int(flush), C.byref(rows), C.byref(ns))
    out = _abi.copy_out(p, rows.value * a.shape[1]) if rows.value > 0 else np.zeros(0, np.float32)
    if p:
        f["free"](C.cast(p, C.c_void_p))
    return (out.reshape(rows.value, a.shape[1]) if rows.value > 0 else out), ns.value
