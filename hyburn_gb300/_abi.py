"""ctypes mirror of ``include/hyburn_gb300.h`` and marshalling of a SimConfig into ``hb_sim_desc``.

The descriptor is what the reference's Rust side would hand over after `SimConfig` parsing and the
batch engine's own initial-state resolution (src/engine/batch_engine/engine.rs:161-247).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import Any, List, Optional, Sequence

import numpy as np

HB_ABI_VERSION = 2

HB_OK = 0
HB_ERR_INVALID_CONFIG = 1
HB_ERR_INVALID_STATE = 2
HB_ERR_BACKEND = 3
HB_ERR_IO = 4
HB_ERR_CUDA = 5
HB_ERR_NONFINITE = 6
HB_ERR_TIMEOUT = 7
HB_ERR_UNSUPPORTED = 8

HB_INT = {"heun": 0, "euler": 1, "euler_stochastic": 2, "heun_stochastic": 3, "rk4": 4, "rk4_stochastic": 5}
STOCHASTIC = {"euler_stochastic", "heun_stochastic", "rk4_stochastic"}

HB_WEIGHTS_SCALAR, HB_WEIGHTS_DENSE, HB_WEIGHTS_CSR = 0, 1, 2

HB_SEM_DELAY_RING = 1 << 0
HB_SEM_SCALAR_DIAGONAL = 1 << 1
HB_SEM_BOLD_PER_POINT = 1 << 2
HB_SEM_NOISE_PER_POINT = 1 << 3
HB_SEM_HYBRID_INTEGRATOR = 1 << 4

HB_RUN_TRAJECTORY = 1 << 0
HB_RUN_CHECK_FINITE = 1 << 1
HB_RUN_DENSE_TC = 1 << 2
HB_RUN_EXACT_SUMS = 1 << 3
HB_RUN_FORCE_RESIDENT = 1 << 8
HB_RUN_FORCE_BLOCKED = 1 << 9
HB_RUN_GLOBAL_RING = 1 << 10
HB_RUN_GENERIC = 1 << 11
HB_RUN_TWO_PHASE = 1 << 16
HB_RUN_NO_PIPE = 1 << 17
HB_RUN_STREAM = 1 << 18
HB_RUN_NO_STREAM = 1 << 19


def HB_RUN_PIPE_LANES(n: int) -> int:
    return (n & 0xf) << 20


def HB_RUN_STREAM_NPT(n: int) -> int:
    return (n & 0x7) << 24


HB_RUN_STREAM_PREFETCH = 1 << 27
HB_RUN_STREAM_BULK = 1 << 7
HB_RUN_PIPE_WIDE = 1 << 28
HB_RUN_DEVICE_TRAJECTORY = 1 << 29
HB_RUN_TEST_UNSET_WAIT = 1 << 30


def HB_RUN_STREAM_CLUSTER(n: int) -> int:
    """Streamed-history kernel: CTAs per sweep point (a thread-block cluster splitting its nodes)."""
    return {1: 1, 2: 2, 4: 3, 8: 4, 3: 5, 5: 6, 6: 7}.get(int(n), 0) << 4


# the run flags that choose a kernel form or its lane counts (what the autotuner chooses)
HB_RUN_KERNEL_CHOICE = (HB_RUN_DENSE_TC | HB_RUN_FORCE_RESIDENT | HB_RUN_FORCE_BLOCKED | HB_RUN_GLOBAL_RING | HB_RUN_GENERIC | (0x7 << 4)
                        | (0xF << 12)
                        | HB_RUN_TWO_PHASE | HB_RUN_NO_PIPE | HB_RUN_STREAM | HB_RUN_NO_STREAM | (0xF << 20)
                        | (0x7 << 24) | HB_RUN_STREAM_PREFETCH | HB_RUN_PIPE_WIDE | HB_RUN_STREAM_BULK)
# the streamed-history kernel's form within those: nodes per consumer thread and L2 prefetch
HB_RUN_STREAM_FORM = (0x7 << 24) | HB_RUN_STREAM_PREFETCH


def HB_RUN_LANES(n: int) -> int:
    return {1: 1, 2: 2, 4: 3, 8: 4}.get(n, 0) << 12


# MODEL_REGISTRY rows of the six hot-path models (src/config.rs:43-49): (nvar, ncvar, nparams)
MODEL_INFO = {
    "Generic2dOscillator": (2, 1, 12),
    "MontbrioPazoRoxin": (2, 2, 7),
    "ReducedWongWang": (1, 1, 8),
    "Kuramoto": (1, 1, 1),
    "JansenRit": (6, 1, 13),
    "WilsonCowan": (2, 1, 22),
}


class hb_subnet_desc(C.Structure):
    _fields_ = [
        ("model", C.c_char_p),
        ("nnodes", C.c_int32),
        ("nmodes", C.c_int32),
        ("params", C.POINTER(C.c_float)),
        ("n_params", C.c_int32),
        ("initial_state", C.POINTER(C.c_float)),
        ("n_initial_state", C.c_int64),
        ("node_params", C.POINTER(C.c_float)),
        ("n_node_params", C.c_int64),
    ]


class hb_projection_desc(C.Structure):
    _fields_ = [
        ("src", C.c_int32),
        ("tgt", C.c_int32),
        ("weights_kind", C.c_int32),
        ("scalar_weight", C.c_float),
        ("dense", C.POINTER(C.c_float)),
        ("dense_rows", C.c_int32),
        ("dense_cols", C.c_int32),
        ("csr_data", C.POINTER(C.c_float)),
        ("csr_indices", C.POINTER(C.c_uint32)),
        ("csr_indptr", C.POINTER(C.c_uint32)),
        ("nnz", C.c_int64),
        ("n_indptr", C.c_int64),
        ("delays", C.POINTER(C.c_uint32)),
        ("n_delays", C.c_int64),
        ("coupling_fn", C.c_char_p),
        ("coupling_params", C.POINTER(C.c_float)),
        ("n_coupling_params", C.c_int32),
        ("cvar_map", C.c_char_p),
    ]


class hb_bold_desc(C.Structure):
    _fields_ = [("bold_period", C.c_int32), ("tr", C.c_double)]


class hb_sim_desc(C.Structure):
    _fields_ = [
        ("dt", C.c_double),
        ("integrator", C.c_int32),
        ("nsig", C.POINTER(C.c_float)),
        ("n_nsig", C.c_int32),
        ("n_subnets", C.c_int32),
        ("subnets", C.POINTER(hb_subnet_desc)),
        ("n_projections", C.c_int32),
        ("projections", C.POINTER(hb_projection_desc)),
        ("n_bold", C.c_int32),
        ("bold", C.POINTER(hb_bold_desc)),
        ("flags", C.c_uint32),
    ]


class hb_sweep_point(C.Structure):
    _fields_ = [
        ("sub_idx", C.c_int32),
        ("param_idx", C.c_int32),
        ("values", C.POINTER(C.c_float)),
        ("n_values", C.c_int32),
    ]


def f32p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def u32p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


@dataclass
class SimDesc:
    """A filled ``hb_sim_desc`` plus the arrays it points into (kept alive here)."""

    desc: hb_sim_desc
    keep: List[Any] = field(default_factory=list)
    noise_row: int = 0           # floats per step (one point) of the noise array
    stochastic: bool = False
    nvars: List[int] = field(default_factory=list)
    nodes: List[int] = field(default_factory=list)


def _arr(x, dtype) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=dtype))


def build_sim_desc(cfg, resolved_states: Sequence[np.ndarray], flags: int = 0) -> SimDesc:
    """Marshal a :class:`hyburn_gb300.config.SimConfig` into ``hb_sim_desc``.

    ``resolved_states[i]`` is subnetwork i's single-point initial state in the batch layout
    ``[nnodes*nmodes, nvar]`` (flattened), as BatchHybridEngine::from_config builds it.
    """
    keep: List[Any] = []
    subs = cfg.network.subnetworks
    projs = cfg.network.projections
    sub_arr = (hb_subnet_desc * max(1, len(subs)))()
    nvars, nodes = [], []
    for i, s in enumerate(subs):
        params = _arr(s.params, np.float32)
        x0 = _arr(resolved_states[i], np.float32).ravel()
        name = s.model.encode()
        keep += [params, x0, name]
        sub_arr[i].model = name
        sub_arr[i].nnodes = int(s.nnodes)
        sub_arr[i].nmodes = int(s.nmodes)
        sub_arr[i].params = f32p(params)
        sub_arr[i].n_params = params.size
        sub_arr[i].initial_state = f32p(x0)
        sub_arr[i].n_initial_state = x0.size
        node_params = getattr(s, "node_params", None)
        if node_params is not None:
            npar = _arr(node_params, np.float32).ravel()
            keep.append(npar)
            sub_arr[i].node_params = f32p(npar)
            sub_arr[i].n_node_params = npar.size
        nv = MODEL_INFO.get(s.model, (0, 0, 0))[0]
        nvars.append(nv)
        nodes.append(int(s.nnodes) * int(s.nmodes))
    proj_arr = (hb_projection_desc * max(1, len(projs)))()
    for k, p in enumerate(projs):
        d = proj_arr[k]
        d.src, d.tgt = int(p.src), int(p.tgt)
        w = p.weights
        if isinstance(w, dict):
            data = _arr(w["data"], np.float32)
            ind = _arr(w["indices"], np.uint32)
            ptr = _arr(w["indptr"], np.uint32)
            keep += [data, ind, ptr]
            d.weights_kind = HB_WEIGHTS_CSR
            d.csr_data, d.csr_indices, d.csr_indptr = f32p(data), u32p(ind), u32p(ptr)
            d.nnz, d.n_indptr = data.size, ptr.size
        elif isinstance(w, (int, float, np.floating)):
            d.weights_kind = HB_WEIGHTS_SCALAR
            d.scalar_weight = float(w)
        else:
            dense = _arr(w, np.float32)
            if dense.ndim != 2:
                dense = dense.reshape(len(w), -1)
            keep.append(dense)
            d.weights_kind = HB_WEIGHTS_DENSE
            d.dense = f32p(dense)
            d.dense_rows, d.dense_cols = dense.shape
        delays = _arr(p.delays if p.delays is not None else [], np.uint32)
        keep.append(delays)
        d.delays = u32p(delays) if delays.size else None
        d.n_delays = delays.size
        fn = (p.coupling_fn or "Linear").encode()
        cp = _arr(p.coupling_params or [], np.float32)
        cm = (p.cvar_map or "0:0").encode()
        keep += [fn, cp, cm]
        d.coupling_fn = fn
        d.coupling_params = f32p(cp) if cp.size else None
        d.n_coupling_params = cp.size
        d.cvar_map = cm
    bolds = [m for m in cfg.monitors if m.monitor_type.lower() == "bold"]
    bold_arr = (hb_bold_desc * max(1, len(bolds)))()
    for k, m in enumerate(bolds):
        bp = m.bold_period
        if bp is None:
            period = m.period if m.period is not None else 2000.0
            bp = int(round(max(period / cfg.dt, 1.0)))
        bold_arr[k].bold_period = int(bp)
        bold_arr[k].tr = float(m.tr if m.tr is not None else 2.0)
    first_nvar = nvars[0] if nvars else 1
    nsig = _arr(cfg.nsig_vec(first_nvar), np.float32)
    keep += [sub_arr, proj_arr, bold_arr, nsig]
    desc = hb_sim_desc()
    desc.dt = float(cfg.dt)
    desc.integrator = HB_INT[cfg.integrator]
    desc.nsig = f32p(nsig)
    desc.n_nsig = nsig.size
    desc.n_subnets = len(subs)
    desc.subnets = C.cast(sub_arr, C.POINTER(hb_subnet_desc))
    desc.n_projections = len(projs)
    desc.projections = C.cast(proj_arr, C.POINTER(hb_projection_desc))
    desc.n_bold = len(bolds)
    desc.bold = C.cast(bold_arr, C.POINTER(hb_bold_desc))
    desc.flags = int(flags)
    row = sum(n * v for n, v in zip(nodes, nvars))
    return SimDesc(desc=desc, keep=keep, noise_row=row, stochastic=cfg.integrator in STOCHASTIC,
                   nvars=nvars, nodes=nodes)


def sweep_points(dims) -> tuple:
    """Marshal SweepPoint dimensions into an ``hb_sweep_point`` array (+ keep-alive list)."""
    arr = (hb_sweep_point * max(1, len(dims)))()
    keep = [arr]
    for k, d in enumerate(dims):
        v = _arr(d.values, np.float32)
        keep.append(v)
        arr[k].sub_idx, arr[k].param_idx = int(d.sub_idx), int(d.param_idx)
        arr[k].values, arr[k].n_values = f32p(v), v.size
    return arr, keep


_LIB = None
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libhyburn_gb300.so")


class hb_group_member(C.Structure):
    _fields_ = [("engine", C.c_void_p), ("sub_idx", C.c_int32), ("param_idx", C.c_int32),
                ("values", C.POINTER(C.c_float)), ("n_values", C.c_int32), ("n_steps", C.c_int64),
                ("run_flags", C.c_uint32), ("noise", C.POINTER(C.c_float)), ("noise_len", C.c_int64)]


class hb_adjoint_out(C.Structure):
    _fields_ = [("loss", C.POINTER(C.c_double)), ("d_gain", C.POINTER(C.c_double)), ("d_A", C.POINTER(C.c_double)),
                ("d_B", C.POINTER(C.c_double)), ("d_a", C.POINTER(C.c_double)), ("fc", C.POINTER(C.c_float)),
                ("y", C.POINTER(C.c_float)), ("forward_ms", C.c_float), ("statistics_ms", C.c_float),
                ("reverse_ms", C.c_float)]


class hb_order_adjoint_out(C.Structure):
    _fields_ = [("loss", C.POINTER(C.c_double)), ("d_gain", C.POINTER(C.c_double)), ("d_omega", C.POINTER(C.c_double)),
                ("d_omega_node", C.POINTER(C.c_double)),
                ("forward_ms", C.c_float), ("prepare_ms", C.c_float), ("reverse_ms", C.c_float)]


class hb_fc_features(C.Structure):
    _fields_ = [("fc", C.POINTER(C.c_float)), ("features", C.POINTER(C.c_float)), ("fcd", C.POINTER(C.c_float)),
                ("fcd_stats", C.POINTER(C.c_float)), ("n_windows", C.c_int32), ("nnodes", C.c_int32),
                ("nvar", C.c_int32), ("ms", C.c_float)]


def load_library():
    """Load the in-tree engine library; raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"hyburn_gb300 engine library not found at {LIB_PATH}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(LIB_PATH)
    P, I32, I64, U32, D = C.c_void_p, C.c_int32, C.c_int64, C.c_uint32, C.c_double
    FP = C.POINTER(C.c_float)
    sig = {
        "hb_abi_version": (I32, []),
        "hb_last_error": (C.c_char_p, []),
        "hb_model_info": (I32, [C.c_char_p, C.POINTER(I32), C.POINTER(I32), C.POINTER(I32)]),
        "hb_engine_create": (I32, [C.POINTER(hb_sim_desc), I32, C.POINTER(P)]),
        "hb_engine_destroy": (None, [P]),
        "hb_engine_run_sweep": (I32, [P, I32, I32, FP, I32, I64, U32, FP, I64, C.POINTER(P)]),
        "hb_engine_run_sweep_multi": (I32, [P, C.POINTER(hb_sweep_point), I32, I64, U32, FP, I64, C.POINTER(P)]),
        "hb_engine_get_state": (I32, [P, I32, FP, I64]),
        "hb_engine_step": (I64, [P]),
        "hb_engine_reset": (I32, [P]),
        "hb_engine_last_kernel_time": (I32, [P, C.POINTER(D), C.POINTER(I64), C.POINTER(I32)]),
        "hb_engine_set_stream": (I32, [P, P]),
        "hb_engine_set_hybrid_integrator": (I32, [P, I32]),
        "hb_engine_prepare": (I32, [P, I32, I32, FP, I32, I64, U32, FP, I64]),
        "hb_engine_execute_prepared": (I32, [P]),
        "hb_group_prepare": (I32, [C.POINTER(hb_group_member), I32, P, C.POINTER(P)]),
        "hb_group_execute": (I32, [P]),
        "hb_group_result": (I32, [P, I32, C.POINTER(P)]),
        "hb_group_last_kernel_time": (I32, [P, C.POINTER(D)]),
        "hb_group_destroy": (None, [P]),
        "hb_engine_adjoint_fc": (I32, [P, FP, I32, I64, FP, I32, C.POINTER(hb_adjoint_out)]),
        "hb_result_n_sweep": (I32, [P]),
        "hb_result_n_subnets": (I32, [P]),
        "hb_result_n_bold": (I32, [P]),
        "hb_result_elapsed_ms": (D, [P]),
        "hb_result_param_values": (FP, [P, C.POINTER(I64)]),
        "hb_result_tavg": (FP, [P, I32, C.POINTER(I64)]),
        "hb_result_final_states": (FP, [P, I32, C.POINTER(I64)]),
        "hb_result_trajectory": (FP, [P, I32, C.POINTER(I64)]),
        "hb_result_bold": (FP, [P, I32, C.POINTER(I64)]),
        "hb_result_free": (None, [P]),
        "hb_npy_write_f32": (I32, [C.c_char_p, FP, C.POINTER(I64), I32]),
        "hb_npy_read_f32": (I32, [C.c_char_p, FP, I64, C.POINTER(I64), I32, C.POINTER(I32), C.POINTER(I64)]),
        "hb_engine_write_tavg": (I32, [P, P, C.c_char_p]),
        "hb_engine_fc_features": (I32, [P, I32, I32, I32, C.POINTER(hb_fc_features)]),
        "hb_engine_adjoint_order": (I32, [P, FP, I32, I64, U32, C.POINTER(hb_order_adjoint_out)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.hb_abi_version() != HB_ABI_VERSION:
        raise RuntimeError("hyburn_gb300 library ABI version mismatch")
    _LIB = lib
    return lib


def copy_out(ptr, n: int, shape=None) -> Optional[np.ndarray]:
    if not ptr or n <= 0:
        return None if not ptr else np.zeros(0, np.float32)
    a = np.ctypeslib.as_array(ptr, shape=(int(n),)).copy()
    return a.reshape(shape) if shape is not None else a
