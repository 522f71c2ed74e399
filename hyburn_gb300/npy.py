"""NPY files as hyburn reads and writes them (``src/io.rs:19-125``) and the batch sweep's output
files (``src/cli.rs:932-973``), through the engine library's C ABI (``hb_npy_*``,
``hb_engine_write_tavg``).

``write_npy_f32(path, data, shape)``  io.rs:88-125: version 1.0 header padded to 64 bytes,
                                      little-endian f32.
``read_npy_f32(path)``                io.rs:25-83: (flat float32 values, shape); '<f8' files are
                                      rounded to f32; trailing whole values beyond the shape's
                                      product are returned too, as in the reference.
``write_tavg(engine, result, dir)``   cli.rs:961-970: ``tavg_sub{i}.npy`` per subnetwork, labelled
                                      [n_sweep, nvar, nnodes*nmodes] over data laid out
                                      [n_sweep, nnodes*nmodes, nvar].
``run_batch_sweep(...)``              cli.rs:932-973: one sweep through a fresh engine, its tavg
                                      files written by the library (hb_engine_write_tavg).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Sequence, Tuple

import numpy as np

from . import _abi
from .config import SimConfig


def _raise(status: int) -> None:
    from .engine import raise_for
    raise_for(status, _abi.load_library().hb_last_error().decode())


def write_npy_f32(path: str, data, shape: Sequence[int]) -> None:
    """io.rs:88-125."""
    lib = _abi.load_library()
    a = np.ascontiguousarray(np.asarray(data, dtype=np.float32).ravel())
    dims = (C.c_int64 * max(1, len(shape)))(*[int(d) for d in shape])
    if int(np.prod([int(d) for d in shape], dtype=np.int64)) > a.size:
        raise ValueError(f"shape {tuple(shape)} needs more values than the {a.size} given")
    _raise(lib.hb_npy_write_f32(os.fsencode(path), _abi.f32p(a), dims, len(shape)))


def read_npy_f32(path: str) -> Tuple[np.ndarray, List[int]]:
    """io.rs:25-83: the values (flat, float32) and the shape."""
    lib = _abi.load_library()
    nd, n = C.c_int32(), C.c_int64()
    dims = (C.c_int64 * 32)()
    _raise(lib.hb_npy_read_f32(os.fsencode(path), None, 0, dims, 32, C.byref(nd), C.byref(n)))
    out = np.empty(max(1, n.value), np.float32)
    _raise(lib.hb_npy_read_f32(os.fsencode(path), _abi.f32p(out), out.size, dims, 32, C.byref(nd), C.byref(n)))
    return out[:n.value], [int(dims[i]) for i in range(nd.value)]


def tavg_shapes(config: SimConfig, n_sweep: int) -> List[Tuple[int, int, int]]:
    """The shape label of each subnetwork's tavg file: (n_sweep, nvar, nnodes*nmodes)."""
    lib = _abi.load_library()
    out = []
    for s in config.network.subnetworks:
        nv, ncv, npar = C.c_int32(), C.c_int32(), C.c_int32()
        _raise(lib.hb_model_info(s.model.encode(), C.byref(nv), C.byref(ncv), C.byref(npar)))
        out.append((int(n_sweep), nv.value, int(s.nnodes) * int(s.nmodes)))
    return out


def write_tavg(config: SimConfig, result, output_dir: str) -> List[str]:
    """cli.rs:947-970 for a result already copied to the host: the directory and its parents are
    created, then tavg_sub{i}.npy per subnetwork. Returns the paths written."""
    os.makedirs(output_dir, exist_ok=True)
    paths = []
    for i, (tavg, shape) in enumerate(zip(result.tavg, tavg_shapes(config, result.n_sweep))):
        p = f"{output_dir}/tavg_sub{i}.npy"
        write_npy_f32(p, tavg, shape)
        paths.append(p)
    return paths


def run_batch_sweep(config: SimConfig, sub_idx: int, param_idx: int, values: Sequence[float], n_steps: int,
                    output: str, noise=None, semantics: int = 0, run_flags: int = 0):
    """cli.rs:932-973: a fresh engine of len(values) points runs the sweep once; the library writes
    output/tavg_sub{i}.npy from the run's result. Returns the BatchSweepResult."""
    from .engine import BatchHybridEngine, SweepParam
    eng = BatchHybridEngine.from_config(config, len(values), semantics=semantics)
    try:
        return eng.run_sweep(SweepParam(sub_idx, param_idx), values, n_steps, noise=noise, run_flags=run_flags,
                             output_dir=output)
    finally:
        eng.close()
