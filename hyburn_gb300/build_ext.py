"""In-tree build of the CUDA engine library ``hyburn_gb300/_lib/libhyburn_gb300.so`` for sm_103a.

The kernels' translation unit is compiled with ``--fmad=false`` (no fused multiply-add, matching
the reference's separately rounded element-wise ops); the host engine is plain C++17. Both
translation units compile in parallel and are linked with the static CUDA runtime.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libhyburn_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

UNITS = [
    ("hb_queue_1.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_dense_tc.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_queue_2.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_queue_4.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_stream_1.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_stream_2.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_stream_4.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_pipe.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_pipe_1024.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_fast_1024.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_fast_512.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_resident_generic.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_kernels.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_single.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_adjoint.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_engine.cu", []),
    ("hb_noalloc.cu", ["--fmad=false"]),
    ("hb_io.cu", []),
    ("hb_features.cu", ["--fmad=false", "-lineinfo"]),
    ("hb_kuradj.cu", ["--fmad=false", "-lineinfo"]),
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def build(verbose: bool = False) -> str:
    os.makedirs(os.path.join(OUT_DIR, "obj"), exist_ok=True)
    nvcc = _nvcc()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"), "-I", CSRC] + ARCH

    def compile_unit(unit):
        src, extra = unit
        obj = os.path.join(OUT_DIR, "obj", src.replace(".cu", ".o"))
        cmd = [nvcc] + common + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    cmd = [nvcc, "-shared", "-cudart", "static", "-Xlinker", "--no-undefined"] + ARCH + ["-o", LIB] + objs + ["-lrt", "-lpthread", "-ldl"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
