"""The Python mirror's view of the C ABI against the header itself (no GPU needed).

- Every descriptor and output struct: ctypes size, and offset and size of each field, equal what a C
  compiler gives for include/hyburn_gb300.h (a program built with gcc prints them).
- Every prototype (each one is bound by the mirror): the number of parameters, the width of each scalar and the
  pointer-ness of each pointer parameter, and the return type, equal the ctypes signature.
A mismatch in either would pass arguments or read results at the wrong place without any error.
"""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

from hyburn_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hyburn_gb300.h")
STRUCTS = [_abi.hb_subnet_desc, _abi.hb_projection_desc, _abi.hb_bold_desc, _abi.hb_sim_desc, _abi.hb_sweep_point,
           _abi.hb_group_member, _abi.hb_adjoint_out, _abi.hb_order_adjoint_out, _abi.hb_fc_features]


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "hyburn_gb300.h"', "int main(void) {"]
    for s in STRUCTS:
        t = s.__name__
        lines.append(f'    printf("{t} %zu\\n", sizeof({t}));')
        for f, _ in s._fields_:
            lines.append(f'    printf("{t}.{f} %zu %zu\\n", offsetof({t}, {f}), sizeof((({t}*)0)->{f}));')
    lines += ["    return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c11", "-Wall", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: tuple(int(x) for x in v) for k, *v in (line.split() for line in out.splitlines())}


@pytest.mark.parametrize("struct", STRUCTS, ids=lambda s: s.__name__)
def test_struct_layout_matches_the_header(c_layout, struct):
    t = struct.__name__
    assert c_layout[t] == (C.sizeof(struct),), f"sizeof({t})"
    for f, _ in struct._fields_:
        d = getattr(struct, f)
        assert c_layout[f"{t}.{f}"] == (d.offset, d.size), f"{t}.{f}: C (offset, size) vs ctypes"


# ---- prototypes ----

SCALARS = {"int32_t": C.c_int32, "hb_status": C.c_int32, "int64_t": C.c_int64, "uint32_t": C.c_uint32,
           "double": C.c_double, "float": C.c_float}


def _prototypes():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    text = re.sub(r"#[^\n]*", "", text)
    out = {}
    for ret, name, params in re.findall(r"([A-Za-z_][\w\s\*]*?)\b(hb_[a-z0-9_]+)\s*\(([^;{}]*?)\)\s*;", text):
        ps = [p.strip() for p in params.split(",")] if params.strip() not in ("", "void") else []
        out[name] = (" ".join(ret.split()), ps)
    return out


def _is_pointer(t):
    return t in (C.c_void_p, C.c_char_p) or (isinstance(t, type) and issubclass(t, C._Pointer))


def _check(kind, c_text, ct):
    """c_text: a C parameter or return type (with or without a parameter name)."""
    if "*" in c_text:
        assert _is_pointer(ct), f"{kind}: C '{c_text}' is a pointer, ctypes {ct}"
        return
    words = c_text.replace("const ", "").split()
    base = words[0]
    if base == "void":
        assert ct is None, f"{kind}: C returns void, ctypes {ct}"
    else:
        assert base in SCALARS, f"{kind}: unexpected C type '{c_text}'"
        assert ct is SCALARS[base], f"{kind}: C '{c_text}' vs ctypes {ct}"


def _bound_functions():
    lib = _abi.load_library()
    from test_zz_no_alloc import _bind
    _bind()
    return lib


def test_every_bound_prototype_matches_the_header():
    lib = _bound_functions()
    protos = _prototypes()
    assert len(protos) >= 30
    checked = 0
    for name, (ret, params) in protos.items():
        fn = getattr(lib, name)
        assert fn.argtypes is not None, f"{name} is declared but the mirror does not bind it"
        assert len(fn.argtypes) == len(params), f"{name}: {len(params)} C parameters, {len(fn.argtypes)} ctypes"
        for i, (p, ct) in enumerate(zip(params, fn.argtypes)):
            _check(f"{name} parameter {i}", p, ct)
        _check(f"{name} return", ret, fn.restype)
        checked += 1
    assert checked == len(protos)
