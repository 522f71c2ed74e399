"""The Rust binding that INTEGRATION.md gives a maintainer (the `hyburn-gb300-sys` block) against the C
header: each `#[repr(C)]` struct has the header's fields in the header's order with matching types, and
each `extern "C"` function the header's parameters with matching types. The header itself is checked
against a C compiler in test_abi_layout.py; the Rust text cannot be compiled here (no Rust toolchain),
so this keeps it from drifting."""
import os
import re

import pytest

from hyburn_gb300 import _abi
from test_abi_layout import STRUCTS, _prototypes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RUST_SCALAR = {"i32": "int32_t", "i64": "int64_t", "u32": "uint32_t", "f32": "float", "f64": "double",
               "hb_status": "int32_t"}
C_SCALAR = {"int32_t": "int32_t", "hb_status": "int32_t", "int64_t": "int64_t", "uint32_t": "uint32_t",
            "float": "float", "double": "double"}


def _sys_block():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```rust\n(.*?)```", text, flags=re.S)
    sys_blocks = [b for b in blocks if "hyburn-gb300-sys/src/lib.rs" in b]
    assert len(sys_blocks) == 1
    return re.sub(r"//[^\n]*", "", sys_blocks[0])


def _rust_kind(t):
    t = t.strip()
    if t.startswith("*"):
        return "ptr"
    return RUST_SCALAR.get(t, t)


def _c_kind(t):
    t = t.replace("const ", "").strip()
    if "*" in t:
        return "ptr"
    return C_SCALAR.get(t.split()[0], t)


def _split_params(s):
    s = " ".join(s.split())
    return [p.strip() for p in s.split(",") if p.strip()] if s else []


def _rust_structs():
    out = {}
    for name, body in re.findall(r"#\[repr\(C\)\]\s*pub struct (hb_\w+)\s*\{(.*?)\}", _sys_block(), flags=re.S):
        fields = re.findall(r"pub (\w+)\s*:\s*([^,]+?)\s*(?:,|$)", " ".join(body.split()))
        if fields:
            out[name] = [(f, _rust_kind(t)) for f, t in fields]
    return out


def _c_field_kind(ct):
    if ct in (_abi.C.c_void_p, _abi.C.c_char_p) or (isinstance(ct, type) and issubclass(ct, _abi.C._Pointer)):
        return "ptr"
    return {_abi.C.c_int32: "int32_t", _abi.C.c_int64: "int64_t", _abi.C.c_uint32: "uint32_t",
            _abi.C.c_float: "float", _abi.C.c_double: "double"}[ct]


@pytest.mark.parametrize("struct", STRUCTS, ids=lambda s: s.__name__)
def test_rust_structs_match_the_header(struct):
    rust = _rust_structs()
    assert struct.__name__ in rust, f"{struct.__name__} missing from the Rust binding"
    want = [(f, _c_field_kind(t)) for f, t in struct._fields_]
    assert rust[struct.__name__] == want


def test_rust_functions_match_the_header():
    protos = _prototypes()
    fns = re.findall(r"pub fn (hb_\w+)\s*\((.*?)\)\s*(?:->\s*([^;]+))?;", _sys_block(), flags=re.S)
    assert {n for n, _, _ in fns} == set(protos), "the Rust block must declare every entry point of the header"
    for name, params, ret in fns:
        assert name in protos, f"{name} is not declared in the header"
        c_ret, c_params = protos[name]
        rp = _split_params(params)
        assert len(rp) == len(c_params), f"{name}: {len(rp)} Rust parameters, {len(c_params)} in C"
        for i, (r, c) in enumerate(zip(rp, c_params)):
            assert _rust_kind(r.split(":", 1)[1]) == _c_kind(c), f"{name} parameter {i}: Rust '{r}' vs C '{c}'"
        want_ret = "void" if c_ret == "void" else _c_kind(c_ret)
        got_ret = "void" if not ret else _rust_kind(ret)
        assert got_ret == want_ret, f"{name} return: Rust '{ret}' vs C '{c_ret}'"
