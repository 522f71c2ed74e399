"""Oracle (test infrastructure only): a byte-level restatement of hyburn's NPY reader and writer,
``src/io.rs`` (writer 88-125, reader 25-83, header scanner 150-228), used by the tests to check
the engine library's ``hb_npy_*`` functions. Pinned by the reference's own round-trip test
(io.rs:238-248) and by numpy's reader and writer (tests/test_npy.py).
"""
from __future__ import annotations

import struct
from typing import List, Sequence, Tuple

import numpy as np

MAGIC = b"\x93NUMPY"


class NpyError(Exception):
    """SimulationError::InvalidState of the reader, with the reference's message."""


def header_text(shape: Sequence[int]) -> str:
    """io.rs:93-112: the header dict, padded so that 10 + len + 1 is a multiple of 64, plus newline."""
    if len(shape) == 1:
        sh = f"({shape[0]},)"
    else:
        sh = "(" + ", ".join(str(int(s)) for s in shape) + ")"
    h = "{'descr': '<f4', 'fortran_order': False, 'shape': " + sh + " }"
    rem = (len(h) + 10 + 1) % 64
    h += " " * (0 if rem == 0 else 64 - rem)
    return h + "\n"


def write_bytes(data: Sequence[float], shape: Sequence[int]) -> bytes:
    """io.rs:88-125: magic, version 1.0, u16 header length, header, little-endian f32 values."""
    h = header_text(shape).encode()
    out = MAGIC + bytes([1, 0]) + struct.pack("<H", len(h)) + h
    n = 1
    for s in shape:
        n *= int(s)
    return out + struct.pack(f"<{n}f", *[float(x) for x in list(data)[:n]])


def find_quoted_value(header: str, key: str):
    """io.rs:154-204: the value of 'key': outside string literals: a tuple's trimmed contents or a
    quoted string's contents; None when absent. Raises NpyError for an unclosed tuple (a panic in
    the reference)."""
    n, kl = len(header), len(key)
    in_string = False
    i = 0
    while i < n:
        ch = header[i]
        if not in_string and ch in "'\"":
            q = ch
            if (i + 1 + kl + 1 < n and header[i + 1:i + 1 + kl] == key and header[i + 1 + kl] == q
                    and header[i + 1 + kl + 1] == ":"):
                rest = header[i + 1 + kl + 2:]
                t = rest.lstrip(" \t\n\r\x0b\x0c")
                if t.startswith("("):
                    depth = 0
                    for k, c in enumerate(t):
                        if c == "(":
                            depth += 1
                        if c == ")":
                            depth -= 1
                        if depth == 0 and c == ")":
                            return t[1:k].strip(" \t\n\r\x0b\x0c")
                    raise NpyError("Failed to parse NPY shape: unclosed tuple")
                if t[:1] in ("'", '"'):
                    end = t.find(t[0], 1)
                    if end >= 0:
                        return t[1:end]
        if ch in "'\"":
            in_string = not in_string
        i += 1
    return None


def _parse_dim(s: str) -> int:
    body = s[1:] if s.startswith("+") else s
    if not body or not body.isdigit() or not body.isascii():
        raise NpyError("Failed to parse NPY shape: invalid digit found in string")
    v = int(body)
    if v >= 1 << 64:
        raise NpyError("Failed to parse NPY shape: number too large to fit in target type")
    return v


def read_bytes(buf: bytes) -> Tuple[List[float], List[int]]:
    """io.rs:25-83 (files shorter than the 10-byte prefix, a panic in the reference, raise
    NpyError('Not a valid .npy file'))."""
    if len(buf) < 10 or buf[:6] != MAGIC:
        raise NpyError("Not a valid .npy file")
    major = buf[6]
    if major < 2:
        header_len = 10 + struct.unpack("<H", buf[8:10])[0]
    else:
        if len(buf) < 12:
            raise NpyError("Not a valid .npy file")
        header_len = 12 + struct.unpack("<I", buf[8:12])[0]
    header = buf[10:min(header_len, len(buf))].decode("utf-8", errors="replace")
    inner = find_quoted_value(header, "shape")
    if inner is None:
        raise NpyError("No 'shape' key in NPY header")
    shape = [_parse_dim(p.strip(" \t\n\r\x0b\x0c")) for p in inner.split(",") if p.strip(" \t\n\r\x0b\x0c")]
    descr = find_quoted_value(header, "descr")
    if descr is None:
        raise NpyError("No 'descr' key in NPY header")
    if descr not in ("<f4", "|f4", "f4", "<f8"):
        raise NpyError(f"Unsupported NPY dtype descriptor: '{descr}', only f32/f64 supported")
    total = 1
    for s in shape:
        total *= s
    data = buf[header_len:] if header_len < len(buf) else b""
    if descr == "<f8":
        if len(data) < total * 8:
            raise NpyError("NPY data truncated (f64)")
        n = len(data) // 8
        with np.errstate(over="ignore"):
            vals = np.frombuffer(data[:8 * n], dtype="<f8").astype(np.float32)  # round to nearest, as `as f32`
        return [float(v) for v in vals], shape
    if len(data) < total * 4:
        raise NpyError("NPY data truncated (f32)")
    n = len(data) // 4
    return list(struct.unpack(f"<{n}f", data[:4 * n])), shape
