"""NPY I/O of the engine library (hb_npy_write_f32 / hb_npy_read_f32, src/io.rs:19-125) and the
batch sweep's tavg_sub{i}.npy files (src/cli.rs:947-970).

The oracle (oracle/npy_ref.py) is pinned first: the reference's round-trip test (io.rs:238-248),
numpy's reader on the oracle's bytes, and the oracle's reader on numpy's files. Then the library
must write the oracle's bytes exactly and read every file (valid or not) as the oracle does."""
import os
import struct

import numpy as np
import pytest

from hyburn_gb300 import npy
from hyburn_gb300.config import InvalidState, IOError_
from oracle import npy_ref

SHAPES = [[], [0], [1], [5], [2, 3], [3, 1], [128, 2, 74], [1, 1, 1, 1], [2, 0, 3],
          [123456789, 0], [1] * 24, [7, 11, 13]]


def _values(shape, seed=0):
    n = int(np.prod(shape, dtype=np.int64))
    return np.random.default_rng(seed).standard_normal(n).astype(np.float32)


# ---- the oracle against the reference's test and numpy ----

def test_oracle_reference_roundtrip():
    # io.rs:238-248: data 1..6, shape [2, 3], written and read back unchanged
    b = npy_ref.write_bytes([1.0, 2.0, 3.0, 4.0, 5.0, 6.0], [2, 3])
    vals, shape = npy_ref.read_bytes(b)
    assert vals == [1.0, 2.0, 3.0, 4.0, 5.0, 6.0] and shape == [2, 3]


@pytest.mark.parametrize("shape", SHAPES[:9])
def test_oracle_bytes_load_in_numpy(tmp_path, shape):
    v = _values(shape)
    b = npy_ref.write_bytes(v, shape)
    assert (len(b) - len(v) * 4) % 64 == 0
    p = tmp_path / "o.npy"
    p.write_bytes(b)
    a = np.load(p)
    assert list(a.shape) == shape and a.dtype == np.float32
    assert np.array_equal(a.ravel(), v)


@pytest.mark.parametrize("dtype", ["<f4", "<f8"])
@pytest.mark.parametrize("version", [(1, 0), (2, 0), (3, 0)])
def test_oracle_reads_numpy_files(tmp_path, dtype, version):
    a = (np.arange(24, dtype=np.float64).reshape(2, 3, 4) / 7.0).astype(dtype)
    p = tmp_path / "n.npy"
    with open(p, "wb") as f:
        np.lib.format.write_array(f, a, version=version)
    vals, shape = npy_ref.read_bytes(p.read_bytes())
    assert shape == [2, 3, 4]
    assert np.array_equal(np.asarray(vals, np.float32), a.astype(np.float32).ravel())


# ---- the library against the oracle ----

@pytest.mark.parametrize("shape", SHAPES)
def test_writer_bytes_equal_oracle(tmp_path, shape):
    v = _values(shape, 1)
    p = str(tmp_path / "w.npy")
    npy.write_npy_f32(p, v, shape)
    assert open(p, "rb").read() == npy_ref.write_bytes(v, shape)


def test_writer_special_values_and_roundtrip(tmp_path):
    v = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, 3.4028235e38, -1.5], np.float32)
    p = str(tmp_path / "s.npy")
    npy.write_npy_f32(p, v, [2, 4])
    assert open(p, "rb").read() == npy_ref.write_bytes(v, [2, 4])
    back, shape = npy.read_npy_f32(p)
    assert shape == [2, 4]
    assert back.tobytes() == v.tobytes()


def _files(tmp_path):
    """(name, bytes) of valid and invalid NPY files."""
    out = []
    a = np.linspace(-2, 3, 30).astype(np.float32).reshape(5, 6)
    for ver in [(1, 0), (2, 0), (3, 0)]:
        for dt in ["<f4", "<f8"]:
            p = tmp_path / f"np_{ver[0]}_{dt[1:]}.npy"
            with open(p, "wb") as f:
                np.lib.format.write_array(f, a.astype(dt), version=ver)
            out.append((p.name, p.read_bytes()))
    f4 = npy_ref.write_bytes(a.ravel(), [5, 6])
    out.append(("trailing", f4 + struct.pack("<3f", 7.0, 8.0, 9.0) + b"\x01\x02"))
    out.append(("truncated", f4[:-5]))
    out.append(("bad_magic", b"\x93NUMPZ" + f4[6:]))
    out.append(("short", f4[:7]))
    out.append(("empty", b""))

    def custom(header, payload=b""):
        h = header.encode()
        return b"\x93NUMPY\x01\x00" + struct.pack("<H", len(h)) + h + payload

    pay = struct.pack("<4f", 1.0, 2.0, 3.0, 4.0)
    out.append(("fortran", custom("{'descr': '<f4', 'fortran_order': True, 'shape': (2, 2), }\n", pay)))
    out.append(("pipe_f4", custom("{'descr': '|f4', 'fortran_order': False, 'shape': (4,), }\n", pay)))
    out.append(("bare_f4", custom("{'descr': 'f4', 'shape': (4,), 'fortran_order': False}\n", pay)))
    out.append(("big_endian", custom("{'descr': '>f4', 'fortran_order': False, 'shape': (4,), }\n", pay)))
    out.append(("int32", custom("{'descr': '<i4', 'fortran_order': False, 'shape': (4,), }\n", pay)))
    out.append(("pipe_f8", custom("{'descr': '|f8', 'fortran_order': False, 'shape': (2,), }\n", pay)))
    out.append(("no_shape", custom("{'descr': '<f4', 'fortran_order': False}\n", pay)))
    out.append(("no_descr", custom("{'fortran_order': False, 'shape': (4,)}\n", pay)))
    out.append(("bad_dim", custom("{'descr': '<f4', 'shape': (2, x), }\n", pay)))
    out.append(("plus_dim", custom("{'descr': '<f4', 'shape': (+2, 2), }\n", pay)))
    out.append(("huge_dim", custom("{'descr': '<f4', 'shape': (99999999999999999999,), }\n", pay)))
    out.append(("unclosed", custom("{'descr': '<f4', 'shape': (2, 2\n", pay)))
    out.append(("scalar", custom("{'descr': '<f4', 'fortran_order': False, 'shape': (), }\n", pay)))
    out.append(("key_in_string", custom("{'note': \"x 'shape': (9,) y\", 'descr': '<f4', 'shape': (4,), }\n", pay)))
    out.append(("dq_keys", custom('{"descr": "<f4", "shape": (2, 2)}\n', pay)))
    out.append(("spaces", custom("{'descr':   '<f4', 'shape':\t(  2 ,  2 , ) }\n", pay)))
    return out


def test_reader_matches_oracle_on_every_file(tmp_path):
    checked = 0
    for name, b in _files(tmp_path):
        p = tmp_path / f"case_{name}.npy"
        p.write_bytes(b)
        try:
            want = npy_ref.read_bytes(b)
        except npy_ref.NpyError as e:
            with pytest.raises(InvalidState) as got:
                npy.read_npy_f32(str(p))
            if "unclosed" not in str(e):
                assert str(e) == str(got.value), name
            checked += 1
            continue
        vals, shape = npy.read_npy_f32(str(p))
        assert shape == want[1], name
        assert vals.tobytes() == np.asarray(want[0], np.float32).tobytes(), name
        checked += 1
    assert checked == len(_files(tmp_path))


def test_reader_missing_file_is_io_error(tmp_path):
    with pytest.raises(IOError_):
        npy.read_npy_f32(str(tmp_path / "absent.npy"))
    with pytest.raises(IOError_):
        npy.write_npy_f32(str(tmp_path / "no_dir" / "x.npy"), [1.0], [1])


def test_write_tavg_labels_shape_over_node_major_data(tmp_path):
    from hyburn_gb300.config import SimConfig
    toml = """
sim_length = 1.0
dt = 0.1
integrator = "heun"
[network]
[[network.subnetworks]]
model = "Generic2dOscillator"
nnodes = 3
params = [1.0, 0.0, -2.0, -10.0, 0.0, 0.02, 3.0, 1.0, 0.0, 1.0, 1.0, 1.0]
initial_state = [0.0, 0.0, 0.0, 0.0, 0.0, 0.0]
[[network.subnetworks]]
model = "JansenRit"
nnodes = 2
params = [3.25, 22.0, 0.1, 0.05, 6.0, 0.0025, 0.56, 135.0, 1.0, 0.8, 0.25, 0.25, 0.22]
initial_state = [0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0]
"""
    cfg = SimConfig.from_toml_str(toml)

    class R:
        n_sweep = 4
        tavg = [_values([4, 3, 2], 3), _values([4, 2, 6], 4)]

    paths = npy.write_tavg(cfg, R, str(tmp_path / "out" / "deep"))
    assert [os.path.basename(p) for p in paths] == ["tavg_sub0.npy", "tavg_sub1.npy"]
    assert open(paths[0], "rb").read() == npy_ref.write_bytes(R.tavg[0], [4, 2, 3])
    assert open(paths[1], "rb").read() == npy_ref.write_bytes(R.tavg[1], [4, 6, 2])


@pytest.mark.gpu
def test_sweep_writes_tavg_files(tmp_path):
    """run_sweep(output_dir=...) writes, through the library, the files the oracle writes for the
    same result; run_batch_sweep (cli.rs:932-973) does the same from a fresh engine."""
    from cases import single_model
    from hyburn_gb300 import BatchHybridEngine, SweepParam
    cfg = single_model("MontbrioPazoRoxin", 6, "rk4", "Linear", (0.3,), weights="csr", delays="per_edge_long",
                       dt=0.05, seed=2)
    vals = [0.1, 0.2, 0.3]
    eng = BatchHybridEngine.from_config(cfg, 3)
    out = tmp_path / "a" / "b"
    r = eng.run_sweep(SweepParam(0, 4), vals, 40, output_dir=str(out))
    eng.close()
    want = npy_ref.write_bytes(r.tavg[0], [3, 2, 6])
    assert (out / "tavg_sub0.npy").read_bytes() == want
    r2 = npy.run_batch_sweep(cfg, 0, 4, vals, 40, str(tmp_path / "cli"))
    assert (tmp_path / "cli" / "tavg_sub0.npy").read_bytes() == npy_ref.write_bytes(r2.tavg[0], [3, 2, 6])
    assert np.array_equal(r.tavg[0], r2.tavg[0])


def test_reader_matches_oracle_on_generated_headers(tmp_path):
    """Seeded random headers built from the pieces the scanner cares about (keys inside and outside
    string literals, either quote, spacing, tuples with odd entries, descriptors, trailing or
    missing data): the library and the oracle agree on every one, value or error."""
    rng = np.random.default_rng(11)
    keys_descr = ["'<f4'", "'|f4'", "'f4'", "'<f8'", "'>f4'", "'<i4'", '"<f4"', "'<f4", "<f4"]
    shapes = ["(3,)", "(1, 3)", "(3, 1, )", "( 3 )", "(+3,)", "(3,x)", "()", "(1, (3))", "3", "(0,)"]
    noise = ["", " ", "'fortran_order': False, ", "'note': \"'shape': (9,)\", ", "'x': 'y', ", '"q": "\'", ']
    checked = 0
    for k in range(300):
        parts = []
        for _ in range(3):
            if rng.random() < 0.5:
                parts.append(noise[rng.integers(len(noise))])
        q = "'" if rng.random() < 0.8 else '"'
        items = [f"{q}descr{q}: {keys_descr[rng.integers(len(keys_descr))]}, ",
                 f"{q}shape{q}:{' ' * int(rng.integers(0, 3))}{shapes[rng.integers(len(shapes))]}, "]
        if rng.random() < 0.1:
            items.pop(int(rng.integers(2)))
        order = rng.permutation(len(items) + len(parts))
        allp = items + parts
        header = "{" + "".join(allp[i] for i in order) + "}\n"
        h = header.encode()
        n_vals = int(rng.integers(0, 6))
        payload = np.arange(n_vals, dtype=np.float32).tobytes() if rng.random() < 0.7 else \
            np.arange(n_vals, dtype=np.float64).tobytes()
        if rng.random() < 0.1:
            payload += b"\x00\x01"
        b = b"\x93NUMPY" + bytes([1 if rng.random() < 0.7 else 2, 0])
        b += struct.pack("<H", len(h)) if b[6] == 1 else struct.pack("<I", len(h))
        b += h + payload
        p = tmp_path / f"g{k}.npy"
        p.write_bytes(b)
        try:
            want = npy_ref.read_bytes(b)
        except npy_ref.NpyError as e:
            with pytest.raises(InvalidState) as got:
                npy.read_npy_f32(str(p))
            if "unclosed" not in str(e):
                assert str(e) == str(got.value), header
            checked += 1
            continue
        vals, shape = npy.read_npy_f32(str(p))
        assert shape == want[1], header
        assert vals.tobytes() == np.asarray(want[0], np.float32).tobytes(), header
        checked += 1
    assert checked == 300
