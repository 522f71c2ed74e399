"""Host-side logic that needs no GPU: the TOML surface (src/config.rs, src/cli.rs:976-998), the
descriptor validation of hb_engine_create, and the C-ABI library's exported symbols."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from hyburn_gb300 import _abi
from hyburn_gb300.config import (InvalidConfig, InvalidState, SimConfig, SweepConfig, Unsupported, parse_sweep_param,
                                 resolve_initial_state, tract_lengths_to_delays)
from hyburn_gb300.engine import BatchHybridEngine

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

TOML = """
sim_length = 1000.0
dt = 0.1
integrator = "heun_stochastic"
nsig = 0.001

[network]
[[network.subnetworks]]
model = "Generic2dOscillator"
nnodes = 3
params = [1.0, 0.0, -2.0, -10.0, 0.0, 0.02, 3.0, 1.0, 0.0, 1.0, 1.0, 1.0]
initial_state = [0.0, 0.5, 0.1, 0.4, 0.2, 0.3]

[[network.projections]]
src = 0
tgt = 0
coupling_fn = "Linear"
coupling_params = [0.01]
tract_lengths = [10.0, 20.0, 25.0]
weights = { data = [1.0, 0.5, 0.25], indices = [1, 2, 0], indptr = [0, 1, 2, 3] }

[[monitors]]
monitor_type = "Bold"
tr = 2.0
"""


def test_parse_toml_defaults():
    cfg = SimConfig.from_toml_str(TOML)
    assert cfg.integrator == "heun_stochastic" and cfg.speed == 3.0 and cfg.backend == "ndarray"
    p = cfg.network.projections[0]
    assert p.cvar_map == "0:0" and p.conn_type == "all_to_all" and p.delays == []
    assert isinstance(p.weights, dict) and p.weights["indptr"] == [0, 1, 2, 3]
    m = cfg.monitors[0]
    assert m.bold_period == 10 and m.tr == 2.0  # serde defaults (config.rs:245-250)
    assert cfg.nsig_vec(2) == [0.001, 0.001]
    cfg.validate()


def test_resolve_delays_from_tract_lengths():  # config.rs:436-452
    cfg = SimConfig.from_toml_str(TOML)
    cfg.resolve_delays()
    assert cfg.network.projections[0].delays == [34, 67, 84]
    assert tract_lengths_to_delays([10.0], 3.0, 0.1) == [34]


def test_validate_errors():
    cfg = SimConfig.from_toml_str(TOML)
    cfg.network.subnetworks[0].params = cfg.network.subnetworks[0].params[:5]
    with pytest.raises(InvalidConfig, match="expects 12 params, got 5"):
        cfg.validate()
    cfg = SimConfig.from_toml_str(TOML.replace("indptr = [0, 1, 2, 3]", "indptr = [0, 1, 3]"))
    with pytest.raises(InvalidConfig, match="CSR indptr length"):
        cfg.validate()
    with pytest.raises(InvalidConfig, match="TOML parse error"):
        SimConfig.from_toml_str("sim_length = [")


def test_parse_sweep_param():  # cli.rs:976-998
    cfg = SimConfig.from_toml_str(TOML)
    assert parse_sweep_param("subnetworks[0].params[1]", cfg) == (0, 1)
    for bad, msg in (("dt", "does not support sweeping dt"), ("subnetworks[3].params[1]", "out of range"),
                     ("coupling.a", "unsupported sweep parameter_name")):
        with pytest.raises(InvalidConfig, match=msg):
            parse_sweep_param(bad, cfg)


def test_sweep_config_range():  # config.rs:486-502
    v = SweepConfig("x", range={"start": 0.0, "step": 0.25, "end": 1.0}).generate_values()
    assert v == [0.0, 0.25, 0.5, 0.75, 1.0]
    assert SweepConfig("x", values=[1, 2]).generate_values() == [1.0, 2.0]
    assert SweepConfig("x", range={"start": 0.0, "step": 0.0, "end": 1.0}).generate_values() == []


def test_initial_state_npy_layouts(tmp_path):  # engine.rs:175-237
    from hyburn_gb300.config import SubnetworkConfig
    a = np.arange(6, dtype=np.float32).reshape(2, 3)  # [nvar, nnodes]
    p = tmp_path / "init.npy"
    np.save(p, a)
    s = SubnetworkConfig("Generic2dOscillator", 3, str(p), [0.0] * 12)
    assert resolve_initial_state(s).tolist() == [0, 3, 1, 4, 2, 5]
    s.nmodes = 2
    assert resolve_initial_state(s).tolist() == [0, 3, 1, 4, 2, 5] * 2
    # [nvar, nnodes, nmodes]: the reference reads data[(v * nnodes * n) * nmodes + m] (engine.rs:207)
    b = np.arange(6, dtype=np.float32).reshape(1, 3, 2)
    np.save(p, b)
    s1 = SubnetworkConfig("Kuramoto", 3, str(p), [1.0], nmodes=2)
    assert resolve_initial_state(s1).tolist() == [0.0, 1.0] * 3
    np.save(p, np.arange(12, dtype=np.float32).reshape(2, 3, 2))
    with pytest.raises(InvalidState, match="out of bounds"):
        resolve_initial_state(s)


# ---- C-ABI library ----

def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "hyburn_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _abi.load_library()
    names = _declared_symbols()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    assert lib.hb_abi_version() == _abi.HB_ABI_VERSION


def test_model_info():
    lib = _abi.load_library()
    nv, nc, npar = C.c_int32(), C.c_int32(), C.c_int32()
    assert lib.hb_model_info(b"JansenRit", C.byref(nv), C.byref(nc), C.byref(npar)) == 0
    assert (nv.value, nc.value, npar.value) == (6, 1, 13)
    assert lib.hb_model_info(b"Epileptor", C.byref(nv), C.byref(nc), C.byref(npar)) == 0
    assert lib.hb_model_info(b"Nope", C.byref(nv), C.byref(nc), C.byref(npar)) == _abi.HB_ERR_INVALID_CONFIG
    assert b"Unknown model" in lib.hb_last_error()


def _cfg_with(**kw):
    cfg = SimConfig.from_toml_str(TOML)
    for k, v in kw.items():
        setattr(cfg.network.subnetworks[0], k, v)
    return cfg


def test_create_rejects_invalid_descriptors_before_touching_the_gpu():
    with pytest.raises(InvalidConfig, match="Unknown model"):
        BatchHybridEngine.from_config(_cfg_with(model="NotAModel"), 2)
    with pytest.raises(Unsupported, match="not batch-native"):
        BatchHybridEngine.from_config(_cfg_with(model="Epileptor", params=[0.0] * 17, initial_state=[0.0] * 18), 2)
    with pytest.raises(InvalidConfig, match="expects 12 params"):
        BatchHybridEngine.from_config(_cfg_with(params=[1.0] * 3), 2)
    with pytest.raises(InvalidConfig, match="initial_state has 4 values"):
        BatchHybridEngine.from_config(_cfg_with(initial_state=[0.0] * 4), 2)
    bad = SimConfig.from_toml_str(TOML.replace("indices = [1, 2, 0]", "indices = [1, 7, 0]"))
    with pytest.raises(InvalidConfig, match="CSR index 7"):
        BatchHybridEngine.from_config(bad, 2)
    cm = SimConfig.from_toml_str(TOML)
    cm.network.projections[0].cvar_map = "1:0"
    with pytest.raises(InvalidConfig, match="cvar_map src index 1"):
        BatchHybridEngine.from_config(cm, 2)
    gt = SimConfig.from_toml_str(TOML)
    gt.network.projections[0].coupling_fn = "PreSigmoidal"
    gt.network.projections[0].coupling_params = [1, 1, 1, 1, 0.5, 1, 1]
    with pytest.raises(Unsupported, match="global_t"):
        BatchHybridEngine.from_config(gt, 2)


def test_new_entry_points_reject_null_arguments_without_a_gpu():
    """NPY, tavg, feature and adjoint entry points validate their arguments before any CUDA call."""
    lib = _abi.load_library()
    assert lib.hb_npy_write_f32(None, None, None, 0) == _abi.HB_ERR_INVALID_STATE
    assert lib.hb_npy_read_f32(None, None, 0, None, 0, None, None) == _abi.HB_ERR_INVALID_STATE
    assert lib.hb_engine_write_tavg(None, None, b"x") == _abi.HB_ERR_INVALID_STATE
    out = _abi.hb_fc_features()
    assert lib.hb_engine_fc_features(None, 0, 0, 1, C.byref(out)) == _abi.HB_ERR_INVALID_STATE
    oa = _abi.hb_order_adjoint_out()
    assert lib.hb_engine_adjoint_order(None, None, 0, 10, 0, C.byref(oa)) == _abi.HB_ERR_INVALID_STATE
    assert lib.hb_engine_set_hybrid_integrator(None, 1) == _abi.HB_ERR_INVALID_STATE
    assert b"NULL" in lib.hb_last_error() or b"null" in lib.hb_last_error()


def test_run_flag_macros_match_the_header():
    """The Python mirror's run-flag helpers give the same bits as the C header's macros: the header
    is compiled with a one-line C program per value (gcc, no GPU)."""
    import os
    import subprocess
    import tempfile
    from hyburn_gb300 import _abi
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    cases = [("HB_RUN_STREAM_CLUSTER", c, _abi.HB_RUN_STREAM_CLUSTER(c)) for c in (1, 2, 3, 4, 5, 6, 8)]
    cases += [("HB_RUN_STREAM_NPT", n, _abi.HB_RUN_STREAM_NPT(n)) for n in (1, 2, 4)]
    cases += [("HB_RUN_PIPE_LANES", n, _abi.HB_RUN_PIPE_LANES(n)) for n in (1, 2, 4, 8)]
    src = "#include <stdio.h>\n#include \"hyburn_gb300.h\"\nint main(void) {\n"
    src += "".join(f'  printf("%u\\n", (unsigned){m}({v}));\n' for m, v, _ in cases) + "  return 0;\n}\n"
    with tempfile.TemporaryDirectory() as d:
        c_path, exe = os.path.join(d, "flags.c"), os.path.join(d, "flags")
        with open(c_path, "w") as f:
            f.write(src)
        subprocess.run(["gcc", "-std=c99", "-I", inc, c_path, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    assert [int(x) for x in out] == [py for _, _, py in cases]
    # distinct codes for the distinct cluster sizes
    codes = [_abi.HB_RUN_STREAM_CLUSTER(c) for c in (1, 2, 3, 4, 5, 6, 8)]
    assert len(set(codes)) == len(codes) and 0 not in codes


def _two_subnets(n0=4, n1=3, weights=0.5, conn="all_to_all", src=0, tgt=1, nmodes=1, params=None, x0=None):
    from hyburn_gb300.config import NetworkConfig, ProjectionConfig, SubnetworkConfig
    g = [1.0, 0.0, -2.0, -10.0, 0.0, 0.02, 3.0, 1.0, 0.0, 1.0, 1.0, 1.0]
    subs = [SubnetworkConfig("Generic2dOscillator", n0, x0 if x0 is not None else [0.1] * (2 * n0 * nmodes),
                             params or g, nmodes=nmodes),
            SubnetworkConfig("Generic2dOscillator", n1, [0.1] * (2 * n1), g)]
    return SimConfig(sim_length=10.0, dt=0.1, network=NetworkConfig(
        subs, [ProjectionConfig(src, tgt, weights, conn_type=conn, coupling_fn="Linear", coupling_params=[0.1])]))


@pytest.mark.parametrize("case,semantics", [
    ("nmodes", 0), ("params", 0), ("initial_state", 0), ("src", 0), ("scalar_sizes", _abi.HB_SEM_SCALAR_DIAGONAL),
    ("dense_rows", 0), ("csr_indptr", 0)])
def test_boundary_errors_carry_the_reference_messages(case, semantics):
    """Where hb_engine_create checks what SimConfig::validate checks (config.rs:286-429), a C caller gets
    the same error kind and text that validate gives (here through the Python mirror's validate)."""
    cfg = {
        "nmodes": lambda: _two_subnets(nmodes=0, x0=[0.1] * 8),
        "params": lambda: _two_subnets(params=[1.0] * 3),
        "initial_state": lambda: _two_subnets(x0=[0.1] * 5),
        "src": lambda: _two_subnets(src=3),
        "scalar_sizes": lambda: _two_subnets(weights=0.5),
        "dense_rows": lambda: _two_subnets(weights=[[1.0] * 4] * 2),
        "csr_indptr": lambda: _two_subnets(weights={"data": [1.0], "indices": [0], "indptr": [0, 1]}, conn="csr"),
    }[case]()
    with pytest.raises(InvalidConfig) as want:
        cfg.validate()
    with pytest.raises(InvalidConfig) as got:
        BatchHybridEngine.from_config(cfg, 2, semantics=semantics)
    assert str(got.value) == str(want.value)


def test_last_error_is_per_thread():
    """hb_last_error() is the calling thread's message (the header's contract): two threads set different
    errors, then each reads its own after the other has set its."""
    import threading
    lib = _abi.load_library()
    gate = threading.Barrier(2)
    got = {}

    def worker(name):
        nv, nc, npar = C.c_int32(), C.c_int32(), C.c_int32()
        assert lib.hb_model_info(name.encode(), C.byref(nv), C.byref(nc), C.byref(npar)) == _abi.HB_ERR_INVALID_CONFIG
        gate.wait()  # both errors are set
        gate.wait()
        got[name] = lib.hb_last_error().decode()

    ts = [threading.Thread(target=worker, args=(n,)) for n in ("ModelOfThreadA", "ModelOfThreadB")]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert "ModelOfThreadA" in got["ModelOfThreadA"] and "ModelOfThreadB" not in got["ModelOfThreadA"]
    assert "ModelOfThreadB" in got["ModelOfThreadB"] and "ModelOfThreadA" not in got["ModelOfThreadB"]
