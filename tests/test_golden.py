"""The committed golden fixtures (tests/golden/*.npz): inputs and oracle outputs of whole runs.

On the CPU: every case has its fixture, the seeded generators still give the stored inputs, and the
oracle still gives the stored outputs (bit for bit where the run has no transcendental function;
otherwise within 1e-6 relative, the room an ulp of the C library's sin/exp/tanh leaves over a few
hundred steps). On the GPU: the CUDA engine, through the C ABI, against the stored FP32 outputs
alone (no oracle runs), at each case's tolerance (rel 1e-5 / abs 1e-6; rel 2e-5 for the
1000-node Kuramoto network, whose phase sums go through sin/cos), and bit for bit with the
reference's summation order (HB_RUN_EXACT_SUMS) on the G2DO sweep cases.
"""
import glob
import os

import numpy as np
import pytest

from golden.make_golden import CASES, build_case, load_case, pack_config, path_of

NAMES = sorted(CASES)
# the BOLD signal cancels near rest; compared with the absolute floor of the engine parity tests
BOLD_ATOL = 2e-5


def close(a, b, rtol, atol, what):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    err = np.abs(a - b) / (atol + rtol * np.abs(b))
    i = int(np.argmax(err)) if err.size else 0
    assert err.size == 0 or err.max() <= 1.0, \
        f"{what}: max scaled error {err.max():.3g} at {i}: got {a.ravel()[i]!r}, golden {b.ravel()[i]!r}"


def outputs(case, tag=""):
    e = case.expected
    fin = [e[f"final{tag}_{i}"] for i in range(len(case.cfg.network.subnetworks))]
    tavg = [e[f"tavg{tag}_{i}"] for i in range(len(case.cfg.network.subnetworks))]
    bold = [e[k] for k in sorted(e) if k.startswith(f"bold{tag}_") and k[len(f"bold{tag}_"):].isdigit()]
    return fin, tavg, bold


def check(result, case, rtol, atol, exact=False):
    fin, tavg, bold = outputs(case)
    for i in range(len(fin)):
        if exact:
            assert np.array_equal(result.final_states[i], fin[i]), f"{case.name}: final[{i}] not bit-identical"
            assert np.array_equal(result.tavg[i], tavg[i]), f"{case.name}: tavg[{i}] not bit-identical"
        else:
            close(result.final_states[i], fin[i], rtol, atol, f"{case.name}: final[{i}]")
            close(result.tavg[i], tavg[i], rtol, atol, f"{case.name}: tavg[{i}]")
    if bold:
        assert result.bold is not None and len(result.bold) == len(bold)
        for m, b in enumerate(bold):
            close(result.bold[m], b, rtol, max(atol, BOLD_ATOL), f"{case.name}: bold[{m}]")
    else:
        assert not result.bold or all(np.asarray(b).size == 0 for b in result.bold)


# ---- CPU ----

def test_every_case_has_its_fixture():
    on_disk = {os.path.basename(p)[:-4] for p in glob.glob(os.path.join(os.path.dirname(path_of("x")), "*.npz"))}
    assert on_disk == set(NAMES)


@pytest.mark.parametrize("name", NAMES)
def test_generators_give_the_stored_inputs(name):
    case, made = load_case(name), build_case(name)
    text0, arr0 = pack_config(case.cfg)
    text1, arr1 = pack_config(made["cfg"])
    assert text0 == text1
    assert sorted(arr0) == sorted(arr1)
    for k in arr0:
        assert np.array_equal(arr0[k], arr1[k]), k
    assert np.array_equal(case.values, np.asarray(made["values"], np.float32))
    assert case.n_steps == made["n_steps"] and case.n_sweep == made["n_sweep"]
    assert (case.noise is None) == (made["noise"] is None)
    if case.noise is not None:
        assert np.array_equal(case.noise, made["noise"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_the_fixture(name):
    from oracle.hb_oracle import OracleEngine
    case = load_case(name)
    r = OracleEngine.from_config(case.cfg, case.n_sweep, semantics=case.semantics).run_sweep(
        case.param, case.values, case.n_steps, noise=case.noise)
    check(r, case, 1e-6, 1e-7, exact=case.bitwise)


@pytest.mark.parametrize("name", NAMES)
def test_fp32_drift_from_fp64_is_small(name):
    """The stored FP32 run stays close to the FP64 twin over these short runs (the per-configuration
    drift over the workloads' full lengths is measured by tests/fp64_drift.py)."""
    case = load_case(name)
    f32, t32, _ = outputs(case)
    f64, t64, _ = outputs(case, "64")
    for a, b in zip(f32 + t32, f64 + t64):
        close(a, b, 1e-3, 1e-4, f"{name}: FP32 vs FP64")


# ---- GPU: the CUDA engine against the stored outputs ----

@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_engine_matches_the_golden_outputs(name):
    from hyburn_gb300 import BatchHybridEngine
    from hyburn_gb300._abi import HB_RUN_EXACT_SUMS
    case = load_case(name)
    eng = BatchHybridEngine.from_config(case.cfg, case.n_sweep, semantics=case.semantics)
    g = eng.run_sweep(case.param, case.values, case.n_steps, noise=case.noise)
    check(g, case, case.rtol, case.atol)
    if case.bitwise:
        eng.reset()
        ex = eng.run_sweep(case.param, case.values, case.n_steps, noise=case.noise, run_flags=HB_RUN_EXACT_SUMS)
        check(ex, case, case.rtol, case.atol, exact=True)
    eng.close()
