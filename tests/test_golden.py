"""The committed golden fixtures (tests/golden/*.npz): inputs and oracle outputs of whole runs.

On the CPU: every case has its fixture, the inputs are still what the seeded generators (or the
reference's example configurations, read through this package's TOML reader) give, the oracle still
gives the stored outputs (bit for bit where the run has no transcendental function; otherwise within
1e-6 relative over the short runs, the room an ulp of the C library's sin/exp/tanh leaves), and the
stored FP32 outputs stay near the FP64 twin.

On the GPU: the CUDA engine, through the C ABI, against the stored FP32 outputs alone (no oracle
runs). Short runs element-wise at each case's tolerance (rel 1e-5 / abs 1e-6; rel 2e-5 for the
1000-node Kuramoto network, whose phase sums go through sin/cos), and bit for bit with the
reference's summation order (HB_RUN_EXACT_SUMS) on the G2DO sweep cases. The reference's example
configurations run for their full length (10 000 to 100 000 steps); there the engine may be no
farther from the FP32 oracle than twice the FP32 oracle's own distance from the FP64 twin, with the
element-wise tolerance as the floor. Kuramoto final phases are compared on the circle.
"""
import glob
import os

import numpy as np
import pytest

from golden.make_golden import CASES, EXAMPLES, REFERENCE_TREE, build_case, difference, load_case, pack_config, path_of

NAMES = sorted(CASES)
# the BOLD signal cancels near rest; compared with the absolute floor of the engine parity tests
BOLD_ATOL = 2e-5


def keys(case, tag=""):
    return sorted(k for k in case.expected if k.split("_")[0] in (f"final{tag}", f"tavg{tag}", f"bold{tag}"))


def check(result, case, rtol, atol, exact=False, bound=None):
    got = {}
    for i in range(len(case.cfg.network.subnetworks)):
        got[f"final_{i}"] = result.final_states[i]
        got[f"tavg_{i}"] = result.tavg[i]
    bold = [k for k in keys(case) if k.startswith("bold_")]
    if bold:
        assert result.bold is not None and len(result.bold) == len(bold), case.name
        for m in range(len(bold)):
            got[f"bold_{m}"] = result.bold[m]
    else:
        assert not result.bold or all(np.asarray(b).size == 0 for b in result.bold), case.name
    for k in keys(case):
        want, have = case.expected[k], np.asarray(got[k])
        assert have.shape == want.shape, (case.name, k, have.shape, want.shape)
        if exact:
            assert np.array_equal(have, want), f"{case.name}: {k} not bit-identical"
            continue
        if not want.size:
            continue
        floor = max(atol, BOLD_ATOL) if k.startswith("bold") else atol
        d = difference(k, have, want, case.cfg)
        if (bound or case.bound) == "fp32":
            limit = max(2.0 * case.drift[k], floor + rtol * float(np.abs(want).max()))
            assert d.max() <= limit, (f"{case.name}: {k} differs from the FP32 oracle by {d.max():.3g}; "
                                      f"the FP32 oracle from FP64 by {case.drift[k]:.3g}")
        else:
            err = d / (floor + rtol * np.abs(want.astype(np.float64)))
            i = int(np.argmax(err))
            assert err.max() <= 1.0, (f"{case.name}: {k} max scaled error {err.max():.3g} at {i}: "
                                      f"got {have.ravel()[i]!r}, golden {want.ravel()[i]!r}")


# ---- CPU ----

def test_every_case_has_its_fixture():
    on_disk = {os.path.basename(p)[:-4] for p in glob.glob(os.path.join(os.path.dirname(path_of("x")), "*.npz"))}
    assert on_disk == set(NAMES)


@pytest.mark.parametrize("name", NAMES)
def test_inputs_are_what_their_source_gives(name):
    if name in EXAMPLES and not os.path.isdir(os.path.join(REFERENCE_TREE, "examples")):
        pytest.skip("the reference's example configurations are not on this machine")
    case, made = load_case(name), build_case(name)
    text0, arr0 = pack_config(case.cfg)
    text1, arr1 = pack_config(made["cfg"])
    assert text0 == text1
    assert sorted(arr0) == sorted(arr1)
    for k in arr0:
        assert np.array_equal(arr0[k], arr1[k]), k
    assert np.array_equal(case.values, np.asarray(made["values"], np.float32))
    assert case.n_steps == made["n_steps"] and case.n_sweep == made["n_sweep"]
    assert (case.param.sub_idx, case.param.param_idx) == (made["param"].sub_idx, made["param"].param_idx)
    assert (case.noise is None) == (made["noise"] is None)
    if case.noise is not None:
        assert np.array_equal(case.noise, made["noise"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_the_fixture(name):
    from oracle.hb_oracle import OracleEngine
    case = load_case(name)
    r = OracleEngine.from_config(case.cfg, case.n_sweep, semantics=case.semantics, n_threads=os.cpu_count()).run_sweep(
        case.param, case.values, case.n_steps, noise=case.noise)
    # short runs within rel 1e-6; the long example runs within their own FP32 error (a C library whose
    # sin/exp differ by an ulp moves a 10^4-step run by no more than FP32 rounding does)
    check(r, case, 1e-6, 1e-7, exact=case.bitwise)


@pytest.mark.parametrize("name", NAMES)
def test_fp32_drift_from_fp64(name):
    """The stored FP32 run against the FP64 twin: the stored drift is the largest difference of the
    stored outputs (short runs), and it stays a small fraction of each output's magnitude."""
    case = load_case(name)
    for k in keys(case):
        want = case.expected[k]
        if k.replace("_", "64_", 1) in case.expected:
            d = difference(k, want, case.expected[k.replace("_", "64_", 1)], case.cfg)
            assert (float(d.max()) if d.size else 0.0) == case.drift[k], (name, k)
        scale = float(np.abs(want).max()) if want.size else 0.0
        assert case.drift[k] <= 5e-3 * scale + 1e-4, (name, k, case.drift[k], scale)


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


@pytest.mark.parametrize("nodes,case", [(76, "refbench_3subnet_76n"), (164, "refbench_3subnet_164n")])
def test_bench_ring3_workload_is_the_golden_case(nodes, case):
    """bench.py's `--workload ring3` line runs the network the golden refbench case checks (its 1024 sweep
    values follow the same formula as the case's fewer). The bench sets the hybrid integrator after
    creation, as the reference's benchmark does; the case creates the engine with the same flag."""
    import bench
    from hyburn_gb300._abi import HB_SEM_HYBRID_INTEGRATOR
    g = load_case(case)
    assert g.semantics == HB_SEM_HYBRID_INTEGRATOR
    cfg, values = bench.ring3_workload(nodes, g.n_sweep, g.n_steps)
    assert pack_config(cfg)[0] == pack_config(g.cfg)[0]
    assert np.array_equal(np.asarray(values, np.float32), g.values)


@pytest.mark.parametrize("model", ["G2DO", "JR", "WC", "MPR"])
def test_bench_single_model_workload_is_the_golden_case(model):
    """bench.py's `--workload single-model` line runs the network the golden refbench_single case checks."""
    import bench
    g = load_case(f"refbench_single_{model.lower()}")
    cfg, (si, pi), values = bench.single_model_workload(model, g.n_sweep, 76)
    assert pack_config(cfg)[0] == pack_config(g.cfg)[0]
    assert (si, pi) == (g.param.sub_idx, g.param.param_idx)
    assert np.array_equal(np.asarray(values, np.float32), g.values)
