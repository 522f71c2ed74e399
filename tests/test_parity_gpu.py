"""Parity of the CUDA engine with the CPU oracle, through the C ABI, on seeded inputs.

Tolerance: |gpu - oracle| <= 1e-6 + 1e-5 * |oracle| element-wise (the FP32 relative bound of the
parity contract). Both sides evaluate the same operations in the same order without fused
multiply-adds; remaining differences come from transcendental functions (CUDA vs C library,
<= 2 ulp) and from the order of mean-field / batch-mean reductions.
"""
import numpy as np
import pytest

from hyburn_gb300 import BatchHybridEngine, SweepParam, SweepPoint, SweepSpec
from hyburn_gb300._abi import (HB_RUN_GENERIC, HB_RUN_GLOBAL_RING, HB_RUN_LANES, HB_RUN_NO_PIPE, HB_RUN_PIPE_LANES,
                               HB_RUN_TWO_PHASE, HB_SEM_BOLD_PER_POINT, HB_SEM_DELAY_RING,
                               HB_SEM_HYBRID_INTEGRATOR, HB_SEM_NOISE_PER_POINT, HB_SEM_SCALAR_DIAGONAL)
from hyburn_gb300.config import InvalidConfig, InvalidState, MonitorConfig, NetworkConfig, ProjectionConfig, SimConfig
from oracle.hb_oracle import OracleEngine

from cases import NATIVE_SWEEP, noise_for, single_model, sub, sweep_values, three_subnet_ring

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-5, 1e-6
# The BOLD signal V0*(k1*(1-q) + k2*(1-q/v) + k3*(1-v)) cancels near rest: one ulp of q or v is about
# V0*k1*6e-8 = 1.7e-6 in signal units, so BOLD series are compared with an absolute floor of
# 2e-5 (about ten ulps of the Balloon-Windkessel state) on top of the relative bound.
BOLD_ATOL = 2e-5
MODELS = ["Generic2dOscillator", "MontbrioPazoRoxin", "ReducedWongWang", "Kuramoto", "JansenRit", "WilsonCowan"]
INTEGRATORS = ["heun", "euler", "euler_stochastic", "heun_stochastic", "rk4", "rk4_stochastic"]


def close(a, b, rtol=RTOL, atol=ATOL, what=""):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    assert np.isfinite(b).all(), f"{what}: oracle produced non-finite values"
    err = np.abs(a - b) / (atol + rtol * np.abs(b))
    i = int(np.argmax(err)) if err.size else 0
    assert err.size == 0 or err.max() <= 1.0, f"{what}: max scaled error {err.max():.3g} at {i}: gpu={a.ravel()[i]!r} oracle={b.ravel()[i]!r}"


def compare(cfg, n_sweep, param, values, n_steps, semantics=0, noise=None, run_flags=0, traj=False, rtol=RTOL,
            atol=ATOL, multi=None):
    eng = BatchHybridEngine.from_config(cfg, n_sweep, semantics=semantics)
    ora = OracleEngine.from_config(cfg, n_sweep, semantics=semantics)
    if multi is not None:
        g = eng.run_sweep_multi(multi, n_steps, noise=noise, run_flags=run_flags | (1 if traj else 0))
        o = ora.run_sweep_multi(multi, n_steps, noise=noise, run_flags=(1 if traj else 0))
    else:
        f = 1 if traj else 0
        g = eng.run_sweep(param, values, n_steps, noise=noise, run_flags=run_flags | f)
        o = ora.run_sweep(param, values, n_steps, noise=noise, run_flags=f)
    for i in range(len(o.tavg)):
        close(g.final_states[i], o.final_states[i], rtol, atol, f"final[{i}]")
        close(g.tavg[i], o.tavg[i], rtol, atol, f"tavg[{i}]")
        if traj:
            close(g.trajectories[i], o.trajectories[i], rtol, atol, f"traj[{i}]")
    if o.bold is not None:
        assert g.bold is not None and len(g.bold) == len(o.bold)
        for m in range(len(o.bold)):
            close(g.bold[m], o.bold[m], rtol, max(atol, BOLD_ATOL), f"bold[{m}]")
    else:
        assert g.bold is None
    assert np.allclose(g.param_values, o.param_values)
    assert eng.step == ora.step
    return eng, ora, g, o


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("integrator", INTEGRATORS)
def test_models_integrators_mean_field(model, integrator):
    """Scalar all-to-all coupling (w * mean over source nodes), native sweep parameter."""
    cfg = single_model(model, 20, integrator, "Linear", (0.05,), nsig=1e-4)
    nz = noise_for(cfg, 120, 4, False, 3) if "stochastic" in integrator else None
    compare(cfg, 4, SweepParam(0, NATIVE_SWEEP[model]), sweep_values(model, 4), 120, noise=nz)


@pytest.mark.parametrize("coupling,cparams,model", [
    ("Linear", (0.1, 0.01), "Generic2dOscillator"),
    ("Sigmoidal", (-1.0, 1.0, 0.0, 1.0, 1.0), "Generic2dOscillator"),
    ("Sigmoidal", (1.0, 0.0, 2.0), "WilsonCowan"),
    ("Difference", (0.1,), "Generic2dOscillator"),
    ("Kuramoto", (1.0,), "Kuramoto"),
    ("ScaledLinear", (0.2, 0.1), "ReducedWongWang"),
    ("HyperbolicTangent", (0.1, 1.0, 0.2, 2.0), "Generic2dOscillator"),
    ("SigmoidalJansenRit", (1.0, 0.005, 0.56, 6.0), "JansenRit"),
    ("SigmoidalJansenRit", (2.0, 0.0, 0.01, 0.56, 6.0), "JansenRit"),
    ("PreSigmoidal", (0.1, 0.5, 1.0, 1.0, 0.5), "Generic2dOscillator"),
    ("Linear", (0.1,), "MontbrioPazoRoxin"),
    ("NotACouplingFunction", (), "Generic2dOscillator"),
])
@pytest.mark.parametrize("weights", ["scalar", "dense", "csr"])
@pytest.mark.parametrize("generic", [False, True])
def test_coupling_functions(coupling, cparams, model, weights, generic):
    """generic=True forces the general resident kernel for networks the specialised kernel serves."""
    cfg = single_model(model, 16, "heun", coupling, cparams, weights=weights)
    compare(cfg, 3, SweepParam(0, NATIVE_SWEEP[model]), sweep_values(model, 3), 100,
            run_flags=HB_RUN_GENERIC if generic else 0)


@pytest.mark.parametrize("weights", ["scalar", "dense", "csr"])
@pytest.mark.parametrize("delay", [1, 3, 7])
def test_compat_single_delay_shift_window(weights, delay):
    """engine.rs:541-589: one delay per projection read from the shift-window history."""
    cfg = single_model("Generic2dOscillator", 12, "heun", "Linear", (0.3,), weights=weights, delays=[delay])
    compare(cfg, 2, SweepParam(0, 1), [0.0, 0.2], 60, traj=True)


def test_compat_two_delays_share_horizon():
    cfg = three_subnet_ring(10, "heun", delays=(2, 5, 0))
    compare(cfg, 3, SweepParam(1, 12), [0.1, 0.2, 0.3], 80)


@pytest.mark.parametrize("weights", ["scalar", "dense", "csr"])
def test_ring_single_delay(weights):
    cfg = single_model("MontbrioPazoRoxin", 12, "rk4", "Linear", (0.2,), weights=weights, delays=[4], dt=0.05)
    compare(cfg, 2, SweepParam(0, 4), [0.0, 0.5], 80, semantics=HB_SEM_DELAY_RING)


@pytest.mark.parametrize("model,coupling,cparams", [
    ("Generic2dOscillator", "Linear", (0.1,)),
    ("Kuramoto", "Kuramoto", (2.0,)),
    ("JansenRit", "SigmoidalJansenRit", (2.0, 0.0, 0.01, 0.56, 6.0)),
    ("MontbrioPazoRoxin", "Linear", (0.5,)),
    ("WilsonCowan", "HyperbolicTangent", (0.2, 1.0, 0.0, 1.0)),
])
@pytest.mark.parametrize("variant", ["generic", "per_step", "two_phase", "pipeline"])
def test_ring_per_edge_delays(model, coupling, cparams, variant):
    """runtime.rs:125-211: CSR with one delay per edge, zero rows after pre()."""
    long = variant == "pipeline"
    cfg = single_model(model, 24, "heun", coupling, cparams, weights="csr",
                       delays="per_edge_long" if long else "per_edge", density=0.3)
    flags = {"generic": HB_RUN_GENERIC, "per_step": HB_RUN_NO_PIPE, "two_phase": HB_RUN_TWO_PHASE,
             "pipeline": 0}[variant]
    compare(cfg, 3, SweepParam(0, NATIVE_SWEEP[model]), sweep_values(model, 3), 400 if long else 150,
            semantics=HB_SEM_DELAY_RING, traj=True, run_flags=flags)


def test_ring_per_edge_global_ring_matches_shared_ring():
    cfg = single_model("Generic2dOscillator", 24, "heun_stochastic", "Linear", (0.2,), weights="csr",
                       delays="per_edge", nsig=1e-3)
    nz = noise_for(cfg, 100, 3, False, 9)
    e1, _, g1, _ = compare(cfg, 3, SweepParam(-1, 0), [0.0, 0.1, 0.2], 100, semantics=HB_SEM_DELAY_RING, noise=nz)
    e2 = BatchHybridEngine.from_config(cfg, 3, semantics=HB_SEM_DELAY_RING)
    g2 = e2.run_sweep(SweepParam(-1, 0), [0.0, 0.1, 0.2], 100, noise=nz, run_flags=HB_RUN_GLOBAL_RING)
    assert np.array_equal(g1.final_states[0], g2.final_states[0])


@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
@pytest.mark.parametrize("semantics", [0, HB_SEM_DELAY_RING])
def test_lane_split_gather(lanes, semantics):
    """The edge list of a node split over 1-8 lanes gives the oracle's coupling (summation order
    differs only by the final lane combine)."""
    cfg = single_model("Kuramoto", 30, "heun", "Kuramoto", (1.5,), weights="csr", delays="per_edge"
                       if semantics else [3], density=0.5)
    compare(cfg, 3, SweepParam(0, 0), [0.8, 1.0, 1.2], 120, semantics=semantics, run_flags=HB_RUN_LANES(lanes))
    cfg = single_model("MontbrioPazoRoxin", 30, "rk4", "Linear", (0.3,), weights="csr", delays="per_edge"
                       if semantics else [2], density=0.5, dt=0.05)
    compare(cfg, 2, SweepParam(0, 4), [0.0, 0.5], 120, semantics=semantics, run_flags=HB_RUN_LANES(lanes))


@pytest.mark.parametrize("flags", [0, HB_RUN_PIPE_LANES(1), HB_RUN_PIPE_LANES(4), HB_RUN_NO_PIPE, HB_RUN_TWO_PHASE,
                                   HB_RUN_TWO_PHASE | HB_RUN_LANES(1), HB_RUN_LANES(2), HB_RUN_GENERIC])
def test_coupling_sweep_batched_workload_small(flags):
    """The batched-sweep workload (coupling scale sweep, per-edge delays, Heun-stochastic), 16 points,
    across the specialised kernel's loop shapes (barriers every K <= min-delay steps)."""
    from hyburn_gb300 import inputs
    cfg, meta = inputs.batched_sweep(n_steps=900, n_points=16)
    nz = inputs.standard_normal((900, 74 * 2), 4)
    compare(cfg, 16, SweepParam(-1, 0), meta["values"], 900, semantics=HB_SEM_DELAY_RING, noise=nz, run_flags=flags,
            traj=True)


def test_three_subnet_ring_with_noise_per_point():
    # nsig is sized by the first subnetwork's nvar (engine.rs:451-452): JansenRit (6 vars) goes first
    cfg = three_subnet_ring(12, "heun_stochastic", delays=(0, 0, 0))
    net = cfg.network
    net.subnetworks = [net.subnetworks[1], net.subnetworks[2], net.subnetworks[0]]
    remap = {1: 0, 2: 1, 0: 2}
    for p in net.projections:
        p.src, p.tgt = remap[p.src], remap[p.tgt]
    cfg.nsig = 1e-4
    nz = noise_for(cfg, 60, 3, True, 5)
    compare(cfg, 3, SweepParam(2, 1), [0.0, 0.1, 0.2], 60, semantics=HB_SEM_NOISE_PER_POINT, noise=nz)


def test_stochastic_subnetwork_wider_than_nsig_is_rejected():
    cfg = three_subnet_ring(12, "heun_stochastic")
    cfg.nsig = 1e-4
    nz = noise_for(cfg, 10, 2, False, 5)
    eng = BatchHybridEngine.from_config(cfg, 2)
    with pytest.raises(InvalidConfig, match="nsig has 2 entries"):
        eng.run_sweep(SweepParam(0, 1), [0.0, 0.1], 10, noise=nz)


def test_mpr_to_kuramoto_cvar_remap():
    subs = [sub("MontbrioPazoRoxin", 8, 1), sub("Kuramoto", 8, 2)]
    projs = [ProjectionConfig(0, 1, 0.5, coupling_fn="Linear", coupling_params=[0.3], cvar_map="1:0"),
             ProjectionConfig(1, 0, 0.4, coupling_fn="Linear", coupling_params=[0.2], cvar_map="0:1"),
             ProjectionConfig(0, 0, 0.3, coupling_fn="Linear", coupling_params=[0.1], cvar_map="0:0,1:1")]
    cfg = SimConfig(sim_length=10.0, dt=0.05, integrator="rk4", network=NetworkConfig(subs, projs))
    compare(cfg, 2, SweepParam(1, 0), [0.8, 1.2], 100)


def test_difference_non_square_rowsums():
    subs = [sub("Generic2dOscillator", 6, 1), sub("Generic2dOscillator", 9, 2)]
    w = np.random.default_rng(3).uniform(0, 1, (9, 6)).astype(np.float32).tolist()
    projs = [ProjectionConfig(0, 1, w, coupling_fn="Difference", coupling_params=[0.05])]
    cfg = SimConfig(sim_length=10.0, dt=0.1, integrator="heun", network=NetworkConfig(subs, projs))
    compare(cfg, 2, SweepParam(1, 1), [0.0, 0.3], 80)


def test_scalar_diagonal_and_hybrid_integrator():
    cfg = three_subnet_ring(8, "heun")
    compare(cfg, 2, SweepParam(0, 1), [0.0, 0.2], 60, semantics=HB_SEM_SCALAR_DIAGONAL | HB_SEM_HYBRID_INTEGRATOR)


def test_hybrid_integrator_set_after_creation():
    """`engine.hybrid_integrator = true` after from_config, as the reference's callers do
    (examples/bench/hyburn_bench_generic_cuda.rs:54): the same run as an engine created with the flag
    (bit for bit) and as the oracle's; set back to false, the configured RK4 again."""
    cfg = three_subnet_ring(8, "rk4")
    p, v = SweepParam(0, 1), [0.0, 0.2]
    eng = BatchHybridEngine.from_config(cfg, 2)
    assert eng.hybrid_integrator is False
    eng.hybrid_integrator = True
    a = eng.run_sweep(p, v, 60)
    b = BatchHybridEngine.from_config(cfg, 2, semantics=HB_SEM_HYBRID_INTEGRATOR).run_sweep(p, v, 60)
    o = OracleEngine.from_config(cfg, 2, semantics=HB_SEM_HYBRID_INTEGRATOR).run_sweep(p, v, 60)
    for i in range(3):
        assert np.array_equal(a.final_states[i], b.final_states[i]) and np.array_equal(a.tavg[i], b.tavg[i])
        close(a.final_states[i], o.final_states[i], what=f"hybrid final[{i}]")
    eng.reset()
    eng.hybrid_integrator = False
    c = eng.run_sweep(p, v, 60)
    d = BatchHybridEngine.from_config(cfg, 2).run_sweep(p, v, 60)
    for i in range(3):
        assert np.array_equal(c.final_states[i], d.final_states[i])


@pytest.mark.parametrize("per_point", [False, True])
@pytest.mark.parametrize("tr,period,n_steps", [(0.002, 10, 250), (0.0015, 10, 257), (0.001, 10, 200), (0.0025, 7, 101)])
def test_bold_monitor(per_point, tr, period, n_steps):
    """bold_monitor.rs:72-227: window mean, BW Euler step, flush of a partial window, TR interpolation."""
    mons = [MonitorConfig("Bold", tr=tr, bold_period=period)]
    cfg = single_model("Generic2dOscillator", 10, "heun", "Linear", (0.1,), monitors=mons)
    sem = HB_SEM_BOLD_PER_POINT if per_point else 0
    compare(cfg, 3, SweepParam(0, 1), [0.0, 0.5, 1.0], n_steps, semantics=sem)


def test_bold_two_monitors_and_consecutive_runs():
    mons = [MonitorConfig("Bold", tr=0.002, bold_period=10), MonitorConfig("Bold", tr=0.0007, bold_period=3)]
    cfg = single_model("WilsonCowan", 10, "rk4", "Linear", (0.5,), monitors=mons)
    eng = BatchHybridEngine.from_config(cfg, 2)
    ora = OracleEngine.from_config(cfg, 2)
    for n in (95, 55, 10):
        g = eng.run_sweep(SweepParam(0, 18), [0.0, 0.5], n)
        o = ora.run_sweep(SweepParam(0, 18), [0.0, 0.5], n)
        for m in range(2):
            close(g.bold[m], o.bold[m], atol=BOLD_ATOL, what=f"bold[{m}] after {n}")
        close(g.final_states[0], o.final_states[0], what="state")


def test_multi_sweep_fallback_and_native():
    cfg = single_model("Generic2dOscillator", 10, "heun", "Linear", (0.1,),
                       monitors=[MonitorConfig("Bold", tr=0.002, bold_period=10)])
    spec = SweepSpec([SweepPoint(0, 1, [-0.5, 0.5]), SweepPoint(0, 9, [0.5, 1.0, 2.0])])
    eng, ora, g, o = compare(cfg, 6, None, None, 80, multi=spec, traj=True)
    # like the reference, the multi run drops the BOLD monitors and keeps its state for the next run
    g2 = eng.run_sweep(SweepParam(0, 1), [0.0] * 6, 20)
    o2 = ora.run_sweep(SweepParam(0, 1), [0.0] * 6, 20)
    assert g2.bold is None and o2.bold is None
    close(g2.final_states[0], o2.final_states[0], what="after multi")
    spec1 = SweepSpec([SweepPoint(0, 1, [-0.5, 0.0, 0.5])])
    compare(cfg, 3, None, None, 50, multi=spec1)


def test_multi_sweep_with_coupling_dimension():
    cfg = single_model("Kuramoto", 16, "rk4", "Kuramoto", (1.0,), weights="csr")
    spec = SweepSpec([SweepPoint(-1, 0, [0.5, 2.0]), SweepPoint(0, 0, [0.9, 1.1])])
    compare(cfg, 4, None, None, 120, multi=spec)


def test_consecutive_runs_continue_state_and_history():
    cfg = single_model("Generic2dOscillator", 12, "heun", "Linear", (0.3,), weights="csr", delays=[5])
    eng = BatchHybridEngine.from_config(cfg, 2)
    ora = OracleEngine.from_config(cfg, 2)
    for n in (7, 13, 1):
        g = eng.run_sweep(SweepParam(0, 1), [0.0, 0.3], n)
        o = ora.run_sweep(SweepParam(0, 1), [0.0, 0.3], n)
        close(g.final_states[0], o.final_states[0], what=f"run of {n}")
        close(g.tavg[0], o.tavg[0], what=f"tavg of {n}")
    assert eng.step == 21


def test_large_point_1000_nodes():
    """Kuramoto, 1000 nodes per point (one 1024-thread CTA per point)."""
    from hyburn_gb300 import inputs
    cfg, meta = inputs.kuramoto_scale(n=1000, n_points=4, n_steps=60, bold=False)
    compare(cfg, 4, SweepParam(-1, 0), [0.0, 0.5, 1.0, 2.0], 60, semantics=HB_SEM_DELAY_RING, rtol=2e-5)


def test_edge_cases_empty_rows_and_long_delays():
    # rows without edges, delays longer than the run, single point, single step
    csr = {"data": [1.0, 0.5], "indices": [2, 0], "indptr": [0, 1, 1, 2, 2]}
    cfg = SimConfig(sim_length=1.0, dt=0.1, integrator="heun",
                    network=NetworkConfig([sub("Generic2dOscillator", 4, 1)],
                                          [ProjectionConfig(0, 0, csr, coupling_fn="Linear", coupling_params=[0.5],
                                                            delays=[3, 40])]))
    compare(cfg, 1, SweepParam(0, 1), [0.1], 20, semantics=HB_SEM_DELAY_RING)
    compare(cfg, 1, SweepParam(0, 1), [0.1], 1, semantics=HB_SEM_DELAY_RING)
    compare(cfg, 1, SweepParam(0, 1), [0.1], 25)


def test_collapsing_pre_into_two_cvar_target_is_rejected():
    """PreSigmoidal dynamic collapses MPR's two cvars into one channel; the reference then narrows
    a missing channel (dfun.rs:449) and panics, so the engine refuses the configuration."""
    from hyburn_gb300.config import Unsupported
    cfg = single_model("MontbrioPazoRoxin", 8, "heun", "PreSigmoidal", (0.1, 0.5, 1.0, 1.0, 0.5, 1.0))
    with pytest.raises(Unsupported):
        BatchHybridEngine.from_config(cfg, 2)


def test_noise_too_short_is_an_error():
    cfg = single_model("Generic2dOscillator", 8, "heun_stochastic", nsig=1e-3)
    eng = BatchHybridEngine.from_config(cfg, 2)
    with pytest.raises(InvalidState, match="noise array too short"):
        eng.run_sweep(SweepParam(0, 1), [0.0, 0.1], 10, noise=np.zeros(5, np.float32))


@pytest.mark.parametrize("integrator", INTEGRATORS)
def test_pipeline_integrators_bold_and_chunked_runs(integrator):
    """Warp-specialised pipeline (all delays >= 17): every integrator, per-point BOLD, and runs
    split across calls (the ring and running sums carry over between launches)."""
    mons = [MonitorConfig("Bold", tr=0.003, bold_period=10)]
    cfg = single_model("Generic2dOscillator", 40, integrator, "Linear", (0.2,), weights="csr",
                       delays="per_edge_long", nsig=1e-3, monitors=mons)
    eng = BatchHybridEngine.from_config(cfg, 3, semantics=HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT)
    ora = OracleEngine.from_config(cfg, 3, semantics=HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT)
    for n in (333, 201):
        nz = noise_for(cfg, n, 3, False, n)
        g = eng.run_sweep(SweepParam(-1, 0), [0.0, 0.1, 0.2], n, noise=nz)
        o = ora.run_sweep(SweepParam(-1, 0), [0.0, 0.1, 0.2], n, noise=nz)
        close(g.final_states[0], o.final_states[0], what=f"final after {n}")
        close(g.tavg[0], o.tavg[0], what=f"tavg after {n}")
        close(g.bold[0], o.bold[0], atol=BOLD_ATOL, what=f"bold after {n}")
    assert eng.last_kernel_time()[2] == 3  # the pipeline ran


def test_prepared_run_matches_host_run():
    from hyburn_gb300 import inputs
    cfg, meta = inputs.batched_sweep(n_steps=200, n_points=8)
    nz = inputs.standard_normal((200, 148), 2)
    eng = BatchHybridEngine.from_config(cfg, 8, semantics=HB_SEM_DELAY_RING)
    g = eng.run_sweep(SweepParam(-1, 0), meta["values"], 200, noise=nz)
    eng.prepare(SweepParam(-1, 0), meta["values"], 200, noise=nz)
    eng.execute_prepared()
    st = eng.states[0]
    assert np.array_equal(st.ravel(), g.final_states[0])
    ms, launches, kind = eng.last_kernel_time()
    assert ms > 0 and launches == 1
