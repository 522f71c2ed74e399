"""Parity with the oracle at the benchmark configurations' own sizes.

Two forms of the check. With HB_RUN_EXACT_SUMS the engine adds every coupling term in the reference's
order with separately rounded products and sums; for models without transcendental functions it must
then equal the FP32 oracle bit for bit, at any length. In the default form the coupling sums are
regrouped (lanes, fused multiply-adds); over tens of thousands of deterministic steps the two FP32
roundings drift apart by more than rel 1e-5 in a few elements (measured: 6.8e-5 in one of 18 944
temporal averages of the deterministic benchmark sweep), so there the bound is the FP32 arithmetic
itself: the engine may be no farther from the FP32 oracle than twice the FP32 oracle's distance from
the FP64 one (largest absolute difference over the output), with rel 1e-5 / abs 1e-6 as the floor.

- The 128-point, 74-node G2DO sweep with per-edge delays, 20 000 Heun steps: deterministic and with
  the shared seeded draws of the benchmark.
- The single G2DO simulation, 74 nodes, mean-field coupling, its full 10 000 steps.
- The uneven MontbrioPazoRoxin grid: each network size (68, 84, 164, 400 nodes) for 20 000 RK4 steps
  at dt 0.05 with per-point eta tables and the coupling scale swept, in one grouped launch; and a
  68-node member for 44 000 steps with BOLD at TR 2 s (two samples).
- Kuramoto, 1000 nodes, 5 % CSR, per-node omega ~ N(0, 1), 4 points x 10 000 steps: phases are
  compared on the circle; a phase that wraps at a different step on each side shifts that node's
  temporal average by exactly 2 pi / T, so the averages are compared after removing whole wraps, and
  such nodes must be rare.
"""
import os

import numpy as np
import pytest

from hyburn_gb300 import BatchHybridEngine, GroupedSweep, SweepParam, inputs
from hyburn_gb300._abi import HB_RUN_EXACT_SUMS, HB_SEM_BOLD_PER_POINT, HB_SEM_DELAY_RING
from oracle.hb_oracle import OracleEngine

from test_parity_gpu import BOLD_ATOL, close

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1


def _mpr_member(n, seed, T, G, eta, tr=2.0):
    cfg, meta = inputs.mpr_grid(n, len(G) * len(eta), T, seed=seed, bold=True, eta_per_point=False)
    cfg.monitors[0].tr = tr
    B = len(G) * len(eta)
    p = np.asarray(cfg.network.subnetworks[0].params, np.float32)
    rows = np.tile(p, (B, n, 1))
    rows[:, :, 2] = np.repeat(np.tile(np.asarray(eta, np.float32), len(G)), n).reshape(B, n)
    cfg.network.subnetworks[0].node_params = rows
    return cfg, np.repeat(np.asarray(G, np.float32), len(eta))


def within_fp32_error(g, o32, o64, what):
    """The engine and the FP32 oracle are two FP32 roundings of the same run, each about as far from the
    FP64 run as the other: the engine's largest distance from the FP32 oracle may be twice the FP32
    oracle's largest distance from FP64, and never needs to be below the usual rel 1e-5 / abs 1e-6."""
    g, o32, o64 = (np.asarray(v, np.float64) for v in (g, o32, o64))
    dg, d32 = np.abs(g - o32).max(), np.abs(o32 - o64).max()
    bound = max(2.0 * d32, 1e-6 + 1e-5 * np.abs(o32).max())
    assert dg <= bound, f"{what}: engine differs from the FP32 oracle by {dg:.3g}, the FP32 oracle from FP64 by {d32:.3g}"


@pytest.mark.parametrize("stochastic", [False, True])
def test_benchmark_sweep_full_size(stochastic):
    """The benchmark sweep, 128 points x 74 nodes x 20 000 steps: bit for bit with the reference's
    summation order, within the FP32 arithmetic's own error in the default (benchmark) form."""
    T, B = 20_000, 128
    cfg, meta = inputs.batched_sweep(n_steps=T, n_points=B, nsig=1e-3 if stochastic else 0.0,
                                     integrator="heun_stochastic" if stochastic else "heun")
    noise = inputs.standard_normal((T, 148), 2) if stochastic else None
    eng = BatchHybridEngine.from_config(cfg, B, semantics=HB_SEM_DELAY_RING)
    ex = eng.run_sweep(SweepParam(-1, 0), meta["values"], T, noise=noise, run_flags=HB_RUN_EXACT_SUMS)
    assert eng.last_kernel_time()[2] == 3  # the benchmark's kernel
    eng.reset()
    g = eng.run_sweep(SweepParam(-1, 0), meta["values"], T, noise=noise)
    o = OracleEngine.from_config(cfg, B, semantics=HB_SEM_DELAY_RING, n_threads=THREADS).run_sweep(
        SweepParam(-1, 0), meta["values"], T, noise=noise)
    o64 = OracleEngine.from_config(cfg, B, semantics=HB_SEM_DELAY_RING, precision="f64", n_threads=THREADS).run_sweep(
        SweepParam(-1, 0), meta["values"], T, noise=noise)
    assert np.array_equal(ex.final_states[0], o.final_states[0]), "final states, reference order"
    assert np.array_equal(ex.tavg[0], o.tavg[0]), "temporal average, reference order"
    within_fp32_error(g.final_states[0], o.final_states[0], o64.final_states[0], "final states")
    within_fp32_error(g.tavg[0], o.tavg[0], o64.tavg[0], "temporal average")


def test_single_simulation_full_size():
    cfg, meta = inputs.plain_single_sim(10_000)
    par = SweepParam(0, 1)
    vals = [cfg.network.subnetworks[0].params[1]]
    g = BatchHybridEngine.from_config(cfg, 1).run_sweep(par, vals, 10_000)
    o = OracleEngine.from_config(cfg, 1).run_sweep(par, vals, 10_000)
    close(g.final_states[0], o.final_states[0], what="final states")
    close(g.tavg[0], o.tavg[0], what="temporal average")


@pytest.mark.parametrize("exact", [True, False])
def test_uneven_mpr_grid_grouped_20000_steps(exact):
    """Every size of the uneven grid for 20 000 RK4 steps in one work-queue launch: bit for bit in the
    reference's summation order (MPR has no transcendental function), within the FP32 error otherwise."""
    T = 20_000
    members, refs, refs64 = [], [], []
    for n in (68, 84, 164, 400):
        cfg, G = _mpr_member(n, 3, T, [0.5, 1.0], [-5.0, -3.5])
        sem = HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT
        members.append((BatchHybridEngine.from_config(cfg, 4, semantics=sem), SweepParam(-1, 0), G, T, None))
        refs.append(OracleEngine.from_config(cfg, 4, semantics=sem, n_threads=THREADS).run_sweep(SweepParam(-1, 0), G, T))
        if not exact:
            refs64.append(OracleEngine.from_config(cfg, 4, semantics=sem, precision="f64", n_threads=THREADS).run_sweep(
                SweepParam(-1, 0), G, T))
    grp = GroupedSweep(members, run_flags=HB_RUN_EXACT_SUMS if exact else 0)
    grp.execute()
    for i, (n, o, r) in enumerate(zip((68, 84, 164, 400), refs, grp.results())):
        if exact:
            assert np.array_equal(r.final_states[0], o.final_states[0]), f"{n} nodes: final states"
            assert np.array_equal(r.tavg[0], o.tavg[0]), f"{n} nodes: temporal average"
        else:
            within_fp32_error(r.final_states[0], o.final_states[0], refs64[i].final_states[0], f"{n} nodes: final states")
            within_fp32_error(r.tavg[0], o.tavg[0], refs64[i].tavg[0], f"{n} nodes: temporal average")
    grp.close()


def test_uneven_mpr_bold_two_samples():
    T = 84_000  # 4.2 s at dt 0.05 ms: BOLD samples at 2 s and 4 s
    cfg, G = _mpr_member(68, 3, T, [0.8], [-4.5])
    sem = HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT
    grp = GroupedSweep([(BatchHybridEngine.from_config(cfg, 1, semantics=sem), SweepParam(-1, 0), G, T, None)])
    grp.execute()
    r = grp.results()[0]
    o = OracleEngine.from_config(cfg, 1, semantics=sem).run_sweep(SweepParam(-1, 0), G, T)
    assert o.bold[0].size == 2 * 68 and r.bold[0].size == 2 * 68
    close(r.final_states[0], o.final_states[0], what="final states")
    close(r.bold[0], o.bold[0], 1e-5, BOLD_ATOL, "BOLD")
    grp.close()


def wrapped_tavg_compare(g_tavg, o_tavg, T, rtol=1e-5, atol=1e-6):
    """Temporal averages of wrapped phases, equal up to whole wraps (2 pi / T each); returns the number
    of nodes whose wrap count differs."""
    d = (np.asarray(g_tavg, np.float64) - np.asarray(o_tavg, np.float64)) * T / (2 * np.pi)
    k = np.round(d)
    rest = (d - k) * 2 * np.pi / T
    err = np.abs(rest) / (atol + rtol * np.abs(np.asarray(o_tavg, np.float64)))
    assert err.max() <= 1.0, f"max scaled error {err.max():.3g} after removing whole wraps"
    return int(np.count_nonzero(k))


def test_kuramoto_1000_nodes_per_node_omega_10000_steps():
    T, B = 10_000, 4
    cfg, meta = inputs.kuramoto_scale(n=1000, n_points=B, n_steps=T, bold=True)
    assert cfg.network.subnetworks[0].node_params is not None
    vals = [0.2, 0.8, 1.4, 2.0]
    sem = HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT
    g = BatchHybridEngine.from_config(cfg, B, semantics=sem).run_sweep(SweepParam(-1, 0), vals, T)
    o = OracleEngine.from_config(cfg, B, semantics=sem, n_threads=THREADS).run_sweep(SweepParam(-1, 0), vals, T)
    d = (np.asarray(g.final_states[0], np.float64) - o.final_states[0] + np.pi) % (2 * np.pi) - np.pi
    err = np.abs(d) / (1e-6 + 1e-5 * np.abs(np.asarray(o.final_states[0], np.float64)))
    assert err.max() <= 1.0, f"final phases: max scaled error {err.max():.3g}"
    moved = wrapped_tavg_compare(g.tavg[0], o.tavg[0], T)
    assert moved <= 0.01 * B * 1000, f"{moved} nodes wrapped at a different step"
