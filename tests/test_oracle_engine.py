"""Engine-level behaviour of the oracle, restating the reference's batch-engine tests
(src/engine/batch_engine/engine.rs:1431-3058) and the semantics the CUDA engine is checked
against (history shift window, per-edge ring, multi-sweep rules)."""
import numpy as np

from hyburn_gb300 import SweepParam, SweepPoint, SweepSpec
from hyburn_gb300._abi import HB_SEM_DELAY_RING, HB_SEM_NOISE_PER_POINT
from hyburn_gb300.config import DEFAULT_PARAMS, NetworkConfig, ProjectionConfig, SimConfig, SubnetworkConfig
from oracle.hb_oracle import OracleEngine

from cases import noise_for, single_model, three_subnet_ring


def g2do_cfg(n=4, integrator="heun", init=None, projections=()):
    init = init if init is not None else [0.0] * (2 * n)
    return SimConfig(sim_length=100.0, dt=0.1, integrator=integrator,
                     network=NetworkConfig([SubnetworkConfig("Generic2dOscillator", n, init,
                                                             list(DEFAULT_PARAMS["Generic2dOscillator"]))],
                                           list(projections)))


def test_batch_engine_g2do_single_subnet():  # engine.rs:1439-1482
    r = OracleEngine(g2do_cfg(), 3).run_sweep(SweepParam(0, 1), [-0.5, 0.0, 0.5], 100)
    assert r.n_sweep == 3
    t = r.tavg[0].reshape(3, -1)
    assert np.isfinite(t).all() and np.isfinite(r.final_states[0]).all()
    assert np.abs(t[0] - t[1]).sum() > 1e-6 and np.abs(t[1] - t[2]).sum() > 1e-6


def test_batch_engine_g2do_sweep_actually_varies():  # engine.rs:1485-1525
    r = OracleEngine(g2do_cfg(2, "euler", [0.1] * 4), 2).run_sweep(SweepParam(0, 1), [-1.0, 1.0], 50)
    t = r.tavg[0].reshape(2, -1)
    assert np.abs(t[0] - t[1]).sum() > 1e-4


def test_non_native_sweep_index_is_ignored():  # dfun.rs:49-72: only I (idx 1) is sweepable for G2DO
    r = OracleEngine(g2do_cfg(2, "euler", [0.1] * 4), 2).run_sweep(SweepParam(0, 9), [0.5, 2.0], 50)
    t = r.tavg[0].reshape(2, -1)
    assert np.array_equal(t[0], t[1])


def test_delay_coupling_changes_output():  # engine.rs:2703-2787
    n = 2
    init = [0.1, 0.2, 0.3, 0.4]

    def cfg(delay):
        subs = [SubnetworkConfig("Generic2dOscillator", n, init, list(DEFAULT_PARAMS["Generic2dOscillator"]))
                for _ in range(2)]
        return SimConfig(sim_length=1.0, dt=0.1, integrator="euler",
                         network=NetworkConfig(subs, [ProjectionConfig(0, 1, 0.1, coupling_fn="Linear",
                                                                       coupling_params=[1.0], delays=[delay])]))

    rd = OracleEngine(cfg(3), 1).run_sweep(SweepParam(0, 1), [0.0], 10)
    r0 = OracleEngine(cfg(0), 1).run_sweep(SweepParam(0, 1), [0.0], 10)
    assert np.abs(rd.tavg[1] - r0.tavg[1]).sum() > 1e-8
    assert np.isfinite(rd.tavg[1]).all() and np.isfinite(r0.tavg[1]).all()


def test_trajectory_recording():  # engine.rs:2790-2838
    cfg = g2do_cfg(2, "euler", [0.1, 0.2, 0.3, 0.4])
    rw = OracleEngine(cfg, 2).run_sweep_with_trajectory(SweepParam(0, 1), [-0.5, 0.5], 10)
    assert rw.trajectories[0].size == 10 * 2 * 2 * 2
    ro = OracleEngine(cfg, 2).run_sweep(SweepParam(0, 1), [-0.5, 0.5], 10)
    assert ro.trajectories is None
    assert np.allclose(rw.tavg[0], ro.tavg[0], atol=1e-6)
    # the trajectory's last step is the final state and its mean is the temporal average
    traj = rw.trajectories[0].reshape(10, -1)
    assert np.array_equal(traj[-1], rw.final_states[0])


def test_threads_match_single_thread():  # engine.rs:2842-2894 (rayon_batch_sweep)
    vals = [-0.5, -0.25, 0.0, 0.25, 0.5, 0.75, 1.0]
    cfg = g2do_cfg(4, "heun", [0.1] * 8)
    a = OracleEngine(cfg, len(vals), n_threads=1).run_sweep(SweepParam(0, 1), vals, 30)
    b = OracleEngine(cfg, len(vals), n_threads=2).run_sweep(SweepParam(0, 1), vals, 30)
    assert np.array_equal(a.tavg[0], b.tavg[0])


def test_sweep_spec_cartesian_product():  # engine.rs:2897-2938
    spec = SweepSpec([SweepPoint(0, 1, [1.0, 2.0]), SweepPoint(0, 2, [10.0, 20.0, 30.0])])
    assert spec.n_sweep() == 6
    p = spec.cartesian_product()
    assert p[0] == [(0, 1, 1.0), (0, 2, 10.0)] and p[1] == [(0, 1, 1.0), (0, 2, 20.0)]
    assert p[3] == [(0, 1, 2.0), (0, 2, 10.0)] and p[5] == [(0, 1, 2.0), (0, 2, 30.0)]
    single = SweepSpec([SweepPoint(0, 1, [0.0, 0.5, 1.0])]).cartesian_product()
    assert single == [[(0, 1, 0.0)], [(0, 1, 0.5)], [(0, 1, 1.0)]]


def test_run_sweep_multi_two_params():  # engine.rs:2941-2991
    spec = SweepSpec([SweepPoint(0, 1, [-1.0, 0.0, 1.0]), SweepPoint(0, 9, [0.5, 2.0])])
    e = OracleEngine(g2do_cfg(2, "euler", [0.1] * 4), spec.n_sweep())
    r = e.run_sweep_multi(spec, 50)
    t = r.tavg[0].reshape(6, -1)
    assert all(np.abs(t[i] - t[i + 1]).sum() > 1e-8 for i in range(5))
    assert np.allclose(r.param_values.reshape(6, 2)[:, 0], [-1, -1, 0, 0, 1, 1])


def test_run_sweep_multi_matches_single():  # engine.rs:2994-3058
    vals = [-0.5, 0.0, 0.5]
    cfg = g2do_cfg(2, "euler", [0.1] * 4)
    a = OracleEngine(cfg, 3).run_sweep(SweepParam(0, 1), vals, 50)
    b = OracleEngine(cfg, 3).run_sweep_multi(SweepSpec([SweepPoint(0, 1, vals)]), 50)
    assert np.allclose(a.tavg[0], b.tavg[0], atol=1e-4)


def test_engine_state_persists_across_runs():  # engine.rs:113 (step) and the state tensors
    cfg = g2do_cfg(3, "heun", [0.2] * 6)
    e1 = OracleEngine(cfg, 2)
    e1.run_sweep(SweepParam(0, 1), [0.1, 0.2], 20)
    r1 = e1.run_sweep(SweepParam(0, 1), [0.1, 0.2], 20)
    assert e1.step == 40
    r2 = OracleEngine(cfg, 2).run_sweep(SweepParam(0, 1), [0.1, 0.2], 40)
    assert np.array_equal(r1.final_states[0], r2.final_states[0])


def test_shift_window_effective_delay_cycles():
    """engine.rs:541-585: with H = d + 1 the delayed read walks back d, d-1, ..., 0, d, ..."""
    n = 1
    cfg = SimConfig(sim_length=2.0, dt=0.1, integrator="euler",
                    network=NetworkConfig([SubnetworkConfig("Kuramoto", n, [0.0], [0.0]),
                                           SubnetworkConfig("Kuramoto", n, [0.0], [0.0])],
                                          [ProjectionConfig(0, 1, 1.0, coupling_fn="Linear", coupling_params=[1.0],
                                                            delays=[3])]))
    # subnetwork 0 runs at omega = 1 (theta_t = 0.1 t); subnetwork 1 integrates its delayed input
    e = OracleEngine(cfg, 1)
    r = e.run_sweep_with_trajectory(SweepParam(0, 0), [1.0], 12)
    th0 = r.trajectories[0].reshape(12)
    th1 = r.trajectories[1].reshape(12)
    inc = np.diff(np.concatenate([[0.0], th1])) / np.float32(0.1)  # coupling seen at each step
    x0 = np.concatenate([[0.0], th0])  # x_s = state at the start of step s
    H = 4
    for s in range(12):
        if s == 0:
            want = x0[0]
        elif 3 > s:
            want = 0.0
        else:
            t_read = s + 1 - H + (s - 3) % H
            want = x0[t_read] if t_read >= 0 else 0.0
        assert abs(inc[s] - want) < 1e-4, (s, inc[s], want)


def test_ring_mode_per_edge_delays_are_true_delays():
    """runtime.rs:162-204: per-edge CSR reads x_{s-d}, zeros before d steps, x_0 at step 0."""
    cfg = SimConfig(sim_length=2.0, dt=0.1, integrator="euler",
                    network=NetworkConfig([SubnetworkConfig("Kuramoto", 2, [0.0, 0.0], [0.0])],
                                          [ProjectionConfig(0, 0, {"data": [1.0, 1.0], "indices": [1, 0], "indptr": [0, 1, 2]},
                                                            coupling_fn="Linear", coupling_params=[1.0], delays=[2, 5])]))
    e = OracleEngine(cfg, 1, semantics=HB_SEM_DELAY_RING)
    r = e.run_sweep_with_trajectory(SweepParam(-1, 0), [1.0], 10)
    th = np.concatenate([[[0.0, 0.0]], r.trajectories[0].reshape(10, 2)])
    inc = np.diff(th, axis=0) / np.float32(0.1)
    for s in range(10):
        for node, src, d in ((0, 1, 2), (1, 0, 5)):
            if s == 0:
                want = th[0, src]
            elif d > s:
                want = 0.0
            else:
                want = th[s - d, src]
            assert abs(inc[s, node] - want) < 1e-4


def test_three_subnet_ring_runs():
    cfg = three_subnet_ring(8, "rk4", delays=(2, 0, 1))
    r = OracleEngine(cfg, 3).run_sweep(SweepParam(0, 1), [0.0, 0.1, 0.2], 30)
    assert all(np.isfinite(t).all() for t in r.tavg)


def test_noise_consumption_shared_vs_per_point():
    cfg = single_model("Generic2dOscillator", 6, "heun_stochastic", nsig=1e-3)
    nz = noise_for(cfg, 20, 3, False, 1)
    a = OracleEngine(cfg, 3).run_sweep(SweepParam(0, 1), [0.0, 0.0, 0.0], 20, noise=nz)
    t = a.final_states[0].reshape(3, -1)
    assert np.array_equal(t[0], t[1])  # shared noise, equal parameters -> identical points
    nzp = np.repeat(nz[:, None, :], 3, axis=1)
    b = OracleEngine(cfg, 3, semantics=HB_SEM_NOISE_PER_POINT).run_sweep(SweepParam(0, 1), [0.0] * 3, 20, noise=nzp)
    assert np.array_equal(a.final_states[0], b.final_states[0])


def test_fp32_vs_fp64_drift_is_small():
    cfg = single_model("Generic2dOscillator", 10, "heun", weights="csr", delays="per_edge")
    vals = [0.0, 0.05]
    a = OracleEngine(cfg, 2, semantics=HB_SEM_DELAY_RING).run_sweep(SweepParam(-1, 0), vals, 200)
    b = OracleEngine(cfg, 2, semantics=HB_SEM_DELAY_RING, precision="f64").run_sweep(SweepParam(-1, 0), vals, 200)
    assert np.allclose(a.final_states[0], b.final_states[0], rtol=1e-4, atol=1e-5)
