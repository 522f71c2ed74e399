"""Functional-connectivity features on the device (hb_engine_fc_features) against the oracle
(oracle/fc_ref.py, a restatement of src/sbi/features/fc.rs and mod.rs:257-280).

CPU: the oracle reproduces the reference's own unit tests (fc.rs:221-296), plus edge cases of the
reference's rules (constant series, one node, one window).
GPU: a sweep run with HB_RUN_DEVICE_TRAJECTORY | HB_RUN_TRAJECTORY keeps its trajectory on the
device and also returns it to the host; the device features must equal the oracle's on the host
copy within FC_ATOL (the device sums products in FP32 over 64-step chunks and in FP64 across
chunks, the reference in FP64 throughout)."""
import math

import numpy as np
import pytest

from oracle import fc_ref

FC_ATOL = 2e-5      # FC entries, FC statistics
FCD_ATOL = 5e-5     # FCD entries (correlations of window FCs) and their statistics


# ---- the oracle against the reference's unit tests ----

def test_kat_fc_identity():
    fc = fc_ref.fc_matrix(np.array([1.0, 1.0, 2.0, 2.0, 3.0, 3.0], np.float32), 3, 2)
    assert np.all(np.abs(fc.ravel() - 1.0) < 1e-5)


def test_kat_fc_anti_correlated():
    fc = fc_ref.fc_matrix(np.array([1.0, -1.0, 2.0, -2.0, 3.0, -3.0], np.float32), 3, 2)
    assert abs(fc[0, 1] + 1.0) < 1e-5


def test_kat_fc_stats():
    fc = np.array([1.0, 0.5, -0.3, 0.5, 1.0, 0.8, -0.3, 0.8, 1.0], np.float32)
    s = fc_ref.fc_stats(fc, 3)
    assert len(s) == 5
    assert abs(s[0] - (0.5 - 0.3 + 0.8) / 3.0) < 1e-5
    assert s[1] >= 0.0 and abs(s[2] + 0.3) < 1e-5 and abs(s[3] - 0.8) < 1e-5


def test_kat_fcd_matrix():
    traj = np.sin(np.arange(30, dtype=np.float32)).astype(np.float32)
    fcd = fc_ref.fcd_matrix(traj, 10, 3, 4, 2)
    assert fcd.shape[0] >= 2 and fcd.shape == (4, 4)  # (10 - 4) / 2 + 1
    assert abs(fcd[0, 0] - 1.0) < 1e-5


def test_kat_homotopic():
    fc = np.array([1.0, 0.1, 0.2, 0.9, 0.1, 1.0, 0.8, 0.3, 0.2, 0.8, 1.0, 0.4, 0.9, 0.3, 0.4, 1.0], np.float32)
    mean, std, n_pairs = fc_ref.homotopic_fc(fc, 4)
    assert n_pairs == 2 and abs(mean - 0.85) < 1e-5
    assert abs(std - math.sqrt((0.05 ** 2 + 0.05 ** 2) / 2.0)) < 1e-5


def test_oracle_rules_constant_series_single_node_single_window():
    # a constant node: deviation 0 -> 1, so its row and its diagonal entry are 0
    y = np.stack([np.full(20, 0.3, np.float32), np.linspace(0, 1, 20).astype(np.float32)], 1)
    fc = fc_ref.fc_matrix(y, 20, 2)
    assert fc[0, 0] == 0.0 and fc[0, 1] == 0.0 and abs(fc[1, 1] - 1.0) < 1e-6
    assert all(math.isnan(v) for v in fc_ref.fc_stats(fc_ref.fc_matrix(y[:, :1], 20, 1), 1))
    assert fc_ref.fcd_matrix(y, 20, 2, 20, 5).shape == (0, 0)   # one window: empty


# ---- the device features against the oracle ----

def _run(cfg, n_pts, n_steps, param, vals, noise=None):
    from hyburn_gb300 import BatchHybridEngine
    from hyburn_gb300._abi import HB_RUN_DEVICE_TRAJECTORY, HB_RUN_TRAJECTORY, HB_SEM_DELAY_RING
    eng = BatchHybridEngine.from_config(cfg, n_pts, semantics=HB_SEM_DELAY_RING)
    r = eng.run_sweep(param, vals, n_steps, noise=noise, run_flags=HB_RUN_DEVICE_TRAJECTORY | HB_RUN_TRAJECTORY)
    return eng, r


def _check(eng, r, cfg, n_pts, window, stride, fcd_atol=FCD_ATOL):
    sub = cfg.network.subnetworks[0]
    from hyburn_gb300.config import MODEL_REGISTRY
    nvar = MODEL_REGISTRY[sub.model][0]
    f = eng.fc_features(0, window, stride)
    fc, feat, fcd, fcds = fc_ref.fc_features(r.trajectories[0], n_pts, sub.nnodes, sub.nmodes, nvar, window, stride)
    np.testing.assert_allclose(f.fc, fc, atol=FC_ATOL, rtol=0)
    np.testing.assert_allclose(f.features, feat, atol=FC_ATOL, rtol=0, equal_nan=True)
    if window:
        assert f.n_windows == (fcd.shape[2] if fcd.ndim == 4 else 0)
        if f.n_windows:
            np.testing.assert_allclose(f.fcd, fcd, atol=fcd_atol, rtol=0)
        np.testing.assert_allclose(f.fcd_stats, fcds, atol=fcd_atol, rtol=0, equal_nan=True)
    return f


@pytest.mark.gpu
@pytest.mark.parametrize("model,n,integ,coupling,cparams", [
    ("Generic2dOscillator", 12, "heun", "Linear", (0.05,)),
    ("JansenRit", 9, "heun", "Sigmoidal", (0.0, 0.1, 0.0, 1.0, 0.05)),
    ("MontbrioPazoRoxin", 16, "rk4", "Linear", (0.3,)),
])
def test_device_fc_features_match_oracle(model, n, integ, coupling, cparams):
    from cases import single_model
    from hyburn_gb300 import SweepParam
    dt = 0.05 if model == "MontbrioPazoRoxin" else 0.1
    cfg = single_model(model, n, integ, coupling, cparams, weights="csr", delays="per_edge_long", dt=dt, seed=3)
    vals = np.linspace(0.0, 0.2, 3).astype(np.float32).tolist()
    eng, r = _run(cfg, 3, 700, SweepParam(-1, 0), vals)
    f = _check(eng, r, cfg, 3, 200, 100)
    assert f.n_windows == 6 and f.ms > 0
    eng.close()


@pytest.mark.gpu
def test_device_fc_features_stochastic_long_and_windows():
    """More steps than one moment slice, windows that straddle slices, a stochastic run."""
    from cases import noise_for, single_model
    from hyburn_gb300 import SweepParam
    cfg = single_model("Generic2dOscillator", 20, "heun_stochastic", "Linear", (0.02,), weights="csr",
                       delays="per_edge_long", nsig=1e-3, seed=4)
    T = 3000
    eng, r = _run(cfg, 2, T, SweepParam(-1, 0), [0.0, 0.1], noise_for(cfg, T, 2, False, 9))
    _check(eng, r, cfg, 2, 1000, 333)   # windows summed directly (gcd 1)
    _check(eng, r, cfg, 2, 1000, 250)   # windows combined from 250-step blocks (four per window)
    _check(eng, r, cfg, 2, 768, 128)    # six 128-step blocks per window
    _check(eng, r, cfg, 2, 0, 1)
    eng.close()


@pytest.mark.gpu
def test_device_fc_features_errors_and_empty_fcd():
    from cases import single_model
    from hyburn_gb300 import BatchHybridEngine, SweepParam
    from hyburn_gb300.config import InvalidState
    cfg = single_model("Generic2dOscillator", 6, "heun", "Linear", (0.05,), weights="csr", delays="per_edge_long", seed=5)
    eng = BatchHybridEngine.from_config(cfg, 2)
    eng.run_sweep(SweepParam(-1, 0), [0.0, 0.1], 50)
    with pytest.raises(InvalidState, match="device trajectory"):
        eng.fc_features()
    eng.close()
    eng, r = _run(cfg, 2, 120, SweepParam(-1, 0), [0.0, 0.1])
    with pytest.raises(InvalidState, match="window_len"):
        eng.fc_features(0, 1, 1)
    with pytest.raises(InvalidState, match="window_len"):
        eng.fc_features(0, 121, 1)
    with pytest.raises(InvalidState, match="stride"):
        eng.fc_features(0, 10, 0)
    f = _check(eng, r, cfg, 2, 100, 50)   # (120 - 100) / 50 + 1 = 1 window: no FCD, NaN stats
    assert f.n_windows == 0 and f.fcd is None and np.isnan(f.fcd_stats).all()
    eng.close()


@pytest.mark.gpu
@pytest.mark.parametrize("n", [2, 3, 5])
def test_device_fc_features_few_nodes(n):
    """Two to five nodes: one to ten upper-triangle values, homotopic pairs n // 2, and the median
    of very short value lists. With three nodes each window FC has three upper-triangle values, and
    the Pearson correlation of two such triples is ill conditioned: FP32 rounding of the FC entries
    (~1e-7) moves it by up to ~5e-5 (measured 5.06e-5), so the FCD bound is 5e-4 there."""
    from cases import single_model
    from hyburn_gb300 import SweepParam
    cfg = single_model("Generic2dOscillator", n, "heun", "Linear", (0.05,), weights="csr", delays="per_edge_long",
                       density=1.0, seed=7)
    eng, r = _run(cfg, 2, 400, SweepParam(-1, 0), [0.0, 0.1])
    _check(eng, r, cfg, 2, 100, 50, fcd_atol=5e-4 if n <= 3 else FCD_ATOL)
    eng.close()
