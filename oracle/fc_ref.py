"""Oracle (test infrastructure only): functional-connectivity features as hyburn computes them,
restated from ``src/sbi/features/fc.rs`` and the FeatureSet::Fc arm of
``src/sbi/features/mod.rs:257-280``, for checking the engine's on-device features
(hb_engine_fc_features). Pinned by the reference's own unit tests (fc.rs:221-296) in
tests/test_fc_features.py. Plain loops in the reference's order where the order changes f32
results (the statistics); numpy FP64 where the reference accumulates in f64.
"""
from __future__ import annotations

import math
from typing import List, Tuple

import numpy as np


def fc_matrix(traj: np.ndarray, n_steps: int, nnodes: int) -> np.ndarray:
    """fc.rs:11-58: Pearson correlation of the [n_steps, nnodes] series; means and deviations over
    n_steps in f64, a deviation below 1e-12 replaced by 1, entries clamped to [-1, 1], f32 out."""
    y = np.asarray(traj, np.float32).reshape(n_steps, nnodes).astype(np.float64)
    means = y.sum(axis=0) / n_steps
    d = y - means
    stds = np.sqrt((d * d).sum(axis=0) / n_steps)
    stds = np.where(stds < 1e-12, 1.0, stds)
    cov = (d.T @ d) / n_steps
    with np.errstate(invalid="ignore"):
        r = cov / np.outer(stds, stds)
    return np.clip(r, -1.0, 1.0).astype(np.float32)


def fc_stats(fc: np.ndarray, nnodes: int) -> List[float]:
    """fc.rs:62-83: mean, std, min, max, median of the upper triangle, f32 sums in row order."""
    m = np.asarray(fc, np.float32).reshape(nnodes, nnodes)
    vals = [m[i, j] for i in range(nnodes) for j in range(i + 1, nnodes)]
    if not vals:
        return [math.nan] * 5
    s = np.float32(0.0)
    for v in vals:
        s = np.float32(s + v)
    mean = np.float32(s / np.float32(len(vals)))
    q = np.float32(0.0)
    for v in vals:
        dv = np.float32(v - mean)
        q = np.float32(q + np.float32(dv * dv))
    var = np.float32(q / np.float32(len(vals)))
    srt = sorted(vals)
    return [float(mean), float(np.sqrt(var)), float(min(vals)), float(max(vals)), float(srt[len(vals) // 2])]


def homotopic_fc(fc: np.ndarray, nnodes: int) -> Tuple[float, float, int]:
    """fc.rs:189-203: mean and std of FC[i][n-1-i] for i < n/2."""
    m = np.asarray(fc, np.float32).reshape(nnodes, nnodes)
    n_pairs = nnodes // 2
    if n_pairs == 0:
        return math.nan, math.nan, 0
    vals = [m[i, nnodes - 1 - i] for i in range(n_pairs)]
    s = np.float32(0.0)
    for v in vals:
        s = np.float32(s + v)
    mean = np.float32(s / np.float32(n_pairs))
    q = np.float32(0.0)
    for v in vals:
        dv = np.float32(v - mean)
        q = np.float32(q + np.float32(dv * dv))
    return float(mean), float(np.sqrt(np.float32(q / np.float32(n_pairs)))), n_pairs


def upper_triangle_correlation(a: np.ndarray, b: np.ndarray, nnodes: int) -> float:
    """fc.rs:144-179 (f64)."""
    iu = np.triu_indices(nnodes, 1)
    va = np.asarray(a, np.float32).reshape(nnodes, nnodes)[iu].astype(np.float64)
    vb = np.asarray(b, np.float32).reshape(nnodes, nnodes)[iu].astype(np.float64)
    n = nnodes * (nnodes - 1) // 2
    with np.errstate(invalid="ignore", divide="ignore"):
        ma, mb = va.sum() / n, vb.sum() / n
    da, db = va - ma, vb - mb
    cov, var_a, var_b = (da * db).sum(), (da * da).sum(), (db * db).sum()
    if var_a <= 0.0 or var_b <= 0.0:
        return 0.0
    return float(np.float32(min(1.0, max(-1.0, cov / (math.sqrt(var_a) * math.sqrt(var_b))))))


def fcd_matrix(traj: np.ndarray, n_steps: int, nnodes: int, window_len: int, stride: int) -> np.ndarray:
    """fc.rs:87-141: FC per window, then correlations of their upper triangles; empty when at most
    one window."""
    assert 1 < window_len <= n_steps and stride > 0
    y = np.asarray(traj, np.float32).reshape(n_steps, nnodes)
    n_windows = max(n_steps - window_len, 0) // stride + 1
    if n_windows <= 1:
        return np.zeros((0, 0), np.float32)
    fcs = []
    for w in range(n_windows):
        start = w * stride
        end = min(start + window_len, n_steps)
        if end - start < 2:
            continue
        fcs.append(fc_matrix(y[start:end], end - start, nnodes))
    nw = len(fcs)
    if nw <= 1:
        return np.zeros((0, 0), np.float32)
    out = np.zeros((nw, nw), np.float32)
    for i in range(nw):
        out[i, i] = 1.0
        for j in range(i + 1, nw):
            out[i, j] = out[j, i] = upper_triangle_correlation(fcs[i], fcs[j], nnodes)
    return out


def node_series(traj_b: np.ndarray, nnodes: int, nmodes: int, nvar: int, var: int) -> np.ndarray:
    """mod.rs:262-271 on one sweep point of the batch engine's trajectory [T][nnodes*nmodes][nvar]:
    the mean over modes (f32, modes in order)."""
    x = np.asarray(traj_b, np.float32).reshape(-1, nnodes, nmodes, nvar)[:, :, :, var]
    s = np.zeros(x.shape[:2], np.float32)
    for m in range(nmodes):
        s = (s + x[:, :, m]).astype(np.float32)
    return (s / np.float32(nmodes)).astype(np.float32)


def fc_features(traj: np.ndarray, n_sweep: int, nnodes: int, nmodes: int, nvar: int, window_len: int = 0,
                stride: int = 1):
    """Per point and variable: FC, the 7 FeatureSet::Fc values, and FCD with its stats
    (None without windows). traj: the batch trajectory [T][n_sweep][nnodes*nmodes][nvar]."""
    t = np.asarray(traj, np.float32).reshape(-1, n_sweep, nnodes * nmodes * nvar)
    T = t.shape[0]
    fc = np.zeros((n_sweep, nvar, nnodes, nnodes), np.float32)
    feat = np.zeros((n_sweep, nvar, 7), np.float32)
    fcd, fcds = [], []
    for b in range(n_sweep):
        fcd.append([]), fcds.append([])
        for v in range(nvar):
            y = node_series(t[:, b], nnodes, nmodes, nvar, v)
            m = fc_matrix(y, T, nnodes)
            fc[b, v] = m
            h = homotopic_fc(m, nnodes)
            feat[b, v] = fc_stats(m, nnodes) + [h[0], h[1]]
            if window_len:
                d = fcd_matrix(y, T, nnodes, window_len, stride)
                fcd[b].append(d)
                fcds[b].append(fc_stats(d, d.shape[0]) if d.shape[0] > 1 else [math.nan] * 5)
    if not window_len:
        return fc, feat, None, None
    return fc, feat, np.asarray(fcd, np.float32), np.asarray(fcds, np.float32)
