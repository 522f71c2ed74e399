"""Seeded synthetic workloads for the batched-simulation benchmarks and parity tests.

No dataset or checkpoint is used: connectomes, tract lengths, initial states and noise draws are
generated with ``numpy.random.default_rng(seed)`` following the recipes of the benchmark
configurations (symmetric, zero diagonal, Bernoulli density, log-normal(0,1) weights normalised to
max 1; uniform tract lengths converted to integer delays with ``ceil(L / speed / dt)``).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Tuple

import numpy as np

from .config import (DEFAULT_PARAMS, MonitorConfig, NetworkConfig, ProjectionConfig, SimConfig, SubnetworkConfig, tract_lengths_to_delays)

G2DO_BENCH_PARAMS = [1.0, 0.0, -2.0, -10.0, 0.0, 0.02, 3.0, 1.0, 0.0, 1.0, 1.0, 1.0]


@dataclass
class Connectome:
    n: int
    data: np.ndarray      # float32 [nnz]
    indices: np.ndarray   # uint32 [nnz] (source node of each edge)
    indptr: np.ndarray    # uint32 [n+1] (rows are target nodes)
    lengths: np.ndarray   # float32 [nnz] tract lengths (mm)

    @property
    def nnz(self) -> int:
        return int(self.data.size)

    def dense(self) -> np.ndarray:
        w = np.zeros((self.n, self.n), np.float32)
        for t in range(self.n):
            for k in range(self.indptr[t], self.indptr[t + 1]):
                w[t, self.indices[k]] = self.data[k]
        return w

    def csr_weights(self) -> dict:
        return {"data": self.data.tolist(), "indices": self.indices.tolist(), "indptr": self.indptr.tolist()}


def connectome(n: int, density: float, seed: int, l_lo: float = 10.0, l_hi: float = 200.0) -> Connectome:
    """Symmetric, zero-diagonal Bernoulli(density) graph with log-normal(0,1) weights / max and
    symmetric uniform tract lengths in [l_lo, l_hi] mm."""
    rng = np.random.default_rng(seed)
    upper = np.triu(rng.random((n, n)) < density, k=1)
    w = np.where(upper, rng.lognormal(0.0, 1.0, (n, n)), 0.0)
    w = w + w.T
    if w.max() > 0:
        w = w / w.max()
    lengths = rng.uniform(l_lo, l_hi, (n, n))
    lengths = np.triu(lengths, 1)
    lengths = lengths + lengths.T
    data, indices, indptr, lens = [], [], [0], []
    for t in range(n):
        cols = np.nonzero(w[t])[0]
        data.extend(w[t, cols])
        indices.extend(cols)
        lens.extend(lengths[t, cols])
        indptr.append(len(data))
    return Connectome(n=n, data=np.asarray(data, np.float32), indices=np.asarray(indices, np.uint32),
                      indptr=np.asarray(indptr, np.uint32), lengths=np.asarray(lens, np.float32))


def uniform_state(n_nodes: int, nvar: int, seed: int, lo: float = -1.0, hi: float = 1.0) -> List[float]:
    """Initial state uniform in [lo, hi] per (node, state var), batch layout [nnodes, nvar]."""
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, (n_nodes, nvar)).astype(np.float32).ravel().tolist()


def standard_normal(shape, seed: int) -> np.ndarray:
    """Raw N(0,1) draws in float32; the engine scales them by sqrt(2*nsig)*sqrt(dt)."""
    return np.random.default_rng(seed).standard_normal(shape, dtype=np.float32)


# ---------------------------------------------------------------------------------------------
# benchmark workloads
# ---------------------------------------------------------------------------------------------

def plain_single_sim(n_steps: int = 10_000) -> Tuple[SimConfig, dict]:
    """G2DO, 74 nodes, Heun dt 0.1, all_to_all Scalar w=0.01 with Linear a=0.01, no delay,
    nsig 0, initial state U[-1,1] (seed 1), batch 1."""
    n = 74
    cfg = SimConfig(
        sim_length=n_steps * 0.1, dt=0.1, integrator="heun", nsig=0.0,
        network=NetworkConfig(
            subnetworks=[SubnetworkConfig("Generic2dOscillator", n, uniform_state(n, 2, 1), list(G2DO_BENCH_PARAMS))],
            projections=[ProjectionConfig(0, 0, 0.01, coupling_fn="Linear", coupling_params=[0.01], cvar_map="0:0")]))
    return cfg, {"n_sweep": 1, "sweep": (0, 1), "values": [0.0], "n_steps": n_steps}


def batched_sweep(n_steps: int = 20_000, n_points: int = 128, n: int = 74, seed: int = 2,
                  coupling_a_max: float = 0.05, nsig: float = 1e-3, integrator: str = "heun_stochastic",
                  per_point_coupling: bool = True) -> Tuple[SimConfig, dict]:
    """The 128-point, 74-node G2DO sweep with sparse delayed coupling.

    Connectome: symmetric, zero diagonal, 20% density, log-normal(0,1) weights / max; tract
    lengths U[10,200] mm at 3 mm/ms with dt 0.1 -> integer delays up to 667 steps (per edge).
    The sweep runs over the Linear coupling scale a in linspace(0, 0.05); the reference can only
    sweep model parameters, so the coupling scale enters as a per-point coupling parameter
    (``coupling_sweep``) of this engine. Heun-stochastic, nsig 1e-3, seeded N(0,1) draws."""
    c = connectome(n, 0.2, seed)
    dt = 0.1
    delays = tract_lengths_to_delays(c.lengths, 3.0, dt)
    cfg = SimConfig(
        sim_length=n_steps * dt, dt=dt, integrator=integrator, nsig=nsig,
        network=NetworkConfig(
            subnetworks=[SubnetworkConfig("Generic2dOscillator", n, uniform_state(n, 2, seed), list(G2DO_BENCH_PARAMS))],
            projections=[ProjectionConfig(0, 0, c.csr_weights(), conn_type="csr", delays=delays,
                                          tract_lengths=c.lengths.tolist(), coupling_fn="Linear",
                                          coupling_params=[0.01], cvar_map="0:0")]))
    values = np.linspace(0.0, coupling_a_max, n_points).astype(np.float32).tolist()
    return cfg, {"n_sweep": n_points, "values": values, "n_steps": n_steps, "connectome": c,
                 "max_delay": int(max(delays)), "min_delay": int(min(delays))}


def mpr_grid(n_nodes: int, n_points: int, n_steps: int, seed: int, dt: float = 0.05,
             bold: bool = True, eta_per_point: bool = True) -> Tuple[SimConfig, dict]:
    """One size of the uneven-batching MPR workload: N nodes, a (G, eta) grid over n_points,
    sparse delayed Linear coupling (U[10,200] mm at 3 mm/ms), RK4, BOLD at TR 2 s.

    The grid has n_eta = the largest divisor of n_points not above its square root values of eta in
    [-6, -3] and n_points / n_eta values of the coupling scale G in [0, 1]; point b = iG * n_eta + i_eta.
    G is swept per point as the Linear coupling scale (``values``); eta enters through per-point
    parameter tables (``node_params`` [n_points, N, 7]) when eta_per_point is set."""
    c = connectome(n_nodes, 0.2, seed)
    delays = tract_lengths_to_delays(c.lengths, 3.0, dt)
    params = list(DEFAULT_PARAMS["MontbrioPazoRoxin"])
    mons = [MonitorConfig("Bold", tr=2.0, bold_period=10)] if bold else []
    rng = np.random.default_rng(seed)
    x0 = np.stack([rng.uniform(0.0, 1.0, n_nodes), rng.uniform(-2.0, 0.0, n_nodes)], 1).astype(np.float32)
    n_eta = max(d for d in range(1, int(np.sqrt(n_points)) + 1) if n_points % d == 0)
    n_g = n_points // n_eta
    g = np.linspace(0.0, 1.0, n_g).astype(np.float32)
    eta = np.linspace(-6.0, -3.0, n_eta).astype(np.float32)
    sub = SubnetworkConfig("MontbrioPazoRoxin", n_nodes, x0.ravel().tolist(), params)
    if eta_per_point:
        rows = np.tile(np.asarray(params, np.float32), (n_points, n_nodes, 1))
        rows[:, :, 2] = np.repeat(np.tile(eta, n_g), n_nodes).reshape(n_points, n_nodes)
        sub.node_params = rows
    cfg = SimConfig(
        sim_length=n_steps * dt, dt=dt, integrator="rk4", nsig=0.0, monitors=mons,
        network=NetworkConfig(
            subnetworks=[sub],
            projections=[ProjectionConfig(0, 0, c.csr_weights(), conn_type="csr", delays=delays,
                                          coupling_fn="Linear", coupling_params=[1.0], cvar_map="0:0")]))
    return cfg, {"n_sweep": n_points, "G": g.tolist(), "eta": eta.tolist(), "values": np.repeat(g, n_eta).tolist(),
                 "n_steps": n_steps, "max_delay": int(max(delays)), "min_delay": int(min(delays))}


def kuramoto_scale(n: int = 1000, n_points: int = 256, n_steps: int = 100_000, seed: int = 5,
                   density: float = 0.05, bold: bool = True, omega_per_node: bool = True) -> Tuple[SimConfig, dict]:
    """Kuramoto, 1000-node 5% CSR connectome, delays from U[10,250] mm at 5 mm/ms, dt 0.1,
    256 points over the coupling scale G, natural frequencies omega ~ N(0,1) per node (``node_params``
    [n, 1]; with omega_per_node off every node keeps the model's omega = 1)."""
    c = connectome(n, density, seed, 10.0, 250.0)
    dt = 0.1
    delays = tract_lengths_to_delays(c.lengths, 5.0, dt)
    rng = np.random.default_rng(seed)
    theta0 = rng.uniform(0.0, 2 * np.pi, n).astype(np.float32)
    mons = [MonitorConfig("Bold", tr=2.0, bold_period=10)] if bold else []
    cfg = SimConfig(
        sim_length=n_steps * dt, dt=dt, integrator="heun", nsig=0.0, monitors=mons,
        network=NetworkConfig(
            subnetworks=[SubnetworkConfig("Kuramoto", n, theta0.tolist(), [1.0])],
            projections=[ProjectionConfig(0, 0, c.csr_weights(), conn_type="csr", delays=delays,
                                          coupling_fn="Kuramoto", coupling_params=[1.0], cvar_map="0:0")]))
    omega = rng.standard_normal(n).astype(np.float32)
    if omega_per_node:
        cfg.network.subnetworks[0].node_params = omega.reshape(n, 1)
    values = np.linspace(0.0, 2.0, n_points).astype(np.float32).tolist()
    return cfg, {"n_sweep": n_points, "values": values, "n_steps": n_steps, "omega": omega,
                 "max_delay": int(max(delays)), "min_delay": int(min(delays))}


def jr_fc_adjoint(n_steps: int = 20_000, n_points: int = 64, n: int = 74, seed: int = 4) -> Tuple[SimConfig, dict]:
    """The FC-adjoint workload: JansenRit, n nodes on the batched-sweep connectome recipe (20 %
    density, tract lengths U[10, 200] mm at 3 mm/ms, dt 0.1 ms), Sigmoidal coupling
    (cmin 0, cmax 0.1, midpoint 0, gain, sigma 0.05) with per-edge delays, Heun, nsig 0, and
    n_points coupling gains in [0.5, 1.5]. Initial state uniform per variable from `seed`."""
    c = connectome(n, 0.2, seed)
    delays = tract_lengths_to_delays(c.lengths, 3.0, 0.1)
    rng = np.random.default_rng(seed)
    ranges = [(-0.5, 0.5), (0.0, 20.0), (0.0, 20.0), (-1.0, 1.0), (-1.0, 1.0), (-1.0, 1.0)]
    x0 = np.stack([rng.uniform(lo, hi, n) for lo, hi in ranges], 1).astype(np.float32).ravel().tolist()
    cfg = SimConfig(
        sim_length=n_steps * 0.1, dt=0.1, integrator="heun", nsig=0.0,
        network=NetworkConfig(
            subnetworks=[SubnetworkConfig("JansenRit", n, x0, list(DEFAULT_PARAMS["JansenRit"]))],
            projections=[ProjectionConfig(0, 0, c.csr_weights(), conn_type="csr", delays=delays,
                                          coupling_fn="Sigmoidal", coupling_params=[0.0, 0.1, 0.0, 1.0, 0.05])]))
    gains = np.linspace(0.5, 1.5, n_points).astype(np.float32)
    return cfg, {"gains": gains, "connectome": c, "min_delay": int(min(delays)), "max_delay": int(max(delays))}



def jr_target_fc(cfg: SimConfig, n_steps: int, gain: float = 1.0, seed: int = 40) -> np.ndarray:
    """Target FC of the FC-adjoint workload: Pearson FC of y1 - y2 of a forward run of the same network
    with coupling gain `gain` from an initial state drawn with `seed` (computed on the GPU)."""
    import copy

    from .engine import BatchHybridEngine
    from ._abi import HB_SEM_DELAY_RING

    c = copy.deepcopy(cfg)
    sub = c.network.subnetworks[0]
    rng = np.random.default_rng(seed)
    ranges = [(-0.5, 0.5), (0.0, 20.0), (0.0, 20.0), (-1.0, 1.0), (-1.0, 1.0), (-1.0, 1.0)]
    sub.initial_state = np.stack([rng.uniform(lo, hi, sub.nnodes) for lo, hi in ranges], 1).astype(np.float32).ravel().tolist()
    eng = BatchHybridEngine.from_config(c, 1, semantics=HB_SEM_DELAY_RING)
    r = eng.adjoint_fc([gain], n_steps, np.eye(sub.nnodes, dtype=np.float32), checkpoint_every=500)
    eng.close()
    return np.asarray(r.fc[0], np.float32)
