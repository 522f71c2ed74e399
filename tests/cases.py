"""Small seeded network configurations shared by the oracle and GPU parity tests."""
from __future__ import annotations

import numpy as np

from hyburn_gb300.config import (DEFAULT_PARAMS, MODEL_REGISTRY, NetworkConfig, ProjectionConfig,
                                 SimConfig, SubnetworkConfig)
from hyburn_gb300.inputs import connectome, tract_lengths_to_delays

INIT_RANGES = {
    "Generic2dOscillator": [(-1.0, 1.0), (-1.0, 1.0)],
    "MontbrioPazoRoxin": [(0.05, 1.0), (-2.0, 0.0)],
    "ReducedWongWang": [(0.05, 0.9)],
    "Kuramoto": [(0.0, 6.0)],
    "JansenRit": [(-0.5, 0.5), (0.0, 20.0), (0.0, 20.0), (-1.0, 1.0), (-1.0, 1.0), (-1.0, 1.0)],
    "WilsonCowan": [(0.0, 0.5), (0.0, 0.5)],
}
# parameter index each model's batch-native dfun accepts as a per-point sweep (dfun.rs:49-72)
NATIVE_SWEEP = {"Generic2dOscillator": 1, "MontbrioPazoRoxin": 4, "ReducedWongWang": 7, "Kuramoto": 0,
                "JansenRit": 12, "WilsonCowan": 18}
SWEEP_VALUES = {"Generic2dOscillator": (-0.5, 0.5), "MontbrioPazoRoxin": (-1.0, 1.0), "ReducedWongWang": (0.2, 0.5),
                "Kuramoto": (0.5, 1.5), "JansenRit": (0.1, 0.3), "WilsonCowan": (0.0, 1.0)}


def init_state(model: str, n: int, seed: int) -> list:
    rng = np.random.default_rng(seed)
    cols = [rng.uniform(lo, hi, n) for lo, hi in INIT_RANGES[model]]
    return np.stack(cols, 1).astype(np.float32).ravel().tolist()


def sub(model: str, n: int, seed: int = 0, params=None) -> SubnetworkConfig:
    return SubnetworkConfig(model, n, init_state(model, n, seed), list(params or DEFAULT_PARAMS[model]))


def sweep_values(model: str, n_sweep: int) -> list:
    lo, hi = SWEEP_VALUES[model]
    return np.linspace(lo, hi, n_sweep).astype(np.float32).tolist()


def single_model(model: str, n: int = 20, integrator: str = "heun", coupling: str = "Linear",
                 cparams=(0.1,), weights="scalar", delays=(), nsig=0.0, seed: int = 0, dt: float = 0.1,
                 monitors=None, density: float = 0.3) -> SimConfig:
    """One subnetwork coupled to itself."""
    if weights == "scalar":
        w = 0.5
    elif weights == "dense":
        c = connectome(n, density, seed + 7)
        w = c.dense().tolist()
    else:
        c = connectome(n, density, seed + 7)
        w = c.csr_weights()
        if delays == "per_edge":
            delays = tract_lengths_to_delays(c.lengths, 30.0, dt)
        elif delays == "per_edge_long":  # every delay >= 17 steps
            delays = tract_lengths_to_delays(c.lengths, 6.0, dt)
    return SimConfig(sim_length=1000.0, dt=dt, integrator=integrator, nsig=nsig, monitors=list(monitors or []),
                     network=NetworkConfig([sub(model, n, seed)],
                                           [ProjectionConfig(0, 0, w, coupling_fn=coupling,
                                                             coupling_params=list(cparams), delays=list(delays))]))


def three_subnet_ring(n: int = 12, integrator: str = "heun", delays=(0, 0, 0)) -> SimConfig:
    """G2DO -> JR -> WC -> G2DO ring (the reference's 3-subnetwork benchmark topology)."""
    subs = [sub("Generic2dOscillator", n, 1), sub("JansenRit", n, 2), sub("WilsonCowan", n, 3)]
    projs = [
        ProjectionConfig(0, 1, 0.05, coupling_fn="Linear", coupling_params=[0.1], delays=[delays[0]]),
        ProjectionConfig(1, 2, connectome(n, 0.4, 5).csr_weights(), coupling_fn="Sigmoidal",
                         coupling_params=[0.0, 1.0, 0.0, 1.0, 1.0], delays=[delays[1]]),
        ProjectionConfig(2, 0, connectome(n, 0.4, 6).dense().tolist(), coupling_fn="Linear",
                         coupling_params=[0.2, 0.01], delays=[delays[2]]),
    ]
    return SimConfig(sim_length=1000.0, dt=0.1, integrator=integrator, network=NetworkConfig(subs, projs))


def noise_for(cfg: SimConfig, n_steps: int, n_sweep: int, per_point: bool, seed: int) -> np.ndarray:
    row = sum(s.nnodes * s.nmodes * MODEL_REGISTRY[s.model][0] for s in cfg.network.subnetworks)
    shape = (n_steps, n_sweep, row) if per_point else (n_steps, row)
    return np.random.default_rng(seed).standard_normal(shape, dtype=np.float32)
