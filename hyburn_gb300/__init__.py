"""GB300-native implementation of hyburn's batched neural-mass simulation step.

The public surface mirrors the reference's engine API (src/engine/batch_engine/engine.rs) and
TOML configuration (src/config.rs); the compute runs in hand-written sm_103a CUDA kernels loaded
from the in-tree C-ABI library ``hyburn_gb300/_lib/libhyburn_gb300.so``.
"""
from .config import (BackendError, DeviceTimeout, InvalidConfig, InvalidState, IOError_, MonitorConfig, NetworkConfig,
                     NonFinite, ProjectionConfig, SimConfig, SimulationError, SubnetworkConfig, SweepConfig,
                     Unsupported, parse_sweep_param)
from .engine import BatchHybridEngine, BatchSweepResult, GroupedSweep, SweepParam, SweepPoint, SweepSpec, noise_shape

__all__ = [
    "BatchHybridEngine", "BatchSweepResult", "GroupedSweep", "SweepParam", "SweepPoint", "SweepSpec", "SimConfig",
    "NetworkConfig", "SubnetworkConfig", "ProjectionConfig", "MonitorConfig", "SweepConfig",
    "parse_sweep_param", "noise_shape", "SimulationError", "InvalidConfig", "InvalidState", "BackendError",
    "IOError_", "NonFinite", "Unsupported", "DeviceTimeout",
]
