"""Host-side mirror of hyburn's ``BatchHybridEngine`` API over the GB300 C-ABI library.

Names, arguments and result layouts follow src/engine/batch_engine/engine.rs so that code written
against the reference reads the same:

    engine = BatchHybridEngine.from_config(config, n_sweep=3)
    result = engine.run_sweep(SweepParam(sub_idx=0, param_idx=1), [-0.5, 0.0, 0.5], 100)
    result.tavg[0]      # flat [n_sweep, nnodes*nmodes, nvar]

Every simulation step runs in the CUDA kernels of ``libhyburn_gb300.so``; there is no host
fallback: if the library or a GPU is missing, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from itertools import product
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _abi
from .config import (BackendError, DeviceTimeout, InvalidConfig, InvalidState, IOError_, NonFinite, SimConfig,
                     SimulationError, Unsupported, resolve_initial_state)


@dataclass
class SweepParam:
    """engine.rs:33-39."""

    sub_idx: int
    param_idx: int


@dataclass
class SweepPoint:
    """engine.rs:41-50."""

    sub_idx: int
    param_idx: int
    values: List[float]


@dataclass
class SweepSpec:
    """engine.rs:52-91."""

    points: List[SweepPoint]

    def n_sweep(self) -> int:
        n = 1
        for p in self.points:
            n *= len(p.values)
        return n

    def cartesian_product(self) -> List[List[Tuple[int, int, float]]]:
        """Last dimension varies fastest (engine.rs:69-90)."""
        out = []
        for combo in product(*[range(len(p.values)) for p in self.points]):
            out.append([(p.sub_idx, p.param_idx, p.values[i]) for p, i in zip(self.points, combo)])
        return out


@dataclass
class BatchSweepResult:
    """engine.rs:14-31; arrays are flat in the reference's memory order."""

    param_values: np.ndarray
    tavg: List[np.ndarray]
    final_states: List[np.ndarray]
    trajectories: Optional[List[np.ndarray]]
    bold: Optional[List[np.ndarray]]
    elapsed_ms: float
    n_sweep: int


_ERRORS = {
    _abi.HB_ERR_INVALID_CONFIG: InvalidConfig,
    _abi.HB_ERR_INVALID_STATE: InvalidState,
    _abi.HB_ERR_BACKEND: BackendError,
    _abi.HB_ERR_IO: IOError_,
    _abi.HB_ERR_CUDA: BackendError,
    _abi.HB_ERR_NONFINITE: NonFinite,
    _abi.HB_ERR_TIMEOUT: DeviceTimeout,
    _abi.HB_ERR_UNSUPPORTED: Unsupported,
}


def raise_for(status: int, message: str) -> None:
    if status == _abi.HB_OK:
        return
    raise _ERRORS.get(status, SimulationError)(message)


def noise_shape(config: SimConfig, n_steps: int, n_sweep: int, semantics: int = 0) -> Tuple[int, ...]:
    """Shape of the standard-normal array a stochastic run consumes."""
    row = 0
    for s in config.network.subnetworks:
        row += s.nnodes * s.nmodes * _abi.MODEL_INFO[s.model][0]
    if semantics & _abi.HB_SEM_NOISE_PER_POINT:
        return (n_steps, n_sweep, row)
    return (n_steps, row)


@dataclass
class FcFeatures:
    """Functional-connectivity features of a device-resident trajectory (hb_engine_fc_features;
    sbi/features/fc.rs, mod.rs:257-280)."""
    fc: np.ndarray                   # [n_sweep, nvar, nnodes, nnodes]
    features: np.ndarray             # [n_sweep, nvar, 7]: mean, std, min, max, median, homotopic mean, std
    fcd: Optional[np.ndarray]        # [n_sweep, nvar, n_windows, n_windows] or None
    fcd_stats: Optional[np.ndarray]  # [n_sweep, nvar, 5] (NaN when there is no FCD) or None
    n_windows: int
    ms: float


@dataclass
class OrderAdjointResult:
    """Time-averaged Kuramoto order parameter and its gradients (hb_engine_adjoint_order)."""
    loss: np.ndarray      # [n_sweep]
    d_gain: np.ndarray    # [n_sweep] dL/da, the coupling scale
    d_omega: np.ndarray   # [n_sweep] dL/domega for a shift of every node's omega (sum of d_omega_node)
    d_omega_node: Optional[np.ndarray] = None  # [n_sweep, nnodes] dL/domega_i
    forward_ms: float = 0.0
    prepare_ms: float = 0.0
    reverse_ms: float = 0.0


@dataclass
class AdjointResult:
    """Loss and gradients of a functional-connectivity fit (hb_engine_adjoint_fc)."""
    loss: np.ndarray          # [n_sweep]
    d_gain: np.ndarray        # [n_sweep]
    d_A: np.ndarray           # [n_sweep, nnodes]
    d_B: np.ndarray           # [n_sweep, nnodes]
    d_a: np.ndarray           # [n_sweep, nnodes]
    fc: np.ndarray            # [n_sweep, nnodes, nnodes]
    y: Optional[np.ndarray]   # [n_steps, n_sweep, nnodes] or None
    forward_ms: float = 0.0
    statistics_ms: float = 0.0
    reverse_ms: float = 0.0


class BatchHybridEngine:
    """src/engine/batch_engine/engine.rs:105-138, backed by the CUDA engine."""

    def __init__(self, config: SimConfig, n_sweep: int, semantics: int = 0):
        self._lib = _abi.load_library()
        self.config = config
        self.n_sweep = int(n_sweep)
        self.semantics = int(semantics)
        states = [resolve_initial_state(s) for s in config.network.subnetworks]
        self._sd = _abi.build_sim_desc(config, states, semantics)
        h = C.c_void_p()
        st = self._lib.hb_engine_create(C.byref(self._sd.desc), self.n_sweep, C.byref(h))
        raise_for(st, self._lib.hb_last_error().decode())
        self._h = h
        self._hybrid = bool(self.semantics & _abi.HB_SEM_HYBRID_INTEGRATOR)
        self.models = [s.model for s in config.network.subnetworks]
        self.tune = "cache"
        self.tuned_flags: Optional[int] = None  # the autotuner's choice the last run used, if any

    def _with_tuned(self, run_flags: int, param: Optional[SweepParam] = None, values=None) -> int:
        """run_flags plus the autotuner's cached kernel choice for this shape, unless the caller chose a
        kernel form itself or tuning is off."""
        self.tuned_flags = None
        if self.tune == "off" or (run_flags & _abi.HB_RUN_KERNEL_CHOICE):
            return run_flags
        from . import autotune
        f = autotune.best_run_flags(self.config, self.n_sweep, self.semantics)
        if f is None and self.tune == "auto" and param is not None:
            f, _ = autotune.tune(self.config, self.n_sweep, param, values, self.semantics)
        self.tuned_flags = f
        return run_flags | (f or 0)

    def _run_tuned(self, call, run_flags: int, param: Optional[SweepParam] = None, values=None) -> int:
        """call(flags), an entry point of the library returning its status, with the autotuner's cached
        kernel choice added. The cache key is the network's shape; it does not see every option of a run
        (trajectories, per-node parameter tables, device memory), so when the engine refuses the cached
        choice for this run (HB_ERR_UNSUPPORTED) the call is made again with the caller's own flags, the
        engine's fixed rules: a cache entry never turns a run those rules serve into an error. Returns the
        flags of the call that ran."""
        flags = self._with_tuned(run_flags, param, values)
        st = call(flags)
        if st == _abi.HB_ERR_UNSUPPORTED and flags != run_flags:
            self.tuned_flags = None
            flags = run_flags
            st = call(flags)
        raise_for(st, self._lib.hb_last_error().decode())
        return flags

    @classmethod
    def from_config(cls, config: SimConfig, n_sweep: int, device=None, semantics: int = 0,
                    tune: str = "cache") -> "BatchHybridEngine":
        """BatchHybridEngine::from_config (engine.rs:145-471).

        `tune` selects how a run that forces no kernel form picks one: "cache" (default) uses the
        autotuner's cached choice for this network shape when there is one, else the engine's fixed
        rules; "auto" also measures the candidates on the first run of an untuned shape
        (hyburn_gb300.autotune.tune) and caches the winner; "off" always uses the fixed rules."""
        eng = cls(config, n_sweep, semantics)
        if tune not in ("cache", "auto", "off"):
            raise ValueError(f"tune must be 'cache', 'auto' or 'off', not {tune!r}")
        eng.tune = tune
        return eng

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.hb_engine_destroy(h)
            self._h = None

    def close(self) -> None:
        self.__del__()

    # ---- runs ----
    def _noise_args(self, noise, n_steps):
        if noise is None:
            return None, 0, None
        a = np.ascontiguousarray(np.asarray(noise, dtype=np.float32))
        return _abi.f32p(a), a.size, a

    def _result(self, r, record_traj: bool) -> BatchSweepResult:
        lib = self._lib
        n = C.c_int64()
        try:
            nsub = lib.hb_result_n_subnets(r)
            pv = _abi.copy_out(lib.hb_result_param_values(r, C.byref(n)), n.value)
            tavg, fin, traj = [], [], []
            for i in range(nsub):
                tavg.append(_abi.copy_out(lib.hb_result_tavg(r, i, C.byref(n)), n.value))
                fin.append(_abi.copy_out(lib.hb_result_final_states(r, i, C.byref(n)), n.value))
                if record_traj:
                    traj.append(_abi.copy_out(lib.hb_result_trajectory(r, i, C.byref(n)), n.value))
            nb = lib.hb_result_n_bold(r)
            bold = None
            if nb > 0:
                bold = []
                for m in range(nb):
                    p = lib.hb_result_bold(r, m, C.byref(n))
                    bold.append(_abi.copy_out(p, n.value) if n.value > 0 else np.zeros(0, np.float32))
            return BatchSweepResult(param_values=pv, tavg=tavg, final_states=fin,
                                    trajectories=traj if record_traj else None, bold=bold,
                                    elapsed_ms=lib.hb_result_elapsed_ms(r), n_sweep=lib.hb_result_n_sweep(r))
        finally:
            lib.hb_result_free(r)

    def run_sweep(self, param: SweepParam, param_values: Sequence[float], n_steps: int,
                  noise=None, run_flags: int = 0, output_dir: Optional[str] = None) -> BatchSweepResult:
        """BatchHybridEngine::run_sweep (engine.rs:477-484). With `output_dir`, the library also
        writes the run's tavg_sub{i}.npy files there (cli.rs:961-970, hb_engine_write_tavg)."""
        vals = np.ascontiguousarray(np.asarray(param_values, dtype=np.float32))
        nptr, nlen, _keep = self._noise_args(noise, n_steps)
        r = C.c_void_p()
        run_flags = self._run_tuned(
            lambda f: self._lib.hb_engine_run_sweep(self._h, int(param.sub_idx), int(param.param_idx), _abi.f32p(vals),
                                                    vals.size, int(n_steps), int(f), nptr, nlen, C.byref(r)),
            run_flags, param, vals)
        if output_dir is not None:
            st = self._lib.hb_engine_write_tavg(self._h, r, os.fsencode(output_dir))
            if st != _abi.HB_OK:
                msg = self._lib.hb_last_error().decode()
                self._lib.hb_result_free(r)
                raise_for(st, msg)
        return self._result(r, bool(run_flags & _abi.HB_RUN_TRAJECTORY))

    def run_sweep_with_trajectory(self, param: SweepParam, param_values, n_steps: int, noise=None,
                                  run_flags: int = 0) -> BatchSweepResult:
        """BatchHybridEngine::run_sweep_with_trajectory (engine.rs:487-494)."""
        return self.run_sweep(param, param_values, n_steps, noise, run_flags | _abi.HB_RUN_TRAJECTORY)

    def run_sweep_multi(self, spec: SweepSpec, n_steps: int, noise=None, run_flags: int = 0) -> BatchSweepResult:
        """BatchHybridEngine::run_sweep_multi (engine.rs:845-851)."""
        arr, keep = _abi.sweep_points(spec.points)
        nptr, nlen, _keep = self._noise_args(noise, n_steps)
        r = C.c_void_p()
        run_flags = self._run_tuned(
            lambda f: self._lib.hb_engine_run_sweep_multi(self._h, arr, len(spec.points), int(n_steps), int(f),
                                                          nptr, nlen, C.byref(r)),
            run_flags)
        return self._result(r, bool(run_flags & _abi.HB_RUN_TRAJECTORY))

    def run_sweep_multi_with_trajectory(self, spec: SweepSpec, n_steps: int, noise=None, run_flags: int = 0):
        return self.run_sweep_multi(spec, n_steps, noise, run_flags | _abi.HB_RUN_TRAJECTORY)

    # ---- state ----
    @property
    def step(self) -> int:
        return int(self._lib.hb_engine_step(self._h))

    @property
    def states(self) -> List[np.ndarray]:
        out = []
        for i, s in enumerate(self.config.network.subnetworks):
            nv = _abi.MODEL_INFO[s.model][0]
            a = np.zeros((self.n_sweep, s.nnodes * s.nmodes, nv), dtype=np.float32)
            st = self._lib.hb_engine_get_state(self._h, i, _abi.f32p(a), a.size)
            raise_for(st, self._lib.hb_last_error().decode())
            out.append(a)
        return out

    def reset(self) -> None:
        raise_for(self._lib.hb_engine_reset(self._h), self._lib.hb_last_error().decode())

    @property
    def hybrid_integrator(self) -> bool:
        """The public field `hybrid_integrator` (engine.rs:125): Heun for Generic2dOscillator
        subnetworks and Euler for the others (engine.rs:697-702). Set it between runs, as callers of
        the reference do after from_config; created from the HB_SEM_HYBRID_INTEGRATOR semantics flag."""
        return bool(self._hybrid)

    @hybrid_integrator.setter
    def hybrid_integrator(self, on: bool) -> None:
        raise_for(self._lib.hb_engine_set_hybrid_integrator(self._h, 1 if on else 0), self._lib.hb_last_error().decode())
        self._hybrid = bool(on)

    def set_stream(self, stream_handle: Optional[int]) -> None:
        raise_for(self._lib.hb_engine_set_stream(self._h, C.c_void_p(stream_handle or 0)),
                  self._lib.hb_last_error().decode())

    def fc_features(self, sub_idx: int = 0, window_len: int = 0, stride: int = 1) -> FcFeatures:
        """FC, FC statistics and, with window_len > 0, FCD of the last run's trajectory, which must
        have been kept on the device (run_flags HB_RUN_DEVICE_TRAJECTORY); computed on the GPU."""
        q = _abi.hb_fc_features()
        st = self._lib.hb_engine_fc_features(self._h, int(sub_idx), int(window_len), int(stride), C.byref(q))
        raise_for(st, self._lib.hb_last_error().decode())
        B, N, nvar, nw = self.n_sweep, q.nnodes, q.nvar, q.n_windows
        fc = np.empty((B, nvar, N, N), np.float32)
        feat = np.empty((B, nvar, 7), np.float32)
        fcd = np.empty((B, nvar, max(nw, 1), max(nw, 1)), np.float32)
        fcds = np.empty((B, nvar, 5), np.float32)
        out = _abi.hb_fc_features()
        out.fc, out.features = _abi.f32p(fc), _abi.f32p(feat)
        out.fcd, out.fcd_stats = _abi.f32p(fcd), _abi.f32p(fcds)
        st = self._lib.hb_engine_fc_features(self._h, int(sub_idx), int(window_len), int(stride), C.byref(out))
        raise_for(st, self._lib.hb_last_error().decode())
        return FcFeatures(fc=fc, features=feat, fcd=fcd if nw else None, fcd_stats=fcds if window_len else None,
                          n_windows=int(nw), ms=float(out.ms))

    def adjoint_order(self, gain_values, n_steps: int, run_flags: int = 0) -> OrderAdjointResult:
        """Kuramoto: loss = time average of the order parameter R over n_steps from the initial state
        (the engine is reset), with the coupling scale a = gain_values[b] per point; gradients with
        respect to a and to omega (per node, and for a shift of all nodes) by the discrete adjoint on the GPU."""
        g = np.ascontiguousarray(np.asarray(gain_values, np.float32))
        B = self.n_sweep
        n = self.config.network.subnetworks[0].nnodes
        loss, dg, dw = (np.zeros(B, np.float64) for _ in range(3))
        dwn = np.zeros((B, n), np.float64)
        out = _abi.hb_order_adjoint_out()
        dp = C.POINTER(C.c_double)
        out.loss, out.d_gain, out.d_omega, out.d_omega_node = (a.ctypes.data_as(dp) for a in (loss, dg, dw, dwn))
        self._run_tuned(lambda f: self._lib.hb_engine_adjoint_order(self._h, _abi.f32p(g), g.size, int(n_steps), int(f),
                                                                     C.byref(out)), run_flags)
        return OrderAdjointResult(loss, dg, dw, dwn, out.forward_ms, out.prepare_ms, out.reverse_ms)

    def adjoint_fc(self, gain_values, n_steps: int, target_fc, checkpoint_every: int = 500,
                   return_y: bool = False) -> AdjointResult:
        """Loss mean((FC - target_fc)^2) of y1 - y2 per sweep point and its gradients with respect to
        the coupling gain and the per-node JansenRit A, B, a (discrete adjoint, FP64 accumulation)."""
        vals = np.ascontiguousarray(np.asarray(gain_values, dtype=np.float32))
        n = self.config.network.subnetworks[0].nnodes
        tgt = np.ascontiguousarray(np.asarray(target_fc, dtype=np.float32).reshape(n, n))
        B = vals.size
        loss, dg = np.zeros(B), np.zeros(B)
        dA, dB, da = np.zeros((B, n)), np.zeros((B, n)), np.zeros((B, n))
        fc = np.zeros((B, n, n), np.float32)
        y = np.zeros((n_steps, B, n), np.float32) if return_y else None
        dp = C.POINTER(C.c_double)
        out = _abi.hb_adjoint_out()
        out.loss, out.d_gain = loss.ctypes.data_as(dp), dg.ctypes.data_as(dp)
        out.d_A, out.d_B, out.d_a = dA.ctypes.data_as(dp), dB.ctypes.data_as(dp), da.ctypes.data_as(dp)
        out.fc = _abi.f32p(fc)
        out.y = _abi.f32p(y) if y is not None else C.POINTER(C.c_float)()
        st = self._lib.hb_engine_adjoint_fc(self._h, _abi.f32p(vals), B, int(n_steps), _abi.f32p(tgt),
                                            int(checkpoint_every), C.byref(out))
        raise_for(st, self._lib.hb_last_error().decode())
        return AdjointResult(loss, dg, dA, dB, da, fc, y, out.forward_ms, out.statistics_ms, out.reverse_ms)

    def prepare(self, param: SweepParam, param_values, n_steps: int, noise=None, run_flags: int = 0) -> None:
        vals = np.ascontiguousarray(np.asarray(param_values, dtype=np.float32))
        nptr, nlen, _keep = self._noise_args(noise, n_steps)
        self._run_tuned(lambda f: self._lib.hb_engine_prepare(self._h, int(param.sub_idx), int(param.param_idx),
                                                               _abi.f32p(vals), vals.size, int(n_steps), int(f), nptr, nlen),
                        run_flags, param, vals)

    def execute_prepared(self) -> None:
        raise_for(self._lib.hb_engine_execute_prepared(self._h), self._lib.hb_last_error().decode())

    def last_kernel_time(self) -> Tuple[float, int, int]:
        ms, n, kind = C.c_double(), C.c_int64(), C.c_int32()
        raise_for(self._lib.hb_engine_last_kernel_time(self._h, C.byref(ms), C.byref(n), C.byref(kind)),
                  self._lib.hb_last_error().decode())
        return ms.value, n.value, kind.value


class GroupedSweep:
    """Several engines' sweeps in one kernel launch replayed from a CUDA graph (hb_group_*).

    ``members`` is a list of ``(engine, SweepParam, values, n_steps, noise)`` tuples; the engines
    may differ in model, node count, connectome, delays, coupling function, sweep values and step
    count. Each member must be one the streamed-history kernel serves: one subnetwork, one sparse
    projection with per-edge delays of at least 15 steps (HB_SEM_DELAY_RING), and no trajectory. The
    launch is a persistent work-queue kernel whose blocks (or thread-block clusters) take (member,
    point) items from a device counter. ``execute()`` restarts every member from its initial state and
    runs all of them; ``results()`` returns one BatchSweepResult per member.
    """

    def __init__(self, members, run_flags: int = 0, stream_handle: Optional[int] = None):
        self._lib = _abi.load_library()
        self._engines = [m[0] for m in members]
        if not (run_flags & _abi.HB_RUN_KERNEL_CHOICE):
            # the autotuner's streamed-history form (nodes per consumer thread, L2 prefetch) when every
            # tuned member chose the same one
            from . import autotune
            picks = {f & _abi.HB_RUN_STREAM_FORM for f in
                     (autotune.best_run_flags(e.config, e.n_sweep, e.semantics) for e in self._engines
                      if e.tune != "off") if f is not None and f & _abi.HB_RUN_STREAM}
            if len(picks) == 1:
                run_flags |= picks.pop()
        keep = []
        arr = (_abi.hb_group_member * len(members))()
        for i, (eng, param, values, n_steps, noise) in enumerate(members):
            vals = np.ascontiguousarray(np.asarray(values, dtype=np.float32))
            keep.append(vals)
            nptr, nlen, nk = eng._noise_args(noise, n_steps)
            keep.append(nk)
            arr[i].engine = eng._h
            arr[i].sub_idx, arr[i].param_idx = int(param.sub_idx), int(param.param_idx)
            arr[i].values, arr[i].n_values = _abi.f32p(vals), vals.size
            arr[i].n_steps, arr[i].run_flags = int(n_steps), int(run_flags)
            arr[i].noise = nptr if nptr is not None else C.POINTER(C.c_float)()
            arr[i].noise_len = nlen
        h = C.c_void_p()
        st = self._lib.hb_group_prepare(arr, len(members), C.c_void_p(stream_handle) if stream_handle else None,
                                        C.byref(h))
        raise_for(st, self._lib.hb_last_error().decode())
        self._h = h

    def execute(self) -> None:
        raise_for(self._lib.hb_group_execute(self._h), self._lib.hb_last_error().decode())

    def results(self) -> List[BatchSweepResult]:
        out = []
        for i, eng in enumerate(self._engines):
            r = C.c_void_p()
            raise_for(self._lib.hb_group_result(self._h, i, C.byref(r)), self._lib.hb_last_error().decode())
            out.append(eng._result(r, False))
        return out

    def last_kernel_time(self) -> float:
        ms = C.c_double()
        raise_for(self._lib.hb_group_last_kernel_time(self._h, C.byref(ms)), self._lib.hb_last_error().decode())
        return ms.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.hb_group_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

