"""hb_noalloc_run_csr_sweep: the sweep entry point that allocates no device memory.

It serves callers that cannot call cudaMalloc — a framework whose own caching allocator or arena
owns the device's memory — by keeping its network tables and history ring in a fixed static
device array instead. These tests give it inputs and outputs that the test itself allocated on
the device, run it twice in a row (the second call reuses the array the first one left behind),
and check both results against the engine's regular entry point within the parity tolerance of
the other GPU tests. The cases cover the history ring in shared memory (74 nodes) and in the
static array with the edge tables read from global memory (1000-node Kuramoto, the [sin, cos]
form of the kernel), a coupling-parameter sweep and a native model-parameter sweep, that the
second call leaves the device's free memory unchanged, and that malformed CSR input, which the
call checks on the device without waiting for it, comes back as NaN outputs.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-5, 1e-6


def _bind():
    from hyburn_gb300 import _abi

    lib = _abi.load_library()
    fn = lib.hb_noalloc_run_csr_sweep
    FP, P = C.POINTER(C.c_float), C.c_void_p
    I32, I64 = C.c_int32, C.c_int64
    fn.restype = I32
    fn.argtypes = [C.c_char_p, FP, I32, I32, P, P, P, P, P, I64, I32, C.c_char_p, FP, I32, I32, I32, FP, I32, C.c_double,
                   I32, FP, I32, P, I64, I64, P, P, P]
    return lib, fn


def _close(a, b, what, period=None):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    d = a - b
    if period is not None:  # phases: distance on the circle
        d = (d + period / 2) % period - period / 2
    err = np.abs(d) / (ATOL + RTOL * np.abs(b))
    assert err.max() <= 1.0, f"{what}: max scaled error {err.max():.3g}"


class _Case:
    """Device copies of one single-projection sweep configuration."""

    def __init__(self, cfg, meta, noise):
        import torch

        from hyburn_gb300.config import MODEL_REGISTRY

        dev = torch.device("cuda", 0)
        c = meta["connectome"]
        proj = cfg.network.projections[0]
        sub = cfg.network.subnetworks[0]
        self.cfg, self.meta, self.noise = cfg, meta, noise
        self.model = sub.model.encode()
        self.n, self.nvar = sub.nnodes, MODEL_REGISTRY[sub.model][0]
        self.nnz = c.nnz
        self.max_delay = int(max(proj.delays))
        self.d_x0 = torch.tensor(np.asarray(sub.initial_state, np.float32), device=dev)
        self.d_indptr = torch.tensor(c.indptr.astype(np.int32), device=dev)
        self.d_indices = torch.tensor(c.indices.astype(np.int32), device=dev)  # same bits as uint32 here
        self.d_delays = torch.tensor(np.asarray(proj.delays, np.int32), device=dev)
        self.d_weights = torch.tensor(c.data, device=dev)
        self.d_noise = torch.tensor(noise, device=dev) if noise is not None else None
        self.params = np.asarray(sub.params, np.float32)
        self.cfn = proj.coupling_fn.encode()
        self.cparams = np.asarray(proj.coupling_params, np.float32)
        self.nsig = np.asarray(cfg.nsig_vec(self.nvar), np.float32)
        self.stream = torch.cuda.current_stream(dev)
        self.dev = dev

    def call(self, fn, sweep_sub, sweep_idx, values, n_steps, d_delays=None):
        import torch

        from hyburn_gb300._abi import HB_INT, f32p

        vals = np.asarray(values, np.float32)
        shape = (vals.size, self.n, self.nvar)
        d_final = torch.full(shape, float("nan"), device=self.dev)
        d_tavg = torch.full(shape, float("nan"), device=self.dev)
        dl = self.d_delays if d_delays is None else d_delays
        st = fn(self.model, f32p(self.params), self.params.size, self.n, self.d_x0.data_ptr(), self.d_indptr.data_ptr(),
                self.d_indices.data_ptr(), dl.data_ptr(), self.d_weights.data_ptr(), self.nnz, self.max_delay,
                self.cfn, f32p(self.cparams), self.cparams.size, sweep_sub, sweep_idx, f32p(vals), vals.size,
                self.cfg.dt, HB_INT[self.cfg.integrator], f32p(self.nsig), self.nsig.size,
                self.d_noise.data_ptr() if self.d_noise is not None else None,
                self.d_noise.numel() if self.d_noise is not None else 0, n_steps, d_final.data_ptr(), d_tavg.data_ptr(),
                C.c_void_p(self.stream.cuda_stream))
        return st, d_final, d_tavg


def test_noalloc_sweep_matches_engine_on_two_consecutive_calls():
    import torch

    from hyburn_gb300 import BatchHybridEngine, SweepParam, inputs
    from hyburn_gb300._abi import HB_SEM_DELAY_RING

    lib, fn = _bind()
    n_steps, n_points, n = 700, 16, 74
    cfg, meta = inputs.batched_sweep(n_steps=n_steps, n_points=n_points)
    case = _Case(cfg, meta, inputs.standard_normal((n_steps, n * 2), 7))
    for call, values in enumerate((meta["values"], list(reversed(meta["values"])))):
        st, d_final, d_tavg = case.call(fn, -1, 0, values, n_steps)
        assert st == 0, lib.hb_last_error().decode()
        torch.cuda.synchronize()
        ref = BatchHybridEngine.from_config(cfg, n_points, semantics=HB_SEM_DELAY_RING).run_sweep(
            SweepParam(-1, 0), np.asarray(values, np.float32), n_steps, noise=case.noise)
        _close(d_final.cpu().numpy().ravel(), ref.final_states[0], f"final states, call {call + 1}")
        _close(d_tavg.cpu().numpy().ravel(), ref.tavg[0], f"temporal average, call {call + 1}")


def test_noalloc_ring_in_static_array_native_sweep_and_free_memory():
    """1000-node Kuramoto, 4 points: the ring (2 MB per point) lives in the static array and the
    50 000 edges are read from global memory; the sweep is over the native parameter omega. The
    second call must not change the device's free memory."""
    import torch

    from hyburn_gb300 import BatchHybridEngine, SweepParam, inputs
    from hyburn_gb300._abi import HB_RUN_NO_STREAM, HB_SEM_DELAY_RING

    lib, fn = _bind()
    n_steps, n_points = 600, 4
    cfg, meta = inputs.kuramoto_scale(n_points=n_points, n_steps=n_steps, bold=False, omega_per_node=False)
    meta = dict(meta, connectome=inputs.connectome(1000, 0.05, 5, 10.0, 250.0))
    case = _Case(cfg, meta, None)
    assert case.max_delay > 400 and case.nnz > 40_000
    eng = BatchHybridEngine.from_config(cfg, n_points, semantics=HB_SEM_DELAY_RING)
    two_pi = 2 * np.pi
    for call, values in enumerate(([0.5, 0.8, 1.1, 1.4], [1.4, 0.2, 0.9, 0.6])):
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st, d_final, d_tavg = case.call(fn, 0, 0, values, n_steps)
        assert st == 0, lib.hb_last_error().decode()
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        if call == 1:
            assert free_after == free_before, f"device free memory changed by {free_before - free_after} bytes"
        eng.reset()
        ref = eng.run_sweep(SweepParam(0, 0), np.asarray(values, np.float32), n_steps, run_flags=HB_RUN_NO_STREAM)
        _close(d_final.cpu().numpy().ravel(), ref.final_states[0], f"final phases, call {call + 1}", period=two_pi)
        _close(d_tavg.cpu().numpy().ravel(), ref.tavg[0], f"temporal average, call {call + 1}")


def test_noalloc_malformed_csr_gives_nan_outputs():
    """A delay above max_delay is caught on the device: the call returns HB_OK without waiting, the
    run uses no edges and both outputs are NaN. A valid call afterwards is unaffected."""
    import torch

    from hyburn_gb300 import inputs

    lib, fn = _bind()
    n_steps, n_points, n = 50, 2, 74
    cfg, meta = inputs.batched_sweep(n_steps=n_steps, n_points=n_points, nsig=0.0, integrator="heun")
    case = _Case(cfg, meta, None)
    bad = case.d_delays.clone()
    bad[3] = case.max_delay + 1
    st, d_final, d_tavg = case.call(fn, -1, 0, [0.01, 0.02], n_steps, d_delays=bad)
    assert st == 0, lib.hb_last_error().decode()
    torch.cuda.synchronize()
    assert torch.isnan(d_final).all() and torch.isnan(d_tavg).all()
    st, d_final, d_tavg = case.call(fn, -1, 0, [0.01, 0.02], n_steps)
    assert st == 0, lib.hb_last_error().decode()
    torch.cuda.synchronize()
    assert torch.isfinite(d_final).all() and torch.isfinite(d_tavg).all()


def test_noalloc_rejects_non_native_model_sweep_and_oversized_sweeps():
    import torch

    lib, fn = _bind()
    from hyburn_gb300._abi import HB_ERR_INVALID_CONFIG, HB_ERR_UNSUPPORTED, f32p

    dev = torch.device("cuda", 0)
    n, n_points, max_delay = 1000, 256, 65000  # ring alone: 256 * 65002 * 1000 * 4 bytes
    d = torch.zeros(n + 1, dtype=torch.int32, device=dev)
    x0 = torch.zeros(n, device=dev)
    out = torch.zeros(n_points * n, device=dev)
    vals = np.zeros(n_points, np.float32)
    params = np.ones(1, np.float32)
    st = fn(b"Kuramoto", f32p(params), 1, n, x0.data_ptr(), d.data_ptr(), None, None, None, 0, max_delay, b"Linear",
            f32p(params), 1, 0, 0, f32p(vals), n_points, 0.1, 0, f32p(params), 1, None, 0, 10, out.data_ptr(),
            out.data_ptr(), None)
    assert st == HB_ERR_UNSUPPORTED
    assert b"scratch" in lib.hb_last_error()
    g2do = np.ones(12, np.float32)
    st = fn(b"Generic2dOscillator", f32p(g2do), 12, n, x0.data_ptr(), d.data_ptr(), None, None, None, 0, 10, b"Linear",
            f32p(params), 1, 0, 3, f32p(vals), 2, 0.1, 0, f32p(params), 1, None, 0, 10, out.data_ptr(),
            out.data_ptr(), None)
    assert st == HB_ERR_INVALID_CONFIG
    assert b"native" in lib.hb_last_error()
