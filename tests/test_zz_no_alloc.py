"""hb_noalloc_run_csr_sweep: the sweep entry point that allocates no device memory.

It serves callers that cannot call cudaMalloc — a framework whose own arena owns the device's
memory, or a loop that cannot afford cudaMalloc's implicit synchronisation — by keeping its
network tables and history ring in a fixed static device array instead. This test gives it
inputs and outputs that the test itself allocated on the device, runs it twice in a row (the
second call reuses the array the first one left behind), and checks both results against the
engine's regular entry point within the parity tolerance of the other GPU tests.
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


def _close(a, b, what):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    err = np.abs(a - b) / (ATOL + RTOL * np.abs(b))
    assert err.max() <= 1.0, f"{what}: max scaled error {err.max():.3g}"


def test_noalloc_sweep_matches_engine_on_two_consecutive_calls():
    import torch

    from hyburn_gb300 import BatchHybridEngine, SweepParam, inputs
    from hyburn_gb300._abi import HB_INT, HB_SEM_DELAY_RING, f32p

    lib, fn = _bind()
    n_steps, n_points, n = 700, 16, 74
    cfg, meta = inputs.batched_sweep(n_steps=n_steps, n_points=n_points)
    c = meta["connectome"]
    proj = cfg.network.projections[0]
    sub = cfg.network.subnetworks[0]
    noise = inputs.standard_normal((n_steps, n * 2), 7)
    dev = torch.device("cuda", 0)
    d_x0 = torch.tensor(np.asarray(sub.initial_state, np.float32), device=dev)
    d_indptr = torch.tensor(c.indptr.astype(np.int32), device=dev)
    d_indices = torch.tensor(c.indices.astype(np.int32), device=dev)  # same bits as uint32 here
    d_delays = torch.tensor(np.asarray(proj.delays, np.int32), device=dev)
    d_weights = torch.tensor(c.data, device=dev)
    d_noise = torch.tensor(noise, device=dev)
    params = np.asarray(sub.params, np.float32)
    cparams = np.asarray(proj.coupling_params, np.float32)
    nsig = np.asarray(cfg.nsig_vec(2), np.float32)
    stream = torch.cuda.current_stream(dev)

    for call, values in enumerate((meta["values"], list(reversed(meta["values"])))):
        vals = np.asarray(values, np.float32)
        d_final = torch.full((n_points, n, 2), float("nan"), device=dev)
        d_tavg = torch.full((n_points, n, 2), float("nan"), device=dev)
        st = fn(b"Generic2dOscillator", f32p(params), params.size, n, d_x0.data_ptr(), d_indptr.data_ptr(),
                d_indices.data_ptr(), d_delays.data_ptr(), d_weights.data_ptr(), c.nnz, int(meta["max_delay"]),
                b"Linear", f32p(cparams), cparams.size, -1, 0, f32p(vals), n_points, cfg.dt,
                HB_INT[cfg.integrator], f32p(nsig), nsig.size, d_noise.data_ptr(), d_noise.numel(), n_steps,
                d_final.data_ptr(), d_tavg.data_ptr(), C.c_void_p(stream.cuda_stream))
        assert st == 0, lib.hb_last_error().decode()
        torch.cuda.synchronize()
        ref = BatchHybridEngine.from_config(cfg, n_points, semantics=HB_SEM_DELAY_RING).run_sweep(
            SweepParam(-1, 0), vals, n_steps, noise=noise)
        _close(d_final.cpu().numpy().ravel(), ref.final_states[0], f"final states, call {call + 1}")
        _close(d_tavg.cpu().numpy().ravel(), ref.tavg[0], f"temporal average, call {call + 1}")


def test_noalloc_rejects_sweeps_larger_than_its_array():
    import torch

    lib, fn = _bind()
    from hyburn_gb300._abi import HB_ERR_UNSUPPORTED, f32p

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
