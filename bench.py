"""Benchmark of the batched neural-mass simulation step on GB300.

Workload (one "step" = one full run of the hot path over one batch):
  Generic2dOscillator, 74 nodes, 128 sweep points over the Linear coupling scale a in
  linspace(0, 0.05); symmetric 20%-dense connectome with log-normal(0,1) weights / max; tract
  lengths U[10, 200] mm at 3 mm/ms with dt 0.1 ms -> per-edge integer delays (up to ~667 steps);
  Heun-stochastic, nsig 1e-3 with a seeded N(0,1) draw array shared by all points, 20 000 steps,
  FP32. All inputs are synthetic (numpy default_rng seeds), no dataset.
Metric: node-steps/s (points x nodes x steps / time), whole job over all ranks.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

value: device-resident run (inputs already in HBM), CUDA events on the engine's stream, L2
flushed between timed iterations. e2e: the public API call (host noise in pinned memory -> H2D,
run, D2H of tavg / final states) timed on the host. The reference arm times the CPU oracle
(restatement of the reference's NdArray path) on all host cores on a bounded sample.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_NODES, N_POINTS, N_STEPS = 74, 128, 20_000
WORKLOAD = "g2do-74n-128pt-csr20pct-per-edge-delays-heun-stochastic-20000steps"
METRIC = "node-steps/s"
FLUSH_BYTES = 512 << 20
KERNEL_NAMES = {1: "point-resident persistent (generic)", 2: "point-resident persistent (single projection)",
                3: "point-resident warp-specialised pipeline"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def issue_roofline(prof, n_run, kern_ms, clocks, hbm):
    """Roofline of the pipeline kernel on the roof that binds it, instruction issue.

    achieved = warp instructions of one launch ÷ the launch's CUDA-event duration; the instruction count
    is the one-launch ncu count of this workload (`smsp__inst_executed.sum`, recorded with the kernel's
    start-up and steady-state instructions per step, scaled to n_run steps); peak = one warp instruction
    per cycle on each of the four schedulers of every SM at the SM clock sampled during the timed
    region. The HBM figure rides along as `hbm`."""
    ss, st = prof.get("warp_instructions_per_step_steady"), prof.get("warp_instructions_startup")
    sms = prof.get("sm_count", 152)
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz") or 2070.0
    out = {"bound": "issue", "unit": "G warp-instructions/s", "kernel_ms_per_launch": kern_ms, "hbm": hbm}
    if ss is None or st is None or not kern_ms:
        out.update(achieved=None, peak=None, frac=None, traffic=hbm["traffic"],
                   note="instruction count not recorded for this kernel build")
        return out
    inst = float(st) + float(ss) * n_run
    achieved = inst / (kern_ms / 1e3) / 1e9
    peak = 4.0 * sms * mhz * 1e6 / 1e9
    out.update(achieved=achieved, peak=peak, frac=achieved / peak, traffic=hbm["traffic"],
               warp_instructions_per_launch=inst, sms_with_work=prof.get("ctas_per_launch"),
               issue_active_ncu=prof.get("issue_active_pct"),
               peak_kind="4 schedulers x %d SMs x %.0f MHz (sampled)" % (sms, mhz))
    return out


def dense_roofline(B, T, ms, clocks, tensor):
    """Roofline of the tensor-core dense kernel on the roof that binds it, instruction issue of its FP32
    epilogue: warp instructions of one launch (the committed one-launch ncu counts per CTA and step,
    profiles/dense_tc_kernel_counts.json, times the launch's CTAs and steps) over the event time, against
    one warp instruction per cycle on the 4 schedulers of every SM at the sampled SM clock. The tensor
    pipe's figures ride along as `tensor`."""
    prof = os.path.join(ROOT, "profiles", "dense_tc_kernel_counts.json")
    out = {"bound": "issue", "unit": "G warp-instructions/s", "tensor": tensor, "traffic": None}
    try:
        d = json.load(open(prof))
    except Exception:
        out.update(achieved=None, peak=None, frac=None, note="instruction counts not recorded")
        return out
    ctas = (B + 127) // 128
    inst = ctas * (d["warp_instructions_per_cta_step"] * T + d["warp_instructions_startup_per_cta"])
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz") or 2070.0
    peak = 4.0 * 152 * mhz * 1e6 / 1e9
    achieved = inst / (ms / 1e3) / 1e9
    out.update(achieved=achieved, peak=peak, frac=achieved / peak, sms_with_work=ctas,
               frac_of_sms_with_work=achieved / (peak * min(ctas, 152) / 152),
               issue_active_ncu=d.get("issue_active_pct"), tensor_pipe_active_ncu=d.get("tensor_pipe_active_pct"),
               peak_kind="4 schedulers x 152 SMs x %.0f MHz (sampled)" % mhz)
    return out


def peaks_tf32():
    """Dense TF32 tensor rate: half the measured bf16 burst rate."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]) / 2.0
    except Exception:
        return 1900.0 / 2.0


class ClockSampler:
    """Samples SM clocks and throttle reasons while the timed region runs: one `nvidia-smi -lms 20`
    process started (and seen answering) before the region, stopped after it; only the samples that
    arrive inside the region are kept."""

    QUERY = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int, period_ms: int = 20):
        self.index = index
        self.period_ms = period_ms
        self.samples = []
        self._all = []
        self._proc = None
        self._thr = None
        self._first = threading.Event()
        self._t0 = self._t1 = None

    def _read(self):
        for line in self._proc.stdout:
            parts = [x.strip() for x in line.strip().split(",")]
            if len(parts) >= 7:
                self._all.append((time.perf_counter(), parts))
                self._first.set()

    def __enter__(self):
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                           "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._thr = threading.Thread(target=self._read, daemon=True)
            self._thr.start()
            self._first.wait(5.0)
        except OSError:
            self._proc = None
        self._t0 = time.perf_counter()
        return self

    def __exit__(self, *a):
        self._t1 = time.perf_counter()
        if self._proc is not None:
            time.sleep(2 * self.period_ms / 1e3)
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
            if self._thr:
                self._thr.join(timeout=5)
        inside = [p for t, p in self._all if self._t0 <= t <= self._t1 + self.period_ms / 1e3]
        self.samples = inside or [p for _, p in self._all[-1:]]

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def workload(n_steps=N_STEPS, n_points=N_POINTS):
    from hyburn_gb300 import inputs

    cfg, meta = inputs.batched_sweep(n_steps=n_steps, n_points=n_points)
    noise = inputs.standard_normal((n_steps, N_NODES * 2), 2)
    return cfg, meta, noise


def workload_config(n_run=N_STEPS) -> dict:
    """The benchmark workload as both arms' lines name it: the same keys and values on each."""
    from hyburn_gb300 import inputs

    _, meta = inputs.batched_sweep(n_steps=1, n_points=1)  # the delays depend on the connectome alone
    return {"workload": WORKLOAD, "points_per_gpu": N_POINTS, "nodes": N_NODES, "steps_per_run": n_run,
            "delays": f"per edge {meta['min_delay']}-{meta['max_delay']} steps",
            "l2": "flushed (512 MiB write) between timed GPU iterations"}


# The reference's published time for its own batch-sweep benchmark, generic BatchHybridEngine on Burn
# CUDA, 1024 points x 1000 steps: (node-steps/s, source) per population size
RING3_PUBLISHED = {76: (6.49e8, "docs/BENCHMARK.md:16-20 (360 ms)"), 164: (1.48e9, "docs/BENCHMARK.md:30-38 (341 ms)")}


def ring3_workload(nnodes: int, n_points: int, n_steps: int):
    """The generic-engine workload of the reference's CUDA benchmark, the one its published 3-population
    times are for (examples/bench/hyburn_bench_generic_cuda.rs:21-56, 116-131): a G2DO -> JansenRit ->
    WilsonCowan ring, `nnodes` nodes per population from a zero state with default parameters, all-to-all
    Scalar weights 0.01 with Linear(1.0) coupling and no delay, Heun at dt 0.1 with the hybrid integrator
    set after from_config (Heun for G2DO, Euler for JansenRit and WilsonCowan); G2DO's I swept as
    -0.5 + i / (n - 1) in f32."""
    from hyburn_gb300.config import DEFAULT_PARAMS, NetworkConfig, ProjectionConfig, SimConfig, SubnetworkConfig
    subs = [SubnetworkConfig(m, nnodes, [0.0] * (nv * nnodes), list(DEFAULT_PARAMS[m]))
            for m, nv in (("Generic2dOscillator", 2), ("JansenRit", 6), ("WilsonCowan", 2))]
    projs = [ProjectionConfig(s, t, 0.01, coupling_fn="Linear", coupling_params=[1.0], delays=[0])
             for s, t in ((0, 1), (1, 2), (2, 0))]
    cfg = SimConfig(sim_length=n_steps * 0.1, dt=0.1, integrator="heun", network=NetworkConfig(subs, projs))
    f = np.float32
    values = [float(f(-0.5) + f(i) / f(max(n_points - 1, 1))) for i in range(n_points)]
    return cfg, values


# The reference's published single-model CUDA times, 256 points x 76 nodes x 1000 steps, in ms per point
# (docs/BENCHMARK.md:50-58; Kuramoto, listed there as ~0.30, is not in the benchmark's model loop)
SINGLE_MODEL_PUBLISHED_MS_PER_POINT = {"G2DO": 0.28, "WC": 0.35, "MPR": 0.37, "JR": 0.41}
SINGLE_MODELS = {"G2DO": ("Generic2dOscillator", 2), "JR": ("JansenRit", 6), "WC": ("WilsonCowan", 2),
                 "MPR": ("MontbrioPazoRoxin", 2)}


def single_model_workload(short: str, n_points: int = 256, nnodes: int = 76):
    """The single-model part of the reference's CUDA benchmark (examples/bench/hyburn_bench_generic_cuda.rs:
    60-107): one population of `nnodes` uncoupled nodes (no projection) from a zero state, default
    parameters (MPR: [1, 1, -5, 15, 0, 1, 0]), Euler at dt 0.1; parameter 1 swept (MPR: 2) as
    -0.5 + i / (n - 1) in f32. Only G2DO's index 1 is batch-native, so for the other models the batch engine
    ignores the sweep (dfun.rs:49-72) and every point runs the same network, as in the reference.
    Returns (config, SweepParam indices, values)."""
    from hyburn_gb300.config import DEFAULT_PARAMS, NetworkConfig, SimConfig, SubnetworkConfig
    model, nvar = SINGLE_MODELS[short]
    params = [1.0, 1.0, -5.0, 15.0, 0.0, 1.0, 0.0] if short == "MPR" else list(DEFAULT_PARAMS[model])
    cfg = SimConfig(sim_length=10.0, dt=0.1, integrator="euler",
                    network=NetworkConfig([SubnetworkConfig(model, nnodes, [0.0] * (nvar * nnodes), params)], []))
    f = np.float32
    values = [float(f(-0.5) + f(i) / f(max(n_points - 1, 1))) for i in range(n_points)]
    return cfg, (0, 2 if short == "MPR" else 1), values


# The reference's published parameter-sweep times of its example configurations on Burn CUDA (RTX 4090),
# 128 points x 74 nodes x 10 000 steps: (node-steps/s, source); the configurations and sweep values are
# those of the committed golden fixtures example_g2do_sweep and example_mpr_sweep
EXAMPLE_SWEEP_PUBLISHED = {"g2do": (5.20e7, "docs/BENCHMARK_EXAMPLES.md:32 (1.82 s)"),
                           "mpr": (3.66e7, "docs/BENCHMARK_EXAMPLES.md:33 (2.59 s)")}


def example_sweep_case(name: str):
    """The reference's example sweep (examples/g2do_sweep.toml with examples/sweep.toml, or
    examples/mpr_sweep.toml with examples/sweep_mpr.toml) as stored in the golden fixture."""
    tests = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests")
    if tests not in sys.path:
        sys.path.insert(0, tests)
    from golden.make_golden import load_case
    return load_case({"g2do": "example_g2do_sweep", "mpr": "example_mpr_sweep"}[name])


def algorithmic_bytes_per_node_step(meta, n_points=N_POINTS) -> float:
    """Delayed reads of the coupling variable (4 B per in-edge), the ring write (4 B) and the
    shared noise draws (2 x 4 B per node per step, read once for all points)."""
    c = meta["connectome"]
    return 4.0 * c.nnz / c.n + 4.0 + 8.0 / n_points


def cpu_reference(n_points, steps_sample, n_threads):
    """Times the CPU oracle on a bounded sample of the workload; returns node-steps/s."""
    from hyburn_gb300 import SweepParam
    from hyburn_gb300._abi import HB_SEM_DELAY_RING
    from oracle.hb_oracle import OracleEngine

    cfg, meta, noise = workload(steps_sample, n_points)
    eng = OracleEngine(cfg, n_points, semantics=HB_SEM_DELAY_RING, n_threads=n_threads)
    t0 = time.perf_counter()
    eng.run_sweep(SweepParam(-1, 0), meta["values"], steps_sample, noise=noise)
    dt = time.perf_counter() - t0
    return n_points * N_NODES * steps_sample / dt, dt


def calibrated_cpu_reference(n_threads, target_s=12.0):
    """Oracle rate on about target_s seconds of the workload: a prefix of its steps when the
    whole run would take longer, else whole runs repeated."""
    rate, dt = cpu_reference(N_POINTS, 100, n_threads)
    steps = int(max(100, min(N_STEPS, rate * target_s / (N_POINTS * N_NODES))))
    reps = 1
    if steps == N_STEPS:
        reps = max(1, int(round(target_s / (N_POINTS * N_NODES * N_STEPS / rate))))
    total_t = 0.0
    for _ in range(reps):
        _, dt = cpu_reference(N_POINTS, steps, n_threads)
        total_t += dt
    rate = reps * N_POINTS * N_NODES * steps / total_t
    sample = f"{reps} run(s) of {N_POINTS} points x {N_NODES} nodes x {steps} steps of the same workload ({total_t:.1f} s)"
    return rate, sample


CPU_BASELINE_NOTE = ("the oracle: a C restatement (-O3, no fused multiply-add) of the reference's NdArray batch "
                     "path, OpenMP over sweep points like rayon_batch_sweep (engine.rs:1363-1429); it is not the "
                     "reference's NdArray code, which the reference publishes at 3.62e6 node-steps/s on 32 EPYC "
                     "cores for a simpler undelayed 128 x 74 G2DO sweep (docs/BENCHMARK_EXAMPLES.md:32)")


def cpu_baseline_line(target_s=12.0):
    """The oracle timed on all host cores (value) and on one core, each on a bounded sample."""
    n_threads = os.cpu_count() or 1
    rate, sample = calibrated_cpu_reference(n_threads, target_s)
    rate1, sample1 = calibrated_cpu_reference(1, target_s)
    return {"value": rate, "unit": "node-steps/s", "cores": n_threads, "kind": "port", "sample": sample,
            "single_thread": {"value": rate1, "cores": 1, "sample": sample1}, "note": CPU_BASELINE_NOTE}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(x: float, world: int, backend_ready: bool) -> float:
    if world == 1 or not backend_ready:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference_arm(args):
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return
    n_threads = os.cpu_count() or 1
    vals = []
    sample = ""
    for _ in range(args.warmup):
        cpu_reference(N_POINTS, 50, n_threads)
    for _ in range(args.steps):
        rate, sample = calibrated_cpu_reference(n_threads, target_s=max(2.0, 30.0 / max(args.steps, 1)))
        vals.append(rate)
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "node-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(),
            "cpu_baseline": {"value": v, "unit": "node-steps/s", "cores": n_threads, "kind": "port",
                             "sample": sample, "note": CPU_BASELINE_NOTE},
            "e2e": {"value": v, "unit": "node-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


class PlainTorchSweep:
    """The batched sweep step as plain per-operation GPU work (the comparator of the fused kernel):
    per step, a gather of the delayed coupling variable of every edge from a [R, B, N] history,
    a scatter-add over targets, the Linear coupling, the G2DO derivatives and the stochastic Heun
    stages as element-wise tensor operations, and the history write — about twenty kernels,
    replayed from a CUDA graph of `graph_steps` steps so that launch overhead does not dominate.
    Ring semantics of runtime.rs:162-204 (current state at step 0, zero before time 0)."""

    def __init__(self, cfg, values, noise, graph_steps=50):
        import torch
        dev = torch.device("cuda")
        sub, proj = cfg.network.subnetworks[0], cfg.network.projections[0]
        n = sub.nnodes
        w = proj.weights
        indptr = np.asarray(w["indptr"])
        self.tgt = torch.tensor(np.repeat(np.arange(n), np.diff(indptr)), device=dev)
        self.src = torch.tensor(np.asarray(w["indices"]), device=dev)
        self.w = torch.tensor(np.asarray(w["data"], np.float32), device=dev)
        self.d = torch.tensor(np.asarray(proj.delays, np.int64), device=dev)
        self.R = int(max(proj.delays)) + 1
        self.B, self.n, self.dt = len(values), n, cfg.dt
        self.a = torch.tensor(np.asarray(values, np.float32), device=dev)[:, None]
        self.b = float(proj.coupling_params[1]) if len(proj.coupling_params) > 1 else 0.0
        self.p = [float(v) for v in sub.params]
        self.scale = float(np.sqrt(2.0 * cfg.nsig) * np.sqrt(cfg.dt))
        self.noise = torch.tensor(np.asarray(noise, np.float32), device=dev).reshape(-1, n, 2)
        x0 = torch.tensor(np.asarray(sub.initial_state, np.float32), device=dev).reshape(n, 2)
        self.x0 = x0[None].expand(self.B, n, 2).contiguous()
        self.graph_steps = graph_steps
        self.x = self.x0.clone()
        self.ring = torch.zeros(self.R, self.B, n, device=dev)
        self.s = torch.zeros((), dtype=torch.int64, device=dev)
        self.graph = None

    def _dfun(self, v, w, c):
        p = self.p
        tau, a_, b_, c_, d_, e_, f_, g_ = max(p[0], 1.1920929e-07), p[2], p[3], p[4], p[5], p[6], p[7], p[8]
        alpha, beta, gamma = p[9], p[10], p[11]
        iext = c * gamma + gamma * p[1]
        v2 = v * v
        dv = (w * alpha + iext - v * v2 * f_ + v2 * e_ + v * g_) * (d_ * tau)
        dw = (v * b_ + v2 * c_ - w * beta + a_) * (d_ / tau)
        return dv, dw

    def _step(self):
        import torch
        s = self.s
        t = s - self.d
        idx = torch.remainder(t, self.R)
        vals = self.ring[idx, :, self.src]                                    # [nnz, B]
        cur = self.x[:, :, 0].t()[self.src]                                   # step 0 reads the current state
        vals = torch.where((s == 0), cur, torch.where((t >= 0)[:, None], vals, torch.zeros_like(vals)))
        g = torch.zeros(self.n, self.B, device=vals.device).index_add_(0, self.tgt, vals * self.w[:, None]).t()
        c = g * self.a + self.b
        nz = self.noise.index_select(0, s.view(1))[0] * self.scale           # [n, 2], shared by all points
        v, w = self.x[..., 0], self.x[..., 1]
        k1v, k1w = self._dfun(v, w, c)
        pv, pw = v + k1v * self.dt + nz[:, 0], w + k1w * self.dt + nz[:, 1]
        k2v, k2w = self._dfun(pv, pw, c)
        v = v + (k1v + k2v) * (0.5 * self.dt) + nz[:, 0]
        w = w + (k1w + k2w) * (0.5 * self.dt) + nz[:, 1]
        self.x.copy_(torch.stack([v, w], -1))
        self.ring.index_copy_(0, torch.remainder(s + 1, self.R).view(1), v[None])
        self.s.add_(1)

    def run(self, n_steps):
        """n_steps steps from the initial state (a multiple of graph_steps)."""
        import torch
        self.x.copy_(self.x0)
        self.ring.zero_()
        self.s.zero_()
        self.ring[0] = self.x0[:, :, 0]
        if self.graph is None:
            st = torch.cuda.Stream()
            st.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(st):
                for _ in range(3):
                    self._step()
            torch.cuda.current_stream().wait_stream(st)
            self.x.copy_(self.x0)
            self.ring.zero_()
            self.s.zero_()
            self.ring[0] = self.x0[:, :, 0]
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph):
                for _ in range(self.graph_steps):
                    self._step()
            self.x.copy_(self.x0)
            self.ring.zero_()
            self.s.zero_()
            self.ring[0] = self.x0[:, :, 0]
        for _ in range(n_steps // self.graph_steps):
            self.graph.replay()
        return self.x


def run_plain_arm(args):
    """The same workload and metric as the default line, computed by PlainTorchSweep on a bounded
    number of steps of the run (the per-step cost is constant)."""
    import torch
    torch.cuda.set_device(0)
    n_run = 2000
    cfg, meta, noise = workload(n_run)
    plain = PlainTorchSweep(cfg, meta["values"], noise)
    plain.run(plain.graph_steps)
    torch.cuda.synchronize()
    times = []
    for _ in range(max(1, args.steps)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        plain.run(n_run)
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = statistics.median(times)
    node_steps = N_POINTS * N_NODES * n_run
    print(json.dumps({"impl": "plain", "metric": METRIC, "value": node_steps / (ms / 1e3), "unit": "node-steps/s",
                      "n_gpus": 1, "steps": args.steps, "warmup": 1, "ms_per_step": ms * N_STEPS / n_run,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                      "data": "synthetic",
                      "config": {"workload": WORKLOAD, "sample": f"{n_run} of {N_STEPS} steps",
                                 "form": "per-operation tensor kernels, 50-step CUDA graphs"}}), flush=True)


def _time_prepared(eng, steps, warmup):
    """CUDA-event time per execute_prepared() of an engine, L2 flushed before each timed run."""
    import torch
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(warmup):
        eng.execute_prepared()
    torch.cuda.synchronize()
    ms = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        eng.execute_prepared()
        ms.append(eng.last_kernel_time()[0])
    return statistics.median(ms), eng.last_kernel_time()[2]


def run_other_workload(args):
    """The other measured configurations (synthetic inputs with the stated shapes), one JSON line."""
    import torch
    from hyburn_gb300 import BatchHybridEngine, GroupedSweep, SweepParam, inputs
    from hyburn_gb300._abi import HB_SEM_BOLD_PER_POINT, HB_SEM_DELAY_RING
    torch.cuda.set_device(0)
    peak, peak_kind = peaks()
    line = {"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "l2": "flushed (512 MiB write) before each timed run"}
    with ClockSampler(0) as clk:
        if args.workload == "single":
            # one simulation: G2DO, 74 nodes, Heun dt 0.1, 10 000 steps, w = 0.01 mean-field Linear coupling
            T = args.run_steps or 10_000
            cfg, meta = inputs.plain_single_sim(T)
            eng = BatchHybridEngine.from_config(cfg, 1)
            eng.prepare(SweepParam(0, 1), [cfg.network.subnetworks[0].params[1]], T)
            ms, kind = _time_prepared(eng, args.steps, args.warmup)
            value = 74 * T / (ms / 1e3)
            # published for examples/g2do_simple.toml, the same network and steps (its initial state from
            # examples/init_g2do_74.npy): CUDA 4.44 s, CPU 0.67 s (docs/BENCHMARK_EXAMPLES.md:15)
            pub_cuda, pub_cpu = 74 * 10_000 / 4.44, 74 * 10_000 / 0.67
            line.update(metric="node-steps/s", value=value, unit="node-steps/s", ms_per_step=ms,
                        vs_baseline=value / pub_cuda if T == 10_000 else None,
                        baseline={"published_node_steps_per_s": pub_cuda, "backend": "Burn CUDA on an RTX 4090 (serial engine)",
                                  "published_cpu_node_steps_per_s": pub_cpu, "source": "docs/BENCHMARK_EXAMPLES.md:15"},
                        config={"workload": f"g2do-74n-1pt-meanfield-heun-{T}steps", "kernel_kind": kind},
                        roofline={"bound": "latency", "note": "one point on one SM; no roofline fraction",
                                  "us_per_integration_step": ms * 1e3 / T})
        elif args.workload == "kuramoto":
            # Kuramoto, 1000 nodes, 5 % CSR, delays U[10,250] mm at 5 mm/ms, 256 points over G, BOLD on
            T = args.run_steps or 10_000
            cfg, meta = inputs.kuramoto_scale(n=1000, n_points=256, n_steps=T, bold=True)
            eng = BatchHybridEngine.from_config(cfg, 256, semantics=HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT)
            from hyburn_gb300._abi import HB_RUN_PIPE_LANES, HB_RUN_STREAM_BULK, HB_RUN_STREAM_CLUSTER, HB_RUN_STREAM_NPT
            eng.prepare(SweepParam(-1, 0), meta["values"], T,
                        run_flags=(HB_RUN_STREAM_CLUSTER(args.stream_cluster) if args.stream_cluster else 0) |
                        HB_RUN_STREAM_NPT(args.stream_npt) | HB_RUN_PIPE_LANES(args.pipe_lanes) |
                        (HB_RUN_STREAM_BULK if args.stream_bulk else 0))
            ms, kind = _time_prepared(eng, args.steps, args.warmup)
            nnz = sum(len(p.weights["data"]) for p in cfg.network.projections)
            bpns = 4.0 * nnz / 1000 + 4.0
            ns = 256 * 1000 * T
            line.update(metric="node-steps/s", value=ns / (ms / 1e3), unit="node-steps/s", ms_per_step=ms,
                        config={"workload": f"kuramoto-1000n-256pt-csr5pct-delays-{meta['min_delay']}-{meta['max_delay']}"
                                            f"-heun-bold-{T}steps (of 100000)", "kernel_kind": kind,
                                "omega": "per node, N(0, 1) (seed 5)",
                                "ctas_per_point": args.stream_cluster or "engine's choice",
                                "nodes_per_consumer_thread": args.stream_npt or "engine's choice",
                                "producer_lanes_per_node": args.pipe_lanes or "engine's choice",
                                "windows_staged_by_bulk_copies": bool(args.stream_bulk)},
                        roofline={"bound": "hbm", "achieved": bpns * ns / (ms / 1e3) / 1e9, "peak": peak,
                                  "unit": "GB/s", "frac": bpns * ns / (ms / 1e3) / 1e9 / peak, "peak_kind": peak_kind,
                                  "algorithmic_bytes_per_node_step": bpns, "traffic": None})
        elif args.workload == "uneven":
            # MPR, {68, 84, 164, 400} nodes x 128 points, (G, eta) grid, RK4 dt 0.05, BOLD TR 2 s, one launch
            T = args.run_steps or 20_000
            members, ns, bytes_ = [], 0, 0.0
            for n in (68, 84, 164, 400):
                # 16 coupling scales G x 8 values of eta per size; eta through per-point parameter tables
                cfg, meta = inputs.mpr_grid(n, 128, T, seed=3, bold=True)
                eng = BatchHybridEngine.from_config(cfg, 128, semantics=HB_SEM_DELAY_RING)
                members.append((eng, SweepParam(-1, 0), meta["values"], T, None))
                nnz = len(cfg.network.projections[0].weights["data"])
                ns += 128 * n * T
                bytes_ += 128 * T * (8.0 * nnz + 8.0 * n)
            from hyburn_gb300._abi import HB_RUN_PIPE_LANES
            from hyburn_gb300._abi import HB_RUN_STREAM_CLUSTER
            g = GroupedSweep(members, run_flags=HB_RUN_PIPE_LANES(args.pipe_lanes) |
                             (HB_RUN_STREAM_CLUSTER(args.stream_cluster) if args.stream_cluster else 0))
            for _ in range(args.warmup):
                g.execute()
            times = []
            for _ in range(args.steps):
                g.execute()
                times.append(g.last_kernel_time())
            ms = statistics.median(times)
            line.update(metric="node-steps/s", value=ns / (ms / 1e3), unit="node-steps/s", ms_per_step=ms,
                        config={"workload": f"mpr-68/84/164/400n-x128pt-(G16xeta8)-csr20pct-per-edge-delays-rk4-dt0.05-bold-"
                                            f"{T}steps (of 1200000), one grouped launch", "kernel_kind": 5,
                                "grid": "per size: G in linspace(0, 1, 16) x eta in linspace(-6, -3, 8)",
                                "producer_lanes_per_node": args.pipe_lanes or "engine's choice",
                                "ctas_per_point_of_split_members": args.stream_cluster or "engine's choice"},
                        roofline={"bound": "hbm", "achieved": bytes_ / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                                  "frac": bytes_ / (ms / 1e3) / 1e9 / peak, "peak_kind": peak_kind,
                                  "algorithmic_bytes_per_node_step": bytes_ / ns, "traffic": None})
        elif args.workload == "kuramoto-adjoint":
            # Kuramoto 1000 nodes x 256 points (the kuramoto workload's network): loss = time average of
            # the order parameter over T steps, gradients w.r.t. the coupling scale and omega
            T = args.run_steps or 2_000
            cfg, meta = inputs.kuramoto_scale(n=1000, n_points=256, n_steps=T, bold=False)
            eng = BatchHybridEngine.from_config(cfg, 256, semantics=HB_SEM_DELAY_RING)
            eng.prepare(SweepParam(-1, 0), meta["values"], T)
            fwd_ms, _ = _time_prepared(eng, args.steps, args.warmup)
            for _ in range(max(1, args.warmup)):
                eng.adjoint_order(meta["values"], T)
            tot, parts = [], None
            for _ in range(args.steps):
                r = eng.adjoint_order(meta["values"], T)
                tot.append(r.forward_ms + r.prepare_ms + r.reverse_ms)
                parts = (r.forward_ms, r.prepare_ms, r.reverse_ms)
            ms = statistics.median(tot)
            eng.close()
            line.update(metric="gradient evaluations/s", value=256 / (ms / 1e3), unit="points/s", ms_per_step=ms,
                        config={"workload": f"kuramoto-1000n-256pt-csr5pct-delays-{meta['min_delay']}-{meta['max_delay']}"
                                            f"-heun-{T}steps-order-parameter-loss",
                                "omega": "per node, N(0, 1) (seed 5)",
                                "gradients": "coupling scale, omega per node", "trajectory": "kept in HBM"},
                        adjoint={"forward_ms": parts[0], "prepare_ms": parts[1], "reverse_ms": parts[2],
                                 "plain_forward_ms": fwd_ms, "fwd_plus_adjoint_over_forward": ms / fwd_ms})
        elif args.workload == "dense":
            # undelayed all-to-all dense coupling (the reference's batched matrix product, engine.rs:609-620):
            # G2DO, 74 nodes, weights U[0, 1) / 74 off the diagonal, Linear coupling swept over the points,
            # Heun, 2 000 steps; the tensor-core path (HB_RUN_DENSE_TC) beside the engine's CUDA-core kernel
            from hyburn_gb300._abi import HB_RUN_DENSE_TC
            from hyburn_gb300.config import NetworkConfig, ProjectionConfig, SimConfig, SubnetworkConfig
            T, n, B = args.run_steps or 2_000, 74, args.dense_points
            rng = np.random.default_rng(7)
            w = (rng.uniform(0.0, 1.0, (n, n)) / n).astype(np.float32)
            np.fill_diagonal(w, 0.0)
            cfg = SimConfig(sim_length=T * 0.1, dt=0.1, integrator="heun", nsig=0.0, network=NetworkConfig(
                [SubnetworkConfig("Generic2dOscillator", n, inputs.uniform_state(n, 2, 7), list(inputs.G2DO_BENCH_PARAMS))],
                [ProjectionConfig(0, 0, w.tolist(), coupling_fn="Linear", coupling_params=[0.1])]))
            vals = np.linspace(0.0, 0.2, B).astype(np.float32)
            res = {}
            for name, flags in (("tensor_core", HB_RUN_DENSE_TC), ("cuda_core", 0)):
                eng = BatchHybridEngine.from_config(cfg, B, tune="off")
                eng.prepare(SweepParam(-1, 0), vals, T, run_flags=flags)
                res[name] = _time_prepared(eng, args.steps, args.warmup)
                eng.close()
            ms, kind = res["tensor_core"]
            ns = B * n * T
            np_, kp = (n + 15) // 16 * 16, (n + 7) // 8 * 8
            issued = 3 * 2 * ((B + 127) // 128 * 128) * np_ * kp * T  # flops the tensor cores execute (3 x TF32, padded)
            useful = 2 * B * n * n * T
            line.update(metric="node-steps/s", value=ns / (ms / 1e3), unit="node-steps/s", ms_per_step=ms,
                        config={"workload": f"g2do-{n}n-{B}pt-dense-undelayed-heun-{T}steps", "kernel_kind": kind},
                        dense={"tensor_core_ms": ms, "cuda_core_ms": res["cuda_core"][0],
                               "cuda_core_kernel_kind": res["cuda_core"][1],
                               "cuda_core_node_steps_per_s": ns / (res["cuda_core"][0] / 1e3),
                               "speedup_over_cuda_core": res["cuda_core"][0] / ms},
                        roofline=dense_roofline(B, T, ms, None, {
                                  "bound": "tensor", "achieved": issued / (ms / 1e3) / 1e12,
                                  "peak": peaks_tf32(), "unit": "TFLOP/s",
                                  "frac": issued / (ms / 1e3) / 1e12 / peaks_tf32(),
                                  "peak_kind": "half the measured dense bf16 burst (TF32 runs at half the bf16 rate)",
                                  "useful_tflops": useful / (ms / 1e3) / 1e12, "traffic": None}))
        elif args.workload == "ring3":
            # the reference's own batch-sweep benchmark (generic engine): 3-population ring, 1024 points x
            # 1000 Heun steps, against its published Burn CUDA time
            T, n, B = args.run_steps or 1000, args.ring_nodes, 1024
            cfg, vals = ring3_workload(n, B, T)
            eng = BatchHybridEngine.from_config(cfg, B)
            eng.hybrid_integrator = True  # as the reference's benchmark sets it (hyburn_bench_generic_cuda.rs:54)
            eng.prepare(SweepParam(0, 1), vals, T)
            ms, kind = _time_prepared(eng, args.steps, args.warmup)
            eng.close()
            ns = B * 3 * n * T
            value = ns / (ms / 1e3)
            pub = RING3_PUBLISHED.get(n)
            line.update(metric="node-steps/s", value=value, unit="node-steps/s", ms_per_step=ms,
                        vs_baseline=(value / pub[0]) if pub and T == 1000 else None,
                        config={"workload": f"ring3-g2do-jr-wc-{n}n-per-population-{B}pt-scalar-heun-{T}steps",
                                "kernel_kind": kind,
                                "integrator": "hybrid: Heun for G2DO, Euler for JansenRit and WilsonCowan",
                                "source": "examples/bench/hyburn_bench_generic_cuda.rs, generic BatchHybridEngine"},
                        baseline={"published_node_steps_per_s": pub[0] if pub else None,
                                  "backend": "Burn CUDA on an RTX 4090, generic BatchHybridEngine with the hybrid "
                                             "integrator", "source": pub[1] if pub else None},
                        roofline={"bound": "latency", "note": "the generic resident kernel's per-step block barrier "
                                  "and mean-field reductions; no DRAM or tensor roof binds (no history, 1 point per CTA)",
                                  "us_per_integration_step": ms * 1e3 / T})
        elif args.workload == "single-model":
            # the single-model part of the reference's CUDA benchmark: 256 uncoupled points x 76 nodes x
            # 1000 Euler steps, against its published ms per point
            T, B, n = args.run_steps or 1000, 256, 76
            cfg, (si, pi), vals = single_model_workload(args.model, B, n)
            eng = BatchHybridEngine.from_config(cfg, B)
            eng.prepare(SweepParam(si, pi), vals, T)
            ms, kind = _time_prepared(eng, args.steps, args.warmup)
            eng.close()
            value = B * n * T / (ms / 1e3)
            pub_ms = SINGLE_MODEL_PUBLISHED_MS_PER_POINT[args.model]
            pub = B * n * T / (pub_ms * B / 1e3)
            line.update(metric="node-steps/s", value=value, unit="node-steps/s", ms_per_step=ms,
                        vs_baseline=value / pub if T == 1000 else None,
                        config={"workload": f"{args.model.lower()}-{n}n-{B}pt-uncoupled-euler-{T}steps",
                                "kernel_kind": kind,
                                "source": "examples/bench/hyburn_bench_generic_cuda.rs, single-model loop"},
                        baseline={"published_node_steps_per_s": pub, "published_ms_per_point": pub_ms,
                                  "backend": "Burn CUDA on an RTX 4090, generic BatchHybridEngine",
                                  "source": "docs/BENCHMARK.md:50-58"},
                        roofline={"bound": "latency", "note": "uncoupled nodes: per-step integration only, no "
                                  "history, no DRAM or tensor roof binds", "us_per_integration_step": ms * 1e3 / T})
        elif args.workload == "example-sweep":
            # the reference's example parameter sweeps, against its published Burn CUDA times; `value` is the
            # device-resident run, `e2e` the public run_sweep call with host values and host results
            case = example_sweep_case(args.example)
            from hyburn_gb300._abi import MODEL_INFO
            B, n = case.n_sweep, case.cfg.network.subnetworks[0].nnodes
            nvar = MODEL_INFO[case.cfg.network.subnetworks[0].model][0]
            T = args.run_steps or case.n_steps
            eng = BatchHybridEngine.from_config(case.cfg, B)
            eng.prepare(case.param, case.values, T)
            ms, kind = _time_prepared(eng, args.steps, args.warmup)
            eng.close()
            eng2 = BatchHybridEngine.from_config(case.cfg, B)
            for _ in range(max(1, args.warmup)):
                eng2.reset()
                eng2.run_sweep(case.param, case.values, T)
            wall = []
            for _ in range(args.steps):
                eng2.reset()
                t0 = time.perf_counter()
                eng2.run_sweep(case.param, case.values, T)
                wall.append(time.perf_counter() - t0)
            eng2.close()
            ns = B * n * T
            value, pub = ns / (ms / 1e3), EXAMPLE_SWEEP_PUBLISHED[args.example]
            line.update(metric="node-steps/s", value=value, unit="node-steps/s", ms_per_step=ms,
                        vs_baseline=value / pub[0] if T == case.n_steps else None,
                        e2e={"value": ns / statistics.median(wall), "unit": "node-steps/s",
                             "h2d_bytes_per_step": 4 * B, "d2h_bytes_per_step": 2 * 4 * B * n * nvar},
                        config={"workload": f"example-{args.example}-sweep-{n}n-{B}pt-{T}steps", "kernel_kind": kind,
                                "source": case.source},
                        baseline={"published_node_steps_per_s": pub[0], "backend": "Burn CUDA on an RTX 4090",
                                  "source": pub[1]},
                        roofline={"bound": "latency", "note": "mean-field coupling without delay: per-step work "
                                  "of one warp per point, no history, no DRAM or tensor roof binds",
                                  "us_per_integration_step": ms * 1e3 / T})
        elif args.workload == "fc":
            # the benchmark sweep (G2DO 74 nodes x 128 points, per-edge delays, Heun-stochastic) with its
            # trajectory kept in HBM and FC / FCD features computed there (windows of 2 000 steps, stride
            # 500), against the same run streaming its trajectory to the host (the reference's per-step copy)
            from hyburn_gb300._abi import HB_RUN_DEVICE_TRAJECTORY, HB_RUN_TRAJECTORY
            T = args.run_steps or 20_000
            W, S = min(2000, T // 2), max(1, min(500, T // 8))
            cfg, meta, noise = workload(T)
            eng = BatchHybridEngine.from_config(cfg, N_POINTS, semantics=HB_SEM_DELAY_RING)
            eng.prepare(SweepParam(-1, 0), meta["values"], T, noise=noise, run_flags=HB_RUN_DEVICE_TRAJECTORY)
            flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
            for _ in range(args.warmup):
                eng.execute_prepared()
                eng.fc_features(0, W, S)
            run_ms, feat_ms, wall = [], [], []
            for _ in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                eng.execute_prepared()
                f = eng.fc_features(0, W, S)
                wall.append((time.perf_counter() - t0) * 1e3)
                run_ms.append(eng.last_kernel_time()[0])
                feat_ms.append(f.ms)
            eng2 = BatchHybridEngine.from_config(cfg, N_POINTS, semantics=HB_SEM_DELAY_RING)
            eng2.run_sweep(SweepParam(-1, 0), meta["values"], min(T, 2000), noise=noise[:min(T, 2000)],
                           run_flags=HB_RUN_TRAJECTORY)
            eng2.reset()
            t0 = time.perf_counter()
            eng2.run_sweep(SweepParam(-1, 0), meta["values"], T, noise=noise, run_flags=HB_RUN_TRAJECTORY)
            host_traj_ms = (time.perf_counter() - t0) * 1e3
            ms = statistics.median(run_ms) + statistics.median(feat_ms)
            ns = N_POINTS * N_NODES * T
            line.update(metric="node-steps/s", value=ns / (ms / 1e3), unit="node-steps/s", ms_per_step=ms,
                        config={"workload": f"g2do-74n-128pt-csr20pct-per-edge-delays-heun-stochastic-{T}steps"
                                            f"-device-trajectory-fc-fcd-w{W}-s{S}", "n_windows": f.n_windows},
                        fc={"run_ms": statistics.median(run_ms), "features_ms": statistics.median(feat_ms),
                            "wall_ms_run_plus_features_with_d2h_of_features": statistics.median(wall),
                            "host_trajectory_run_ms": host_traj_ms,
                            "trajectory_bytes": T * N_POINTS * N_NODES * 2 * 4})
            eng.close()
            eng2.close()
        else:
            # adjoint: JR 74 nodes x 64 points, Sigmoidal delayed CSR coupling, Heun dt 0.1, 20 000 steps,
            # FC loss of y1 - y2; gradients w.r.t. the coupling gain and per-node A, B, a
            T, n, B = args.run_steps or 20_000, 74, 64
            cfg, meta = inputs.jr_fc_adjoint(T, B, n)
            gains = meta["gains"]
            eng = BatchHybridEngine.from_config(cfg, B, semantics=HB_SEM_DELAY_RING)
            eng.prepare(SweepParam(-1, 3), gains, T)
            fwd_ms, _ = _time_prepared(eng, args.steps, args.warmup)
            eng.reset()
            target = inputs.jr_target_fc(cfg, T)
            K = 500
            for _ in range(max(1, args.warmup)):
                eng.adjoint_fc(gains, T, target, checkpoint_every=K)
            tot, parts = [], None
            for _ in range(args.steps):
                r = eng.adjoint_fc(gains, T, target, checkpoint_every=K)
                tot.append(r.forward_ms + r.statistics_ms + r.reverse_ms)
                parts = (r.forward_ms, r.statistics_ms, r.reverse_ms)
            ms = statistics.median(tot)
            line.update(metric="gradient evaluations/s", value=B / (ms / 1e3), unit="points/s", ms_per_step=ms,
                        higher_is_better=True,
                        config={"workload": f"jr-74n-64pt-sigmoidal-csr-delays-heun-{T}steps-fc-loss",
                                "gradients": "coupling gain, per-node A, B, a",
                                "checkpoint_every": K, "target_fc": "FC of y1 - y2 of a seeded forward run (gain 1, initial state seed 40)"},
                        adjoint={"forward_ms": parts[0], "statistics_ms": parts[1], "reverse_ms": parts[2],
                                 "plain_forward_ms": fwd_ms, "fwd_plus_adjoint_over_forward": ms / fwd_ms})
    line["clocks"] = clk.summary()
    if args.workload == "dense" and line.get("roofline", {}).get("bound") == "issue":
        # the issue peak at the SM clock sampled during the timed region
        r = line["roofline"]
        line["roofline"] = dense_roofline(args.dense_points, args.run_steps or 2_000, line["ms_per_step"],
                                          line["clocks"], r["tensor"])
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference", "plain"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--run-steps", type=int, default=None,
                    help="integration steps per run (smaller values only for profiler captures)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--lanes", type=int, default=0, help="threads per node (0: the engine's choice)")
    ap.add_argument("--two-phase", action="store_true", help="batch each block's gathers before its updates")
    ap.add_argument("--no-pipe", action="store_true", help="do not use the warp-specialised pipeline")
    ap.add_argument("--pipe-lanes", type=int, default=0,
                    help="pipeline and streamed-history kernels: producer threads per node (0: engine's choice)")
    ap.add_argument("--stream-cluster", type=int, default=0,
                    help="streamed-history kernel: CTAs per sweep point, 1-6 or 8 (0: the engine's choice); "
                         "uneven workload: the grouped launch's cluster size (0: the engine's choice)")
    ap.add_argument("--stream-bulk", action="store_true",
                    help="Kuramoto workload: stage the gathered windows by the bulk-copy engine (HB_RUN_STREAM_BULK)")
    ap.add_argument("--dense-points", type=int, default=1024, help="dense workload: sweep points")
    ap.add_argument("--stream-npt", type=int, default=0,
                    help="streamed-history kernel: nodes per consumer thread, 1/2/4 (0: engine's choice)")
    ap.add_argument("--ring-nodes", type=int, default=76, help="ring3 workload: nodes per population (76 or 164)")
    ap.add_argument("--model", default="G2DO", choices=sorted(SINGLE_MODELS), help="single-model workload: the model")
    ap.add_argument("--example", default="g2do", choices=sorted(EXAMPLE_SWEEP_PUBLISHED),
                    help="example-sweep workload: the reference's example sweep")
    ap.add_argument("--workload", default="sweep", choices=["sweep", "single", "uneven", "adjoint", "kuramoto", "kuramoto-adjoint",
                                                          "fc", "dense", "ring3", "single-model",
                                                          "example-sweep"],
                    help="sweep: the 128-point batched sweep (default); the others are the remaining "
                         "measured configurations, one JSON line each")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference_arm(args)
        return
    if args.impl == "plain":
        run_plain_arm(args)
        return
    if args.workload != "sweep":
        run_other_workload(args)
        return
    if args.run_steps is None:
        args.run_steps = N_STEPS

    import torch

    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    backend_ready = False
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        backend_ready = True

    from hyburn_gb300 import BatchHybridEngine, SweepParam
    from hyburn_gb300._abi import HB_SEM_DELAY_RING

    n_run = args.run_steps
    cfg, meta, noise = workload(n_run)
    param = SweepParam(-1, 0)
    eng = BatchHybridEngine.from_config(cfg, N_POINTS, semantics=HB_SEM_DELAY_RING)
    stream = torch.cuda.Stream()
    eng.set_stream(stream.cuda_stream)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    # ---- device-resident runs (value) ----
    from hyburn_gb300._abi import HB_RUN_LANES
    from hyburn_gb300._abi import HB_RUN_NO_PIPE, HB_RUN_PIPE_LANES, HB_RUN_TWO_PHASE
    run_flags = ((HB_RUN_LANES(args.lanes) if args.lanes else 0) | (HB_RUN_TWO_PHASE if args.two_phase else 0)
                 | (HB_RUN_NO_PIPE if args.no_pipe else 0) | HB_RUN_PIPE_LANES(args.pipe_lanes))
    eng.prepare(param, meta["values"], n_run, noise=noise, run_flags=run_flags)
    for _ in range(args.warmup):
        eng.execute_prepared()
    torch.cuda.synchronize()
    if backend_ready:
        torch.distributed.barrier()
    times, kern = [], []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                eng.execute_prepared()
                e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            ms_k, launches, kind = eng.last_kernel_time()
            kern.append((ms_k, launches))
        torch.cuda.synchronize()
    if backend_ready:
        torch.distributed.barrier()
    total_ms = reduce_max(sum(times), world, backend_ready)
    node_steps = N_POINTS * N_NODES * n_run
    value = world * node_steps * args.steps / (total_ms / 1e3)

    # dominant kernel: the resident simulation kernel, its launches timed on the engine stream
    kern_ms = sum(k for k, _ in kern) / max(1, sum(n for _, n in kern))
    bpns = algorithmic_bytes_per_node_step(meta)
    achieved = bpns * node_steps / (kern_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    traffic, prof_d = None, {}
    prof = os.path.join(ROOT, "profiles", "resident_pipe_kernel_traffic.json")
    if os.path.exists(prof):
        try:
            prof_d = json.load(open(prof))
            traffic = prof_d.get("dram_bytes_per_launch")
        except Exception:
            traffic, prof_d = None, {}

    # ---- end to end through the public API (pinned host noise, H2D, run, D2H) ----
    e2e = None
    h2d = noise.nbytes + 4 * N_POINTS
    d2h = 2 * 4 * N_POINTS * N_NODES * 2
    if not args.no_e2e:
        pinned = torch.from_numpy(noise).pin_memory()
        host_noise = pinned.numpy()
        eng2 = BatchHybridEngine.from_config(cfg, N_POINTS, semantics=HB_SEM_DELAY_RING)
        for _ in range(max(1, args.warmup)):
            eng2.reset()
            eng2.run_sweep(param, meta["values"], n_run, noise=host_noise, run_flags=run_flags)
        torch.cuda.synchronize()
        if backend_ready:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            eng2.reset()
            r = eng2.run_sweep(param, meta["values"], n_run, noise=host_noise, run_flags=run_flags)
        e2e_s = reduce_max(time.perf_counter() - t0, world, backend_ready)
        e2e = world * node_steps * args.steps / e2e_s

    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": "node-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(n_run),
        "impl_detail": {"kernel": KERNEL_NAMES.get(kind, str(kind)), "parallelism": f"sweep points sharded, {world} replica(s)"},
        "roofline": issue_roofline(prof_d, n_run, kern_ms, clocks,
                                   {"bound": "hbm (notional: the history lives in shared memory)", "achieved": achieved,
                                    "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                                    "peak_kind": peak_kind, "algorithmic_bytes_per_node_step": bpns}),
        "e2e": {"value": e2e, "unit": "node-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(sum(n for _, n in kern)),
        "clocks": clocks,
    }
    # the CPU baseline is timed at N = 1 only, so that no GPU of a multi-rank job idles meanwhile
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_line()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if backend_ready:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
