/*
 * hyburn_gb300.h — C ABI of the GB300-native batched neural-mass simulation engine.
 *
 * This library replaces the `BatchHybridEngine` step of hyburn 0.2.0 (Rust crate) for
 * `--backend cuda`. Every entry point below names the reference item it stands in for,
 * by the file path inside the hyburn project.
 *
 * Conventions (mirroring the reference's engine contract, src/engine/batch_engine/engine.rs):
 *   - All functions return an `hb_status`; the message of the last failure on the calling
 *     thread is returned by `hb_last_error()` (thread-local, valid until the next call).
 *   - Status codes mirror `SimulationError` (src/error.rs:6-25) plus CUDA/numeric/timeout codes.
 *   - Engines are not thread-safe (one CUDA stream each); distinct engines may be driven from
 *     distinct threads.
 *   - Result buffers are owned by the library until `hb_result_free`.
 *   - Layouts are those of `BatchSweepResult` (engine.rs:15-31): tavg / final states are
 *     [n_sweep, nnodes*nmodes, nvar] (memory order of the batch engine's state tensor),
 *     trajectories [n_steps, n_sweep, nnodes*nmodes, nvar], BOLD [n_tr, nnodes] per monitor in
 *     batch-mean mode or [n_sweep, n_tr, nnodes] in per-point mode.
 *   - All simulation arithmetic is FP32.
 */
#ifndef HYBURN_GB300_H
#define HYBURN_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HB_ABI_VERSION 2

/* ---- status codes: src/error.rs:6-25 (SimulationError) + device-side codes ---- */
typedef int32_t hb_status;
#define HB_OK                   0
#define HB_ERR_INVALID_CONFIG   1  /* SimulationError::InvalidConfig */
#define HB_ERR_INVALID_STATE    2  /* SimulationError::InvalidState */
#define HB_ERR_BACKEND          3  /* SimulationError::BackendError */
#define HB_ERR_IO               4  /* SimulationError::IOError */
#define HB_ERR_CUDA             5  /* a CUDA runtime call failed */
#define HB_ERR_NONFINITE        6  /* a state value became NaN/Inf on the device (checked runs) */
#define HB_ERR_TIMEOUT          7  /* a bounded device-side wait gave up */
#define HB_ERR_UNSUPPORTED      8  /* valid for the reference, not implemented by this engine */

/* ---- integrators: src/engine/integrator.rs:14-23 (IntegratorKind, same order) ---- */
#define HB_INT_HEUN              0
#define HB_INT_EULER             1
#define HB_INT_EULER_STOCHASTIC  2
#define HB_INT_HEUN_STOCHASTIC   3
#define HB_INT_RK4               4
#define HB_INT_RK4_STOCHASTIC    5

/* ---- weight kinds: src/config.rs (WeightsConfig) ---- */
#define HB_WEIGHTS_SCALAR 0
#define HB_WEIGHTS_DENSE  1
#define HB_WEIGHTS_CSR    2

/* ---- semantics flags (hb_sim_desc.flags) ----
 * Default (0) reproduces the batch engine exactly, including its documented quirks:
 * one delay per projection (`delays.first()`, engine.rs:410) read from the shift-window
 * history (engine.rs:541-551, 565-589), Scalar weights as w*mean over source nodes
 * (engine.rs:602-608), noise shared by all sweep points (engine.rs:729-745) and BOLD driven
 * by the mean over sweep points (engine.rs:786-801). */
#define HB_SEM_DELAY_RING       (1u << 0) /* true ring-buffer delays, per edge for CSR with
                                             len(delays)==nnz (src/engine/runtime.rs:55-85,125-211) */
#define HB_SEM_SCALAR_DIAGONAL  (1u << 1) /* Scalar weights as w*I (construction.rs:639-655) */
#define HB_SEM_BOLD_PER_POINT   (1u << 2) /* one BOLD series per sweep point */
#define HB_SEM_NOISE_PER_POINT  (1u << 3) /* noise array carries an independent draw per point */
#define HB_SEM_HYBRID_INTEGRATOR (1u << 4) /* BatchHybridEngine::hybrid_integrator = true (engine.rs:697-702) */

/* ---- run flags (hb_engine_run_* `run_flags`) ---- */
#define HB_RUN_TRAJECTORY   (1u << 0) /* run_sweep_with_trajectory (engine.rs:487-494) */
#define HB_RUN_CHECK_FINITE (1u << 1) /* fail with HB_ERR_NONFINITE if a state becomes NaN/Inf */
/* undelayed dense coupling (the batched matrix product of engine.rs:609-620) on the tensor cores: 128 sweep
   points per CTA, X * W^T by tcgen05.mma in three TF32 products (FP32 accumulation). For one subnetwork coupled
   to itself through one projection without delay, Linear / Sigmoidal / ScaledLinear coupling, a model with one
   coupling variable, up to 112 nodes, no monitors, trajectories or node_params; HB_ERR_UNSUPPORTED otherwise. */
#define HB_RUN_DENSE_TC     (1u << 2)
/* sparse coupling sums in the reference's order: one thread per target node adds its edges' terms in CSR order,
   each product and each sum rounded (no fused multiply-add), as the reference's per-edge loop
   (runtime.rs:162-204); slower than the default, which splits a node's edges over lanes and fuses the
   multiply-adds (results agree within the FP32 rounding of the sum). With it, a model without transcendental
   functions reproduces the FP32 reference arithmetic bit for bit. */
#define HB_RUN_EXACT_SUMS   (1u << 3)
/* streamed-history kernel, warp-cooperative gather: each lane stages its edge's window of history into
   shared memory with the bulk-copy engine (cp.async.bulk, completion on a per-warp mbarrier, bounded
   waits) instead of loading it; refused when the warp-cooperative gather is not in use */
#define HB_RUN_STREAM_BULK    (1u << 7)
#define HB_RUN_FORCE_RESIDENT (1u << 8) /* kernel choice: point-resident persistent kernel */
#define HB_RUN_FORCE_BLOCKED  (1u << 9) /* kernel choice: time-blocked tiled kernel */
#define HB_RUN_GLOBAL_RING    (1u << 10) /* resident kernel: keep the history ring in global memory */
#define HB_RUN_GENERIC        (1u << 11) /* resident kernel: use the general form even for one-projection networks */
#define HB_RUN_TWO_PHASE      (1u << 16) /* specialised kernel: batch a block's gathers before its serial updates */
#define HB_RUN_NO_PIPE        (1u << 17) /* do not use the warp-specialised producer/consumer pipeline */
#define HB_RUN_STREAM         (1u << 18) /* keep the history in HBM (streamed-history pipeline) even when it fits shared memory */
#define HB_RUN_NO_STREAM      (1u << 19) /* never use the streamed-history pipeline */
/* pipeline and streamed-history kernels: producer threads per node (1, 2, 4 or 8; a streamed-history
   CTA with fewer producers than nodes x lanes runs its producers over several rounds per block); 0 lets
   the engine choose. HB_RUN_EXACT_SUMS overrides it with one. */
#define HB_RUN_PIPE_LANES(n)  ((uint32_t)((n) & 0xf) << 20)
/* streamed-history kernel: nodes per consumer thread (1: 512 threads, 2: 1024 threads, 4: 768 threads
   with two edge windows in flight per producer; 0 lets the engine choose). A grouped launch uses 4 when
   every member asks for it. */
#define HB_RUN_STREAM_NPT(n)  ((uint32_t)((n) & 0x7) << 24)
/* streamed-history kernel: CTAs per sweep point (1, 2, 3, 4, 5, 6 or 8; 0 lets the engine choose). With
   more than one, each point's nodes are split over a thread-block cluster of that many CTAs, so that fewer
   points are in flight and their histories stay in L2; the CTAs of a point exchange the history through
   global memory and signal each finished block of steps to each other. The engine's choice takes the
   size whose resident clusters keep the histories in flight within about 100 MB of L2 with the most SMs
   busy. Grouped launches use one. */
#define HB_RUN_STREAM_CLUSTER(n) \
    ((uint32_t)((n) == 1 ? 1 : (n) == 2 ? 2 : (n) == 4 ? 3 : (n) == 8 ? 4 : (n) == 3 ? 5 : (n) == 5 ? 6 : (n) == 6 ? 7 : 0) << 4)
/* streamed-history kernel: prefetch the history runs of upcoming edges into L2 */
#define HB_RUN_STREAM_PREFETCH (1u << 27)
/* warp-specialised pipeline: use its 1024-thread form (room for eight producer threads per node) */
#define HB_RUN_PIPE_WIDE      (1u << 28)
/* keep every step's state of the run in device memory ([n_steps][n_sweep][state]) for
 * hb_engine_fc_features, with no host copy (the reference copies each step to the host,
 * engine.rs:779-782); HB_ERR_UNSUPPORTED when it does not fit the device's free memory */
#define HB_RUN_DEVICE_TRAJECTORY (1u << 29)
/* test hook of the bounded device-side waits: the warp-specialised pipeline kernel also waits once on
 * an mbarrier phase that nothing completes; the wait gives up after a fixed number of polls, the run
 * finishes unchanged and returns HB_ERR_TIMEOUT. Other kernels ignore the flag. */
#define HB_RUN_TEST_UNSET_WAIT (1u << 30)
/* resident kernel: threads per node sharing its edge list (1, 2, 4 or 8); 0 lets the engine choose */
#define HB_RUN_LANES(n) ((uint32_t)((n) == 1 ? 1 : (n) == 2 ? 2 : (n) == 4 ? 3 : (n) == 8 ? 4 : 0) << 12)

/* One subnetwork: SubnetworkConfig (src/config.rs:129-142) after the batch engine resolved its
 * initial state (engine.rs:161-247). */
typedef struct hb_subnet_desc {
    const char*  model;          /* "Generic2dOscillator", "MontbrioPazoRoxin", "ReducedWongWang",
                                    "Kuramoto", "JansenRit", "WilsonCowan" (config.rs:43-49) */
    int32_t      nnodes;
    int32_t      nmodes;
    const float* params;         /* model parameters, config.rs:43-72 sizes */
    int32_t      n_params;
    const float* initial_state;  /* one point, [nnodes*nmodes, nvar] node-major (engine.rs:239-243) */
    int64_t      n_initial_state;
    /* Extension (the reference takes one parameter row per subnetwork); NULL / 0 for none.
     * Parameter rows per node, [nnodes*nmodes][n_params] shared by all sweep points or
     * [n_sweep][nnodes*nmodes][n_params] one table per point. They replace `params` node by node;
     * a swept model parameter (the native sweep index, or the per-point overrides of a multi-parameter
     * sweep) still takes its sweep value at every node. */
    const float* node_params;
    int64_t      n_node_params;
} hb_subnet_desc;

/* One projection: ProjectionConfig (src/config.rs:158-184). */
typedef struct hb_projection_desc {
    int32_t         src;
    int32_t         tgt;
    int32_t         weights_kind;    /* HB_WEIGHTS_* */
    float           scalar_weight;   /* HB_WEIGHTS_SCALAR */
    const float*    dense;           /* HB_WEIGHTS_DENSE: [tgt_nodes, src_nodes] row-major */
    int32_t         dense_rows;
    int32_t         dense_cols;
    const float*    csr_data;        /* HB_WEIGHTS_CSR: rows are target nodes */
    const uint32_t* csr_indices;
    const uint32_t* csr_indptr;      /* length n_indptr (tgt_nodes + 1) */
    int64_t         nnz;
    int64_t         n_indptr;
    const uint32_t* delays;          /* integration steps; may be NULL when n_delays == 0 */
    int64_t         n_delays;
    const char*     coupling_fn;     /* CouplingFnConfig::from_name_and_params (coupling.rs:114-202) */
    const float*    coupling_params;
    int32_t         n_coupling_params;
    const char*     cvar_map;        /* "0:0" or "0:0,1:1" (construction.rs:337-349) */
} hb_projection_desc;

/* One BOLD monitor: MonitorConfig with monitor_type == "Bold" (config.rs:206-229, engine.rs:419-449). */
typedef struct hb_bold_desc {
    int32_t bold_period;   /* neural steps per Balloon-Windkessel step */
    double  tr;            /* repetition time in seconds */
} hb_bold_desc;

/* SimConfig (src/config.rs:83-114) as the batch engine consumes it. */
typedef struct hb_sim_desc {
    double                     dt;              /* ms */
    int32_t                    integrator;      /* HB_INT_* */
    const float*               nsig;            /* NsigConfig::to_vec(first nvar) (config.rs:16-24) */
    int32_t                    n_nsig;
    int32_t                    n_subnets;
    const hb_subnet_desc*      subnets;
    int32_t                    n_projections;
    const hb_projection_desc*  projections;
    int32_t                    n_bold;
    const hb_bold_desc*        bold;
    uint32_t                   flags;           /* HB_SEM_* */
} hb_sim_desc;

/* One sweep dimension: SweepPoint (engine.rs:41-50). */
typedef struct hb_sweep_point {
    int32_t      sub_idx;
    int32_t      param_idx;
    const float* values;
    int32_t      n_values;
} hb_sweep_point;

typedef struct hb_engine hb_engine;
typedef struct hb_result hb_result;

/* ---- library ---- */
/* HB_ABI_VERSION of the built library (no reference counterpart: the FFI crate checks it at load). */
int32_t     hb_abi_version(void);
/* The calling thread's message for the last failed call: the text of the SimulationError
 * (error.rs:6-25) that the reference would return. Valid until the thread's next call. */
const char* hb_last_error(void);

/* Number of state variables / coupling variables / parameters of a model name
 * (config.rs:43-49, MODEL_REGISTRY); returns HB_ERR_INVALID_CONFIG for unknown names. */
hb_status hb_model_info(const char* model, int32_t* nvar, int32_t* ncvar, int32_t* n_params);

/* ---- engine lifecycle ---- */

/* BatchHybridEngine::from_config(SimConfig, n_sweep, device) (engine.rs:145-471).
 * Validates the descriptor, builds the device-side projection tables and uploads them. */
hb_status hb_engine_create(const hb_sim_desc* desc, int32_t n_sweep, hb_engine** out);

/* Drop of BatchHybridEngine (engine.rs:105-138; the reference frees on scope exit). Accepts NULL. */
void hb_engine_destroy(hb_engine* engine);

/* BatchHybridEngine::run_sweep / run_sweep_with_trajectory (engine.rs:477-494, 496-842).
 * `values` has n_sweep entries. `noise` holds standard-normal draws (the raw N(0,1) samples
 * that generate_noise_reproducible scales by sqrt(2*nsig)*sqrt(dt), integrator.rs:170-198):
 *   shared (default):  [n_steps, sum_over_subnets(nnodes*nmodes*nvar)]
 *   HB_SEM_NOISE_PER_POINT: [n_steps, n_sweep, sum_over_subnets(nnodes*nmodes*nvar)]
 * It is required for stochastic integrators and ignored otherwise (may be NULL).
 * The engine keeps its state, history and step counter across calls, like the reference. */
hb_status hb_engine_run_sweep(hb_engine* engine, int32_t sub_idx, int32_t param_idx,
                              const float* values, int32_t n_values, int64_t n_steps,
                              uint32_t run_flags, const float* noise, int64_t noise_len,
                              hb_result** out);

/* BatchHybridEngine::run_sweep_multi / run_sweep_multi_with_trajectory (engine.rs:845-1348):
 * Cartesian product of the dimensions (last dimension fastest, engine.rs:69-90). Like the
 * reference, this runs a fresh engine seeded from sweep point 0's current state, with no BOLD
 * monitors. The product size must equal the engine's n_sweep. */
hb_status hb_engine_run_sweep_multi(hb_engine* engine, const hb_sweep_point* dims, int32_t n_dims,
                                    int64_t n_steps, uint32_t run_flags,
                                    const float* noise, int64_t noise_len, hb_result** out);

/* Current batched state of one subnetwork (BatchHybridEngine::states, engine.rs:109):
 * [n_sweep, nnodes*nmodes, nvar] written into `out` (len floats). */
hb_status hb_engine_get_state(hb_engine* engine, int32_t sub_idx, float* out, int64_t len);

/* BatchHybridEngine::step (engine.rs:113). */
int64_t   hb_engine_step(const hb_engine* engine);

/* Restore the state, history, step counter and BOLD monitors of a freshly created engine
 * (no reference counterpart: lets a caller repeat a run without re-uploading the network). */
hb_status hb_engine_reset(hb_engine* engine);

/* Milliseconds of device time of the last run's simulation kernels, measured with CUDA events
 * on the engine's stream, and the number of kernel launches of that run (no reference counterpart;
 * BatchSweepResult::elapsed_ms, engine.rs:28, is the host wall time of the whole call). */
hb_status hb_engine_last_kernel_time(const hb_engine* engine, double* ms, int64_t* launches,
                                     int32_t* kernel_kind);

/* Use a caller-provided CUDA stream (cudaStream_t passed as void*) for subsequent runs; NULL
 * restores the engine's own stream (no reference counterpart: Burn owns its device queue). */
hb_status hb_engine_set_stream(hb_engine* engine, void* cuda_stream);

/* Replaces an assignment to the public field `BatchHybridEngine::hybrid_integrator`
 * (engine.rs:125, read by the step at engine.rs:697-702; callers set it after from_config, e.g.
 * examples/bench/hyburn_bench_generic_cuda.rs:54). on != 0: Heun for Generic2dOscillator
 * subnetworks and Euler for the others, whatever the configured integrator; 0: the configured
 * integrator for every subnetwork. Same as creating the engine with or without
 * HB_SEM_HYBRID_INTEGRATOR; takes effect at the next run or prepare. */
hb_status hb_engine_set_hybrid_integrator(hb_engine* engine, int32_t on);

/* ---- device-resident runs (inputs already in HBM; used to time the kernels alone) ---- */

/* Upload the sweep values and noise of a run once; later `hb_engine_execute_prepared` calls
 * reset the engine and run all steps on the device without host transfers (no reference
 * counterpart; the same run as hb_engine_run_sweep, engine.rs:477-484, minus the copies). */
hb_status hb_engine_prepare(hb_engine* engine, int32_t sub_idx, int32_t param_idx,
                            const float* values, int32_t n_values, int64_t n_steps,
                            uint32_t run_flags, const float* noise, int64_t noise_len);
hb_status hb_engine_execute_prepared(hb_engine* engine);

/* ---- one sweep without any device allocation (no counterpart in the reference) ----
 * For callers that cannot call cudaMalloc: a host framework whose own caching allocator or arena
 * owns the device's memory (a foreign allocation fails once the arena has reserved the device, or
 * fragments it), or code running where allocating is not allowed. It runs the hot-path shape —
 * one subnetwork coupled to itself through one CSR projection with one delay per edge
 * (ring-buffer semantics of HB_SEM_DELAY_RING), shared noise, no monitors — on inputs and outputs
 * the caller already holds in device memory:
 *   d_x0 [nnodes*nvar] (one point, node-major), CSR rows = target nodes: d_indptr [nnodes+1]
 *   (int32), d_indices / d_delays / d_weights [nnz], d_noise [n_steps, nnodes*nvar] standard
 *   normal draws (stochastic integrators only), outputs d_final_states / d_tavg
 *   [n_sweep, nnodes, nvar]. Host arrays: model and coupling parameters, nsig, sweep_values.
 * sweep_sub_idx 0 sweeps model parameter sweep_param_idx, which must be the model's native sweep
 * index (the batch engine's dfun.rs:49-72; any other index is HB_ERR_INVALID_CONFIG here), -1
 * sweeps coupling parameter sweep_param_idx.
 * Network tables and the history ring live in one static device array of
 * HB_NOALLOC_SCRATCH_BYTES that every GPU loading the library keeps until exit; sweeps needing
 * more are rejected with HB_ERR_UNSUPPORTED. The first call on a device resolves that array's
 * address. All calls share the array: calls that overlap on the GPU race and must be serialised
 * by the caller. The call returns once its work is enqueued on cuda_stream and makes no explicit
 * synchronisation (its parameter tables are copied from pageable host memory, which the driver
 * stages and for which it may wait on the stream). The CSR input (indptr monotone from 0 to nnz,
 * source indices below nnodes, delays at most max_delay) is checked on the device: a malformed
 * one makes the run use no edges and fills both outputs with NaN. */
#define HB_NOALLOC_SCRATCH_BYTES (64u << 20)
hb_status hb_noalloc_run_csr_sweep(
    const char* model, const float* params, int32_t n_params, int32_t nnodes, const float* d_x0,
    const int32_t* d_indptr, const uint32_t* d_indices, const uint32_t* d_delays, const float* d_weights,
    int64_t nnz, int32_t max_delay, const char* coupling_fn, const float* coupling_params,
    int32_t n_coupling_params, int32_t sweep_sub_idx, int32_t sweep_param_idx, const float* sweep_values,
    int32_t n_sweep, double dt, int32_t integrator, const float* nsig, int32_t n_nsig,
    const float* d_noise, int64_t noise_len, int64_t n_steps, float* d_final_states, float* d_tavg,
    void* cuda_stream);

/* ---- grouped launch: several engines' sweeps in one kernel launch (no counterpart in the reference) ----
 * The reference runs each network size as its own BatchHybridEngine, one after the other. A grouped
 * launch runs the sweeps of several engines — different models, node counts, connectomes, delays,
 * coupling functions, sweep values and step counts — as one launch of a persistent work-queue
 * kernel: CTAs, or thread-block clusters (HB_RUN_STREAM_CLUSTER in the members' run flags, else
 * chosen by the engine), take (member, point) items from a device counter, members with the most
 * work per CTA first, so short points fill the SMs that long ones leave free; a member with at
 * least 100 nodes per CTA runs each point split over a cluster. Every member needs one subnetwork
 * coupled to itself through one CSR projection with per-edge delays (HB_SEM_DELAY_RING) of at
 * least 15 steps.
 * hb_group_prepare resets every member engine, uploads its tables and noise, and captures the
 * member resets, the launch and the batch-mean BOLD reductions in a CUDA graph;
 * hb_group_execute replays it (each member restarts from its initial state) and completes the
 * members' BOLD series; hb_group_result returns member i's BatchSweepResult of the last execute.
 * The member engines must not be used elsewhere while the group exists. */
typedef struct hb_group_member {
    hb_engine*   engine;
    int32_t      sub_idx;      /* SweepParam of this member's sweep (as hb_engine_run_sweep) */
    int32_t      param_idx;
    const float* values;       /* n_values == the engine's n_sweep */
    int32_t      n_values;
    int64_t      n_steps;
    uint32_t     run_flags;    /* HB_RUN_CHECK_FINITE; no trajectories */
    const float* noise;        /* host standard-normal draws as for hb_engine_run_sweep, or NULL */
    int64_t      noise_len;
} hb_group_member;
typedef struct hb_group hb_group;

hb_status hb_group_prepare(const hb_group_member* members, int32_t n_members, void* cuda_stream, hb_group** out);
hb_status hb_group_execute(hb_group* group);
hb_status hb_group_result(hb_group* group, int32_t member, hb_result** out);
hb_status hb_group_last_kernel_time(const hb_group* group, double* ms);
void      hb_group_destroy(hb_group* group);

/* ---- adjoint of a functional-connectivity loss (no counterpart in the reference, which has no adjoint) ----
 * For an engine with one JansenRit subnetwork coupled to itself through one CSR projection with
 * per-edge delays (HB_SEM_DELAY_RING), Sigmoidal or Linear coupling and the deterministic Heun
 * or RK4 integrator: sweep point b runs n_steps from the engine's initial state with the coupling gain
 * gain_values[b] (Sigmoidal `a`, Linear `a`); y = y1 - y2; FC = Pearson correlation over the
 * post-step states t = 1..n_steps; loss_b = mean over i, j of (FC_ij - target_fc_ij)^2 with a
 * symmetric target_fc [nnodes][nnodes]. Outputs (any pointer may be NULL): loss [n_sweep],
 * d_gain [n_sweep], d_A / d_B / d_a [n_sweep][nnodes] (the JansenRit A, B, a taken per node),
 * fc [n_sweep][nnodes][nnodes], y [n_steps][n_sweep][nnodes]. The gradients are those of the
 * discrete FP32 step (discrete adjoint), summed in FP32 within a checkpoint segment and in FP64
 * across segments. checkpoint_every > 0: the reverse sweep re-computes the forward run from
 * checkpoints taken every checkpoint_every steps; <= 0: the forward keeps every step (32 B per
 * node-step) when that takes at most a quarter of the free device memory, else checkpoints every
 * 500 steps. The engine's state is left reset. */
typedef struct hb_adjoint_out {
    double* loss;
    double* d_gain;
    double* d_A;
    double* d_B;
    double* d_a;
    float*  fc;
    float*  y;
    float   forward_ms;     /* device time of the forward run with checkpoints */
    float   statistics_ms;  /* FC, loss and the per-step loss sources */
    float   reverse_ms;     /* re-computation and reverse sweep */
} hb_adjoint_out;
hb_status hb_engine_adjoint_fc(hb_engine* engine, const float* gain_values, int32_t n_values, int64_t n_steps,
                               const float* target_fc, int32_t checkpoint_every, hb_adjoint_out* out);

/* ---- adjoint of the time-averaged Kuramoto order parameter (no counterpart in the reference) ----
 * For an engine with one Kuramoto subnetwork (one mode) coupled to itself through one CSR projection
 * with per-edge delays (HB_SEM_DELAY_RING), Kuramoto coupling and deterministic Heun: the engine is
 * reset and runs n_steps with the coupling scale a = gain_values[b] for sweep point b, keeping
 * every step's phase on the device; loss_b = (1/n_steps) sum_{t=1..n_steps} R_b(t) with
 * R = |mean_j exp(i theta_j)|. Omega may be one value per node (hb_subnet_desc.node_params). Outputs (any
 * pointer may be NULL): loss, d_gain = dL/da and d_omega = dL/domega (the gradient with respect to a
 * shift of every node's omega), [n_sweep] each, d_omega_node = dL/domega_i [n_sweep][nnodes], and the
 * device times of the forward run, the preparation
 * (sin / cos rows, order parameter) and the reverse sweep. run_flags (HB_RUN_*) choose the forward's
 * kernel form as for hb_engine_run_sweep; the pipeline and streamed-history forms also hand the
 * coupling sums of every step to the reverse sweep, which otherwise gathers them again. The phase
 * wrap to [0, 2 pi) is taken with derivative 1 (the loss depends on the phases only through sin
 * and cos). */
typedef struct hb_order_adjoint_out {
    double* loss;
    double* d_gain;
    double* d_omega;       /* [n_sweep]: dL/domega for one omega shared by all nodes (the sum of d_omega_node) */
    double* d_omega_node;  /* [n_sweep][nnodes]: dL/domega_i per node (omega per node from hb_subnet_desc.node_params) */
    float   forward_ms, prepare_ms, reverse_ms;
} hb_order_adjoint_out;
hb_status hb_engine_adjoint_order(hb_engine* engine, const float* gain_values, int32_t n_values, int64_t n_steps,
                                  uint32_t run_flags, hb_order_adjoint_out* out);

/* ---- functional-connectivity features on the device (sbi/features/fc.rs, mod.rs:257-280) ----
 * From the trajectory of the engine's last run, which must have used HB_RUN_DEVICE_TRAJECTORY, for
 * every sweep point and state variable of subnetwork sub_idx: the node series (mean over modes)
 * over all the run's steps, its FC matrix (fc_matrix, fc.rs:11-58), the FeatureSet::Fc values
 * (fc_stats of FC's upper triangle: mean, std, min, max, median; homotopic mean and std), and, with
 * window_len > 0, the FCD matrix of windows [w * stride, w * stride + window_len) (fcd_matrix,
 * fc.rs:87-141) and its fc_stats. n_windows = (n_steps - window_len) / stride + 1, reported as 0
 * (FCD empty, fcd_stats NaN) when it is 1. window_len outside [2, n_steps] or stride < 1 (assertion
 * failures in the reference) return HB_ERR_INVALID_STATE. Any output pointer may be NULL; with all
 * four NULL the call only validates and reports n_windows, nnodes and nvar (a size query). */
typedef struct hb_fc_features {
    float*  fc;          /* [n_sweep][nvar][nnodes][nnodes] */
    float*  features;    /* [n_sweep][nvar][7] */
    float*  fcd;         /* [n_sweep][nvar][n_windows][n_windows] */
    float*  fcd_stats;   /* [n_sweep][nvar][5] */
    int32_t n_windows;   /* out */
    int32_t nnodes;      /* out */
    int32_t nvar;        /* out */
    float   ms;          /* out: device time of the feature kernels */
} hb_fc_features;
hb_status hb_engine_fc_features(hb_engine* engine, int32_t sub_idx, int32_t window_len, int32_t stride,
                                hb_fc_features* out);

/* ---- results: BatchSweepResult (engine.rs:15-31) ---- */
int32_t      hb_result_n_sweep(const hb_result* r);
int32_t      hb_result_n_subnets(const hb_result* r);
int32_t      hb_result_n_bold(const hb_result* r);
double       hb_result_elapsed_ms(const hb_result* r);
const float* hb_result_param_values(const hb_result* r, int64_t* len);
const float* hb_result_tavg(const hb_result* r, int32_t sub_idx, int64_t* len);
const float* hb_result_final_states(const hb_result* r, int32_t sub_idx, int64_t* len);
const float* hb_result_trajectory(const hb_result* r, int32_t sub_idx, int64_t* len); /* NULL if not recorded */
const float* hb_result_bold(const hb_result* r, int32_t monitor_idx, int64_t* len);
void         hb_result_free(hb_result* r);

/* ---- NPY files (io.rs:19-125) ---- */

/* write_npy_f32 (io.rs:88-125): `ndim` dimensions in `shape`, their product of values from `data`;
 * version 1.0 header "{'descr': '<f4', 'fortran_order': False, 'shape': (...) }" padded with spaces
 * to a 64-byte multiple, little-endian f32 values. HB_ERR_IO when the file cannot be written. */
hb_status hb_npy_write_f32(const char* path, const float* data, const int64_t* shape, int32_t ndim);

/* read_npy_f32 (io.rs:25-83): with out == NULL, a size query (n_values, ndim and up to max_ndim
 * entries of shape); otherwise also the values into out[capacity]. Descriptors '<f4', '|f4', 'f4'
 * and '<f8' (rounded to f32); 'fortran_order' is ignored; every whole value after the header is
 * returned, so n_values can exceed the shape's product when the file has trailing bytes.
 * HB_ERR_IO when the file cannot be read, HB_ERR_INVALID_STATE for the format errors of the
 * reference ("Not a valid .npy file", "No 'shape' key in NPY header", "Failed to parse NPY shape",
 * "Unsupported NPY dtype descriptor", "NPY data truncated (f32|f64)") and for files shorter than
 * the fixed 10-byte prefix. */
hb_status hb_npy_read_f32(const char* path, float* out, int64_t capacity, int64_t* shape, int32_t max_ndim,
                          int32_t* ndim, int64_t* n_values);

/* The batch sweep's output files (cli.rs:947-970): `output_dir` and its parents are created, then
 * tavg_sub{i}.npy per subnetwork i of the result, labelled [n_sweep, nvar, nnodes*nmodes] over data
 * laid out [n_sweep, nnodes*nmodes, nvar], as the reference writes them. */
hb_status hb_engine_write_tavg(const hb_engine* engine, const hb_result* result, const char* output_dir);

#ifdef __cplusplus
}
#endif

#endif /* HYBURN_GB300_H */
