// hb_device.h — device-side network description shared by the host engine and the kernels.
//
// The host engine (hb_engine.cu) lowers a validated hb_sim_desc into these flat tables once per
// engine (projections, CSR rows with packed per-edge delays and precomputed ring offsets) and
// once per run (per-point model and coupling parameters, noise, BOLD schedules). Kernels read
// the DevNet from global memory and keep a copy in shared memory.
#pragma once
#include <cstdint>

#define HB_MAX_SUB 8
#define HB_MAX_PROJ 16
#define HB_MAX_BOLD 4
#define HB_PSTRIDE 32   // floats per (subnetwork, point) parameter row: params + derived constants
#define HB_NCP 16       // floats per resolved coupling-function parameter row
#define HB_MAX_THREADS 1024
#define HB_MAX_IN 4       // incoming projections per subnetwork
#define HB_STREAM_K 8     // steps per block of the streamed-history kernel (needs every delay >= 2K - 1)

// model ids (order of the host registry)
enum { HBM_G2DO = 0, HBM_MPR = 1, HBM_RWW = 2, HBM_KURAMOTO = 3, HBM_JR = 4, HBM_WC = 5 };

// effective integrators (engine.rs:697-771); HBI_HEUN_DET is the deterministic Heun arm
enum { HBI_HEUN_DET = 0, HBI_EULER = 1, HBI_EULER_STOCH = 2, HBI_HEUN_STOCH = 3, HBI_RK4 = 4, HBI_RK4_STOCH = 5 };

// coupling functions (coupling.rs:52-71)
enum { HBC_LINEAR = 0, HBC_SIGMOIDAL, HBC_DIFFERENCE, HBC_KURAMOTO, HBC_SCALED_LINEAR, HBC_TANH, HBC_SJR, HBC_PRESIG };

// weighted-sum kinds
enum { HBK_MEAN = 0, HBK_DIAG = 1, HBK_SPARSE = 2 };

// delay read modes
//  HBD_COMPAT: one delay per projection, batch engine shift window (engine.rs:541-589)
//  HBD_RING:   one delay per projection, true ring (runtime.rs:235-252)
//  HBD_EDGE:   per-edge delays, true ring, zero rows after pre() (runtime.rs:162-204)
enum { HBD_COMPAT = 0, HBD_RING = 1, HBD_EDGE = 2 };

// derived-constant slots in a parameter row (computed on the host in f32 with the C library)
#define HB_D_WC_SIG_E_OFF 24
#define HB_D_WC_SIG_I_OFF 25

struct DevSub {
    int model, nm, nvar, ncvar;
    int thread_off;   // resident kernel: first thread of this subnetwork (warp aligned)
    int col_off;      // first ring column (columns are [node][cvar])
    int state_off;    // offset of this subnetwork in a point's packed state [nm][nvar]
    int noise_off;    // offset in a noise row
    int integ, sweep_form;
    int lanes;        // threads per node (edge lists split over `lanes` lanes, power of two <= 8)
    int lanes_log2;
    int n_in;
    int in_idx[HB_MAX_IN];
    int n_mean_out;   // mean-field projections whose source is this subnetwork
    int mean_out[HB_MAX_PROJ];
    const float* params;   // [B][HB_PSTRIDE]
    const float* node_params;  // [B or 1][nm][HB_PSTRIDE] per-node rows (extension), or nullptr
    int node_pp;               // node_params holds one table per sweep point
};

// parameter row of node `n` of sweep point `b` of a subnetwork: its node row when the subnetwork has
// per-node parameters, else the point's row
__host__ __device__ inline const float* hb_param_row(const DevSub& s, int b, int n) {
    return s.node_params ? s.node_params + ((size_t)(s.node_pp ? b : 0) * s.nm + n) * HB_PSTRIDE
                         : s.params + (size_t)b * HB_PSTRIDE;
}

struct DevProj {
    int src, tgt, kind, dmode, delay, nsrc, ntgt;
    int cfk, pre_cpu, ncv, pc, oc, has_rowsums;
    int direct, ncm;
    int cm_s[4], cm_cpl[4];
    int mean_slot;        // MEAN: index of its partial-sum slot
    int smem_edges;       // resident kernel: edge offset inside the shared-memory copy, -1 if global
    int maxd;             // largest edge delay (per-edge mode)
    float w;
    float cp[HB_NCP];
    const float* cp_pp;   // [B][HB_NCP] when the coupling parameters are swept, else nullptr
    const int* rowptr;    // [ntgt + 1]
    const int* porder;    // producer order of the target nodes (pipeline and streamed-history kernels): per node slice,
                          // the slice's local node ids by decreasing in-degree, so that a warp's lanes get similar
                          // edge counts; nullptr for the identity
    const uint32_t* edges; // (delay << 16) | src node
    const int* eoff;       // ring offset of each edge: src column - delay * cols (per-edge mode) or src column
    const float* ew;
    const float* rowsums;
};

struct DevNet {
    int n_sub, n_proj, n_mean;
    int B;                // sweep points
    int H;                // horizon (batch: max delay + 1 or 0; ring: max delay + 1)
    int R;                // ring length (slots)
    int cols;             // ring columns per point = sum nm * ncvar
    int state_len;        // floats per point of packed state = sum nm * nvar
    int noise_row;        // floats per step (per point) of the noise array
    int total_edges;
    float dt, dt_half, dt_sixth, dt_h2;
    float noise_scale[8]; // sqrt(2*nsig[v]) * sqrt(dt)
    DevSub sub[HB_MAX_SUB];
    DevProj proj[HB_MAX_PROJ];
};

// BOLD emission schedule entry: emit output `out` when run-local sample `k` is produced
struct BoldEmit {
    int k;       // run-local sample index
    int out;     // run-local output row
    int interp;  // 1: prev + (cur - prev) * w ; 0: cur
    float w;
};

struct DevBold {
    int n;                 // number of monitors
    int per_point;         // 1: one series per point
    int period[HB_MAX_BOLD];
    int n_full[HB_MAX_BOLD];      // full windows in this run
    int partial[HB_MAX_BOLD];     // steps of the flushed partial window (0 if none)
    float dt_full[HB_MAX_BOLD];   // BW step (s) of a full window
    float dt_part[HB_MAX_BOLD];   // BW step (s) of the partial window
    int n_emit[HB_MAX_BOLD];
    const BoldEmit* emit[HB_MAX_BOLD];
    float* out[HB_MAX_BOLD];      // per point: [B][n_out_run][N0]; batch mean: [n_out_run][N0]
    int n_out_run[HB_MAX_BOLD];
    float* bw[HB_MAX_BOLD];       // BW state [5][B or 1][N0]: s, f, v, q, previous signal
    float* win[HB_MAX_BOLD];      // batch mean: window sums [W][B][N0]
    float* acc[HB_MAX_BOLD];      // running window sum [B][N0] carried between launches
    int n0;                       // nodes of subnetwork 0
};

// per-launch arguments of the simulation kernels
struct RunArgs {
    int64_t s0;           // absolute step of the first step of this launch
    int n_steps;          // steps in this launch
    int64_t run_s0;       // absolute step at which the current run started
    int64_t run_steps;    // total steps of the run
    float* state;         // [B][state_len]
    float* tavg;          // [B][state_len]
    float* ring;          // [B][R][cols] global ring (scratch)
    const float* noise;   // noise rows of this launch: [n_steps][row] or [n_steps][B][row]
    int noise_per_point;
    float* traj;          // [n_steps][B][state_len] or nullptr
    float* gx_out;        // [n_steps][B][nm][2] the two coupling sums of every step (Kuramoto), or nullptr
    int ring_in_smem;     // resident kernel: ring cached in shared memory
    int smem_edges;       // resident kernel: edges cached in shared memory
    int sync_every;       // specialised kernel: steps between CTA barriers (<= smallest delay, R >= H + sync_every)
    int two_phase;        // specialised kernel: batch the gathers of a block before its serial updates
    int pipe_lanes;       // pipeline kernels: producer threads per node in the steady state
    int stream_rp;        // streamed-history kernel: ring positions per node (time t at t mod stream_rp)
    int stream_noise_smem;// streamed-history kernel: noise rows staged through shared memory
    int stream_prefetch;  // streamed-history kernel: prefetch the history run of the edge this many lane strides ahead (0: off)
    int stream_cluster;   // streamed-history kernel: CTAs per sweep point (a thread-block cluster splitting its nodes; 0 or 1: one)
    int load_ring;        // copy the global ring into shared memory at launch start
    int store_ring;       // copy the shared ring back at launch end
    int* flags;           // [0]: non-finite seen, [1]: bounds error
    int check_finite;
    int test_unset_wait;  // pipeline kernel: one bounded wait on a barrier nothing completes (timeout test)
    int exact_sums;       // coupling sums term by term in edge order, product and sum rounded apart (HB_RUN_EXACT_SUMS)
    int stream_wgather;   // streamed-history kernel: warp-cooperative gathers (a warp per node, 8 lanes per edge
                          // window; 0: one thread per edge window)
    int stream_bulk;      // warp-cooperative gathers staged by the bulk-copy engine (HB_RUN_STREAM_BULK)
    DevBold bold;
};

// one network's sweep inside a grouped launch of the streamed-history work-queue kernel
struct StreamJob {
    const DevNet* net;
    RunArgs args;
    int first_block;   // first work item of this job (items are numbered job by job)
    int n_points;      // its sweep points (one work item each)
    int model, pre;    // model id and coupling pre() form (0: identity, 1: [sin, cos]) of its kernel path
    int split;         // 1: each work item is one point split over the launch's cluster (args.stream_cluster
                       // = the cluster size); 0: each item is cluster-size points, one per CTA
};

// the FC-loss adjoint's buffers and sizes (hb_adjoint.cu); device pointers
struct HbAdjointLaunch {
    int B, N, T, R, K, CK, n_ck, cfk, gain_idx, nnz, store_all;
    int slices;        // time slices of the moment pass (hb_adjoint_moment_slices)
    int pipelined;     // forward, re-computation and reverse as producer / consumer pipelines (every delay >= 2K - 1)
    int dmin;          // smallest edge delay (steps)
    int rk4;           // deterministic RK4 (else Heun)
    float dt_h2, dt_sixth;
    float dt, dt_half;
    const float* x0;
    const int* rowptr; const uint32_t* edges; const float* ew;
    const int* cptr; const int* ctgt; const int* cdel; const float* cw;
    float *Y, *S, *ck_state, *ck_ring, *scratch, *mu_ring;
    float* lam_g;      // [B][N*6] lambda between the checkpoint segments' reverse launches
    const float* target;
    float *mean, *sdev, *coef, *rk, *M, *fc;
    double *loss, *gG, *gA, *gB, *ga;
    double* moments;   // [B][slices][W * W + W] partial moments of y, W = N rounded up to 4
};

// FC / FCD features of a device trajectory (hb_features.cu); device pointers
struct HbFeatLaunch {
    const float* traj;   // [T][B][state_len]
    int T, B, state_len, off, nnodes, nmodes, nvar;
    int window, stride, n_windows;  // FCD windows (n_windows >= 2), else n_windows = 0
    int b0, nb;          // this batch: points b0 .. b0 + nb - 1
    int fc_slices, win_slices;
    int block_len;       // > 0: FCD window moments from blocks of this many steps (divides window and stride)
    float* fc;           // [B][nvar][nnodes][nnodes]
    float* feat;         // [B][nvar][7]: mean, std, min, max, median of FC's upper triangle; homotopic mean, std
    float* fcd;          // [B][nvar][n_windows][n_windows]
    float* fcd_stats;    // [B][nvar][5]
    double* part;        // moments workspace: nb * nvar * (ranges of the largest pass) * hb_fc_part_len(nnodes)
    float* ut;           // nb * nvar * n_windows * nnodes (nnodes - 1) / 2 window-FC upper triangles
    double* ut_mv;       // nb * nvar * n_windows * 2: mean and centred sum of squares of each
};
cudaError_t hb_launch_fc_features(const HbFeatLaunch& L, cudaStream_t st);
size_t hb_fc_part_len(int nnodes);  // doubles of one range's moments in HbFeatLaunch::part

// the Kuramoto order-parameter adjoint (hb_kuradj.cu); device pointers
struct HbKuraAdjLaunch {
    const float* traj;   // [T][B][N] phases after each step
    const float* x0;     // [B][N] initial phases
    int B, N, T, K;      // K: steps per reverse block (<= 8 and <= every delay)
    int maxd;            // largest edge delay
    float dt;
    const float* k;      // [B] the coupling's a / N as the engine resolves it
    const int* rowptr; const uint32_t* edges; const float* ew;          // CSR by target
    const int* cptr; const int* ctgt; const int* cdel; const float* cw;  // CSC by source
    const float* cs;     // [T][B][N][2] the forward's coupling sums S, C of every step, or nullptr
    float* sc;           // [B][N][T + 1][2] sin, cos of every phase
    float* z;            // [B][T][2] mean cos, mean sin after each step
    float* nu;           // [B][N][T][2] the pulled adjoint terms
    double* loss; double* gA; double* gW;  // [B]
    double* gWn;         // [B][N] dL/domega_i per node, or nullptr
};
cudaError_t hb_launch_kura_adjoint(const HbKuraAdjLaunch& L, int phase, cudaStream_t st);

// time slices of the moment pass for B points of T steps: enough blocks to fill the SMs three times
// over, at most 16, each slice at least 64 steps
inline int hb_adjoint_moment_slices(int B, int T) {
    int s = (456 + B - 1) / B;
    if (s > 16) s = 16;
    if (s > T / 64) s = T / 64;
    return s < 1 ? 1 : s;
}
