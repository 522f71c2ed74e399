// hb_noalloc.cu — a sweep entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host framework whose own caching allocator or arena owns
// every byte of device memory (a foreign allocation would fail once the arena has reserved the
// device, or fragment it), or code that runs where allocation is not allowed, such as a callback
// that may not synchronise the device. For them, hb_noalloc_run_csr_sweep runs the hot-path
// network shape — one subnetwork coupled to itself through one CSR projection with one delay per
// edge — on inputs and outputs the caller already holds in device memory. Everything else the
// kernel needs (its network tables, per-point parameter rows and the coupling-variable history
// ring) lives in one file-scope device array of HB_NOALLOC_SCRATCH_BYTES bytes, which every GPU
// that loads this library keeps until exit.
//
// The array's address is resolved once per device with cudaGetSymbolAddress (host code may not
// use the symbol itself as a device address); the first call on a device does that set-up. All
// calls share the array and it keeps the last call's contents: this file clears the status flags
// each call; the ring needs no clearing because the kernel never reads a time before the run's
// first step. Calls that overlap on the GPU race on the array and must be serialised by the
// caller. The call makes no explicit synchronisation: the CSR input is checked on the device, and a
// malformed one turns the run into an edge-free one whose outputs are NaN. Its small parameter
// tables go to the array by cudaMemcpyAsync from pageable host memory, which the CUDA driver
// stages before the call returns (and for which it may wait on the stream).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "hb_device.h"
#include "hyburn_gb300.h"

cudaError_t hb_launch_resident(int model, int fast, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem,
                               cudaStream_t st);
int hb_resident_smem_budget(int model, int fast, int threads);

static __device__ __align__(256) unsigned char g_noalloc_scratch[HB_NOALLOC_SCRATCH_BYTES];

// records the message returned by hb_last_error() (defined with the other entry points)
void hb_internal_set_error(const char* msg);

namespace {

hb_status nfail(hb_status st, const char* msg) {
    hb_internal_set_error(msg);
    return st;
}

std::mutex g_setup_mu;
void* g_scratch_addr[64] = {nullptr};

// device address of the scratch array on the current device (resolved once per device)
hb_status scratch_address(unsigned char** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nfail(HB_ERR_CUDA, "no current CUDA device");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return nfail(HB_ERR_CUDA, cudaGetErrorString(e));
        g_scratch_addr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_scratch_addr[dev]);
    return HB_OK;
}

// packs (delay << 16 | src) and the ring offset of every edge; flags malformed CSR input
__global__ void pack_edges_kernel(const int32_t* __restrict__ indptr, const uint32_t* __restrict__ indices,
                                  const uint32_t* __restrict__ delays, int64_t nnz, int nnodes, int max_delay, int ncv,
                                  int cols, uint32_t* __restrict__ edges, int* __restrict__ eoff, int* __restrict__ flags) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k <= nnodes) {
        int v = indptr[k];
        if (v < 0 || (int64_t)v > nnz || (k == 0 && v != 0) || (k == nnodes && (int64_t)v != nnz) ||
            (k < nnodes && indptr[k + 1] < v))
            atomicOr(flags + 1, 1);
    }
    if (k >= nnz) return;
    uint32_t src = indices[k], d = delays[k];
    if (src >= (uint32_t)nnodes || d > (uint32_t)max_delay) {
        atomicOr(flags + 1, 2);
        src = 0;
        d = 0;
    }
    edges[k] = (d << 16) | src;
    eoff[k] = (int)src * ncv - (int)d * cols;
}

__global__ void replicate_kernel(const float* __restrict__ x0, int per, int B, float* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (int64_t)per * B) out[i] = x0[i % per];
}

// After pack_edges_kernel: when it flagged the CSR input as malformed, every target row of the
// projection is pointed at an empty edge range, so the run that follows reads only in-bounds memory.
__global__ void guard_kernel(DevNet* __restrict__ net, int* __restrict__ empty_rows, int nnodes,
                             const int* __restrict__ flags) {
    if (!flags[1]) return;
    for (int i = threadIdx.x; i <= nnodes; i += blockDim.x) empty_rows[i] = 0;
    if (threadIdx.x == 0) net->proj[0].rowptr = empty_rows;
}

// tavg = sum / n_steps; both outputs become NaN when the CSR input was malformed
__global__ void finish_kernel(float* __restrict__ tavg, float* __restrict__ fin, int64_t n, float s,
                              const int* __restrict__ flags) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (flags[1]) {
        tavg[i] = __int_as_float(0x7fc00000);
        fin[i] = __int_as_float(0x7fc00000);
    } else {
        tavg[i] = tavg[i] * s;
    }
}

struct ModelRow { const char* name; int id, nvar, ncvar, nparams, native; };
const ModelRow k_rows[6] = {{"Generic2dOscillator", HBM_G2DO, 2, 1, 12, 1}, {"MontbrioPazoRoxin", HBM_MPR, 2, 2, 7, 4},
                            {"ReducedWongWang", HBM_RWW, 1, 1, 8, 7},       {"Kuramoto", HBM_KURAMOTO, 1, 1, 1, 0},
                            {"JansenRit", HBM_JR, 6, 1, 13, 12},            {"WilsonCowan", HBM_WC, 2, 1, 22, 18}};

// coupling functions with an identity or [sin, cos] pre(): resolved parameter rows as the kernels read them
bool coupling_row(const char* name, const float* cp, int n, int n_src, float* row, int* kind) {
    auto P = [&](int i, float d) { return n > i ? cp[i] : d; };
    for (int i = 0; i < HB_NCP; i++) row[i] = 0.0f;
    if (!name || !strcmp(name, "Linear")) { *kind = HBC_LINEAR; row[0] = P(0, 1.0f); row[1] = P(1, 0.0f); }
    else if (!strcmp(name, "ScaledLinear")) { *kind = HBC_SCALED_LINEAR; row[0] = P(0, 1.0f); row[1] = P(1, 0.0f); }
    else if (!strcmp(name, "Difference")) { *kind = HBC_LINEAR; row[0] = P(0, 1.0f); row[1] = 0.0f; }
    else if (!strcmp(name, "Sigmoidal")) {
        *kind = HBC_SIGMOIDAL;
        if (n >= 5) { row[0] = cp[0]; row[1] = cp[1]; row[2] = cp[2]; row[3] = cp[3]; row[4] = cp[4]; }
        else { row[0] = -1.0f; row[1] = P(0, 1.0f); row[2] = P(1, 0.0f); row[3] = 1.0f; row[4] = P(2, 1.0f); }
    } else if (!strcmp(name, "Kuramoto")) { *kind = HBC_KURAMOTO; row[0] = P(0, 1.0f); row[1] = row[0] / (float)n_src; }
    else return false;
    return true;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

extern "C" hb_status hb_noalloc_run_csr_sweep(
    const char* model, const float* params, int32_t n_params, int32_t nnodes, const float* d_x0,
    const int32_t* d_indptr, const uint32_t* d_indices, const uint32_t* d_delays, const float* d_weights, int64_t nnz,
    int32_t max_delay, const char* coupling_fn, const float* coupling_params, int32_t n_coupling_params,
    int32_t sweep_sub_idx, int32_t sweep_param_idx, const float* sweep_values, int32_t n_sweep, double dt,
    int32_t integrator, const float* nsig, int32_t n_nsig, const float* d_noise, int64_t noise_len, int64_t n_steps,
    float* d_final_states, float* d_tavg, void* cuda_stream) {
    const ModelRow* mr = nullptr;
    for (const auto& r : k_rows)
        if (model && !strcmp(model, r.name)) mr = &r;
    if (!mr) return nfail(HB_ERR_INVALID_CONFIG, "unknown or unsupported model");
    if (n_params < mr->nparams || n_params > 24 || !params) return nfail(HB_ERR_INVALID_CONFIG, "wrong number of model parameters");
    if (nnodes < 1 || nnodes > 1024 || n_sweep < 1 || n_steps < 1 || !(dt > 0.0))
        return nfail(HB_ERR_INVALID_CONFIG, "nnodes must be 1..1024, n_sweep >= 1, n_steps >= 1, dt > 0");
    if (n_steps > (int64_t)0x7fffffff) return nfail(HB_ERR_UNSUPPORTED, "n_steps above 2^31-1");
    if (max_delay < 0 || max_delay > 65535 || nnz < 0) return nfail(HB_ERR_INVALID_CONFIG, "max_delay must be 0..65535");
    if (!d_x0 || !d_indptr || (nnz > 0 && (!d_indices || !d_delays || !d_weights)) || !d_final_states || !d_tavg || !sweep_values)
        return nfail(HB_ERR_INVALID_STATE, "a required pointer is NULL");
    if (integrator < 0 || integrator > 5) return nfail(HB_ERR_INVALID_CONFIG, "unknown integrator");
    const bool stoch = integrator == HB_INT_EULER_STOCHASTIC || integrator == HB_INT_HEUN_STOCHASTIC || integrator == HB_INT_RK4_STOCHASTIC;
    if (stoch && (!d_noise || noise_len < n_steps * (int64_t)nnodes * mr->nvar || n_nsig < mr->nvar))
        return nfail(HB_ERR_INVALID_STATE, "stochastic integration needs noise [n_steps, nnodes*nvar] and nsig[nvar]");
    cudaStream_t st = (cudaStream_t)cuda_stream;

    // ---- network constants (engine.rs:253-257 horizon, ring semantics: runtime.rs:55-85) ----
    const int nvar = mr->nvar, ncv = mr->ncvar;
    const int H = max_delay + 1, R = H + 1, cols = nnodes * ncv;
    const int B = n_sweep;
    const size_t ring_stride = ((size_t)R * cols + 3) & ~(size_t)3;
    // ---- scratch layout and its size limit ----
    size_t off = 0;
    const size_t o_net = off;      off = align256(off + sizeof(DevNet));
    const size_t o_params = off;   off = align256(off + (size_t)B * HB_PSTRIDE * 4);
    const size_t o_cp = off;       off = align256(off + (size_t)B * HB_NCP * 4);
    const size_t o_edges = off;    off = align256(off + (size_t)std::max<int64_t>(nnz, 1) * 4);
    const size_t o_eoff = off;     off = align256(off + (size_t)std::max<int64_t>(nnz, 1) * 4);
    const size_t o_flags = off;    off = align256(off + 16);
    const size_t o_empty = off;    off = align256(off + ((size_t)nnodes + 1) * 4);
    const size_t o_ring = off;     off = align256(off + (size_t)B * ring_stride * 4);
    if (off > (size_t)HB_NOALLOC_SCRATCH_BYTES) {
        char msg[256];
        snprintf(msg, sizeof msg, "this sweep needs %zu bytes of scratch; hb_noalloc_run_csr_sweep holds at most %u",
                 off, (unsigned)HB_NOALLOC_SCRATCH_BYTES);
        return nfail(HB_ERR_UNSUPPORTED, msg);
    }
    unsigned char* scratch = nullptr;
    hb_status s = scratch_address(&scratch);
    if (s) return s;
    DevNet* d_net = reinterpret_cast<DevNet*>(scratch + o_net);
    int* d_flags = reinterpret_cast<int*>(scratch + o_flags);

    // ---- per-point parameter rows (dfun.rs:49-72 native sweep index) and coupling rows ----
    std::vector<float> prow((size_t)B * HB_PSTRIDE, 0.0f), cprow((size_t)B * HB_NCP, 0.0f);
    float cp0[HB_NCP];
    int cfk = HBC_LINEAR;
    if (!coupling_row(coupling_fn, coupling_params, n_coupling_params, nnodes, cp0, &cfk))
        return nfail(HB_ERR_UNSUPPORTED, "coupling function must be Linear, ScaledLinear, Difference, Sigmoidal or Kuramoto");
    if (cfk == HBC_KURAMOTO && ncv != 1) return nfail(HB_ERR_UNSUPPORTED, "Kuramoto coupling needs one coupling variable");
    const bool coupling_sweep = sweep_sub_idx == -1;
    if (sweep_sub_idx != 0 && !coupling_sweep) return nfail(HB_ERR_INVALID_CONFIG, "sweep_sub_idx must be 0 or -1");
    if (coupling_sweep && (sweep_param_idx < 0 || sweep_param_idx >= n_coupling_params))
        return nfail(HB_ERR_INVALID_CONFIG, "coupling sweep index out of range");
    if (!coupling_sweep && sweep_param_idx != mr->native)
        return nfail(HB_ERR_INVALID_CONFIG, "a model-parameter sweep takes the model's native sweep index only");
    const bool native = !coupling_sweep;
    std::vector<float> cpb(coupling_params, coupling_params + std::max(0, n_coupling_params));
    for (int b = 0; b < B; b++) {
        float* row = &prow[(size_t)b * HB_PSTRIDE];
        for (int k = 0; k < n_params; k++) row[k] = params[k];
        if (native) row[sweep_param_idx] = sweep_values[b];
        if (mr->id == HBM_WC) {
            row[HB_D_WC_SIG_E_OFF] = 1.0f / (1.0f + expf(row[6] * row[7]));
            row[HB_D_WC_SIG_I_OFF] = 1.0f / (1.0f + expf(row[10] * row[11]));
        }
        int kind;
        if (coupling_sweep) {
            cpb[sweep_param_idx] = sweep_values[b];
            coupling_row(coupling_fn, cpb.data(), n_coupling_params, nnodes, &cprow[(size_t)b * HB_NCP], &kind);
        }
    }

    // ---- device network description (the specialised single-projection kernel's tables) ----
    DevNet net;
    memset(&net, 0, sizeof net);
    net.n_sub = 1; net.n_proj = 1; net.n_mean = 0; net.B = B; net.H = H; net.R = R; net.cols = cols;
    net.state_len = nnodes * nvar; net.noise_row = nnodes * nvar; net.total_edges = (int)nnz;
    const float dtf = (float)dt;
    net.dt = dtf; net.dt_half = dtf * 0.5f; net.dt_sixth = dtf / 6.0f; net.dt_h2 = dtf / 2.0f;
    for (int v = 0; v < 8; v++) net.noise_scale[v] = (stoch && v < n_nsig) ? sqrtf(2.0f * nsig[v]) * sqrtf(dtf) : 0.0f;
    const double deg = nnz / (double)nnodes;
    int L = deg < 6 ? 1 : deg < 12 ? 2 : deg < 32 ? 4 : 8;
    while (L > 1 && (nnodes * L + 31) / 32 * 32 > 1024) L >>= 1;
    DevSub& sb = net.sub[0];
    sb.model = mr->id; sb.nm = nnodes; sb.nvar = nvar; sb.ncvar = ncv;
    sb.thread_off = 0; sb.col_off = 0; sb.state_off = 0; sb.noise_off = 0;
    const bool use_heun = integrator == HB_INT_HEUN;
    sb.integ = use_heun ? HBI_HEUN_DET : integrator == HB_INT_EULER ? HBI_EULER : integrator == HB_INT_EULER_STOCHASTIC ? HBI_EULER_STOCH
             : integrator == HB_INT_HEUN_STOCHASTIC ? HBI_HEUN_STOCH : integrator == HB_INT_RK4 ? HBI_RK4 : HBI_RK4_STOCH;
    sb.sweep_form = native ? 1 : 0;
    sb.lanes = L; sb.lanes_log2 = L == 1 ? 0 : L == 2 ? 1 : L == 4 ? 2 : 3;
    sb.n_in = 1; sb.in_idx[0] = 0; sb.n_mean_out = 0;
    sb.params = reinterpret_cast<const float*>(scratch + o_params);
    DevProj& pj = net.proj[0];
    pj.src = 0; pj.tgt = 0; pj.kind = HBK_SPARSE; pj.dmode = HBD_EDGE; pj.delay = 0; pj.nsrc = nnodes; pj.ntgt = nnodes;
    pj.cfk = cfk; pj.pre_cpu = 1; pj.ncv = ncv; pj.pc = cfk == HBC_KURAMOTO ? 2 : ncv; pj.oc = ncv; pj.has_rowsums = 0;
    pj.direct = 1; pj.ncm = 1; pj.mean_slot = -1; pj.maxd = max_delay; pj.w = 0.0f;
    memcpy(pj.cp, cp0, sizeof cp0);
    pj.cp_pp = coupling_sweep ? reinterpret_cast<const float*>(scratch + o_cp) : nullptr;
    pj.rowptr = d_indptr;
    pj.edges = reinterpret_cast<const uint32_t*>(scratch + o_edges);
    pj.eoff = reinterpret_cast<const int*>(scratch + o_eoff);
    pj.ew = d_weights;
    pj.rowsums = nullptr;
    const int threads = (nnodes * L + 31) / 32 * 32;
    const int budget = hb_resident_smem_budget(mr->id, cfk == HBC_KURAMOTO ? 1 : 0, threads);
    if (budget < 0) return nfail(HB_ERR_CUDA, "cannot query the kernel's shared-memory limit");
    const size_t ring_bytes = ((size_t)R * cols * 4 + 15) & ~(size_t)15, edge_bytes = ((size_t)nnz * 8 + 15) & ~(size_t)15;
    int ring_in_smem = 0, edges_in_smem = 0;
    if (ring_bytes + edge_bytes + 64 <= (size_t)budget) { ring_in_smem = 1; edges_in_smem = 1; }
    else if (ring_bytes + 64 <= (size_t)budget) ring_in_smem = 1;
    else if (edge_bytes + 64 <= (size_t)budget) edges_in_smem = 1;
    pj.smem_edges = edges_in_smem ? 0 : -1;
    const size_t smem = (ring_in_smem ? ring_bytes : 0) + (edges_in_smem ? edge_bytes : 0) + 64;

    auto cu = [&](cudaError_t e) -> hb_status { return e == cudaSuccess ? HB_OK : nfail(HB_ERR_CUDA, cudaGetErrorString(e)); };
    if ((s = cu(cudaMemcpyAsync(d_net, &net, sizeof net, cudaMemcpyHostToDevice, st)))) return s;
    if ((s = cu(cudaMemcpyAsync(scratch + o_params, prow.data(), prow.size() * 4, cudaMemcpyHostToDevice, st)))) return s;
    if (coupling_sweep && (s = cu(cudaMemcpyAsync(scratch + o_cp, cprow.data(), cprow.size() * 4, cudaMemcpyHostToDevice, st)))) return s;
    if ((s = cu(cudaMemsetAsync(d_flags, 0, 16, st)))) return s;
    {
        const int64_t work = std::max<int64_t>(nnz, nnodes + 1);
        pack_edges_kernel<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(d_indptr, d_indices, d_delays, nnz, nnodes, max_delay, ncv, cols,
                                                                        reinterpret_cast<uint32_t*>(scratch + o_edges),
                                                                        reinterpret_cast<int*>(scratch + o_eoff), d_flags);
        if ((s = cu(cudaGetLastError()))) return s;
        guard_kernel<<<1, 256, 0, st>>>(d_net, reinterpret_cast<int*>(scratch + o_empty), nnodes, d_flags);
        if ((s = cu(cudaGetLastError()))) return s;
        const int64_t n = (int64_t)B * nnodes * nvar;
        replicate_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d_x0, nnodes * nvar, B, d_final_states);
        if ((s = cu(cudaGetLastError()))) return s;
    }
    RunArgs a;
    memset(&a, 0, sizeof a);
    a.s0 = 0; a.n_steps = (int)n_steps; a.run_s0 = 0; a.run_steps = n_steps;
    a.state = d_final_states; a.tavg = d_tavg;
    a.ring = reinterpret_cast<float*>(scratch + o_ring);
    a.noise = stoch ? d_noise : d_final_states;  // not read by deterministic integrators
    a.noise_per_point = 0;
    a.traj = nullptr;
    a.ring_in_smem = ring_in_smem; a.smem_edges = edges_in_smem ? (int)nnz : 0;
    a.sync_every = 1; a.two_phase = 0; a.pipe_lanes = 1;
    a.load_ring = 0; a.store_ring = 0;
    a.flags = d_flags; a.check_finite = 0;
    a.bold.n = 0;
    if ((s = cu(hb_launch_resident(mr->id, cfk == HBC_KURAMOTO ? 1 : 0, d_net, a, B, threads, smem, st)))) return s;
    const int64_t n = (int64_t)B * nnodes * nvar;
    finish_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d_tavg, d_final_states, n, 1.0f / (float)n_steps, d_flags);
    if ((s = cu(cudaGetLastError()))) return s;
    return HB_OK;
}
