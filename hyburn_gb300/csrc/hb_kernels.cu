// hb_kernels.cu — batch-mean BOLD kernels and the launch dispatch of the simulation kernels.
//
// The point-resident persistent kernel lives in hb_resident.cuh (instantiated per model and
// launch bound in hb_resident_{256,512,1024}.cu). The batch-mean BOLD monitor (mean over sweep
// points of var0, engine.rs:786-801) runs after the simulation kernel from per-point window
// sums: bold_reduce_kernel averages over points, bold_bw_kernel integrates the
// Balloon-Windkessel ODE per node and applies the TR down-sampling schedule.
#include <cuda_runtime.h>
#include "hb_models.cuh"

namespace hb {

// batch-mean BOLD, stage 1: mean over sweep points of each window sum -> means[w][n]
__global__ void bold_reduce_kernel(const float* __restrict__ win, int n_windows, int B, int N0, float* __restrict__ means) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)n_windows * N0) return;
    int w = (int)(i / N0), n = (int)(i % N0);
    const float* p = win + (size_t)w * B * N0 + n;
    float acc = 0.0f;
    for (int bb = 0; bb < B; bb++) acc += p[(size_t)bb * N0];
    means[i] = acc / (float)B;
}

// batch-mean BOLD, stage 2: one thread per node walks the windows in order (bold_monitor.rs:86-106)
__global__ void bold_bw_kernel(DevBold bold, int m, const float* __restrict__ means, int n_windows) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int N0 = bold.n0;
    if (n >= N0) return;
    float* bw = bold.bw[m];
    float bs = bw[n], bf = bw[N0 + n], bv = bw[2 * N0 + n], bq = bw[3 * N0 + n], prev = bw[4 * N0 + n];
    const BoldEmit* em = bold.emit[m];
    int j = 0;
    for (int w = 0; w < n_windows; w++) {
        bool full = w < bold.n_full[m];
        int cnt = full ? bold.period[m] : bold.partial[m];
        float avg = means[(size_t)w * N0 + n] / (float)cnt;
        bw_step(bs, bf, bv, bq, avg, full ? bold.dt_full[m] : bold.dt_part[m]);
        float cur = bw_signal(bv, bq);
        while (j < bold.n_emit[m] && em[j].k < w) j++;
        for (; j < bold.n_emit[m] && em[j].k == w; j++) {
            float val = em[j].interp ? prev + (cur - prev) * em[j].w : cur;
            bold.out[m][(size_t)em[j].out * N0 + n] = val;
        }
        prev = cur;
    }
    bw[n] = bs; bw[N0 + n] = bf; bw[2 * N0 + n] = bv; bw[3 * N0 + n] = bq; bw[4 * N0 + n] = prev;
}

}  // namespace hb

// ---- launch wrappers (called by the host engine) ----
cudaError_t hb_launch_resident_256(int model, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
cudaError_t hb_launch_resident_512(int model, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
cudaError_t hb_launch_resident_1024(int model, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
int hb_resident_budget_256(int model);
int hb_resident_budget_512(int model);
int hb_resident_budget_1024(int model);

cudaError_t hb_launch_fast_512(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
cudaError_t hb_launch_fast_1024(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
int hb_fast_budget_512(int model, int pre);
int hb_fast_budget_1024(int model, int pre);

// fast >= 0 selects the specialised single-projection kernel with that pre() kind
cudaError_t hb_launch_resident(int model, int fast, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem,
                               cudaStream_t st) {
    if (fast >= 0) {
        if (threads <= 512) return hb_launch_fast_512(model, fast, d_net, a, B, threads, smem, st);
        return hb_launch_fast_1024(model, fast, d_net, a, B, threads, smem, st);
    }
    if (threads <= 256) return hb_launch_resident_256(model, d_net, a, B, threads, smem, st);
    if (threads <= 512) return hb_launch_resident_512(model, d_net, a, B, threads, smem, st);
    return hb_launch_resident_1024(model, d_net, a, B, threads, smem, st);
}

// dynamic shared memory available to a resident launch of `threads` threads
int hb_resident_smem_budget(int model, int fast, int threads) {
    if (fast >= 0) return threads <= 512 ? hb_fast_budget_512(model, fast) : hb_fast_budget_1024(model, fast);
    if (threads <= 256) return hb_resident_budget_256(model);
    if (threads <= 512) return hb_resident_budget_512(model);
    return hb_resident_budget_1024(model);
}

cudaError_t hb_launch_bold_batch_mean(const DevBold& bold, int m, int n_windows, int B, float* means, cudaStream_t st) {
    if (n_windows <= 0) return cudaSuccess;
    int64_t total = (int64_t)n_windows * bold.n0;
    int blocks = (int)((total + 255) / 256);
    hb::bold_reduce_kernel<<<blocks, 256, 0, st>>>(bold.win[m], n_windows, B, bold.n0, means);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    hb::bold_bw_kernel<<<(bold.n0 + 127) / 128, 128, 0, st>>>(bold, m, means, n_windows);
    return cudaGetLastError();
}

