// hb_kuradj.cu — discrete adjoint of the time-averaged Kuramoto order parameter.
//
// Scope: one Kuramoto subnetwork coupled to itself through one CSR projection with per-edge delays
// (ring semantics of runtime.rs:162-204), Kuramoto coupling c_i = k (cos th_i S_i - sin th_i C_i)
// with k = a / N and S_i, C_i the weighted sums of sin and cos of the delayed source phases
// (coupling.rs Kuramoto arm), dth = omega + c (dfun.rs), deterministic Heun with the coupling held
// over the step, so th(s + 1) = wrap(th(s) + dt (omega + c(s))). The loss of sweep point b is
//     L_b = (1 / T) sum_{t=1..T} R(t),   R = |mean_j exp(i th_j)|,
// and the gradients are dL_b/da (the coupling scale swept over the points) and dL_b/domega.
//
// The forward is the engine's own run with every step's phase kept in device memory
// (HB_RUN_DEVICE_TRAJECTORY). Then:
//   kura_prep_kernel     sin and cos of every phase into node rows, time contiguous:
//                        sc [B][N][T + 1][2] (t = 0 is the initial phase)
//   kura_order_kernel    the order parameter's components per step: z [B][T][2] (t = 1..T)
//   kura_reverse_kernel  one CTA per point, one thread per node, in blocks of K steps from the end:
//                        (A) each node reads S, C of the block's steps (written by the forward's
//                        consumers, else gathered again over its in-edges) and pulls
//                        sum_e w_e nu_tgt(s + d_e) over its out-edges, two windows in flight;
//                        (B) each node runs the
//                        block's steps of
//                          lambda(s) = lambda(s+1) (1 + dt dc/dth) + cos th P_c + sin th P_s + dR/dth / T
//                        writing nu(s) = lambda(s+1) dt k (cos th(s), sin th(s)) for the pulls of
//                        earlier steps. With every delay >= K the pulled values were written in an
//                        earlier block. The gradients are summed in FP32 per block, FP64 across.
#include <cuda_runtime.h>
#include <cstdint>

#include "hb_device.h"

namespace {

constexpr int KB_TILE_T = 64;  // steps per prep tile

// [B][T][N] post-step phases (+ initial phases) -> sc [B][N][T + 1][2], via a shared tile of
// 64 steps x 32 nodes so that both the reads and the writes are contiguous
__global__ void kura_prep_kernel(const float* __restrict__ traj, const float* __restrict__ x0, int B, int N, int T,
                                 float* __restrict__ sc) {
    __shared__ float tile[KB_TILE_T][33];
    const int b = blockIdx.z, n0 = blockIdx.y * 32, t0 = blockIdx.x * KB_TILE_T;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int tt = w; tt < KB_TILE_T; tt += nw) {
        const int t = t0 + tt, n = n0 + lane;
        float th = 0.0f;
        if (t <= T && n < N) th = (t == 0) ? x0[(size_t)b * N + n] : traj[((size_t)(t - 1) * B + b) * N + n];
        tile[tt][lane] = th;
    }
    __syncthreads();
    // each warp writes whole node rows: lane l covers steps l and l + 32 of the tile
    for (int nn = w; nn < 32; nn += nw) {
        const int n = n0 + nn;
        if (n >= N) continue;
        float2* row = reinterpret_cast<float2*>(sc) + ((size_t)b * N + n) * (T + 1);
        for (int tt = lane; tt < KB_TILE_T; tt += 32) {
            const int t = t0 + tt;
            if (t > T) break;
            const float th = tile[tt][nn];
            row[t] = make_float2(sinf(th), cosf(th));
        }
    }
}

// z [B][T][2]: (mean cos, mean sin) of the phases after step t = 1..T; one warp per step
__global__ void kura_order_kernel(const float* __restrict__ traj, int B, int N, int T, float* __restrict__ z) {
    const int b = blockIdx.y;
    const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (t >= T) return;
    const float* row = traj + ((size_t)t * B + b) * N;
    double c = 0.0, s = 0.0;
    for (int n = lane; n < N; n += 32) {
        const float th = row[n];
        c += (double)cosf(th);
        s += (double)sinf(th);
    }
    for (int o = 16; o > 0; o >>= 1) {
        c += __shfl_xor_sync(0xffffffffu, c, o);
        s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    if (lane == 0) {
        z[((size_t)b * T + t) * 2] = (float)(c / N);
        z[((size_t)b * T + t) * 2 + 1] = (float)(s / N);
    }
}

__device__ __forceinline__ uint32_t kb_cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// every thread of every CTA of the cluster (release / acquire at cluster scope)
__device__ __forceinline__ void kb_cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}
// a double in the shared memory of CTA `rank` of the cluster, at the offset of `p` in this CTA
__device__ __forceinline__ double kb_ld_remote(const double* p, uint32_t rank) {
    uint32_t ra;
    double v;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"((uint32_t)__cvta_generic_to_shared(p)), "r"(rank));
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(ra) : "memory");
    return v;
}

// One point's reverse sweep, its nodes split over the C CTAs of a cluster (CTA r owns nodes
// [N r / C, N (r + 1) / C)); C = 1 is one CTA per point. Per block of K steps from the end:
// (A) the S, C of the block's steps for the owned nodes, and the pulls sum_e w_e nu_tgt(s + d_e) over
// their out-edges, gathered by whole warps: warp w takes owned nodes w, w + nwarp, ..., 32 out-edges at
// a time; lane j decodes out-edge j, and the 8 lanes of slot (lane / 8) read one edge's window of nu as
// 8 consecutive entries (lane % 8 = the block step), 4 edges per load instruction; (B) the lambda chain
// of each owned node (one thread per node). The ends of the blocks are cluster barriers, so the nu that
// a CTA writes in (B) is visible to every CTA's pulls of the next block; with every delay >= K those
// pulls read only such values. C CTAs per point keep fewer points in flight, so that their windows of
// nu stay in L2.
__global__ void __launch_bounds__(1024) kura_reverse_kernel(HbKuraAdjLaunch L, int C) {
    // S [K][ns], C [K][ns], pulled cos / sin sums [K][ns] each, (sin, cos) of the owned phases [K][ns]
    extern __shared__ __align__(16) float kb[];
    __shared__ float2 zk[8];   // the order parameter's (mean cos, mean sin) that each block step's source reads
    __shared__ double red[3][32];
    __shared__ double part[3];  // this CTA's loss and gradient sums, read by rank 0
    const int rank = C > 1 ? (int)kb_cluster_rank() : 0;
    const int b = (int)blockIdx.x / C, N = L.N, T = L.T, K = L.K;
    const int n0 = (int)(((long long)N * rank) / C), ns = (int)(((long long)N * (rank + 1)) / C) - n0;
    const int tid = threadIdx.x, i = n0 + tid;  // phase (B): thread tid owns node i
    const bool act = tid < ns;
    float* Sb = kb;
    float* Cb = kb + (size_t)K * ns;
    float* Pcb = Cb + (size_t)K * ns;
    float* Psb = Pcb + (size_t)K * ns;
    float2* Thb = reinterpret_cast<float2*>(Psb + (size_t)K * ns);
    const float2* sc = reinterpret_cast<const float2*>(L.sc) + (size_t)b * N * (T + 1);
    float2* nu = reinterpret_cast<float2*>(L.nu) + (size_t)b * N * T;
    const float2* zb = reinterpret_cast<const float2*>(L.z) + (size_t)b * T;
    const float dt = L.dt, k = L.k[b], inv_n = 1.0f / (float)N;
    const float srcw = 1.0f / ((float)T * (float)N);
    // the loss: the time average of R (FP64), summed by the point's first CTA
    double lsum = 0.0;
    if (rank == 0)
        for (int t = tid; t < T; t += blockDim.x) {
            const float2 zz = zb[t];
            lsum += sqrt((double)zz.x * zz.x + (double)zz.y * zz.y);
        }
    // dR(t)/dth_i / T at the phase th (t >= 1), the order parameter of step t - 1 given
    auto source_z = [&](float2 zz, float c, float s) {
        const float R = sqrtf(zz.x * zz.x + zz.y * zz.y);
        return R > 0.0f ? srcw * (zz.y * c - zz.x * s) / R : 0.0f;
    };
    auto source = [&](int t, float c, float s) { return source_z(zb[t - 1], c, s); };
    const int r0 = act ? L.rowptr[i] : 0, r1 = act ? L.rowptr[i + 1] : 0;
    float lam = 0.0f;
    if (act) {
        const float2 th = sc[(size_t)i * (T + 1) + T];
        lam = source(T, th.y, th.x);
    }
    const int lane = tid & 31, wid = tid >> 5, nwarp = (int)(blockDim.x >> 5);
    const int slot = lane >> 3, stp = lane & 7;
    double gA = 0.0, gW = 0.0;
    const int n_blocks = (T + K - 1) / K;
    for (int blk = 0; blk < n_blocks; blk++) {
        const int s_top = T - 1 - blk * K, nb = (s_top + 1) < K ? (s_top + 1) : K;
        // (A) the order parameter and the owned phases' sin / cos of the block's steps, off the lambda chain
        if (tid < nb && s_top - tid >= 1) zk[tid] = zb[s_top - tid - 1];
        if (act)
            for (int j = 0; j < nb; j++) Thb[j * ns + tid] = sc[(size_t)i * (T + 1) + (s_top - j)];
        // (A) S, C of the block's steps (the forward's, else gathered again over the in-edges)
        if (act) {
            if (L.cs) {
                const float2* cs = reinterpret_cast<const float2*>(L.cs);
                for (int j = 0; j < nb; j++) {
                    const float2 v = cs[((size_t)(s_top - j) * L.B + b) * N + i];
                    Sb[j * ns + tid] = v.x;
                    Cb[j * ns + tid] = v.y;
                }
            } else {
                float sS[8], sC[8];
#pragma unroll
                for (int j = 0; j < 8; j++) { sS[j] = 0.0f; sC[j] = 0.0f; }
                for (int e = r0; e < r1; e++) {
                    const uint32_t m = L.edges[e];
                    const int d = (int)(m >> 16), src = (int)(m & 0xffffu);
                    const float w = L.ew[e];
                    const float2* rs = sc + (size_t)src * (T + 1);
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        if (j < nb) {
                            const int s = s_top - j;
                            const int t = (s == 0) ? 0 : s - d;  // step 0 reads the current state
                            if (t >= 0) {
                                const float2 v = rs[t];
                                sS[j] += w * v.x;
                                sC[j] += w * v.y;
                            }
                        }
                    }
                }
#pragma unroll
                for (int j = 0; j < 8; j++)
                    if (j < nb) { Sb[j * ns + tid] = sS[j]; Cb[j * ns + tid] = sC[j]; }
            }
        }
        // (A) the pulls over the owned nodes' out-edges, whole warps at a time; lanes past a node's
        // out-edges, past the block or past the run's last step take weight 0 (their clamped reads
        // stay inside the node rows)
        for (int l = wid; l < ns; l += nwarp) {
            const int node = n0 + l;
            const int c0 = L.cptr[node], c1 = L.cptr[node + 1];
            float pc = 0.0f, ps = 0.0f;
            for (int eb = c0; eb < c1; eb += 32) {
                const int cnt = (c1 - eb) < 32 ? (c1 - eb) : 32;
                int tg = 0, top = 0;
                float w = 0.0f;
                if (lane < cnt) {
                    tg = L.ctgt[eb + lane];
                    top = s_top + L.cdel[eb + lane];  // time of the value that block step 0 pulls
                    w = L.cw[eb + lane];
                }
                float2 v[8];
                float wv[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int kk = 4 * u + slot;
                    const int tgk = __shfl_sync(0xffffffffu, tg, kk);
                    const int tt = __shfl_sync(0xffffffffu, top, kk) - stp;
                    const float wk = __shfl_sync(0xffffffffu, w, kk);
                    const bool ok = kk < cnt && stp < nb && tt <= T - 1;
                    const int tc = tt > T - 1 ? T - 1 : (tt < 0 ? 0 : tt);
                    v[u] = nu[(size_t)tgk * T + tc];
                    wv[u] = ok ? wk : 0.0f;
                }
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    pc += wv[u] == 0.0f ? 0.0f : wv[u] * v[u].x;
                    ps += wv[u] == 0.0f ? 0.0f : wv[u] * v[u].y;
                }
            }
            pc += __shfl_xor_sync(0xffffffffu, pc, 8);
            pc += __shfl_xor_sync(0xffffffffu, pc, 16);
            ps += __shfl_xor_sync(0xffffffffu, ps, 8);
            ps += __shfl_xor_sync(0xffffffffu, ps, 16);
            if (slot == 0 && stp < nb) {
                Pcb[stp * ns + l] = pc;
                Psb[stp * ns + l] = ps;
            }
        }
        __syncthreads();
        // (B) the block's steps of the lambda chain
        if (act) {
            float fa = 0.0f, fw = 0.0f;
            for (int j = 0; j < nb; j++) {
                const int s = s_top - j;
                const float2 th = Thb[j * ns + tid];  // (sin, cos)
                const float S = Sb[j * ns + tid], Cc = Cb[j * ns + tid];
                const float tcs = th.y * S - th.x * Cc;  // c / k
                fa += lam * dt * tcs * inv_n;
                fw += lam * dt;
                nu[(size_t)i * T + s] = make_float2(lam * dt * k * th.y, lam * dt * k * th.x);
                if (s >= 1) {
                    const float q = k * (-th.x * S - th.y * Cc);  // dc/dth
                    const float pb = th.y * Pcb[j * ns + tid] + th.x * Psb[j * ns + tid];
                    lam = lam * (1.0f + dt * q) + pb + source_z(zk[j], th.y, th.x);
                }
            }
            gA += fa;
            gW += fw;
        }
        // nu of this block in every CTA of the point before the pulls of the next
        if (C > 1) kb_cluster_barrier();
        else __syncthreads();
    }
    if (act && L.gWn) L.gWn[(size_t)b * N + i] = gW;
    // block sums of the loss and the two gradients (FP64), then the point's CTAs in rank order
    double v3[3] = {lsum, gA, gW};
#pragma unroll
    for (int q = 0; q < 3; q++)
        for (int o = 16; o > 0; o >>= 1) v3[q] += __shfl_xor_sync(0xffffffffu, v3[q], o);
    if ((tid & 31) == 0)
        for (int q = 0; q < 3; q++) red[q][tid >> 5] = v3[q];
    __syncthreads();
    if (tid == 0) {
        double s3[3] = {0.0, 0.0, 0.0};
        for (int wv = 0; wv < nwarp; wv++)
            for (int q = 0; q < 3; q++) s3[q] += red[q][wv];
        for (int q = 0; q < 3; q++) part[q] = s3[q];
    }
    if (C > 1) kb_cluster_barrier();
    else __syncthreads();
    if (rank == 0 && tid == 0) {
        double s3[3] = {0.0, 0.0, 0.0};
        for (int r = 0; r < C; r++)
            for (int q = 0; q < 3; q++) s3[q] += C > 1 ? kb_ld_remote(&part[q], (uint32_t)r) : part[q];
        L.loss[b] = s3[0] / T;
        L.gA[b] = s3[1];
        L.gW[b] = s3[2];
    }
    // no CTA leaves while the first may still read its partial sums
    if (C > 1) kb_cluster_barrier();
}

}  // namespace

cudaError_t hb_launch_kura_adjoint(const HbKuraAdjLaunch& L, int phase, cudaStream_t st) {
    if (phase == 0) {
        dim3 g1((L.T + 1 + KB_TILE_T - 1) / KB_TILE_T, (L.N + 31) / 32, L.B);
        kura_prep_kernel<<<g1, 256, 0, st>>>(L.traj, L.x0, L.B, L.N, L.T, L.sc);
        dim3 g2((L.T + 7) / 8, L.B);
        kura_order_kernel<<<g2, 256, 0, st>>>(L.traj, L.B, L.N, L.T, L.z);
        return cudaGetLastError();
    }
    // CTAs per point: among 1..8 (at least 64 nodes per CTA), the size whose resident clusters keep the
    // points' windows of nu (N x (largest delay + 2K) entries each) within about 100 MB of L2, then the
    // most SMs busy
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const double window = (double)L.N * (L.maxd + 2 * L.K) * 8.0;
    int C = 1;
    double best = -1.0;
    bool best_fit = false;
    for (int c = 1; c <= 8; c++) {
        if (c > 1 && L.N / c < 64) break;
        const int ns = (L.N + c - 1) / c;
        const size_t sm = (size_t)6 * L.K * ns * sizeof(float);
        cudaError_t e = cudaFuncSetAttribute(kura_reverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        int cap = sms;
        if (c > 1) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)(c * 64));
            cfg.blockDim = dim3(1024);
            cfg.dynamicSmemBytes = sm;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = (unsigned)c;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            if (cudaOccupancyMaxActiveClusters(&cap, kura_reverse_kernel, &cfg) != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
        }
        if (cap <= 0) continue;
        const double inflight = cap < L.B ? cap : L.B;
        const bool fit = inflight * window <= 100e6;
        const double score = inflight * c;
        if (best < 0 || (fit && !best_fit) || (fit == best_fit && score > best)) {
            best = score;
            best_fit = fit;
            C = c;
        }
    }
    const int ns = (L.N + C - 1) / C;
    const size_t sm = (size_t)6 * L.K * ns * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(kura_reverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    if (C == 1) {
        kura_reverse_kernel<<<L.B, 1024, sm, st>>>(L, 1);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(L.B * C));
    cfg.blockDim = dim3(1024);
    cfg.dynamicSmemBytes = sm;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kura_reverse_kernel, L, C);
}
