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

__global__ void __launch_bounds__(1024) kura_reverse_kernel(HbKuraAdjLaunch L) {
    extern __shared__ __align__(16) float kb[];  // S [K][N], C [K][N], P [K][N]
    const int b = blockIdx.x, N = L.N, T = L.T, K = L.K;
    const int i = threadIdx.x;
    const bool act = i < N;
    float* Sb = kb;
    float* Cb = kb + (size_t)K * N;
    float* Pb = Cb + (size_t)K * N;
    const float2* sc = reinterpret_cast<const float2*>(L.sc) + (size_t)b * N * (T + 1);
    float2* nu = reinterpret_cast<float2*>(L.nu) + (size_t)b * N * T;
    const float2* zb = reinterpret_cast<const float2*>(L.z) + (size_t)b * T;
    const float dt = L.dt, k = L.k[b], inv_n = 1.0f / (float)N;
    const float srcw = 1.0f / ((float)T * (float)N);
    // the loss: the time average of R (FP64)
    double lsum = 0.0;
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
        const float2 zz = zb[t];
        lsum += sqrt((double)zz.x * zz.x + (double)zz.y * zz.y);
    }
    // dR(t)/dth_i / T at the phase th (t >= 1)
    auto source = [&](int t, float c, float s) {
        const float2 zz = zb[t - 1];
        const float R = sqrtf(zz.x * zz.x + zz.y * zz.y);
        return R > 0.0f ? srcw * (zz.y * c - zz.x * s) / R : 0.0f;
    };
    const int r0 = act ? L.rowptr[i] : 0, r1 = act ? L.rowptr[i + 1] : 0;
    const int c0 = act ? L.cptr[i] : 0, c1 = act ? L.cptr[i + 1] : 0;
    float lam = 0.0f;
    if (act) {
        const float2 th = sc[(size_t)i * (T + 1) + T];
        lam = source(T, th.y, th.x);
    }
    double gA = 0.0, gW = 0.0;
    const int n_blocks = (T + K - 1) / K;
    for (int blk = 0; blk < n_blocks; blk++) {
        const int s_top = T - 1 - blk * K, nb = (s_top + 1) < K ? (s_top + 1) : K;
        // (A) S, C of the block's steps (the forward's, else gathered again over the in-edges), and
        // the pulls over the out-edges, two windows in flight per iteration
        if (act) {
            if (L.cs) {
                const float2* cs = reinterpret_cast<const float2*>(L.cs);
                for (int j = 0; j < nb; j++) {
                    const float2 v = cs[((size_t)(s_top - j) * L.B + b) * N + i];
                    Sb[j * N + i] = v.x;
                    Cb[j * N + i] = v.y;
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
                    if (j < nb) { Sb[j * N + i] = sS[j]; Cb[j * N + i] = sC[j]; }
            }
            float pc[8], ps[8];
#pragma unroll
            for (int j = 0; j < 8; j++) { pc[j] = 0.0f; ps[j] = 0.0f; }
            int e = c0;
            for (; e + 1 < c1; e += 2) {
                const int tg0 = L.ctgt[e], d0 = L.cdel[e], tg1 = L.ctgt[e + 1], d1 = L.cdel[e + 1];
                const float w0 = L.cw[e], w1 = L.cw[e + 1];
                const float2* rn0 = nu + (size_t)tg0 * T;
                const float2* rn1 = nu + (size_t)tg1 * T;
                float2 v0[8], v1[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const int t0 = s_top - j + d0, t1 = s_top - j + d1;
                    v0[j] = (j < nb && t0 <= T - 1) ? rn0[t0] : make_float2(0.0f, 0.0f);
                    v1[j] = (j < nb && t1 <= T - 1) ? rn1[t1] : make_float2(0.0f, 0.0f);
                }
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    pc[j] += w0 * v0[j].x;
                    ps[j] += w0 * v0[j].y;
                    pc[j] += w1 * v1[j].x;
                    ps[j] += w1 * v1[j].y;
                }
            }
            if (e < c1) {
                const int tg = L.ctgt[e], d = L.cdel[e];
                const float w = L.cw[e];
                const float2* rn = nu + (size_t)tg * T;
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const int t = s_top - j + d;
                    if (j < nb && t <= T - 1) {
                        const float2 v = rn[t];
                        pc[j] += w * v.x;
                        ps[j] += w * v.y;
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < 8; j++) {
                if (j < nb) {
                    const float2 th = sc[(size_t)i * (T + 1) + (s_top - j)];
                    Pb[j * N + i] = th.y * pc[j] + th.x * ps[j];
                }
            }
        }
        __syncthreads();
        // (B) the block's steps of the lambda chain
        if (act) {
            float fa = 0.0f, fw = 0.0f;
            for (int j = 0; j < nb; j++) {
                const int s = s_top - j;
                const float2 th = sc[(size_t)i * (T + 1) + s];  // (sin, cos)
                const float S = Sb[j * N + i], C = Cb[j * N + i];
                const float tcs = th.y * S - th.x * C;           // c / k
                fa += lam * dt * tcs * inv_n;
                fw += lam * dt;
                nu[(size_t)i * T + s] = make_float2(lam * dt * k * th.y, lam * dt * k * th.x);
                if (s >= 1) {
                    const float q = k * (-th.x * S - th.y * C);  // dc/dth
                    lam = lam * (1.0f + dt * q) + Pb[j * N + i] + source(s, th.y, th.x);
                }
            }
            gA += fa;
            gW += fw;
        }
        __syncthreads();  // nu of this block before the pulls of the next
    }
    if (act && L.gWn) L.gWn[(size_t)b * N + i] = gW;
    // block sums of the loss and the two gradients (FP64)
    __shared__ double red[3][32];
    double v[3] = {lsum, gA, gW};
#pragma unroll
    for (int q = 0; q < 3; q++)
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < 3; q++) red[q][threadIdx.x >> 5] = v[q];
    __syncthreads();
    if (threadIdx.x == 0) {
        double s3[3] = {0.0, 0.0, 0.0};
        for (int wv = 0; wv < (int)(blockDim.x >> 5); wv++)
            for (int q = 0; q < 3; q++) s3[q] += red[q][wv];
        L.loss[b] = s3[0] / T;
        L.gA[b] = s3[1];
        L.gW[b] = s3[2];
    }
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
    const int threads = (L.N + 31) / 32 * 32;
    const size_t sm = (size_t)3 * L.K * L.N * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(kura_reverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    kura_reverse_kernel<<<L.B, threads, sm, st>>>(L);
    return cudaGetLastError();
}
