// hb_moments.cuh — second moments of N time series over a range of steps: the building block of
// Pearson functional connectivity, shared by the FC-loss adjoint (hb_adjoint.cu) and the FC / FCD
// features (hb_features.cu).
#pragma once
#include <cstdint>

namespace hb {

constexpr int MOM_CHUNK = 64;  // steps summed in FP32 before an FP64 accumulation (default)

// Sums over t in [t_lo, t_hi) of z_i(t) z_j(t) and of z_k(t), where z_k(t) = load(t, k) - shift[k],
// for N series padded to W = 4 ceil(N / 4). Written to P as Q [W][W] (full, symmetric), then S [W].
// Products are summed in FP32 over chunks of CHUNK steps and in FP64 across chunks; each thread
// owns a 4 x 4 tile of Q's upper triangle (several passes over the range when the tiles outnumber
// the threads). zs: CHUNK * W floats of 16-byte aligned shared memory; shift: W floats of shared
// memory, written before the call (the first barrier inside orders it). Needs N <= blockDim.x and
// blockDim.x a multiple of 32; every thread of the block calls it.
template <int CHUNK = MOM_CHUNK, class Load>
__device__ __forceinline__ void series_moments(const Load& load, int N, int t_lo, int t_hi, const float* shift,
                                               float* zs, double* P) {
    const int tid = threadIdx.x, nth = blockDim.x;
    const int N4 = (N + 3) / 4, W = N4 * 4;
    double ssum = 0.0;
    const int n_tiles = N4 * (N4 + 1) / 2;
    for (int base = 0; base < n_tiles; base += nth) {
        const int tile = base + tid;
        int bi = -1, bj = -1;
        if (tile < n_tiles) {
            int rem = tile;
            bi = 0;
            while (rem >= N4 - bi) { rem -= N4 - bi; bi++; }
            bj = bi + rem;
        }
        double acc[4][4];
        float part4[4][4];
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int v = 0; v < 4; v++) acc[u][v] = 0.0;
        for (int t0 = t_lo; t0 < t_hi; t0 += CHUNK) {
            const int nt = (t_hi - t0) < CHUNK ? (t_hi - t0) : CHUNK;
            __syncthreads();
            // one step per warp at a time, its lanes along the series (no index division)
            for (int tt = tid >> 5; tt < CHUNK; tt += nth >> 5)
                for (int k = tid & 31; k < W; k += 32) {
                    float z = 0.0f;
                    if (tt < nt && k < N) z = load(t0 + tt, k) - shift[k];
                    zs[tt * W + k] = z;
                }
            __syncthreads();
            if (base == 0 && tid < N) {
                float s1 = 0.0f;
                for (int tt = 0; tt < nt; tt++) s1 += zs[tt * W + tid];
                ssum += s1;
            }
            if (bi < 0) continue;
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) part4[u][v] = 0.0f;
            for (int tt = 0; tt < nt; tt++) {
                const float4 zi = *reinterpret_cast<const float4*>(zs + tt * W + bi * 4);
                const float4 zj = *reinterpret_cast<const float4*>(zs + tt * W + bj * 4);
                const float ai[4] = {zi.x, zi.y, zi.z, zi.w}, aj[4] = {zj.x, zj.y, zj.z, zj.w};
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int v = 0; v < 4; v++) part4[u][v] = __fmaf_rn(ai[u], aj[v], part4[u][v]);
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) acc[u][v] += part4[u][v];
        }
        if (bi >= 0) {
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    P[(size_t)(bi * 4 + u) * W + bj * 4 + v] = acc[u][v];
                    P[(size_t)(bj * 4 + v) * W + bi * 4 + u] = acc[u][v];
                }
        }
    }
    if (tid < W) P[(size_t)W * W + tid] = tid < N ? ssum : 0.0;
}

}  // namespace hb
