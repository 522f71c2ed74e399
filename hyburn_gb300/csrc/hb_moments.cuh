// hb_moments.cuh — second moments of N time series over a range of steps: the building block of
// Pearson functional connectivity, shared by the FC-loss adjoint (hb_adjoint.cu) and the FC / FCD
// features (hb_features.cu).
#pragma once
#include <cstdint>

namespace hb {

constexpr int MOM_CHUNK = 64;  // steps summed in FP32 before an FP64 accumulation (default)

// the 4 x 4 tile (bi, bj) of the upper triangle owned by a thread, or (-1, -1)
__device__ __forceinline__ void moment_tile(int tile, int N4, int n_tiles, int& bi, int& bj) {
    bi = -1;
    bj = -1;
    if (tile < n_tiles) {
        int rem = tile;
        bi = 0;
        while (rem >= N4 - bi) { rem -= N4 - bi; bi++; }
        bj = bi + rem;
    }
}

// products of one staged chunk (nt rows of W shifted values) for tile (bi, bj), summed in FP32 and
// added to the FP64 accumulators; the column sum of the thread's series when it owns one
__device__ __forceinline__ void moment_chunk(const float* zs, int W, int nt, int bi, int bj, bool col, double& ssum,
                                             double (&acc)[4][4]) {
    if (col) {
        float s1 = 0.0f;
        for (int tt = 0; tt < nt; tt++) s1 += zs[tt * W + threadIdx.x];
        ssum += s1;
    }
    if (bi < 0) return;
    float part4[4][4];
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

__device__ __forceinline__ void moment_store(double* P, int W, int bi, int bj, const double (&acc)[4][4]) {
    if (bi < 0) return;
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) {
            P[(size_t)(bi * 4 + u) * W + bj * 4 + v] = acc[u][v];
            P[(size_t)(bj * 4 + v) * W + bi * 4 + u] = acc[u][v];
        }
}

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
        int bi, bj;
        moment_tile(base + tid, N4, n_tiles, bi, bj);
        double acc[4][4];
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
            moment_chunk(zs, W, nt, bi, bj, base == 0 && tid < N, ssum, acc);
        }
        moment_store(P, W, bi, bj, acc);
    }
    if (tid < W) P[(size_t)W * W + tid] = tid < N ? ssum : 0.0;
}

__device__ __forceinline__ void cp_async_f32(float* dst, const float* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N_PENDING>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N_PENDING) : "memory"); }

// series_moments for series that are plain strided loads, y_k(t) = base[t * ts + k * ks]: the next
// chunk is copied into shared memory (cp.async) while the current one is multiplied. Each thread
// shifts the values it copied once its copies have landed. zs: 2 * CHUNK * W floats of 16-byte
// aligned shared memory. Same results as series_moments with the same arguments.
template <int CHUNK = MOM_CHUNK>
__device__ __forceinline__ void series_moments_strided(const float* base, size_t ts, int ks, int N, int t_lo, int t_hi,
                                                       const float* shift, float* zs, double* P) {
    const int tid = threadIdx.x, nth = blockDim.x;
    const int N4 = (N + 3) / 4, W = N4 * 4;
    double ssum = 0.0;
    const int n_tiles = N4 * (N4 + 1) / 2;
    const int n_chunks = t_hi > t_lo ? (t_hi - t_lo + CHUNK - 1) / CHUNK : 0;
    // stage chunk c into buffer c & 1: copies of this thread's rows and lanes, zeros past the range
    auto stage = [&](int c) {
        float* buf = zs + (size_t)(c & 1) * CHUNK * W;
        const int t0 = t_lo + c * CHUNK;
        const int nt = (t_hi - t0) < CHUNK ? (t_hi - t0) : CHUNK;
        for (int tt = tid >> 5; tt < CHUNK; tt += nth >> 5)
            for (int k = tid & 31; k < W; k += 32) {
                if (tt < nt && k < N) cp_async_f32(buf + tt * W + k, base + (size_t)(t0 + tt) * ts + (size_t)k * ks);
                else buf[tt * W + k] = 0.0f;
            }
        cp_async_commit();
    };
    for (int pass = 0; pass < n_tiles; pass += nth) {
        int bi, bj;
        moment_tile(pass + tid, N4, n_tiles, bi, bj);
        double acc[4][4];
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int v = 0; v < 4; v++) acc[u][v] = 0.0;
        __syncthreads();  // the buffers are free (previous pass) and the shifts are written
        if (n_chunks > 0) stage(0);
        for (int c = 0; c < n_chunks; c++) {
            if (c + 1 < n_chunks) {
                stage(c + 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            float* buf = zs + (size_t)(c & 1) * CHUNK * W;
            const int t0 = t_lo + c * CHUNK;
            const int nt = (t_hi - t0) < CHUNK ? (t_hi - t0) : CHUNK;
            for (int tt = tid >> 5; tt < nt; tt += nth >> 5)
                for (int k = tid & 31; k < N; k += 32) buf[tt * W + k] -= shift[k];
            __syncthreads();
            moment_chunk(buf, W, nt, bi, bj, pass == 0 && tid < N, ssum, acc);
            __syncthreads();  // buffer c & 1 is restaged at chunk c + 2
        }
        moment_store(P, W, bi, bj, acc);
    }
    if (tid < W) P[(size_t)W * W + tid] = tid < N ? ssum : 0.0;
}

}  // namespace hb
