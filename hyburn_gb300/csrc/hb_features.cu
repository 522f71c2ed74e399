// hb_features.cu — functional-connectivity features of a trajectory kept in device memory
// (HB_RUN_DEVICE_TRAJECTORY), so that no step's state crosses to the host: the FeatureSet::Fc arm
// of sbi/features/mod.rs:257-280 and sbi/features/fc.rs:11-186.
//
// For every sweep point b and state variable v, the node series is the mean over modes,
//     y_n(t) = (sum_m x[t][b][n * nmodes + m][v]) / nmodes   (f32, modes in order, mod.rs:262-271),
// and
//   FC       Pearson correlation over all steps (fc.rs:11-58): means and deviations over T (not
//            T - 1), a deviation below 1e-12 replaced by 1, every entry (the diagonal included)
//            cov / (sd_i sd_j) clamped to [-1, 1];
//   features fc_stats of FC's upper triangle (mean, std, min, max, median; fc.rs:62-83) and the
//            homotopic mean and std of FC[i][N-1-i] (fc.rs:189-203): 7 values per (b, v);
//   FCD      FC of each window [w * stride, w * stride + window) (fc.rs:87-141; when window and
//            stride share a divisor G >= 64, from moments of G-step blocks computed once and
//            combined per window by the parallel-axis formula), then the Pearson
//            correlation of every pair of window FCs' upper triangles (fc.rs:144-179; FP32
//            products of the centred values, summed in FP64), diagonal 1;
//            and fc_stats of that matrix (fc.rs:182-187).
// Moments use hb::series_moments (FP32 sums over chunks of steps, FP64 across chunks) on the series
// shifted by the FP64 mean of the range's first 64 steps rounded to f32, so that a constant series
// gives exactly zero deviation, as in the reference. The statistics use the reference's f32
// summation order (one thread); the median is the k-th smallest value, found by bisection on the
// values' ordered bit patterns.
#include <cuda_runtime.h>
#include <cstdint>

#include "hb_device.h"
#include "hb_moments.cuh"

namespace {

// one range's moments in the workspace: Q [W][W], S [W] (sums of y - shift), the shift [W]
__host__ __device__ __forceinline__ size_t part_len(int N) {
    const size_t W = (size_t)(N + 3) / 4 * 4;
    return W * W + 2 * W;
}

// the upper-triangle entry u (row-major, i < j) of an N x N matrix as (i, j)
__device__ __forceinline__ void ut_index(size_t u, int N, int& i, int& j) {
    i = (int)((2.0 * N - 1.0 - sqrt((2.0 * N - 1.0) * (2.0 * N - 1.0) - 8.0 * (double)u)) * 0.5);
    while (i > 0 && (size_t)i * N - (size_t)i * (i + 1) / 2 > u) i--;
    while ((size_t)(i + 1) * N - (size_t)(i + 1) * (i + 2) / 2 <= u) i++;
    j = (int)(u - ((size_t)i * N - (size_t)i * (i + 1) / 2)) + i + 1;
}

// moments of range r = blockIdx.y / slices ([r * stride, r * stride + len)), slice blockIdx.y % slices,
// of point-variable blockIdx.x of the batch
template <int CHUNK, int MAXT>
__global__ void __launch_bounds__(MAXT, MAXT <= 256 ? 3 : 1) feat_moments_kernel(HbFeatLaunch L, int n_ranges, int stride, int len,
                                                            int slices) {
    extern __shared__ __align__(16) float zs[];  // [2][CHUNK][W] chunks of y - shift, then shift[W]
    const int bv = blockIdx.x, b = L.b0 + bv / L.nvar, v = bv - (bv / L.nvar) * L.nvar;
    const int r = blockIdx.y / slices, sl = blockIdx.y - r * slices;
    const int N = L.nnodes, W = (N + 3) / 4 * 4;
    const int start = r * stride;
    const int Tc = ((len + slices - 1) / slices + CHUNK - 1) / CHUNK * CHUNK;
    const int t_lo = start + sl * Tc, t_end = start + len;
    const int t_hi = (t_lo + Tc) < t_end ? (t_lo + Tc) : t_end;
    float* shift = zs + 2 * CHUNK * W;
    // the series of point b, variable v: x[t * tstride + n * nstride + m * nvar]
    const float* x0 = L.traj + (size_t)b * L.state_len + L.off + v;
    const size_t tstride = (size_t)L.B * L.state_len;
    const int nvar = L.nvar, nmodes = L.nmodes, nstride = L.nmodes * L.nvar;
    const float fm = (float)nmodes;
    auto load = [=](int t, int n) {
        const float* x = x0 + (size_t)t * tstride + (size_t)n * nstride;
        if (nmodes == 1) return x[0];  // (0 + x) / 1 == x up to the sign of zero
        float s = 0.0f;
        for (int m = 0; m < nmodes; m++) s += x[(size_t)m * nvar];
        return s / fm;
    };
    const int n0 = len < 64 ? len : 64;
    for (int k = threadIdx.x; k < W; k += blockDim.x) {
        double c = 0.0;
        if (k < N) {
            for (int t = 0; t < n0; t++) c += (double)load(start + t, k);
            c /= n0;
        }
        shift[k] = (float)c;
    }
    double* P = L.part + (((size_t)bv * n_ranges + r) * slices + sl) * part_len(N);
    if (nmodes == 1) hb::series_moments_strided<CHUNK>(x0, tstride, nvar, N, t_lo, t_hi, shift, zs, P);
    else hb::series_moments<CHUNK>(load, N, t_lo, t_hi, shift, zs, P);
    for (int k = threadIdx.x; k < W; k += blockDim.x) P[(size_t)W * W + W + k] = (double)shift[k];
}

// FC of range blockIdx.y from its slices' moments: the full matrix into `full` and / or the upper
// triangle (row-major, i < j) into `ut`
__global__ void feat_corr_kernel(HbFeatLaunch L, int n_ranges, int len, int slices, float* full, float* ut) {
    extern __shared__ __align__(16) double ms[];  // mean [W], 1 / sd [W]
    const int bv = blockIdx.x, r = blockIdx.y;
    const int N = L.nnodes, W = (N + 3) / 4 * 4;
    const size_t pl = part_len(N);
    const double* P0 = L.part + ((size_t)bv * n_ranges + r) * slices * pl;
    double* mean = ms;
    double* rsd = ms + W;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        double s1 = 0.0, s2 = 0.0;
        for (int q = 0; q < slices; q++) {
            s1 += P0[q * pl + (size_t)W * W + k];
            s2 += P0[q * pl + (size_t)k * W + k];
        }
        const double m = s1 / len, var = s2 / len - m * m;
        double d = sqrt(var > 0.0 ? var : 0.0);
        if (d < 1e-12) d = 1.0;  // constant series (fc.rs:35-37)
        mean[k] = m;
        rsd[k] = 1.0 / d;
    }
    __syncthreads();
    const size_t rr = (size_t)bv * n_ranges + r;
    const size_t n_ut = (size_t)N * (N - 1) / 2;
    const double rlen = 1.0 / len;
    if (full) {
        for (int q = threadIdx.x; q < N * N; q += blockDim.x) {
            const int i = q / N, j = q - (q / N) * N;
            double qs = 0.0;
            for (int s = 0; s < slices; s++) qs += P0[s * pl + (size_t)i * W + j];
            double c = (qs * rlen - mean[i] * mean[j]) * rsd[i] * rsd[j];
            c = c < -1.0 ? -1.0 : (c > 1.0 ? 1.0 : c);
            full[rr * N * N + q] = (float)c;
        }
    } else {
        // upper triangle only, in its row-major order
        for (size_t u = threadIdx.x; u < n_ut; u += blockDim.x) {
            int i, j;
            ut_index(u, N, i, j);
            double qs = 0.0;
            for (int s = 0; s < slices; s++) qs += P0[s * pl + (size_t)i * W + j];
            double c = (qs * rlen - mean[i] * mean[j]) * rsd[i] * rsd[j];
            c = c < -1.0 ? -1.0 : (c > 1.0 ? 1.0 : c);
            ut[rr * n_ut + u] = (float)c;
        }
    }
}

// FC upper triangle of window w = blockIdx.y from the moments of its K consecutive blocks of G
// steps (blocks w * (stride / G) ...), combined exactly by the parallel-axis formula: with block
// means mu_q = shift_q + S_q / G and the window mean mu,
//   M_ij = sum_q (Q_q,ij - S_q,i S_q,j / G) + G sum_q (mu_q,i - mu_i)(mu_q,j - mu_j),  cov = M / (K G).
// A series constant over the window has M = 0 exactly (each block's shift is its value).
__global__ void feat_corr_blocks_kernel(HbFeatLaunch L, int n_blocks, int G, int K, int step) {
    extern __shared__ __align__(16) double sb[];  // S [K][W], S / G [K][W], mu_q - mu [K][W], 1/sd [W]
    const int bv = blockIdx.x, w = blockIdx.y;
    const int N = L.nnodes, W = (N + 3) / 4 * 4;
    const size_t pl = part_len(N);
    const double* P0 = L.part + ((size_t)bv * n_blocks + (size_t)w * step) * pl;
    double* S = sb;
    double* Sg = sb + (size_t)K * W;
    double* dq = Sg + (size_t)K * W;
    double* rsd = dq + (size_t)K * W;
    const double g = (double)G, rg = 1.0 / g, rlen = 1.0 / ((double)K * G);
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        double m = 0.0;
        for (int q = 0; q < K; q++) {
            const double sq = P0[q * pl + (size_t)W * W + k];
            S[q * W + k] = sq;
            Sg[q * W + k] = sq * rg;
            const double mb = P0[q * pl + (size_t)W * W + W + k] + sq * rg;
            dq[q * W + k] = mb;
            m += mb;
        }
        m /= K;
        double M = 0.0;
        for (int q = 0; q < K; q++) {
            const double d = dq[q * W + k] - m;
            dq[q * W + k] = d;
            M += P0[q * pl + (size_t)k * W + k] - S[q * W + k] * Sg[q * W + k] + g * d * d;
        }
        double sd = sqrt(M > 0.0 ? M * rlen : 0.0);
        if (sd < 1e-12) sd = 1.0;
        rsd[k] = 1.0 / sd;
    }
    __syncthreads();
    const size_t n_ut = (size_t)N * (N - 1) / 2;
    float* out = L.ut + ((size_t)bv * L.n_windows + w) * n_ut;
    for (size_t u = threadIdx.x; u < n_ut; u += blockDim.x) {
        int i, j;
        ut_index(u, N, i, j);
        double M = 0.0;
        for (int q = 0; q < K; q++)
            M += P0[q * pl + (size_t)i * W + j] - S[q * W + i] * Sg[q * W + j] + g * dq[q * W + i] * dq[q * W + j];
        double c = M * rlen * rsd[i] * rsd[j];
        c = c < -1.0 ? -1.0 : (c > 1.0 ? 1.0 : c);
        out[u] = (float)c;
    }
}

template <class T>
__device__ __forceinline__ T block_sum(T x, T* red) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[w] = x;
    __syncthreads();
    T s = 0;
    for (int i = 0; i < nw; i++) s += red[i];
    return s;
}

// mean and centred sum of squares of each window FC's upper triangle (FP64)
__global__ void feat_ut_moments_kernel(HbFeatLaunch L) {
    __shared__ double red[32];
    const size_t n_ut = (size_t)L.nnodes * (L.nnodes - 1) / 2;
    const size_t w = (size_t)blockIdx.x * L.n_windows + blockIdx.y;
    const float* a = L.ut + w * n_ut;
    double s = 0.0;
    for (size_t k = threadIdx.x; k < n_ut; k += blockDim.x) s += (double)a[k];
    const double m = block_sum(s, red) / (double)n_ut;
    double q = 0.0;
    for (size_t k = threadIdx.x; k < n_ut; k += blockDim.x) {
        const double d = (double)a[k] - m;
        q += d * d;
    }
    const double qq = block_sum(q, red);
    if (threadIdx.x == 0) { L.ut_mv[2 * w] = m; L.ut_mv[2 * w + 1] = qq; }
    // the centred values, rounded to f32, for the pair products of feat_fcd_kernel
    float* ac = L.ut + w * n_ut;
    for (size_t k = threadIdx.x; k < n_ut; k += blockDim.x) ac[k] = (float)((double)ac[k] - m);
}

// row i = blockIdx.y of the FCD matrix of point-variable blockIdx.x (fc.rs:130-139, 144-179)
__global__ void feat_fcd_kernel(HbFeatLaunch L) {
    __shared__ double red[32];
    const int nw = L.n_windows, i = blockIdx.y, bv = blockIdx.x;
    const size_t n_ut = (size_t)L.nnodes * (L.nnodes - 1) / 2;
    const float* ai = L.ut + ((size_t)bv * nw + i) * n_ut;  // centred
    const double vi = L.ut_mv[2 * ((size_t)bv * nw + i) + 1];
    float* F = L.fcd + ((size_t)L.b0 * L.nvar + bv) * nw * nw;
    if (threadIdx.x == 0) F[(size_t)i * nw + i] = 1.0f;
    for (int j = i + 1; j < nw; j++) {
        const float* aj = L.ut + ((size_t)bv * nw + j) * n_ut;
        const double vj = L.ut_mv[2 * ((size_t)bv * nw + j) + 1];
        // FP32 products summed per thread in runs of 64, FP64 across runs and threads
        double c = 0.0;
        for (size_t k0 = threadIdx.x; k0 < n_ut; k0 += 64 * (size_t)blockDim.x) {
            float part = 0.0f;
            for (size_t k = k0; k < n_ut && k < k0 + 64 * (size_t)blockDim.x; k += blockDim.x) part = __fmaf_rn(ai[k], aj[k], part);
            c += part;
        }
        c = block_sum(c, red);
        if (threadIdx.x == 0) {
            double r = 0.0;
            if (vi > 0.0 && vj > 0.0) {
                r = c / (sqrt(vi) * sqrt(vj));
                r = r < -1.0 ? -1.0 : (r > 1.0 ? 1.0 : r);
            }
            F[(size_t)i * nw + j] = (float)r;
            F[(size_t)j * nw + i] = (float)r;
        }
    }
}

__device__ __forceinline__ uint32_t order_key(float x) {
    const uint32_t u = __float_as_uint(x);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float key_value(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// fc_stats (fc.rs:62-83) of the upper triangle of the n x n matrix blockIdx.x of `mats` into
// stats[blockIdx.x * sstride .. + 5], and, when homo is set, homotopic_fc (fc.rs:189-203) into
// homo[blockIdx.x * sstride .. + 2]
__global__ void feat_stats_kernel(const float* mats, int n, float* stats, int sstride, float* homo) {
    __shared__ int cnt_red[32];
    const float* M = mats + (size_t)blockIdx.x * n * n;
    float* S = stats + (size_t)blockIdx.x * sstride;
    const long long nut = (long long)n * (n - 1) / 2;
    const float qnan = __int_as_float(0x7fc00000);
    if (nut == 0) {
        if (threadIdx.x < 5) S[threadIdx.x] = qnan;
    } else {
        if (threadIdx.x == 0) {
            float sum = 0.0f, mn = __int_as_float(0x7f800000), mx = -__int_as_float(0x7f800000);
            for (int i = 0; i < n; i++)
                for (int j = i + 1; j < n; j++) {
                    const float x = M[(size_t)i * n + j];
                    sum += x;
                    mn = fminf(mn, x);
                    mx = fmaxf(mx, x);
                }
            const float mean = sum / (float)nut;
            float var = 0.0f;
            for (int i = 0; i < n; i++)
                for (int j = i + 1; j < n; j++) {
                    const float d = M[(size_t)i * n + j] - mean;
                    var += d * d;
                }
            var = var / (float)nut;
            S[0] = mean;
            S[1] = sqrtf(var);
            S[2] = mn;
            S[3] = mx;
        }
        __syncthreads();
        // median: sorted[nut / 2], the smallest key whose count of keys <= it exceeds nut / 2
        const long long k = nut / 2;
        uint32_t lo = 0u, hi = 0xffffffffu;
        while (lo < hi) {
            const uint32_t mid = lo + (hi - lo) / 2;
            int c = 0;
            for (long long q = threadIdx.x; q < (long long)n * n; q += blockDim.x) {
                const int i = (int)(q / n), j = (int)(q - (q / n) * n);
                if (i < j && order_key(M[q]) <= mid) c++;
            }
            const long long total = block_sum<int>(c, cnt_red);
            if (total > k) hi = mid;
            else lo = mid + 1;
        }
        if (threadIdx.x == 0) S[4] = key_value(lo);
    }
    if (homo && threadIdx.x == 0) {
        float* H = homo + (size_t)blockIdx.x * sstride;
        const int np = n / 2;
        if (np == 0) { H[0] = qnan; H[1] = qnan; }
        else {
            float sum = 0.0f;
            for (int i = 0; i < np; i++) sum += M[(size_t)i * n + (n - 1 - i)];
            const float mean = sum / (float)np;
            float var = 0.0f;
            for (int i = 0; i < np; i++) {
                const float d = M[(size_t)i * n + (n - 1 - i)] - mean;
                var += d * d;
            }
            H[0] = mean;
            H[1] = sqrtf(var / (float)np);
        }
    }
}

template <int CHUNK, int MAXT>
cudaError_t launch_moments(const HbFeatLaunch& L, int n_ranges, int stride, int len, int slices, cudaStream_t st) {
    const int W = (L.nnodes + 3) / 4 * 4;
    const size_t sm = ((size_t)2 * CHUNK + 1) * W * sizeof(float) + 16;
    cudaError_t e = cudaFuncSetAttribute(feat_moments_kernel<CHUNK, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    feat_moments_kernel<CHUNK, MAXT><<<dim3(L.nb * L.nvar, n_ranges * slices), MAXT, sm, st>>>(L, n_ranges, stride, len, slices);
    return cudaGetLastError();
}

// 256 threads (three blocks per SM) while the 4 x 4 tiles fit one pass, else one thread per node
cudaError_t moments(const HbFeatLaunch& L, int n_ranges, int stride, int len, int slices, cudaStream_t st) {
    const int n4 = (L.nnodes + 3) / 4;
    if (n4 * (n4 + 1) / 2 <= 256) return launch_moments<64, 256>(L, n_ranges, stride, len, slices, st);
    if (L.nnodes <= 512) return launch_moments<32, 512>(L, n_ranges, stride, len, slices, st);
    return launch_moments<16, 1024>(L, n_ranges, stride, len, slices, st);
}

}  // namespace

size_t hb_fc_part_len(int nnodes) { return part_len(nnodes); }

cudaError_t hb_launch_fc_features(const HbFeatLaunch& L, cudaStream_t st) {
    const int N = L.nnodes, W = (N + 3) / 4 * 4, nbv = L.nb * L.nvar;
    if (N < 1 || N > 1024) return cudaErrorInvalidValue;
    cudaError_t e;
    // static FC over all steps, its statistics and homotopic values
    if ((e = moments(L, 1, 0, L.T, L.fc_slices, st)) != cudaSuccess) return e;
    float* fc_b = L.fc + (size_t)L.b0 * L.nvar * N * N;
    feat_corr_kernel<<<dim3(nbv, 1), 256, 2 * W * sizeof(double), st>>>(L, 1, L.T, L.fc_slices, fc_b, nullptr);
    feat_stats_kernel<<<nbv, 256, 0, st>>>(fc_b, N, L.feat + (size_t)L.b0 * L.nvar * 7, 7, L.feat + (size_t)L.b0 * L.nvar * 7 + 5);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (L.n_windows < 2) return cudaSuccess;
    // FCD: window FCs, their pairwise correlations, statistics
    const int nw = L.n_windows;
    if (L.block_len > 0) {
        // moments of blocks of block_len steps, each window the sum of window / block_len of them
        const int G = L.block_len, K = L.window / G, step = L.stride / G;
        const int n_blocks = (nw - 1) * step + K;
        if ((e = moments(L, n_blocks, G, G, 1, st)) != cudaSuccess) return e;
        const size_t sm = ((size_t)3 * K + 1) * W * sizeof(double);
        if ((e = cudaFuncSetAttribute(feat_corr_blocks_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)) != cudaSuccess)
            return e;
        feat_corr_blocks_kernel<<<dim3(nbv, nw), 256, sm, st>>>(L, n_blocks, G, K, step);
    } else {
        if ((e = moments(L, nw, L.stride, L.window, L.win_slices, st)) != cudaSuccess) return e;
        feat_corr_kernel<<<dim3(nbv, nw), 256, 2 * W * sizeof(double), st>>>(L, nw, L.window, L.win_slices, nullptr, L.ut);
    }
    feat_ut_moments_kernel<<<dim3(nbv, nw), 256, 0, st>>>(L);
    feat_fcd_kernel<<<dim3(nbv, nw), 256, 0, st>>>(L);
    feat_stats_kernel<<<nbv, 256, 0, st>>>(L.fcd + (size_t)L.b0 * L.nvar * nw * nw, nw,
                                            L.fcd_stats + (size_t)L.b0 * L.nvar * 5, 5, nullptr);
    return cudaGetLastError();
}
