// hb_adjoint.cu — discrete adjoint of the batched step for a functional-connectivity loss.
//
// Scope: one Jansen–Rit subnetwork coupled to itself through one CSR projection with per-edge
// delays (ring semantics of runtime.rs:125-211), Sigmoidal or Linear coupling, deterministic Heun
// (engine.rs:710-720). The loss of sweep point b is
//     L_b = mean_{i,j} (FC_ij - FCt_ij)^2,   FC = Pearson correlation over t = 1..T of y = y1 - y2,
// and the gradients are dL_b/dG (the coupling function's gain: Sigmoidal `a`, Linear `a`) and
// dL_b/dA_i, dL_b/dB_i, dL_b/da_i for every node i (the Jansen–Rit parameters taken per node).
//
// Kernels (one CTA per sweep point unless stated):
//   adj_forward_kernel  the forward run as the engine computes it (same dfun, same op order), writing
//                       y(t) and, every CK steps, a checkpoint of the state and the delay ring
//   adj_stats_kernel    means, deviations, FC, the loss, and the coefficients of dL/dy(t)
//   adj_source_kernel   dL/dy_k(t) = coef_k * (sum_j M_kj z_j(t) - r_k z_k(t))   (grid: points x time tiles)
//   adj_backward_kernel per checkpoint segment, last to first: recompute the segment forward from its
//                       checkpoint (keeping x(s) and the coupling sum g(s)), then the reverse sweep
//                       lambda(s) = lambda(s+1) * dx(s+1)/dx(s) + delayed-coupling terms + dL/dx(s).
// The delayed coupling adjoint is pulled, not scattered: mu(s) = dL/dg(s) of every node goes into a
// ring like the forward history, and source node j adds sum over its out-edges e of
// w_e * mu_tgt(e)(s + d_e) to its lambda at time s. With every delay >= K the values pulled at
// step s were written at least K reverse steps earlier, so one barrier per K steps suffices, as in
// the forward kernels. The result is deterministic (no atomics). Parameter gradients accumulate in
// FP64 over the run.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>

#include "hb_device.h"
#include "hb_models.cuh"

namespace {

constexpr int NV = 6;  // Jansen–Rit state variables

struct AdjArgs {
    int B, N, T, R, K, CK, n_ck;
    int cfk;              // HBC_SIGMOIDAL or HBC_LINEAR
    int gain_idx;         // index of the gain in the resolved coupling row (Sigmoidal 3, Linear 0)
    float dt, dt_half;
    const float* x0;      // [B][N*6] initial states
    const int* rowptr;    // CSR by target [N+1]
    const uint32_t* edges;// (delay << 16) | src
    const float* ew;
    const int* cptr;      // CSC by source [N+1]
    const int* ctgt;      // target of each out-edge
    const int* cdel;      // its delay
    const float* cw;      // its weight
    float* Y;             // [T][B][N]   y(t) = y1 - y2 at t = 1..T (row t-1)
    float* S;             // [T][B][N]   dL/dy(t)
    float* ck_state;      // [n_ck][B][N*6]
    float* ck_ring;       // [n_ck][B][R*N]
    float* scratch;       // [B][CK][N][8]  x(s), g(s) of the segment being reversed
    float* mu_ring;       // [B][R*N]
    // statistics
    const float* target;  // [N][N] target FC
    float* mean;          // [B][N]
    float* sdev;          // [B][N]
    float* coef;          // [B][N]
    float* rk;            // [B][N]
    float* M;             // [B][N][N] (column j major: M[b][j][k])
    float* fc;            // [B][N][N]
    double* loss;         // [B]
    // gradients
    double* gG;           // [B]
    double* gA;           // [B][N]
    double* gB;           // [B][N]
    double* ga;           // [B][N]
};

__device__ __forceinline__ float coupling_post(int cfk, const float* cp, float g) {
    float gx[4] = {g, 0.f, 0.f, 0.f}, xi[2] = {0.f, 0.f}, out[4] = {0.f, 0.f, 0.f, 0.f};
    hb::post(cfk, cp, 0, gx, 1, xi, 1, 0.0f, out);
    return out[0];
}

// dc/dg and dc/dgain of the coupling output at the weighted sum g
__device__ __forceinline__ void coupling_post_grad(int cfk, const float* cp, float g, float& dc_dg, float& dc_dgain) {
    if (cfk == HBC_SIGMOIDAL) {
        const float cmin = cp[0], cmax = cp[1], mid = cp[2], a = cp[3], sigma = cp[4];
        float sh = (g + (-mid)) / sigma;
        float q = 1.0f / (expf(-(sh * a)) + 1.0f);
        float dq = q * (1.0f - q);
        dc_dg = (cmax - cmin) * dq * a / sigma;
        dc_dgain = (cmax - cmin) * dq * sh;
    } else {  // Linear: a * g + b
        dc_dg = cp[0];
        dc_dgain = g;
    }
}

// Jansen–Rit sigmoid values and their derivatives with respect to their arguments at state y
__device__ __forceinline__ void jr_sigmoids(const float* p, const float* y, float* sv, float* dsv) {
    const float J = p[7], v0 = p[4], nu_max = p[5], r = p[6], a1 = p[8], a3 = p[10];
    const float two_nu_max = 2.0f * nu_max;
    float args[3] = {y[1] - y[2], y[0] * (a1 * J), y[0] * (a3 * J)};
#pragma unroll
    for (int q = 0; q < 3; q++) {
        float arg = ((-args[q]) + v0) * r;
        const float E = expf(arg);
        float denom = E + 1.0f;
        sv[q] = (1.0f * two_nu_max) / denom;
        dsv[q] = sv[q] * r / (1.0f + 1.0f / E);  // E / (1 + E) without cancellation; 0 when E underflows
    }
}

// u^T (df/dy) at state y (dfun.rs Jansen–Rit arm), and u . df/dc0, u . df/dA, u . df/dB, u . df/da
__device__ __forceinline__ void jr_vjp(const float* p, const float* y, float c0, const float* u, float* out,
                                       float& u_c, float& u_A, float& u_B, float& u_a) {
    const float A = p[0], B = p[1], a = p[2], b = p[3], J = p[7];
    const float a1 = p[8], a2 = p[9], a3 = p[10], a4 = p[11], mu = p[12];
    float sv[3], dsv[3];
    jr_sigmoids(p, y, sv, dsv);
    const float Aa = A * a;
    out[0] = u[3] * (-(a * a)) + u[4] * (Aa * (a2 * J) * dsv[1] * (a1 * J)) + u[5] * ((B * b) * (a4 * J) * dsv[2] * (a3 * J));
    out[1] = u[3] * (Aa * dsv[0]) + u[4] * (-(a * a));
    out[2] = -u[3] * (Aa * dsv[0]) + u[5] * (-(b * b));
    out[3] = u[0] + u[3] * (-2.0f * a);
    out[4] = u[1] + u[4] * (-2.0f * a);
    out[5] = u[2] + u[5] * (-2.0f * b);
    const float Mv = (sv[1] * (a2 * J) + mu) + c0;
    u_c = u[4] * Aa;
    u_A = u[3] * (a * sv[0]) + u[4] * (a * Mv);
    u_B = u[5] * (b * (sv[2] * (a4 * J)));
    u_a = u[3] * (A * sv[0] - 2.0f * y[3] - 2.0f * a * y[0]) + u[4] * (A * Mv - 2.0f * y[4] - 2.0f * a * y[1]);
}

// coupling sum of target i at step s from the delay ring [R][N] (runtime.rs:162-204 reads)
__device__ __forceinline__ float gather_ring(const float* ring, const AdjArgs& A, int i, int s) {
    float g = 0.0f;
    const int R = A.R;
    for (int e = A.rowptr[i]; e < A.rowptr[i + 1]; e++) {
        const uint32_t m = A.edges[e];
        const int d = (int)(m >> 16), src = (int)(m & 0xffffu);
        int t;
        if (s == 0) t = 0;
        else if (d > s) continue;
        else t = s - d;
        g += A.ew[e] * ring[(t % R) * A.N + src];
    }
    return g;
}

// one deterministic Heun step of node state x with coupling c (engine.rs:710-720, no clamp for JR)
__device__ __forceinline__ void heun_step(const float* p, float* x, float c, float dt, float dt_half) {
    float cc[2] = {c, 0.0f}, k1[NV], k2[NV], tmp[NV];
    hb::dfun(HBM_JR, p, 0, x, cc, k1);
#pragma unroll
    for (int v = 0; v < NV; v++) tmp[v] = x[v] + k1[v] * dt;
    hb::dfun(HBM_JR, p, 0, tmp, cc, k2);
#pragma unroll
    for (int v = 0; v < NV; v++) x[v] = x[v] + (k1[v] + k2[v]) * dt_half;
}

__device__ __forceinline__ void load_params(const DevNet& net, int b, float* prm, float* cp) {
    const float* pr = net.sub[0].params + (size_t)b * HB_PSTRIDE;
#pragma unroll
    for (int i = 0; i < 13; i++) prm[i] = pr[i];
    const DevProj& P = net.proj[0];
    const float* c = P.cp_pp ? P.cp_pp + (size_t)b * HB_NCP : P.cp;
#pragma unroll
    for (int i = 0; i < 8; i++) cp[i] = c[i];
}

// forward steps [s_begin, s_end) of node i from the ring in shared memory; K-step barrier blocks.
// mode 0: write y(t) (and checkpoints at multiples of CK); mode 1: keep x(s), g(s) in the scratch.
__device__ void forward_steps(float* ring, const AdjArgs& A, int b, int i, bool act, float* x, const float* prm,
                              const float* cp, int s_begin, int s_end, int mode) {
    const int N = A.N, R = A.R;
    for (int s = s_begin; s < s_end; s++) {
        if ((s - s_begin) % A.K == 0) {
            __syncthreads();
            if (mode == 0 && s % A.CK == 0) {
                const int k = s / A.CK;
                float* cr = A.ck_ring + ((size_t)k * A.B + b) * (size_t)R * N;
                for (int q = threadIdx.x; q < R * N; q += blockDim.x) cr[q] = ring[q];
                if (act) {
                    float* cs = A.ck_state + ((size_t)k * A.B + b) * N * NV + (size_t)i * NV;
#pragma unroll
                    for (int v = 0; v < NV; v++) cs[v] = x[v];
                }
                __syncthreads();
            }
        }
        if (!act) continue;
        const float g = gather_ring(ring, A, i, s);
        if (mode == 1) {
            float* sc = A.scratch + (((size_t)b * A.CK + (s - s_begin)) * N + i) * 8;
#pragma unroll
            for (int v = 0; v < NV; v++) sc[v] = x[v];
            sc[6] = g;
        }
        heun_step(prm, x, coupling_post(A.cfk, cp, g), A.dt, A.dt_half);
        ring[((s + 1) % R) * N + i] = x[0];
        if (mode == 0) A.Y[((size_t)s * A.B + b) * N + i] = x[1] - x[2];
    }
}

__global__ void adj_forward_kernel(const DevNet* __restrict__ gnet, AdjArgs A) {
    extern __shared__ __align__(16) float ring[];
    const int b = blockIdx.x, i = threadIdx.x, N = A.N;
    const DevNet& net = *gnet;
    const bool act = i < N;
    float prm[13], cp[8], x[NV];
    load_params(net, b, prm, cp);
    for (int q = threadIdx.x; q < A.R * N; q += blockDim.x) ring[q] = 0.0f;
    __syncthreads();
#pragma unroll
    for (int v = 0; v < NV; v++) x[v] = act ? A.x0[(size_t)b * N * NV + i * NV + v] : 0.0f;
    if (act) ring[i] = x[0];
    forward_steps(ring, A, b, i, act, x, prm, cp, 0, A.T, 0);
}

// ---- statistics of y, FC, loss, and the coefficients of dL/dy ----
__global__ void adj_stats_kernel(AdjArgs A) {
    extern __shared__ __align__(16) float zs[];  // [32][N] chunk of z
    const int b = blockIdx.x, N = A.N, T = A.T;
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int i = tid; i < N; i += nth) {
        double s = 0.0;
        for (int t = 0; t < T; t++) s += A.Y[((size_t)t * A.B + b) * N + i];
        const double m = s / T;
        double v = 0.0;
        for (int t = 0; t < T; t++) { double d = A.Y[((size_t)t * A.B + b) * N + i] - m; v += d * d; }
        A.mean[(size_t)b * N + i] = (float)m;
        A.sdev[(size_t)b * N + i] = (float)sqrt(v / T);
    }
    __syncthreads();
    const int n_pairs = N * (N + 1) / 2;
    constexpr int PPT = 8;  // pairs per thread per pass over y
    float* fc = A.fc + (size_t)b * N * N;
    for (int base = 0; base < n_pairs; base += PPT * nth) {
        int pi[PPT], pj[PPT];
        double acc[PPT];
#pragma unroll
        for (int q = 0; q < PPT; q++) {
            int p = base + tid + q * nth;
            pi[q] = -1; pj[q] = -1; acc[q] = 0.0;
            if (p < n_pairs) {  // p -> (i, j), i <= j, row-major upper triangle
                int ii = 0, rem = p;
                while (rem >= N - ii) { rem -= N - ii; ii++; }
                pi[q] = ii; pj[q] = ii + rem;
            }
        }
        for (int t0 = 0; t0 < T; t0 += 32) {
            const int nt = (T - t0) < 32 ? (T - t0) : 32;
            __syncthreads();
            for (int q = tid; q < nt * N; q += nth) {
                const int tt = q / N, k = q - tt * N;
                const float sd = A.sdev[(size_t)b * N + k];
                zs[q] = sd > 0.0f ? (A.Y[((size_t)(t0 + tt) * A.B + b) * N + k] - A.mean[(size_t)b * N + k]) / sd : 0.0f;
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < PPT; q++) {
                if (pi[q] < 0) continue;
                float part = 0.0f;
                for (int tt = 0; tt < nt; tt++) part += zs[tt * N + pi[q]] * zs[tt * N + pj[q]];
                acc[q] += part;
            }
        }
#pragma unroll
        for (int q = 0; q < PPT; q++) {
            if (pi[q] < 0) continue;
            float v = (float)(acc[q] / T);
            if (pi[q] == pj[q]) v = 1.0f;
            fc[pi[q] * N + pj[q]] = v;
            fc[pj[q] * N + pi[q]] = v;
        }
    }
    __syncthreads();
    // loss, M (off-diagonal dL/dFC), r_k, coef_k
    double* red = reinterpret_cast<double*>(zs);
    double part = 0.0;
    const double inv_n2 = 1.0 / ((double)N * N);
    float* Mb = A.M + (size_t)b * N * N;
    for (int q = tid; q < N * N; q += nth) {
        const int k = q / N, j = q - k * N;
        const double d = (double)fc[q] - (double)A.target[q];
        part += d * d;
        Mb[(size_t)j * N + k] = (k == j) ? 0.0f : (float)(2.0 * d * inv_n2);
    }
    red[tid] = part;
    __syncthreads();
    for (int o = nth >> 1; o > 0; o >>= 1) {
        if (tid < o) red[tid] += red[tid + o];
        __syncthreads();
    }
    if (tid == 0) A.loss[b] = red[0] * inv_n2;
    for (int k = tid; k < N; k += nth) {
        double r = 0.0;
        for (int j = 0; j < N; j++) r += (double)Mb[(size_t)j * N + k] * fc[k * N + j];
        A.rk[(size_t)b * N + k] = (float)r;
        const float sd = A.sdev[(size_t)b * N + k];
        A.coef[(size_t)b * N + k] = sd > 0.0f ? 2.0f / ((float)T * sd) : 0.0f;
    }
}

// dL/dy_k(t) for a tile of 64 time steps of one point: block (threads k = 0..N-1) x (TW rows)
__global__ void adj_source_kernel(AdjArgs A) {
    extern __shared__ __align__(16) float sm[];
    const int b = blockIdx.x, N = A.N;
    const int t0 = blockIdx.y * 64;
    const int nt = (A.T - t0) < 64 ? (A.T - t0) : 64;
    float* Ms = sm;               // [N][N], M[j][k]
    float* zs = sm + N * N;       // [64][N]
    const float* Mb = A.M + (size_t)b * N * N;
    for (int q = threadIdx.x; q < N * N; q += blockDim.x) Ms[q] = Mb[q];
    for (int q = threadIdx.x; q < nt * N; q += blockDim.x) {
        const int tt = q / N, k = q - tt * N;
        const float sd = A.sdev[(size_t)b * N + k];
        zs[q] = sd > 0.0f ? (A.Y[((size_t)(t0 + tt) * A.B + b) * N + k] - A.mean[(size_t)b * N + k]) / sd : 0.0f;
    }
    __syncthreads();
    const int kpad = (N + 31) / 32 * 32;
    const int k = threadIdx.x % kpad, w = threadIdx.x / kpad, TW = blockDim.x / kpad;
    if (k >= N) return;
    const float ck = A.coef[(size_t)b * N + k], rk = A.rk[(size_t)b * N + k];
    for (int tt = w; tt < nt; tt += TW) {
        float acc = 0.0f;
        for (int j = 0; j < N; j++) acc += Ms[j * N + k] * zs[tt * N + j];
        A.S[((size_t)(t0 + tt) * A.B + b) * N + k] = ck * (acc - rk * zs[tt * N + k]);
    }
}

__global__ void adj_backward_kernel(const DevNet* __restrict__ gnet, AdjArgs A) {
    extern __shared__ __align__(16) float ring[];  // forward ring during recompute, mu ring during reversal
    const int b = blockIdx.x, i = threadIdx.x, N = A.N, R = A.R, T = A.T;
    const DevNet& net = *gnet;
    const bool act = i < N;
    float prm[13], cp[8];
    load_params(net, b, prm, cp);
    const float h = A.dt, hh = A.dt_half;
    double lam[NV];  // adjoint state, carried in FP64 across the reverse sweep
#pragma unroll
    for (int v = 0; v < NV; v++) lam[v] = 0.0;
    if (act) {
        const float sT = A.S[((size_t)(T - 1) * A.B + b) * N + i];
        lam[1] = sT;
        lam[2] = -(double)sT;
    }
    double gA = 0.0, gB = 0.0, ga = 0.0, gG = 0.0;
    float* mu_g = A.mu_ring + (size_t)b * R * N;
    for (int q = threadIdx.x; q < R * N; q += blockDim.x) mu_g[q] = 0.0f;
    for (int seg = A.n_ck - 1; seg >= 0; seg--) {
        const int s_begin = seg * A.CK, s_end = (s_begin + A.CK) < T ? (s_begin + A.CK) : T;
        // (a) recompute the segment forward from its checkpoint
        __syncthreads();
        {
            const float* cr = A.ck_ring + ((size_t)seg * A.B + b) * (size_t)R * N;
            for (int q = threadIdx.x; q < R * N; q += blockDim.x) ring[q] = cr[q];
        }
        float x[NV];
#pragma unroll
        for (int v = 0; v < NV; v++) x[v] = act ? A.ck_state[((size_t)seg * A.B + b) * N * NV + (size_t)i * NV + v] : 0.0f;
        forward_steps(ring, A, b, i, act, x, prm, cp, s_begin, s_end, 1);
        // (b) the mu ring of the later segments into shared memory
        __syncthreads();
        for (int q = threadIdx.x; q < R * N; q += blockDim.x) ring[q] = mu_g[q];
        // (c) reverse sweep
        for (int s = s_end - 1; s >= s_begin; s--) {
            if ((s_end - 1 - s) % A.K == 0) __syncthreads();
            if (!act) continue;
            const float* sc = A.scratch + (((size_t)b * A.CK + (s - s_begin)) * N + i) * 8;
            float xs[NV];
#pragma unroll
            for (int v = 0; v < NV; v++) xs[v] = sc[v];
            const float g = sc[6];
            const float c = coupling_post(A.cfk, cp, g);
            float cc[2] = {c, 0.0f}, k1[NV], p[NV];
            hb::dfun(HBM_JR, prm, 0, xs, cc, k1);
#pragma unroll
            for (int v = 0; v < NV; v++) p[v] = xs[v] + k1[v] * h;
            // adjoint of k2 = f(p): u2 = h/2 lam
            float u2[NV], vp[NV], u1[NV], vx[NV];
#pragma unroll
            for (int v = 0; v < NV; v++) u2[v] = (float)(hh * lam[v]);
            float uc2, uA2, uB2, ua2, uc1, uA1, uB1, ua1;
            jr_vjp(prm, p, c, u2, vp, uc2, uA2, uB2, ua2);
#pragma unroll
            for (int v = 0; v < NV; v++) u1[v] = (float)(hh * lam[v] + (double)(h * vp[v]));
            jr_vjp(prm, xs, c, u1, vx, uc1, uA1, uB1, ua1);
#pragma unroll
            for (int v = 0; v < NV; v++) lam[v] = lam[v] + ((double)vp[v] + (double)vx[v]);
            const float mu_c = uc1 + uc2;
            float dc_dg, dc_dgain;
            coupling_post_grad(A.cfk, cp, g, dc_dg, dc_dgain);
            gA += (double)uA1 + (double)uA2;
            gB += (double)uB1 + (double)uB2;
            ga += (double)ua1 + (double)ua2;
            gG += (double)mu_c * (double)dc_dgain;
            ring[(s % R) * N + i] = mu_c * dc_dg;
            // lambda(s) for s >= 1: delayed-coupling terms pulled from later steps, then dL/dx(s)
            if (s >= 1) {
                float pull = 0.0f;
                for (int e = A.cptr[i]; e < A.cptr[i + 1]; e++) {
                    const int tt = s + A.cdel[e];
                    if (tt <= T - 1) pull += A.cw[e] * ring[(tt % R) * N + A.ctgt[e]];
                }
                lam[0] += pull;
                const float src = A.S[((size_t)(s - 1) * A.B + b) * N + i];
                lam[1] += src;
                lam[2] -= src;
            }
        }
        __syncthreads();
        for (int q = threadIdx.x; q < R * N; q += blockDim.x) mu_g[q] = ring[q];
    }
    if (act) {
        A.gA[(size_t)b * N + i] = gA;
        A.gB[(size_t)b * N + i] = gB;
        A.ga[(size_t)b * N + i] = ga;
    }
    // gain gradient: sum over nodes
    __syncthreads();
    double* red = reinterpret_cast<double*>(ring);
    red[threadIdx.x] = act ? gG : 0.0;
    __syncthreads();
    for (int o = blockDim.x >> 1; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) A.gG[b] = red[0];
}

}  // namespace

// ---- launch interface used by the engine (hb_engine.cu) ----
struct HbAdjointLaunch {
    int B, N, T, R, K, CK, n_ck, cfk, gain_idx;
    float dt, dt_half;
    const float* x0;
    const int* rowptr; const uint32_t* edges; const float* ew;
    const int* cptr; const int* ctgt; const int* cdel; const float* cw;
    float *Y, *S, *ck_state, *ck_ring, *scratch, *mu_ring;
    const float* target;
    float *mean, *sdev, *coef, *rk, *M, *fc;
    double *loss, *gG, *gA, *gB, *ga;
};

cudaError_t hb_launch_adjoint(const DevNet* d_net, const HbAdjointLaunch& L, int phase, cudaStream_t st) {
    AdjArgs A;
    A.B = L.B; A.N = L.N; A.T = L.T; A.R = L.R; A.K = L.K; A.CK = L.CK; A.n_ck = L.n_ck;
    A.cfk = L.cfk; A.gain_idx = L.gain_idx; A.dt = L.dt; A.dt_half = L.dt_half;
    A.x0 = L.x0; A.rowptr = L.rowptr; A.edges = L.edges; A.ew = L.ew;
    A.cptr = L.cptr; A.ctgt = L.ctgt; A.cdel = L.cdel; A.cw = L.cw;
    A.Y = L.Y; A.S = L.S; A.ck_state = L.ck_state; A.ck_ring = L.ck_ring; A.scratch = L.scratch; A.mu_ring = L.mu_ring;
    A.target = L.target; A.mean = L.mean; A.sdev = L.sdev; A.coef = L.coef; A.rk = L.rk; A.M = L.M; A.fc = L.fc;
    A.loss = L.loss; A.gG = L.gG; A.gA = L.gA; A.gB = L.gB; A.ga = L.ga;
    const int threads = (L.N + 31) / 32 * 32;
    const size_t ring_bytes = (size_t)L.R * L.N * sizeof(float);
    if (phase == 0) {
        if (cudaFuncSetAttribute(adj_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ring_bytes) != cudaSuccess)
            return cudaGetLastError();
        adj_forward_kernel<<<L.B, threads, ring_bytes, st>>>(d_net, A);
    } else if (phase == 1) {
        const size_t sm = std::max((size_t)32 * L.N * sizeof(float), (size_t)512 * sizeof(double));
        adj_stats_kernel<<<L.B, 512, sm, st>>>(A);
        const size_t sm2 = ((size_t)L.N * L.N + 64 * (size_t)L.N) * sizeof(float);
        if (cudaFuncSetAttribute(adj_source_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2) != cudaSuccess)
            return cudaGetLastError();
        const int kpad = (L.N + 31) / 32 * 32;
        const int tw = std::max(1, 512 / kpad);
        dim3 grid(L.B, (L.T + 63) / 64);
        adj_source_kernel<<<grid, kpad * tw, sm2, st>>>(A);
    } else {
        const size_t sm = std::max(ring_bytes, (size_t)threads * sizeof(double));
        if (cudaFuncSetAttribute(adj_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
            return cudaGetLastError();
        adj_backward_kernel<<<L.B, threads, sm, st>>>(d_net, A);
    }
    return cudaGetLastError();
}
