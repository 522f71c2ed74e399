// hb_adjoint.cu — discrete adjoint of the batched step for a functional-connectivity loss.
//
// Scope: one Jansen–Rit subnetwork coupled to itself through one CSR projection with per-edge
// delays (ring semantics of runtime.rs:125-211), Sigmoidal or Linear coupling, deterministic Heun
// (engine.rs:710-720) or RK4 (the engine's stage order, coupling held over the step). The loss of
// sweep point b is
//     L_b = mean_{i,j} (FC_ij - FCt_ij)^2,   FC = Pearson correlation over t = 1..T of y = y1 - y2,
// and the gradients are dL_b/dG (the coupling function's gain: Sigmoidal `a`, Linear `a`) and
// dL_b/dA_i, dL_b/dB_i, dL_b/da_i for every node i (the Jansen–Rit parameters taken per node).
//
// Kernels (one CTA per sweep point unless stated):
//   adj_forward_kernel  the forward run as the engine computes it (same dfun, same op order), writing
//                       y(t) and, every CK steps, a checkpoint of the state and the delay ring
//   adj_moments_kernel  moments of y over one time slice (grid: points x up to 16 slices)
//   adj_fc_kernel       adds the slices: means, deviations, FC, the loss, the coefficients of dL/dy(t)
//   adj_source_kernel   dL/dy_k(t) = coef_k * (sum_j M_kj z_j(t) - r_k z_k(t))   (grid: points x 128-step tiles)
//   adj_backward_kernel per checkpoint segment, last to first: recompute the segment forward from its
//                       checkpoint (keeping x(s) and the coupling sum g(s)), then the reverse sweep
//                       lambda(s) = lambda(s+1) * dx(s+1)/dx(s) + delayed-coupling terms + dL/dx(s).
// The delayed coupling adjoint is pulled, not scattered: mu(s) = dL/dg(s) of every node goes into a
// ring like the forward history, and source node j adds sum over its out-edges e of
// w_e * mu_tgt(e)(s + d_e) to its lambda at time s. With every delay >= K the values pulled at
// step s were written at least K reverse steps earlier, so one barrier per K steps suffices, as in
// the forward kernels. The result is deterministic (no atomics). Parameter gradients are summed in
// FP32 within a checkpoint segment and in FP64 across segments (FP64 arithmetic is slow on this
// part, so it is kept out of the per-step work).
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>

#include "hb_device.h"
#include "hb_models.cuh"
#include "hb_moments.cuh"

namespace {

constexpr int NV = 6;  // Jansen–Rit state variables

struct AdjArgs {
    int B, N, T, R, K, CK, n_ck;
    int store_all;        // 1: the forward keeps x(s), g(s) of every step (CK == T), no re-computation
    int cfk;              // HBC_SIGMOIDAL or HBC_LINEAR
    int gain_idx;         // index of the gain in the resolved coupling row (Sigmoidal 3, Linear 0)
    float dt, dt_half;
    int rk4;              // 1: deterministic RK4, 0: deterministic Heun
    float dt_h2, dt_sixth;// dt / 2 and dt / 6 as the engine's RK4 uses them
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
    float* lam_g;         // [B][N*6] lambda carried between the segments' reverse launches
    int seg_begin, seg_end, seg_last;  // the segment one reverse or re-computation launch covers (seg_last: the
                                       // run's last segment, where the reverse starts)
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

// Jansen–Rit sigmoid values and their derivatives with respect to their arguments at state y, with
// the hardware exponential and division (a few ulp): for the reverse coefficients, where the
// linearisation point, not bit-exactness with the forward, is what matters
__device__ __forceinline__ void jr_sigmoids_fast(const float* p, const float* y, float* sv, float* dsv) {
    const float J = p[7], v0 = p[4], nu_max = p[5], r = p[6], a1 = p[8], a3 = p[10];
    const float two_nu_max = 2.0f * nu_max;
    float args[3] = {y[1] - y[2], y[0] * (a1 * J), y[0] * (a3 * J)};
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const float arg = ((-args[q]) + v0) * r;
        const float E = __expf(arg);
        const float inv = __fdividef(1.0f, E + 1.0f);
        sv[q] = two_nu_max * inv;
        dsv[q] = sv[q] * r * (1.0f - inv);  // E / (1 + E) = 1 - 1 / (1 + E)
    }
}

// coupling output c(g) and its slopes dc/dg, dc/dgain from one exponential
__device__ __forceinline__ float coupling_post_and_grad(int cfk, const float* cp, float g, float& dc_dg, float& dc_dgain) {
    if (cfk == HBC_SIGMOIDAL) {
        const float cmin = cp[0], cmax = cp[1], mid = cp[2], a = cp[3], sigma = cp[4];
        const float sh = (g + (-mid)) / sigma;
        const float q = 1.0f / (expf(-(sh * a)) + 1.0f);
        const float dq = (cmax - cmin) * (q * (1.0f - q));
        dc_dg = dq * a / sigma;
        dc_dgain = dq * sh;
        return q * (cmax - cmin) + cmin;
    }
    dc_dg = cp[0];
    dc_dgain = g;
    return g * cp[0] + cp[1];
}

// The lambda-independent part of one reverse step at state x(s) with coupling sum g(s): the nonzero
// Jacobian factors of the Jansen-Rit arm at x and at the Heun predictor p = x + h f(x), the parameter
// derivative factors there, and the coupling slopes. With them the step's adjoint is a short chain of
// multiply-adds in lambda (jr_lin_step), so the transcendental work of step s - 1 can be done while
// step s is still in flight.
struct JrCoef {
    float q1x, q2x, p0x, q1p, q2p, p0p;     // J factors: d f4/d y0, d f5/d y0, d f3/d y1 at x and at p
    float aAx, aAp, aMx, aMp;               // d f3/dA = a sv0, d f4/dA = a M at x and p
    float bBx, bBp;                         // d f5/dB at x and p
    float a3x, a4x, a3p, a4p;               // d f3/da, d f4/da at x and p
    float dcdg, dcdgain;                    // coupling output slopes
};

__device__ __forceinline__ JrCoef jr_coef(const float* prm, const float* cp, int cfk, const float* xs, float g, float h) {
    const float A = prm[0], B = prm[1], a = prm[2], b = prm[3], J = prm[7];
    const float a1 = prm[8], a2 = prm[9], a3 = prm[10], a4 = prm[11], mu = prm[12];
    JrCoef k;
    const float c = coupling_post_and_grad(cfk, cp, g, k.dcdg, k.dcdgain);
    float sv[3], dsv[3];
    jr_sigmoids_fast(prm, xs, sv, dsv);
    // k1 = f(x, c) from the same sigmoid values, in the operation order of dfun.rs's Jansen-Rit arm
    float k1[NV], p[NV];
    {
        k1[0] = xs[3];
        k1[1] = xs[4];
        k1[2] = xs[5];
        float d3 = sv[0] * (A * a);
        d3 = d3 - xs[3] * (2.0f * a);
        d3 = d3 - xs[0] * (a * a);
        k1[3] = d3;
        float mt = sv[1] * (a2 * J);
        mt = mt + mu;
        mt = mt + c;
        float d4 = mt * (A * a);
        d4 = d4 - xs[4] * (2.0f * a);
        d4 = d4 - xs[1] * (a * a);
        k1[4] = d4;
        float d5 = sv[2] * (a4 * J);
        d5 = d5 * (B * b);
        d5 = d5 - xs[5] * (2.0f * b);
        d5 = d5 - xs[2] * (b * b);
        k1[5] = d5;
    }
#pragma unroll
    for (int v = 0; v < NV; v++) p[v] = xs[v] + k1[v] * h;
    const float Aa = A * a, Bb = B * b;
    k.q1x = Aa * (a2 * J) * dsv[1] * (a1 * J);
    k.q2x = Bb * (a4 * J) * dsv[2] * (a3 * J);
    k.p0x = Aa * dsv[0];
    float Mx = (sv[1] * (a2 * J) + mu) + c;
    k.aAx = a * sv[0];
    k.aMx = a * Mx;
    k.bBx = b * (sv[2] * (a4 * J));
    k.a3x = A * sv[0] - 2.0f * xs[3] - 2.0f * a * xs[0];
    k.a4x = A * Mx - 2.0f * xs[4] - 2.0f * a * xs[1];
    jr_sigmoids_fast(prm, p, sv, dsv);
    k.q1p = Aa * (a2 * J) * dsv[1] * (a1 * J);
    k.q2p = Bb * (a4 * J) * dsv[2] * (a3 * J);
    k.p0p = Aa * dsv[0];
    float Mp = (sv[1] * (a2 * J) + mu) + c;
    k.aAp = a * sv[0];
    k.aMp = a * Mp;
    k.bBp = b * (sv[2] * (a4 * J));
    k.a3p = A * sv[0] - 2.0f * p[3] - 2.0f * a * p[0];
    k.a4p = A * Mp - 2.0f * p[4] - 2.0f * a * p[1];
    return k;
}

// adjoint of one Heun step (engine.rs:710-720) given the coefficients: lambda(s+1) -> lambda(s)
// (without the delayed-coupling and loss terms), mu_c = dL/dc(s), and the parameter terms
__device__ __forceinline__ void jr_lin_step(const JrCoef& k, const float* prm, float h, float hh, float* lam,
                                            float& mu_c, float& tA, float& tB, float& ta) {
    const float A = prm[0], a = prm[2], b = prm[3];
    const float na2 = -(a * a), nb2 = -(b * b), m2a = -2.0f * a, m2b = -2.0f * b;
    float u2[NV], vp[NV], u1[NV], vx[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) u2[v] = hh * lam[v];
    vp[0] = u2[3] * na2 + u2[4] * k.q1p + u2[5] * k.q2p;
    vp[1] = u2[3] * k.p0p + u2[4] * na2;
    vp[2] = -u2[3] * k.p0p + u2[5] * nb2;
    vp[3] = u2[0] + u2[3] * m2a;
    vp[4] = u2[1] + u2[4] * m2a;
    vp[5] = u2[2] + u2[5] * m2b;
#pragma unroll
    for (int v = 0; v < NV; v++) u1[v] = hh * lam[v] + h * vp[v];
    vx[0] = u1[3] * na2 + u1[4] * k.q1x + u1[5] * k.q2x;
    vx[1] = u1[3] * k.p0x + u1[4] * na2;
    vx[2] = -u1[3] * k.p0x + u1[5] * nb2;
    vx[3] = u1[0] + u1[3] * m2a;
    vx[4] = u1[1] + u1[4] * m2a;
    vx[5] = u1[2] + u1[5] * m2b;
#pragma unroll
    for (int v = 0; v < NV; v++) lam[v] = lam[v] + (vp[v] + vx[v]);
    mu_c = (u1[4] + u2[4]) * (A * a);
    tA = (u1[3] * k.aAx + u1[4] * k.aMx) + (u2[3] * k.aAp + u2[4] * k.aMp);
    tB = u1[5] * k.bBx + u2[5] * k.bBp;
    ta = (u1[3] * k.a3x + u1[4] * k.a4x) + (u2[3] * k.a3p + u2[4] * k.a4p);
}

// The lambda-independent part of one reverse RK4 step: the Jacobian and parameter factors of the
// Jansen-Rit arm at the four stage states x1 = x, x2 = x + h/2 k1, x3 = x + h/2 k2, x4 = x + h k3
// (k_i = f(x_i, c), with the hardware exponential like jr_coef), and the coupling slopes.
struct JrCoef4 {
    float q1[4], q2[4], p0[4];          // J factors: d f4/d y0, d f5/d y0, d f3/d y1
    float aA[4], aM[4], bB[4];          // d f3/dA = a sv0, d f4/dA = a M, d f5/dB
    float a3[4], a4[4];                 // d f3/da, d f4/da
    float dcdg, dcdgain;
};

// factors of one stage state y, and f(y, c) into k
__device__ __forceinline__ void jr_stage(const float* prm, const float* y, float c, JrCoef4& k, int i, float* f) {
    const float A = prm[0], B = prm[1], a = prm[2], b = prm[3], J = prm[7];
    const float a1 = prm[8], a2 = prm[9], a3 = prm[10], a4 = prm[11], mu = prm[12];
    float sv[3], dsv[3];
    jr_sigmoids_fast(prm, y, sv, dsv);
    const float Aa = A * a, Bb = B * b;
    k.q1[i] = Aa * (a2 * J) * dsv[1] * (a1 * J);
    k.q2[i] = Bb * (a4 * J) * dsv[2] * (a3 * J);
    k.p0[i] = Aa * dsv[0];
    const float M = (sv[1] * (a2 * J) + mu) + c;
    k.aA[i] = a * sv[0];
    k.aM[i] = a * M;
    k.bB[i] = b * (sv[2] * (a4 * J));
    k.a3[i] = A * sv[0] - 2.0f * y[3] - 2.0f * a * y[0];
    k.a4[i] = A * M - 2.0f * y[4] - 2.0f * a * y[1];
    if (f) {
        f[0] = y[3];
        f[1] = y[4];
        f[2] = y[5];
        f[3] = (sv[0] * Aa - y[3] * (2.0f * a)) - y[0] * (a * a);
        f[4] = (M * Aa - y[4] * (2.0f * a)) - y[1] * (a * a);
        f[5] = ((sv[2] * (a4 * J)) * Bb - y[5] * (2.0f * b)) - y[2] * (b * b);
    }
}

__device__ __forceinline__ JrCoef4 jr_coef_rk4(const float* prm, const float* cp, int cfk, const float* xs, float g,
                                               float h, float h2) {
    JrCoef4 k;
    const float c = coupling_post_and_grad(cfk, cp, g, k.dcdg, k.dcdgain);
    float f[NV], y[NV];
    jr_stage(prm, xs, c, k, 0, f);
#pragma unroll
    for (int v = 0; v < NV; v++) y[v] = xs[v] + f[v] * h2;
    jr_stage(prm, y, c, k, 1, f);
#pragma unroll
    for (int v = 0; v < NV; v++) y[v] = xs[v] + f[v] * h2;
    jr_stage(prm, y, c, k, 2, f);
#pragma unroll
    for (int v = 0; v < NV; v++) y[v] = xs[v] + f[v] * h;
    jr_stage(prm, y, c, k, 3, nullptr);
    return k;
}

// u^T J at stage i
__device__ __forceinline__ void jr_vjp4(const JrCoef4& k, int i, const float* u, float na2, float nb2, float m2a,
                                        float m2b, float* v) {
    v[0] = u[3] * na2 + u[4] * k.q1[i] + u[5] * k.q2[i];
    v[1] = u[3] * k.p0[i] + u[4] * na2;
    v[2] = -u[3] * k.p0[i] + u[5] * nb2;
    v[3] = u[0] + u[3] * m2a;
    v[4] = u[1] + u[4] * m2a;
    v[5] = u[2] + u[5] * m2b;
}

// adjoint of one RK4 step given the coefficients: lambda(s+1) -> lambda(s) (without the
// delayed-coupling and loss terms), mu_c = dL/dc(s), and the parameter terms. With a_i the adjoint
// of k_i and g_i = a_i^T J(x_i): a4 = h/6 lam, a3 = h/3 lam + h g4, a2 = h/3 lam + h/2 g3,
// a1 = h/6 lam + h/2 g2, lambda(s) = lam + g1 + g2 + g3 + g4.
__device__ __forceinline__ void jr_lin_step_rk4(const JrCoef4& k, const float* prm, float h, float h2, float h6,
                                                float* lam, float& mu_c, float& tA, float& tB, float& ta) {
    const float A = prm[0], a = prm[2], b = prm[3];
    const float na2 = -(a * a), nb2 = -(b * b), m2a = -2.0f * a, m2b = -2.0f * b;
    const float h3 = 2.0f * h6;
    float ai[NV], gi[NV], gsum[NV];
    float c4 = 0.0f;
    tA = 0.0f;
    tB = 0.0f;
    ta = 0.0f;
#pragma unroll
    for (int v = 0; v < NV; v++) ai[v] = h6 * lam[v];                 // a4
#pragma unroll
    for (int st = 3; st >= 0; st--) {
        jr_vjp4(k, st, ai, na2, nb2, m2a, m2b, gi);
        c4 += ai[4];
        tA += ai[3] * k.aA[st] + ai[4] * k.aM[st];
        tB += ai[5] * k.bB[st];
        ta += ai[3] * k.a3[st] + ai[4] * k.a4[st];
#pragma unroll
        for (int v = 0; v < NV; v++) gsum[v] = (st == 3) ? gi[v] : gsum[v] + gi[v];
        if (st == 3) {
#pragma unroll
            for (int v = 0; v < NV; v++) ai[v] = h3 * lam[v] + h * gi[v];   // a3
        } else if (st == 2) {
#pragma unroll
            for (int v = 0; v < NV; v++) ai[v] = h3 * lam[v] + h2 * gi[v];  // a2
        } else if (st == 1) {
#pragma unroll
            for (int v = 0; v < NV; v++) ai[v] = h6 * lam[v] + h2 * gi[v];  // a1
        }
    }
#pragma unroll
    for (int v = 0; v < NV; v++) lam[v] = lam[v] + gsum[v];
    mu_c = c4 * (A * a);
}

// coupling sum of target i at step 0: every edge reads the current state (runtime.rs:166-170)
__device__ __forceinline__ float gather_step0(const float* ring, const AdjArgs& A, int i, int lane, int L) {
    float g = 0.0f;
    for (int e = A.rowptr[i] + lane; e < A.rowptr[i + 1]; e += L) {
        const uint32_t m = A.edges[e];
        g += A.ew[e] * ring[(int)(m & 0xffffu)];
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

// one deterministic RK4 step (the engine's stage order: x + k h/2, x + k h/2, x + k h, then
// x + (k1 + 2 k2 + 2 k3 + k4) h/6 summed left to right; no clamp for JR)
__device__ __forceinline__ void rk4_step(const float* p, float* x, float c, float dt, float h2, float h6) {
    float cc[2] = {c, 0.0f}, k1[NV], k2[NV], k3[NV], k4[NV], tmp[NV];
    hb::dfun(HBM_JR, p, 0, x, cc, k1);
#pragma unroll
    for (int v = 0; v < NV; v++) tmp[v] = x[v] + k1[v] * h2;
    hb::dfun(HBM_JR, p, 0, tmp, cc, k2);
#pragma unroll
    for (int v = 0; v < NV; v++) tmp[v] = x[v] + k2[v] * h2;
    hb::dfun(HBM_JR, p, 0, tmp, cc, k3);
#pragma unroll
    for (int v = 0; v < NV; v++) tmp[v] = x[v] + k3[v] * dt;
    hb::dfun(HBM_JR, p, 0, tmp, cc, k4);
#pragma unroll
    for (int v = 0; v < NV; v++) {
        float sacc = k1[v] + k2[v] * 2.0f;
        sacc = sacc + k3[v] * 2.0f;
        sacc = sacc + k4[v];
        x[v] = x[v] + sacc * h6;
    }
}

template <bool RK4>
__device__ __forceinline__ void adj_step(const AdjArgs& A, const float* prm, float* x, float c) {
    if constexpr (RK4) rk4_step(prm, x, c, A.dt, A.dt_h2, A.dt_sixth);
    else heun_step(prm, x, c, A.dt, A.dt_half);
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

__device__ __forceinline__ float lane_sum(float v, int L) {
    for (int o = L >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// shared-memory tables: CSR rows of the targets (ring offsets src - d*N) and, for the reverse
// sweep, the out-edges of the sources (ring offsets d*N + tgt)
struct AdjTables {
    const int* rowptr;
    const int* eoff;
    const float* ew;
    const int* cptr;
    const int* coff;
    const float* cw;
};

__device__ AdjTables stage_tables(const AdjArgs& A, unsigned char* smem, size_t off, bool reverse) {
    const int N = A.N, nnz = A.rowptr[N];
    int* rp = reinterpret_cast<int*>(smem + off);
    int* eo = rp + (N + 1);
    float* w = reinterpret_cast<float*>(eo + nnz);
    for (int q = threadIdx.x; q <= N; q += blockDim.x) rp[q] = A.rowptr[q];
    for (int q = threadIdx.x; q < nnz; q += blockDim.x) {
        const uint32_t m = A.edges[q];
        eo[q] = (int)(m & 0xffffu) - (int)(m >> 16) * N;
        w[q] = A.ew[q];
    }
    AdjTables t{rp, eo, w, nullptr, nullptr, nullptr};
    if (reverse) {
        int* cp = reinterpret_cast<int*>(w + nnz);
        int* co = cp + (N + 1);
        float* cw = reinterpret_cast<float*>(co + nnz);
        for (int q = threadIdx.x; q <= N; q += blockDim.x) cp[q] = A.cptr[q];
        for (int q = threadIdx.x; q < nnz; q += blockDim.x) { co[q] = A.cdel[q] * N + A.ctgt[q]; cw[q] = A.cw[q]; }
        t.cptr = cp; t.coff = co; t.cw = cw;
    }
    return t;
}

// forward steps [s_begin, s_end) in blocks of K steps, from the ring in shared memory. The ring starts
// zeroed, so a time before 0 reads 0 (runtime.rs:171-176), and every step after 0 reads time s - d at
// ring offset (s mod R) * N + src - d * N, wrapped once. Every delay is >= K, so the K coupling sums
// of a block read only times published before it:
//   phase A (all threads, L lanes per node): the block's coupling sums into gbuf[K][N];
//   phase B (thread t = node t): the K serial Heun steps, publishing x0 into the ring.
// mode 0: write y(t) (and checkpoints at multiples of CK, or every step's x, g when store_all);
// mode 1: keep x(s), g(s) in the scratch. x holds the state of node threadIdx.x.
template <bool RK4>
__device__ void forward_steps(float* ring, float* gbuf, const AdjArgs& A, const AdjTables& tb, int b, int L, float* x,
                              const float* prm, const float* cp, int s_begin, int s_end, int mode) {
    const int N = A.N, R = A.R, RN = A.R * A.N, K = A.K;
    const int t = threadIdx.x;
    const int gi = t / L, gl = t - (t / L) * L;
    const bool gact = gi < N, uact = t < N;
    const int e0 = gact ? tb.rowptr[gi] : 0, e1 = gact ? tb.rowptr[gi + 1] : 0;
    for (int s0 = s_begin; s0 < s_end; s0 += K) {
        const int nb = (s_end - s0) < K ? (s_end - s0) : K;
        __syncthreads();
        if (mode == 0 && !A.store_all && s0 % A.CK == 0) {
            const int k = s0 / A.CK;
            float* cr = A.ck_ring + ((size_t)k * A.B + b) * (size_t)RN;
            for (int q = t; q < RN; q += blockDim.x) cr[q] = ring[q];
            if (uact) {
                float* cs = A.ck_state + ((size_t)k * A.B + b) * N * NV + (size_t)t * NV;
#pragma unroll
                for (int v = 0; v < NV; v++) cs[v] = x[v];
            }
        }
        // phase A
        int slot = s0 % R;
        for (int j = 0; j < nb; j++) {
            float part = 0.0f;
            if (gact) {
                if (s0 + j == 0) part = gather_step0(ring, A, gi, gl, L);
                else {
                    const int base = slot * N;
                    for (int e = e0 + gl; e < e1; e += L) {
                        int a = base + tb.eoff[e];
                        a += (a < 0) ? RN : 0;
                        part += tb.ew[e] * ring[a];
                    }
                }
            }
            part = lane_sum(part, L);
            if (gact && gl == 0) gbuf[j * N + gi] = part;
            slot = (slot + 1 == R) ? 0 : slot + 1;
        }
        __syncthreads();
        // phase B
        if (uact) {
            slot = s0 % R;
            for (int j = 0; j < nb; j++) {
                const int s = s0 + j;
                const float g = gbuf[j * N + t];
                if (mode == 1 || A.store_all) {
                    float* sc = A.scratch + (((size_t)b * A.CK + (s - s_begin)) * N + t) * 8;
#pragma unroll
                    for (int v = 0; v < NV; v++) sc[v] = x[v];
                    sc[6] = g;
                }
                adj_step<RK4>(A, prm, x, coupling_post(A.cfk, cp, g));
                const int next = (slot + 1 == R) ? 0 : slot + 1;
                ring[next * N + t] = x[0];
                if (mode == 0) A.Y[((size_t)s * A.B + b) * N + t] = x[1] - x[2];
                slot = next;
            }
        }
    }
}

__device__ __forceinline__ size_t tables_size(int N, int nnz) { return (size_t)(N + 1) * 4 + (size_t)nnz * 8; }

constexpr int ADJ_BAR_FULL0 = 1, ADJ_BAR_EMPTY0 = 3;  // named barriers 1-2 and 3-4 (0 is __syncthreads)

__device__ __forceinline__ void bar_sync(int id, int count) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory"); }
__device__ __forceinline__ void bar_arrive(int id, int count) { asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory"); }

// The forward with every step's state kept (store_all) as a producer / consumer pipeline, when every
// delay is at least 2K - 1 steps: the first n_cons threads are consumers (thread t integrates node t),
// the others producers (L lanes per node) that gather block k + 1's coupling sums into one of two
// buffers while the consumers integrate block k from the other; named barriers hand the buffers
// over. The values read for block k + 1 are at least K steps old when block k starts, so the
// consumers of block k never write them. Per step the same operations in the same order as
// forward_steps (mode 0).
constexpr int ADJ_BAR_CONS = 5;  // named barrier of the consumer threads alone

// The forward steps [s_begin, s_end) as a producer / consumer pipeline, when every delay is at least
// 2K - 1 steps: the first n_cons threads are consumers (thread t integrates node t), the others
// producers (L lanes per node) that gather block k + 1's coupling sums into one of two buffers while
// the consumers integrate block k from the other; named barriers hand the buffers over. The values
// read for block k + 1 are at least K steps old when block k starts, so the consumers of block k never
// write them. Per step the same operations in the same order as forward_steps. mode 0: the run's
// forward (y(t); every step's x, g when store_all, else a checkpoint of the state and the ring at each
// multiple of CK, taken by the consumers before they write the block); mode 1: re-computation of one
// segment from its checkpoint, keeping x(s), g(s) in the scratch (rows relative to s_begin).
template <bool RK4>
__device__ void forward_pipelined(float* ring, float* gbuf2, const AdjArgs& A, const AdjTables& tb, int b, int L,
                                  float* x, const float* prm, const float* cp, int n_cons, int s_begin, int s_end,
                                  int mode) {
    const int N = A.N, R = A.R, RN = A.R * A.N, K = A.K;
    const int t = threadIdx.x, nthreads = blockDim.x;
    const int n_blocks = (s_end - s_begin + K - 1) / K;
    if (t >= n_cons) {
        const int p = t - n_cons;
        const int gi = p / L, gl = p - (p / L) * L;
        const bool gact = gi < N;
        const int e0 = gact ? tb.rowptr[gi] : 0, e1 = gact ? tb.rowptr[gi + 1] : 0;
        for (int blk = 0; blk < n_blocks; blk++) {
            const int buf = blk & 1;
            if (blk >= 2) bar_sync(ADJ_BAR_EMPTY0 + buf, nthreads);
            const int s0 = s_begin + blk * K, nb = (s_end - s0) < K ? (s_end - s0) : K;
            float* gb = gbuf2 + (size_t)buf * K * N;
            int slot = s0 % R;
            for (int j = 0; j < nb; j++) {
                float part = 0.0f;
                if (gact) {
                    if (s0 + j == 0) part = gather_step0(ring, A, gi, gl, L);
                    else {
                        const int base = slot * N;
                        for (int e = e0 + gl; e < e1; e += L) {
                            int a = base + tb.eoff[e];
                            a += (a < 0) ? RN : 0;
                            part += tb.ew[e] * ring[a];
                        }
                    }
                }
                part = lane_sum(part, L);
                if (gact && gl == 0) gb[j * N + gi] = part;
                slot = (slot + 1 == R) ? 0 : slot + 1;
            }
            bar_arrive(ADJ_BAR_FULL0 + buf, nthreads);
        }
    } else {
        const bool uact = t < N;
        for (int blk = 0; blk < n_blocks; blk++) {
            const int buf = blk & 1;
            bar_sync(ADJ_BAR_FULL0 + buf, nthreads);
            const int s0 = s_begin + blk * K, nb = (s_end - s0) < K ? (s_end - s0) : K;
            if (mode == 0 && !A.store_all && s0 % A.CK == 0) {
                // checkpoint: the ring holds every time before s0 and no consumer has written block s0 yet
                const int k = s0 / A.CK;
                float* cr = A.ck_ring + ((size_t)k * A.B + b) * (size_t)RN;
                for (int q = t; q < RN; q += n_cons) cr[q] = ring[q];
                if (uact) {
                    float* cs = A.ck_state + ((size_t)k * A.B + b) * N * NV + (size_t)t * NV;
#pragma unroll
                    for (int v = 0; v < NV; v++) cs[v] = x[v];
                }
                bar_sync(ADJ_BAR_CONS, n_cons);
            }
            const float* gb = gbuf2 + (size_t)buf * K * N;
            if (uact) {
                int slot = s0 % R;
                for (int j = 0; j < nb; j++) {
                    const int s = s0 + j;
                    const float g = gb[j * N + t];
                    if (mode == 1 || A.store_all) {
                        float* sc = A.scratch + (((size_t)b * A.CK + (s - s_begin)) * N + t) * 8;
#pragma unroll
                        for (int v = 0; v < NV; v++) sc[v] = x[v];
                        sc[6] = g;
                    }
                    adj_step<RK4>(A, prm, x, coupling_post(A.cfk, cp, g));
                    const int next = (slot + 1 == R) ? 0 : slot + 1;
                    ring[next * N + t] = x[0];
                    if (mode == 0) A.Y[((size_t)s * A.B + b) * N + t] = x[1] - x[2];
                    slot = next;
                }
            }
            bar_arrive(ADJ_BAR_EMPTY0 + buf, nthreads);
        }
    }
}

template <bool RK4>
__global__ void adj_forward_kernel(const DevNet* __restrict__ gnet, AdjArgs A, int L, int n_cons) {
    extern __shared__ __align__(16) unsigned char smem[];
    float* ring = reinterpret_cast<float*>(smem);
    const int b = blockIdx.x, N = A.N, RN = A.R * A.N;
    const DevNet& net = *gnet;
    float prm[13], cp[8], x[NV];
    load_params(net, b, prm, cp);
    for (int q = threadIdx.x; q < RN; q += blockDim.x) ring[q] = 0.0f;
    const AdjTables tb = stage_tables(A, smem, (size_t)RN * 4, false);
    float* gbuf = reinterpret_cast<float*>(smem + (((size_t)RN * 4 + tables_size(N, A.rowptr[N]) + 15) & ~(size_t)15));
    __syncthreads();
    const bool uact = (int)threadIdx.x < N;
#pragma unroll
    for (int v = 0; v < NV; v++) x[v] = uact ? A.x0[(size_t)b * N * NV + threadIdx.x * NV + v] : 0.0f;
    if (uact) ring[threadIdx.x] = x[0];
    if (n_cons > 0) {
        __syncthreads();
        forward_pipelined<RK4>(ring, gbuf, A, tb, b, L, x, prm, cp, n_cons, 0, A.T, 0);
    } else {
        forward_steps<RK4>(ring, gbuf, A, tb, b, L, x, prm, cp, 0, A.T, 0);
    }
}

// Re-computation of one checkpoint segment [A.seg_begin, A.seg_end) as the forward's pipeline, from
// the segment's checkpoint (state and ring), keeping x(s), g(s) in the scratch for the reverse.
template <bool RK4>
__global__ void adj_recompute_kernel(const DevNet* __restrict__ gnet, AdjArgs A, int L, int n_cons) {
    extern __shared__ __align__(16) unsigned char smem[];
    float* ring = reinterpret_cast<float*>(smem);
    const int b = blockIdx.x, N = A.N, RN = A.R * A.N;
    const int seg = A.seg_begin / A.CK;
    const DevNet& net = *gnet;
    float prm[13], cp[8], x[NV];
    load_params(net, b, prm, cp);
    const float* cr = A.ck_ring + ((size_t)seg * A.B + b) * (size_t)RN;
    for (int q = threadIdx.x; q < RN; q += blockDim.x) ring[q] = cr[q];
    const AdjTables tb = stage_tables(A, smem, (size_t)RN * 4, false);
    float* gbuf = reinterpret_cast<float*>(smem + (((size_t)RN * 4 + tables_size(N, A.rowptr[N]) + 15) & ~(size_t)15));
    const bool uact = (int)threadIdx.x < N;
#pragma unroll
    for (int v = 0; v < NV; v++) x[v] = uact ? A.ck_state[((size_t)seg * A.B + b) * N * NV + threadIdx.x * NV + v] : 0.0f;
    __syncthreads();
    forward_pipelined<RK4>(ring, gbuf, A, tb, b, L, x, prm, cp, n_cons, A.seg_begin, A.seg_end, 1);
}

// ---- statistics of y, FC, loss, and the coefficients of dL/dy ----
// One pass over y in S time slices per point (grid: points x slices): moments of y - c_i with the
// shift c_i = mean of the first 64 steps, summed in FP32 over chunks of 64 steps and in FP64 across
// chunks, written per slice; adj_fc_kernel adds the slices and forms FC, the loss and the
// coefficients of dL/dy. Each thread owns a 4 x 4 tile of the upper triangle of the product matrix.
using hb::MOM_CHUNK;

__device__ __forceinline__ float moment_shift(const AdjArgs& A, int b, int k) {
    const int n0 = A.T < 64 ? A.T : 64;
    float c = 0.0f;
    for (int t = 0; t < n0; t++) c += A.Y[((size_t)t * A.B + b) * A.N + k];
    return c / (float)n0;
}

__global__ void adj_moments_kernel(AdjArgs A, double* part, int slices) {
    extern __shared__ __align__(16) float zs[];  // [2][MOM_CHUNK][W] chunks of y - shift, then shift[W]
    const int b = blockIdx.x, sl = blockIdx.y, N = A.N, T = A.T;
    const int W = (N + 3) / 4 * 4;
    const int Tc = ((T + slices - 1) / slices + MOM_CHUNK - 1) / MOM_CHUNK * MOM_CHUNK;
    const int t_lo = sl * Tc, t_hi = (t_lo + Tc) < T ? (t_lo + Tc) : T;
    float* shift = zs + 2 * MOM_CHUNK * W;
    double* P = part + ((size_t)b * slices + sl) * ((size_t)W * W + W);  // Q [W][W], then S [W]
    for (int k = threadIdx.x; k < W; k += blockDim.x) shift[k] = k < N ? moment_shift(A, b, k) : 0.0f;
    hb::series_moments_strided(A.Y + (size_t)b * N, (size_t)A.B * N, 1, N, t_lo, t_hi, shift, zs, P);
}

__global__ void adj_fc_kernel(AdjArgs A, const double* part, int slices) {
    extern __shared__ __align__(16) double red[];  // [nth], then dsum [W], dsq [W]
    const int b = blockIdx.x, N = A.N, T = A.T;
    const int tid = threadIdx.x, nth = blockDim.x;
    const int W = (N + 3) / 4 * 4;
    double* dsum = red + nth;
    double* dsq = dsum + W;
    const double* P0 = part + (size_t)b * slices * ((size_t)W * W + W);
    for (int k = tid; k < N; k += nth) {
        double s1 = 0.0, s2 = 0.0;
        for (int sl = 0; sl < slices; sl++) {
            const double* P = P0 + (size_t)sl * ((size_t)W * W + W);
            s1 += P[(size_t)W * W + k];
            s2 += P[(size_t)k * W + k];
        }
        dsum[k] = s1;
        dsq[k] = s2;
        const double m = s1 / T, v = s2 / T - m * m;
        A.mean[(size_t)b * N + k] = (float)(moment_shift(A, b, k) + m);
        A.sdev[(size_t)b * N + k] = (float)sqrt(v > 0.0 ? v : 0.0);
    }
    __syncthreads();
    float* fc = A.fc + (size_t)b * N * N;
    for (int q = tid; q < N * N; q += nth) {
        const int ii = q / N, jj = q - ii * N;
        double qs = 0.0;
        for (int sl = 0; sl < slices; sl++) qs += P0[(size_t)sl * ((size_t)W * W + W) + (size_t)ii * W + jj];
        const double mi = dsum[ii] / T, mj = dsum[jj] / T;
        const double vi = dsq[ii] / T - mi * mi, vj = dsq[jj] / T - mj * mj;
        const double cov = qs / T - mi * mj;
        const double den = sqrt(vi > 0.0 ? vi : 0.0) * sqrt(vj > 0.0 ? vj : 0.0);
        fc[q] = (ii == jj) ? 1.0f : (float)(den > 0.0 ? cov / den : 0.0);
    }
    __syncthreads();
    // loss, M (off-diagonal dL/dFC), r_k, coef_k
    double part_l = 0.0;
    const double inv_n2 = 1.0 / ((double)N * N);
    float* Mb = A.M + (size_t)b * N * N;
    for (int q = tid; q < N * N; q += nth) {
        const int k = q / N, j = q - k * N;
        const double d = (double)fc[q] - (double)A.target[q];
        part_l += d * d;
        Mb[(size_t)j * N + k] = (k == j) ? 0.0f : (float)(2.0 * d * inv_n2);
    }
    red[tid] = part_l;
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
// Time steps per source tile, time steps per thread, and the padded row length of the transposed
// tile (a multiple of 4 for float4 reads; 132 spreads the transposing writes over 8 banks).
constexpr int SRC_TS = 128, SRC_TT = 16, SRC_ROW = 132;

__global__ void adj_source_kernel(AdjArgs A) {
    extern __shared__ __align__(16) float sm[];
    const int b = blockIdx.x, N = A.N;
    const int t0 = blockIdx.y * SRC_TS;
    const int nt = (A.T - t0) < SRC_TS ? (A.T - t0) : SRC_TS;
    float* Ms = sm;                                  // [N][N], M[j][k]
    float* zt = sm + ((N * N + 3) & ~3);             // [N][SRC_ROW], z_j(t0 + tt) normalised
    const float* Mb = A.M + (size_t)b * N * N;
    for (int q = threadIdx.x; q < N * N; q += blockDim.x) Ms[q] = Mb[q];
    for (int q = threadIdx.x; q < SRC_TS * N; q += blockDim.x) {
        const int tt = q / N, k = q - tt * N;
        float z = 0.0f;
        if (tt < nt) {
            const float sd = A.sdev[(size_t)b * N + k];
            z = sd > 0.0f ? (A.Y[((size_t)(t0 + tt) * A.B + b) * N + k] - A.mean[(size_t)b * N + k]) / sd : 0.0f;
        }
        zt[k * SRC_ROW + tt] = z;
    }
    __syncthreads();
    const int kpad = (N + 31) / 32 * 32;
    const int k = threadIdx.x % kpad, w = threadIdx.x / kpad;
    const int tt0 = w * SRC_TT;
    if (k >= N || tt0 >= nt) return;
    float acc[SRC_TT];
#pragma unroll
    for (int q = 0; q < SRC_TT; q++) acc[q] = 0.0f;
    for (int j = 0; j < N; j++) {
        const float m = Ms[j * N + k];
        const float4* zj = reinterpret_cast<const float4*>(zt + j * SRC_ROW + tt0);
#pragma unroll
        for (int q = 0; q < SRC_TT / 4; q++) {
            const float4 z = zj[q];
            acc[4 * q + 0] = __fmaf_rn(m, z.x, acc[4 * q + 0]);
            acc[4 * q + 1] = __fmaf_rn(m, z.y, acc[4 * q + 1]);
            acc[4 * q + 2] = __fmaf_rn(m, z.z, acc[4 * q + 2]);
            acc[4 * q + 3] = __fmaf_rn(m, z.w, acc[4 * q + 3]);
        }
    }
    const float ck = A.coef[(size_t)b * N + k], rk = A.rk[(size_t)b * N + k];
    const float* zk = zt + k * SRC_ROW + tt0;
#pragma unroll
    for (int q = 0; q < SRC_TT; q++)
        if (tt0 + q < nt) A.S[((size_t)(t0 + tt0 + q) * A.B + b) * N + k] = ck * (acc[q] - rk * zk[q]);
}

template <class C>
__device__ __forceinline__ C shfl_coef(const C& k, int src_lane, int L) {
    C o;
    const float* in = reinterpret_cast<const float*>(&k);
    float* out = reinterpret_cast<float*>(&o);
#pragma unroll
    for (int q = 0; q < (int)(sizeof(C) / 4); q++) out[q] = __shfl_sync(0xffffffffu, in[q], src_lane, L);
    return o;
}

// the reverse-step coefficients and their linear step for Heun (JrCoef) or RK4 (JrCoef4)
template <bool RK4>
struct RevStep;
template <>
struct RevStep<false> {
    using Coef = JrCoef;
    static __device__ __forceinline__ Coef coef(const AdjArgs& A, const float* prm, const float* cp, const float* xs, float g) {
        return jr_coef(prm, cp, A.cfk, xs, g, A.dt);
    }
    static __device__ __forceinline__ void lin(const AdjArgs& A, const Coef& k, const float* prm, float* lam, float& mu_c,
                                               float& tA, float& tB, float& ta) {
        jr_lin_step(k, prm, A.dt, A.dt_half, lam, mu_c, tA, tB, ta);
    }
};
template <>
struct RevStep<true> {
    using Coef = JrCoef4;
    static __device__ __forceinline__ Coef coef(const AdjArgs& A, const float* prm, const float* cp, const float* xs, float g) {
        return jr_coef_rk4(prm, cp, A.cfk, xs, g, A.dt, A.dt_h2);
    }
    static __device__ __forceinline__ void lin(const AdjArgs& A, const Coef& k, const float* prm, float* lam, float& mu_c,
                                               float& tA, float& tB, float& ta) {
        jr_lin_step_rk4(k, prm, A.dt, A.dt_h2, A.dt_sixth, lam, mu_c, tA, tB, ta);
    }
};

template <bool RK4>
__global__ void adj_backward_kernel(const DevNet* __restrict__ gnet, AdjArgs A, int L) {
    using RS = RevStep<RK4>;
    extern __shared__ __align__(16) unsigned char smem[];
    float* ring = reinterpret_cast<float*>(smem);  // forward ring during recompute, mu ring during reversal
    const int b = blockIdx.x, N = A.N, R = A.R, T = A.T, RN = A.R * A.N;
    const int i = threadIdx.x / L, lane = threadIdx.x - (threadIdx.x / L) * L;
    const DevNet& net = *gnet;
    const bool act = i < N;
    float prm[13], cp[8];
    load_params(net, b, prm, cp);
    const int nnz = A.rowptr[N];
    const AdjTables tb = stage_tables(A, smem, (size_t)RN * 4, true);
    float* gbuf = reinterpret_cast<float*>(smem + (((size_t)RN * 4 + 2 * tables_size(N, nnz) + 15) & ~(size_t)15));
    __syncthreads();  // the tables are staged by other threads than the ones reading a node's range
    float lam[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) lam[v] = 0.0f;
    if (act) {
        const float sT = A.S[((size_t)(T - 1) * A.B + b) * N + i];
        lam[1] = sT;
        lam[2] = -sT;
    }
    // gradients: FP32 sums over one checkpoint segment, added into FP64 totals once per segment
    double gA = 0.0, gB = 0.0, ga = 0.0, gG = 0.0;
    float* mu_g = A.mu_ring + (size_t)b * RN;
    for (int q = threadIdx.x; q < RN; q += blockDim.x) mu_g[q] = 0.0f;
    const int c0 = act ? tb.cptr[i] : 0, c1 = act ? tb.cptr[i + 1] : 0;
    for (int seg = A.n_ck - 1; seg >= 0; seg--) {
        const int s_begin = seg * A.CK, s_end = (s_begin + A.CK) < T ? (s_begin + A.CK) : T;
        // (a) recompute the segment forward from its checkpoint (unless the forward kept every step)
        __syncthreads();
        if (!A.store_all) {
            const float* cr = A.ck_ring + ((size_t)seg * A.B + b) * (size_t)RN;
            for (int q = threadIdx.x; q < RN; q += blockDim.x) ring[q] = cr[q];
            float x[NV];
            const bool uact = (int)threadIdx.x < N;
#pragma unroll
            for (int v = 0; v < NV; v++)
                x[v] = uact ? A.ck_state[((size_t)seg * A.B + b) * N * NV + (size_t)threadIdx.x * NV + v] : 0.0f;
            forward_steps<RK4>(ring, gbuf, A, tb, b, L, x, prm, cp, s_begin, s_end, 1);
        }
        // (b) the mu ring of the later segments into shared memory
        __syncthreads();
        for (int q = threadIdx.x; q < RN; q += blockDim.x) ring[q] = mu_g[q];
        // (c) reverse sweep in groups of L steps: lane l of a node computes the coefficients of step
        // s_hi - l, then the L steps run in order with the coefficients shuffled from their lane.
        // mu(t) of a time never reached (t > T - 1) reads as the ring's initial 0.
        float sA = 0.0f, sB = 0.0f, sa = 0.0f, sG = 0.0f;
        int slot = (s_end - 1) % R;
        for (int s_hi = s_end - 1; s_hi >= s_begin; s_hi -= L) {
            typename RS::Coef mine;
            float src_mine = 0.0f;
            const int sl = s_hi - lane;
            if (act && sl >= s_begin) {
                const float* sc = A.scratch + (((size_t)b * A.CK + (sl - s_begin)) * N + i) * 8;
                float xs[NV];
#pragma unroll
                for (int v = 0; v < NV; v++) xs[v] = sc[v];
                mine = RS::coef(A, prm, cp, xs, sc[6]);
                if (sl >= 1) src_mine = A.S[((size_t)(sl - 1) * A.B + b) * N + i];
            } else {
                mine = typename RS::Coef{};
            }
            for (int j = 0; j < L; j++) {
                const int s = s_hi - j;
                if (s < s_begin) break;
                if ((s_end - 1 - s) % A.K == 0) __syncthreads();
                float pull = 0.0f;
                if (act && s >= 1) {
                    const int base = slot * N;
                    for (int e = c0 + lane; e < c1; e += L) {
                        int a = base + tb.coff[e];
                        a -= (a >= RN) ? RN : 0;
                        pull += tb.cw[e] * ring[a];
                    }
                }
                pull = lane_sum(pull, L);
                const typename RS::Coef kc = shfl_coef(mine, j, L);
                const float src = __shfl_sync(0xffffffffu, src_mine, j, L);
                if (act) {
                    float mu_c, tA, tB, ta;
                    RS::lin(A, kc, prm, lam, mu_c, tA, tB, ta);
                    sA += tA;
                    sB += tB;
                    sa += ta;
                    sG += mu_c * kc.dcdgain;
                    if (lane == 0) ring[slot * N + i] = mu_c * kc.dcdg;
                    // lambda(s) for s >= 1: delayed-coupling terms pulled from later steps, then dL/dx(s)
                    if (s >= 1) {
                        lam[0] += pull;
                        lam[1] += src;
                        lam[2] -= src;
                    }
                }
                slot = (slot == 0) ? R - 1 : slot - 1;
            }
        }
        gA += sA; gB += sB; ga += sa; gG += sG;
        __syncthreads();
        for (int q = threadIdx.x; q < RN; q += blockDim.x) mu_g[q] = ring[q];
    }
    if (act && lane == 0) {
        A.gA[(size_t)b * N + i] = gA;
        A.gB[(size_t)b * N + i] = gB;
        A.ga[(size_t)b * N + i] = ga;
    }
    // gain gradient: sum over nodes
    __syncthreads();
    double* red = reinterpret_cast<double*>(smem);
    red[threadIdx.x] = (act && lane == 0) ? gG : 0.0;
    __syncthreads();
    for (int o = blockDim.x >> 1; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) A.gG[b] = red[0];
}

// The reverse sweep when the forward kept every step (one segment) and every delay is at least 2K
// steps, as a producer / consumer pipeline: the first n_cons threads are consumers (L lanes per node:
// coefficients lane-parallel, the lambda chain, the mu ring writes), the others producers (L lanes
// per node) that pull the delayed-coupling sums sum_e w_e mu_tgt(e)(s + d_e) of block k + 1 into
// one of two buffers while the consumers run block k. The mu values a producer pulls for block
// k + 1 belong to steps the consumers finished before block k began. Per step the same operations,
// lanes and summation order as adj_backward_kernel, so the gradients are bitwise the same.
constexpr int ADJ_PIPE_MAXT = 640;  // register budget: 102 per thread

template <bool RK4>
__global__ void __launch_bounds__(ADJ_PIPE_MAXT, 1) adj_backward_pipe_kernel(const DevNet* __restrict__ gnet, AdjArgs A,
                                                                            int L, int n_cons) {
    using RS = RevStep<RK4>;
    extern __shared__ __align__(16) unsigned char smem[];
    float* ring = reinterpret_cast<float*>(smem);  // mu ring
    const int b = blockIdx.x, N = A.N, R = A.R, T = A.T, RN = A.R * A.N, K = A.K;
    const int nthreads = blockDim.x;
    const DevNet& net = *gnet;
    float prm[13], cp[8];
    load_params(net, b, prm, cp);
    const int nnz = A.rowptr[N];
    const AdjTables tb = stage_tables(A, smem, (size_t)RN * 4, true);
    float* pbuf = reinterpret_cast<float*>(smem + (((size_t)RN * 4 + 2 * tables_size(N, nnz) + 15) & ~(size_t)15));
    // the segment [sb, se) of this launch: the run's last segment starts from mu = 0 (steps past the end
    // read 0) and lambda = dL/dx(T - 1); earlier segments continue the later ones' mu ring and lambda
    const int sb = A.seg_begin, se = A.seg_end;
    float* mu_g = A.mu_ring + (size_t)b * RN;
    for (int q = threadIdx.x; q < RN; q += nthreads) ring[q] = A.seg_last ? 0.0f : mu_g[q];
    __syncthreads();
    const int n_blocks = (se - sb + K - 1) / K;
    double gG = 0.0;
    bool owner = false;
    if ((int)threadIdx.x >= n_cons) {
        const int p = threadIdx.x - n_cons;
        const int i = p / L, lane = p - (p / L) * L;
        const bool act = i < N;
        const int c0 = act ? tb.cptr[i] : 0, c1 = act ? tb.cptr[i + 1] : 0;
        for (int blk = 0; blk < n_blocks; blk++) {
            const int buf = blk & 1;
            if (blk >= 2) bar_sync(ADJ_BAR_EMPTY0 + buf, nthreads);
            const int s_top = se - 1 - blk * K, nb = (s_top - sb + 1) < K ? (s_top - sb + 1) : K;
            float* pb = pbuf + (size_t)buf * K * N;
            for (int j = 0; j < nb; j++) {
                const int s = s_top - j;
                float pull = 0.0f;
                if (act && s >= 1) {
                    const int base = (s % R) * N;
                    for (int e = c0 + lane; e < c1; e += L) {
                        int a = base + tb.coff[e];
                        a -= (a >= RN) ? RN : 0;
                        pull += tb.cw[e] * ring[a];
                    }
                }
                pull = lane_sum(pull, L);
                if (act && lane == 0) pb[j * N + i] = pull;
            }
            bar_arrive(ADJ_BAR_FULL0 + buf, nthreads);
        }
    } else {
        const int i = threadIdx.x / L, lane = threadIdx.x - (threadIdx.x / L) * L;
        const bool act = i < N;
        owner = act && lane == 0;
        float lam[NV];
#pragma unroll
        for (int v = 0; v < NV; v++) lam[v] = 0.0f;
        if (act) {
            if (A.seg_last) {
                const float sT = A.S[((size_t)(T - 1) * A.B + b) * N + i];
                lam[1] = sT;
                lam[2] = -sT;
            } else {
#pragma unroll
                for (int v = 0; v < NV; v++) lam[v] = A.lam_g[((size_t)b * N + i) * NV + v];
            }
        }
        float sA = 0.0f, sB = 0.0f, sa = 0.0f, sG = 0.0f;
        for (int blk = 0; blk < n_blocks; blk++) {
            const int buf = blk & 1;
            bar_sync(ADJ_BAR_FULL0 + buf, nthreads);
            const int s_top = se - 1 - blk * K, nb = (s_top - sb + 1) < K ? (s_top - sb + 1) : K;
            const float* pb = pbuf + (size_t)buf * K * N;
            for (int g = 0; g < nb; g += L) {
                const int s_hi = s_top - g;
                typename RS::Coef mine;
                float src_mine = 0.0f;
                const int sl = s_hi - lane;
                if (act && g + lane < nb) {
                    const float* sc = A.scratch + (((size_t)b * A.CK + (sl - sb)) * N + i) * 8;
                    float xs[NV];
#pragma unroll
                    for (int v = 0; v < NV; v++) xs[v] = sc[v];
                    mine = RS::coef(A, prm, cp, xs, sc[6]);
                    if (sl >= 1) src_mine = A.S[((size_t)(sl - 1) * A.B + b) * N + i];
                } else {
                    mine = typename RS::Coef{};
                }
                for (int j = 0; j < L; j++) {
                    const int jj = g + j;
                    if (jj >= nb) break;
                    const int s = s_top - jj;
                    const typename RS::Coef kc = shfl_coef(mine, j, L);
                    const float src = __shfl_sync(0xffffffffu, src_mine, j, L);
                    if (act) {
                        float mu_c, tA, tB, ta;
                        RS::lin(A, kc, prm, lam, mu_c, tA, tB, ta);
                        sA += tA;
                        sB += tB;
                        sa += ta;
                        sG += mu_c * kc.dcdgain;
                        if (lane == 0) ring[(s % R) * N + i] = mu_c * kc.dcdg;
                        if (s >= 1) {
                            lam[0] += pb[jj * N + i];
                            lam[1] += src;
                            lam[2] -= src;
                        }
                    }
                }
            }
            bar_arrive(ADJ_BAR_EMPTY0 + buf, nthreads);
        }
        // FP32 sums within the segment, FP64 across segments
        if (owner) {
            const size_t gi = (size_t)b * N + i;
            A.gA[gi] = (A.seg_last ? 0.0 : A.gA[gi]) + (double)sA;
            A.gB[gi] = (A.seg_last ? 0.0 : A.gB[gi]) + (double)sB;
            A.ga[gi] = (A.seg_last ? 0.0 : A.ga[gi]) + (double)sa;
            gG = (double)sG;
            if (sb > 0) {
#pragma unroll
                for (int v = 0; v < NV; v++) A.lam_g[gi * NV + v] = lam[v];
            }
        }
    }
    // the mu ring for the next (earlier) segment
    if (sb > 0) {
        __syncthreads();
        for (int q = threadIdx.x; q < RN; q += nthreads) mu_g[q] = ring[q];
    }
    // gain gradient: sum over nodes, a tree over the next power of two of the block (zeros past it)
    __syncthreads();
    int p2 = 1;
    while (p2 < nthreads) p2 <<= 1;
    double* red = reinterpret_cast<double*>(smem);
    for (int q = threadIdx.x; q < p2; q += nthreads) red[q] = 0.0;
    __syncthreads();
    if (owner) red[threadIdx.x] = gG;
    __syncthreads();
    for (int o = p2 >> 1; o > 0; o >>= 1) {
        for (int q = threadIdx.x; q < o; q += nthreads) red[q] += red[q + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) A.gG[b] = (A.seg_last ? 0.0 : A.gG[b]) + red[0];
}

}  // namespace

// ---- launch interface used by the engine (hb_engine.cu) ----

cudaError_t hb_launch_adjoint(const DevNet* d_net, const HbAdjointLaunch& L, int phase, cudaStream_t st) {
    AdjArgs A;
    A.B = L.B; A.N = L.N; A.T = L.T; A.R = L.R; A.K = L.K; A.CK = L.CK; A.n_ck = L.n_ck; A.store_all = L.store_all;
    A.cfk = L.cfk; A.gain_idx = L.gain_idx; A.dt = L.dt; A.dt_half = L.dt_half;
    A.rk4 = L.rk4; A.dt_h2 = L.dt_h2; A.dt_sixth = L.dt_sixth;
    A.x0 = L.x0; A.rowptr = L.rowptr; A.edges = L.edges; A.ew = L.ew;
    A.cptr = L.cptr; A.ctgt = L.ctgt; A.cdel = L.cdel; A.cw = L.cw;
    A.Y = L.Y; A.S = L.S; A.ck_state = L.ck_state; A.ck_ring = L.ck_ring; A.scratch = L.scratch; A.mu_ring = L.mu_ring;
    A.lam_g = L.lam_g;
    A.seg_begin = 0; A.seg_end = L.T; A.seg_last = 1;
    A.target = L.target; A.mean = L.mean; A.sdev = L.sdev; A.coef = L.coef; A.rk = L.rk; A.M = L.M; A.fc = L.fc;
    A.loss = L.loss; A.gG = L.gG; A.gA = L.gA; A.gB = L.gB; A.ga = L.ga;
    // lanes per node: a power of two up to 4 within 1024 threads; the block a power of two for the
    // final reduction
    int lanes = 1;
    while (lanes < 4 && L.N * lanes * 2 <= 1024) lanes *= 2;
    int threads = 32;
    while (threads < L.N * lanes) threads *= 2;
    const int nnz = L.nnz;
    const size_t ring_bytes = (size_t)L.R * L.N * sizeof(float);
    const size_t tab1 = (size_t)(L.N + 1) * 4 + (size_t)nnz * 8;
    const size_t gbuf_bytes = (size_t)L.K * L.N * sizeof(float) + 16;
    if (phase == 0) {
        // pipelined: one consumer thread per node (warp aligned), then lanes producer threads per node
        const int n_cons = L.pipelined ? (L.N + 31) / 32 * 32 : 0;
        const int fthreads = L.pipelined ? n_cons + (L.N * lanes + 31) / 32 * 32 : threads;
        const size_t sm = ring_bytes + tab1 + (L.pipelined ? 2 * gbuf_bytes : gbuf_bytes);
        auto kf = L.rk4 ? adj_forward_kernel<true> : adj_forward_kernel<false>;
        if (cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
            return cudaGetLastError();
        kf<<<L.B, fthreads, sm, st>>>(d_net, A, lanes, n_cons);
    } else if (phase == 1) {
        const size_t W = (size_t)(L.N + 3) / 4 * 4;
        const size_t sm = (2 * MOM_CHUNK + 1) * W * sizeof(float) + 16;
        if (cudaFuncSetAttribute(adj_moments_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
            return cudaGetLastError();
        const int n_tiles = (int)(W / 4 * (W / 4 + 1) / 2);
        adj_moments_kernel<<<dim3(L.B, L.slices), n_tiles <= 256 ? 256 : 512, sm, st>>>(A, L.moments, L.slices);
        adj_fc_kernel<<<L.B, 512, (512 + 2 * W) * sizeof(double), st>>>(A, L.moments, L.slices);
        const size_t sm2 = ((((size_t)L.N * L.N + 3) & ~(size_t)3) + (size_t)SRC_ROW * L.N) * sizeof(float);
        if (cudaFuncSetAttribute(adj_source_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2) != cudaSuccess)
            return cudaGetLastError();
        const int kpad = (L.N + 31) / 32 * 32;
        dim3 grid(L.B, (L.T + SRC_TS - 1) / SRC_TS);
        adj_source_kernel<<<grid, kpad * (SRC_TS / SRC_TT), sm2, st>>>(A);
    } else {
        const int rl = lanes;
        // pipelined reverse: one segment, every delay >= 2K, coefficient groups inside a block
        const int pc = (L.N * rl + 31) / 32 * 32, pthreads = 2 * pc;
        const size_t psm = std::max(((ring_bytes + 2 * tab1 + 15) & ~(size_t)15) + 2 * (size_t)L.K * L.N * sizeof(float),
                                    (size_t)1024 * sizeof(double));
        int max_sm = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&max_sm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (L.pipelined && L.dmin >= 2 * L.K && L.K % rl == 0 && pthreads <= ADJ_PIPE_MAXT && psm <= (size_t)max_sm) {
            auto kp = L.rk4 ? adj_backward_pipe_kernel<true> : adj_backward_pipe_kernel<false>;
            if (cudaFuncSetAttribute(kp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psm) != cudaSuccess)
                return cudaGetLastError();
            if (L.store_all) {
                kp<<<L.B, pthreads, psm, st>>>(d_net, A, rl, pc);
                return cudaGetLastError();
            }
            // checkpointed: the segments last to first, each re-computed from its checkpoint by the forward
            // pipeline into one of two scratch buffers, then reversed. The re-computation of segment k - 1
            // runs on a second stream, on SMs the reverse of segment k leaves idle (one CTA per point each),
            // so only the last segment's re-computation adds to the reverse time.
            const int n_cons = (L.N + 31) / 32 * 32;
            const int fthreads = n_cons + (L.N * lanes + 31) / 32 * 32;
            const size_t fsm = ring_bytes + tab1 + 2 * gbuf_bytes;
            auto kr = L.rk4 ? adj_recompute_kernel<true> : adj_recompute_kernel<false>;
            if (cudaFuncSetAttribute(kr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsm) != cudaSuccess)
                return cudaGetLastError();
            const size_t seg_floats = (size_t)L.B * L.CK * L.N * 8;
            auto seg_args = [&](int seg) {
                AdjArgs a2 = A;
                a2.seg_begin = seg * L.CK;
                a2.seg_end = (seg + 1) * L.CK < L.T ? (seg + 1) * L.CK : L.T;
                a2.seg_last = seg == L.n_ck - 1 ? 1 : 0;
                a2.scratch = L.scratch + (size_t)(seg & 1) * seg_floats;
                return a2;
            };
            cudaStream_t s2 = nullptr;
            cudaEvent_t ev_start = nullptr, rc[2] = {nullptr, nullptr}, bk[2] = {nullptr, nullptr};
            cudaError_t ce = cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking);
            if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&ev_start, cudaEventDisableTiming);
            for (int q = 0; q < 2 && ce == cudaSuccess; q++) ce = cudaEventCreateWithFlags(&rc[q], cudaEventDisableTiming);
            for (int q = 0; q < 2 && ce == cudaSuccess; q++) ce = cudaEventCreateWithFlags(&bk[q], cudaEventDisableTiming);
            if (ce == cudaSuccess) ce = cudaEventRecord(ev_start, st);
            if (ce == cudaSuccess) ce = cudaStreamWaitEvent(s2, ev_start, 0);
            const int last = L.n_ck - 1;
            if (ce == cudaSuccess) {
                kr<<<L.B, fthreads, fsm, s2>>>(d_net, seg_args(last), lanes, n_cons);
                ce = cudaGetLastError();
            }
            if (ce == cudaSuccess) ce = cudaEventRecord(rc[last & 1], s2);
            for (int seg = last; seg >= 0 && ce == cudaSuccess; seg--) {
                ce = cudaStreamWaitEvent(st, rc[seg & 1], 0);
                if (ce != cudaSuccess) break;
                kp<<<L.B, pthreads, psm, st>>>(d_net, seg_args(seg), rl, pc);
                ce = cudaGetLastError();
                if (ce == cudaSuccess) ce = cudaEventRecord(bk[seg & 1], st);
                if (ce == cudaSuccess && seg > 0) {
                    // the buffer of segment seg - 1 was last read by the reverse of segment seg + 1
                    ce = cudaStreamWaitEvent(s2, bk[(seg - 1) & 1], 0);
                    if (ce == cudaSuccess) {
                        kr<<<L.B, fthreads, fsm, s2>>>(d_net, seg_args(seg - 1), lanes, n_cons);
                        ce = cudaGetLastError();
                    }
                    if (ce == cudaSuccess) ce = cudaEventRecord(rc[(seg - 1) & 1], s2);
                }
            }
            for (auto* ev : {&ev_start, &rc[0], &rc[1], &bk[0], &bk[1]})
                if (*ev) cudaEventDestroy(*ev);
            if (s2) cudaStreamDestroy(s2);
            return ce;
        }
        int rthreads = 32;
        while (rthreads < L.N * rl) rthreads *= 2;
        const size_t sm = std::max(ring_bytes + 2 * tab1 + gbuf_bytes, (size_t)rthreads * sizeof(double));
        auto kb = L.rk4 ? adj_backward_kernel<true> : adj_backward_kernel<false>;
        if (cudaFuncSetAttribute(kb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
            return cudaGetLastError();
        kb<<<L.B, rthreads, sm, st>>>(d_net, A, rl);
    }
    return cudaGetLastError();
}
