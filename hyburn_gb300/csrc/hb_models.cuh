// hb_models.cuh — per-node model derivatives, clamps and coupling pre/post on the device.
//
// Each function evaluates the same binary operations, in the same order, as the reference's
// batch tensor expressions (src/engine/batch_engine/dfun.rs:271-516, coupling.rs:204-444). This
// translation unit is compiled with --fmad=false so that no multiply-add is contracted: every
// product and sum is rounded separately, as in the reference's element-wise tensor ops.
#pragma once
#include "hb_device.h"

namespace hb {

__device__ __forceinline__ float maxf_(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float minf_(float a, float b) { return a < b ? a : b; }

// dfun of one node. `p` is the (sub, point) parameter row; `sweep_form` selects the expression
// used when the model's native sweep parameter arrives as a per-point tensor (dfun.rs:49-72).
__device__ __forceinline__ void dfun(int model, const float* p, int sweep_form, const float* x, const float* c,
                                     float* dx) {
    switch (model) {
    case HBM_G2DO: {
        const float eps = 1.1920929e-07f;
        float tau_g = p[0];
        tau_g = tau_g > eps ? tau_g : eps;
        float a_g = p[2], b_g = p[3], c_g = p[4], d_g = p[5], e_g = p[6], f_g = p[7], g_g = p[8];
        float alpha = p[9], beta = p[10], gamma = p[11];
        float dtau = d_g * tau_g;
        float d_over_tau = d_g / tau_g;
        float v = x[0], w = x[1], c0 = c[0];
        float i_ext_term;
        if (sweep_form) i_ext_term = (c0 + p[1]) * gamma;
        else { float gi = gamma * p[1]; i_ext_term = c0 * gamma + gi; }
        float v2 = v * v;
        float v3 = v * v2;
        float t = w * alpha;
        t = t + i_ext_term;
        t = t - v3 * f_g;
        t = t + v2 * e_g;
        t = t + v * g_g;
        dx[0] = t * dtau;
        float u = v * b_g;
        u = u + v2 * c_g;
        u = u - w * beta;
        u = u + a_g;
        dx[1] = u * d_over_tau;
        break;
    }
    case HBM_MPR: {
        const float eps = 1.1920929e-07f;
        float tau = p[0];
        tau = tau > eps ? tau : eps;
        float delta = p[1], eta = p[2], j = p[3], i_ext = p[4], cr = p[5], cv = p[6];
        float r = x[0], v = x[1], c_r = c[0], c_v = c[1];
        const float pi = 3.14159265358979323846f;
        float inv_tau = 1.0f / tau;
        float dr = r * v;
        dr = dr * 2.0f;
        dr = dr + delta / (pi * tau);
        dx[0] = dr * inv_tau;
        float v2 = v * v, r2 = r * r;
        float k = pi * pi;
        k = k * tau;
        k = k * tau;
        float dv = v2 - r2 * k;
        if (sweep_form) { dv = dv + eta; dv = dv + p[4]; }
        else dv = dv + (eta + i_ext);
        dv = dv + r * (j * tau);
        dv = dv + c_r * cr;
        dv = dv + c_v * cv;
        dx[1] = dv * inv_tau;
        break;
    }
    case HBM_RWW: {
        float a = p[0], b = p[1], d = p[2], gamma = p[3], tau_s = p[4], w = p[5], j_n = p[6];
        float s = x[0], c0 = c[0];
        float xx = s * (w * j_n);
        xx = xx + p[7];
        xx = xx + c0 * j_n;
        float ax_b = xx * a + (-b);
        float e = expf(ax_b * (-d));
        float denom = (-e) + 1.0f;
        float h = ax_b / denom;
        float t1 = (-s) * (1.0f / tau_s);
        float t2 = ((-s) + 1.0f) * h;
        t2 = t2 * gamma;
        dx[0] = t1 + t2;
        break;
    }
    case HBM_KURAMOTO:
        dx[0] = c[0] + p[0];
        break;
    case HBM_JR: {
        float A = p[0], B = p[1], a = p[2], b = p[3], v0 = p[4], nu_max = p[5], r = p[6], J = p[7];
        float a1 = p[8], a2 = p[9], a3 = p[10], a4 = p[11], mu = p[12];
        float y0 = x[0], y1 = x[1], y2 = x[2], y3 = x[3], y4 = x[4], y5 = x[5], c0 = c[0];
        float two_nu_max = 2.0f * nu_max;
        float args[3] = {y1 - y2, y0 * (a1 * J), y0 * (a3 * J)};
        float sv[3];
#pragma unroll
        for (int q = 0; q < 3; q++) {
            float arg = (-args[q]) + v0;
            arg = arg * r;
            float denom = expf(arg) + 1.0f;
            sv[q] = (1.0f * two_nu_max) / denom;
        }
        dx[0] = y3;
        dx[1] = y4;
        dx[2] = y5;
        float d3 = sv[0] * (A * a);
        d3 = d3 - y3 * (2.0f * a);
        d3 = d3 - y0 * (a * a);
        dx[3] = d3;
        float mt = sv[1] * (a2 * J);
        mt = mt + (sweep_form ? p[12] : mu);
        mt = mt + c0;
        float d4 = mt * (A * a);
        d4 = d4 - y4 * (2.0f * a);
        d4 = d4 - y1 * (a * a);
        dx[4] = d4;
        float d5 = sv[2] * (a4 * J);
        d5 = d5 * (B * b);
        d5 = d5 - y5 * (2.0f * b);
        d5 = d5 - y2 * (b * b);
        dx[5] = d5;
        break;
    }
    case HBM_WC: {
        const float eps = 1.1920929e-07f;
        float c_ee = p[0], c_ei = p[1], c_ie = p[2], c_ii = p[3];
        float tau_e = p[4], tau_i = p[5];
        tau_e = tau_e > eps ? tau_e : eps;
        tau_i = tau_i > eps ? tau_i : eps;
        float a_e = p[6], b_e = p[7], ce = p[8], theta_e = p[9];
        float a_i = p[10], b_i = p[11], ci = p[12], theta_i = p[13];
        float r_e = p[14], r_i = p[15], k_e = p[16], k_i = p[17];
        float q = p[19], alpha_e = p[20], alpha_i = p[21];
        float sig_e_off = p[HB_D_WC_SIG_E_OFF], sig_i_off = p[HB_D_WC_SIG_I_OFF];
        float e = x[0], iv = x[1], c0 = c[0];
        float xe = e * c_ee - iv * c_ei;
        xe = xe - theta_e;
        xe = xe + c0;
        xe = xe + p[18];
        xe = xe * alpha_e;
        float xi = e * c_ie - iv * c_ii;
        xi = xi + q;
        xi = xi - theta_i;
        xi = xi * alpha_i;
        float ea = expf((xe + (-b_e)) * (-a_e));
        float sig_e = 1.0f / (ea + 1.0f);
        float s_e = (sig_e - sig_e_off) * ce;
        float ia = expf((xi + (-b_i)) * (-a_i));
        float sig_i = 1.0f / (ia + 1.0f);
        float s_i = (sig_i - sig_i_off) * ci;
        float de = (-e) + (e * (-r_e) + k_e) * s_e;
        dx[0] = de * (1.0f / tau_e);
        float di = (-iv) + (iv * (-r_i) + k_i) * s_i;
        dx[1] = di * (1.0f / tau_i);
        break;
    }
    }
}

// clamp_batch (dfun.rs:170-239)
__device__ __forceinline__ void clamp(int model, float* x) {
    switch (model) {
    case HBM_WC:
        x[0] = maxf_(minf_(x[0], 1.0f), 0.0f);
        x[1] = maxf_(minf_(x[1], 1.0f), 0.0f);
        break;
    case HBM_MPR:
        x[0] = maxf_(x[0], 0.0f);
        break;
    case HBM_RWW:
        x[0] = maxf_(minf_(x[0], 1.0f), 0.0f);
        break;
    case HBM_KURAMOTO: {
        const float two_pi = 2.0f * 3.14159265358979323846f;
        x[0] = x[0] - floorf(x[0] / two_pi) * two_pi;
        break;
    }
    default:
        break;
    }
}

// Resolved coupling parameter slots (host fills DevProj::cp / cp_pp in this layout):
//  LINEAR/SCALED_LINEAR: a=0 b=1 | SIGMOIDAL: cmin=0 cmax=1 mid=2 a=3 sigma=4
//  DIFFERENCE: a=0 | KURAMOTO: a=0, a/n_src=1 | TANH: a=0 b=1 mid=2 sigma=3
//  SJR: a=0 classic=1 cmin=2 cmax=3 r=4 mid=5 e0=6 v0=7 | PRESIG: h=0 q=1 g=2 p=3 theta=4 dynamic=5

// pre() of one source row (coupling.rs:204-258 tensor form; 268-321 per-edge CPU form).
// ncv <= 2 and the channel count <= 4; loops are unrolled to those bounds so that every array
// stays in registers.
__device__ __forceinline__ void pre(int cfk, const float* cp, int cpu_form, const float* x, int ncv, float* out) {
    switch (cfk) {
    case HBC_KURAMOTO: {
        float s0 = sinf(x[0]), c0 = cosf(x[0]);
        if (ncv == 1) { out[0] = s0; out[1] = c0; }
        else {
            float s1 = sinf(x[1]), c1 = cosf(x[1]);
            if (cpu_form) { out[0] = s0; out[1] = c0; out[2] = s1; out[3] = c1; }
            else { out[0] = s0; out[1] = s1; out[2] = c0; out[3] = c1; }
        }
        break;
    }
    case HBC_TANH:
#pragma unroll
        for (int c = 0; c < 2; c++) {
            if (c < ncv) {
                if (cpu_form) { float inner = (x[c] * cp[1] - cp[2]) / cp[3]; out[c] = cp[0] * (1.0f + tanhf(inner)); }
                else { float inner = (x[c] * cp[1] + (-cp[2])) / cp[3]; out[c] = (tanhf(inner) + 1.0f) * cp[0]; }
            }
        }
        break;
    case HBC_SJR: {
        float x0 = x[0], x1 = ncv >= 2 ? x[1] : 0.0f;
        float diff = x0 - x1;
        bool classic = cp[1] != 0.0f;
        if (cpu_form) {
            if (classic) { float sh = (diff - cp[5]) * (-cp[4]); float den = expf(sh) + 1.0f; out[0] = cp[2] + (cp[3] - cp[2]) / den; }
            else { float sh = (diff - cp[7]) * (-cp[4]); float den = expf(sh) + 1.0f; out[0] = cp[0] * 2.0f * cp[6] / den; }
        } else {
            if (classic) { float sh = (diff + (-cp[5])) * (-cp[4]); float den = expf(sh) + 1.0f; out[0] = (1.0f / den) * (cp[3] - cp[2]) + cp[2]; }
            else { float sh = (diff + (-cp[7])) * (-cp[4]); float den = expf(sh) + 1.0f; out[0] = (1.0f / den) * ((cp[0] * 2.0f) * cp[6]); }
        }
        break;
    }
    case HBC_PRESIG:
        if (cp[5] != 0.0f) {
            float x0 = x[0], x1 = ncv >= 2 ? x[1] : 0.0f;
            float inner = cpu_form ? (cp[3] * x0 - x1) : (x0 * cp[3] - x1);
            out[0] = (tanhf(inner * cp[2]) + cp[1]) * cp[0];
        } else {
#pragma unroll
            for (int c = 0; c < 2; c++) {
                if (c < ncv) {
                    float inner = cpu_form ? (cp[3] * x[c] - cp[4]) : (x[c] * cp[3] + (-cp[4]));
                    out[c] = (tanhf(inner * cp[2]) + cp[1]) * cp[0];
                }
            }
        }
        break;
    default:  // Linear, Sigmoidal, ScaledLinear, Difference: identity
        out[0] = x[0];
        if (ncv > 1) out[1] = x[1];
        break;
    }
}

// post_with_target (coupling.rs:323-399, engine.rs:621-633); returns the output channel count
__device__ __forceinline__ int post(int cfk, const float* cp, int has_rowsums, const float* gx, int pc,
                                    const float* xi, int tgt_ncv, float rowsum, float* out) {
    switch (cfk) {
    case HBC_LINEAR:
#pragma unroll
        for (int c = 0; c < 4; c++) if (c < pc) out[c] = gx[c] * cp[0] + cp[1];
        return pc;
    case HBC_SIGMOIDAL:
#pragma unroll
        for (int c = 0; c < 4; c++) {
            if (c < pc) {
                float sh = (gx[c] + (-cp[2])) / cp[4];
                float ex = -(sh * cp[3]);
                float den = expf(ex) + 1.0f;
                out[c] = (1.0f / den) * (cp[1] - cp[0]) + cp[0];
            }
        }
        return pc;
    case HBC_SCALED_LINEAR:
#pragma unroll
        for (int c = 0; c < 4; c++) if (c < pc) out[c] = (gx[c] + (-cp[1])) * cp[0];
        return pc;
    case HBC_DIFFERENCE:
        if (has_rowsums) {
#pragma unroll
            for (int c = 0; c < 2; c++) if (c < pc) out[c] = (gx[c] - xi[c] * rowsum) * cp[0];
        } else {
#pragma unroll
            for (int c = 0; c < 4; c++) if (c < pc) out[c] = gx[c] * cp[0];
        }
        return pc;
    case HBC_KURAMOTO:
        if (tgt_ncv == 1) {
            float t = cosf(xi[0]) * gx[0] - sinf(xi[0]) * gx[1];
            out[0] = t * cp[1];
        } else {
            float t0 = cosf(xi[0]) * gx[0] - sinf(xi[0]) * gx[2];
            float t1 = cosf(xi[1]) * gx[1] - sinf(xi[1]) * gx[3];
            out[0] = t0 * cp[1];
            out[1] = t1 * cp[1];
        }
        return tgt_ncv;
    case HBC_SJR:
        if (cp[1] != 0.0f) out[0] = gx[0] * cp[0];
        else out[0] = gx[0];
        return pc;
    default:
#pragma unroll
        for (int c = 0; c < 4; c++) if (c < pc) out[c] = gx[c];
        return pc;
    }
}

// compile-time model facts (MODEL = -1: decided at run time)
__host__ __device__ constexpr int c_nvar(int m) { return m == HBM_G2DO ? 2 : m == HBM_MPR ? 2 : m == HBM_RWW ? 1 : m == HBM_KURAMOTO ? 1 : m == HBM_JR ? 6 : m == HBM_WC ? 2 : 6; }
__host__ __device__ constexpr int c_ncvar(int m) { return m == HBM_MPR ? 2 : (m >= 0 ? 1 : 2); }
// parameter-row entries a model reads (WilsonCowan also reads the two derived constants at 24, 25)
__host__ __device__ constexpr int c_nparams_used(int m) {
    return m == HBM_G2DO ? 12 : m == HBM_MPR ? 7 : m == HBM_RWW ? 8 : m == HBM_KURAMOTO ? 1 : m == HBM_JR ? 13 : m == HBM_WC ? 26 : HB_PSTRIDE;
}

template <int MODEL>
__device__ __forceinline__ void dfun_m(int model, const float* p, int sweep_form, const float* x, const float* c, float* dx) {
    dfun(MODEL >= 0 ? MODEL : model, p, sweep_form, x, c, dx);
}

template <int MODEL>
__device__ __forceinline__ void clamp_m(int model, float* x) {
    clamp(MODEL >= 0 ? MODEL : model, x);
}

__device__ __forceinline__ float pick4(const float* a, int i) {
    return i == 0 ? a[0] : (i == 1 ? a[1] : (i == 2 ? a[2] : a[3]));
}

// Balloon-Windkessel forward Euler step of one node (bold.rs:106-150), default parameters
__device__ __forceinline__ void bw_step(float& s_, float& f_, float& v_, float& q_, float input, float dt_f) {
    const float tau_s = 1.54f, tau_f = 0.50f, tau_0 = 1.02f, alpha = 0.32f, e0 = 0.34f;
    float kappa = 1.0f / tau_s, gamma = 1.0f / tau_f, tau_inv = 1.0f / tau_0;
    float z = input > 0.0f ? input : 0.0f;
    float s = s_, f = f_, v = v_, q = q_;
    float fs = f > 1e-6f ? f : 1e-6f;
    float vs = v > 1e-6f ? v : 1e-6f;
    float ds = z - kappa * s - gamma * (fs - 1.0f);
    float df = s;
    float va = powf(vs, 1.0f / alpha);
    float dv = tau_inv * (fs - va);
    float dq = tau_inv * (fs * (1.0f - powf(1.0f - e0, 1.0f / fs)) / e0 - va * (q / vs));
    float sn = s + dt_f * ds, fn = fs + dt_f * df, vn = vs + dt_f * dv, qn = q + dt_f * dq;
    s_ = sn > 0.0f ? sn : 0.0f;
    f_ = fn > 1e-6f ? fn : 1e-6f;
    v_ = vn > 1e-6f ? vn : 1e-6f;
    q_ = qn > 0.0f ? qn : 0.0f;
}

// BoldModel::signal (bold.rs:153-166)
__device__ __forceinline__ float bw_signal(float v_, float q) {
    float v = v_ > 1e-6f ? v_ : 1e-6f;
    return 4.0f * (7.0f * (1.0f - q) + 2.0f * (1.0f - q / v) + 2.0f * (1.0f - v));
}

}  // namespace hb
