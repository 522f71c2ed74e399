/*
 * hb_oracle.c — CPU oracle for hyburn's batched simulation step (TEST INFRASTRUCTURE).
 *
 * This file is the checker, not the product: only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference legs load it. The CUDA engine never calls into it.
 *
 * It restates, operation for operation and in the same floating-point order, the reference's
 * NdArray path of `BatchHybridEngine` (hyburn 0.2.0, Rust):
 *   - setup                     src/engine/batch_engine/engine.rs:145-471
 *   - step loop                 src/engine/batch_engine/engine.rs:540-804
 *   - multi-parameter sweeps    src/engine/batch_engine/engine.rs:53-91, 862-1348
 *   - batch dfuns / clamps      src/engine/batch_engine/dfun.rs:32-97, 99-133, 170-239, 271-516
 *   - coupling pre/post         src/engine/coupling.rs:114-444
 *   - noise scaling             src/engine/integrator.rs:170-198
 *   - Balloon-Windkessel BOLD   src/engine/bold.rs:22-166, src/engine/bold_monitor.rs:49-227
 *   - per-edge ring delays      src/engine/runtime.rs:55-85, 125-211 (HB_SEM_DELAY_RING)
 * The history of the default (batch) mode is the literal shift window of engine.rs:541-551,
 * not a closed-form index, so that the device path's index arithmetic is checked against it.
 *
 * Built twice: FP32 (HBO_REAL=float, symbols hbo_*) and an FP64 twin (HBO_REAL=double,
 * symbols hbo64_*) used to report drift against a higher-precision integration.
 * Compile with -ffp-contract=off so that no multiply-add is fused (Rust does not fuse either).
 *
 * Pinning: the reference's own known-answer tests (dfuns, clamps, coupling pre/post, BOLD, sweep
 * order, ring semantics; restated in tests/test_oracle_kat.py, tests/test_config_ref.py,
 * tests/test_integrator_ref.py, tests/test_sparse_ref.py) pin the units and the engine semantics.
 * Whole trajectories are unpinned against the reference itself: it is Rust, no Rust toolchain is
 * available to run it, and its TVB trajectory files are git-LFS pointers. The fixtures in
 * tests/golden/ keep this oracle's own outputs from drifting; they are not the reference's outputs.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#include <stdarg.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "hyburn_gb300.h"

#ifndef HBO_REAL
#define HBO_REAL float
#endif
#ifndef HBO_PREFIX
#define HBO_PREFIX hbo_
#endif
#define HBO_CAT2(a, b) a##b
#define HBO_CAT(a, b) HBO_CAT2(a, b)
#define HBO(name) HBO_CAT(HBO_PREFIX, name)

typedef HBO_REAL real;

#if defined(HBO_DOUBLE)
#define R_EXP exp
#define R_SIN sin
#define R_COS cos
#define R_TANH tanh
#define R_SQRT sqrt
#define R_POW pow
#define R_FLOOR floor
#define R_PI ((real)3.14159265358979323846)
#else
#define R_EXP expf
#define R_SIN sinf
#define R_COS cosf
#define R_TANH tanhf
#define R_SQRT sqrtf
#define R_POW powf
#define R_FLOOR floorf
#define R_PI ((real)3.14159265358979323846f)
#endif

#define EXPORT __attribute__((visibility("default")))

static __thread char g_err[512];
static void set_err(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}
EXPORT const char* HBO(last_error)(void) { return g_err; }

/* ------------------------------------------------------------------------------------------ */
/* models: config.rs:43-49 registry, construction.rs:57-89 names                              */
/* ------------------------------------------------------------------------------------------ */
enum { M_G2DO = 0, M_MPR, M_RWW, M_KURAMOTO, M_JR, M_WC, M_COUNT };
static const char* k_model_names[M_COUNT] = {
    "Generic2dOscillator", "MontbrioPazoRoxin", "ReducedWongWang", "Kuramoto", "JansenRit", "WilsonCowan"};
static const int k_nvar[M_COUNT] = {2, 2, 1, 1, 6, 2};
static const int k_ncvar[M_COUNT] = {1, 2, 1, 1, 1, 1};
static const int k_nparams[M_COUNT] = {12, 7, 8, 1, 13, 22};
/* Sweepable parameter of the batch-native dfun (dfun.rs:49-72). */
static const int k_native_sweep[M_COUNT] = {1, 4, 7, 0, 12, 18};
/* First entry of each model CVAR list (src/model/NAME.rs): JR couples through state var 1. */
static const int k_cvar0[M_COUNT] = {0, 0, 0, 0, 1, 0};

static int model_from_name(const char* name) {
    if (!name) return -1;
    for (int i = 0; i < M_COUNT; i++)
        if (strcmp(name, k_model_names[i]) == 0) return i;
    return -1;
}

/* position of state var t in the model's CVAR list, or 0 if absent (engine.rs:389-392) */
static int cvar_position(int model, int t) {
    if (model == M_MPR) return (t == 0) ? 0 : (t == 1 ? 1 : 0);
    return (k_cvar0[model] == t) ? 0 : 0;
}

/* Batch dfun of one node (dfun.rs:271-516). `sweep_form` selects the batch-native sweep
 * expression (the swept parameter arrives as a per-point tensor) used when the swept index is
 * the model's native one; otherwise the scalar-parameter expression. */
static void dfun_node(int model, const real* p, int sweep_form, const real* x, const real* c, real* dx) {
    switch (model) {
    case M_G2DO: {
        real tau_g = p[0];
        tau_g = tau_g > (real)FLT_EPSILON ? tau_g : (real)FLT_EPSILON;
        real a_g = p[2], b_g = p[3], c_g = p[4], d_g = p[5], e_g = p[6], f_g = p[7], g_g = p[8];
        real alpha = p[9], beta = p[10], gamma = p[11];
        real dtau = d_g * tau_g;
        real d_over_tau = d_g / tau_g;
        real v = x[0], w = x[1], c0 = c[0];
        real i_ext_term;
        if (sweep_form) i_ext_term = (c0 + p[1]) * gamma;
        else { real gi = gamma * p[1]; i_ext_term = c0 * gamma + gi; }
        real v2 = v * v;
        real v3 = v * v2;
        real t = w * alpha;
        t = t + i_ext_term;
        t = t - v3 * f_g;
        t = t + v2 * e_g;
        t = t + v * g_g;
        dx[0] = t * dtau;
        real u = v * b_g;
        u = u + v2 * c_g;
        u = u - w * beta;
        u = u + a_g;
        dx[1] = u * d_over_tau;
        break;
    }
    case M_MPR: {
        real tau = p[0];
        tau = tau > (real)FLT_EPSILON ? tau : (real)FLT_EPSILON;
        real delta = p[1], eta = p[2], j = p[3], i_ext = p[4], cr = p[5], cv = p[6];
        real r = x[0], v = x[1], c_r = c[0], c_v = c[1];
        real pi = R_PI;
        real inv_tau = (real)1 / tau;
        real dr = r * v;
        dr = dr * (real)2;
        dr = dr + delta / (pi * tau);
        dx[0] = dr * inv_tau;
        real v2 = v * v, r2 = r * r;
        real k = pi * pi;
        k = k * tau;
        k = k * tau;
        real dv = v2 - r2 * k;
        if (sweep_form) {
            dv = dv + eta;
            dv = dv + p[4];
        } else {
            dv = dv + (eta + i_ext);
        }
        dv = dv + r * (j * tau);
        dv = dv + c_r * cr;
        dv = dv + c_v * cv;
        dx[1] = dv * inv_tau;
        break;
    }
    case M_RWW: {
        real a = p[0], b = p[1], d = p[2], gamma = p[3], tau_s = p[4], w = p[5], j_n = p[6];
        real s = x[0], c0 = c[0];
        real xx = s * (w * j_n);
        xx = xx + p[7];
        xx = xx + c0 * j_n;
        real ax_b = xx * a + (-b);
        real e = R_EXP(ax_b * (-d));
        real denom = (-e) + (real)1;
        real h = ax_b / denom;
        real t1 = (-s) * ((real)1 / tau_s);
        real t2 = ((-s) + (real)1) * h;
        t2 = t2 * gamma;
        dx[0] = t1 + t2;
        break;
    }
    case M_KURAMOTO: {
        dx[0] = c[0] + p[0];
        break;
    }
    case M_JR: {
        real A = p[0], B = p[1], a = p[2], b = p[3], v0 = p[4], nu_max = p[5], r = p[6], J = p[7];
        real a1 = p[8], a2 = p[9], a3 = p[10], a4 = p[11], mu = p[12];
        real y0 = x[0], y1 = x[1], y2 = x[2], y3 = x[3], y4 = x[4], y5 = x[5], c0 = c[0];
        real two_nu_max = (real)2 * nu_max;
        real sv[3];
        real args[3];
        args[0] = y1 - y2;
        args[1] = y0 * (a1 * J);
        args[2] = y0 * (a3 * J);
        for (int q = 0; q < 3; q++) {
            real arg = (-args[q]) + v0;
            arg = arg * r;
            real denom = R_EXP(arg) + (real)1;
            sv[q] = ((real)1 * two_nu_max) / denom;
        }
        dx[0] = y3;
        dx[1] = y4;
        dx[2] = y5;
        real d3 = sv[0] * (A * a);
        d3 = d3 - y3 * ((real)2 * a);
        d3 = d3 - y0 * (a * a);
        dx[3] = d3;
        real mt = sv[1] * (a2 * J);
        mt = mt + (sweep_form ? p[12] : mu);
        mt = mt + c0;
        real d4 = mt * (A * a);
        d4 = d4 - y4 * ((real)2 * a);
        d4 = d4 - y1 * (a * a);
        dx[4] = d4;
        real d5 = sv[2] * (a4 * J);
        d5 = d5 * (B * b);
        d5 = d5 - y5 * ((real)2 * b);
        d5 = d5 - y2 * (b * b);
        dx[5] = d5;
        break;
    }
    case M_WC: {
        real c_ee = p[0], c_ei = p[1], c_ie = p[2], c_ii = p[3];
        real tau_e = p[4], tau_i = p[5];
        tau_e = tau_e > (real)FLT_EPSILON ? tau_e : (real)FLT_EPSILON;
        tau_i = tau_i > (real)FLT_EPSILON ? tau_i : (real)FLT_EPSILON;
        real a_e = p[6], b_e = p[7], ce = p[8], theta_e = p[9];
        real a_i = p[10], b_i = p[11], ci = p[12], theta_i = p[13];
        real r_e = p[14], r_i = p[15], k_e = p[16], k_i = p[17];
        real q = p[19], alpha_e = p[20], alpha_i = p[21];
        real sig_e_off = (real)1 / ((real)1 + R_EXP(a_e * b_e));
        real sig_i_off = (real)1 / ((real)1 + R_EXP(a_i * b_i));
        real e = x[0], iv = x[1], c0 = c[0];
        real xe = e * c_ee - iv * c_ei;
        xe = xe - theta_e;
        xe = xe + c0;
        xe = xe + p[18];
        xe = xe * alpha_e;
        real xi = e * c_ie - iv * c_ii;
        xi = xi + q;
        xi = xi - theta_i;
        xi = xi * alpha_i;
        real ea = R_EXP((xe + (-b_e)) * (-a_e));
        real sig_e = (real)1 / (ea + (real)1);
        real s_e = (sig_e - sig_e_off) * ce;
        real ia = R_EXP((xi + (-b_i)) * (-a_i));
        real sig_i = (real)1 / (ia + (real)1);
        real s_i = (sig_i - sig_i_off) * ci;
        real de = (-e) + (e * (-r_e) + k_e) * s_e;
        dx[0] = de * ((real)1 / tau_e);
        real di = (-iv) + (iv * (-r_i) + k_i) * s_i;
        dx[1] = di * ((real)1 / tau_i);
        (void)sweep_form;
        break;
    }
    }
}

/* clamp_batch (dfun.rs:170-239) for the six hot-path models */
static void clamp_node(int model, real* x) {
    switch (model) {
    case M_WC:
        for (int v = 0; v < 2; v++) { real t = x[v]; t = t < (real)1 ? t : (real)1; x[v] = t > (real)0 ? t : (real)0; }
        break;
    case M_MPR:
        x[0] = x[0] > (real)0 ? x[0] : (real)0;
        break;
    case M_RWW: { real t = x[0]; t = t < (real)1 ? t : (real)1; x[0] = t > (real)0 ? t : (real)0; break; }
    case M_KURAMOTO: {
        real two_pi = (real)2 * R_PI;
        x[0] = x[0] - R_FLOOR(x[0] / two_pi) * two_pi;
        break;
    }
    default: break;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* coupling functions: coupling.rs:52-202                                                     */
/* ------------------------------------------------------------------------------------------ */
enum { C_LINEAR = 0, C_SIGMOIDAL, C_DIFFERENCE, C_KURAMOTO, C_SCALED_LINEAR, C_TANH, C_SJR, C_PRESIG };

typedef struct {
    int kind;
    real a, b;                       /* Linear, ScaledLinear, Difference(a) */
    real cmin, cmax, midpoint, sigma; /* Sigmoidal / Tanh / SJR */
    int use_classic;                 /* SJR */
    real r, e0, v0;                  /* SJR */
    real h, q, g, p, theta;          /* PreSigmoidal */
    int dynamic, global_t;
    int n_src;                       /* Kuramoto normalisation */
    int has_rowsums;                 /* Difference non-square */
} ocfn;

static int cfn_parse(const char* name, const float* cp, int n, ocfn* f) {
    memset(f, 0, sizeof *f);
#define P(i, d) ((n) > (i) ? (real)cp[i] : (real)(d))
    if (name && strcmp(name, "Linear") == 0) { f->kind = C_LINEAR; f->a = P(0, 1.0); f->b = P(1, 0.0); }
    else if (name && strcmp(name, "Sigmoidal") == 0) {
        f->kind = C_SIGMOIDAL;
        if (n >= 5) { f->cmin = cp[0]; f->cmax = cp[1]; f->midpoint = cp[2]; f->a = cp[3]; f->sigma = cp[4]; }
        else { f->cmin = -1; f->cmax = P(0, 1.0); f->midpoint = P(1, 0.0); f->a = 1; f->sigma = P(2, 1.0); }
    } else if (name && strcmp(name, "Difference") == 0) { f->kind = C_DIFFERENCE; f->a = P(0, 1.0); }
    else if (name && strcmp(name, "Kuramoto") == 0) { f->kind = C_KURAMOTO; f->a = P(0, 1.0); f->n_src = 1; }
    else if (name && strcmp(name, "ScaledLinear") == 0) { f->kind = C_SCALED_LINEAR; f->a = P(0, 1.0); f->b = P(1, 0.0); }
    else if (name && strcmp(name, "HyperbolicTangent") == 0) {
        f->kind = C_TANH; f->a = P(0, 1.0); f->b = P(1, 1.0); f->midpoint = P(2, 0.0); f->sigma = P(3, 1.0);
    } else if (name && strcmp(name, "SigmoidalJansenRit") == 0) {
        f->kind = C_SJR;
        if (n >= 5) { f->a = cp[0]; f->use_classic = 1; f->cmin = cp[1]; f->cmax = cp[2]; f->r = cp[3]; f->midpoint = cp[4]; f->e0 = (real)0.005f; f->v0 = (real)6.0f; }
        else { f->a = P(0, 1.0); f->use_classic = 0; f->cmin = 0; f->cmax = (real)0.005f; f->r = P(2, 0.56f); f->midpoint = 6; f->e0 = P(1, 0.005f); f->v0 = P(3, 6.0); }
    } else if (name && strcmp(name, "PreSigmoidal") == 0) {
        f->kind = C_PRESIG; f->h = P(0, 1.0); f->q = P(1, 1.0); f->g = P(2, 1.0); f->p = P(3, 1.0); f->theta = P(4, 0.5);
        f->dynamic = (n > 5 && cp[5] != 0.0f); f->global_t = (n > 6 && cp[6] != 0.0f);
    } else {
        return 0;
    }
#undef P
    return 1;
}

/* CouplingFnConfig of a projection for given parameters, after the engine's construction-time
 * rewrites (engine.rs:277-283, 327-368) */
static void resolve_cfn(const char* name, const float* cp, int ncp, int diff_mode, int n_src, ocfn* f) {
    if (!cfn_parse(name, cp, ncp, f)) {
        /* engine.rs:277-279: unknown names fall back to Linear{a:1,b:0} */
        memset(f, 0, sizeof *f); f->kind = C_LINEAR; f->a = 1; f->b = 0;
    }
    if (f->kind == C_KURAMOTO) f->n_src = n_src;
    if (f->kind == C_DIFFERENCE) {
        real a = f->a;
        if (diff_mode == 1) { memset(f, 0, sizeof *f); f->kind = C_LINEAR; f->a = a; f->b = 0; }
        else if (diff_mode == 2) f->has_rowsums = 1;
    }
}

/* number of channels produced by pre() for `ncv` source coupling variables */
static int pre_channels(const ocfn* f, int ncv) {
    if (f->kind == C_KURAMOTO) return 2 * ncv;
    if (f->kind == C_SJR) return 1;
    if (f->kind == C_PRESIG && f->dynamic) return 1;
    return ncv;
}

/* pre() of one source row in the tensor form (coupling.rs:204-258) when cpu_form == 0, or the
 * per-edge CPU form (coupling.rs:268-321) when cpu_form == 1. */
static void pre_row(const ocfn* f, const real* x, int ncv, int cpu_form, real* out) {
    switch (f->kind) {
    case C_LINEAR: case C_SIGMOIDAL: case C_SCALED_LINEAR: case C_DIFFERENCE:
        for (int c = 0; c < ncv; c++) out[c] = x[c];
        break;
    case C_KURAMOTO:
        if (cpu_form) { for (int c = 0; c < ncv; c++) { out[2 * c] = R_SIN(x[c]); out[2 * c + 1] = R_COS(x[c]); } }
        else { for (int c = 0; c < ncv; c++) { out[c] = R_SIN(x[c]); out[ncv + c] = R_COS(x[c]); } }
        break;
    case C_TANH:
        for (int c = 0; c < ncv; c++) {
            if (cpu_form) { real inner = (x[c] * f->b - f->midpoint) / f->sigma; out[c] = f->a * ((real)1 + R_TANH(inner)); }
            else { real inner = (x[c] * f->b + (-f->midpoint)) / f->sigma; out[c] = (R_TANH(inner) + (real)1) * f->a; }
        }
        break;
    case C_SJR: {
        real x0 = x[0], x1 = ncv >= 2 ? x[1] : (real)0;
        real diff = x0 - x1;
        if (cpu_form) {
            if (f->use_classic) { real sh = (diff - f->midpoint) * (-f->r); real den = R_EXP(sh) + (real)1; out[0] = f->cmin + (f->cmax - f->cmin) / den; }
            else { real sh = (diff - f->v0) * (-f->r); real den = R_EXP(sh) + (real)1; out[0] = f->a * (real)2 * f->e0 / den; }
        } else {
            if (f->use_classic) { real sh = (diff + (-f->midpoint)) * (-f->r); real den = R_EXP(sh) + (real)1; out[0] = ((real)1 / den) * (f->cmax - f->cmin) + f->cmin; }
            else { real sh = (diff + (-f->v0)) * (-f->r); real den = R_EXP(sh) + (real)1; out[0] = ((real)1 / den) * ((f->a * (real)2) * f->e0); }
        }
        break;
    }
    case C_PRESIG:
        if (f->dynamic) {
            real x0 = x[0], x1 = ncv >= 2 ? x[1] : (real)0;
            real inner = cpu_form ? (f->p * x0 - x1) : (x0 * f->p - x1);
            out[0] = (R_TANH(inner * f->g) + f->q) * f->h;
        } else {
            for (int c = 0; c < ncv; c++) {
                real inner = cpu_form ? (f->p * x[c] - f->theta) : (x[c] * f->p + (-f->theta));
                out[c] = (R_TANH(inner * f->g) + f->q) * f->h;
            }
        }
        break;
    }
}

/* post_with_target (coupling.rs:323-399, engine.rs:621-633) of one target row; returns the
 * number of output channels. */
static int post_row(const ocfn* f, const real* gx, int pc, const real* xi, int tgt_ncv, real rowsum, real* out) {
    switch (f->kind) {
    case C_LINEAR:
        for (int c = 0; c < pc; c++) out[c] = gx[c] * f->a + f->b;
        return pc;
    case C_SIGMOIDAL:
        for (int c = 0; c < pc; c++) {
            real sh = (gx[c] + (-f->midpoint)) / f->sigma;
            real ex = -(sh * f->a);
            real den = R_EXP(ex) + (real)1;
            out[c] = ((real)1 / den) * (f->cmax - f->cmin) + f->cmin;
        }
        return pc;
    case C_SCALED_LINEAR:
        for (int c = 0; c < pc; c++) out[c] = (gx[c] + (-f->b)) * f->a;
        return pc;
    case C_DIFFERENCE:
        if (f->has_rowsums) { for (int c = 0; c < pc; c++) out[c] = (gx[c] - xi[c] * rowsum) * f->a; }
        else { for (int c = 0; c < pc; c++) out[c] = gx[c] * f->a; }
        return pc;
    case C_KURAMOTO: {
        real s = f->a / (real)f->n_src;
        for (int c = 0; c < tgt_ncv; c++) {
            real t = R_COS(xi[c]) * gx[c] - R_SIN(xi[c]) * gx[tgt_ncv + c];
            out[c] = t * s;
        }
        return tgt_ncv;
    }
    case C_SJR:
        if (f->use_classic) { for (int c = 0; c < pc; c++) out[c] = gx[c] * f->a; }
        else { for (int c = 0; c < pc; c++) out[c] = gx[c]; }
        return pc;
    default:
        for (int c = 0; c < pc; c++) out[c] = gx[c];
        return pc;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Balloon-Windkessel: bold.rs:22-166, bold_monitor.rs:49-227                                 */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
    int nnodes, bold_period;
    double tr, dt_neural;
    float *s, *f, *v, *q;   /* BW state is f32 in the reference (bold.rs:11-20) */
    float* acc;
    int count;
    double* times; int64_t n_times, cap_times;
    float* data; int64_t n_data, cap_data;
} obold;

static void bold_init(obold* m, int nnodes, int period, double tr, double dt) {
    memset(m, 0, sizeof *m);
    m->nnodes = nnodes; m->bold_period = period < 1 ? 1 : period; m->tr = tr; m->dt_neural = dt;
    m->s = calloc(nnodes, 4); m->f = malloc(nnodes * 4); m->v = malloc(nnodes * 4); m->q = malloc(nnodes * 4);
    m->acc = calloc(nnodes, 4);
    for (int i = 0; i < nnodes; i++) { m->f[i] = 1.0f; m->v[i] = 1.0f; m->q[i] = 1.0f; }
}
static void bold_free(obold* m) {
    free(m->s); free(m->f); free(m->v); free(m->q); free(m->acc); free(m->times); free(m->data);
    memset(m, 0, sizeof *m);
}

/* BoldModel::step (bold.rs:106-150): forward Euler with the default parameters */
static void bw_step(float* s_, float* f_, float* v_, float* q_, int n, const float* input, double dt) {
    float dt_f = (float)dt;
    const float tau_s = 1.54f, tau_f = 0.50f, tau_0 = 1.02f, alpha = 0.32f, e0 = 0.34f;
    float kappa = 1.0f / tau_s, gamma = 1.0f / tau_f, tau_inv = 1.0f / tau_0;
    for (int i = 0; i < n; i++) {
        float z = input[i] > 0.0f ? input[i] : 0.0f;
        float s = s_[i], f = f_[i], v = v_[i], q = q_[i];
        float fs = f > 1e-6f ? f : 1e-6f;
        float vs = v > 1e-6f ? v : 1e-6f;
        float ds = z - kappa * s - gamma * (fs - 1.0f);
        float df = s;
        float va = powf(vs, 1.0f / alpha);
        float dv = tau_inv * (fs - va);
        float dq = tau_inv * (fs * (1.0f - powf(1.0f - e0, 1.0f / fs)) / e0 - powf(vs, 1.0f / alpha) * (q / vs));
        float sn = s + dt_f * ds, fn = fs + dt_f * df, vn = vs + dt_f * dv, qn = q + dt_f * dq;
        s_[i] = sn > 0.0f ? sn : 0.0f;
        f_[i] = fn > 1e-6f ? fn : 1e-6f;
        v_[i] = vn > 1e-6f ? vn : 1e-6f;
        q_[i] = qn > 0.0f ? qn : 0.0f;
    }
}

/* BoldModel::signal (bold.rs:153-166) */
static void bw_signal(const float* v_, const float* q_, int n, float* out) {
    const float v0 = 4.0f, k1 = 7.0f, k2 = 2.0f, k3 = 2.0f;
    for (int i = 0; i < n; i++) {
        float v = v_[i] > 1e-6f ? v_[i] : 1e-6f;
        float q = q_[i];
        out[i] = v0 * (k1 * (1.0f - q) + k2 * (1.0f - q / v) + k3 * (1.0f - v));
    }
}

static void bold_push_sample(obold* m, double t) {
    if (m->n_times == m->cap_times) { m->cap_times = m->cap_times ? 2 * m->cap_times : 64; m->times = realloc(m->times, m->cap_times * sizeof(double)); }
    m->times[m->n_times++] = t;
    if (m->n_data + m->nnodes > m->cap_data) { m->cap_data = (m->cap_data + m->nnodes) * 2; m->data = realloc(m->data, m->cap_data * sizeof(float)); }
    bw_signal(m->v, m->q, m->nnodes, m->data + m->n_data);
    m->n_data += m->nnodes;
}

/* BoldMonitor::accumulate (bold_monitor.rs:72-107) */
static void bold_accumulate(obold* m, const float* input) {
    for (int i = 0; i < m->nnodes; i++) m->acc[i] += input[i];
    m->count += 1;
    if (m->count >= m->bold_period) {
        float* avg = malloc((size_t)m->nnodes * sizeof(float));
        for (int i = 0; i < m->nnodes; i++) avg[i] = m->acc[i] / (float)m->count;
        double dt_bold = m->dt_neural * (double)m->count;
        bw_step(m->s, m->f, m->v, m->q, m->nnodes, avg, dt_bold / 1000.0);
        double t = (double)m->n_times * dt_bold + dt_bold;
        bold_push_sample(m, t);
        memset(m->acc, 0, m->nnodes * 4);
        m->count = 0;
        free(avg);
    }
}

/* BoldMonitor::downsample_to_tr (bold_monitor.rs:123-203); returns number of output rows */
static int64_t bold_downsample(const obold* m, float** out) {
    int n = m->nnodes;
    *out = NULL;
    if (m->n_times == 0) return 0;
    double dt_bold = m->dt_neural * (double)m->bold_period;
    double tr_ms = m->tr * 1000.0;
    if (tr_ms <= 0.0 || fabs(tr_ms - dt_bold) < 1e-6) {
        *out = malloc(m->n_data * sizeof(float));
        memcpy(*out, m->data, m->n_data * sizeof(float));
        return m->n_times;
    }
    double max_t = m->times[m->n_times - 1];
    int64_t n_out = max_t >= tr_ms ? (int64_t)floor(max_t / tr_ms) : 0;
    float* o = malloc((size_t)(n_out * n + 1) * sizeof(float));
    int64_t ns = m->n_times;
    for (int64_t j = 0; j < n_out; j++) {
        double tt = (double)(j + 1) * tr_ms;
        float* row = o + j * n;
        if (tt <= m->times[0]) { for (int i = 0; i < n; i++) row[i] = m->data[i]; continue; }
        int64_t idx = 0;
        for (int64_t k = 1; k < ns; k++) {
            if (m->times[k] > tt) { idx = k - 1; break; }
            idx = k;
        }
        if (idx + 1 >= ns) { for (int i = 0; i < n; i++) row[i] = m->data[idx * n + i]; continue; }
        double t0 = m->times[idx], t1 = m->times[idx + 1];
        double w = fabs(t1 - t0) < 1e-12 ? 0.0 : (tt - t0) / (t1 - t0);
        if (w < 0.0) w = 0.0;
        if (w > 1.0) w = 1.0;
        for (int i = 0; i < n; i++) {
            float a = m->data[idx * n + i], b = m->data[(idx + 1) * n + i];
            row[i] = a + (b - a) * (float)w;
        }
    }
    *out = o;
    return n_out;
}

/* BoldMonitor::flush (bold_monitor.rs:207-227) */
static int64_t bold_flush(obold* m, float** out) {
    if (m->count > 0) {
        float* avg = malloc((size_t)m->nnodes * sizeof(float));
        for (int i = 0; i < m->nnodes; i++) avg[i] = m->acc[i] / (float)m->count;
        double dt_bold = m->dt_neural * (double)m->count;
        bw_step(m->s, m->f, m->v, m->q, m->nnodes, avg, dt_bold / 1000.0);
        double t = (double)m->n_times * (m->dt_neural * (double)m->bold_period) + dt_bold;
        bold_push_sample(m, t);
        memset(m->acc, 0, m->nnodes * 4);
        m->count = 0;
        free(avg);
    }
    return bold_downsample(m, out);
}

/* ------------------------------------------------------------------------------------------ */
/* engine                                                                                     */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
    int model, nnodes, nmodes, nm, nvar, ncvar;
    float params[32];
    int nparams;
    float* x0; /* [nm*nvar] */
    float* node_params;  /* extension of this engine: [nm][nparams] or [B][nm][nparams] rows per node, or NULL */
    int node_pp;         /* node_params holds one table per sweep point */
} osub;

enum { W_MEAN = 0, W_DIAG, W_DENSE, W_CSR };

typedef struct {
    int src, tgt;
    int wkind;
    real w;                     /* MEAN / DIAG */
    real* dense;                /* W_DENSE: [ntgt][nsrc] */
    int nnz;
    real* csr_w; int* csr_idx; int* csr_ptr; uint32_t* edelay;
    int per_edge;
    uint32_t delay;
    ocfn cf;
    char cf_name[32];
    float cf_params[16];
    int n_cf_params;
    int diff_mode;              /* 0: none, 1: Difference became Linear{a,0}, 2: Difference with rowsums */
    real* rowsums;              /* [ntgt] when cf.has_rowsums */
    int direct;
    int ncm; int cm_s[8]; int cm_cpl[8];
} oproj;

typedef struct {
    int nsub, nproj, nbold;
    osub sub[16];
    oproj* proj;
    hb_bold_desc bold_cfg[8];
    double dt_ms;
    real dt;
    int integrator;
    uint32_t flags;
    float nsig[16]; int n_nsig;
    int n_sweep;
    int horizon;               /* batch: 0 if no delay else max+1; ring: max+1 */
    /* dynamic */
    real* x[16];               /* [B][nm][nvar] */
    real* hist[16];            /* [B][nm][nvar][H] */
    int64_t step;
    obold* monitors;           /* batch-mean: nbold monitors; per point: nbold*B */
    int n_monitors;
    /* last result */
    float* r_tavg[16]; float* r_final[16]; float* r_traj[16]; int64_t r_traj_len[16];
    float* r_bold[8]; int64_t r_bold_len[8];
    float* r_params; int64_t r_params_len;
    int r_nbold;
} oengine;

typedef struct {
    int mode;                 /* 0 none, 1 native sweep form, 2 per-point params */
    real* pp;                 /* [B][nparams] */
    char swept[32];           /* parameters that pp overrides (they override per-node rows too) */
} osweep;

/* per-point coupling functions of swept projections (an extension: the reference cannot sweep
 * coupling parameters, cli.rs:976-998) */
typedef struct {
    ocfn* cf[64];             /* [proj] -> [B] or NULL */
} ocsweep;

static int parse_cvar_map(const char* s, int* ps, int* pt, int maxn) {
    int n = 0;
    if (!s) s = "0:0";
    const char* c = s;
    while (*c && n < maxn) {
        const char* e = strchr(c, ',');
        size_t len = e ? (size_t)(e - c) : strlen(c);
        char buf[64];
        if (len >= sizeof buf) len = sizeof buf - 1;
        memcpy(buf, c, len); buf[len] = 0;
        /* trim */
        char* b = buf; while (*b == ' ' || *b == '\t') b++;
        char* z = b + strlen(b); while (z > b && (z[-1] == ' ' || z[-1] == '\t')) *--z = 0;
        if (*b) {
            char* colon = strchr(b, ':');
            int a = 0, t = 0;
            if (colon && !strchr(colon + 1, ':')) {
                char* endp;
                *colon = 0;
                long v1 = strtol(b, &endp, 10); if (*endp || endp == b || v1 < 0) v1 = 0;
                long v2 = strtol(colon + 1, &endp, 10); if (*endp || endp == colon + 1 || v2 < 0) v2 = 0;
                a = (int)v1; t = (int)v2;
            }
            ps[n] = a; pt[n] = t; n++;
        }
        if (!e) break;
        c = e + 1;
    }
    return n;
}

EXPORT void HBO(engine_destroy)(oengine* e);
EXPORT void HBO(engine_reset)(oengine* e);

EXPORT oengine* HBO(engine_create)(const hb_sim_desc* d, int32_t n_sweep, int32_t* status) {
    *status = HB_OK;
    if (!d || n_sweep < 1 || d->n_subnets < 1 || d->n_subnets > 16 || d->n_bold > 8) {
        set_err("invalid descriptor"); *status = HB_ERR_INVALID_CONFIG; return NULL;
    }
    oengine* e = calloc(1, sizeof *e);
    e->nsub = d->n_subnets; e->nproj = d->n_projections; e->dt_ms = d->dt; e->dt = (real)(float)d->dt;
    e->integrator = d->integrator; e->flags = d->flags; e->n_sweep = n_sweep;
    e->n_nsig = d->n_nsig > 16 ? 16 : d->n_nsig;
    for (int i = 0; i < e->n_nsig; i++) e->nsig[i] = d->nsig[i];
    int ring = (d->flags & HB_SEM_DELAY_RING) != 0;
    for (int i = 0; i < e->nsub; i++) {
        const hb_subnet_desc* s = &d->subnets[i];
        osub* o = &e->sub[i];
        o->model = model_from_name(s->model);
        if (o->model < 0) { set_err("Unknown model: %s", s->model ? s->model : "(null)"); *status = HB_ERR_INVALID_CONFIG; HBO(engine_destroy)(e); return NULL; }
        o->nnodes = s->nnodes; o->nmodes = s->nmodes; o->nm = s->nnodes * s->nmodes;
        o->nvar = k_nvar[o->model]; o->ncvar = k_ncvar[o->model];
        o->nparams = s->n_params;
        if (s->n_params < k_nparams[o->model] || s->n_params > 32) { set_err("subnetwork %d: model expects %d params, got %d", i, k_nparams[o->model], s->n_params); *status = HB_ERR_INVALID_CONFIG; HBO(engine_destroy)(e); return NULL; }
        for (int k = 0; k < s->n_params; k++) o->params[k] = s->params[k];
        if (s->n_initial_state != (int64_t)o->nm * o->nvar) { set_err("subnetwork %d: initial state has %lld values, expected %d", i, (long long)s->n_initial_state, o->nm * o->nvar); *status = HB_ERR_INVALID_CONFIG; HBO(engine_destroy)(e); return NULL; }
        o->x0 = malloc(sizeof(float) * o->nm * o->nvar);
        memcpy(o->x0, s->initial_state, sizeof(float) * o->nm * o->nvar);
        if (s->n_node_params > 0) {
            int64_t per = (int64_t)o->nm * s->n_params;
            if (!s->node_params || (s->n_node_params != per && s->n_node_params != per * n_sweep)) {
                set_err("subnetwork %d: node_params has %lld values", i, (long long)s->n_node_params);
                *status = HB_ERR_INVALID_CONFIG; HBO(engine_destroy)(e); return NULL;
            }
            o->node_params = malloc(sizeof(float) * (size_t)s->n_node_params);
            memcpy(o->node_params, s->node_params, sizeof(float) * (size_t)s->n_node_params);
            o->node_pp = s->n_node_params != per || n_sweep == 1;
        }
    }
    /* horizon: engine.rs:253-257 (batch) / construction.rs:596-601 (ring) */
    int max_delay = 0;
    for (int p = 0; p < d->n_projections; p++)
        for (int64_t k = 0; k < d->projections[p].n_delays; k++)
            if ((int)d->projections[p].delays[k] > max_delay) max_delay = (int)d->projections[p].delays[k];
    e->horizon = ring ? max_delay + 1 : (max_delay == 0 ? 0 : max_delay + 1);

    e->proj = calloc(d->n_projections > 0 ? d->n_projections : 1, sizeof(oproj));
    for (int p = 0; p < d->n_projections; p++) {
        const hb_projection_desc* pd = &d->projections[p];
        oproj* o = &e->proj[p];
        if (pd->src < 0 || pd->src >= e->nsub || pd->tgt < 0 || pd->tgt >= e->nsub) { set_err("projection %d: bad src/tgt", p); *status = HB_ERR_INVALID_CONFIG; HBO(engine_destroy)(e); return NULL; }
        o->src = pd->src; o->tgt = pd->tgt;
        int nsrc = e->sub[o->src].nm, ntgt = e->sub[o->tgt].nm;
        snprintf(o->cf_name, sizeof o->cf_name, "%s", pd->coupling_fn ? pd->coupling_fn : "Linear");
        o->n_cf_params = pd->n_coupling_params > 16 ? 16 : pd->n_coupling_params;
        for (int k = 0; k < o->n_cf_params; k++) o->cf_params[k] = pd->coupling_params[k];
        resolve_cfn(o->cf_name, o->cf_params, o->n_cf_params, 0, nsrc, &o->cf);
        o->delay = pd->n_delays > 0 ? pd->delays[0] : 0;
        if (pd->weights_kind == HB_WEIGHTS_SCALAR) {
            o->wkind = (d->flags & HB_SEM_SCALAR_DIAGONAL) ? W_DIAG : W_MEAN;
            o->w = pd->scalar_weight;
        } else if (pd->weights_kind == HB_WEIGHTS_DENSE) {
            o->wkind = W_DENSE;
            o->dense = malloc(sizeof(real) * (size_t)ntgt * nsrc);
            for (int64_t k = 0; k < (int64_t)ntgt * nsrc; k++) o->dense[k] = pd->dense[k];
        } else {
            /* CSR: the batch engine densifies (engine.rs:298-322); the ring mode keeps the serial
             * engine's CSR path (runtime.rs:103-211) */
            if (!ring) {
                o->wkind = W_DENSE;
                o->dense = calloc((size_t)ntgt * nsrc, sizeof(real));
                for (int t = 0; t < ntgt; t++)
                    for (uint32_t k = pd->csr_indptr[t]; k < pd->csr_indptr[t + 1]; k++)
                        o->dense[(size_t)t * nsrc + pd->csr_indices[k]] = pd->csr_data[k];
            } else {
                o->wkind = W_CSR;
                o->nnz = (int)pd->nnz;
                o->csr_w = malloc(sizeof(real) * (o->nnz + 1));
                o->csr_idx = malloc(sizeof(int) * (o->nnz + 1));
                o->csr_ptr = malloc(sizeof(int) * (ntgt + 1));
                for (int k = 0; k < o->nnz; k++) { o->csr_w[k] = pd->csr_data[k]; o->csr_idx[k] = (int)pd->csr_indices[k]; }
                for (int t = 0; t <= ntgt; t++) o->csr_ptr[t] = (int)pd->csr_indptr[t];
                o->per_edge = (pd->n_delays == pd->nnz && pd->nnz > 0);
                if (o->per_edge) { o->edelay = malloc(sizeof(uint32_t) * o->nnz); memcpy(o->edelay, pd->delays, sizeof(uint32_t) * o->nnz); }
            }
        }
        /* Difference preprocessing: engine.rs:327-368 (batch) / construction.rs:700-730 (serial) */
        if (o->cf.kind == C_DIFFERENCE) {
            if (o->wkind == W_MEAN || o->wkind == W_DIAG) {
                o->w = 0; o->diff_mode = 1;
            } else if (o->wkind == W_DENSE) {
                if (ntgt == nsrc) {
                    for (int i = 0; i < ntgt; i++) {
                        real rs = 0;
                        for (int j = 0; j < nsrc; j++) rs = rs + o->dense[(size_t)i * nsrc + j];
                        o->dense[(size_t)i * nsrc + i] -= rs;
                    }
                    o->diff_mode = 1;
                } else {
                    o->rowsums = malloc(sizeof(real) * ntgt);
                    for (int i = 0; i < ntgt; i++) {
                        real rs = 0;
                        for (int j = 0; j < nsrc; j++) rs = rs + o->dense[(size_t)i * nsrc + j];
                        o->rowsums[i] = rs;
                    }
                    o->diff_mode = 2;
                }
            } else {
                /* serial engine: the preprocessing touches a zero placeholder matrix, so CSR
                 * Difference acts as Linear{a, b: 0} on the raw CSR weights */
                o->diff_mode = 1;
            }
            resolve_cfn(o->cf_name, o->cf_params, o->n_cf_params, o->diff_mode, nsrc, &o->cf);
        }
        /* cvar map: engine.rs:370-392, 637-664 */
        int cs[8], ct[8];
        o->ncm = parse_cvar_map(pd->cvar_map, cs, ct, 8);
        int src_ncvar = e->sub[o->src].ncvar, tgt_ncvar = e->sub[o->tgt].ncvar;
        for (int k = 0; k < o->ncm; k++) {
            if (cs[k] >= src_ncvar) { set_err("Projection %d cvar_map src index %d >= src_ncvar %d", p, cs[k], src_ncvar); *status = HB_ERR_INVALID_CONFIG; HBO(engine_destroy)(e); return NULL; }
            if (ct[k] >= tgt_ncvar) { set_err("Projection %d cvar_map tgt index %d >= tgt_ncvar %d", p, ct[k], tgt_ncvar); *status = HB_ERR_INVALID_CONFIG; HBO(engine_destroy)(e); return NULL; }
            o->cm_s[k] = cs[k];
            o->cm_cpl[k] = cvar_position(e->sub[o->tgt].model, ct[k]);
        }
        o->direct = (tgt_ncvar == src_ncvar && o->ncm == 1 && cs[0] == 0 && ct[0] == 0);
        if (o->cf.kind == C_PRESIG && o->cf.global_t) { set_err("PreSigmoidal global_t is not supported"); *status = HB_ERR_UNSUPPORTED; HBO(engine_destroy)(e); return NULL; }
        if (o->cf.kind == C_PRESIG && o->cf.dynamic && src_ncvar < 2) { set_err("PreSigmoidal dynamic needs two source cvars"); *status = HB_ERR_UNSUPPORTED; HBO(engine_destroy)(e); return NULL; }
    }
    e->nbold = d->n_bold;
    for (int m = 0; m < d->n_bold; m++) e->bold_cfg[m] = d->bold[m];
    /* dynamic state */
    for (int i = 0; i < e->nsub; i++) {
        osub* o = &e->sub[i];
        e->x[i] = malloc(sizeof(real) * (size_t)n_sweep * o->nm * o->nvar);
        if (e->horizon > 0) e->hist[i] = calloc((size_t)n_sweep * o->nm * o->nvar * e->horizon, sizeof(real));
    }
    HBO(engine_reset)(e);
    return e;
}

EXPORT void HBO(engine_reset)(oengine* e) {
    int B = e->n_sweep, H = e->horizon;
    for (int i = 0; i < e->nsub; i++) {
        osub* o = &e->sub[i];
        int per = o->nm * o->nvar;
        for (int b = 0; b < B; b++)
            for (int k = 0; k < per; k++) e->x[i][(size_t)b * per + k] = o->x0[k];
        if (H > 0) {
            memset(e->hist[i], 0, sizeof(real) * (size_t)B * per * H);
            for (int b = 0; b < B; b++)
                for (int k = 0; k < per; k++) e->hist[i][((size_t)b * per + k) * H + 0] = o->x0[k];
        }
    }
    e->step = 0;
    if (e->monitors) { for (int m = 0; m < e->n_monitors; m++) bold_free(&e->monitors[m]); free(e->monitors); }
    e->monitors = NULL; e->n_monitors = 0;
    if (e->nbold > 0) {
        int per_point = (e->flags & HB_SEM_BOLD_PER_POINT) != 0;
        e->n_monitors = per_point ? e->nbold * B : e->nbold;
        e->monitors = calloc(e->n_monitors, sizeof(obold));
        for (int m = 0; m < e->n_monitors; m++) {
            const hb_bold_desc* bc = &e->bold_cfg[per_point ? m / B : m];
            bold_init(&e->monitors[m], e->sub[0].nnodes, bc->bold_period, bc->tr, e->dt_ms);
        }
    }
}

static void free_results(oengine* e) {
    for (int i = 0; i < 16; i++) { free(e->r_tavg[i]); free(e->r_final[i]); free(e->r_traj[i]); e->r_tavg[i] = e->r_final[i] = e->r_traj[i] = NULL; e->r_traj_len[i] = 0; }
    for (int m = 0; m < 8; m++) { free(e->r_bold[m]); e->r_bold[m] = NULL; e->r_bold_len[m] = 0; }
    free(e->r_params); e->r_params = NULL; e->r_params_len = 0; e->r_nbold = 0;
}

EXPORT void HBO(engine_destroy)(oengine* e) {
    if (!e) return;
    for (int i = 0; i < e->nsub; i++) { free(e->sub[i].x0); free(e->sub[i].node_params); free(e->x[i]); free(e->hist[i]); }
    for (int p = 0; p < e->nproj && e->proj; p++) {
        oproj* o = &e->proj[p];
        free(o->dense); free(o->csr_w); free(o->csr_idx); free(o->csr_ptr); free(o->edelay); free(o->rowsums);
    }
    free(e->proj);
    if (e->monitors) { for (int m = 0; m < e->n_monitors; m++) bold_free(&e->monitors[m]); free(e->monitors); }
    free_results(e);
    free(e);
}

/* effective integrator of a subnetwork: engine.rs:697-771 */
enum { I_HEUN_DET = 100 };
static int effective_integrator(const oengine* e, int model) {
    int use_heun = (e->flags & HB_SEM_HYBRID_INTEGRATOR) ? (model == M_G2DO) : (e->integrator == HB_INT_HEUN);
    if (use_heun) return I_HEUN_DET;
    if (e->integrator == HB_INT_HEUN) return HB_INT_EULER; /* `_ =>` arm */
    return e->integrator;
}

typedef struct {
    real* gx; real* pre; real* cv; real* out; real* cpl[16];
    real* k1; real* k2; real* k3; real* k4; real* tmp; real* noise;
} oscratch;

/* couplings of all subnetworks for point b at the current step (engine.rs:554-674, ring mode:
 * runtime.rs:88-211) */
static void compute_couplings(const oengine* e, int b, const ocsweep* cs, oscratch* sc) {
    int B = e->n_sweep, H = e->horizon;
    int ring = (e->flags & HB_SEM_DELAY_RING) != 0;
    int64_t step = e->step;
    for (int i = 0; i < e->nsub; i++) memset(sc->cpl[i], 0, sizeof(real) * e->sub[i].nm * e->sub[i].ncvar);
    (void)B;
    for (int p = 0; p < e->nproj; p++) {
        const oproj* o = &e->proj[p];
        const ocfn* cf = (cs && cs->cf[p]) ? &cs->cf[p][b] : &o->cf;
        const osub* S = &e->sub[o->src];
        const osub* T = &e->sub[o->tgt];
        int nsrc = S->nm, ntgt = T->nm;
        int ncv = S->ncvar < S->nvar ? S->ncvar : S->nvar;
        int pc = pre_channels(cf, ncv);
        const real* xs = e->x[o->src] + (size_t)b * S->nm * S->nvar;
        const real* xt = e->x[o->tgt] + (size_t)b * T->nm * T->nvar;
        const real* hs = H > 0 ? e->hist[o->src] + (size_t)b * S->nm * S->nvar * H : NULL;
        real* gx = sc->gx;
        memset(gx, 0, sizeof(real) * ntgt * pc);
        if (o->wkind == W_CSR && o->per_edge) {
            /* runtime.rs:162-204: per-edge ring reads, zero rows after pre() */
            real row[8], pv[16];
            for (int t = 0; t < ntgt; t++) {
                for (int k = o->csr_ptr[t]; k < o->csr_ptr[t + 1]; k++) {
                    int s = o->csr_idx[k];
                    uint32_t dl = o->edelay[k];
                    if (dl == 0 || step == 0) {
                        for (int c = 0; c < ncv; c++) row[c] = xs[s * S->nvar + c];
                        pre_row(cf, row, ncv, 1, pv);
                    } else if ((int64_t)dl > step) {
                        for (int c = 0; c < pc; c++) pv[c] = 0;
                    } else {
                        int slot = (int)((step - dl + H) % H);
                        for (int c = 0; c < ncv; c++) row[c] = hs[((size_t)s * S->nvar + c) * H + slot];
                        pre_row(cf, row, ncv, 1, pv);
                    }
                    real wk = o->csr_w[k];
                    for (int c = 0; c < pc; c++) gx[t * pc + c] += wk * pv[c];
                }
            }
        } else {
            /* delayed cvar rows of all source nodes, then pre() (tensor form) */
            real* cv = sc->cv;
            uint32_t dl = o->delay;
            for (int s = 0; s < nsrc; s++) {
                for (int c = 0; c < ncv; c++) {
                    real v;
                    if (dl == 0 || step == 0) v = xs[s * S->nvar + c];
                    else if ((int64_t)dl <= step) {
                        int slot = ring ? (int)((step - dl) % H) : (int)((step - dl + H) % H);
                        v = hs[((size_t)s * S->nvar + c) * H + slot];
                    } else v = 0;
                    cv[s * ncv + c] = v;
                }
            }
            real* pre = sc->pre;
            for (int s = 0; s < nsrc; s++) pre_row(cf, cv + s * ncv, ncv, 0, pre + s * pc);
            if (o->wkind == W_MEAN) {
                /* mean_dim(1) * weight, broadcast over target nodes (engine.rs:602-608) */
                real m[16];
                for (int c = 0; c < pc; c++) {
                    real acc = 0;
                    for (int s = 0; s < nsrc; s++) acc = acc + pre[s * pc + c];
                    m[c] = (acc / (real)nsrc) * o->w;
                }
                for (int t = 0; t < ntgt; t++) for (int c = 0; c < pc; c++) gx[t * pc + c] = m[c];
            } else if (o->wkind == W_DIAG) {
                for (int t = 0; t < ntgt; t++) for (int c = 0; c < pc; c++) gx[t * pc + c] = o->w * pre[t * pc + c];
            } else if (o->wkind == W_DENSE) {
                for (int t = 0; t < ntgt; t++)
                    for (int c = 0; c < pc; c++) {
                        real acc = 0;
                        for (int s = 0; s < nsrc; s++) acc = acc + o->dense[(size_t)t * nsrc + s] * pre[s * pc + c];
                        gx[t * pc + c] = acc;
                    }
            } else {
                /* sparse_csr_matvec (sparse.rs:29-52) */
                for (int t = 0; t < ntgt; t++)
                    for (int c = 0; c < pc; c++) {
                        real acc = 0;
                        for (int k = o->csr_ptr[t]; k < o->csr_ptr[t + 1]; k++) acc = acc + o->csr_w[k] * pre[o->csr_idx[k] * pc + c];
                        gx[t * pc + c] = acc;
                    }
            }
        }
        /* post_with_target + remap + accumulate */
        real out[16], xi[8];
        int tgt_ncv = T->ncvar;
        real* cp = sc->cpl[o->tgt];
        for (int t = 0; t < ntgt; t++) {
            for (int c = 0; c < tgt_ncv && c < T->nvar; c++) xi[c] = xt[t * T->nvar + c];
            real rs = cf->has_rowsums ? o->rowsums[t] : 0;
            int oc = post_row(cf, gx + t * pc, pc, xi, tgt_ncv, rs, out);
            if (o->direct) {
                for (int c = 0; c < tgt_ncv && c < oc; c++) cp[t * tgt_ncv + c] = cp[t * tgt_ncv + c] + out[c];
            } else {
                real tmp[8] = {0};
                for (int k = 0; k < o->ncm; k++) {
                    int s = o->cm_s[k], cpl = o->cm_cpl[k];
                    if (s < S->ncvar && cpl < tgt_ncv) tmp[cpl] += out[s];
                }
                for (int c = 0; c < tgt_ncv; c++) cp[t * tgt_ncv + c] = cp[t * tgt_ncv + c] + tmp[c];
            }
        }
    }
}

static void dfun_sub(const oengine* e, int i, const osweep* sw, int b, const real* x, const real* cpl, real* dx) {
    const osub* S = &e->sub[i];
    real p[32];
    int sweep_form = 0;
    if (sw[i].mode == 0) { for (int k = 0; k < S->nparams; k++) p[k] = S->params[k]; }
    else { for (int k = 0; k < S->nparams; k++) p[k] = sw[i].pp[(size_t)b * S->nparams + k]; sweep_form = (sw[i].mode == 1); }
    if (!S->node_params) {
        for (int n = 0; n < S->nm; n++) dfun_node(S->model, p, sweep_form, x + n * S->nvar, cpl + n * S->ncvar, dx + n * S->nvar);
        return;
    }
    /* per-node rows (an extension: the reference has one row per subnetwork): the node's row, with the
     * swept parameters of point b taking their sweep values as above */
    real q[32];
    for (int n = 0; n < S->nm; n++) {
        const float* nr = S->node_params + ((size_t)(S->node_pp ? b : 0) * S->nm + n) * S->nparams;
        for (int k = 0; k < S->nparams; k++) q[k] = (sw[i].mode != 0 && sw[i].swept[k]) ? p[k] : (real)nr[k];
        dfun_node(S->model, q, sweep_form, x + n * S->nvar, cpl + n * S->ncvar, dx + n * S->nvar);
    }
}

static void clamp_sub(const osub* S, real* x) {
    for (int n = 0; n < S->nm; n++) clamp_node(S->model, x + n * S->nvar);
}

static int64_t noise_row(const oengine* e) {
    int64_t r = 0;
    for (int i = 0; i < e->nsub; i++) r += (int64_t)e->sub[i].nm * e->sub[i].nvar;
    return r;
}

/* integrate subnetwork i of point b (engine.rs:677-783) */
static void integrate_sub(const oengine* e, int i, const osweep* sw, int b, const real* cpl, const float* noise_t, oscratch* sc) {
    const osub* S = &e->sub[i];
    int per = S->nm * S->nvar;
    real* x = e->x[i] + (size_t)b * per;
    real dt = e->dt;
    real *k1 = sc->k1, *k2 = sc->k2, *k3 = sc->k3, *k4 = sc->k4, *tmp = sc->tmp, *nz = sc->noise;
    int integ = effective_integrator(e, S->model);
    int stoch = (integ == HB_INT_EULER_STOCHASTIC || integ == HB_INT_HEUN_STOCHASTIC || integ == HB_INT_RK4_STOCHASTIC);
    if (stoch) {
        /* generate_noise_reproducible scaling: raw * (sqrt(2*nsig[v]) * sqrt(dt)) */
        real sqrt_dt = R_SQRT(dt);
        for (int n = 0; n < S->nm; n++)
            for (int v = 0; v < S->nvar; v++) {
                real scale = R_SQRT((real)2 * (real)e->nsig[v]) * sqrt_dt;
                nz[n * S->nvar + v] = (real)noise_t[n * S->nvar + v] * scale;
            }
    }
    dfun_sub(e, i, sw, b, x, cpl, k1);
    switch (integ) {
    case I_HEUN_DET:
        for (int k = 0; k < per; k++) tmp[k] = x[k] + k1[k] * dt;
        clamp_sub(S, tmp);
        dfun_sub(e, i, sw, b, tmp, cpl, k2);
        for (int k = 0; k < per; k++) x[k] = x[k] + (k1[k] + k2[k]) * (dt * (real)0.5);
        break;
    case HB_INT_EULER:
        for (int k = 0; k < per; k++) x[k] = x[k] + k1[k] * dt;
        break;
    case HB_INT_EULER_STOCHASTIC:
        for (int k = 0; k < per; k++) x[k] = (x[k] + k1[k] * dt) + nz[k];
        break;
    case HB_INT_HEUN_STOCHASTIC:
        for (int k = 0; k < per; k++) tmp[k] = (x[k] + k1[k] * dt) + nz[k];
        clamp_sub(S, tmp);
        dfun_sub(e, i, sw, b, tmp, cpl, k2);
        for (int k = 0; k < per; k++) x[k] = (x[k] + (k1[k] + k2[k]) * (dt * (real)0.5)) + nz[k];
        break;
    case HB_INT_RK4:
    case HB_INT_RK4_STOCHASTIC: {
        real h2 = dt / (real)2, h6 = dt / (real)6;
        for (int k = 0; k < per; k++) tmp[k] = x[k] + k1[k] * h2;
        clamp_sub(S, tmp);
        dfun_sub(e, i, sw, b, tmp, cpl, k2);
        for (int k = 0; k < per; k++) tmp[k] = x[k] + k2[k] * h2;
        clamp_sub(S, tmp);
        dfun_sub(e, i, sw, b, tmp, cpl, k3);
        for (int k = 0; k < per; k++) tmp[k] = x[k] + k3[k] * dt;
        clamp_sub(S, tmp);
        dfun_sub(e, i, sw, b, tmp, cpl, k4);
        for (int k = 0; k < per; k++) {
            real s = k1[k] + k2[k] * (real)2;
            s = s + k3[k] * (real)2;
            s = s + k4[k];
            x[k] = x[k] + s * h6;
        }
        if (integ == HB_INT_RK4_STOCHASTIC) for (int k = 0; k < per; k++) x[k] = x[k] + nz[k];
        break;
    }
    }
    clamp_sub(S, x);
}

static int validate_run(oengine* e, const float* noise, int64_t noise_len, int64_t n_steps) {
    int integ = e->integrator;
    int stoch = (integ == HB_INT_EULER_STOCHASTIC || integ == HB_INT_HEUN_STOCHASTIC || integ == HB_INT_RK4_STOCHASTIC);
    if (stoch) {
        int64_t row = noise_row(e) * ((e->flags & HB_SEM_NOISE_PER_POINT) ? e->n_sweep : 1);
        if (!noise || noise_len < row * n_steps) { set_err("noise array too short: %lld < %lld", (long long)noise_len, (long long)(row * n_steps)); return HB_ERR_INVALID_STATE; }
        for (int i = 0; i < e->nsub; i++) if (e->sub[i].nvar > e->n_nsig) { set_err("nsig has %d entries, subnetwork %d has nvar %d", e->n_nsig, i, e->sub[i].nvar); return HB_ERR_INVALID_CONFIG; }
    }
    return HB_OK;
}

/* the step loop of run_sweep_internal (engine.rs:540-842) */
static int run_loop(oengine* e, const osweep* sw, const ocsweep* cs, int64_t n_steps, int record_traj, const float* noise, int n_threads) {
    int B = e->n_sweep, H = e->horizon;
    int ring = (e->flags & HB_SEM_DELAY_RING) != 0;
    int per_point_noise = (e->flags & HB_SEM_NOISE_PER_POINT) != 0;
    int per_point_bold = (e->flags & HB_SEM_BOLD_PER_POINT) != 0;
    int64_t nrow = noise_row(e);
    int64_t sub_off[17]; sub_off[0] = 0;
    for (int i = 0; i < e->nsub; i++) sub_off[i + 1] = sub_off[i] + (int64_t)e->sub[i].nm * e->sub[i].nvar;
    real* tavg[16];
    for (int i = 0; i < e->nsub; i++) {
        tavg[i] = calloc((size_t)B * e->sub[i].nm * e->sub[i].nvar, sizeof(real));
        if (record_traj) { e->r_traj_len[i] = n_steps * B * e->sub[i].nm * e->sub[i].nvar; e->r_traj[i] = malloc(sizeof(float) * (size_t)(e->r_traj_len[i] ? e->r_traj_len[i] : 1)); }
    }
    int maxn = 1, maxpc = 4;
    for (int i = 0; i < e->nsub; i++) if (e->sub[i].nm * e->sub[i].nvar > maxn) maxn = e->sub[i].nm * e->sub[i].nvar;
    int nb0 = e->sub[0].nnodes;
    float* bold_in = calloc((size_t)nb0 * (per_point_bold ? B : 1), sizeof(float));
    if (n_threads < 1) n_threads = 1;
#pragma omp parallel num_threads(n_threads)
    {
        oscratch sc;
        sc.gx = malloc(sizeof(real) * maxn * maxpc); sc.pre = malloc(sizeof(real) * maxn * maxpc);
        sc.cv = malloc(sizeof(real) * maxn * maxpc); sc.out = malloc(sizeof(real) * maxn * maxpc);
        for (int i = 0; i < e->nsub; i++) sc.cpl[i] = malloc(sizeof(real) * e->sub[i].nm * e->sub[i].ncvar);
        sc.k1 = malloc(sizeof(real) * maxn); sc.k2 = malloc(sizeof(real) * maxn); sc.k3 = malloc(sizeof(real) * maxn);
        sc.k4 = malloc(sizeof(real) * maxn); sc.tmp = malloc(sizeof(real) * maxn); sc.noise = malloc(sizeof(real) * maxn);
        for (int64_t t = 0; t < n_steps; t++) {
#pragma omp for schedule(static)
            for (int b = 0; b < B; b++) {
                /* 0. history (engine.rs:541-551 shift window; runtime.rs:55-85 ring slot) */
                if (H > 0) {
                    for (int i = 0; i < e->nsub; i++) {
                        const osub* S = &e->sub[i];
                        int per = S->nm * S->nvar;
                        real* hb = e->hist[i] + (size_t)b * per * H;
                        const real* xb = e->x[i] + (size_t)b * per;
                        if (ring) {
                            int slot = (int)(e->step % H);
                            for (int k = 0; k < per; k++) hb[(size_t)k * H + slot] = xb[k];
                        } else {
                            for (int k = 0; k < per; k++) {
                                memmove(hb + (size_t)k * H, hb + (size_t)k * H + 1, sizeof(real) * (H - 1));
                                hb[(size_t)k * H + H - 1] = xb[k];
                            }
                        }
                    }
                }
                /* 1. coupling */
                compute_couplings(e, b, cs, &sc);
                /* 2. integrate each subnetwork */
                for (int i = 0; i < e->nsub; i++) {
                    const float* nt = NULL;
                    if (noise) nt = noise + (per_point_noise ? (t * B + b) * nrow : t * nrow) + sub_off[i];
                    integrate_sub(e, i, sw, b, sc.cpl[i], nt, &sc);
                    const osub* S = &e->sub[i];
                    int per = S->nm * S->nvar;
                    real* xb = e->x[i] + (size_t)b * per;
                    real* ta = tavg[i] + (size_t)b * per;
                    for (int k = 0; k < per; k++) ta[k] = ta[k] + xb[k];
                    if (record_traj) {
                        float* tr = e->r_traj[i] + ((size_t)t * B + b) * per;
                        for (int k = 0; k < per; k++) tr[k] = (float)xb[k];
                    }
                }
            }
#pragma omp single
            {
                /* 3. BOLD input: var0 mean over modes and sweep points (engine.rs:786-801) */
                if (e->n_monitors > 0) {
                    const osub* S = &e->sub[0];
                    if (per_point_bold) {
                        for (int b = 0; b < B; b++)
                            for (int n = 0; n < S->nnodes; n++) {
                                real acc = 0;
                                for (int m = 0; m < S->nmodes; m++) acc = acc + e->x[0][((size_t)b * S->nm + n * S->nmodes + m) * S->nvar];
                                bold_in[b * nb0 + n] = (float)(acc / (real)S->nmodes);
                            }
                        for (int m = 0; m < e->n_monitors; m++) bold_accumulate(&e->monitors[m], bold_in + (m % B) * nb0);
                    } else {
                        for (int n = 0; n < S->nnodes; n++) {
                            real acc = 0;
                            for (int b = 0; b < B; b++) {
                                real am = 0;
                                for (int m = 0; m < S->nmodes; m++) am = am + e->x[0][((size_t)b * S->nm + n * S->nmodes + m) * S->nvar];
                                acc = acc + am / (real)S->nmodes;
                            }
                            bold_in[n] = (float)(acc / (real)B);
                        }
                        for (int m = 0; m < e->n_monitors; m++) bold_accumulate(&e->monitors[m], bold_in);
                    }
                }
                e->step += 1;
            }
        }
        free(sc.gx); free(sc.pre); free(sc.cv); free(sc.out);
        for (int i = 0; i < e->nsub; i++) free(sc.cpl[i]);
        free(sc.k1); free(sc.k2); free(sc.k3); free(sc.k4); free(sc.tmp); free(sc.noise);
    }
    free(bold_in);
    /* results: tavg * (1/n_steps) and final states (engine.rs:812-823) */
    real inv = (real)1 / (real)n_steps;
    for (int i = 0; i < e->nsub; i++) {
        int64_t len = (int64_t)B * e->sub[i].nm * e->sub[i].nvar;
        e->r_tavg[i] = malloc(sizeof(float) * len);
        e->r_final[i] = malloc(sizeof(float) * len);
        for (int64_t k = 0; k < len; k++) { e->r_tavg[i][k] = (float)(tavg[i][k] * inv); e->r_final[i][k] = (float)e->x[i][k]; }
        free(tavg[i]);
    }
    /* BOLD flush (bold_monitor.rs:207-227) */
    e->r_nbold = 0;
    if (e->n_monitors > 0) {
        if (per_point_bold) {
            for (int m = 0; m < e->nbold; m++) {
                float* parts[4096]; int64_t rows[4096]; int64_t tot = 0;
                int nb = B < 4096 ? B : 4096;
                for (int b = 0; b < nb; b++) { rows[b] = bold_flush(&e->monitors[m * B + b], &parts[b]); tot += rows[b] * nb0; }
                e->r_bold[m] = malloc(sizeof(float) * (tot ? tot : 1));
                int64_t off = 0;
                for (int b = 0; b < nb; b++) { memcpy(e->r_bold[m] + off, parts[b], sizeof(float) * rows[b] * nb0); off += rows[b] * nb0; free(parts[b]); }
                e->r_bold_len[m] = tot;
            }
        } else {
            for (int m = 0; m < e->nbold; m++) {
                int64_t rows = bold_flush(&e->monitors[m], &e->r_bold[m]);
                e->r_bold_len[m] = rows * nb0;
            }
        }
        e->r_nbold = e->nbold;
    }
    return HB_OK;
}

/* per-point coupling functions of projection p with coupling parameter k set to values[b]
 * (single sweep) or to the Cartesian values of the listed dimensions (multi sweep) */
static int coupling_sweep_table(const oengine* e, int p, int k, const float* values,
                                const hb_sweep_point* dims, int n_dims, ocsweep* cs) {
    const oproj* o = &e->proj[p];
    int B = e->n_sweep;
    if (!dims && (k < 0 || k >= o->n_cf_params)) { set_err("projection %d has %d coupling params, cannot sweep index %d", p, o->n_cf_params, k); return HB_ERR_INVALID_CONFIG; }
    cs->cf[p] = malloc(sizeof(ocfn) * B);
    float prm[16];
    for (int b = 0; b < B; b++) {
        memcpy(prm, o->cf_params, sizeof prm);
        if (!dims) prm[k] = values[b];
        else {
            int64_t rem = b;
            float vals[64];
            for (int d = n_dims - 1; d >= 0; d--) { int64_t idx = rem % dims[d].n_values; rem /= dims[d].n_values; vals[d] = dims[d].values[idx]; }
            for (int d = 0; d < n_dims; d++)
                if (dims[d].sub_idx == -1 - p) {
                    if (dims[d].param_idx < 0 || dims[d].param_idx >= o->n_cf_params) { set_err("projection %d has %d coupling params, cannot sweep index %d", p, o->n_cf_params, dims[d].param_idx); free(cs->cf[p]); cs->cf[p] = NULL; return HB_ERR_INVALID_CONFIG; }
                    prm[dims[d].param_idx] = vals[d];
                }
        }
        resolve_cfn(o->cf_name, prm, o->n_cf_params, o->diff_mode, e->sub[o->src].nm, &cs->cf[p][b]);
    }
    return HB_OK;
}

/* run_sweep / run_sweep_with_trajectory (engine.rs:477-494) */
EXPORT int32_t HBO(engine_run_sweep)(oengine* e, int32_t sub_idx, int32_t param_idx, const float* values, int32_t n_values,
                                     int64_t n_steps, uint32_t run_flags, const float* noise, int64_t noise_len, int32_t n_threads) {
    free_results(e);
    if (n_values != e->n_sweep) { set_err("expected %d sweep values, got %d", e->n_sweep, n_values); return HB_ERR_INVALID_STATE; }
    if (sub_idx >= e->nsub || sub_idx < -e->nproj) { set_err("subnetwork index %d out of range", sub_idx); return HB_ERR_INVALID_CONFIG; }
    int st = validate_run(e, noise, noise_len, n_steps);
    if (st) return st;
    osweep sw[16];
    memset(sw, 0, sizeof sw);
    ocsweep cs;
    memset(&cs, 0, sizeof cs);
    if (sub_idx < 0) {
        int p = -1 - sub_idx;
        st = coupling_sweep_table(e, p, param_idx, values, NULL, 0, &cs);
        if (st) return st;
    } else if (param_idx == k_native_sweep[e->sub[sub_idx].model]) {
        const osub* S = &e->sub[sub_idx];
        sw[sub_idx].mode = 1;
        sw[sub_idx].swept[param_idx] = 1;
        sw[sub_idx].pp = malloc(sizeof(real) * (size_t)e->n_sweep * S->nparams);
        for (int b = 0; b < e->n_sweep; b++) {
            for (int k = 0; k < S->nparams; k++) sw[sub_idx].pp[(size_t)b * S->nparams + k] = S->params[k];
            sw[sub_idx].pp[(size_t)b * S->nparams + param_idx] = values[b];
        }
    }
    e->r_params = malloc(sizeof(float) * n_values);
    memcpy(e->r_params, values, sizeof(float) * n_values);
    e->r_params_len = n_values;
    st = run_loop(e, sw, &cs, n_steps, (run_flags & HB_RUN_TRAJECTORY) != 0, noise, n_threads);
    for (int i = 0; i < 16; i++) free(sw[i].pp);
    for (int p = 0; p < 64; p++) free(cs.cf[p]);
    return st;
}

/* run_sweep_multi (engine.rs:862-1348) */
EXPORT int32_t HBO(engine_run_sweep_multi)(oengine* e, const hb_sweep_point* dims, int32_t n_dims, int64_t n_steps,
                                           uint32_t run_flags, const float* noise, int64_t noise_len, int32_t n_threads) {
    free_results(e);
    int64_t n = 1;
    for (int d = 0; d < n_dims; d++) n *= dims[d].n_values;
    if (n_dims == 0 || n == 0) { set_err("empty sweep"); return HB_ERR_INVALID_STATE; }
    if (n != e->n_sweep) { set_err("Cartesian product has %lld points, engine has %d", (long long)n, e->n_sweep); return HB_ERR_INVALID_STATE; }
    for (int d = 0; d < n_dims; d++) if (dims[d].sub_idx < -e->nproj || dims[d].sub_idx >= e->nsub) { set_err("subnetwork index out of range"); return HB_ERR_INVALID_CONFIG; }
    if (n_dims > 64) { set_err("too many sweep dimensions"); return HB_ERR_INVALID_CONFIG; }
    int st = validate_run(e, noise, noise_len, n_steps);
    if (st) return st;
    int B = e->n_sweep;
    /* fresh engine seeded by sweep point 0's current state, no BOLD monitors */
    for (int i = 0; i < e->nsub; i++) {
        osub* S = &e->sub[i];
        int per = S->nm * S->nvar;
        for (int k = 0; k < per; k++) S->x0[k] = (float)e->x[i][k];
    }
    e->nbold = 0;
    HBO(engine_reset)(e);
    /* expanded values per dimension (engine.rs:921-940) */
    osweep sw[16];
    memset(sw, 0, sizeof sw);
    int cnt[16] = {0};
    ocsweep cs;
    memset(&cs, 0, sizeof cs);
    for (int d = 0; d < n_dims; d++) {
        if (dims[d].sub_idx >= 0) { cnt[dims[d].sub_idx]++; continue; }
        int p = -1 - dims[d].sub_idx;
        if (!cs.cf[p]) {
            st = coupling_sweep_table(e, p, 0, NULL, dims, n_dims, &cs);
            if (st) { for (int q = 0; q < 64; q++) free(cs.cf[q]); return st; }
        }
    }
    for (int i = 0; i < e->nsub; i++) {
        if (!cnt[i]) continue;
        osub* S = &e->sub[i];
        sw[i].pp = malloc(sizeof(real) * (size_t)B * S->nparams);
        for (int b = 0; b < B; b++) for (int k = 0; k < S->nparams; k++) sw[i].pp[(size_t)b * S->nparams + k] = S->params[k];
        sw[i].mode = 2;
        if (cnt[i] == 1) {
            int d0 = 0; while (dims[d0].sub_idx != i) d0++;
            sw[i].mode = (dims[d0].param_idx == k_native_sweep[S->model]) ? 1 : 0;
        }
        for (int d = 0; d < n_dims && sw[i].mode != 0; d++)
            if (dims[d].sub_idx == i && dims[d].param_idx >= 0 && dims[d].param_idx < S->nparams) sw[i].swept[dims[d].param_idx] = 1;
    }
    e->r_params = malloc(sizeof(float) * (size_t)B * n_dims);
    e->r_params_len = (int64_t)B * n_dims;
    float vals[64];
    for (int b = 0; b < B; b++) {
        /* Cartesian point b, last dimension fastest (engine.rs:69-90) */
        int64_t rem = b;
        for (int d = n_dims - 1; d >= 0; d--) {
            int64_t idx = rem % dims[d].n_values;
            rem /= dims[d].n_values;
            vals[d] = dims[d].values[idx];
            e->r_params[(size_t)b * n_dims + d] = vals[d];
        }
        /* overrides in dimension order: a later dimension wins for a repeated index (dfun.rs:113-118) */
        for (int d = 0; d < n_dims; d++) {
            int i = dims[d].sub_idx;
            if (i < 0) continue;
            osub* S = &e->sub[i];
            if (sw[i].mode == 0) continue;
            if (dims[d].param_idx >= 0 && dims[d].param_idx < S->nparams) sw[i].pp[(size_t)b * S->nparams + dims[d].param_idx] = vals[d];
        }
    }
    st = run_loop(e, sw, &cs, n_steps, (run_flags & HB_RUN_TRAJECTORY) != 0, noise, n_threads);
    for (int i = 0; i < 16; i++) free(sw[i].pp);
    for (int p = 0; p < 64; p++) free(cs.cf[p]);
    return st;
}

EXPORT int64_t HBO(engine_step)(const oengine* e) { return e->step; }
EXPORT int32_t HBO(engine_n_bold)(const oengine* e) { return e->r_nbold; }
EXPORT const float* HBO(result_tavg)(const oengine* e, int32_t i, int64_t* len) { *len = (int64_t)e->n_sweep * e->sub[i].nm * e->sub[i].nvar; return e->r_tavg[i]; }
EXPORT const float* HBO(result_final)(const oengine* e, int32_t i, int64_t* len) { *len = (int64_t)e->n_sweep * e->sub[i].nm * e->sub[i].nvar; return e->r_final[i]; }
EXPORT const float* HBO(result_traj)(const oengine* e, int32_t i, int64_t* len) { *len = e->r_traj_len[i]; return e->r_traj[i]; }
EXPORT const float* HBO(result_bold)(const oengine* e, int32_t m, int64_t* len) { *len = e->r_bold_len[m]; return e->r_bold[m]; }
EXPORT const float* HBO(result_params)(const oengine* e, int64_t* len) { *len = e->r_params_len; return e->r_params; }

/* ------------------------------------------------------------------------------------------ */
/* unit entry points for the reference's known-answer tests                                   */
/* ------------------------------------------------------------------------------------------ */

/* one dfun evaluation for `n` nodes (state [n][nvar], coupling [n][ncvar]) with the scalar
 * parameter form, or the batch-native sweep form when sweep_form != 0 */
EXPORT int32_t HBO(dfun)(const char* model, const float* params, int32_t n_params, int32_t sweep_form,
                         const float* state, const float* coupling, int32_t n, float* out) {
    int m = model_from_name(model);
    if (m < 0) { set_err("Unknown model: %s", model ? model : "(null)"); return HB_ERR_INVALID_CONFIG; }
    real p[32], x[8], c[4], dx[8] = {0};
    for (int k = 0; k < n_params && k < 32; k++) p[k] = params[k];
    for (int i = 0; i < n; i++) {
        for (int v = 0; v < k_nvar[m]; v++) x[v] = state[i * k_nvar[m] + v];
        for (int v = 0; v < k_ncvar[m]; v++) c[v] = coupling[i * k_ncvar[m] + v];
        dfun_node(m, p, sweep_form, x, c, dx);
        for (int v = 0; v < k_nvar[m]; v++) out[i * k_nvar[m] + v] = (float)dx[v];
    }
    return HB_OK;
}

EXPORT int32_t HBO(clamp)(const char* model, float* state, int32_t n) {
    int m = model_from_name(model);
    if (m < 0) { set_err("Unknown model"); return HB_ERR_INVALID_CONFIG; }
    real x[8];
    for (int i = 0; i < n; i++) {
        for (int v = 0; v < k_nvar[m]; v++) x[v] = state[i * k_nvar[m] + v];
        clamp_node(m, x);
        for (int v = 0; v < k_nvar[m]; v++) state[i * k_nvar[m] + v] = (float)x[v];
    }
    return HB_OK;
}

/* pre() over `rows` rows of `ncv` values; returns the channel count in *pc */
EXPORT int32_t HBO(coupling_pre)(const char* name, const float* cp, int32_t ncp, int32_t cpu_form,
                                 const float* x, int32_t rows, int32_t ncv, float* out, int32_t* pc) {
    ocfn f;
    if (!cfn_parse(name, cp, ncp, &f)) { set_err("unknown coupling function"); return HB_ERR_INVALID_CONFIG; }
    int c = pre_channels(&f, ncv);
    real xr[8], o[16];
    for (int r = 0; r < rows; r++) {
        for (int k = 0; k < ncv; k++) xr[k] = x[r * ncv + k];
        pre_row(&f, xr, ncv, cpu_form, o);
        for (int k = 0; k < c; k++) out[r * c + k] = (float)o[k];
    }
    *pc = c;
    return HB_OK;
}

/* post_with_target over `rows` rows; x_i may be NULL, rowsums may be NULL */
EXPORT int32_t HBO(coupling_post)(const char* name, const float* cp, int32_t ncp, int32_t n_src,
                                  const float* gx, int32_t rows, int32_t pc, const float* xi, int32_t tgt_ncv,
                                  const float* rowsums, float* out, int32_t* oc) {
    ocfn f;
    if (!cfn_parse(name, cp, ncp, &f)) { set_err("unknown coupling function"); return HB_ERR_INVALID_CONFIG; }
    if (f.kind == C_KURAMOTO) f.n_src = n_src;
    if (f.kind == C_DIFFERENCE && rowsums) f.has_rowsums = 1;
    real g[16], xr[8], o[16];
    int c = 0;
    for (int r = 0; r < rows; r++) {
        for (int k = 0; k < pc; k++) g[k] = gx[r * pc + k];
        for (int k = 0; k < tgt_ncv; k++) xr[k] = xi ? xi[r * tgt_ncv + k] : 0;
        c = post_row(&f, g, pc, xr, tgt_ncv, rowsums ? rowsums[r] : 0, o);
        for (int k = 0; k < c; k++) out[r * c + k] = (float)o[k];
    }
    *oc = c;
    return HB_OK;
}

/* BoldModel: `n_steps` Euler steps of size dt (s) under a constant input; returns the signal
 * after each step in out[n_steps][nnodes] */
EXPORT void HBO(bold_model_run)(int32_t nnodes, const float* input, double dt, int32_t n_steps, float* out) {
    obold m;
    bold_init(&m, nnodes, 1, 0.0, 1.0);
    for (int k = 0; k < n_steps; k++) {
        bw_step(m.s, m.f, m.v, m.q, nnodes, input, dt);
        bw_signal(m.v, m.q, nnodes, out + (size_t)k * nnodes);
    }
    bold_free(&m);
}

/* BoldMonitor: feed inputs[n_steps][nnodes]; returns the flushed, TR-downsampled series (rows
 * in *rows, library-owned until hbo_free) and the number of raw samples in *n_samples */
EXPORT float* HBO(bold_monitor_run)(int32_t nnodes, int32_t bold_period, double tr, double dt_neural,
                                    const float* inputs, int32_t n_steps, int32_t flush,
                                    int64_t* rows, int64_t* n_samples) {
    obold m;
    bold_init(&m, nnodes, bold_period, tr, dt_neural);
    for (int k = 0; k < n_steps; k++) bold_accumulate(&m, inputs + (size_t)k * nnodes);
    float* out = NULL;
    *rows = flush ? bold_flush(&m, &out) : bold_downsample(&m, &out);
    *n_samples = m.n_times;
    bold_free(&m);
    return out;
}

EXPORT void HBO(free)(void* p) { free(p); }
