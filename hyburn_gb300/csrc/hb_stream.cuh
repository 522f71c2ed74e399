// hb_stream.cuh — point-resident pipeline whose delayed history lives in HBM.
//
// For one subnetwork coupled to itself through one CSR projection with per-edge delays
// (ring semantics of runtime.rs:125-211) when the history ring of a point does not fit shared
// memory (hundreds of nodes, delays of hundreds to thousands of steps). One CTA owns one sweep
// point. The history is stored per point as [node][RP + 2K][PCH] floats: for each source node the
// coupling-function pre() channels (PCH = ncvar for identity pre, 2 = sin, cos for Kuramoto) of
// consecutive time steps are adjacent, so the K = 8 delayed values an edge contributes to a block
// of 8 steps are one contiguous 32·PCH-byte run that touches one or two 32-byte sectors, not eight.
// Time t sits at position t mod RP; positions [RP, RP + K) mirror [0, K) so that a run of K
// positions never wraps, and [RP + K, RP + 2K) pads the row for aligned vector reads. Negative times read zero: the ring is zeroed at the start of a fresh
// run and RP > max delay + 2K keeps a position from being reused before its last reader.
//
// Warp specialisation as in resident_pipe_kernel: consumer threads (NPT nodes each) run the
// serial model updates of block i from a shared-memory double buffer while producer threads
// gather the coupling sums (and stage the noise draws) of block i + 1. With every delay >= 2K - 1
// the producers of block i + 1 read only times published by the consumers before they finished
// block i - 1, which the named barrier EMPTY[buf] orders before the producers start.
#pragma once
#include <cuda_runtime.h>
#include "hb_resident.cuh"

namespace hb {

// one model step of node state x from the coupling sums gx and the scaled noise nz
// (post() then the integrator stages of engine.rs:697-771 and the final clamp)
template <int MODEL>
__device__ __forceinline__ void stream_node_step(const DevProj& P, const float* cp, int integ, const float* prm,
                                                 int sweep_form, float rowsum, const float* gx, const float* nz,
                                                 float* x, float dt, float dt_half, float h2, float h6) {
    constexpr int NVAR = c_nvar(MODEL), NCV = c_ncvar(MODEL);
    float cc[2] = {0.0f, 0.0f};
    {
        float out[4] = {0.f, 0.f, 0.f, 0.f};
        float xi[2] = {x[0], NCV > 1 ? x[NCV - 1] : 0.0f};
        int oc = post(P.cfk, cp, P.has_rowsums, gx, P.pc, xi, NCV, rowsum, out);
        if (P.direct) {
            cc[0] = out[0];
            if (NCV > 1 && oc > 1) cc[1] = out[1];
        } else {
            for (int jj = 0; jj < P.ncm; jj++) {
                int sidx = P.cm_s[jj], cpl = P.cm_cpl[jj];
                if (sidx < NCV && cpl < NCV) {
                    float o = pick4(out, sidx);
                    if (cpl == 0) cc[0] += o; else cc[1] += o;
                }
            }
        }
    }
    float k1[NVAR], k2[NVAR], tmp[NVAR];
    dfun(MODEL, prm, sweep_form, x, cc, k1);
    if (integ == HBI_HEUN_STOCH) {
#pragma unroll
        for (int v = 0; v < NVAR; v++) tmp[v] = (x[v] + k1[v] * dt) + nz[v];
        clamp(MODEL, tmp);
        dfun(MODEL, prm, sweep_form, tmp, cc, k2);
#pragma unroll
        for (int v = 0; v < NVAR; v++) x[v] = (x[v] + (k1[v] + k2[v]) * dt_half) + nz[v];
    } else if (integ == HBI_HEUN_DET) {
#pragma unroll
        for (int v = 0; v < NVAR; v++) tmp[v] = x[v] + k1[v] * dt;
        clamp(MODEL, tmp);
        dfun(MODEL, prm, sweep_form, tmp, cc, k2);
#pragma unroll
        for (int v = 0; v < NVAR; v++) x[v] = x[v] + (k1[v] + k2[v]) * dt_half;
    } else if (integ == HBI_EULER) {
#pragma unroll
        for (int v = 0; v < NVAR; v++) x[v] = x[v] + k1[v] * dt;
    } else if (integ == HBI_EULER_STOCH) {
#pragma unroll
        for (int v = 0; v < NVAR; v++) x[v] = (x[v] + k1[v] * dt) + nz[v];
    } else {
        float k3[NVAR], k4[NVAR];
#pragma unroll
        for (int v = 0; v < NVAR; v++) tmp[v] = x[v] + k1[v] * h2;
        clamp(MODEL, tmp);
        dfun(MODEL, prm, sweep_form, tmp, cc, k2);
#pragma unroll
        for (int v = 0; v < NVAR; v++) tmp[v] = x[v] + k2[v] * h2;
        clamp(MODEL, tmp);
        dfun(MODEL, prm, sweep_form, tmp, cc, k3);
#pragma unroll
        for (int v = 0; v < NVAR; v++) tmp[v] = x[v] + k3[v] * dt;
        clamp(MODEL, tmp);
        dfun(MODEL, prm, sweep_form, tmp, cc, k4);
#pragma unroll
        for (int v = 0; v < NVAR; v++) {
            float sacc = k1[v] + k2[v] * 2.0f;
            sacc = sacc + k3[v] * 2.0f;
            sacc = sacc + k4[v];
            x[v] = x[v] + sacc * h6;
        }
        if (integ == HBI_RK4_STOCH) {
#pragma unroll
            for (int v = 0; v < NVAR; v++) x[v] = x[v] + nz[v];
        }
    }
    clamp(MODEL, x);
}

// BOLD input of node n at absolute step s (bold_monitor.rs:72-227): window sums, and per point the
// Balloon-Windkessel step and the TR emissions of a completed window
__device__ __forceinline__ void stream_bold_sample(const RunArgs& a, int b, int B, int n, int64_t s, float x0,
                                                   float* bacc, int* bcnt) {
    const int N0 = a.bold.n0;
    const int64_t rel = s - a.run_s0;
#pragma unroll
    for (int m = 0; m < HB_MAX_BOLD; m++) {
        if (m >= a.bold.n) break;
        bacc[m] = bacc[m] + x0;
        bcnt[m] += 1;
        bool full = bcnt[m] >= a.bold.period[m];
        bool last_partial = !full && (rel == a.run_steps - 1) && a.bold.partial[m] > 0;
        if (!(full || last_partial)) continue;
        int kk = full ? (int)((rel + 1) / a.bold.period[m] - 1) : a.bold.n_full[m];
        if (a.bold.per_point) {
            float avg = bacc[m] / (float)bcnt[m];
            float* bw = a.bold.bw[m];
            const size_t stride = (size_t)B * N0, idx = (size_t)b * N0 + n;
            float bs = bw[idx], bf = bw[stride + idx], bv = bw[2 * stride + idx], bq = bw[3 * stride + idx];
            float prev = bw[4 * stride + idx];
            bw_step(bs, bf, bv, bq, avg, full ? a.bold.dt_full[m] : a.bold.dt_part[m]);
            float cur = bw_signal(bv, bq);
            const BoldEmit* em = a.bold.emit[m];
            for (int q = lower_bound_emit(em, a.bold.n_emit[m], kk); q < a.bold.n_emit[m] && em[q].k == kk; q++) {
                float val = em[q].interp ? prev + (cur - prev) * em[q].w : cur;
                a.bold.out[m][((size_t)b * a.bold.n_out_run[m] + em[q].out) * N0 + n] = val;
            }
            bw[idx] = bs; bw[stride + idx] = bf; bw[2 * stride + idx] = bv; bw[3 * stride + idx] = bq;
            bw[4 * stride + idx] = cur;
        } else {
            a.bold.win[m][((size_t)kk * B + b) * N0 + n] = bacc[m];
        }
        bacc[m] = 0.0f;
        bcnt[m] = 0;
    }
}

// pre() channels of a node's new value at ring position pos (and its mirror below K)
template <int PRE, int NCV, int PCH>
__device__ __forceinline__ void stream_publish(float* ring, int n, int RPX, int RP, int pos, const float* x) {
    float v[PCH];
    if (PRE == PRE_KURA) { v[0] = sinf(x[0]); v[PCH - 1] = cosf(x[0]); }
    else {
#pragma unroll
        for (int c = 0; c < PCH; c++) v[c] = x[c];
    }
    float* r = ring + ((size_t)n * RPX + pos) * PCH;
    if (PCH == 2) *reinterpret_cast<float2*>(r) = make_float2(v[0], v[PCH - 1]);
    else r[0] = v[0];
    if (pos < HB_STREAM_K) {
        float* m = r + (size_t)RP * PCH;
        if (PCH == 2) *reinterpret_cast<float2*>(m) = make_float2(v[0], v[PCH - 1]);
        else m[0] = v[0];
    }
}

// The K = 8 consecutive history entries (PCH channels each) starting at q, read with 16-byte
// aligned vector loads from the aligned address at or below q and realigned in registers: 3 loads
// instead of 8 for one channel, 5 instead of 8 for two. Rows are padded by 2K positions, so
// the widest read stays inside the node's own row.
template <int PCH>
__device__ __forceinline__ void stream_window(const float* q, float (&v)[HB_STREAM_K][PCH]) {
    constexpr int K = HB_STREAM_K;
    const uintptr_t addr = reinterpret_cast<uintptr_t>(q);
    const float4* b4 = reinterpret_cast<const float4*>(addr & ~(uintptr_t)15);
    const int sh = (int)((addr >> 2) & 3);  // floats between the aligned base and q
    if (PCH == 1) {
        float f[12];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const float4 u = b4[i];
            f[4 * i] = u.x; f[4 * i + 1] = u.y; f[4 * i + 2] = u.z; f[4 * i + 3] = u.w;
        }
        float g[10];
#pragma unroll
        for (int i = 0; i < 10; i++) g[i] = (sh & 1) ? f[i + 1] : f[i];
#pragma unroll
        for (int j = 0; j < K; j++) v[j][0] = (sh & 2) ? g[j + 2] : g[j];
    } else {
        // q is 8-byte aligned: sh is 0 or 2
        float f[20];
#pragma unroll
        for (int i = 0; i < 5; i++) {
            const float4 u = b4[i];
            f[4 * i] = u.x; f[4 * i + 1] = u.y; f[4 * i + 2] = u.z; f[4 * i + 3] = u.w;
        }
#pragma unroll
        for (int j = 0; j < K; j++)
#pragma unroll
            for (int c = 0; c < PCH; c++) v[j][c] = sh ? f[2 * j + c + 2] : f[2 * j + c];
    }
}

// One edge's contribution to the K coupling sums of a block: the window of its source's history
// starting `delay` steps before the block's first step, times the weight, added to acc (fused
// multiply-adds: the regrouped sum; with EXACT a rounded product and a rounded sum per term, the
// reference's operations). At step 0 the edge also reads the current state (runtime.rs:166-170).
template <int PCH, bool EXACT = false>
__device__ __forceinline__ void stream_edge_acc(const float* ring, uint32_t m, float w, int sbm, int RP, int RPX,
                                                bool first_step, float (&acc)[HB_STREAM_K][PCH]) {
    const int d = (int)(m >> 16), src = (int)(m & 0xffffu);
    int pos = sbm - d;
    pos += (pos < 0) ? RP : 0;
    float v[HB_STREAM_K][PCH];
    stream_window<PCH>(ring + ((size_t)src * RPX + pos) * PCH, v);
#pragma unroll
    for (int j = 0; j < HB_STREAM_K; j++)
#pragma unroll
        for (int c = 0; c < PCH; c++) acc[j][c] = EXACT ? acc[j][c] + w * v[j][c] : __fmaf_rn(w, v[j][c], acc[j][c]);
    if (first_step) {
        const float* q0 = ring + (size_t)src * RPX * PCH;
#pragma unroll
        for (int c = 0; c < PCH; c++) acc[0][c] += w * q0[c];
    }
}

// L2 prefetch of the window of edge ep (when it is below e1)
template <int PCH>
__device__ __forceinline__ void stream_edge_prefetch(const float* ring, const uint32_t* ed, int ep, int e1, int sbm, int RP,
                                                     int RPX) {
    if (ep >= e1) return;
    const uint32_t mp = ed[ep];
    int pp = sbm - (int)(mp >> 16);
    pp += (pp < 0) ? RP : 0;
    const float* qp = ring + ((size_t)(mp & 0xffffu) * RPX + pp) * PCH;
    prefetch_l2(qp);
    prefetch_l2(qp + (HB_STREAM_K * PCH - 1));
}

// ---- one sweep point split over the CTAs of a thread-block cluster ----
#define HB_BAR_CONS 5  // named barrier of the consumer threads alone

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// every thread of every CTA of the cluster (release / acquire at cluster scope)
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}
// arrive (release at cluster scope) on the mbarrier at the same shared-memory offset in CTA `rank`
__device__ __forceinline__ void fence_cluster() { asm volatile("fence.acq_rel.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_remote(const uint64_t* bar, uint32_t rank) {
    uint32_t ra;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(smem_addr(bar)), "r"(rank));
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(ra) : "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// wait (acquire at cluster scope) for the phase of parity `parity`, for at most 200 ms; false when the
// time ran out. After a timeout in the block (*gave_up set) later waits return at once, so a fault in
// the cluster's signalling costs one bounded wait, not one per block.
__device__ __forceinline__ bool mbar_try_cluster(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done) : "r"(smem_addr(bar)), "r"(parity) : "memory");
    return done != 0;
}
__device__ __forceinline__ bool mbar_wait_cluster(uint64_t* bar, uint32_t parity, volatile int* gave_up) {
    if (mbar_try_cluster(bar, parity)) return true;  // the common case: no clock read
    if (*gave_up) return false;
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try_cluster(bar, parity)) return true;
        __nanosleep(64);  // a waiting warp leaves the issue slots to the consumers
        if (global_ns() - t0 > 200000000ull || *gave_up) {
            *gave_up = 1;
            return false;
        }
    }
}
// The CTAs of a cluster-split point signal each finished block on four barriers (block mod 4) in every
// CTA. A barrier's phase then only ever collects one arrival per CTA for the same block: a CTA can
// arrive for block j + 4 only after its producers saw every CTA's arrival for block j + 2, which each CTA
// made after its arrivals for block j.
#define HB_HIST_BARS 4
// consumers of a cluster-split point after finishing block `blk`: their history writes made visible at
// cluster scope, then one arrival per CTA on every CTA's barrier of the block, made by C consumer threads
// in parallel
__device__ __forceinline__ void stream_signal_block(uint64_t* hbar, int blk, int C, int n_cons) {
    fence_cluster();
    named_sync(HB_BAR_CONS, n_cons);
    if ((int)threadIdx.x < C) mbar_arrive_remote(hbar + (blk & (HB_HIST_BARS - 1)), threadIdx.x);
}

// Consumer steps for Heun (deterministic or stochastic) with Linear coupling delivered directly, no
// trajectory and no BOLD, one node per thread: one straight-line loop with the operations of
// stream_node_step in the same order.
template <int MODEL, bool STOCH, bool SF, bool NOISE_SMEM>
__device__ __forceinline__ void stream_consume_heun_linear(float* x, float* tv, const float* prm, const float* cp,
                                                           const float* nscale, float dt, float dt_half,
                                                           const float* gxbuf, const float* nzbuf, const float* noise_g,
                                                           size_t nstride, float* ring, int n, int l, bool active, int ns,
                                                           int RPX, int RP, int wpos, int n_steps, int n_blocks,
                                                           int nthreads, int C, uint64_t* hbar, int n_cons) {
    constexpr int NVAR = c_nvar(MODEL), NCV = c_ncvar(MODEL), K = HB_STREAM_K;
    const float ca = cp[0], cb = cp[1];
    float nsc[NVAR];
#pragma unroll
    for (int v = 0; v < NVAR; v++) nsc[v] = nscale[v];
    for (int blk = 0; blk < n_blocks; blk++) {
        const int buf = blk & 1;
        named_sync(HB_BAR_FULL0 + buf, nthreads);
        const int it0 = blk * K;
        const int nb = (n_steps - it0) < K ? (n_steps - it0) : K;
        const float* gb = gxbuf + (size_t)buf * K * ns * NCV + (size_t)l * NCV;
        const float* nbuf = nzbuf + (size_t)buf * K * ns * NVAR + (size_t)l * NVAR;
#pragma unroll 1
        for (int j = 0; j < nb; j++) {
            const int pos = wpos;
            wpos = (wpos + 1 == RP) ? 0 : wpos + 1;
            if (!active) continue;  // threads past the last node only take part in the barriers
            float cc[2] = {0.0f, 0.0f};
            cc[0] = gb[(size_t)j * ns * NCV] * ca + cb;
            if (NCV > 1) cc[1] = gb[(size_t)j * ns * NCV + 1] * ca + cb;
            float nz[NVAR];
#pragma unroll
            for (int v = 0; v < NVAR; v++) {
                if (!STOCH) nz[v] = 0.0f;
                else if (NOISE_SMEM) nz[v] = nbuf[(size_t)j * ns * NVAR + v] * nsc[v];
                else nz[v] = __ldcs(noise_g + (size_t)(it0 + j) * nstride + (size_t)n * NVAR + v) * nsc[v];
            }
            float k1[NVAR], k2[NVAR], tmp[NVAR];
            dfun(MODEL, prm, SF ? 1 : 0, x, cc, k1);
#pragma unroll
            for (int v = 0; v < NVAR; v++) tmp[v] = STOCH ? (x[v] + k1[v] * dt) + nz[v] : x[v] + k1[v] * dt;
            clamp(MODEL, tmp);
            dfun(MODEL, prm, SF ? 1 : 0, tmp, cc, k2);
#pragma unroll
            for (int v = 0; v < NVAR; v++)
                x[v] = STOCH ? (x[v] + (k1[v] + k2[v]) * dt_half) + nz[v] : x[v] + (k1[v] + k2[v]) * dt_half;
            clamp(MODEL, x);
#pragma unroll
            for (int v = 0; v < NVAR; v++) tv[v] = tv[v] + x[v];
            stream_publish<PRE_ID, NCV, NCV>(ring, n, RPX, RP, pos, x);
        }
        __threadfence_block();
        named_arrive(HB_BAR_EMPTY0 + buf, nthreads);
        if (C > 1) stream_signal_block(hbar, blk, C, n_cons);
    }
}

// steps from absolute step s (included) to the next step at which stream_bold_sample emits: a monitor's
// window of period steps closes (its count `cnt` before step s), or the run's last step closes a partial
// window
__device__ __forceinline__ int stream_bold_until(const RunArgs& a, const int* cnt, int64_t s) {
    int u = 0x7fffffff;
    bool partial = false;
#pragma unroll
    for (int m = 0; m < HB_MAX_BOLD; m++)
        if (m < a.bold.n) {
            u = min(u, a.bold.period[m] - cnt[m]);
            partial |= a.bold.partial[m] > 0;
        }
    if (partial) u = min(u, (int)(a.run_steps - (s - a.run_s0)));
    return u;
}

// the Kuramoto phase wrap x - floor(x / 2pi) * 2pi (clamp(), dfun.rs:170-239). For 0 < x < 2pi the
// quotient rounds to a value below 1 (x <= 2pi - 2^-21 gives x / 2pi <= 1 - 2^-24 after rounding), so
// the floor is 0 and the result is x itself: the division runs only when the phase left that interval.
__device__ __forceinline__ float kura_wrap(float v) {
    const float two_pi = 2.0f * 3.14159265358979323846f;
    if (v > 0.0f && v < two_pi) return v;
    return v - floorf(v / two_pi) * two_pi;
}

// Consumer steps for the Kuramoto model with Kuramoto coupling delivered directly and Heun integration
// (deterministic or stochastic), NPT nodes per thread, writing the trajectory and the coupling sums when
// asked (as the general loop does): the operations of stream_node_step in the same order, with two exact
// shortcuts. The corrector's derivative
// equals the predictor's (c + omega does not depend on the phase, dfun.rs:480-492), so the predictor
// state is not formed; and the sin / cos of the phase that post() takes (coupling.rs:323-399) are the
// values the previous step published (sinf / cosf of the same float), so each step evaluates them once.
// Per-point BOLD is sampled as in the general loop.
template <int NPT, bool STOCH, bool NOISE_SMEM, bool OUTS>
__device__ __forceinline__ void stream_consume_kuramoto(float (&x)[NPT][1], float (&tv)[NPT][1], const bool (&active)[NPT],
                                                        const float (&om)[NPT], float cpk, float nsc, float dt_half,
                                                        const float* gxbuf, const float* nzbuf, const float* noise_g,
                                                        size_t nstride, float* ring, int n0, int t, int n_cons, int ns,
                                                        int RPX, int RP, int wpos, int64_t s, const RunArgs& a, int b, int B,
                                                        int N, size_t state_len,
                                                        float (&bacc)[NPT][HB_MAX_BOLD], int (&bcnt)[NPT][HB_MAX_BOLD],
                                                        int n_blocks, int nthreads, int C, uint64_t* hbar) {
    constexpr int K = HB_STREAM_K;
    float sn[NPT], cs[NPT];
#pragma unroll
    for (int q = 0; q < NPT; q++) { sn[q] = sinf(x[q][0]); cs[q] = cosf(x[q][0]); }
    // BOLD: the window sums grow every step; the window counts and the emissions (stream_bold_sample) are
    // settled only at the steps where a monitor's window closes or the run's last step emits a partial
    // window. `until` counts the steps to the next such step (the current one included); `pend` the steps
    // whose counts are not yet added.
    const bool bold = a.bold.n > 0;
    int until = bold ? stream_bold_until(a, bcnt[0], s) : 0, pend = 0;
    for (int blk = 0; blk < n_blocks; blk++) {
        const int buf = blk & 1;
        named_sync(HB_BAR_FULL0 + buf, nthreads);
        const int it0 = blk * K;
        const int nb = (a.n_steps - it0) < K ? (a.n_steps - it0) : K;
        const float2* gb = reinterpret_cast<const float2*>(gxbuf) + (size_t)buf * K * ns;
        const float* nbuf = nzbuf + (size_t)buf * K * ns;
#pragma unroll 1
        for (int j = 0; j < nb; j++, s++) {
            const int pos = wpos;
            wpos = (wpos + 1 == RP) ? 0 : wpos + 1;
#pragma unroll
            for (int q = 0; q < NPT; q++) {
                if (!active[q]) continue;
                const int l = t + q * n_cons, n = n0 + l;
                const float2 g = gb[(size_t)j * ns + l];
                if (OUTS && a.gx_out) __stcs(reinterpret_cast<float2*>(a.gx_out) + ((size_t)(it0 + j) * B + b) * N + n, g);
                float nz = 0.0f;
                if (STOCH) nz = (NOISE_SMEM ? nbuf[(size_t)j * ns + l] : __ldcs(noise_g + (size_t)(it0 + j) * nstride + n)) * nsc;
                const float ct = cs[q] * g.x;
                const float st = sn[q] * g.y;
                const float cc = (ct - st) * cpk;
                const float k1 = cc + om[q];
                float xn = STOCH ? (x[q][0] + (k1 + k1) * dt_half) + nz : x[q][0] + (k1 + k1) * dt_half;
                xn = kura_wrap(xn);
                x[q][0] = xn;
                tv[q][0] = tv[q][0] + xn;
                if (OUTS && a.traj) __stcs(a.traj + ((size_t)(it0 + j) * B + b) * state_len + n, xn);
                if (bold) {
                    if (until == 1) {
#pragma unroll
                        for (int m = 0; m < HB_MAX_BOLD; m++) bcnt[q][m] += pend;
                        stream_bold_sample(a, b, B, n, s, xn, bacc[q], bcnt[q]);
                    } else {
#pragma unroll
                        for (int m = 0; m < HB_MAX_BOLD; m++)
                            if (m < a.bold.n) bacc[q][m] = bacc[q][m] + xn;
                    }
                }
                sn[q] = sinf(xn);
                cs[q] = cosf(xn);
                float* r = ring + ((size_t)n * RPX + pos) * 2;
                *reinterpret_cast<float2*>(r) = make_float2(sn[q], cs[q]);
                if (pos < K) *reinterpret_cast<float2*>(r + (size_t)RP * 2) = make_float2(sn[q], cs[q]);
            }
            if (bold) {
                if (until == 1) {
                    pend = 0;
                    until = stream_bold_until(a, bcnt[0], s + 1);
                } else {
                    pend++;
                    until--;
                }
            }
        }
        __threadfence_block();
        named_arrive(HB_BAR_EMPTY0 + buf, nthreads);
        if (C > 1) stream_signal_block(hbar, blk, C, n_cons);
    }
#pragma unroll
    for (int q = 0; q < NPT; q++)
#pragma unroll
        for (int m = 0; m < HB_MAX_BOLD; m++) bcnt[q][m] += pend;
}

// copy of a network description into shared memory by all threads of the block (no barrier)
__device__ __forceinline__ void stream_load_net(DevNet& net, const DevNet* __restrict__ gnet) {
    const int* src = reinterpret_cast<const int*>(gnet);
    int* dst = reinterpret_cast<int*>(&net);
    for (int i = threadIdx.x; i < (int)(sizeof(DevNet) / 4); i += blockDim.x) dst[i] = src[i];
}

// One sweep point b of a network, or with a.stream_cluster = C > 1 the slice of its nodes that CTA
// `rank` of the point's cluster owns. `net` is the block's shared-memory copy of the network's
// description, filled by the caller and published with a block barrier before this call.
template <int MODEL, int PRE, int NPT, int MAXT>
__device__ __forceinline__ void stream_point(DevNet& net, const RunArgs& a, const int b, const int rank) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ __align__(8) uint64_t hist_bar[HB_HIST_BARS];  // cluster-split: all CTAs finished block j (j mod 4)
    __shared__ int hist_gave_up;                              // cluster-split: a wait on hist_bar timed out
    constexpr int NVAR = c_nvar(MODEL), NCV = c_ncvar(MODEL);
    constexpr int PCH = (PRE == PRE_KURA) ? 2 : NCV;
    constexpr int K = HB_STREAM_K;
    constexpr int UNR = (MAXT > 768) ? 1 : 2;  // edges in flight per producer thread (register budget)
    constexpr int DB = (MAXT > 768) ? 1 : 8;   // edge descriptors loaded per batch (register budget)
    const int t = threadIdx.x, nthreads = blockDim.x;
    const int nm = net.sub[0].nm;  // nodes of the network (history rows)
    const int C = a.stream_cluster > 1 ? a.stream_cluster : 1;
    const int n0 = (int)(((long long)nm * rank) / C);                  // this CTA's nodes n0 .. n0 + ns - 1
    const int ns = (int)(((long long)nm * (rank + 1)) / C) - n0;
    const int RP = a.stream_rp, RPX = RP + 2 * K;
    const int n_cons = (((ns + NPT - 1) / NPT + 31) >> 5) << 5;
    const int n_prod = nthreads - n_cons;
    float* ring = a.ring + (size_t)b * nm * RPX * PCH;

    // shared layout: gx buffers [2][K][ns][PCH] | noise buffers [2][K][ns*NVAR] | rowptr | edges | weights
    size_t off = 0;
    float* gxbuf = reinterpret_cast<float*>(smem);
    off += (size_t)2 * K * ns * PCH * sizeof(float);
    float* nzbuf = reinterpret_cast<float*>(smem + off);
    if (a.stream_noise_smem) off += (size_t)2 * K * ns * NVAR * sizeof(float);
    off = (off + 15) & ~(size_t)15;
    int* s_rowptr = reinterpret_cast<int*>(smem + off);
    off += (size_t)(ns + 1) * 4;
    off = (off + 15) & ~(size_t)15;
    uint32_t* s_edges = reinterpret_cast<uint32_t*>(smem + off);
    off += (size_t)a.smem_edges * 4;
    float* s_ew = reinterpret_cast<float*>(smem + off);
    off += (size_t)a.smem_edges * 4;
    off = (off + 15) & ~(size_t)15;
    // with several nodes per consumer thread, every node's parameter row [nm][PU] (its node row when the
    // subnetwork has per-node parameters, else the point's row)
    constexpr int PU = c_nparams_used(MODEL);
    float* s_prm = reinterpret_cast<float*>(smem + off);
    if (NPT > 1) off += (size_t)ns * PU * 4;
    off = (off + 15) & ~(size_t)15;
    int* s_porder = reinterpret_cast<int*>(smem + off);  // [ns] producer order of the slice's nodes
    off += (size_t)ns * 4;
    off = (off + 15) & ~(size_t)15;
    // bulk-staged gathers: per producer warp 32 window slots of BSLOT bytes, then one mbarrier per warp
    constexpr int BSLOT = PCH == 2 ? 80 : 48;  // an 8-step window from the 16-byte boundary at or below it
    unsigned char* s_stage = smem + off;
    uint64_t* s_sbar = reinterpret_cast<uint64_t*>(smem + off + (size_t)(n_prod >> 5) * 32 * BSLOT);

    // a fresh run starts from a zero history (zero rows after pre() for d > s, runtime.rs:166-176);
    // each CTA clears its own nodes' rows
    if (a.s0 == 0) {
        float4* r4 = reinterpret_cast<float4*>(ring + (size_t)n0 * RPX * PCH);
        const size_t n4 = ((size_t)ns * RPX * PCH) >> 2;
        for (size_t i = t; i < n4; i += nthreads) r4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (C > 1 && t == 0) {
        for (int q = 0; q < HB_HIST_BARS; q++) mbar_init(&hist_bar[q], (uint32_t)C);
        hist_gave_up = 0;
        mbar_init_fence();
    }
    __syncthreads();
    const DevProj& P = net.proj[0];
    // row bounds of this CTA's target nodes; relative to the shared-memory copy of its edges when
    // they fit there
    const bool edges_smem = a.smem_edges > 0;
    const int e_first = P.rowptr[n0];
    for (int i = t; i <= ns; i += nthreads) s_rowptr[i] = P.rowptr[n0 + i] - (edges_smem ? e_first : 0);
    if (edges_smem) {
        const int cnt = P.rowptr[n0 + ns] - e_first;
        for (int i = t; i < cnt; i += nthreads) { s_edges[i] = P.edges[e_first + i]; s_ew[i] = P.ew[e_first + i]; }
    }
    const uint32_t* __restrict__ ed = edges_smem ? s_edges : P.edges;
    const float* __restrict__ ew = edges_smem ? s_ew : P.ew;
    const int integ = net.sub[0].integ;
    const bool stoch = (integ == HBI_EULER_STOCH || integ == HBI_HEUN_STOCH || integ == HBI_RK4_STOCH);
    float cp[8];
    {
        const float* c = P.cp_pp ? P.cp_pp + (size_t)b * HB_NCP : P.cp;
#pragma unroll
        for (int i = 0; i < 8; i++) cp[i] = c[i];
    }
    const int B = net.B;
    const float* noise_base = a.noise + (a.noise_per_point ? (size_t)b * net.noise_row : 0);
    const size_t nstride = (size_t)(a.noise_per_point ? B : 1) * net.noise_row;
    const int n_blocks = (a.n_steps + K - 1) / K;
    const bool is_consumer = t < n_cons;
    const bool first_launch_of_run = (a.s0 == a.run_s0);

    // consumer state: local nodes t, t + n_cons, ... (network nodes n0 + those)
    float x[NPT][NVAR], tv[NPT][NVAR];
    size_t st_base[NPT];
    bool active[NPT];
#pragma unroll
    for (int q = 0; q < NPT; q++) {
        const int n = n0 + t + q * n_cons;
        active[q] = is_consumer && t + q * n_cons < ns;
        st_base[q] = (size_t)b * net.state_len + (size_t)(active[q] ? n : 0) * NVAR;
#pragma unroll
        for (int v = 0; v < NVAR; v++) {
            x[q][v] = active[q] ? a.state[st_base[q] + v] : 0.0f;
            tv[q][v] = (active[q] && !first_launch_of_run) ? a.tavg[st_base[q] + v] : 0.0f;
        }
        if (active[q]) stream_publish<PRE, NCV, PCH>(ring, n, RPX, RP, (int)(a.s0 % RP), x[q]);
    }
    if (NPT > 1)
        for (int i = t; i < ns * PU; i += nthreads) s_prm[i] = hb_param_row(net.sub[0], b, n0 + i / PU)[i % PU];
    for (int i = t; i < ns; i += nthreads) s_porder[i] = P.porder ? P.porder[n0 + i] : i;
    // the history every CTA of the point reads (cleared rows, the published start state) and the
    // barriers of the cluster are ready
    if (C > 1) cluster_barrier();
    else __syncthreads();

    if (!is_consumer) {
        // ================= producers =================
        const int p = t - n_cons;
        uint32_t bulk_phase = 0;  // bulk-staged gathers: chunks this warp has staged (its mbarrier's phase)
        if (a.stream_wgather && a.stream_bulk) {
            if ((p & 31) == 0) {
                mbar_init(s_sbar + (p >> 5), 1);
                mbar_init_fence();
            }
            __syncwarp();
        }
        const int PL = a.pipe_lanes;  // threads per node (power of two <= 8)
        const int pf = a.stream_prefetch;
        const int items = ns * PL;
        const int rounds = (items + n_prod - 1) / n_prod;
        const int row_len = ns * NVAR;  // this CTA's part of a noise row
        for (int blk = 0; blk < n_blocks; blk++) {
            const int buf = blk & 1;
            if (blk >= 2) named_sync(HB_BAR_EMPTY0 + buf, nthreads);
            // block blk reads the history up to the first step of block blk - 1, which every CTA of the
            // point has published once it finished block blk - 2
            if (C > 1 && blk >= 2 &&
                !mbar_wait_cluster(&hist_bar[(blk - 2) & (HB_HIST_BARS - 1)], (uint32_t)(((blk - 2) >> 2) & 1), &hist_gave_up))
                atomicOr(a.flags + 1, 4);
            const int it0 = blk * K;
            const int nb = (a.n_steps - it0) < K ? (a.n_steps - it0) : K;
            const int64_t sb = a.s0 + it0;
            const int sbm = (int)(sb % RP);
            float* gb = gxbuf + (size_t)buf * K * ns * PCH;
            if (a.stream_wgather && a.stream_bulk) {
                // the warp-cooperative gather with each chunk's windows staged by the bulk-copy engine: lane j
                // copies edge j's window (BSLOT bytes from the 16-byte boundary at or below its first entry,
                // which stays inside the node's row) into its slot of the warp's staging area; lane 0 posts
                // the chunk's byte count on the warp's mbarrier, whose phase completes when every copy has
                // landed (bounded wait); the 8 lanes of a slot then read the window's entries from shared
                // memory. The reads of one chunk finish (warp barrier, proxy fence) before the next chunk's
                // copies overwrite the slots.
                const int lane = t & 31, wid = p >> 5, nwarp = n_prod >> 5;
                const int slot = lane >> 3, stp = lane & (K - 1);
                unsigned char* stg = s_stage + (size_t)wid * 32 * BSLOT;
                uint64_t* sbar = s_sbar + wid;
                for (int i = wid; i < ns; i += nwarp) {
                    const int node = s_porder[i];
                    const int e0 = s_rowptr[node], e1 = s_rowptr[node + 1];
                    float acc[PCH];
#pragma unroll
                    for (int c = 0; c < PCH; c++) acc[c] = 0.0f;
                    for (int eb = e0; eb < e1; eb += 32) {
                        const int cnt = (e1 - eb) < 32 ? (e1 - eb) : 32;
                        uint32_t src = 0, shift = 0;
                        float w = 0.0f;
                        if (lane == 0)
                            asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
                                         ::"r"(smem_addr(sbar)), "r"((uint32_t)(cnt * BSLOT)) : "memory");
                        __syncwarp();
                        if (lane < cnt) {
                            const uint32_t m = ed[eb + lane];
                            int pos = sbm - (int)(m >> 16);
                            pos += (pos < 0) ? RP : 0;
                            src = m & 0xffffu;
                            const size_t off_f = ((size_t)src * RPX + (size_t)pos) * PCH;  // floats
                            shift = (uint32_t)(off_f & 3);
                            w = ew[eb + lane];
                            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                                         ::"r"(smem_addr(stg + lane * BSLOT)), "l"(ring + (off_f - shift)), "r"((uint32_t)BSLOT),
                                           "r"(smem_addr(sbar))
                                         : "memory");
                        }
                        if (!mbar_wait(sbar, bulk_phase & 1u)) atomicOr(a.flags + 1, 4);
                        bulk_phase++;
#pragma unroll
                        for (int u = 0; u < 8; u++) {
                            const int k = 4 * u + slot;
                            const uint32_t shk = __shfl_sync(0xffffffffu, shift, k);
                            const float wk = __shfl_sync(0xffffffffu, w, k);
                            const float* q = reinterpret_cast<const float*>(stg + k * BSLOT) + shk + stp * PCH;
                            if (k < cnt) {
                                if (PCH == 2) {
                                    acc[0] = __fmaf_rn(wk, q[0], acc[0]);
                                    acc[PCH - 1] = __fmaf_rn(wk, q[1], acc[PCH - 1]);
                                } else acc[0] = __fmaf_rn(wk, q[0], acc[0]);
                            }
                        }
                        if (sb == 0) {
                            // step 0 also reads the current state (runtime.rs:166-170)
#pragma unroll
                            for (int u = 0; u < 8; u++) {
                                const int k = 4 * u + slot;
                                const uint32_t sk = __shfl_sync(0xffffffffu, src, k);
                                const float wk = __shfl_sync(0xffffffffu, w, k);
                                if (stp == 0 && k < cnt) {
                                    const float* q0 = ring + (size_t)sk * RPX * PCH;
#pragma unroll
                                    for (int c = 0; c < PCH; c++) acc[c] += wk * q0[c];
                                }
                            }
                        }
                        __syncwarp();
                    }
#pragma unroll
                    for (int c = 0; c < PCH; c++) {
                        acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 8);
                        acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 16);
                    }
                    if (slot == 0 && stp < nb) {
#pragma unroll
                        for (int c = 0; c < PCH; c++) gb[((size_t)stp * ns + node) * PCH + c] = acc[c];
                    }
                }
            } else if (a.stream_wgather) {
                // warp-cooperative gather: warp w takes the slice's nodes w, w + nwarp, ... in producer order
                // (decreasing in-degree), 32 of the node's edges at a time. Lane j decodes edge j of the chunk
                // (history offset of its window, weight); the window of chunk edge k = 4u + slot is then read
                // by the 8 lanes of that slot, lane (slot, stp) taking entry stp (step stp of the block), so
                // one load instruction covers 4 edges as 4 runs of 32 PCH contiguous bytes; each lane sums
                // its step over its slot's edges, and the 4 slots' sums are added by shuffles.
                const int lane = t & 31, wid = p >> 5, nwarp = n_prod >> 5;
                const int slot = lane >> 3, stp = lane & (K - 1);
                for (int i = wid; i < ns; i += nwarp) {
                    const int node = s_porder[i];
                    const int e0 = s_rowptr[node], e1 = s_rowptr[node + 1];
                    float acc[PCH];
#pragma unroll
                    for (int c = 0; c < PCH; c++) acc[c] = 0.0f;
                    for (int eb = e0; eb < e1; eb += 32) {
                        const int cnt = (e1 - eb) < 32 ? (e1 - eb) : 32;
                        // lanes past the row read entries RP + K .. RP + 2K - 1 of row 0, which nothing writes
                        // (cleared when a run starts), with weight 0
                        uint32_t off = (uint32_t)(RP + K) * PCH, src = 0;
                        float w = 0.0f;
                        if (lane < cnt) {
                            const uint32_t m = ed[eb + lane];
                            int pos = sbm - (int)(m >> 16);
                            pos += (pos < 0) ? RP : 0;
                            src = m & 0xffffu;
                            off = (src * (uint32_t)RPX + (uint32_t)pos) * PCH;
                            w = ew[eb + lane];
                        }
                        float v[8][PCH], wk[8];
#pragma unroll
                        for (int u = 0; u < 8; u++) {
                            const int k = 4 * u + slot;  // lanes with k >= cnt read the zero entries
                            const uint32_t o = __shfl_sync(0xffffffffu, off, k) + (uint32_t)(stp * PCH);
                            wk[u] = __shfl_sync(0xffffffffu, w, k);
                            if (PCH == 2) {
                                const float2 f = *reinterpret_cast<const float2*>(ring + o);
                                v[u][0] = f.x;
                                v[u][PCH - 1] = f.y;
                            } else v[u][0] = ring[o];
                        }
#pragma unroll
                        for (int u = 0; u < 8; u++)
#pragma unroll
                            for (int c = 0; c < PCH; c++) acc[c] = __fmaf_rn(wk[u], v[u][c], acc[c]);
                        if (sb == 0) {
                            // step 0 also reads the current state (runtime.rs:166-170)
#pragma unroll
                            for (int u = 0; u < 8; u++) {
                                const int k = 4 * u + slot;
                                const uint32_t sk = __shfl_sync(0xffffffffu, src, k);
                                if (stp == 0 && k < cnt) {
                                    const float* q0 = ring + (size_t)sk * RPX * PCH;
#pragma unroll
                                    for (int c = 0; c < PCH; c++) acc[c] += wk[u] * q0[c];
                                }
                            }
                        }
                    }
#pragma unroll
                    for (int c = 0; c < PCH; c++) {
                        acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 8);
                        acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 16);
                    }
                    if (slot == 0 && stp < nb) {
#pragma unroll
                        for (int c = 0; c < PCH; c++) gb[((size_t)stp * ns + node) * PCH + c] = acc[c];
                    }
                }
            } else {
                for (int r = 0; r < rounds; r++) {
                    const int item = p + r * n_prod;
                    const int islot = item / PL, lane = item - (item / PL) * PL;
                    const int node = islot < ns ? s_porder[islot] : islot;
                    float acc[K][PCH];
#pragma unroll
                    for (int j = 0; j < K; j++)
#pragma unroll
                        for (int c = 0; c < PCH; c++) acc[j][c] = 0.0f;
                    if (node < ns) {
                        const int e0 = s_rowptr[node], e1 = s_rowptr[node + 1];
                        if constexpr (DB == 1) {
#pragma unroll UNR
                            for (int e = e0 + lane; e < e1; e += PL) {
                                if (pf) stream_edge_prefetch<PCH>(ring, ed, e + pf * PL, e1, sbm, RP, RPX);
                                if (a.exact_sums) stream_edge_acc<PCH, true>(ring, ed[e], ew[e], sbm, RP, RPX, sb == 0, acc);
                                else stream_edge_acc<PCH>(ring, ed[e], ew[e], sbm, RP, RPX, sb == 0, acc);
                            }
                        } else {
                            // the edge descriptors DB at a time, loaded together, so that their latency is
                            // paid once per batch instead of before every window read; the batch is
                            // consumed in order by rotating it through registers
                            for (int eb = e0 + lane; eb < e1; eb += DB * PL) {
                                uint32_t mb[DB];
                                float wb[DB];
#pragma unroll
                                for (int u = 0; u < DB; u++) {
                                    const int e = eb + u * PL;
                                    mb[u] = (e < e1) ? ed[e] : 0u;
                                    wb[u] = (e < e1) ? ew[e] : 0.0f;
                                }
                                const int cnt = (e1 - eb + PL - 1) / PL < DB ? (e1 - eb + PL - 1) / PL : DB;
#pragma unroll UNR
                                for (int u = 0; u < cnt; u++) {
                                    const uint32_t m = mb[0];
                                    const float w = wb[0];
#pragma unroll
                                    for (int q = 0; q + 1 < DB; q++) { mb[q] = mb[q + 1]; wb[q] = wb[q + 1]; }
                                    if (pf) stream_edge_prefetch<PCH>(ring, ed, eb + (u + pf) * PL, e1, sbm, RP, RPX);
                                    if (a.exact_sums) stream_edge_acc<PCH, true>(ring, m, w, sbm, RP, RPX, sb == 0, acc);
                                    else stream_edge_acc<PCH>(ring, m, w, sbm, RP, RPX, sb == 0, acc);
                                }
                            }
                        }
                    }
                    for (int o = PL >> 1; o > 0; o >>= 1) {
#pragma unroll
                        for (int j = 0; j < K; j++)
#pragma unroll
                            for (int c = 0; c < PCH; c++) acc[j][c] += __shfl_xor_sync(0xffffffffu, acc[j][c], o);
                    }
                    if (node < ns && lane == 0) {
#pragma unroll
                        for (int j = 0; j < K; j++)
                            if (j < nb) {
#pragma unroll
                                for (int c = 0; c < PCH; c++) gb[((size_t)j * ns + node) * PCH + c] = acc[j][c];
                            }
                    }
                }
            }
            if (stoch && a.stream_noise_smem) {
                float* nbuf = nzbuf + (size_t)buf * K * row_len;
                const float* src = noise_base + (size_t)it0 * nstride + (size_t)n0 * NVAR;
                if (C == 1 && !a.noise_per_point && ((reinterpret_cast<uintptr_t>(src) & 15) == 0)) {
                    const int total = nb * row_len, n4 = total >> 2;
                    const float4* s4 = reinterpret_cast<const float4*>(src);
                    float4* d4 = reinterpret_cast<float4*>(nbuf);
                    for (int i = p; i < n4; i += n_prod) d4[i] = __ldcs(s4 + i);
                    for (int i = (n4 << 2) + p; i < total; i += n_prod) nbuf[i] = __ldcs(src + i);
                    // the rows of the block four blocks ahead into L2, one 128-byte line per thread
                    if (it0 + 4 * K < a.n_steps) {
                        const int ahead = (a.n_steps - it0 - 4 * K) < K ? (a.n_steps - it0 - 4 * K) : K;
                        const int lines = (ahead * row_len + 31) >> 5;
                        for (int l = p; l < lines; l += n_prod) prefetch_l2(src + (size_t)4 * K * nstride + (size_t)l * 32);
                    }
                } else {
                    for (int jj = 0; jj < nb; jj++)
                        for (int i = p; i < row_len; i += n_prod) nbuf[jj * row_len + i] = __ldcs(src + (size_t)jj * nstride + i);
                }
            }
            named_arrive(HB_BAR_FULL0 + buf, nthreads);
        }
        // the consumers' arrivals on EMPTY after the last two blocks have no producer block to wait for
        // them; they are matched here, so that the named barriers end the point as they started (the
        // work-queue kernel runs several points in one CTA)
        for (int q = n_blocks - 2 > 0 ? n_blocks - 2 : 0; q < n_blocks; q++) named_sync(HB_BAR_EMPTY0 + (q & 1), nthreads);
    } else {
        // ================= consumers =================
        const int sweep_form = net.sub[0].sweep_form;
        float prm[HB_PSTRIDE];  // one node per thread: its row in registers
        {
            const float* pr = hb_param_row(net.sub[0], b, active[0] ? n0 + t : 0);
#pragma unroll
            for (int i = 0; i < HB_PSTRIDE; i++) prm[i] = (NPT == 1 && i < PU) ? pr[i] : 0.0f;
        }
        float rowsum[NPT];
#pragma unroll
        for (int q = 0; q < NPT; q++) rowsum[q] = (P.has_rowsums && active[q]) ? P.rowsums[n0 + t + q * n_cons] : 0.0f;
        const float dt = net.dt, dt_half = net.dt_half, h2 = net.dt_h2, h6 = net.dt_sixth;
        const int N0 = a.bold.n0;
        float bacc[NPT][HB_MAX_BOLD];
        int bcnt[NPT][HB_MAX_BOLD];
#pragma unroll
        for (int q = 0; q < NPT; q++)
#pragma unroll
            for (int m = 0; m < HB_MAX_BOLD; m++) {
                bacc[q][m] = 0.0f;
                bcnt[q][m] = 0;
                if (m < a.bold.n) {
                    bcnt[q][m] = (int)((a.s0 - a.run_s0) % a.bold.period[m]);
                    if (active[q] && !first_launch_of_run) bacc[q][m] = a.bold.acc[m][(size_t)b * N0 + n0 + t + q * n_cons];
                }
            }
        int64_t s = a.s0;
        int wpos = (int)((a.s0 + 1) % RP);
        const bool straight = NPT == 1 && PRE == PRE_ID && (integ == HBI_HEUN_STOCH || integ == HBI_HEUN_DET) &&
                              P.cfk == HBC_LINEAR && P.direct && P.pc == NCV && !P.has_rowsums && a.traj == nullptr &&
                              a.bold.n == 0;
        if (straight) {
            const int n = n0 + t;
            float nscale[8];
#pragma unroll
            for (int v = 0; v < 8; v++) nscale[v] = net.noise_scale[v];
            const bool ns_smem = a.stream_noise_smem != 0;
            float* x0 = x[0];
            float* tv0 = tv[0];
#define HB_SC(ST, SF, NS) stream_consume_heun_linear<MODEL, ST, SF, NS>(x0, tv0, prm, cp, nscale, dt, dt_half, gxbuf, nzbuf, noise_base, nstride, ring, n, t, active[0], ns, RPX, RP, wpos, a.n_steps, n_blocks, nthreads, C, hist_bar, n_cons)
            if (integ == HBI_HEUN_STOCH) {
                if (ns_smem) { if (sweep_form) HB_SC(true, true, true); else HB_SC(true, false, true); }
                else { if (sweep_form) HB_SC(true, true, false); else HB_SC(true, false, false); }
            } else {
                if (sweep_form) HB_SC(false, true, true); else HB_SC(false, false, true);
            }
#undef HB_SC
        }
        const bool kura = MODEL == HBM_KURAMOTO && PRE == PRE_KURA && (integ == HBI_HEUN_STOCH || integ == HBI_HEUN_DET) &&
                          P.cfk == HBC_KURAMOTO && P.direct;
        if constexpr (MODEL == HBM_KURAMOTO && PRE == PRE_KURA) {
            if (kura) {
                float om[NPT];
#pragma unroll
                for (int q = 0; q < NPT; q++) om[q] = NPT == 1 ? prm[0] : s_prm[(size_t)(active[q] ? t + q * n_cons : 0) * PU];
                const float nsc = net.noise_scale[0];
#define HB_SK(ST, NS) if (a.traj || a.gx_out) stream_consume_kuramoto<NPT, ST, NS, true>(HB_SK_ARGS); else stream_consume_kuramoto<NPT, ST, NS, false>(HB_SK_ARGS)
#define HB_SK_ARGS x, tv, active, om, cp[1], nsc, dt_half, gxbuf, nzbuf, noise_base, nstride, ring, n0, t, n_cons, ns, RPX, RP, wpos, s, a, b, B, nm, (size_t)net.state_len, bacc, bcnt, n_blocks, nthreads, C, hist_bar
                if (integ == HBI_HEUN_STOCH) {
                    if (a.stream_noise_smem) HB_SK(true, true);
                    else HB_SK(true, false);
                } else HB_SK(false, false);
#undef HB_SK
#undef HB_SK_ARGS
            }
        }
        const bool general = !straight && !(kura && MODEL == HBM_KURAMOTO && PRE == PRE_KURA);
        for (int blk = 0; blk < (general ? n_blocks : 0); blk++) {
            const int buf = blk & 1;
            named_sync(HB_BAR_FULL0 + buf, nthreads);
            const int it0 = blk * K;
            const int nb = (a.n_steps - it0) < K ? (a.n_steps - it0) : K;
            const float* gb = gxbuf + (size_t)buf * K * ns * PCH;
            const float* nbuf = nzbuf + (size_t)buf * K * ns * NVAR;
#pragma unroll 1
            for (int j = 0; j < nb; j++, s++) {
#pragma unroll
                for (int q = 0; q < NPT; q++) {
                    if (!active[q]) continue;
                    const int l = t + q * n_cons, n = n0 + l;  // local and network node
                    float gx[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                    for (int c = 0; c < PCH; c++) gx[c] = gb[((size_t)j * ns + l) * PCH + c];
                    if (PCH == 2 && a.gx_out)
                        __stcs(reinterpret_cast<float2*>(a.gx_out) + ((size_t)(it0 + j) * B + b) * nm + n,
                               make_float2(gx[0], gx[PCH - 1]));
                    float nz[NVAR];
#pragma unroll
                    for (int v = 0; v < NVAR; v++) {
                        if (!stoch) nz[v] = 0.0f;
                        else if (a.stream_noise_smem) nz[v] = nbuf[(size_t)j * ns * NVAR + l * NVAR + v] * net.noise_scale[v];
                        else nz[v] = __ldcs(noise_base + (size_t)(it0 + j) * nstride + n * NVAR + v) * net.noise_scale[v];
                    }
                    const float* pq = NPT == 1 ? prm : s_prm + (size_t)l * PU;
                    stream_node_step<MODEL>(P, cp, integ, pq, sweep_form, rowsum[q], gx, nz, x[q], dt, dt_half, h2, h6);
#pragma unroll
                    for (int v = 0; v < NVAR; v++) tv[q][v] = tv[q][v] + x[q][v];
                    if (a.traj) {
                        float* tr = a.traj + ((size_t)(it0 + j) * B + b) * net.state_len + (size_t)n * NVAR;
#pragma unroll
                        for (int v = 0; v < NVAR; v++) __stcs(tr + v, x[q][v]);
                    }
                    if (a.bold.n > 0) stream_bold_sample(a, b, B, n, s, x[q][0], bacc[q], bcnt[q]);
                    stream_publish<PRE, NCV, PCH>(ring, n, RPX, RP, wpos, x[q]);
                }
                wpos = (wpos + 1 == RP) ? 0 : wpos + 1;
            }
            __threadfence_block();
            named_arrive(HB_BAR_EMPTY0 + buf, nthreads);
            if (C > 1) stream_signal_block(hist_bar, blk, C, n_cons);
        }
#pragma unroll
        for (int q = 0; q < NPT; q++) {
            if (!active[q]) continue;
            bool bad = false;
#pragma unroll
            for (int v = 0; v < NVAR; v++) {
                a.state[st_base[q] + v] = x[q][v];
                a.tavg[st_base[q] + v] = tv[q][v];
                bad |= !isfinite(x[q][v]);
            }
            if (a.check_finite && bad) atomicOr(a.flags, 1);
#pragma unroll
            for (int m = 0; m < HB_MAX_BOLD; m++)
                if (m < a.bold.n) a.bold.acc[m][(size_t)b * N0 + n0 + t + q * n_cons] = bacc[q][m];
        }
    }
    // no CTA of a cluster-split point leaves while another may still arrive on its barriers
    if (C > 1) cluster_barrier();
}

template <int MODEL, int PRE, int NPT, int MAXT>
__global__ void __launch_bounds__(MAXT, 1) stream_pipe_kernel(const DevNet* __restrict__ gnet, RunArgs a) {
    __shared__ DevNet net;
    stream_load_net(net, gnet);
    __syncthreads();
    // a cluster of a.stream_cluster CTAs per point (consecutive blocks), else one CTA per point
    const int C = a.stream_cluster > 1 ? a.stream_cluster : 1;
    stream_point<MODEL, PRE, NPT, MAXT>(net, a, (int)blockIdx.x / C, C > 1 ? (int)cluster_rank() : 0);
}


// Several networks' sweeps — different models, node counts, connectomes, delays and step counts — in
// one launch of a persistent kernel: each block (or thread-block cluster) takes the next work item from
// a device counter until the items run out, and runs it through the path of the job's model and
// coupling form. Items are numbered job by job with the jobs ordered by decreasing work per item, so
// the longest start first and the short ones fill the SMs that finish early (greedy longest-first
// scheduling). The counter is zeroed before every launch.
// Launched with clusters of C CTAs, a job marked split gives each item one point whose nodes the C
// CTAs share (stream_point's cluster form: fewer points in flight, histories in L2); another job's item
// is C consecutive points, one per CTA. The cluster's first CTA takes the item and the others read it
// from its shared memory after a cluster barrier; every item ends with a cluster barrier.
__device__ __forceinline__ uint32_t cluster_size() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ int ld_remote_int(const int* p, uint32_t rank) {
    uint32_t ra;
    int v;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(smem_addr(p)), "r"(rank));
    asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(ra) : "memory");
    return v;
}
template <int NPT, int MAXT>
__global__ void __launch_bounds__(MAXT, 1) stream_queue_kernel(const StreamJob* __restrict__ jobs, int n_jobs, int n_items,
                                                              int* __restrict__ counter) {
    __shared__ DevNet net;
    __shared__ RunArgs sa;
    __shared__ int s_item, s_job;
    const int C = (int)cluster_size();
    const int rank = C > 1 ? (int)cluster_rank() : 0;
    for (;;) {
        if (threadIdx.x == 0 && rank == 0) {
            const int it = atomicAdd(counter, 1);
            int j = 0;
            while (j + 1 < n_jobs && it >= jobs[j + 1].first_block) j++;
            s_item = it;
            s_job = j;
        }
        if (C > 1) {
            cluster_barrier();
            if (threadIdx.x == 0 && rank != 0) {
                s_item = ld_remote_int(&s_item, 0);
                s_job = ld_remote_int(&s_job, 0);
            }
        }
        __syncthreads();
        const int it = s_item;
        if (it >= n_items) break;
        const StreamJob* J = jobs + s_job;
        {
            const int* src = reinterpret_cast<const int*>(&J->args);
            int* dst = reinterpret_cast<int*>(&sa);
            for (int i = threadIdx.x; i < (int)(sizeof(RunArgs) / 4); i += blockDim.x) dst[i] = src[i];
        }
        stream_load_net(net, J->net);
        __syncthreads();
        const bool split = C > 1 && J->split;
        const int local = it - J->first_block;
        const int b = split ? local : local * C + rank;
        bool ran = false;  // stream_point ran (and, on a split item, ended with its cluster barrier)
        if (b < J->n_points) {
            const int r = split ? rank : 0;
            ran = true;
            switch (J->model * 2 + (J->pre == PRE_KURA ? 1 : 0)) {
            case 0: stream_point<0, PRE_ID, NPT, MAXT>(net, sa, b, r); break;
            case 1: stream_point<0, PRE_KURA, NPT, MAXT>(net, sa, b, r); break;
            case 2: stream_point<1, PRE_ID, NPT, MAXT>(net, sa, b, r); break;
            case 4: stream_point<2, PRE_ID, NPT, MAXT>(net, sa, b, r); break;
            case 5: stream_point<2, PRE_KURA, NPT, MAXT>(net, sa, b, r); break;
            case 6: stream_point<3, PRE_ID, NPT, MAXT>(net, sa, b, r); break;
            case 7: stream_point<3, PRE_KURA, NPT, MAXT>(net, sa, b, r); break;
            case 8: stream_point<4, PRE_ID, NPT, MAXT>(net, sa, b, r); break;
            case 9: stream_point<4, PRE_KURA, NPT, MAXT>(net, sa, b, r); break;
            case 10: stream_point<5, PRE_ID, NPT, MAXT>(net, sa, b, r); break;
            case 11: stream_point<5, PRE_KURA, NPT, MAXT>(net, sa, b, r); break;
            default: ran = false; break;  // MontbrioPazoRoxin has two coupling variables: no [sin, cos] form (refused on the host)
            }
        }
        // a split point that ran ends with stream_point's cluster barrier; every other item ends with one
        // here, so no rank reads the item slot of rank 0 after rank 0 has taken the next item (every rank
        // of a split item sees the same point and job, so all of them take the same branch)
        if (C > 1 && !(split && ran)) cluster_barrier();
        __syncthreads();  // shared memory and the item slot are reused by the next item
    }
    // no CTA leaves while another may still read the first CTA's item slot
    if (C > 1) cluster_barrier();
}

template <int NPT, int MAXT>
int stream_queue_max_dynamic_smem() {
    static int cached = -1;
    if (cached >= 0) return cached;
    int dev = 0, optin = 0;
    cudaFuncAttributes fa;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&fa, stream_queue_kernel<NPT, MAXT>) != cudaSuccess) return -1;
    int maxdyn = optin - (int)fa.sharedSizeBytes;
    if (cudaFuncSetAttribute(stream_queue_kernel<NPT, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxdyn) != cudaSuccess)
        return -1;
    cached = maxdyn;
    return cached;
}

// persistent grid: as many blocks (clusters of C blocks) of the queue kernel as fit on the device at once
template <int NPT, int MAXT>
int stream_queue_grid(int threads, size_t smem, int C) {
    if (stream_queue_max_dynamic_smem<NPT, MAXT>() < 0) return -1;
    if (C > 1) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)(C * 64));
        cfg.blockDim = dim3((unsigned)threads);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)C;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, stream_queue_kernel<NPT, MAXT>, &cfg) != cudaSuccess) {
            cudaGetLastError();
            return -1;
        }
        return n * C;
    }
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, stream_queue_kernel<NPT, MAXT>, threads, smem) != cudaSuccess) return -1;
    return sms * (per_sm > 0 ? per_sm : 1);
}

template <int NPT, int MAXT>
cudaError_t launch_stream_queue(const StreamJob* d_jobs, int n_jobs, int n_items, int* counter, int blocks, int threads,
                                size_t smem, int C, cudaStream_t st) {
    int maxdyn = stream_queue_max_dynamic_smem<NPT, MAXT>();
    if (maxdyn < 0) return cudaErrorInvalidConfiguration;
    if ((long long)smem > maxdyn || threads > MAXT || blocks < 1 || C < 1 || C > 8) return cudaErrorInvalidValue;
    if (C == 1) {
        if (blocks > n_items) blocks = n_items;
        stream_queue_kernel<NPT, MAXT><<<blocks, threads, smem, st>>>(d_jobs, n_jobs, n_items, counter);
        return cudaGetLastError();
    }
    if (blocks / C > n_items) blocks = n_items * C;
    blocks = blocks / C * C;
    if (blocks < C) return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, stream_queue_kernel<NPT, MAXT>, d_jobs, n_jobs, n_items, counter);
}

template <int MODEL, int PRE, int NPT, int MAXT>
int stream_max_dynamic_smem() {
    static int cached = -1;
    if (cached >= 0) return cached;
    int dev = 0, optin = 0;
    cudaFuncAttributes fa;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&fa, stream_pipe_kernel<MODEL, PRE, NPT, MAXT>) != cudaSuccess) return -1;
    int maxdyn = optin - (int)fa.sharedSizeBytes;
    if (cudaFuncSetAttribute(stream_pipe_kernel<MODEL, PRE, NPT, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxdyn) != cudaSuccess)
        return -1;
    cached = maxdyn;
    return cached;
}

// thread-block clusters of C CTAs that can be resident at once (one point each), or -1
template <int MODEL, int PRE, int NPT, int MAXT>
int stream_cluster_capacity(int C, int threads, size_t smem) {
    if (stream_max_dynamic_smem<MODEL, PRE, NPT, MAXT>() < 0) return -1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(C * 64));
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, stream_pipe_kernel<MODEL, PRE, NPT, MAXT>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return n;
}

template <int MODEL, int PRE, int NPT, int MAXT>
cudaError_t launch_stream(const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st) {
    int maxdyn = stream_max_dynamic_smem<MODEL, PRE, NPT, MAXT>();
    if (maxdyn < 0) return cudaErrorInvalidConfiguration;
    if ((long long)smem > maxdyn || threads > MAXT) return cudaErrorInvalidValue;
    const int C = a.stream_cluster > 1 ? a.stream_cluster : 1;
    if (C == 1) {
        stream_pipe_kernel<MODEL, PRE, NPT, MAXT><<<B, threads, smem, st>>>(d_net, a);
        return cudaGetLastError();
    }
    if (C > 8) return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(B * C));
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, stream_pipe_kernel<MODEL, PRE, NPT, MAXT>, d_net, a);
}

}  // namespace hb

// one translation unit per (NPT, MAXT): nodes per consumer thread and the launch bound
cudaError_t hb_launch_stream_1(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
cudaError_t hb_launch_stream_2(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
cudaError_t hb_launch_stream_4(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
int hb_stream_budget_1(int model, int pre);
int hb_stream_clusters_1(int model, int pre, int C, int threads, size_t smem);
int hb_stream_clusters_2(int model, int pre, int C, int threads, size_t smem);
int hb_stream_clusters_4(int model, int pre, int C, int threads, size_t smem);
int hb_stream_budget_2(int model, int pre);
int hb_stream_budget_4(int model, int pre);
cudaError_t hb_launch_stream_queue_1(const StreamJob* d_jobs, int n_jobs, int n_items, int* counter, int blocks, int threads, size_t smem, int C, cudaStream_t st);
int hb_stream_queue_grid_1(int threads, size_t smem, int C);
cudaError_t hb_launch_stream_queue_2(const StreamJob* d_jobs, int n_jobs, int n_items, int* counter, int blocks, int threads, size_t smem, int C, cudaStream_t st);
int hb_stream_queue_grid_2(int threads, size_t smem, int C);
cudaError_t hb_launch_stream_queue_4(const StreamJob* d_jobs, int n_jobs, int n_items, int* counter, int blocks, int threads, size_t smem, int C, cudaStream_t st);
int hb_stream_queue_grid_4(int threads, size_t smem, int C);
int hb_stream_queue_budget_1();
int hb_stream_queue_budget_2();
int hb_stream_queue_budget_4();

#define HB_STREAM_UNIT(NPT_, MAXT_)                                                                                  \
    cudaError_t hb_launch_stream_##NPT_(int model, int pre, const DevNet* d_net, const RunArgs& a, int B,            \
                                        int threads, size_t smem, cudaStream_t st) {                                 \
        using F = cudaError_t (*)(const DevNet*, const RunArgs&, int, int, size_t, cudaStream_t);                    \
        static const F tab[12] = {                                                                                   \
            hb::launch_stream<0, hb::PRE_ID, NPT_, MAXT_>, hb::launch_stream<0, hb::PRE_KURA, NPT_, MAXT_>,          \
            hb::launch_stream<1, hb::PRE_ID, NPT_, MAXT_>, hb::launch_stream<1, hb::PRE_KURA, NPT_, MAXT_>,          \
            hb::launch_stream<2, hb::PRE_ID, NPT_, MAXT_>, hb::launch_stream<2, hb::PRE_KURA, NPT_, MAXT_>,          \
            hb::launch_stream<3, hb::PRE_ID, NPT_, MAXT_>, hb::launch_stream<3, hb::PRE_KURA, NPT_, MAXT_>,          \
            hb::launch_stream<4, hb::PRE_ID, NPT_, MAXT_>, hb::launch_stream<4, hb::PRE_KURA, NPT_, MAXT_>,          \
            hb::launch_stream<5, hb::PRE_ID, NPT_, MAXT_>, hb::launch_stream<5, hb::PRE_KURA, NPT_, MAXT_>};         \
        int i = model * 2 + (pre == hb::PRE_KURA ? 1 : 0);                                                           \
        if (i < 0 || i >= 12) return cudaErrorInvalidValue;                                                          \
        return tab[i](d_net, a, B, threads, smem, st);                                                               \
    }                                                                                                                \
    int hb_stream_clusters_##NPT_(int model, int pre, int C, int threads, size_t smem) {                             \
        using H = int (*)(int, int, size_t);                                                                         \
        static const H tab[12] = {                                                                                   \
            hb::stream_cluster_capacity<0, hb::PRE_ID, NPT_, MAXT_>, hb::stream_cluster_capacity<0, hb::PRE_KURA, NPT_, MAXT_>, \
            hb::stream_cluster_capacity<1, hb::PRE_ID, NPT_, MAXT_>, hb::stream_cluster_capacity<1, hb::PRE_KURA, NPT_, MAXT_>, \
            hb::stream_cluster_capacity<2, hb::PRE_ID, NPT_, MAXT_>, hb::stream_cluster_capacity<2, hb::PRE_KURA, NPT_, MAXT_>, \
            hb::stream_cluster_capacity<3, hb::PRE_ID, NPT_, MAXT_>, hb::stream_cluster_capacity<3, hb::PRE_KURA, NPT_, MAXT_>, \
            hb::stream_cluster_capacity<4, hb::PRE_ID, NPT_, MAXT_>, hb::stream_cluster_capacity<4, hb::PRE_KURA, NPT_, MAXT_>, \
            hb::stream_cluster_capacity<5, hb::PRE_ID, NPT_, MAXT_>, hb::stream_cluster_capacity<5, hb::PRE_KURA, NPT_, MAXT_>}; \
        int i = model * 2 + (pre == hb::PRE_KURA ? 1 : 0);                                                           \
        if (i < 0 || i >= 12) return -1;                                                                             \
        return tab[i](C, threads, smem);                                                                             \
    }                                                                                                                \
    int hb_stream_budget_##NPT_(int model, int pre) {                                                                \
        using G = int (*)();                                                                                         \
        static const G tab[12] = {                                                                                   \
            hb::stream_max_dynamic_smem<0, hb::PRE_ID, NPT_, MAXT_>, hb::stream_max_dynamic_smem<0, hb::PRE_KURA, NPT_, MAXT_>, \
            hb::stream_max_dynamic_smem<1, hb::PRE_ID, NPT_, MAXT_>, hb::stream_max_dynamic_smem<1, hb::PRE_KURA, NPT_, MAXT_>, \
            hb::stream_max_dynamic_smem<2, hb::PRE_ID, NPT_, MAXT_>, hb::stream_max_dynamic_smem<2, hb::PRE_KURA, NPT_, MAXT_>, \
            hb::stream_max_dynamic_smem<3, hb::PRE_ID, NPT_, MAXT_>, hb::stream_max_dynamic_smem<3, hb::PRE_KURA, NPT_, MAXT_>, \
            hb::stream_max_dynamic_smem<4, hb::PRE_ID, NPT_, MAXT_>, hb::stream_max_dynamic_smem<4, hb::PRE_KURA, NPT_, MAXT_>, \
            hb::stream_max_dynamic_smem<5, hb::PRE_ID, NPT_, MAXT_>, hb::stream_max_dynamic_smem<5, hb::PRE_KURA, NPT_, MAXT_>}; \
        int i = model * 2 + (pre == hb::PRE_KURA ? 1 : 0);                                                           \
        if (i < 0 || i >= 12) return -1;                                                                             \
        return tab[i]();                                                                                             \
    }

// one translation unit per (NPT, MAXT) for the work-queue kernel of grouped launches
#define HB_QUEUE_UNIT(NPT_, MAXT_)                                                                                   \
    cudaError_t hb_launch_stream_queue_##NPT_(const StreamJob* d_jobs, int n_jobs, int n_items, int* counter,        \
                                              int blocks, int threads, size_t smem, int C, cudaStream_t st) {        \
        return hb::launch_stream_queue<NPT_, MAXT_>(d_jobs, n_jobs, n_items, counter, blocks, threads, smem, C, st); \
    }                                                                                                                \
    int hb_stream_queue_budget_##NPT_() { return hb::stream_queue_max_dynamic_smem<NPT_, MAXT_>(); }                  \
    int hb_stream_queue_grid_##NPT_(int threads, size_t smem, int C) {                                               \
        return hb::stream_queue_grid<NPT_, MAXT_>(threads, smem, C);                                                 \
    }
