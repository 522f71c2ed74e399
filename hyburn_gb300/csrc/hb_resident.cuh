// hb_resident.cuh — the point-resident persistent simulation kernel (the "plain" form).
//
// One CTA owns one sweep point for a whole launch: every node of every subnetwork, `lanes`
// threads per node (warp aligned per subnetwork). State, temporal average and BOLD window sums
// stay in registers across steps. The coupling-variable history ring ([R][cols], only the cvars)
// stays in shared memory when it fits, otherwise in global memory. Each CSR edge carries a
// precomputed ring offset (source column - delay * cols), so a delayed read is one add, one
// wrap and one load. The edges of a node are split over its `lanes` lanes and the partial sums
// are combined with a butterfly; the model update is evaluated identically by all lanes of the
// node and lane 0 alone publishes results.
//
// Synchronisation: one __syncthreads per step separates publishing x_s into ring slot s % R
// from the coupling gather; R >= H + 1 so the write of step s + 1 never hits a slot that a
// slower thread may still read at step s.
//
// Template parameters: MODEL (a fixed model id, or -1 for networks mixing models) and MAXT
// (the launch bound, which sets the register budget).
#pragma once
#include <type_traits>
#include <cuda_runtime.h>
#include "hb_models.cuh"

namespace hb {

enum { PRE_ID = 0, PRE_KURA = 1, PRE_GEN = 2 };

__device__ __forceinline__ int wrap_add(int a, int wrap) { return a < 0 ? a + wrap : a; }

// noise rows are fetched into L2 this many steps ahead of their use
#define HB_NOISE_L2_AHEAD 8

__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// single-delay projection at step s: false when the source rows are the zero tensor (zeros before
// pre(), engine.rs:580-584 / runtime.rs:246-249); dd is the read-back distance in steps
__device__ __forceinline__ bool single_delay(const DevProj& P, int64_t s, int H, int& dd) {
    int d = P.delay;
    if (d == 0 || s == 0) { dd = 0; return true; }
    if ((int64_t)d > s) return false;
    if (P.dmode == HBD_COMPAT) {
        // window index (s - d + H) % H of the shift-window history holds x_{s+1+idx-H}
        dd = H - 1 - (int)((s - d) % H);
        return (int64_t)dd <= s;
    }
    dd = d;
    return true;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ int lower_bound_emit(const BoldEmit* e, int n, int k) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (e[mid].k < k) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// gx[c] += sum over edges e = e0 + lane, e0 + lane + L, ... of w_e * pre(ring[base + off_e])
template <int PRE>
__device__ __forceinline__ void gather(const float* __restrict__ ring, const int* __restrict__ eoff,
                                       const float* __restrict__ ew, int e0, int e1, int lane, int L, int base,
                                       int wrap, int ncv, int cfk, const float* cp, int cpu_form, float* gx) {
    if (PRE == PRE_ID) {
        float a0 = 0.0f, a1 = 0.0f;
        if (ncv == 1) {
#pragma unroll 4
            for (int e = e0 + lane; e < e1; e += L) {
                int a = wrap_add(base + eoff[e], wrap);
                a0 += ew[e] * ring[a];
            }
        } else {
#pragma unroll 2
            for (int e = e0 + lane; e < e1; e += L) {
                int a = wrap_add(base + eoff[e], wrap);
                float w = ew[e];
                a0 += w * ring[a];
                a1 += w * ring[a + 1];
            }
        }
        gx[0] += a0;
        gx[1] += a1;
    } else if (PRE == PRE_KURA) {  // one cvar: [sin, cos]
        float a0 = 0.0f, a1 = 0.0f;
#pragma unroll 2
        for (int e = e0 + lane; e < e1; e += L) {
            int a = wrap_add(base + eoff[e], wrap);
            float w = ew[e], v = ring[a];
            a0 += w * sinf(v);
            a1 += w * cosf(v);
        }
        gx[0] += a0;
        gx[1] += a1;
    } else {
        for (int e = e0 + lane; e < e1; e += L) {
            int a = wrap_add(base + eoff[e], wrap);
            float cv[2] = {ring[a], ncv > 1 ? ring[a + 1] : 0.0f}, pv[4] = {0.f, 0.f, 0.f, 0.f};
            pre(cfk, cp, cpu_form, cv, ncv, pv);
            float w = ew[e];
#pragma unroll
            for (int c = 0; c < 4; c++) gx[c] += w * pv[c];
        }
    }
}

// per-edge delays during the first max-delay steps: the delay of every edge is checked (zero rows
// after pre() for d > s, current state for d == 0 or s == 0, runtime.rs:166-176)
__device__ __forceinline__ void gather_early(const float* __restrict__ ring, const DevProj& P, int e0, int e1,
                                             int lane, int L, int64_t s, int slot, int R, int cols, int scol,
                                             int sncv, const float* cp, float* gx) {
    for (int e = e0 + lane; e < e1; e += L) {
        uint32_t m = P.edges[e];
        int d = (int)(m >> 16), src = (int)(m & 0xffffu);
        int dd = d;
        if (d == 0 || s == 0) dd = 0;
        else if ((int64_t)d > s) continue;
        int row = slot - dd;
        row = row < 0 ? row + R : row;
        const float* rr = ring + row * cols + scol + src * sncv;
        float cv[2] = {rr[0], P.ncv > 1 ? rr[1] : 0.0f}, pv[4] = {0.f, 0.f, 0.f, 0.f};
        pre(P.cfk, cp, P.pre_cpu, cv, P.ncv, pv);
        float w = P.ew[e];
#pragma unroll
        for (int c = 0; c < 4; c++) gx[c] += w * pv[c];
    }
}

template <int MODEL, int MAXT>
__global__ void __launch_bounds__(MAXT, 1) resident_kernel(const DevNet* __restrict__ gnet, RunArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ DevNet net;
    {
        const int* src = reinterpret_cast<const int*>(gnet);
        int* dst = reinterpret_cast<int*>(&net);
        for (int i = threadIdx.x; i < (int)(sizeof(DevNet) / 4); i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();

    const int b = blockIdx.x;
    const int t = threadIdx.x;
    const int wlane = t & 31, warp = t >> 5;
    const int R = net.R, cols = net.cols, H = net.H, B = net.B;
    const int ring_words = R * cols;
    const size_t ring_stride = (size_t)((ring_words + 3) & ~3);  // per-point stride, 16-byte aligned

    size_t off = 0;
    float* ring;
    if (a.ring_in_smem) { ring = reinterpret_cast<float*>(smem); off = (size_t)ring_words * sizeof(float); }
    else ring = a.ring + (size_t)b * ring_stride;
    off = (off + 15) & ~(size_t)15;
    int* s_eoff = reinterpret_cast<int*>(smem + off);
    off += (size_t)a.smem_edges * 4;
    float* s_ew = reinterpret_cast<float*>(smem + off);
    off += (size_t)a.smem_edges * 4;
    off = (off + 15) & ~(size_t)15;
    float* s_part = reinterpret_cast<float*>(smem + off);  // [2][n_mean][32 warps][4]

    if (a.ring_in_smem && a.load_ring) {
        const float4* g = reinterpret_cast<const float4*>(a.ring + (size_t)b * ring_stride);
        float4* r4 = reinterpret_cast<float4*>(ring);
        const int n4 = ring_words >> 2;
        for (int i = t; i < n4; i += blockDim.x) r4[i] = g[i];
        for (int i = (n4 << 2) + t; i < ring_words; i += blockDim.x) ring[i] = a.ring[(size_t)b * ring_stride + i];
    }
    for (int p = 0; p < net.n_proj; p++) {
        const DevProj& P = net.proj[p];
        if (P.kind != HBK_SPARSE || P.smem_edges < 0) continue;
        const int nnz = P.rowptr[P.ntgt];
        for (int i = t; i < nnz; i += blockDim.x) {
            s_eoff[P.smem_edges + i] = P.eoff[i];
            s_ew[P.smem_edges + i] = P.ew[i];
        }
    }

    // ---- role: lane `lane` of node n of subnetwork k ----
    int k = 0;
    for (int i = 1; i < net.n_sub; i++)
        if (t >= net.sub[i].thread_off) k = i;
    const int model = MODEL >= 0 ? MODEL : net.sub[k].model;
    const int nm = net.sub[k].nm, nvar = MODEL >= 0 ? c_nvar(MODEL) : net.sub[k].nvar;
    const int ncvar = MODEL >= 0 ? c_ncvar(MODEL) : net.sub[k].ncvar;
    const int L = net.sub[k].lanes;
    const int local = t - net.sub[k].thread_off;
    const int n = local >> net.sub[k].lanes_log2;
    const int lane = local & (L - 1);
    const bool active = n < nm;
    const bool lead = active && lane == 0;
    const int nn = active ? n : 0;
    const int col_off = net.sub[k].col_off, integ = net.sub[k].integ, sweep_form = net.sub[k].sweep_form;
    const int mycol = col_off + nn * ncvar;

    float prm[HB_PSTRIDE];
    {
        const float* pr = hb_param_row(net.sub[k], b, nn);
#pragma unroll
        for (int i = 0; i < HB_PSTRIDE; i++) prm[i] = (i < c_nparams_used(MODEL)) ? pr[i] : 0.0f;
    }
    float x[6], tv[6];
    const size_t st_base = (size_t)b * net.state_len + net.sub[k].state_off + (size_t)nn * nvar;
    const bool first_launch_of_run = (a.s0 == a.run_s0);
#pragma unroll
    for (int v = 0; v < 6; v++) {
        x[v] = (active && v < nvar) ? a.state[st_base + v] : 0.0f;
        tv[v] = (active && v < nvar && !first_launch_of_run) ? a.tavg[st_base + v] : 0.0f;
    }
    // row bounds of the incoming sparse projections
    const int n_in = net.sub[k].n_in;
    int re0[HB_MAX_IN], re1[HB_MAX_IN];
#pragma unroll
    for (int q = 0; q < HB_MAX_IN; q++) {
        re0[q] = re1[q] = 0;
        if (q < n_in) {
            const DevProj& P = net.proj[net.sub[k].in_idx[q]];
            if (P.kind == HBK_SPARSE && active) { re0[q] = P.rowptr[n]; re1[q] = P.rowptr[n + 1]; }
        }
    }
    // noise stream of this node
    const bool stoch = (integ == HBI_EULER_STOCH || integ == HBI_HEUN_STOCH || integ == HBI_RK4_STOCH);
    const float* nptr = a.noise + (a.noise_per_point ? (size_t)b * net.noise_row : 0) + net.sub[k].noise_off + (size_t)nn * nvar;
    const size_t nstride = (size_t)(a.noise_per_point ? B : 1) * net.noise_row;
    float nz_next[6];
#pragma unroll
    for (int v = 0; v < 6; v++) nz_next[v] = (stoch && active && v < nvar) ? __ldcs(nptr + v) : 0.0f;
    // BOLD (subnetwork 0, nmodes == 1)
    const bool bold_thread = (k == 0) && lead && a.bold.n > 0;
    const int N0 = a.bold.n0;
    float bacc[HB_MAX_BOLD];
    int bcnt[HB_MAX_BOLD];
#pragma unroll
    for (int m = 0; m < HB_MAX_BOLD; m++) {
        bacc[m] = 0.0f;
        bcnt[m] = 0;
        if (m < a.bold.n) {
            bcnt[m] = (int)((a.s0 - a.run_s0) % a.bold.period[m]);
            if (bold_thread && !first_launch_of_run) bacc[m] = a.bold.acc[m][(size_t)b * N0 + n];
        }
    }
    __syncthreads();

    int64_t s = a.s0;
    int slot = (int)(s % R);
    const int n_mean = net.n_mean;
    for (int it = 0; it < a.n_steps; ++it, ++s) {
        const int buf = it & 1;
        // ---- 1. publish x_s (first ncvar state vars, engine.rs:570) into ring slot s % R ----
        if (lead) {
            ring[slot * cols + mycol] = x[0];
            if (ncvar > 1) ring[slot * cols + mycol + 1] = x[1];
        }
        // ---- mean-field partial sums of projections whose source is this subnetwork ----
        for (int q = 0; q < net.sub[k].n_mean_out; q++) {
            const DevProj& P = net.proj[net.sub[k].mean_out[q]];
            const float* cp = P.cp_pp ? P.cp_pp + (size_t)b * HB_NCP : P.cp;
            float pv[4] = {0.f, 0.f, 0.f, 0.f};
            int dd;
            bool ok = single_delay(P, s, H, dd);
            if (lead) {
                float cv[2] = {0.0f, 0.0f};
                if (ok) {
                    int row = slot - dd;
                    row = row < 0 ? row + R : row;
                    cv[0] = dd == 0 ? x[0] : ring[row * cols + mycol];
                    if (P.ncv > 1) cv[1] = dd == 0 ? x[1] : ring[row * cols + mycol + 1];
                }
                pre(P.cfk, cp, 0, cv, P.ncv, pv);
            }
#pragma unroll
            for (int c = 0; c < 4; c++) {
                if (c < P.pc) {
                    float sum = warp_sum(pv[c]);
                    if (wlane == 0) s_part[((buf * n_mean + P.mean_slot) * 32 + warp) * 4 + c] = sum;
                }
            }
        }
        // noise of this step was prefetched one step ahead
        float nz[6];
#pragma unroll
        for (int v = 0; v < 6; v++) nz[v] = nz_next[v] * net.noise_scale[v];
        if (stoch && it + 1 < a.n_steps) {
            nptr += nstride;
#pragma unroll
            for (int v = 0; v < 6; v++) nz_next[v] = (active && v < nvar) ? __ldcs(nptr + v) : 0.0f;
            if (lead && it + HB_NOISE_L2_AHEAD < a.n_steps) prefetch_l2(nptr + (HB_NOISE_L2_AHEAD - 1) * nstride);
        }
        __syncthreads();

        // ---- 2. coupling into this subnetwork (engine.rs:557-674) ----
        float cc[2] = {0.0f, 0.0f};
#pragma unroll
        for (int q = 0; q < HB_MAX_IN; q++) {
            if (q >= n_in) break;
            const DevProj& P = net.proj[net.sub[k].in_idx[q]];
            const float* cp = P.cp_pp ? P.cp_pp + (size_t)b * HB_NCP : P.cp;
            const int scol = net.sub[P.src].col_off, sncv = net.sub[P.src].ncvar;
            float gx[4] = {0.f, 0.f, 0.f, 0.f};
            if (P.kind == HBK_MEAN) {
                const int w0 = net.sub[P.src].thread_off >> 5;
                const int w1 = (net.sub[P.src].thread_off + P.nsrc * net.sub[P.src].lanes + 31) >> 5;
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    if (c < P.pc) {
                        float acc = 0.0f;
                        for (int w = w0; w < w1; w++) acc += s_part[((buf * n_mean + P.mean_slot) * 32 + w) * 4 + c];
                        gx[c] = (acc / (float)P.nsrc) * P.w;
                    }
                }
            } else if (P.kind == HBK_DIAG) {
                int dd;
                bool ok = single_delay(P, s, H, dd);
                int row = slot - (ok ? dd : 0);
                row = row < 0 ? row + R : row;
                const float* rr = ring + row * cols + scol + nn * sncv;
                float cv[2] = {ok ? rr[0] : 0.0f, (ok && P.ncv > 1) ? rr[1] : 0.0f}, pv[4] = {0.f, 0.f, 0.f, 0.f};
                pre(P.cfk, cp, 0, cv, P.ncv, pv);
#pragma unroll
                for (int c = 0; c < 4; c++) gx[c] = P.w * pv[c];
            } else {
                const int* eo = P.smem_edges >= 0 ? s_eoff + P.smem_edges : P.eoff;
                const float* ew = P.smem_edges >= 0 ? s_ew + P.smem_edges : P.ew;
                const int pk = (P.cfk == HBC_KURAMOTO && P.ncv == 1) ? PRE_KURA
                             : ((P.cfk == HBC_TANH || P.cfk == HBC_SJR || P.cfk == HBC_PRESIG || P.cfk == HBC_KURAMOTO) ? PRE_GEN : PRE_ID);
                if (P.dmode == HBD_EDGE) {
                    if (s < (int64_t)P.maxd || s == 0) {
                        gather_early(ring, P, re0[q], re1[q], lane, L, s, slot, R, cols, scol, sncv, cp, gx);
                    } else {
                        const int base = slot * cols;
                        if (pk == PRE_ID) gather<PRE_ID>(ring, eo, ew, re0[q], re1[q], lane, L, base, ring_words, P.ncv, P.cfk, cp, P.pre_cpu, gx);
                        else if (pk == PRE_KURA) gather<PRE_KURA>(ring, eo, ew, re0[q], re1[q], lane, L, base, ring_words, P.ncv, P.cfk, cp, P.pre_cpu, gx);
                        else gather<PRE_GEN>(ring, eo, ew, re0[q], re1[q], lane, L, base, ring_words, P.ncv, P.cfk, cp, P.pre_cpu, gx);
                    }
                } else {
                    int dd;
                    bool ok = single_delay(P, s, H, dd);
                    if (ok) {
                        int row = slot - dd;
                        row = row < 0 ? row + R : row;
                        const int base = row * cols;
                        if (pk == PRE_ID) gather<PRE_ID>(ring, eo, ew, re0[q], re1[q], lane, L, base, 0, P.ncv, P.cfk, cp, 0, gx);
                        else if (pk == PRE_KURA) gather<PRE_KURA>(ring, eo, ew, re0[q], re1[q], lane, L, base, 0, P.ncv, P.cfk, cp, 0, gx);
                        else gather<PRE_GEN>(ring, eo, ew, re0[q], re1[q], lane, L, base, 0, P.ncv, P.cfk, cp, 0, gx);
                    } else {
                        // every source row is the zero tensor: sum of w_e * pre(0) in edge order
                        float zero[2] = {0.0f, 0.0f}, pz[4] = {0.f, 0.f, 0.f, 0.f};
                        pre(P.cfk, cp, 0, zero, P.ncv, pz);
                        for (int e = re0[q] + lane; e < re1[q]; e += L) {
                            float w = ew[e];
#pragma unroll
                            for (int c = 0; c < 4; c++) gx[c] += w * pz[c];
                        }
                    }
                }
                // combine the lanes of this node
                for (int o = L >> 1; o > 0; o >>= 1) {
#pragma unroll
                    for (int c = 0; c < 4; c++) gx[c] += __shfl_xor_sync(0xffffffffu, gx[c], o);
                }
            }
            if (active) {
                float out[4] = {0.f, 0.f, 0.f, 0.f};
                float rs = P.has_rowsums ? P.rowsums[n] : 0.0f;
                int oc = post(P.cfk, cp, P.has_rowsums, gx, P.pc, x, ncvar, rs, out);
                if (P.direct) {
                    cc[0] = cc[0] + out[0];
                    if (ncvar > 1 && oc > 1) cc[1] = cc[1] + out[1];
                } else {
                    float t0 = 0.0f, t1 = 0.0f;
                    for (int j = 0; j < P.ncm; j++) {
                        int sidx = P.cm_s[j], cpl = P.cm_cpl[j];
                        if (sidx < sncv && cpl < ncvar) {
                            float o = pick4(out, sidx);
                            if (cpl == 0) t0 += o; else t1 += o;
                        }
                    }
                    cc[0] = cc[0] + t0;
                    if (ncvar > 1) cc[1] = cc[1] + t1;
                }
            }
        }

        // ---- 3. integrate (engine.rs:677-783) ----
        if (active) {
            float k1[6], k2[6], tmp[6];
            const float dt = net.dt;
            dfun_m<MODEL>(model, prm, sweep_form, x, cc, k1);
            switch (integ) {
            case HBI_HEUN_DET:
#pragma unroll
                for (int v = 0; v < 6; v++) tmp[v] = x[v] + k1[v] * dt;
                clamp_m<MODEL>(model, tmp);
                dfun_m<MODEL>(model, prm, sweep_form, tmp, cc, k2);
#pragma unroll
                for (int v = 0; v < 6; v++) x[v] = x[v] + (k1[v] + k2[v]) * net.dt_half;
                break;
            case HBI_EULER:
#pragma unroll
                for (int v = 0; v < 6; v++) x[v] = x[v] + k1[v] * dt;
                break;
            case HBI_EULER_STOCH:
#pragma unroll
                for (int v = 0; v < 6; v++) x[v] = (x[v] + k1[v] * dt) + nz[v];
                break;
            case HBI_HEUN_STOCH:
#pragma unroll
                for (int v = 0; v < 6; v++) tmp[v] = (x[v] + k1[v] * dt) + nz[v];
                clamp_m<MODEL>(model, tmp);
                dfun_m<MODEL>(model, prm, sweep_form, tmp, cc, k2);
#pragma unroll
                for (int v = 0; v < 6; v++) x[v] = (x[v] + (k1[v] + k2[v]) * net.dt_half) + nz[v];
                break;
            default: {  // RK4 / RK4 stochastic
                float k3[6], k4[6];
                const float h2 = net.dt_h2, h6 = net.dt_sixth;
#pragma unroll
                for (int v = 0; v < 6; v++) tmp[v] = x[v] + k1[v] * h2;
                clamp_m<MODEL>(model, tmp);
                dfun_m<MODEL>(model, prm, sweep_form, tmp, cc, k2);
#pragma unroll
                for (int v = 0; v < 6; v++) tmp[v] = x[v] + k2[v] * h2;
                clamp_m<MODEL>(model, tmp);
                dfun_m<MODEL>(model, prm, sweep_form, tmp, cc, k3);
#pragma unroll
                for (int v = 0; v < 6; v++) tmp[v] = x[v] + k3[v] * dt;
                clamp_m<MODEL>(model, tmp);
                dfun_m<MODEL>(model, prm, sweep_form, tmp, cc, k4);
#pragma unroll
                for (int v = 0; v < 6; v++) {
                    float sacc = k1[v] + k2[v] * 2.0f;
                    sacc = sacc + k3[v] * 2.0f;
                    sacc = sacc + k4[v];
                    x[v] = x[v] + sacc * h6;
                }
                if (integ == HBI_RK4_STOCH) {
#pragma unroll
                    for (int v = 0; v < 6; v++) x[v] = x[v] + nz[v];
                }
                break;
            }
            }
            clamp_m<MODEL>(model, x);
#pragma unroll
            for (int v = 0; v < 6; v++) tv[v] = tv[v] + x[v];
            if (a.traj && lane == 0) {
                float* tr = a.traj + ((size_t)it * B + b) * net.state_len + net.sub[k].state_off + (size_t)n * nvar;
#pragma unroll
                for (int v = 0; v < 6; v++) if (v < nvar) __stcs(tr + v, x[v]);
            }
        }

        // ---- 4. BOLD monitors on var0 of subnetwork 0 (engine.rs:786-801) ----
        if (bold_thread) {
            const int64_t rel = s - a.run_s0;
#pragma unroll
            for (int m = 0; m < HB_MAX_BOLD; m++) {
                if (m >= a.bold.n) break;
                bacc[m] = bacc[m] + x[0];
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
                    for (int j = lower_bound_emit(em, a.bold.n_emit[m], kk); j < a.bold.n_emit[m] && em[j].k == kk; j++) {
                        float val = em[j].interp ? prev + (cur - prev) * em[j].w : cur;
                        a.bold.out[m][((size_t)b * a.bold.n_out_run[m] + em[j].out) * N0 + n] = val;
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
        slot = (slot + 1 == R) ? 0 : slot + 1;
    }

    // ---- launch end: persist state, running sums and the shared ring ----
    if (lead) {
        bool bad = false;
#pragma unroll
        for (int v = 0; v < 6; v++) {
            if (v < nvar) {
                a.state[st_base + v] = x[v];
                a.tavg[st_base + v] = tv[v];
                bad |= !isfinite(x[v]);
            }
        }
        if (a.check_finite && bad) atomicOr(a.flags, 1);
    }
    if (bold_thread) {
#pragma unroll
        for (int m = 0; m < HB_MAX_BOLD; m++)
            if (m < a.bold.n) a.bold.acc[m][(size_t)b * N0 + n] = bacc[m];
    }
    if (a.ring_in_smem && a.store_ring) {
        __syncthreads();
        float4* g = reinterpret_cast<float4*>(a.ring + (size_t)b * ring_stride);
        const float4* r4 = reinterpret_cast<const float4*>(ring);
        const int n4 = ring_words >> 2;
        for (int i = t; i < n4; i += blockDim.x) g[i] = r4[i];
        for (int i = (n4 << 2) + t; i < ring_words; i += blockDim.x) a.ring[(size_t)b * ring_stride + i] = ring[i];
    }
}

// ---------------------------------------------------------------------------------------------
// Specialised form for the dominant network shape: one subnetwork coupled to itself through one
// sparse (CSR or dense) projection whose pre() is the identity or Kuramoto's [sin, cos]. The
// projection's constants, the point's coupling parameters and the node's row bounds live in
// registers; the step is publish -> barrier -> lane-split gather -> butterfly -> post -> update.
// ---------------------------------------------------------------------------------------------
template <int MODEL, int PRE, int MAXT>
__global__ void __launch_bounds__(MAXT, 1) resident_fast_kernel(const DevNet* __restrict__ gnet, RunArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ DevNet net;
    {
        const int* src = reinterpret_cast<const int*>(gnet);
        int* dst = reinterpret_cast<int*>(&net);
        for (int i = threadIdx.x; i < (int)(sizeof(DevNet) / 4); i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    constexpr int NVAR = c_nvar(MODEL), NCV = c_ncvar(MODEL);
    const int b = blockIdx.x, t = threadIdx.x;
    const int R = net.R, cols = net.cols, H = net.H, B = net.B;
    const int ring_words = R * cols;
    const size_t ring_stride = (size_t)((ring_words + 3) & ~3);
    const DevProj& P = net.proj[0];

    size_t off = 0;
    float* ring;
    if (a.ring_in_smem) { ring = reinterpret_cast<float*>(smem); off = (size_t)ring_words * sizeof(float); }
    else ring = a.ring + (size_t)b * ring_stride;
    off = (off + 15) & ~(size_t)15;
    int* s_eoff = reinterpret_cast<int*>(smem + off);
    off += (size_t)a.smem_edges * 4;
    float* s_ew = reinterpret_cast<float*>(smem + off);

    if (a.ring_in_smem && a.load_ring) {
        const float4* g = reinterpret_cast<const float4*>(a.ring + (size_t)b * ring_stride);
        float4* r4 = reinterpret_cast<float4*>(ring);
        const int n4 = ring_words >> 2;
        for (int i = t; i < n4; i += blockDim.x) r4[i] = g[i];
        for (int i = (n4 << 2) + t; i < ring_words; i += blockDim.x) ring[i] = a.ring[(size_t)b * ring_stride + i];
    }
    const bool edges_smem = P.smem_edges >= 0;
    if (edges_smem) {
        const int nnz = P.rowptr[P.ntgt];
        for (int i = t; i < nnz; i += blockDim.x) { s_eoff[i] = P.eoff[i]; s_ew[i] = P.ew[i]; }
    }
    const int* __restrict__ eo = edges_smem ? s_eoff : P.eoff;
    const float* __restrict__ ew = edges_smem ? s_ew : P.ew;

    const int L = net.sub[0].lanes;
    const int n = t >> net.sub[0].lanes_log2;
    const int lane = t & (L - 1);
    const int nm = net.sub[0].nm;
    const bool active = n < nm;
    const bool lead = active && lane == 0;
    const int nn = active ? n : 0;
    const int mycol = nn * NCV;
    const int integ = net.sub[0].integ, sweep_form = net.sub[0].sweep_form;
    const int cfk = P.cfk, pc = P.pc, direct = P.direct, dmode = P.dmode, maxd = P.maxd, has_rowsums = P.has_rowsums;

    float prm[HB_PSTRIDE];
    {
        const float* pr = hb_param_row(net.sub[0], b, nn);
#pragma unroll
        for (int i = 0; i < HB_PSTRIDE; i++) prm[i] = (i < c_nparams_used(MODEL)) ? pr[i] : 0.0f;
    }
    float cp[8];
    {
        const float* c = P.cp_pp ? P.cp_pp + (size_t)b * HB_NCP : P.cp;
#pragma unroll
        for (int i = 0; i < 8; i++) cp[i] = c[i];
    }
    const float rowsum = (has_rowsums && active) ? P.rowsums[n] : 0.0f;
    const int e0 = active ? P.rowptr[n] : 0, e1 = active ? P.rowptr[n + 1] : 0;

    float x[NVAR], tv[NVAR];
    const size_t st_base = (size_t)b * net.state_len + (size_t)nn * NVAR;
    const bool first_launch_of_run = (a.s0 == a.run_s0);
#pragma unroll
    for (int v = 0; v < NVAR; v++) {
        x[v] = active ? a.state[st_base + v] : 0.0f;
        tv[v] = (active && !first_launch_of_run) ? a.tavg[st_base + v] : 0.0f;
    }
    const bool stoch = (integ == HBI_EULER_STOCH || integ == HBI_HEUN_STOCH || integ == HBI_RK4_STOCH);
    const float* nptr = a.noise + (a.noise_per_point ? (size_t)b * net.noise_row : 0) + (size_t)nn * NVAR;
    const size_t nstride = (size_t)(a.noise_per_point ? B : 1) * net.noise_row;
    float nscale[NVAR];
#pragma unroll
    for (int v = 0; v < NVAR; v++) nscale[v] = net.noise_scale[v];
    const bool bold_thread = lead && a.bold.n > 0;
    const int N0 = a.bold.n0;
    float bacc[HB_MAX_BOLD];
    int bcnt[HB_MAX_BOLD];
#pragma unroll
    for (int m = 0; m < HB_MAX_BOLD; m++) {
        bacc[m] = 0.0f;
        bcnt[m] = 0;
        if (m < a.bold.n) {
            bcnt[m] = (int)((a.s0 - a.run_s0) % a.bold.period[m]);
            if (bold_thread && !first_launch_of_run) bacc[m] = a.bold.acc[m][(size_t)b * N0 + n];
        }
    }
    const float dt = net.dt, dt_half = net.dt_half, h2 = net.dt_h2, h6 = net.dt_sixth;
    __syncthreads();

    // ---- time loop ----
    // Every edge delay is >= sync_every, so the coupling of a block of KBLK <= sync_every steps
    // [s0, s0 + KBLK) reads only times < s0 (or time 0 at s == 0), all published before the block's
    // barrier, and R >= H + KBLK keeps a warp that runs ahead off the slots a slower warp still
    // reads. Two loop shapes: per-step (gather then update, one step at a time) and two-phase
    // (phase A issues all gathers and noise loads of the block at once, phase B runs the serial
    // updates from a register queue).
    constexpr int PCH = (PRE == PRE_KURA) ? 2 : NCV;
    constexpr int KB = (NVAR <= 2) ? 8 : 4;
    const bool two_phase = a.two_phase != 0;
    const int KBLK = two_phase ? (a.sync_every < KB ? a.sync_every : KB) : a.sync_every;
    int64_t s = a.s0;
    int slot = (int)(s % R);
    if (lead) {
        ring[slot * cols + mycol] = x[0];
        if (NCV > 1) ring[slot * cols + mycol + 1] = x[1];
    }
    auto coupling_sum = [&](int64_t sj, int sl, float* gx) {
        if (dmode == HBD_EDGE) {
            if (sj < (int64_t)maxd || sj == 0) gather_early(ring, P, e0, e1, lane, L, sj, sl, R, cols, 0, NCV, cp, gx);
            else gather<PRE>(ring, eo, ew, e0, e1, lane, L, sl * cols, ring_words, NCV, cfk, cp, P.pre_cpu, gx);
        } else {
            int dd;
            if (single_delay(P, sj, H, dd)) {
                int row = sl - dd;
                row = row < 0 ? row + R : row;
                gather<PRE>(ring, eo, ew, e0, e1, lane, L, row * cols, 0, NCV, cfk, cp, 0, gx);
            } else {
                float zero[2] = {0.0f, 0.0f}, pz[4] = {0.f, 0.f, 0.f, 0.f};
                pre(cfk, cp, 0, zero, NCV, pz);
                for (int e = e0 + lane; e < e1; e += L) {
                    float w = ew[e];
#pragma unroll
                    for (int c = 0; c < 4; c++) gx[c] += w * pz[c];
                }
            }
        }
    };
    // one model step from the coupling sums gx and the scaled noise nz; publishes x_{s+1}
    auto update = [&](const float* gx, const float* nz, int it, int64_t sj, int sl_next) {
        float cc[2] = {0.0f, 0.0f};
        {
            float out[4] = {0.f, 0.f, 0.f, 0.f};
            float xi[2] = {x[0], NCV > 1 ? x[NCV - 1] : 0.0f};
            int oc = post(cfk, cp, has_rowsums, gx, pc, xi, NCV, rowsum, out);
            if (direct) {
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
#pragma unroll
        for (int v = 0; v < NVAR; v++) tv[v] = tv[v] + x[v];
        if (a.traj && lead) {
            float* tr = a.traj + ((size_t)it * B + b) * net.state_len + (size_t)n * NVAR;
#pragma unroll
            for (int v = 0; v < NVAR; v++) __stcs(tr + v, x[v]);
        }
        if (bold_thread) {
            const int64_t rel = sj - a.run_s0;
#pragma unroll
            for (int m = 0; m < HB_MAX_BOLD; m++) {
                if (m >= a.bold.n) break;
                bacc[m] = bacc[m] + x[0];
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
        if (lead) {
            ring[sl_next * cols + mycol] = x[0];
            if (NCV > 1) ring[sl_next * cols + mycol + 1] = x[1];
        }
    };

    if (!two_phase) {
        int until_sync = 0;
        for (int it = 0; it < a.n_steps; ++it, ++s) {
            if (until_sync == 0) {
                __syncthreads();
                until_sync = KBLK;
            }
            --until_sync;
            float gx[4] = {0.f, 0.f, 0.f, 0.f};
            coupling_sum(s, slot, gx);
            float nz[NVAR];
            if (stoch) {
                const float* np = nptr + (size_t)it * nstride;
#pragma unroll
                for (int v = 0; v < NVAR; v++) nz[v] = active ? __ldcs(np + v) * nscale[v] : 0.0f;
                if (lead && it + HB_NOISE_L2_AHEAD < a.n_steps) prefetch_l2(np + HB_NOISE_L2_AHEAD * nstride);
            } else {
#pragma unroll
                for (int v = 0; v < NVAR; v++) nz[v] = 0.0f;
            }
            for (int o = L >> 1; o > 0; o >>= 1) {
#pragma unroll
                for (int c = 0; c < PCH; c++) gx[c] += __shfl_xor_sync(0xffffffffu, gx[c], o);
            }
            const int sl1 = (slot + 1 == R) ? 0 : slot + 1;
            update(gx, nz, it, s, sl1);
            slot = sl1;
        }
    } else {
        for (int it0 = 0; it0 < a.n_steps; it0 += KBLK) {
            const int nb = (a.n_steps - it0) < KBLK ? (a.n_steps - it0) : KBLK;
            __syncthreads();
            // phase A: coupling sums and noise of the block, into a register queue
            float gxs[KB][PCH];
            float nzs[KB][NVAR];
#pragma unroll
            for (int j = 0; j < KB; j++) {
                float gx[4] = {0.f, 0.f, 0.f, 0.f};
                if (j < nb) {
                    int sl = slot + j;
                    sl = sl >= R ? sl - R : sl;
                    coupling_sum(s + j, sl, gx);
                }
#pragma unroll
                for (int c = 0; c < PCH; c++) gxs[j][c] = gx[c];
#pragma unroll
                for (int v = 0; v < NVAR; v++)
                    nzs[j][v] = (stoch && active && j < nb) ? __ldcs(nptr + (size_t)(it0 + j) * nstride + v) * nscale[v] : 0.0f;
            }
            if (stoch && lead && it0 + KBLK * HB_NOISE_L2_AHEAD < a.n_steps)
                prefetch_l2(nptr + (size_t)(it0 + KBLK * HB_NOISE_L2_AHEAD) * nstride);
            if (L > 1) {
#pragma unroll
                for (int j = 0; j < KB; j++) {
                    for (int o = L >> 1; o > 0; o >>= 1) {
#pragma unroll
                        for (int c = 0; c < PCH; c++) gxs[j][c] += __shfl_xor_sync(0xffffffffu, gxs[j][c], o);
                    }
                }
            }
            // phase B: serial updates, popping the queue front (not unrolled: one copy of the update)
#pragma unroll 1
            for (int j = 0; j < nb; j++) {
                float gx[4] = {0.f, 0.f, 0.f, 0.f}, nz[NVAR];
#pragma unroll
                for (int c = 0; c < PCH; c++) gx[c] = gxs[0][c];
#pragma unroll
                for (int v = 0; v < NVAR; v++) nz[v] = nzs[0][v];
#pragma unroll
                for (int q = 0; q < KB - 1; q++) {
#pragma unroll
                    for (int c = 0; c < PCH; c++) gxs[q][c] = gxs[q + 1][c];
#pragma unroll
                    for (int v = 0; v < NVAR; v++) nzs[q][v] = nzs[q + 1][v];
                }
                int sl1 = slot + j + 1;
                sl1 = sl1 >= R ? sl1 - R : sl1;
                update(gx, nz, it0 + j, s + j, sl1);
            }
            s += nb;
            slot += nb;
            slot = slot >= R ? slot - R : slot;
        }
    }

    if (lead) {
        bool bad = false;
#pragma unroll
        for (int v = 0; v < NVAR; v++) {
            a.state[st_base + v] = x[v];
            a.tavg[st_base + v] = tv[v];
            bad |= !isfinite(x[v]);
        }
        if (a.check_finite && bad) atomicOr(a.flags, 1);
    }
    if (bold_thread) {
#pragma unroll
        for (int m = 0; m < HB_MAX_BOLD; m++)
            if (m < a.bold.n) a.bold.acc[m][(size_t)b * N0 + n] = bacc[m];
    }
    if (a.ring_in_smem && a.store_ring) {
        __syncthreads();
        float4* g = reinterpret_cast<float4*>(a.ring + (size_t)b * ring_stride);
        const float4* r4 = reinterpret_cast<const float4*>(ring);
        const int n4 = ring_words >> 2;
        for (int i = t; i < n4; i += blockDim.x) g[i] = r4[i];
        for (int i = (n4 << 2) + t; i < ring_words; i += blockDim.x) a.ring[(size_t)b * ring_stride + i] = ring[i];
    }
}

template <int MODEL, int PRE, int MAXT>
int fast_max_dynamic_smem() {
    static int cached = -1;
    if (cached >= 0) return cached;
    int dev = 0, optin = 0;
    cudaFuncAttributes fa;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&fa, resident_fast_kernel<MODEL, PRE, MAXT>) != cudaSuccess) return -1;
    int maxdyn = optin - (int)fa.sharedSizeBytes;
    if (cudaFuncSetAttribute(resident_fast_kernel<MODEL, PRE, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxdyn) != cudaSuccess)
        return -1;
    cached = maxdyn;
    return cached;
}

template <int MODEL, int PRE, int MAXT>
cudaError_t launch_fast(const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st) {
    int maxdyn = fast_max_dynamic_smem<MODEL, PRE, MAXT>();
    if (maxdyn < 0) return cudaErrorInvalidConfiguration;
    if ((long long)smem > maxdyn) return cudaErrorInvalidValue;
    resident_fast_kernel<MODEL, PRE, MAXT><<<B, threads, smem, st>>>(d_net, a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Warp-specialised pipeline for the same network shape when every edge delay is >= 2 * PK - 1.
// Consumer warps (one thread per node) run the serial model updates of block i from a shared
// double buffer while producer warps compute the coupling sums and stage the noise of block
// i + 1. Producers of block i + 1 read times <= s0(i+1) + PK - 1 - dmin <= s0(i) - 1... that is,
// only ring entries published by consumers no later than block i - 1, which the named barrier
// EMPTY[buf] orders before the producers start. Named barriers: FULL[buf] (producers arrive,
// consumers wait) and EMPTY[buf] (consumers arrive, producers wait). The ring holds H + 2*PK
// slots so a consumer's writes never land on a slot a producer may still read.
// ---------------------------------------------------------------------------------------------
#define HB_PIPE_K 8
#define HB_PIPE_PRODUCER_WARPS 8
#define HB_BAR_FULL0 1
#define HB_BAR_EMPTY0 3

__device__ __forceinline__ void named_sync(int id, int count) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory"); }
__device__ __forceinline__ void named_arrive(int id, int count) { asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory"); }

// ---- bulk-copy engine (cp.async.bulk) with mbarrier completion, for contiguous 16-byte aligned runs ----
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// one thread: expect `bytes` on the barrier and start the copy global -> shared that delivers them
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
                 ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
// wait for the phase of parity `parity` with an iteration limit; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit = 1 << 22) {
    for (int it = 0; it < limit; it++) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done) : "r"(smem_addr(bar)), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

// Consumer steps of the pipeline for the common case — Heun (deterministic or stochastic), Linear or
// Sigmoidal coupling (CFK) delivered to the first coupling variables, no BOLD — as one straight-line
// loop: the per-step branches of the general consumer (integrator, coupling function, channel map,
// monitors) are resolved by the template arguments, with the same operations in the same order
// (post() for the coupling). With traj set, each step's state of node n goes to
// traj + step * traj_stride.
template <int MODEL, int NVAR, int NCV, bool STOCH, bool SWEEP_FORM, int CFK>
__device__ __forceinline__ void pipe_consume_heun_linear(float* x, float* tv, const float* prm, const float* cp,
                                                         const float* nscale, float dt, float dt_half,
                                                         const float* gxbuf, const float* nzbuf, float* ring,
                                                         int n, bool active, int nm, int cols, int R, int slot,
                                                         int n_steps, int n_blocks, int nthreads, uint64_t* nbar,
                                                         int* err, float* traj, size_t traj_stride, bool mirror) {
    constexpr int PK = HB_PIPE_K;
    const float ca = cp[0], cb = cp[1], c2 = cp[2], c3 = cp[3], c4 = cp[4];
    float ns[NVAR];
#pragma unroll
    for (int v = 0; v < NVAR; v++) ns[v] = nscale[v];
    for (int blk = 0; blk < n_blocks; blk++) {
        const int buf = blk & 1;
        named_sync(HB_BAR_FULL0 + buf, nthreads);
        if (STOCH && nbar && !mbar_wait(nbar + buf, (uint32_t)((blk >> 1) & 1))) atomicOr(err, 4);
        const int nb = (n_steps - blk * PK) < PK ? (n_steps - blk * PK) : PK;
        const float* gb = gxbuf + (size_t)buf * PK * nm * NCV + (size_t)n * NCV;
        const float* nbuf = nzbuf + (size_t)buf * PK * nm * NVAR + (size_t)n * NVAR;
        // the block's steps unrolled: the shared-memory reads of every step's coupling sums and draws
        // do not depend on the state, so they can issue ahead of the state's dependency chain
#pragma unroll
        for (int j = 0; j < PK; j++) {
            if (j >= nb) break;
            slot = (slot + 1 == R) ? 0 : slot + 1;
            if (!active) continue;  // threads past the last node only take part in the barriers
            float cc[2] = {0.0f, 0.0f};
#pragma unroll
            for (int c = 0; c < NCV; c++) {
                const float g = gb[(size_t)j * nm * NCV + c];
                if (CFK == HBC_SIGMOIDAL) {
                    const float sh = (g + (-c2)) / c4;
                    const float ex = -(sh * c3);
                    const float den = expf(ex) + 1.0f;
                    cc[c] = (1.0f / den) * (cb - ca) + ca;
                } else {
                    cc[c] = g * ca + cb;
                }
            }
            float nz[NVAR];
#pragma unroll
            for (int v = 0; v < NVAR; v++) nz[v] = STOCH ? nbuf[(size_t)j * nm * NVAR + v] * ns[v] : 0.0f;
            float k1[NVAR], k2[NVAR], tmp[NVAR];
            dfun(MODEL, prm, SWEEP_FORM ? 1 : 0, x, cc, k1);
            if (STOCH) {
#pragma unroll
                for (int v = 0; v < NVAR; v++) tmp[v] = (x[v] + k1[v] * dt) + nz[v];
            } else {
#pragma unroll
                for (int v = 0; v < NVAR; v++) tmp[v] = x[v] + k1[v] * dt;
            }
            clamp(MODEL, tmp);
            dfun(MODEL, prm, SWEEP_FORM ? 1 : 0, tmp, cc, k2);
            if (STOCH) {
#pragma unroll
                for (int v = 0; v < NVAR; v++) x[v] = (x[v] + (k1[v] + k2[v]) * dt_half) + nz[v];
            } else {
#pragma unroll
                for (int v = 0; v < NVAR; v++) x[v] = x[v] + (k1[v] + k2[v]) * dt_half;
            }
            clamp(MODEL, x);
#pragma unroll
            for (int v = 0; v < NVAR; v++) tv[v] = tv[v] + x[v];
            ring[slot * cols + n * NCV] = x[0];
            if (NCV > 1) ring[slot * cols + n * NCV + 1] = x[1];
            if (mirror && slot < PK) {
                ring[(slot + R) * cols + n * NCV] = x[0];
                if (NCV > 1) ring[(slot + R) * cols + n * NCV + 1] = x[1];
            }
            if (traj) {
                float* tr = traj + (size_t)(blk * PK + j) * traj_stride;
#pragma unroll
                for (int v = 0; v < NVAR; v++) __stcs(tr + v, x[v]);
            }
        }
        named_arrive(HB_BAR_EMPTY0 + buf, nthreads);
    }
}

template <int MODEL, int PRE, int MAXT>
__global__ void __launch_bounds__(MAXT, 1) resident_pipe_kernel(const DevNet* __restrict__ gnet, RunArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ __align__(8) uint64_t noise_bar[2];  // bulk-copy completion of the two noise buffers
    __shared__ __align__(8) uint64_t unset_bar;     // HB_RUN_TEST_UNSET_WAIT: a barrier nothing completes
    __shared__ DevNet net;
    {
        const int* src = reinterpret_cast<const int*>(gnet);
        int* dst = reinterpret_cast<int*>(&net);
        for (int i = threadIdx.x; i < (int)(sizeof(DevNet) / 4); i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    constexpr int NVAR = c_nvar(MODEL), NCV = c_ncvar(MODEL);
    constexpr int PCH = (PRE == PRE_KURA) ? 2 : NCV;
    constexpr int PK = HB_PIPE_K;
    const int b = blockIdx.x, t = threadIdx.x, nthreads = blockDim.x;
    const int R = net.R, cols = net.cols, H = net.H, B = net.B;
    const int ring_words = R * cols;
    const size_t ring_stride = (size_t)((ring_words + 3) & ~3);
    const DevProj& P = net.proj[0];
    const int nm = net.sub[0].nm;
    const int n_cons = ((nm + 31) >> 5) << 5;      // consumer threads (warp aligned)
    const int n_prod = nthreads - n_cons;

    // shared layout: ring | gx buffers [2][PK][nm][PCH] | noise buffers [2][PK][nm*NVAR] | edges
    size_t off = 0;
    float* ring;
    // a ring in shared memory carries PK mirror slots after its R slots (slot R + q holds slot q), so that
    // a producer's window of PK consecutive slots never wraps
    const bool mirror = a.ring_in_smem != 0;
    if (a.ring_in_smem) { ring = reinterpret_cast<float*>(smem); off = (size_t)(ring_words + PK * cols) * sizeof(float); }
    else ring = a.ring + (size_t)b * ring_stride;
    off = (off + 15) & ~(size_t)15;
    float* gxbuf = reinterpret_cast<float*>(smem + off);
    off += (size_t)2 * PK * nm * PCH * sizeof(float);
    float* nzbuf = reinterpret_cast<float*>(smem + off);
    {
        const int ig = net.sub[0].integ;  // noise buffers only for stochastic integrators
        if (ig == HBI_EULER_STOCH || ig == HBI_HEUN_STOCH || ig == HBI_RK4_STOCH) off += (size_t)2 * PK * nm * NVAR * sizeof(float);
    }
    off = (off + 15) & ~(size_t)15;
    int* s_rowptr = reinterpret_cast<int*>(smem + off);
    off += (size_t)(nm + 1) * 4;
    off = (off + 15) & ~(size_t)15;
    int* s_eoff = reinterpret_cast<int*>(smem + off);
    off += (size_t)a.smem_edges * 4;
    float* s_ew = reinterpret_cast<float*>(smem + off);

    if (a.ring_in_smem && a.load_ring) {
        const float4* g = reinterpret_cast<const float4*>(a.ring + (size_t)b * ring_stride);
        float4* r4 = reinterpret_cast<float4*>(ring);
        const int n4 = ring_words >> 2;
        for (int i = t; i < n4; i += nthreads) r4[i] = g[i];
        for (int i = (n4 << 2) + t; i < ring_words; i += nthreads) ring[i] = a.ring[(size_t)b * ring_stride + i];
        for (int i = t; i < PK * cols; i += nthreads) ring[ring_words + i] = a.ring[(size_t)b * ring_stride + i];
    }
    for (int i = t; i <= nm; i += nthreads) s_rowptr[i] = P.rowptr[i];
    const bool edges_smem = P.smem_edges >= 0;
    if (edges_smem) {
        const int nnz = P.rowptr[P.ntgt];
        for (int i = t; i < nnz; i += nthreads) { s_eoff[i] = P.eoff[i]; s_ew[i] = P.ew[i]; }
    }
    const int* __restrict__ eo = edges_smem ? s_eoff : P.eoff;
    const float* __restrict__ ew = edges_smem ? s_ew : P.ew;
    const int cfk = P.cfk, maxd = P.maxd, dmode = P.dmode;
    const int integ = net.sub[0].integ;
    const bool stoch = (integ == HBI_EULER_STOCH || integ == HBI_HEUN_STOCH || integ == HBI_RK4_STOCH);
    float cp[8];
    {
        const float* c = P.cp_pp ? P.cp_pp + (size_t)b * HB_NCP : P.cp;
#pragma unroll
        for (int i = 0; i < 8; i++) cp[i] = c[i];
    }
    const float* noise_base = a.noise + (a.noise_per_point ? (size_t)b * net.noise_row : 0);
    const size_t nstride = (size_t)(a.noise_per_point ? B : 1) * net.noise_row;
    const int n_blocks = (a.n_steps + PK - 1) / PK;
    const bool is_consumer = t < n_cons;
    // noise shared by all points, rows a multiple of 16 bytes: each block's rows are one contiguous
    // aligned run, copied by the bulk-copy engine (one elected producer thread per block)
    const bool use_bulk = stoch && !a.noise_per_point && (net.noise_row % 4) == 0 &&
                          ((reinterpret_cast<uintptr_t>(noise_base) & 15) == 0) && ((reinterpret_cast<uintptr_t>(nzbuf) & 15) == 0);
    if (use_bulk && t == 0) {
        mbar_init(&noise_bar[0], 1);
        mbar_init(&noise_bar[1], 1);
        mbar_init_fence();
    }
    // test hook: one bounded wait on a barrier phase that nothing completes; it gives up after 4096
    // polls and reports the timeout like a real one, and the run then proceeds unchanged
    if (a.test_unset_wait && t == 0) {
        mbar_init(&unset_bar, 1);
        mbar_init_fence();
        if (!mbar_wait(&unset_bar, 0, 1 << 12)) atomicOr(a.flags + 1, 4);
    }

    // consumers publish x_{s0} before the first barrier
    const int n = t;
    const bool active = is_consumer && n < nm;
    float x[NVAR], tv[NVAR];
    const size_t st_base = (size_t)b * net.state_len + (size_t)(active ? n : 0) * NVAR;
    const bool first_launch_of_run = (a.s0 == a.run_s0);
    int slot = (int)(a.s0 % R);
#pragma unroll
    for (int v = 0; v < NVAR; v++) {
        x[v] = active ? a.state[st_base + v] : 0.0f;
        tv[v] = (active && !first_launch_of_run) ? a.tavg[st_base + v] : 0.0f;
    }
    if (active) {
        ring[slot * cols + n * NCV] = x[0];
        if (NCV > 1) ring[slot * cols + n * NCV + 1] = x[1];
        if (mirror && slot < PK) {
            ring[(slot + R) * cols + n * NCV] = x[0];
            if (NCV > 1) ring[(slot + R) * cols + n * NCV + 1] = x[1];
        }
    }
    __syncthreads();

    if (!is_consumer) {
        // ================= producers =================
        const int p = t - n_cons;
        const int row_len = nm * NVAR;
        // node-major assignment for the steady state: node p / PL, lane p % PL (PL a power of two)
        const int PL = a.pipe_lanes;
        const int pslot = p / PL, plane = p - (p / PL) * PL;
        const int pnode = (P.porder && pslot < nm) ? P.porder[pslot] : pslot;
        const bool pactive = pnode < nm;
        const int pe0 = pactive ? s_rowptr[pnode] : 0, pe1 = pactive ? s_rowptr[pnode + 1] : 0;
        const int early_until = (dmode == HBD_EDGE) ? maxd : P.delay;
        const int doff = (dmode == HBD_RING) ? -P.delay * cols : 0;  // single delay: uniform row offset
        for (int blk = 0; blk < n_blocks; blk++) {
            const int buf = blk & 1;
            if (blk >= 2) named_sync(HB_BAR_EMPTY0 + buf, nthreads);
            const int it0 = blk * PK;
            const int nb = (a.n_steps - it0) < PK ? (a.n_steps - it0) : PK;
            const int64_t sb = a.s0 + it0;
            int slb = (int)(sb % R);
            float* gb = gxbuf + (size_t)buf * PK * nm * PCH;
            const bool early = (sb < (int64_t)early_until) || sb == 0 || dmode == HBD_COMPAT;
            if (!early) {
                // every edge reads PK consecutive rows at its column: one offset/weight load per edge.
                // The per-lane partial sums are already regrouped relative to the source-order sum
                // of the reference (lanes, then a butterfly), so the multiply-adds are fused here;
                // the difference is one rounding per term, inside the parity tolerance.
                float acc[PK][PCH];
#pragma unroll
                for (int j = 0; j < PK; j++)
#pragma unroll
                    for (int c = 0; c < PCH; c++) acc[j][c] = 0.0f;
                const int base = slb * cols + doff;
                // EXACT (HB_RUN_EXACT_SUMS, one lane per node): each term rounded as a product and then a sum,
                // in edge order, as the reference; otherwise fused multiply-adds
                auto edge_loop = [&](auto exact_tag) {
                    constexpr bool EXACT = decltype(exact_tag)::value;
                    auto term = [&](int j, float w, int aj) {
                        const float v = ring[aj];
                        if (PRE == PRE_KURA) { acc[j][0] += w * sinf(v); acc[j][PCH - 1] += w * cosf(v); }
                        else if (EXACT) {
                            acc[j][0] = acc[j][0] + w * v;
                            if (NCV > 1) acc[j][PCH - 1] = acc[j][PCH - 1] + w * ring[aj + 1];
                        } else {
                            acc[j][0] = __fmaf_rn(w, v, acc[j][0]);
                            if (NCV > 1) acc[j][PCH - 1] = __fmaf_rn(w, ring[aj + 1], acc[j][PCH - 1]);
                        }
                    };
                    for (int e = pe0 + plane; e < pe1; e += PL) {
                        int a0 = base + eo[e];
                        a0 = a0 < 0 ? a0 + ring_words : a0;
                        const float w = ew[e];
                        if (mirror || a0 + (PK - 1) * cols < ring_words) {
#pragma unroll
                            for (int j = 0; j < PK; j++) term(j, w, a0 + j * cols);
                        } else {
#pragma unroll
                            for (int j = 0; j < PK; j++) {
                                int aj = a0 + j * cols;
                                aj = aj >= ring_words ? aj - ring_words : aj;
                                term(j, w, aj);
                            }
                        }
                    }
                };
                if (a.exact_sums) edge_loop(std::true_type());
                else edge_loop(std::false_type());
                for (int o = PL >> 1; o > 0; o >>= 1) {
#pragma unroll
                    for (int j = 0; j < PK; j++)
#pragma unroll
                        for (int c = 0; c < PCH; c++) acc[j][c] += __shfl_xor_sync(0xffffffffu, acc[j][c], o);
                }
                if (pactive && plane == 0) {
#pragma unroll
                    for (int j = 0; j < PK; j++)
                        if (j < nb) {
#pragma unroll
                            for (int c = 0; c < PCH; c++) gb[((size_t)j * nm + pnode) * PCH + c] = acc[j][c];
                        }
                }
            } else {
                // early steps: per (step, node) items with the delay checks of each edge
                int j = p / nm, nd = p - (p / nm) * nm;
                while (j < nb) {
                    const int64_t sj = sb + j;
                    int sl = slb + j;
                    sl = sl >= R ? sl - R : sl;
                    const int e0 = s_rowptr[nd], e1 = s_rowptr[nd + 1];
                    float gx[4] = {0.f, 0.f, 0.f, 0.f};
                    if (dmode == HBD_EDGE) {
                        if (sj < (int64_t)maxd || sj == 0) gather_early(ring, P, e0, e1, 0, 1, sj, sl, R, cols, 0, NCV, cp, gx);
                        else gather<PRE>(ring, eo, ew, e0, e1, 0, 1, sl * cols, ring_words, NCV, cfk, cp, P.pre_cpu, gx);
                    } else {
                        int dd;
                        if (single_delay(P, sj, H, dd)) {
                            int row = sl - dd;
                            row = row < 0 ? row + R : row;
                            gather<PRE>(ring, eo, ew, e0, e1, 0, 1, row * cols, 0, NCV, cfk, cp, 0, gx);
                        } else {
                            float zero[2] = {0.0f, 0.0f}, pz[4] = {0.f, 0.f, 0.f, 0.f};
                            pre(cfk, cp, 0, zero, NCV, pz);
                            for (int e = e0; e < e1; e++) {
                                float w = ew[e];
#pragma unroll
                                for (int c = 0; c < 4; c++) gx[c] += w * pz[c];
                            }
                        }
                    }
#pragma unroll
                    for (int c = 0; c < PCH; c++) gb[((size_t)j * nm + nd) * PCH + c] = gx[c];
                    nd += n_prod;
                    while (nd >= nm) { nd -= nm; j++; }
                }
            }
            if (stoch) {
                // raw draws of the block's rows; consumers apply the per-variable scale
                float* nbuf = nzbuf + (size_t)buf * PK * row_len;
                const float* src = noise_base + (size_t)it0 * nstride;
                if (use_bulk) {
                    if (p == 0) bulk_copy_g2s(nbuf, src, (uint32_t)(nb * row_len * 4), &noise_bar[buf]);
                    if (it0 + 4 * PK < a.n_steps) {
                        const int ahead = (a.n_steps - it0 - 4 * PK) < PK ? (a.n_steps - it0 - 4 * PK) : PK;
                        const int lines = (ahead * row_len + 31) >> 5;
                        for (int l = p; l < lines; l += n_prod) prefetch_l2(src + (size_t)4 * PK * nstride + (size_t)l * 32);
                    }
                } else if (!a.noise_per_point && ((reinterpret_cast<uintptr_t>(src) & 15) == 0)) {
                    const int total = nb * row_len, n4 = total >> 2;
                    const float4* s4 = reinterpret_cast<const float4*>(src);
                    float4* d4 = reinterpret_cast<float4*>(nbuf);
                    for (int i = p; i < n4; i += n_prod) d4[i] = __ldcs(s4 + i);
                    for (int i = (n4 << 2) + p; i < total; i += n_prod) nbuf[i] = __ldcs(src + i);
                    // the noise rows of the block four blocks ahead into L2, one 128-byte line per thread
                    if (it0 + 4 * PK < a.n_steps) {
                        const int ahead = (a.n_steps - it0 - 4 * PK) < PK ? (a.n_steps - it0 - 4 * PK) : PK;
                        const int lines = (ahead * row_len + 31) >> 5;
                        for (int l = p; l < lines; l += n_prod) prefetch_l2(src + (size_t)4 * PK * nstride + (size_t)l * 32);
                    }
                } else {
                    for (int jj = 0; jj < nb; jj++)
                        for (int i = p; i < row_len; i += n_prod) nbuf[jj * row_len + i] = __ldcs(src + (size_t)jj * nstride + i);
                }
            }
            named_arrive(HB_BAR_FULL0 + buf, nthreads);
        }
    } else {
        // ================= consumers =================
        const int sweep_form = net.sub[0].sweep_form;
        const int pc = P.pc, direct = P.direct, has_rowsums = P.has_rowsums;
        const float rowsum = (has_rowsums && active) ? P.rowsums[n] : 0.0f;
        float prm[HB_PSTRIDE];
        {
            const float* pr = hb_param_row(net.sub[0], b, active ? n : 0);
#pragma unroll
            for (int i = 0; i < HB_PSTRIDE; i++) prm[i] = (i < c_nparams_used(MODEL)) ? pr[i] : 0.0f;
        }
        const float dt = net.dt, dt_half = net.dt_half, h2 = net.dt_h2, h6 = net.dt_sixth;
        const bool bold_thread = active && a.bold.n > 0;
        const int N0 = a.bold.n0;
        float bacc[HB_MAX_BOLD];
        int bcnt[HB_MAX_BOLD];
#pragma unroll
        for (int m = 0; m < HB_MAX_BOLD; m++) {
            bacc[m] = 0.0f;
            bcnt[m] = 0;
            if (m < a.bold.n) {
                bcnt[m] = (int)((a.s0 - a.run_s0) % a.bold.period[m]);
                if (bold_thread && !first_launch_of_run) bacc[m] = a.bold.acc[m][(size_t)b * N0 + n];
            }
        }
        int64_t s = a.s0;
        const bool straight = PRE == PRE_ID && (integ == HBI_HEUN_STOCH || integ == HBI_HEUN_DET) &&
                              (cfk == HBC_LINEAR || cfk == HBC_SIGMOIDAL) && direct && pc == NCV && !has_rowsums &&
                              a.bold.n == 0;
        if (straight) {
            float* trj = a.traj ? a.traj + (size_t)b * net.state_len + (size_t)n * NVAR : nullptr;
            const size_t trs = (size_t)B * net.state_len;
            float nscale[8];
#pragma unroll
            for (int v = 0; v < 8; v++) nscale[v] = net.noise_scale[v];
            uint64_t* nb_ = use_bulk ? noise_bar : nullptr;
#define HB_STRAIGHT(ST, SF, CF) pipe_consume_heun_linear<MODEL, NVAR, NCV, ST, SF, CF>(x, tv, prm, cp, nscale, dt, dt_half, gxbuf, nzbuf, ring, n, active, nm, cols, R, slot, a.n_steps, n_blocks, nthreads, nb_, a.flags + 1, trj, trs, mirror)
            if (cfk == HBC_SIGMOIDAL) {
                if (integ == HBI_HEUN_STOCH) { if (sweep_form) HB_STRAIGHT(true, true, HBC_SIGMOIDAL); else HB_STRAIGHT(true, false, HBC_SIGMOIDAL); }
                else { if (sweep_form) HB_STRAIGHT(false, true, HBC_SIGMOIDAL); else HB_STRAIGHT(false, false, HBC_SIGMOIDAL); }
            } else {
                if (integ == HBI_HEUN_STOCH) { if (sweep_form) HB_STRAIGHT(true, true, HBC_LINEAR); else HB_STRAIGHT(true, false, HBC_LINEAR); }
                else { if (sweep_form) HB_STRAIGHT(false, true, HBC_LINEAR); else HB_STRAIGHT(false, false, HBC_LINEAR); }
            }
#undef HB_STRAIGHT
        }
        for (int blk = 0; blk < (straight ? 0 : n_blocks); blk++) {
            const int buf = blk & 1;
            named_sync(HB_BAR_FULL0 + buf, nthreads);
            if (use_bulk && !mbar_wait(&noise_bar[buf], (uint32_t)((blk >> 1) & 1))) atomicOr(a.flags + 1, 4);
            const int it0 = blk * PK;
            const int nb = (a.n_steps - it0) < PK ? (a.n_steps - it0) : PK;
            const float* gb = gxbuf + (size_t)buf * PK * nm * PCH;
            const float* nbuf = nzbuf + (size_t)buf * PK * nm * NVAR;
#pragma unroll 1
            for (int j = 0; j < nb; j++, s++) {
                if (active) {
                    float gx[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                    for (int c = 0; c < PCH; c++) gx[c] = gb[((size_t)j * nm + n) * PCH + c];
                    if (PCH == 2 && a.gx_out)
                        __stcs(reinterpret_cast<float2*>(a.gx_out) + ((size_t)(it0 + j) * B + b) * nm + n,
                               make_float2(gx[0], gx[PCH - 1]));
                    float nz[NVAR];
#pragma unroll
                    for (int v = 0; v < NVAR; v++) nz[v] = stoch ? nbuf[(size_t)j * nm * NVAR + n * NVAR + v] * net.noise_scale[v] : 0.0f;
                    float cc[2] = {0.0f, 0.0f};
                    {
                        float out[4] = {0.f, 0.f, 0.f, 0.f};
                        float xi[2] = {x[0], NCV > 1 ? x[NCV - 1] : 0.0f};
                        int oc = post(cfk, cp, has_rowsums, gx, pc, xi, NCV, rowsum, out);
                        if (direct) {
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
#pragma unroll
                    for (int v = 0; v < NVAR; v++) tv[v] = tv[v] + x[v];
                    const int it = it0 + j;
                    if (a.traj) {
                        float* tr = a.traj + ((size_t)it * B + b) * net.state_len + (size_t)n * NVAR;
#pragma unroll
                        for (int v = 0; v < NVAR; v++) __stcs(tr + v, x[v]);
                    }
                    if (bold_thread) {
                        const int64_t rel = s - a.run_s0;
#pragma unroll
                        for (int m = 0; m < HB_MAX_BOLD; m++) {
                            if (m >= a.bold.n) break;
                            bacc[m] = bacc[m] + x[0];
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
                    int sl1 = slot + 1;
                    sl1 = sl1 >= R ? sl1 - R : sl1;
                    ring[sl1 * cols + n * NCV] = x[0];
                    if (NCV > 1) ring[sl1 * cols + n * NCV + 1] = x[1];
                    if (mirror && sl1 < PK) {
                        ring[(sl1 + R) * cols + n * NCV] = x[0];
                        if (NCV > 1) ring[(sl1 + R) * cols + n * NCV + 1] = x[1];
                    }
                }
                slot = (slot + 1 == R) ? 0 : slot + 1;
            }
            named_arrive(HB_BAR_EMPTY0 + buf, nthreads);
        }
        if (active) {
            bool bad = false;
#pragma unroll
            for (int v = 0; v < NVAR; v++) {
                a.state[st_base + v] = x[v];
                a.tavg[st_base + v] = tv[v];
                bad |= !isfinite(x[v]);
            }
            if (a.check_finite && bad) atomicOr(a.flags, 1);
        }
        if (bold_thread) {
#pragma unroll
            for (int m = 0; m < HB_MAX_BOLD; m++)
                if (m < a.bold.n) a.bold.acc[m][(size_t)b * N0 + n] = bacc[m];
        }
    }
    __syncthreads();
    if (a.ring_in_smem && a.store_ring) {
        float4* g = reinterpret_cast<float4*>(a.ring + (size_t)b * ring_stride);
        const float4* r4 = reinterpret_cast<const float4*>(ring);
        const int n4 = ring_words >> 2;
        for (int i = t; i < n4; i += nthreads) g[i] = r4[i];
        for (int i = (n4 << 2) + t; i < ring_words; i += nthreads) a.ring[(size_t)b * ring_stride + i] = ring[i];
    }
}

template <int MODEL, int PRE, int MAXT>
int pipe_max_dynamic_smem() {
    static int cached = -1;
    if (cached >= 0) return cached;
    int dev = 0, optin = 0;
    cudaFuncAttributes fa;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&fa, resident_pipe_kernel<MODEL, PRE, MAXT>) != cudaSuccess) return -1;
    int maxdyn = optin - (int)fa.sharedSizeBytes;
    if (cudaFuncSetAttribute(resident_pipe_kernel<MODEL, PRE, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxdyn) != cudaSuccess)
        return -1;
    cached = maxdyn;
    return cached;
}

template <int MODEL, int PRE, int MAXT>
cudaError_t launch_pipe(const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st) {
    int maxdyn = pipe_max_dynamic_smem<MODEL, PRE, MAXT>();
    if (maxdyn < 0) return cudaErrorInvalidConfiguration;
    if ((long long)smem > maxdyn || threads > MAXT) return cudaErrorInvalidValue;
    resident_pipe_kernel<MODEL, PRE, MAXT><<<B, threads, smem, st>>>(d_net, a);
    return cudaGetLastError();
}

// dynamic shared memory available to resident_kernel<MODEL, MAXT> on this device (sets the opt-in)
template <int MODEL, int MAXT>
int resident_max_dynamic_smem() {
    static int cached = -1;
    if (cached >= 0) return cached;
    int dev = 0, optin = 0;
    cudaFuncAttributes fa;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&fa, resident_kernel<MODEL, MAXT>) != cudaSuccess) return -1;
    int maxdyn = optin - (int)fa.sharedSizeBytes;
    if (cudaFuncSetAttribute(resident_kernel<MODEL, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxdyn) != cudaSuccess)
        return -1;
    cached = maxdyn;
    return cached;
}

template <int MODEL, int MAXT>
cudaError_t launch_resident(const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st) {
    int maxdyn = resident_max_dynamic_smem<MODEL, MAXT>();
    if (maxdyn < 0) return cudaErrorInvalidConfiguration;
    if ((long long)smem > maxdyn) return cudaErrorInvalidValue;
    resident_kernel<MODEL, MAXT><<<B, threads, smem, st>>>(d_net, a);
    return cudaGetLastError();
}

}  // namespace hb

// per-MAXT entry points (one translation unit each)
cudaError_t hb_launch_resident_256(int model, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
cudaError_t hb_launch_resident_512(int model, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
cudaError_t hb_launch_resident_1024(int model, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
int hb_resident_budget_256(int model);
int hb_resident_budget_512(int model);
int hb_resident_budget_1024(int model);

#define HB_RESIDENT_UNIT(MAXT)                                                                                      \
    cudaError_t hb_launch_resident_##MAXT(int model, const DevNet* d_net, const RunArgs& a, int B, int threads,     \
                                          size_t smem, cudaStream_t st) {                                            \
        (void)model;                                                                                                 \
        return hb::launch_resident<-1, MAXT>(d_net, a, B, threads, smem, st);                                        \
    }                                                                                                                \
    int hb_resident_budget_##MAXT(int model) {                                                                       \
        (void)model;                                                                                                 \
        return hb::resident_max_dynamic_smem<-1, MAXT>();                                                            \
    }

cudaError_t hb_launch_fast_512(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
cudaError_t hb_launch_fast_1024(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
int hb_fast_budget_512(int model, int pre);
int hb_fast_budget_1024(int model, int pre);

#define HB_FAST_UNIT(MAXT)                                                                                          \
    cudaError_t hb_launch_fast_##MAXT(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, \
                                      size_t smem, cudaStream_t st) {                                                \
        constexpr int MAXT_ = MAXT;                                                                                  \
        using F = cudaError_t (*)(const DevNet*, const RunArgs&, int, int, size_t, cudaStream_t);                   \
        F f = nullptr;                                                                                               \
        switch (model * 2 + (pre == hb::PRE_KURA ? 1 : 0)) {                                                         \
        case 0: f = hb::launch_fast<0, hb::PRE_ID, MAXT_>; break;                                                    \
        case 1: f = hb::launch_fast<0, hb::PRE_KURA, MAXT_>; break;                                                  \
        case 2: f = hb::launch_fast<1, hb::PRE_ID, MAXT_>; break;                                                    \
        case 3: f = hb::launch_fast<1, hb::PRE_KURA, MAXT_>; break;                                                  \
        case 4: f = hb::launch_fast<2, hb::PRE_ID, MAXT_>; break;                                                    \
        case 5: f = hb::launch_fast<2, hb::PRE_KURA, MAXT_>; break;                                                  \
        case 6: f = hb::launch_fast<3, hb::PRE_ID, MAXT_>; break;                                                    \
        case 7: f = hb::launch_fast<3, hb::PRE_KURA, MAXT_>; break;                                                  \
        case 8: f = hb::launch_fast<4, hb::PRE_ID, MAXT_>; break;                                                    \
        case 9: f = hb::launch_fast<4, hb::PRE_KURA, MAXT_>; break;                                                  \
        case 10: f = hb::launch_fast<5, hb::PRE_ID, MAXT_>; break;                                                   \
        case 11: f = hb::launch_fast<5, hb::PRE_KURA, MAXT_>; break;                                                 \
        default: return cudaErrorInvalidValue;                                                                       \
        }                                                                                                            \
        return f(d_net, a, B, threads, smem, st);                                                                    \
    }                                                                                                                \
    int hb_fast_budget_##MAXT(int model, int pre) {                                                                  \
        constexpr int MAXT_ = MAXT;                                                                                  \
        switch (model * 2 + (pre == hb::PRE_KURA ? 1 : 0)) {                                                         \
        case 0: return hb::fast_max_dynamic_smem<0, hb::PRE_ID, MAXT_>();                                            \
        case 1: return hb::fast_max_dynamic_smem<0, hb::PRE_KURA, MAXT_>();                                          \
        case 2: return hb::fast_max_dynamic_smem<1, hb::PRE_ID, MAXT_>();                                            \
        case 3: return hb::fast_max_dynamic_smem<1, hb::PRE_KURA, MAXT_>();                                          \
        case 4: return hb::fast_max_dynamic_smem<2, hb::PRE_ID, MAXT_>();                                            \
        case 5: return hb::fast_max_dynamic_smem<2, hb::PRE_KURA, MAXT_>();                                          \
        case 6: return hb::fast_max_dynamic_smem<3, hb::PRE_ID, MAXT_>();                                            \
        case 7: return hb::fast_max_dynamic_smem<3, hb::PRE_KURA, MAXT_>();                                          \
        case 8: return hb::fast_max_dynamic_smem<4, hb::PRE_ID, MAXT_>();                                            \
        case 9: return hb::fast_max_dynamic_smem<4, hb::PRE_KURA, MAXT_>();                                          \
        case 10: return hb::fast_max_dynamic_smem<5, hb::PRE_ID, MAXT_>();                                           \
        case 11: return hb::fast_max_dynamic_smem<5, hb::PRE_KURA, MAXT_>();                                         \
        default: return -1;                                                                                          \
        }                                                                                                            \
    }

cudaError_t hb_launch_pipe_512(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
cudaError_t hb_launch_pipe_1024(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
int hb_pipe_budget_512(int model, int pre);
int hb_pipe_budget_1024(int model, int pre);

#define HB_PIPE_UNIT(MAXT_)                                                                                         \
    cudaError_t hb_launch_pipe_##MAXT_(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, \
                                       size_t smem, cudaStream_t st) {                                               \
        using F = cudaError_t (*)(const DevNet*, const RunArgs&, int, int, size_t, cudaStream_t);                    \
        static const F tab[12] = {                                                                                   \
            hb::launch_pipe<0, hb::PRE_ID, MAXT_>, hb::launch_pipe<0, hb::PRE_KURA, MAXT_>,                          \
            hb::launch_pipe<1, hb::PRE_ID, MAXT_>, hb::launch_pipe<1, hb::PRE_KURA, MAXT_>,                          \
            hb::launch_pipe<2, hb::PRE_ID, MAXT_>, hb::launch_pipe<2, hb::PRE_KURA, MAXT_>,                          \
            hb::launch_pipe<3, hb::PRE_ID, MAXT_>, hb::launch_pipe<3, hb::PRE_KURA, MAXT_>,                          \
            hb::launch_pipe<4, hb::PRE_ID, MAXT_>, hb::launch_pipe<4, hb::PRE_KURA, MAXT_>,                          \
            hb::launch_pipe<5, hb::PRE_ID, MAXT_>, hb::launch_pipe<5, hb::PRE_KURA, MAXT_>};                         \
        int i = model * 2 + (pre == hb::PRE_KURA ? 1 : 0);                                                           \
        if (model < 0 || i >= 12) return cudaErrorInvalidValue;                                                      \
        return tab[i](d_net, a, B, threads, smem, st);                                                               \
    }                                                                                                                \
    int hb_pipe_budget_##MAXT_(int model, int pre) {                                                                 \
        using G = int (*)();                                                                                         \
        static const G tab[12] = {                                                                                   \
            hb::pipe_max_dynamic_smem<0, hb::PRE_ID, MAXT_>, hb::pipe_max_dynamic_smem<0, hb::PRE_KURA, MAXT_>,      \
            hb::pipe_max_dynamic_smem<1, hb::PRE_ID, MAXT_>, hb::pipe_max_dynamic_smem<1, hb::PRE_KURA, MAXT_>,      \
            hb::pipe_max_dynamic_smem<2, hb::PRE_ID, MAXT_>, hb::pipe_max_dynamic_smem<2, hb::PRE_KURA, MAXT_>,      \
            hb::pipe_max_dynamic_smem<3, hb::PRE_ID, MAXT_>, hb::pipe_max_dynamic_smem<3, hb::PRE_KURA, MAXT_>,      \
            hb::pipe_max_dynamic_smem<4, hb::PRE_ID, MAXT_>, hb::pipe_max_dynamic_smem<4, hb::PRE_KURA, MAXT_>,      \
            hb::pipe_max_dynamic_smem<5, hb::PRE_ID, MAXT_>, hb::pipe_max_dynamic_smem<5, hb::PRE_KURA, MAXT_>};     \
        int i = model * 2 + (pre == hb::PRE_KURA ? 1 : 0);                                                           \
        if (model < 0 || i >= 12) return -1;                                                                         \
        return tab[i]();                                                                                             \
    }
