// hb_kernels.cu — simulation kernels of the batched neural-mass engine (sm_103a).
//
// resident_kernel: the persistent "plain" form. One CTA owns one sweep point for a whole launch
//   (all subnetworks, one thread per node, warp-aligned per subnetwork). State, temporal average
//   and BOLD window sums stay in registers across steps; the coupling-variable history ring
//   (only the cvars, [R][cols]) stays in shared memory when it fits, otherwise in global memory;
//   CSR rows with packed per-edge delays are cached in shared memory. One __syncthreads per step
//   separates publishing x_s into the ring from the coupling gather; the ring holds R >= H + 1
//   slots so that the next step's write never lands on a slot still being read.
// bold_reduce_kernel / bold_bw_kernel: the batch-mean BOLD monitor (mean over sweep points of
//   var0, engine.rs:786-801) from per-point window sums, then the Balloon-Windkessel ODE and
//   the TR down-sampling schedule.
#include <cuda_runtime.h>
#include "hb_models.cuh"

namespace hb {

__device__ __forceinline__ int ring_back(int slot, int dd, int R) {
    int i = slot - dd;
    return i < 0 ? i + R : i;
}

// delay offset of a single-delay projection at step s: returns false when the source row is the
// zero tensor (zeros before pre(), engine.rs:580-584 / runtime.rs:246-249)
__device__ __forceinline__ bool single_delay(const DevProj& P, int64_t s, int H, int& dd) {
    int d = P.delay;
    if (d == 0 || s == 0) { dd = 0; return true; }
    if ((int64_t)d > s) return false;
    if (P.dmode == HBD_COMPAT) {
        // the window index (s - d + H) % H of the shift-window history holds x_{s+1+idx-H}
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

template <int MAXT>
__global__ void __launch_bounds__(MAXT, 1)
resident_kernel(const DevNet* __restrict__ gnet, RunArgs a) {
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
    const int lane = t & 31, warp = t >> 5;
    const int R = net.R, cols = net.cols, H = net.H, B = net.B;

    size_t off = 0;
    float* ring;
    if (a.ring_in_smem) { ring = reinterpret_cast<float*>(smem); off = (size_t)R * cols * sizeof(float); }
    else ring = a.ring + (size_t)b * R * cols;
    off = (off + 15) & ~(size_t)15;
    uint32_t* s_edges = reinterpret_cast<uint32_t*>(smem + off);
    off += (size_t)a.smem_edges * 4;
    float* s_ew = reinterpret_cast<float*>(smem + off);
    off += (size_t)a.smem_edges * 4;
    off = (off + 15) & ~(size_t)15;
    float* s_part = reinterpret_cast<float*>(smem + off);  // [2][n_mean][32 warps][4]

    if (a.ring_in_smem && a.load_ring) {
        const float* g = a.ring + (size_t)b * R * cols;
        int n = R * cols;
        for (int i = t; i < n; i += blockDim.x) ring[i] = g[i];
    }
    for (int p = 0; p < net.n_proj; p++) {
        const DevProj& P = net.proj[p];
        if (P.kind != HBK_SPARSE || P.smem_edges < 0) continue;
        int nnz = P.rowptr[P.ntgt];
        for (int i = t; i < nnz; i += blockDim.x) {
            s_edges[P.smem_edges + i] = P.edges[i];
            s_ew[P.smem_edges + i] = P.ew[i];
        }
    }

    // role of this thread: node n of subnetwork k
    int k = 0;
    for (int i = 1; i < net.n_sub; i++)
        if (t >= net.sub[i].thread_off) k = i;
    const int model = net.sub[k].model, nm = net.sub[k].nm, nvar = net.sub[k].nvar, ncvar = net.sub[k].ncvar;
    const int col_off = net.sub[k].col_off, integ = net.sub[k].integ, sweep_form = net.sub[k].sweep_form;
    const int n = t - net.sub[k].thread_off;
    const bool active = n < nm;
    const int nn = active ? n : 0;

    float prm[HB_PSTRIDE];
    {
        const float* pr = net.sub[k].params + (size_t)b * HB_PSTRIDE;
#pragma unroll
        for (int i = 0; i < HB_PSTRIDE; i++) prm[i] = pr[i];
    }
    float x[6], tv[6];
    const size_t st_base = (size_t)b * net.state_len + net.sub[k].state_off + (size_t)nn * nvar;
    const bool first_launch_of_run = (a.s0 == a.run_s0);
#pragma unroll
    for (int v = 0; v < 6; v++) {
        x[v] = (active && v < nvar) ? a.state[st_base + v] : 0.0f;
        tv[v] = (active && v < nvar && !first_launch_of_run) ? a.tavg[st_base + v] : 0.0f;
    }
    // BOLD (subnetwork 0, nmodes == 1)
    const bool bold_thread = (k == 0) && active && a.bold.n > 0;
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
        if (active) {
            float* wr = ring + (size_t)slot * cols + col_off + n * ncvar;
            wr[0] = x[0];
            if (ncvar > 1) wr[1] = x[1];
        }
        // ---- mean-field partial sums of projections whose source is this subnetwork ----
        for (int p = 0; p < net.n_proj; p++) {
            const DevProj& P = net.proj[p];
            if (P.kind != HBK_MEAN || P.src != k) continue;
            const float* cp = P.cp_pp ? P.cp_pp + (size_t)b * HB_NCP : P.cp;
            float pv[4] = {0.f, 0.f, 0.f, 0.f};
            int dd;
            bool ok = single_delay(P, s, H, dd);
            if (active) {
                float cv[2] = {0.0f, 0.0f};
                if (ok) {
                    const float* rr = ring + (size_t)ring_back(slot, dd, R) * cols + col_off + n * ncvar;
                    cv[0] = dd == 0 ? x[0] : rr[0];
                    if (P.ncv > 1) cv[1] = dd == 0 ? x[1] : rr[1];
                }
                pre(P.cfk, cp, 0, cv, P.ncv, pv);
            }
#pragma unroll
            for (int c = 0; c < 4; c++) {
                if (c < P.pc) {
                    float sum = warp_sum(pv[c]);
                    if (lane == 0) s_part[((buf * n_mean + P.mean_slot) * 32 + warp) * 4 + c] = sum;
                }
            }
        }
        // noise draws of this step (issued before the barrier to hide their latency)
        float nz[6];
        if (integ == HBI_EULER_STOCH || integ == HBI_HEUN_STOCH || integ == HBI_RK4_STOCH) {
            const float* row = a.noise + ((size_t)it * (a.noise_per_point ? B : 1) + (a.noise_per_point ? b : 0)) * net.noise_row
                               + net.sub[k].noise_off + (size_t)nn * nvar;
#pragma unroll
            for (int v = 0; v < 6; v++) nz[v] = (active && v < nvar) ? __ldcs(row + v) * net.noise_scale[v] : 0.0f;
        }
        __syncthreads();

        // ---- 2. coupling into this subnetwork (engine.rs:557-674) ----
        float cc[2] = {0.0f, 0.0f};
        const int n_in = net.sub[k].n_in;
        for (int q = 0; q < n_in; q++) {
            const DevProj& P = net.proj[net.sub[k].in_idx[q]];
            const float* cp = P.cp_pp ? P.cp_pp + (size_t)b * HB_NCP : P.cp;
            const int scol = net.sub[P.src].col_off, sncv = net.sub[P.src].ncvar;
            float gx[4] = {0.f, 0.f, 0.f, 0.f};
            if (P.kind == HBK_MEAN) {
                const int w0 = net.sub[P.src].thread_off >> 5;
                const int w1 = (net.sub[P.src].thread_off + P.nsrc + 31) >> 5;
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    if (c < P.pc) {
                        float acc = 0.0f;
                        for (int w = w0; w < w1; w++) acc += s_part[((buf * n_mean + P.mean_slot) * 32 + w) * 4 + c];
                        gx[c] = (acc / (float)P.nsrc) * P.w;
                    }
                }
            } else if (active) {
                if (P.kind == HBK_DIAG) {
                    int dd;
                    bool ok = single_delay(P, s, H, dd);
                    float cv[2] = {0.0f, 0.0f}, pv[4] = {0.f, 0.f, 0.f, 0.f};
                    const float* rr = ring + (size_t)ring_back(slot, ok ? dd : 0, R) * cols + scol + n * sncv;
                    if (ok) { cv[0] = rr[0]; if (P.ncv > 1) cv[1] = rr[1]; }
                    pre(P.cfk, cp, 0, cv, P.ncv, pv);
#pragma unroll
                    for (int c = 0; c < 4; c++) if (c < P.pc) gx[c] = P.w * pv[c];
                } else {
                    const uint32_t* ed = P.smem_edges >= 0 ? s_edges + P.smem_edges : P.edges;
                    const float* ew = P.smem_edges >= 0 ? s_ew + P.smem_edges : P.ew;
                    const int e0 = P.rowptr[n], e1 = P.rowptr[n + 1];
                    if (P.dmode == HBD_EDGE) {
                        const bool early = (s == 0) || (s < (int64_t)H);
                        const int cpu_form = P.pre_cpu;
                        if (P.cfk != HBC_KURAMOTO && P.cfk != HBC_TANH && P.cfk != HBC_SJR && P.cfk != HBC_PRESIG && P.ncv == 1) {
                            // identity pre(): plain weighted gather
                            float acc = 0.0f;
                            for (int e = e0; e < e1; e++) {
                                uint32_t m = ed[e];
                                int d = (int)(m >> 16), src = (int)(m & 0xffffu);
                                int dd = d;
                                if (early) {
                                    if (d == 0 || s == 0) dd = 0;
                                    else if ((int64_t)d > s) continue;
                                }
                                acc += ew[e] * ring[(size_t)ring_back(slot, dd, R) * cols + scol + src * sncv];
                            }
                            gx[0] = acc;
                        } else {
                            for (int e = e0; e < e1; e++) {
                                uint32_t m = ed[e];
                                int d = (int)(m >> 16), src = (int)(m & 0xffffu);
                                int dd = d;
                                if (early) {
                                    if (d == 0 || s == 0) dd = 0;
                                    else if ((int64_t)d > s) continue;
                                }
                                const float* rr = ring + (size_t)ring_back(slot, dd, R) * cols + scol + src * sncv;
                                float cv[2] = {rr[0], 0.0f}, pv[4] = {0.f, 0.f, 0.f, 0.f};
                                if (P.ncv > 1) cv[1] = rr[1];
                                pre(P.cfk, cp, cpu_form, cv, P.ncv, pv);
                                float wk = ew[e];
#pragma unroll
                                for (int c = 0; c < 4; c++) if (c < P.pc) gx[c] += wk * pv[c];
                            }
                        }
                    } else {
                        int dd;
                        bool ok = single_delay(P, s, H, dd);
                        const float* rbase = ring + (size_t)ring_back(slot, ok ? dd : 0, R) * cols + scol;
                        for (int e = e0; e < e1; e++) {
                            uint32_t m = ed[e];
                            int src = (int)(m & 0xffffu);
                            float cv[2] = {0.0f, 0.0f}, pv[4] = {0.f, 0.f, 0.f, 0.f};
                            if (ok) { cv[0] = rbase[src * sncv]; if (P.ncv > 1) cv[1] = rbase[src * sncv + 1]; }
                            pre(P.cfk, cp, 0, cv, P.ncv, pv);
                            float wk = ew[e];
#pragma unroll
                            for (int c = 0; c < 4; c++) if (c < P.pc) gx[c] += wk * pv[c];
                        }
                    }
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
                        if (sidx < net.sub[P.src].ncvar && cpl < ncvar) {
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
            dfun(model, prm, sweep_form, x, cc, k1);
            switch (integ) {
            case HBI_HEUN_DET:
#pragma unroll
                for (int v = 0; v < 6; v++) tmp[v] = x[v] + k1[v] * dt;
                clamp(model, tmp);
                dfun(model, prm, sweep_form, tmp, cc, k2);
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
                clamp(model, tmp);
                dfun(model, prm, sweep_form, tmp, cc, k2);
#pragma unroll
                for (int v = 0; v < 6; v++) x[v] = (x[v] + (k1[v] + k2[v]) * net.dt_half) + nz[v];
                break;
            default: {  // RK4 / RK4 stochastic
                float k3[6], k4[6];
                const float h2 = net.dt_h2, h6 = net.dt_sixth;
#pragma unroll
                for (int v = 0; v < 6; v++) tmp[v] = x[v] + k1[v] * h2;
                clamp(model, tmp);
                dfun(model, prm, sweep_form, tmp, cc, k2);
#pragma unroll
                for (int v = 0; v < 6; v++) tmp[v] = x[v] + k2[v] * h2;
                clamp(model, tmp);
                dfun(model, prm, sweep_form, tmp, cc, k3);
#pragma unroll
                for (int v = 0; v < 6; v++) tmp[v] = x[v] + k3[v] * dt;
                clamp(model, tmp);
                dfun(model, prm, sweep_form, tmp, cc, k4);
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
            clamp(model, x);
#pragma unroll
            for (int v = 0; v < 6; v++) tv[v] = tv[v] + x[v];
            if (a.traj) {
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
    if (active) {
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
        float* g = a.ring + (size_t)b * R * cols;
        int nr = R * cols;
        for (int i = t; i < nr; i += blockDim.x) g[i] = ring[i];
    }
}

// batch-mean BOLD, stage 1: mean over sweep points of each window sum -> means[w][n]
__global__ void bold_reduce_kernel(const float* __restrict__ win, int n_windows, int B, int N0, float* __restrict__ means) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)n_windows * N0) return;
    int w = (int)(i / N0), n = (int)(i % N0);
    const float* p = win + (size_t)w * B * N0 + n;
    float acc = 0.0f;
    for (int bb = 0; bb < B; bb++) acc += p[(size_t)bb * N0];
    means[i] = acc / (float)B;
}

// batch-mean BOLD, stage 2: one thread per node walks the windows in order (bold_monitor.rs:86-106)
__global__ void bold_bw_kernel(DevBold bold, int m, const float* __restrict__ means, int n_windows) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int N0 = bold.n0;
    if (n >= N0) return;
    float* bw = bold.bw[m];
    float bs = bw[n], bf = bw[N0 + n], bv = bw[2 * N0 + n], bq = bw[3 * N0 + n], prev = bw[4 * N0 + n];
    const BoldEmit* em = bold.emit[m];
    int j = 0;
    for (int w = 0; w < n_windows; w++) {
        bool full = w < bold.n_full[m];
        int cnt = full ? bold.period[m] : bold.partial[m];
        float avg = means[(size_t)w * N0 + n] / (float)cnt;
        bw_step(bs, bf, bv, bq, avg, full ? bold.dt_full[m] : bold.dt_part[m]);
        float cur = bw_signal(bv, bq);
        while (j < bold.n_emit[m] && em[j].k < w) j++;
        for (; j < bold.n_emit[m] && em[j].k == w; j++) {
            float val = em[j].interp ? prev + (cur - prev) * em[j].w : cur;
            bold.out[m][(size_t)em[j].out * N0 + n] = val;
        }
        prev = cur;
    }
    bw[n] = bs; bw[N0 + n] = bf; bw[2 * N0 + n] = bv; bw[3 * N0 + n] = bq; bw[4 * N0 + n] = prev;
}

}  // namespace hb

// ---- launch wrappers (called by the host engine) ----
// largest dynamic shared-memory request a resident_kernel<MAXT> launch may make on this device
template <int MAXT>
static int resident_max_dynamic_smem() {
    static int cached = -1;
    if (cached >= 0) return cached;
    int dev = 0, optin = 0;
    cudaFuncAttributes fa;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&fa, hb::resident_kernel<MAXT>) != cudaSuccess) return -1;
    int maxdyn = optin - (int)fa.sharedSizeBytes;
    if (cudaFuncSetAttribute(hb::resident_kernel<MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxdyn) != cudaSuccess)
        return -1;
    cached = maxdyn;
    return cached;
}

template <int MAXT>
static cudaError_t launch_resident_t(const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st) {
    int maxdyn = resident_max_dynamic_smem<MAXT>();
    if (maxdyn < 0) return cudaGetLastError() != cudaSuccess ? cudaGetLastError() : cudaErrorInvalidConfiguration;
    if ((long long)smem > maxdyn) return cudaErrorInvalidValue;
    hb::resident_kernel<MAXT><<<B, threads, smem, st>>>(d_net, a);
    return cudaGetLastError();
}

cudaError_t hb_launch_resident(const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st) {
    if (threads <= 256) return launch_resident_t<256>(d_net, a, B, threads, smem, st);
    return launch_resident_t<1024>(d_net, a, B, threads, smem, st);
}

// dynamic shared memory available to the resident kernel for a CTA of `threads` threads
int hb_resident_smem_budget(int threads) {
    int v = threads <= 256 ? resident_max_dynamic_smem<256>() : resident_max_dynamic_smem<1024>();
    return v;
}

cudaError_t hb_launch_bold_batch_mean(const DevBold& bold, int m, int n_windows, int B, float* means, cudaStream_t st) {
    if (n_windows <= 0) return cudaSuccess;
    int64_t total = (int64_t)n_windows * bold.n0;
    int blocks = (int)((total + 255) / 256);
    hb::bold_reduce_kernel<<<blocks, 256, 0, st>>>(bold.win[m], n_windows, B, bold.n0, means);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    hb::bold_bw_kernel<<<(bold.n0 + 127) / 128, 128, 0, st>>>(bold, m, means, n_windows);
    return cudaGetLastError();
}

int hb_resident_static_smem() {
    cudaFuncAttributes attr;
    if (cudaFuncGetAttributes(&attr, hb::resident_kernel<1024>) != cudaSuccess) return -1;
    return (int)attr.sharedSizeBytes;
}
