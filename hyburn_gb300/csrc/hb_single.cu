// hb_single.cu — one warp per sweep point for networks without delays or edges.
//
// For one subnetwork coupled to itself through one projection of Scalar weights without delay —
// the mean-field form w * mean over source nodes (engine.rs:602-608) or the diagonal form w * x_i
// (construction.rs:639-655) — a sweep point of up to 128 nodes fits one warp: lane l holds nodes
// l, l + 32, l + 64, l + 96 in registers, the mean over source nodes is a warp butterfly sum, and
// a step needs no block barrier and no history. Blocks of one warp, so up to 32 points share an
// SM. The plain single simulation (one point, 74 nodes, mean-field coupling) runs here.
#include <cuda_runtime.h>

#include "hb_device.h"
#include "hb_models.cuh"
#include "hb_stream.cuh"

namespace {

// Heun (deterministic or stochastic) with Linear coupling delivered directly: the update of the
// lane's M nodes stage by stage (k1 of all, then the predictor of all, ...), so that their
// dependency chains overlap. Same operations in the same order as the general update.
template <int MODEL, int M, bool STOCH, bool SF>
__device__ __forceinline__ void heun_linear_nodes(float (&x)[M][hb::c_nvar(MODEL)], const float* prm, float cc0, float cc1,
                                                  const float (&nz)[M][hb::c_nvar(MODEL)], float dt, float dt_half) {
    constexpr int NVAR = hb::c_nvar(MODEL);
    float cc[2] = {cc0, cc1};
    float k1[M][NVAR], k2[M][NVAR], tmp[M][NVAR];
#pragma unroll
    for (int q = 0; q < M; q++) hb::dfun(MODEL, prm, SF ? 1 : 0, x[q], cc, k1[q]);
#pragma unroll
    for (int q = 0; q < M; q++) {
#pragma unroll
        for (int v = 0; v < NVAR; v++) tmp[q][v] = STOCH ? (x[q][v] + k1[q][v] * dt) + nz[q][v] : x[q][v] + k1[q][v] * dt;
        hb::clamp(MODEL, tmp[q]);
    }
#pragma unroll
    for (int q = 0; q < M; q++) hb::dfun(MODEL, prm, SF ? 1 : 0, tmp[q], cc, k2[q]);
#pragma unroll
    for (int q = 0; q < M; q++) {
#pragma unroll
        for (int v = 0; v < NVAR; v++)
            x[q][v] = STOCH ? (x[q][v] + (k1[q][v] + k2[q][v]) * dt_half) + nz[q][v] : x[q][v] + (k1[q][v] + k2[q][v]) * dt_half;
        hb::clamp(MODEL, x[q]);
    }
}

template <int MODEL, int M, bool STOCH, bool SF>
__device__ __forceinline__ void single_warp_straight(const DevProj& P, const float* prm, const float* cp, float (&x)[M][hb::c_nvar(MODEL)],
                                                     float (&tv)[M][hb::c_nvar(MODEL)], const bool (&act)[M], int lane, int n_steps,
                                                     const float* nbase, size_t nstride, const float* noise_scale, float dt,
                                                     float dt_half) {
    constexpr int NVAR = hb::c_nvar(MODEL), NCV = hb::c_ncvar(MODEL);
    const float ca = cp[0], cb = cp[1], w = P.w, nsrc = (float)P.nsrc;
    const bool mean = P.kind == HBK_MEAN;
    float ns[NVAR];
#pragma unroll
    for (int v = 0; v < NVAR; v++) ns[v] = noise_scale[v];
    float nz_next[M][NVAR];
#pragma unroll
    for (int q = 0; q < M; q++)
#pragma unroll
        for (int v = 0; v < NVAR; v++) nz_next[q][v] = (STOCH && act[q]) ? __ldcs(nbase + (size_t)(lane + 32 * q) * NVAR + v) : 0.0f;
    for (int it = 0; it < n_steps; it++) {
        float nz[M][NVAR];
#pragma unroll
        for (int q = 0; q < M; q++)
#pragma unroll
            for (int v = 0; v < NVAR; v++) nz[q][v] = nz_next[q][v] * ns[v];
        if (STOCH && it + 1 < n_steps) {
            const float* np = nbase + (size_t)(it + 1) * nstride;
#pragma unroll
            for (int q = 0; q < M; q++)
#pragma unroll
                for (int v = 0; v < NVAR; v++) nz_next[q][v] = act[q] ? __ldcs(np + (size_t)(lane + 32 * q) * NVAR + v) : 0.0f;
        }
        if (mean) {
            float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
            for (int q = 0; q < M; q++) {
                if (!act[q]) continue;
                s0 += x[q][0];
                if (NCV > 1) s1 += x[q][1];
            }
            s0 = hb::warp_sum(s0);
            if (NCV > 1) s1 = hb::warp_sum(s1);
            const float c0 = ((s0 / nsrc) * w) * ca + cb;
            const float c1 = NCV > 1 ? ((s1 / nsrc) * w) * ca + cb : 0.0f;
            heun_linear_nodes<MODEL, M, STOCH, SF>(x, prm, c0, c1, nz, dt, dt_half);
        } else {
            // diagonal form: each node's own coupling value
            float xs[M][NVAR];
#pragma unroll
            for (int q = 0; q < M; q++) {
#pragma unroll
                for (int v = 0; v < NVAR; v++) xs[q][v] = x[q][v];
            }
#pragma unroll
            for (int q = 0; q < M; q++) {
                float one[1][NVAR], n1[1][NVAR];
#pragma unroll
                for (int v = 0; v < NVAR; v++) { one[0][v] = xs[q][v]; n1[0][v] = nz[q][v]; }
                const float c0 = (w * xs[q][0]) * ca + cb;
                const float c1 = NCV > 1 ? (w * xs[q][1]) * ca + cb : 0.0f;
                heun_linear_nodes<MODEL, 1, STOCH, SF>(one, prm, c0, c1, n1, dt, dt_half);
#pragma unroll
                for (int v = 0; v < NVAR; v++) x[q][v] = one[0][v];
            }
        }
#pragma unroll
        for (int q = 0; q < M; q++)
#pragma unroll
            for (int v = 0; v < NVAR; v++) tv[q][v] = act[q] ? tv[q][v] + x[q][v] : 0.0f;
    }
}

template <int MODEL, int M>
__global__ void __launch_bounds__(32) single_warp_kernel(const DevNet* __restrict__ gnet, RunArgs a) {
    constexpr int NVAR = hb::c_nvar(MODEL), NCV = hb::c_ncvar(MODEL);
    __shared__ DevProj P;
    __shared__ float noise_scale[8];
    {
        const int* src = reinterpret_cast<const int*>(&gnet->proj[0]);
        int* dst = reinterpret_cast<int*>(&P);
        for (int i = threadIdx.x; i < (int)(sizeof(DevProj) / 4); i += 32) dst[i] = src[i];
        if (threadIdx.x < 8) noise_scale[threadIdx.x] = gnet->noise_scale[threadIdx.x];
    }
    __syncwarp();
    const int b = blockIdx.x, lane = threadIdx.x;
    const int nm = gnet->sub[0].nm, state_len = gnet->state_len, B = gnet->B;
    const int integ = gnet->sub[0].integ, sweep_form = gnet->sub[0].sweep_form;
    const float dt = gnet->dt, dt_half = gnet->dt_half, h2 = gnet->dt_h2, h6 = gnet->dt_sixth;
    const bool stoch = (integ == HBI_EULER_STOCH || integ == HBI_HEUN_STOCH || integ == HBI_RK4_STOCH);
    float prm[HB_PSTRIDE];
    {
        const float* pr = gnet->sub[0].params + (size_t)b * HB_PSTRIDE;
#pragma unroll
        for (int i = 0; i < HB_PSTRIDE; i++) prm[i] = (i < hb::c_nparams_used(MODEL)) ? pr[i] : 0.0f;
    }
    float cp[8];
    {
        const float* c = P.cp_pp ? P.cp_pp + (size_t)b * HB_NCP : P.cp;
#pragma unroll
        for (int i = 0; i < 8; i++) cp[i] = c[i];
    }
    const bool mean = P.kind == HBK_MEAN;
    const float inv_scale_w = P.w;
    const float nsrc = (float)P.nsrc;
    const bool first_launch_of_run = (a.s0 == a.run_s0);
    float x[M][NVAR], tv[M][NVAR];
    bool act[M];
#pragma unroll
    for (int q = 0; q < M; q++) {
        const int n = lane + 32 * q;
        act[q] = n < nm;
        const size_t base = (size_t)b * state_len + (size_t)(act[q] ? n : 0) * NVAR;
#pragma unroll
        for (int v = 0; v < NVAR; v++) {
            x[q][v] = act[q] ? a.state[base + v] : 0.0f;
            tv[q][v] = (act[q] && !first_launch_of_run) ? a.tavg[base + v] : 0.0f;
        }
    }
    const float* nbase = a.noise + (a.noise_per_point ? (size_t)b * gnet->noise_row : 0);
    const size_t nstride = (size_t)(a.noise_per_point ? B : 1) * gnet->noise_row;
    const bool straight = (integ == HBI_HEUN_STOCH || integ == HBI_HEUN_DET) && P.cfk == HBC_LINEAR && P.direct &&
                          P.pc == NCV && !P.has_rowsums;
    if (straight) {
        if (integ == HBI_HEUN_STOCH) {
            if (sweep_form) single_warp_straight<MODEL, M, true, true>(P, prm, cp, x, tv, act, lane, a.n_steps, nbase, nstride, noise_scale, dt, dt_half);
            else single_warp_straight<MODEL, M, true, false>(P, prm, cp, x, tv, act, lane, a.n_steps, nbase, nstride, noise_scale, dt, dt_half);
        } else {
            if (sweep_form) single_warp_straight<MODEL, M, false, true>(P, prm, cp, x, tv, act, lane, a.n_steps, nbase, nstride, noise_scale, dt, dt_half);
            else single_warp_straight<MODEL, M, false, false>(P, prm, cp, x, tv, act, lane, a.n_steps, nbase, nstride, noise_scale, dt, dt_half);
        }
    }
    float nz_next[M][NVAR];
#pragma unroll
    for (int q = 0; q < M; q++)
#pragma unroll
        for (int v = 0; v < NVAR; v++)
            nz_next[q][v] = (!straight && stoch && act[q]) ? __ldcs(nbase + (size_t)(lane + 32 * q) * NVAR + v) : 0.0f;
    for (int it = 0; it < (straight ? 0 : a.n_steps); it++) {
        // coupling sum: mean over source nodes of pre(x_s), or pre(x_i) of the node itself
        float gmean[4] = {0.f, 0.f, 0.f, 0.f};
        if (mean) {
            float part[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int q = 0; q < M; q++) {
                if (!act[q]) continue;
                float cv[2] = {x[q][0], NCV > 1 ? x[q][1] : 0.0f}, pv[4] = {0.f, 0.f, 0.f, 0.f};
                hb::pre(P.cfk, cp, 0, cv, P.ncv, pv);
#pragma unroll
                for (int c = 0; c < 4; c++) part[c] += pv[c];
            }
#pragma unroll
            for (int c = 0; c < 4; c++) {
                if (c < P.pc) gmean[c] = (hb::warp_sum(part[c]) / nsrc) * inv_scale_w;
            }
        }
        float nz[M][NVAR];
#pragma unroll
        for (int q = 0; q < M; q++)
#pragma unroll
            for (int v = 0; v < NVAR; v++) nz[q][v] = nz_next[q][v] * noise_scale[v];
        if (stoch && it + 1 < a.n_steps) {
            const float* np = nbase + (size_t)(it + 1) * nstride;
#pragma unroll
            for (int q = 0; q < M; q++)
#pragma unroll
                for (int v = 0; v < NVAR; v++)
                    nz_next[q][v] = act[q] ? __ldcs(np + (size_t)(lane + 32 * q) * NVAR + v) : 0.0f;
        }
#pragma unroll
        for (int q = 0; q < M; q++) {
            if (!act[q]) continue;
            float gx[4];
            if (mean) {
#pragma unroll
                for (int c = 0; c < 4; c++) gx[c] = gmean[c];
            } else {
                float cv[2] = {x[q][0], NCV > 1 ? x[q][1] : 0.0f}, pv[4] = {0.f, 0.f, 0.f, 0.f};
                hb::pre(P.cfk, cp, 0, cv, P.ncv, pv);
#pragma unroll
                for (int c = 0; c < 4; c++) gx[c] = P.w * pv[c];
            }
            hb::stream_node_step<MODEL>(P, cp, integ, prm, sweep_form, 0.0f, gx, nz[q], x[q], dt, dt_half, h2, h6);
#pragma unroll
            for (int v = 0; v < NVAR; v++) tv[q][v] = tv[q][v] + x[q][v];
        }
    }
    bool bad = false;
#pragma unroll
    for (int q = 0; q < M; q++) {
        if (!act[q]) continue;
        const size_t base = (size_t)b * state_len + (size_t)(lane + 32 * q) * NVAR;
#pragma unroll
        for (int v = 0; v < NVAR; v++) {
            a.state[base + v] = x[q][v];
            a.tavg[base + v] = tv[q][v];
            bad |= !isfinite(x[q][v]);
        }
    }
    if (a.check_finite && bad) atomicOr(a.flags, 1);
}

template <int MODEL, int M>
cudaError_t launch_single(const DevNet* d_net, const RunArgs& a, int B, cudaStream_t st) {
    single_warp_kernel<MODEL, M><<<B, 32, 0, st>>>(d_net, a);
    return cudaGetLastError();
}

}  // namespace

// nodes per lane M = ceil(nodes / 32) in 1..4
cudaError_t hb_launch_single(int model, int m, const DevNet* d_net, const RunArgs& a, int B, cudaStream_t st) {
    using F = cudaError_t (*)(const DevNet*, const RunArgs&, int, cudaStream_t);
    static const F tab[6][4] = {
        {launch_single<0, 1>, launch_single<0, 2>, launch_single<0, 3>, launch_single<0, 4>},
        {launch_single<1, 1>, launch_single<1, 2>, launch_single<1, 3>, launch_single<1, 4>},
        {launch_single<2, 1>, launch_single<2, 2>, launch_single<2, 3>, launch_single<2, 4>},
        {launch_single<3, 1>, launch_single<3, 2>, launch_single<3, 3>, launch_single<3, 4>},
        {launch_single<4, 1>, launch_single<4, 2>, launch_single<4, 3>, launch_single<4, 4>},
        {launch_single<5, 1>, launch_single<5, 2>, launch_single<5, 3>, launch_single<5, 4>}};
    if (model < 0 || model > 5 || m < 1 || m > 4) return cudaErrorInvalidValue;
    return tab[model][m - 1](d_net, a, B, st);
}
