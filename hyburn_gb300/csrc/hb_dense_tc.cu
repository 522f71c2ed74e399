// hb_dense_tc.cu — undelayed dense coupling on the fifth-generation tensor cores (tcgen05).
//
// The batch engine computes the coupling of a Dense projection without delay as a batched
// matrix product over the sweep points, gx[b, tgt] = sum_src W[tgt, src] * x[b, src]
// (engine.rs:609-620). Here one CTA owns M = 128 sweep points and all N nodes of the network and,
// every step, forms the whole [128 x N] product D = X * W^T with tcgen05.mma (kind::tf32, FP32
// accumulation in tensor memory), issued by one thread. For single-precision agreement the
// product is split into three TF32 products, X_hi W_hi + X_hi W_lo + X_lo W_hi, with
// v_hi = v with its low 13 mantissa bits cleared (exactly what the tensor core reads of an FP32
// operand) and v_lo = v - v_hi; the dropped X_lo W_lo term and the truncation of the lo parts are
// below 2^-21 of each product.
//
// Layout: A = X [128 points][KP sources] and B = W [NP targets][KP sources], both K-major in the
// no-swizzle core-matrix layout (8 rows x 16 bytes per core matrix, core matrices K-adjacent at 128
// bytes, 8-row groups at KP / 4 * 128 bytes), in shared memory; W is arranged on the host once. Tensor
// memory holds, for lane = point, the accumulator D (NP columns), the state x [node][var] and its
// running sum over the run (NPN * nvar columns each, NPN = N rounded up to 16). The CTA runs four
// warpgroups; a warp may only touch the 32 tensor-memory lanes of its quarter (warp % 4), so thread
// (warpgroup g, row r) owns point r and the 8-node chunks g, g + 4, g + 8, ... of that point. After the
// product of a step each thread reads its chunks of its point's row of D, applies the coupling
// post-function and the integrator stages node by node (the same operations in the same order as the
// other kernels; the coupling is held over the stages, engine.rs:697-771), writes the new state back
// and rebuilds its part of the row of X.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "hb_stream.cuh"

namespace hb {
namespace {

constexpr int TC_M = 128;    // sweep points per CTA (the MMA's M)
constexpr int TC_WG = 4;     // warpgroups per CTA, splitting each point's nodes
constexpr int TC_CH = 8;     // nodes per tensor-memory chunk

// byte offset of element (row r, column k) in the K-major no-swizzle core-matrix layout with KP columns
__device__ __forceinline__ uint32_t cm_off(int r, int k, int KP) {
    return (uint32_t)((((r >> 3) * (KP >> 2) + (k >> 2)) << 7) + ((r & 7) << 4) + ((k & 3) << 2));
}

// shared-memory matrix descriptor: start address, leading (K) and stride (M / N) byte offsets of the
// core matrices, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3fffu);
    d |= (uint64_t)((lbo >> 4) & 0x3fffu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3fffu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor of kind::tf32: D f32, A and B tf32, both K-major, N and M
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc) : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 8 consecutive tensor-memory columns of this thread's lane
__device__ __forceinline__ void tc_ld8(uint32_t taddr, float* v) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tc_st8(uint32_t taddr, const float* v) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};"
                 ::"r"(taddr), "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
                   "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
                   "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
                 : "memory");
}

// this thread's row of X for nodes c .. c + 7 (value v of node c + i in v[i]; zero past the last node)
__device__ __forceinline__ void write_x_row(unsigned char* ahi, unsigned char* alo, int row, int c, int KP, const float* v) {
#pragma unroll
    for (int q = 0; q < TC_CH; q += 4) {
        if (c + q >= KP) break;
        float4 h, l;
        float* hp = &h.x;
        float* lp = &l.x;
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const float x = v[q + u];
            const float xh = __uint_as_float(__float_as_uint(x) & 0xffffe000u);
            hp[u] = xh;
            lp[u] = x - xh;
        }
        const uint32_t o = cm_off(row, c + q, KP);
        *reinterpret_cast<float4*>(ahi + o) = h;
        *reinterpret_cast<float4*>(alo + o) = l;
    }
}

template <int MODEL>
__global__ void __launch_bounds__(TC_M * TC_WG, 1) dense_tc_kernel(const DevNet* __restrict__ gnet, RunArgs a,
                                                           const float* __restrict__ wtiles, int NP, int KP, int NPN,
                                                           int ncols) {
    extern __shared__ __align__(128) unsigned char smem[];  // W_hi | W_lo | X_hi | X_lo
    __shared__ DevNet net;
    __shared__ __align__(8) uint64_t mma_bar;
    __shared__ uint32_t tmem_base_s;
    for (int i = threadIdx.x; i < (int)(sizeof(DevNet) / 4); i += blockDim.x)
        reinterpret_cast<int*>(&net)[i] = reinterpret_cast<const int*>(gnet)[i];
    constexpr int NVAR = c_nvar(MODEL);
    const int t = threadIdx.x, warp = t >> 5;
    const int row = ((warp & 3) << 5) | (t & 31), grp = warp >> 2;  // point row of the tile, node-chunk group
    const size_t wbytes = (size_t)NP * KP * 4, abytes = (size_t)TC_M * KP * 4;
    unsigned char* whi = smem;
    unsigned char* wlo = smem + wbytes;
    unsigned char* ahi = smem + 2 * wbytes;
    unsigned char* alo = ahi + abytes;
    {
        const uint4* src = reinterpret_cast<const uint4*>(wtiles);
        uint4* dst = reinterpret_cast<uint4*>(smem);
        const int n16 = (int)(2 * wbytes / 16), a16 = (int)(2 * abytes / 16);
        for (int i = t; i < n16; i += blockDim.x) dst[i] = src[i];
        uint4* az = reinterpret_cast<uint4*>(ahi);
        for (int i = t; i < a16; i += blockDim.x) az[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base_s)),
                     "r"(ncols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (t == 0) {
        mbar_init(&mma_bar, 1);
        mbar_init_fence();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    const int N = net.sub[0].nm, B = net.B;
    const int b = blockIdx.x * TC_M + row;  // this thread's sweep point
    const bool active = b < B;
    const int bb = active ? b : 0;
    const uint32_t tlane = tmem_base_s + ((uint32_t)((warp & 3) * 32) << 16);
    const int c_first = grp * TC_CH, c_step = TC_WG * TC_CH;
    const uint32_t tD = tlane, tX = tlane + (uint32_t)NP, tV = tlane + (uint32_t)(NP + NVAR * NPN);
    const DevProj& P = net.proj[0];
    const int integ = net.sub[0].integ, sweep_form = net.sub[0].sweep_form;
    float prm[HB_PSTRIDE];
    {
        const float* pr = net.sub[0].params + (size_t)bb * HB_PSTRIDE;
#pragma unroll
        for (int i = 0; i < HB_PSTRIDE; i++) prm[i] = (i < c_nparams_used(MODEL)) ? pr[i] : 0.0f;
    }
    float cp[8];
    {
        const float* c = P.cp_pp ? P.cp_pp + (size_t)bb * HB_NCP : P.cp;
#pragma unroll
        for (int i = 0; i < 8; i++) cp[i] = c[i];
    }
    const float dt = net.dt, dt_half = net.dt_half, h2 = net.dt_h2, h6 = net.dt_sixth;
    const float* noise_base = a.noise + (a.noise_per_point ? (size_t)bb * net.noise_row : 0);
    const size_t nstride = (size_t)(a.noise_per_point ? B : 1) * net.noise_row;
    const size_t st_base = (size_t)bb * net.state_len;
    const bool first_launch_of_run = (a.s0 == a.run_s0);

    // the start state and running sums into tensor memory, X of the first step into shared memory
    for (int c = c_first; c < NPN; c += c_step) {
        float xr[TC_CH * NVAR], vr[TC_CH * NVAR], x0[TC_CH];
#pragma unroll
        for (int i = 0; i < TC_CH; i++) {
            const int n = c + i;
            const bool ok = active && n < N;
#pragma unroll
            for (int v = 0; v < NVAR; v++) {
                xr[i * NVAR + v] = ok ? a.state[st_base + (size_t)n * NVAR + v] : 0.0f;
                vr[i * NVAR + v] = (ok && !first_launch_of_run) ? a.tavg[st_base + (size_t)n * NVAR + v] : 0.0f;
            }
            x0[i] = xr[i * NVAR];
        }
#pragma unroll
        for (int v = 0; v < NVAR; v++) {
            tc_st8(tX + (uint32_t)(c * NVAR + v * TC_CH), xr + v * TC_CH);
            tc_st8(tV + (uint32_t)(c * NVAR + v * TC_CH), vr + v * TC_CH);
        }
        write_x_row(ahi, alo, row, c, KP, x0);
    }
    tc_wait_st();

    const uint32_t idesc = idesc_tf32(TC_M, NP);
    const uint32_t sbo = (uint32_t)(KP >> 2) << 7;
    const uint32_t s_whi = smem_addr(whi), s_wlo = smem_addr(wlo), s_ahi = smem_addr(ahi), s_alo = smem_addr(alo);
    bool bad = false;
    // the step loop with the integrator fixed at compile time: only that integrator's code is live in the
    // instruction cache while the 8 node updates of a chunk run unrolled
    auto run_steps = [&](auto integ_tag) {
        constexpr int IG = decltype(integ_tag)::value;
        constexpr bool STOCH = IG == HBI_EULER_STOCH || IG == HBI_HEUN_STOCH || IG == HBI_RK4_STOCH;
        for (int s = 0; s < a.n_steps; s++) {
            // X of this step visible to the tensor core; the last step's reads of D finished
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
            if (t == 0) {
                tc_fence_after();
                const int nk = KP >> 3;
                for (int kk = 0; kk < nk; kk++)
                    tc_mma(tD, smem_desc(s_ahi + kk * 256, 128, sbo), smem_desc(s_whi + kk * 256, 128, sbo), idesc, kk > 0);
                for (int kk = 0; kk < nk; kk++)
                    tc_mma(tD, smem_desc(s_ahi + kk * 256, 128, sbo), smem_desc(s_wlo + kk * 256, 128, sbo), idesc, 1);
                for (int kk = 0; kk < nk; kk++)
                    tc_mma(tD, smem_desc(s_alo + kk * 256, 128, sbo), smem_desc(s_whi + kk * 256, 128, sbo), idesc, 1);
                tc_commit(&mma_bar);
            }
            if (!mbar_wait(&mma_bar, (uint32_t)(s & 1))) atomicOr(a.flags + 1, 4);
            tc_fence_after();
            for (int c = c_first; c < NPN; c += c_step) {
                float dr[TC_CH], xr[TC_CH * NVAR], x0[TC_CH];
                tc_ld8(tD + (uint32_t)c, dr);
#pragma unroll
                for (int v = 0; v < NVAR; v++) tc_ld8(tX + (uint32_t)(c * NVAR + v * TC_CH), xr + v * TC_CH);
                tc_wait_ld();
#pragma unroll
                for (int i = 0; i < TC_CH; i++) {
                    const int n = c + i;
                    float* x = xr + i * NVAR;
                    if (active && n < N) {
                        float gx[4] = {dr[i], 0.0f, 0.0f, 0.0f};
                        float nz[NVAR];
#pragma unroll
                        for (int v = 0; v < NVAR; v++)
                            nz[v] = STOCH ? noise_base[(size_t)s * nstride + (size_t)n * NVAR + v] * net.noise_scale[v] : 0.0f;
                        stream_node_step<MODEL>(P, cp, IG, prm, sweep_form, 0.0f, gx, nz, x, dt, dt_half, h2, h6);
                    }
                    x0[i] = (active && n < N) ? x[0] : 0.0f;
                }
#pragma unroll
                for (int v = 0; v < NVAR; v++) tc_st8(tX + (uint32_t)(c * NVAR + v * TC_CH), xr + v * TC_CH);
                write_x_row(ahi, alo, row, c, KP, x0);
                // running sums, one variable block at a time (padded nodes and rows past the batch hold
                // zero states, so adding them changes nothing)
#pragma unroll
                for (int v = 0; v < NVAR; v++) {
                    float vr[TC_CH];
                    tc_ld8(tV + (uint32_t)(c * NVAR + v * TC_CH), vr);
                    tc_wait_ld();
#pragma unroll
                    for (int i = 0; i < TC_CH; i++) vr[i] = vr[i] + xr[v * TC_CH + i];
                    tc_st8(tV + (uint32_t)(c * NVAR + v * TC_CH), vr);
                }
            }
            tc_wait_st();
        }
    };
    switch (integ) {
    case HBI_HEUN_DET: run_steps(std::integral_constant<int, HBI_HEUN_DET>()); break;
    case HBI_HEUN_STOCH: run_steps(std::integral_constant<int, HBI_HEUN_STOCH>()); break;
    case HBI_EULER: run_steps(std::integral_constant<int, HBI_EULER>()); break;
    case HBI_EULER_STOCH: run_steps(std::integral_constant<int, HBI_EULER_STOCH>()); break;
    case HBI_RK4: run_steps(std::integral_constant<int, HBI_RK4>()); break;
    default: run_steps(std::integral_constant<int, HBI_RK4_STOCH>()); break;
    }
    // state and running sums out
    for (int c = c_first; c < NPN; c += c_step) {
        float xr[TC_CH * NVAR], vr[TC_CH * NVAR];
#pragma unroll
        for (int v = 0; v < NVAR; v++) {
            tc_ld8(tX + (uint32_t)(c * NVAR + v * TC_CH), xr + v * TC_CH);
            tc_ld8(tV + (uint32_t)(c * NVAR + v * TC_CH), vr + v * TC_CH);
        }
        tc_wait_ld();
#pragma unroll
        for (int i = 0; i < TC_CH; i++) {
            const int n = c + i;
            if (!active || n >= N) continue;
#pragma unroll
            for (int v = 0; v < NVAR; v++) {
                a.state[st_base + (size_t)n * NVAR + v] = xr[i * NVAR + v];
                a.tavg[st_base + (size_t)n * NVAR + v] = vr[i * NVAR + v];
                bad |= !isfinite(xr[i * NVAR + v]);
            }
        }
    }
    if (a.check_finite && bad) atomicOr(a.flags, 1);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base_s), "r"(ncols) : "memory");
    }
}

template <int MODEL>
cudaError_t launch_dense_tc(const DevNet* d_net, const RunArgs& a, int B, const float* wtiles, int NP, int KP, int NPN,
                            cudaStream_t st) {
    const int ncols_need = NP + 2 * c_nvar(MODEL) * NPN;
    int ncols = 32;
    while (ncols < ncols_need) ncols <<= 1;
    if (ncols > 512) return cudaErrorInvalidValue;
    const size_t smem = (size_t)2 * NP * KP * 4 + (size_t)2 * TC_M * KP * 4;
    cudaError_t e = cudaFuncSetAttribute(dense_tc_kernel<MODEL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dense_tc_kernel<MODEL><<<(B + TC_M - 1) / TC_M, TC_M * TC_WG, smem, st>>>(d_net, a, wtiles, NP, KP, NPN, ncols);
    return cudaGetLastError();
}

}  // namespace
}  // namespace hb

// Host side: W arranged in the core-matrix layout as the hi and lo TF32 parts ([2][NP x KP] floats),
// and the launch. Models with one coupling variable and tensor memory for their state: G2DO, RWW,
// JansenRit, WilsonCowan.
int hb_dense_tc_tmem_columns(int model, int nm) {
    static const int nvar[6] = {2, 2, 1, 1, 6, 2};
    if (model < 0 || model > 5) return 1 << 30;
    const int NP = (nm + 15) / 16 * 16;
    return NP + 2 * nvar[model] * NP;
}

void hb_dense_tc_tiles(const float* w, int nm, int NP, int KP, float* out) {
    for (size_t i = 0; i < (size_t)2 * NP * KP; i++) out[i] = 0.0f;
    for (int r = 0; r < nm; r++)
        for (int k = 0; k < nm; k++) {
            const float x = w[(size_t)r * nm + k];
            uint32_t u;
            memcpy(&u, &x, 4);
            u &= 0xffffe000u;
            float hi;
            memcpy(&hi, &u, 4);
            const size_t o = ((size_t)((r >> 3) * (KP >> 2) + (k >> 2)) << 5) + ((r & 7) << 2) + (k & 3);
            out[o] = hi;
            out[(size_t)NP * KP + o] = x - hi;
        }
}

cudaError_t hb_launch_dense_tc(int model, const DevNet* d_net, const RunArgs& a, int B, const float* wtiles, int NP, int KP,
                               int NPN, cudaStream_t st) {
    switch (model) {
    case HBM_G2DO: return hb::launch_dense_tc<HBM_G2DO>(d_net, a, B, wtiles, NP, KP, NPN, st);
    case HBM_RWW: return hb::launch_dense_tc<HBM_RWW>(d_net, a, B, wtiles, NP, KP, NPN, st);
    case HBM_JR: return hb::launch_dense_tc<HBM_JR>(d_net, a, B, wtiles, NP, KP, NPN, st);
    case HBM_WC: return hb::launch_dense_tc<HBM_WC>(d_net, a, B, wtiles, NP, KP, NPN, st);
    default: return cudaErrorInvalidValue;
    }
}
