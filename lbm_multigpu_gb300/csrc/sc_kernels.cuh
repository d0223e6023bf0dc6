/*
 * sc_kernels.cuh -- the stream-collide kernels, templated on the storage
 * format S and on the population layout BLK (structure-of-arrays or blocks of
 * 32 nodes, Level::blocked).  lbm_kernels.cu instantiates the
 * structure-of-arrays kernels and lbm_blocked.cu the blocked ones, so the two
 * sets compile in parallel.
 *
 * k_stream_collide is the hot kernel: one thread per lattice node, a warp
 * spans 32 consecutive x of one row, so every population load and store of a
 * warp touches one aligned run of 32 elements (x-shifted pulls straddle two
 * runs, the neighbour warp's part is then an L2 hit).  It fuses, per node and
 * per step, what the reference spreads over update_inn/update_top/update_bot
 * (LR7:1127-1628):
 *   pull streaming (LR7:1445-1491) with the z halo planes replaced by a
 *   periodic index wrap inside one domain,
 *   full-way bounce-back (LR7:1493-1526), or half-way bounce-back through
 *   per-node link masks,
 *   inlet/outlet rebuilds (LR7:1531-1561), the moving lid,
 *   MRT/BGK collision with Smagorinsky (LR7:583-711, DI3:599-832),
 *   running statistics (LR7:1567-1584),
 *   the coarse-moment export for the refinement (LR7:1590-1605).
 * The momentum exchange on the body (LR7:1607-1626) is summed by a separate
 * kernel, k_force_list, from the same populations.
 */
#pragma once

#include <algorithm>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "d3q19.cuh"
#include "lbm_kernels.cuh"
#include "sgs_infer.cuh"

namespace lbm {

/* ---- storage formats: FP32, FP64, and FP16/BF16 holding f - off with FP32
 * math; off is the equilibrium at the level's reference velocity (Level::off),
 * so the stored numbers are small deviations and keep their relative precision */
template <class S> struct Fmt;
template <> struct Fmt<float> {
    using T = float;
    static __device__ __forceinline__ float ld(const float* p, float) { return __ldg(p); }
    static __device__ __forceinline__ void st(float* p, float v, float) { *p = v; }
};
template <> struct Fmt<double> {
    using T = double;
    static __device__ __forceinline__ double ld(const double* p, float) { return __ldg(p); }
    static __device__ __forceinline__ void st(double* p, double v, float) { *p = v; }
};
template <> struct Fmt<__half> {
    using T = float;
    static __device__ __forceinline__ float ld(const __half* p, float off) { return __half2float(__ldg(p)) + off; }
    static __device__ __forceinline__ void st(__half* p, float v, float off) { *p = __float2half_rn(v - off); }
};
template <> struct Fmt<__nv_bfloat16> {
    using T = float;
    static __device__ __forceinline__ float ld(const __nv_bfloat16* p, float off) {
        return __bfloat162float(__ldg(p)) + off;
    }
    static __device__ __forceinline__ void st(__nv_bfloat16* p, float v, float off) {
        *p = __float2bfloat16_rn(v - off);
    }
};

/* Element offsets of the pulled populations, split into a z term, a y term,
 * an x term and a population term so that a pull is the sum of four table
 * entries:
 *   structure-of-arrays  q qstride + z plane + y pitch + x
 *   blocked              32 q + 19 (z plane + y pitch) + (x / 32) 608 + x % 32
 * In the blocked layout the population term is a compile-time constant, so
 * the 19 pulls and the 19 stores of a node need no per-population address
 * arithmetic beyond an immediate offset. */
template <bool BLK> struct Lay;
template <> struct Lay<false> {
    static __device__ __forceinline__ unsigned zt(const Level& L, unsigned z) { return z * unsigned(L.plane); }
    static __device__ __forceinline__ unsigned yt(const Level& L, unsigned y) { return y * unsigned(L.pitch); }
    static __device__ __forceinline__ unsigned xt(unsigned x) { return x; }
    static __device__ __forceinline__ unsigned qt(const Level& L, int q) { return unsigned(q) * unsigned(L.qstride); }
};
template <> struct Lay<true> {
    static __device__ __forceinline__ unsigned zt(const Level& L, unsigned z) { return z * unsigned(L.plane) * 19u; }
    static __device__ __forceinline__ unsigned yt(const Level& L, unsigned y) { return y * unsigned(L.pitch) * 19u; }
    static __device__ __forceinline__ unsigned xt(unsigned x) { return (x >> 5) * BLOCK_ELEMS + (x & 31u); }
    static __device__ __forceinline__ unsigned qt(const Level&, int q) { return unsigned(q) << 5; }
};

/* FEAT: compile-time features, chosen at launch from the configuration and
 * the node types present, so a channel kernel carries no lid code (whose
 * 19-entry temporaries would otherwise set every variant's register count) */
constexpr int FEAT_HALFWAY = 1, FEAT_LID = 2, FEAT_CLAMP = 4, FEAT_XBC = 8;
/* the node update of one node (x, y, z) inside the level */
template <class S, int FEAT, bool BLK>
__device__ __forceinline__ void sc_node(const Level& L, const StepParams& p, const S* __restrict__ fA,
                                        S* __restrict__ fB, const uint8_t* __restrict__ mask,
                                        float* __restrict__ stats, float* __restrict__ mom_export,
                                        const uint32_t* __restrict__ links, const int x, const int y, const int z) {
    using F = Fmt<S>;
    using T = typename F::T;
    using A = Lay<BLK>;
    /* 32-bit element offsets: a level holds fewer than 2^31 elements per
     * buffer (checked at allocation) */
    const unsigned qs = unsigned(L.qstride);
    const unsigned plane = unsigned(L.plane), pitch = unsigned(L.pitch);
    const unsigned c = z * plane + y * pitch + x;
    const int mbyte = mask[c];
    const int type = mbyte & TYPE_MASK;
    /* under half-way bounce-back nothing pulls from a solid node, which still
     * runs the full-way branch below: an early return here would make the
     * population loads of every warp wait for the mask byte */
    constexpr bool HALFWAY = (FEAT & FEAT_HALFWAY) != 0;
    /* periodic neighbours; only boundary nodes, whose pulled values the
     * reference discards or bounces, ever wrap in x or y */
    constexpr bool cl = (FEAT & FEAT_CLAMP) != 0;
    const unsigned xm = (x == 0) ? (cl ? 0 : L.nx - 1) : x - 1;
    const unsigned xp = (x == L.nx - 1) ? (cl ? x : 0) : x + 1;
    const unsigned ym = (y == 0) ? (cl ? 0 : L.ny - 1) : y - 1;
    const unsigned yp = (y == L.ny - 1) ? (cl ? y : 0) : y + 1;
    const unsigned zm = (z == 0) ? (cl ? 0 : L.nz - 1) : z - 1;
    const unsigned zp = (z == L.nz - 1) ? (cl ? z : 0) : z + 1;
    const unsigned zb[3] = {A::zt(L, zm), A::zt(L, z), A::zt(L, zp)};
    const unsigned yb[3] = {A::yt(L, ym), A::yt(L, y), A::yt(L, yp)};
    const unsigned xs[3] = {A::xt(xm), A::xt(unsigned(x)), A::xt(xp)};
    /* element offset of this node's population 0 */
    const unsigned self = zb[1] + yb[1] + xs[1];

    T f[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        /* pull: the value arriving from x - c_q */
        const unsigned src = A::qt(L, q) + zb[1 - cz(q)] + yb[1 - cy(q)] + xs[1 - cx(q)];
        f[q] = F::ld(fA + src, L.off[q]);
    }
    if (HALFWAY && (mbyte & NEAR_SOLID)) {
        /* a population that would come from a solid node is the node's own
         * post-collision population of the opposite direction, reflected
         * half-way to the solid; links has bit q set for those q */
        const uint32_t lk = links[c];
#pragma unroll
        for (int q = 1; q < 19; ++q)
            if (lk & (1u << q)) f[q] = F::ld(fA + A::qt(L, opp(q)) + self, L.off[opp(q)]);
    }

    if (type == WALL || type == BODY) {
        /* full-way bounce-back (LR7:1493-1526); the momentum exchange of BODY
         * nodes is summed by k_force_list from the same fA */
#pragma unroll
        for (int q = 0; q < 19; ++q) F::st(fB + A::qt(L, q) + self, f[opp(q)], L.off[q]);
    } else {
        if (type >= WEST_INLET && type <= NORTH_OUTLET) {
            /* rebuild from the neighbour's stored post-collision state */
            unsigned nb;
            if (type == WEST_INLET) nb = zb[1] + yb[1] + xs[2];
            else if (type == EAST_OUTLET) nb = zb[1] + yb[1] + xs[0];
            else if (type == SOUTH_INLET) nb = zb[1] + yb[2] + xs[1];
            else nb = zb[1] + yb[0] + xs[1];
#pragma unroll
            for (int q = 0; q < 19; ++q) f[q] = F::ld(fA + A::qt(L, q) + nb, L.off[q]);
            T uin = T(p.u_in);
            if (p.noise_amp != 0.f) {
                const uint32_t cell = uint32_t((z * L.ny + y) * L.nx + x);
                const float xi = philox_uniform(p.noise_seed, cell, uint32_t(p.t));
                uin = uin + T(p.u_in) * T(p.noise_amp) * (T(2) * T(xi) - T(1));
            }
            extrap<T>(type, f, T(p.rho_out), uin);
        } else if ((FEAT & FEAT_LID) && type == LID) {
            lid<T>(f, p.lid_face, T(p.lid_u[0]), T(p.lid_u[1]), T(p.lid_u[2]), p.lid_quirk != 0);
        } else if ((FEAT & FEAT_XBC) && type >= DIR_WEST) {
            alt_boundary<T>(type, f, x, y, z, L.nx, L.ny, L.nz, T(p.u_in), p.t);
        }
        T dp = T(p.dpdy_dev ? *p.dpdy_dev : p.dpdy);
        if (y > p.dyn_y1) dp = T(0);
        collide<T>(p.model, f, T(p.omega), p.les != 0, T(p.cs), dp);

        if (p.stats_on && p.t >= p.start_av) {
            /* vel_av / vel_fluc (LR7:1018-1058): running mean, then variance */
            T u = 0, v = 0;
#pragma unroll
            for (int q = 0; q < 19; ++q) {
                if (cx(q)) u += T(cx(q)) * f[q];
                if (cy(q)) v += T(cy(q)) * f[q];
            }
            float* au = stats;
            float* av = stats + qs;
            const float w = p.stats_weight;
            if (p.t < p.start_fluc) {
                const float n = float(p.t - p.start_av);
                au[c] = (au[c] * n + float(u) * w) / (n + w);
                av[c] = (av[c] * n + float(v) * w) / (n + w);
            } else {
                float* fu = stats + 2 * (size_t)qs;
                float* fv = stats + 3 * (size_t)qs;
                const float n = float(p.t - p.start_fluc);
                const float du = (float(u) - au[c]) * (float(u) - au[c]);
                const float dv = (float(v) - av[c]) * (float(v) - av[c]);
                fu[c] = (fu[c] * n + du * w) / (n + w);
                fv[c] = (fv[c] * n + dv * w) / (n + w);
            }
        }
#pragma unroll
        for (int q = 0; q < 19; ++q) F::st(fB + A::qt(L, q) + self, f[q], L.off[q]);
    }

    if (p.exp_nx > 0) {
        /* moments for the coarse->fine interpolation (LR7:1590-1605):
         * post-collision for fluid nodes, the pulled values at bounce-back nodes */
        const int ex = x - p.exp_x0, ey = y - p.exp_y0;
        if (ex >= 0 && ex < p.exp_nx && ey >= 0 && ey < p.exp_ny) {
            float ff[19], mom[9];
#pragma unroll
            for (int q = 0; q < 19; ++q) ff[q] = float(f[q]);
            physical_moments<float>(ff, mom);
            const unsigned ne = unsigned(p.exp_nx * p.exp_ny * L.nz);
            const unsigned ce = (unsigned(z) * p.exp_ny + ey) * p.exp_nx + ex;
#pragma unroll
            for (int i = 0; i < 9; ++i) mom_export[i * ne + ce] = mom[i];
        }
    }
}

template <class S, int FEAT, bool BLK>
__global__ void __launch_bounds__(SC_BX* SC_BY) k_stream_collide(const Level L, const StepParams p,
                                                                  const S* __restrict__ fA, S* __restrict__ fB,
                                                                  const uint8_t* __restrict__ mask,
                                                                  float* __restrict__ stats,
                                                                  float* __restrict__ mom_export,
                                                                  const uint32_t* __restrict__ links) {
    const int x = blockIdx.x * SC_BX + threadIdx.x;
    const int y = blockIdx.y * SC_BY + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= L.nx || y >= L.ny) return;
    sc_node<S, FEAT, BLK>(L, p, fA, fB, mask, stats, mom_export, links, x, y, z);
}

/* The stream-collide step with the learned subgrid closure in place of the
 * Smagorinsky model: the node update of k_stream_collide (pull, half-way or
 * full-way bounce-back, inlet/outlet rebuild with inlet noise, running
 * statistics; no lid, no clamped edges, no refinement export), with the
 * eddy viscosity of every node from the MLP evaluated on the tensor cores
 * for the whole 32 x 4 tile at once.  Persistent blocks walk the tiles so
 * that each block stages the weights and allocates its TMEM once per launch.
 * MRT collision (LR7:583-711) at tau_eff = tau0 + 3 nu_t; FP32 arithmetic. */
constexpr int MLP_BY = 4; /* tile 32 x 4: one M = 128 MMA per layer */
template <class S, bool HALFWAY, bool BLK>
__global__ void __launch_bounds__(SC_BX* MLP_BY, 6) k_stream_collide_mlp(const Level L, const StepParams p,
                                                                      const S* __restrict__ fA, S* __restrict__ fB,
                                                                      const uint8_t* __restrict__ mask,
                                                                      float* __restrict__ stats,
                                                                      const uint32_t* __restrict__ links,
                                                                      const unsigned char* __restrict__ blob,
                                                                      int* __restrict__ err) {
    using F = Fmt<S>;
    using A = Lay<BLK>;
    constexpr int ROWS = SC_BX * MLP_BY;
    extern __shared__ unsigned char dsm[];
    sgs::InferSmem<ROWS>& sm = *reinterpret_cast<sgs::InferSmem<ROWS>*>(
        (reinterpret_cast<uintptr_t>(dsm) + 1023) & ~uintptr_t(1023));
#if defined(__CUDA_ARCH__)
    sgs::infer_setup<ROWS>(sm, blob);
    const unsigned qs = unsigned(L.qstride);
    const unsigned plane = unsigned(L.plane), pitch = unsigned(L.pitch);
    const int tiles_x = L.pitch / SC_BX, tiles_y = (L.ny + MLP_BY - 1) / MLP_BY;
    const int ntiles = tiles_x * tiles_y * L.nz;
    const float tau0 = 1.f / p.omega, inv_t0 = p.omega;
    for (int g = blockIdx.x; g < ntiles; g += gridDim.x) {
        const int z = g / (tiles_x * tiles_y), r = g - z * tiles_x * tiles_y;
        const int x = (r % tiles_x) * SC_BX + int(threadIdx.x), y = (r / tiles_x) * MLP_BY + int(threadIdx.y);
        const bool live = x < L.nx && y < L.ny;
        float f[19];
        int type = FLUID;
        unsigned c = 0, self = 0;
        if (live) {
            c = unsigned(z) * plane + unsigned(y) * pitch + unsigned(x);
            const int mbyte = mask[c];
            type = mbyte & TYPE_MASK;
            const unsigned xm = (x == 0) ? L.nx - 1 : x - 1, xp = (x == L.nx - 1) ? 0 : x + 1;
            const unsigned ym = (y == 0) ? L.ny - 1 : y - 1, yp = (y == L.ny - 1) ? 0 : y + 1;
            const unsigned zm = (z == 0) ? L.nz - 1 : z - 1, zp = (z == L.nz - 1) ? 0 : z + 1;
            const unsigned zb[3] = {A::zt(L, zm), A::zt(L, z), A::zt(L, zp)};
            const unsigned yb[3] = {A::yt(L, ym), A::yt(L, y), A::yt(L, yp)};
            const unsigned xs[3] = {A::xt(xm), A::xt(unsigned(x)), A::xt(xp)};
            self = zb[1] + yb[1] + xs[1];
#pragma unroll
            for (int q = 0; q < 19; ++q)
                f[q] = F::ld(fA + A::qt(L, q) + zb[1 - cz(q)] + yb[1 - cy(q)] + xs[1 - cx(q)], L.off[q]);
            if (HALFWAY && (mbyte & NEAR_SOLID)) {
                const uint32_t lk = links[c];
#pragma unroll
                for (int q = 1; q < 19; ++q)
                    if (lk & (1u << q)) f[q] = F::ld(fA + A::qt(L, opp(q)) + self, L.off[opp(q)]);
            }
            if (type >= WEST_INLET && type <= NORTH_OUTLET) {
                unsigned nb;
                if (type == WEST_INLET) nb = zb[1] + yb[1] + xs[2];
                else if (type == EAST_OUTLET) nb = zb[1] + yb[1] + xs[0];
                else if (type == SOUTH_INLET) nb = zb[1] + yb[2] + xs[1];
                else nb = zb[1] + yb[0] + xs[1];
#pragma unroll
                for (int q = 0; q < 19; ++q) f[q] = F::ld(fA + A::qt(L, q) + nb, L.off[q]);
                float uin = p.u_in;
                if (p.noise_amp != 0.f) {
                    const uint32_t cell = uint32_t((z * L.ny + y) * L.nx + x);
                    const float xi = philox_uniform(p.noise_seed, cell, uint32_t(p.t));
                    uin = uin + p.u_in * p.noise_amp * (2.f * xi - 1.f);
                }
                extrap<float>(type, f, p.rho_out, uin);
            }
        } else {
#pragma unroll
            for (int q = 0; q < 19; ++q) f[q] = wq(q);
        }
        /* the closure for the whole tile */
        float rho, p6[6], xf[sgs::NIN];
        pi_neq<float>(f, rho, p6);
        const float sc = -1.5f / rho;
#pragma unroll
        for (int k = 0; k < 6; ++k) p6[k] *= sc;
        sgs::features_fast(p6, tau0, inv_t0, xf);
        const float nu = sgs::infer_nu<ROWS>(sm, xf, err);
        if (!live) continue;
        if (type == WALL || type == BODY) {
#pragma unroll
            for (int q = 0; q < 19; ++q) F::st(fB + A::qt(L, q) + self, f[opp(q)], L.off[q]);
            continue;
        }
        collide_mrt<MRT>(f, 1.f / (tau0 + 3.f * nu), false, 0.f, 0.f);
        if (p.stats_on && p.t >= p.start_av) {
            float u = 0, v = 0;
#pragma unroll
            for (int q = 0; q < 19; ++q) {
                if (cx(q)) u += float(cx(q)) * f[q];
                if (cy(q)) v += float(cy(q)) * f[q];
            }
            float* au = stats;
            float* av = stats + qs;
            const float w = p.stats_weight;
            if (p.t < p.start_fluc) {
                const float n = float(p.t - p.start_av);
                au[c] = (au[c] * n + u * w) / (n + w);
                av[c] = (av[c] * n + v * w) / (n + w);
            } else {
                float* fu = stats + 2 * (size_t)qs;
                float* fv = stats + 3 * (size_t)qs;
                const float n = float(p.t - p.start_fluc);
                fu[c] = (fu[c] * n + (u - au[c]) * (u - au[c]) * w) / (n + w);
                fv[c] = (fv[c] * n + (v - av[c]) * (v - av[c]) * w) / (n + w);
            }
        }
#pragma unroll
        for (int q = 0; q < 19; ++q) F::st(fB + A::qt(L, q) + self, f[q], L.off[q]);
    }
    sgs::infer_teardown<ROWS>(sm);
#endif
}

#define LBM_DISPATCH3(storage, KERNEL_CALL)                                  \
    switch (storage) {                                                       \
        case STORE_F32: { using S = float; KERNEL_CALL; } break;             \
        case STORE_F16: { using S = __half; KERNEL_CALL; } break;            \
        case STORE_BF16: { using S = __nv_bfloat16; KERNEL_CALL; } break;    \
        default: return cudaErrorInvalidValue;                               \
    }

/* the stream-collide launch of one layout; FP64 storage only in the
 * structure-of-arrays layout */
template <bool BLK>
inline cudaError_t launch_sc_layout(const Level& L, const StepParams& p, const void* fA, void* fB,
                                    const uint8_t* mask, float* stats, float* mom_export, cudaStream_t s,
                                    const uint32_t* links) {
    const dim3 block(SC_BX, SC_BY), grid = sc_grid(L);
    const int feat = (p.halfway ? FEAT_HALFWAY : 0) | (p.has_lid ? FEAT_LID : 0) | (p.pull_clamp ? FEAT_CLAMP : 0) |
                     (p.has_xbc ? FEAT_XBC : 0);
#define LBM_SC_CALL(FT)                                                                                          \
    (k_stream_collide<S, FT, BLK><<<grid, block, 0, s>>>(L, p, (const S*)fA, (S*)fB, mask, stats, mom_export, \
                                                          links))
#define LBM_SC(FT)                                                                   \
    if constexpr (BLK) {                                                             \
        LBM_DISPATCH3(L.storage, LBM_SC_CALL(FT))                                    \
    } else {                                                                         \
        if (L.storage == STORE_F64) {                                                \
            using S = double;                                                        \
            LBM_SC_CALL(FT);                                                         \
        } else {                                                                     \
            LBM_DISPATCH3(L.storage, LBM_SC_CALL(FT))                                \
        }                                                                            \
    }
    switch (feat) {
        case 0: LBM_SC(0); break;
        case 1: LBM_SC(1); break;
        case 2: LBM_SC(2); break;
        case 3: LBM_SC(3); break;
        case 4: LBM_SC(4); break;
        case 5: LBM_SC(5); break;
        case 6: LBM_SC(6); break;
        case 7: LBM_SC(7); break;
        /* alternate boundaries, with every combination of the others */
        case 8: LBM_SC(8); break;
        case 9: LBM_SC(9); break;
        case 10: LBM_SC(10); break;
        case 11: LBM_SC(11); break;
        case 12: LBM_SC(12); break;
        case 13: LBM_SC(13); break;
        case 14: LBM_SC(14); break;
        case 15: LBM_SC(15); break;
        default: return cudaErrorInvalidValue;
    }
#undef LBM_SC
#undef LBM_SC_CALL
    return cudaGetLastError();
}

template <class S, bool HW, bool BLK>
static cudaError_t sc_mlp_t(const Level& L, const StepParams& p, const void* fA, void* fB, const uint8_t* mask,
                            float* stats, const uint32_t* links, const void* blob, int* err, cudaStream_t s) {
    const size_t smem = sgs::infer_dyn_smem<SC_BX * MLP_BY>();
    static cudaError_t attr = cudaErrorNotReady;
    static int grid = 0;
    if (attr == cudaErrorNotReady) {
        attr = cudaFuncSetAttribute(k_stream_collide_mlp<S, HW, BLK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    int(smem));
        /* all of the unified L1 / shared array as shared memory, so that the
         * register limit (6 blocks of 128 threads at 80 registers) decides */
        if (attr == cudaSuccess)
            attr = cudaFuncSetAttribute(k_stream_collide_mlp<S, HW, BLK>,
                                        cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        /* resident blocks per SM from the kernel's own limits: registers,
         * shared memory, threads, and TMEM (64 columns of 512 per block) */
        cudaFuncAttributes fa{};
        int dev = 0, sms = 0, regs_sm = 0, smem_sm = 0;
        if (attr == cudaSuccess) attr = cudaFuncGetAttributes(&fa, k_stream_collide_mlp<S, HW, BLK>);
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        const int threads = SC_BX * MLP_BY;
        const int regs_block = ((fa.numRegs > 0 ? fa.numRegs : 255) * 32 + 255) / 256 * 256 * (threads / 32);
        int nb = regs_sm / (regs_block > 0 ? regs_block : 1);
        nb = std::min(nb, int(smem_sm / (smem + fa.sharedSizeBytes + 1024)));
        nb = std::min(nb, 2048 / threads);
        nb = std::min(nb, 512 / sgs::tmem_cols<SC_BX * MLP_BY>());
        nb = nb < 1 ? 1 : nb;
        grid = (sms > 0 ? sms : 152) * nb;
    }
    if (attr != cudaSuccess) return attr;
    const int ntiles = (L.pitch / SC_BX) * ((L.ny + MLP_BY - 1) / MLP_BY) * L.nz;
    k_stream_collide_mlp<S, HW, BLK><<<grid < ntiles ? grid : ntiles, dim3(SC_BX, MLP_BY), smem, s>>>(
        L, p, (const S*)fA, (S*)fB, mask, stats, links, (const unsigned char*)blob, err);
    return cudaGetLastError();
}

/* the closure's stream-collide launch of one layout (FP32, FP16, BF16) */
template <bool BLK>
inline cudaError_t launch_sc_mlp_layout(const Level& L, const StepParams& p, const void* fA, void* fB,
                                        const uint8_t* mask, float* stats, const uint32_t* links, const void* blob,
                                        int* err, cudaStream_t s) {
    switch (L.storage) {
        case STORE_F32:
            return p.halfway ? sc_mlp_t<float, true, BLK>(L, p, fA, fB, mask, stats, links, blob, err, s)
                             : sc_mlp_t<float, false, BLK>(L, p, fA, fB, mask, stats, links, blob, err, s);
        case STORE_F16:
            return p.halfway ? sc_mlp_t<__half, true, BLK>(L, p, fA, fB, mask, stats, links, blob, err, s)
                             : sc_mlp_t<__half, false, BLK>(L, p, fA, fB, mask, stats, links, blob, err, s);
        case STORE_BF16:
            return p.halfway ? sc_mlp_t<__nv_bfloat16, true, BLK>(L, p, fA, fB, mask, stats, links, blob, err, s)
                             : sc_mlp_t<__nv_bfloat16, false, BLK>(L, p, fA, fB, mask, stats, links, blob, err, s);
        default: return cudaErrorInvalidValue;
    }
}

/* the blocked-layout launches (lbm_blocked.cu) */
cudaError_t launch_sc_blocked(const Level& L, const StepParams& p, const void* fA, void* fB, const uint8_t* mask,
                              float* stats, float* mom_export, cudaStream_t s, const uint32_t* links);
cudaError_t launch_sc_mlp_blocked(const Level& L, const StepParams& p, const void* fA, void* fB,
                                  const uint8_t* mask, float* stats, const uint32_t* links, const void* blob, int* err,
                                  cudaStream_t s);

}  // namespace lbm
