/*
 * sc_kernels.cuh -- the stream-collide kernels, templated on the storage
 * format S and on the population layout LAY (Level::blocked: structure of
 * arrays, or blocks of 32 nodes).  lbm_kernels.cu instantiates the
 * structure-of-arrays kernels and lbm_blocked.cu the blocked ones, so that
 * the two sets compile in parallel.
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
 * so the stored numbers are small deviations and keep their relative precision.
 * ld / st convert between stored values and populations; ldr / str / st2 move
 * stored values as they are (st2: two adjacent elements with one store). */
template <class S> struct Fmt;
template <> struct Fmt<float> {
    using T = float;
    static __device__ __forceinline__ float ldr(const float* p) { return __ldg(p); }
    static __device__ __forceinline__ void str(float* p, float v) { *p = v; }
    static __device__ __forceinline__ void st2(float* p, float a, float b) {
        *reinterpret_cast<float2*>(p) = make_float2(a, b);
    }
    static __device__ __forceinline__ float ld(const float* p, float) { return __ldg(p); }
    static __device__ __forceinline__ void st(float* p, float v, float) { *p = v; }
};
template <> struct Fmt<double> {
    using T = double;
    static __device__ __forceinline__ double ldr(const double* p) { return __ldg(p); }
    static __device__ __forceinline__ void str(double* p, double v) { *p = v; }
    static __device__ __forceinline__ void st2(double* p, double a, double b) {
        *reinterpret_cast<double2*>(p) = make_double2(a, b);
    }
    static __device__ __forceinline__ double ld(const double* p, float) { return __ldg(p); }
    static __device__ __forceinline__ void st(double* p, double v, float) { *p = v; }
};
template <> struct Fmt<__half> {
    using T = float;
    static __device__ __forceinline__ float ldr(const __half* p) { return __half2float(__ldg(p)); }
    static __device__ __forceinline__ void str(__half* p, float v) { *p = __float2half_rn(v); }
    static __device__ __forceinline__ void st2(__half* p, float a, float b) {
        *reinterpret_cast<__half2*>(p) = __floats2half2_rn(a, b);
    }
    static __device__ __forceinline__ float ld(const __half* p, float off) { return ldr(p) + off; }
    static __device__ __forceinline__ void st(__half* p, float v, float off) { str(p, v - off); }
};
template <> struct Fmt<__nv_bfloat16> {
    using T = float;
    static __device__ __forceinline__ float ldr(const __nv_bfloat16* p) { return __bfloat162float(__ldg(p)); }
    static __device__ __forceinline__ void str(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }
    static __device__ __forceinline__ void st2(__nv_bfloat16* p, float a, float b) {
        *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(a, b);
    }
    static __device__ __forceinline__ float ld(const __nv_bfloat16* p, float off) { return ldr(p) + off; }
    static __device__ __forceinline__ void st(__nv_bfloat16* p, float v, float off) { str(p, v - off); }
};

/* Per-node addressing of the populations in the two layouts (Level):
 *   0 structure-of-arrays: q qstride + z plane + y pitch + x, each pull the
 *     sum of a population, a z, a y and an x term;
 *   1 blocked: a node's populations sit at compile-time offsets from its
 *     block position, pair_qoff(q) + 2 (x % 32) (population 0 at x % 32),
 *     and a neighbour's at a signed offset of a few elements in x and of
 *     19 pitch / 19 plane in y / z.  The pull of population q is then one
 *     base pointer plus the sum of at most three per-thread offsets plus an
 *     immediate, and the stores of a node one base pointer plus immediates.
 * pull(f, q): the population q arriving from x - c_q; own(f, q): this
 * node's population q; at(f, q, cn): population q of node cn (the
 * neighbours of the inlet / outlet rebuilds). */
template <int LAY> struct NodeIdx;
template <> struct NodeIdx<0> {
    unsigned zb[3], yb[3], xs[3], qs, self;
    __device__ __forceinline__ NodeIdx(const Level& L, unsigned xm, unsigned x, unsigned xp, unsigned ym, unsigned y,
                                       unsigned yp, unsigned zm, unsigned z, unsigned zp) {
        const unsigned plane = unsigned(L.plane), pitch = unsigned(L.pitch);
        zb[0] = zm * plane, zb[1] = z * plane, zb[2] = zp * plane;
        yb[0] = ym * pitch, yb[1] = y * pitch, yb[2] = yp * pitch;
        xs[0] = xm, xs[1] = x, xs[2] = xp;
        qs = unsigned(L.qstride);
        self = zb[1] + yb[1] + x;
    }
    template <class P> __device__ __forceinline__ P* pull(P* f, int q) const {
        return f + (unsigned(q) * qs + zb[1 - cz(q)] + yb[1 - cy(q)] + xs[1 - cx(q)]);
    }
    template <class P> __device__ __forceinline__ P* own(P* f, int q) const { return f + (unsigned(q) * qs + self); }
    template <class P> __device__ __forceinline__ P* at(P* f, int q, unsigned cn) const {
        return f + (unsigned(q) * qs + cn);
    }
};
template <> struct NodeIdx<1> {
    unsigned base, lane;
    int dx[3], dy[3], dz[3]; /* element offsets to the x-1 / x / x+1 (y, z) neighbours' pair slots */
    __device__ __forceinline__ NodeIdx(const Level& L, unsigned xm, unsigned x, unsigned xp, unsigned ym, unsigned y,
                                       unsigned yp, unsigned zm, unsigned z, unsigned zp) {
        const int ry = int(L.pitch) * 19, rz = int(L.plane) * 19;
        lane = x & 31u;
        const unsigned xq = (x >> 5) * BLOCK_ELEMS + 2u * lane;
        base = z * unsigned(rz) + y * unsigned(ry) + xq;
        dx[0] = int((xm >> 5) * BLOCK_ELEMS + 2u * (xm & 31u)) - int(xq);
        dx[1] = 0;
        dx[2] = int((xp >> 5) * BLOCK_ELEMS + 2u * (xp & 31u)) - int(xq);
        dy[0] = (int(ym) - int(y)) * ry, dy[1] = 0, dy[2] = (int(yp) - int(y)) * ry;
        dz[0] = (int(zm) - int(z)) * rz, dz[1] = 0, dz[2] = (int(zp) - int(z)) * rz;
    }
    /* the neighbour part is summed in 32 bits (the element index stays below
     * 2^31) and widened once; the population's constant offset is added to
     * the 64-bit pointer, where it becomes the load's immediate */
    template <class P> __device__ __forceinline__ P* pull(P* f, int q) const {
        if (q == 0) return f + (base - lane);
        return (f + (base + unsigned(dz[1 - cz(q)] + dy[1 - cy(q)] + dx[1 - cx(q)]))) + pair_qoff(q);
    }
    template <class P> __device__ __forceinline__ P* own(P* f, int q) const {
        return q == 0 ? f + (base - lane) : (f + base) + pair_qoff(q);
    }
    template <class P> __device__ __forceinline__ P* at(P* f, int q, unsigned cn) const {
        return f + ((cn >> 5) * BLOCK_ELEMS + pair_qoff(q) + (q == 0 ? 1u : 2u) * (cn & 31u));
    }
};

/* the 19 values g of this node into buffer f: raw stored values (RAW) or
 * populations with the format's offsets removed; the blocked layout writes
 * each opposite pair with one store */
template <class S, int LAY, bool RAW>
__device__ __forceinline__ void store19(const Level& L, S* __restrict__ f, const NodeIdx<LAY>& n,
                                        const typename Fmt<S>::T g[19]) {
    using F = Fmt<S>;
    if constexpr (LAY == 1) {
        F::str(n.own(f, 0), RAW ? g[0] : g[0] - L.off[0]);
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const int q1 = pair_first(k), q2 = opp(q1);
            F::st2(n.own(f, q1), RAW ? g[q1] : g[q1] - L.off[q1], RAW ? g[q2] : g[q2] - L.off[q2]);
        }
    } else {
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            if (RAW) F::str(n.own(f, q), g[q]);
            else F::st(n.own(f, q), g[q], L.off[q]);
        }
    }
}

/* FEAT: compile-time features, chosen at launch from the configuration and
 * the node types present, so a channel kernel carries no lid code (whose
 * 19-entry temporaries would otherwise set every variant's register count) */
constexpr int FEAT_HALFWAY = 1, FEAT_LID = 2, FEAT_CLAMP = 4, FEAT_XBC = 8;
/* FP16 / BF16 with LR7's MRT and no body force: the deviation collision
 * only (other models convert to populations and back) */
constexpr int FEAT_DEVMRT = 16;
/* the relaxation time of each node from the learned closure's last refresh
 * (StepParams::nu) instead of the LES setting */
constexpr int FEAT_NUBUF = 32;

/* FP16 / BF16 nodes collide their stored deviations (no offsets on the way
 * in and out) */
#ifndef LBM_SC_DEV
#define LBM_SC_DEV 1
#endif
/* resident blocks per SM the register allocation must allow (0: no bound)
 * for the FP16 / BF16 deviation kernels without lid or alternate
 * boundaries: 10 blocks of 128 threads, 48 registers, no spills (measured
 * 3 % faster than 9 blocks at 55 registers on the 512 x 128 x 128 channel) */
#ifndef LBM_SC_MINB
#define LBM_SC_MINB 10
#endif

/* the collision, statistics, store and moment export of a non-solid node;
 * f holds populations, or for DEV their stored deviations */
template <class S, int LAY, bool DEVMRT, bool NUBUF>
__device__ __forceinline__ void sc_collide_store(const Level& L, const StepParams& p, S* __restrict__ fB,
                                                 float* __restrict__ stats, float* __restrict__ mom_export,
                                                 const NodeIdx<LAY>& n, typename Fmt<S>::T f[19], unsigned c,
                                                 const int x, const int y, const int z) {
    using T = typename Fmt<S>::T;
    constexpr bool DEV = LBM_SC_DEV && sizeof(S) == 2;
    const unsigned qs = unsigned(L.qstride);
    /* the learned closure's eddy viscosity of this node from its last
     * refresh, or the configured relaxation */
    const float om = NUBUF ? 1.f / (p.tau0 + 3.f * p.nu[c]) : p.omega;
    const bool les = !NUBUF && p.les != 0;
    if constexpr (DEV && DEVMRT) {
        collide_mrt_dev<T>(f, T(om), les, T(p.tau0), T(p.smag_k), T(L.u_ref));
    } else {
        T dp = T(p.dpdy_dev ? *p.dpdy_dev : p.dpdy);
        if (y > p.dyn_y1) dp = T(0);
        if (DEV) {
#pragma unroll
            for (int q = 0; q < 19; ++q) f[q] += L.off[q];
        }
        collide<T>(p.model, f, T(om), les, T(p.cs), dp);
        if (DEV) {
#pragma unroll
            for (int q = 0; q < 19; ++q) f[q] -= L.off[q];
        }
    }
    if (p.stats_on && p.t >= p.start_av) {
        /* vel_av / vel_fluc (LR7:1018-1058): running mean, then variance */
        T u = 0, v = 0;
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            const T g = DEV ? f[q] + L.off[q] : f[q];
            if (cx(q)) u += T(cx(q)) * g;
            if (cy(q)) v += T(cy(q)) * g;
        }
        float* au = stats;
        float* av = stats + qs;
        const float w = p.stats_weight;
        if (p.t < p.start_fluc) {
            const float nn = float(p.t - p.start_av);
            au[c] = (au[c] * nn + float(u) * w) / (nn + w);
            av[c] = (av[c] * nn + float(v) * w) / (nn + w);
        } else {
            float* fu = stats + 2 * (size_t)qs;
            float* fv = stats + 3 * (size_t)qs;
            const float nn = float(p.t - p.start_fluc);
            const float du = (float(u) - au[c]) * (float(u) - au[c]);
            const float dv = (float(v) - av[c]) * (float(v) - av[c]);
            fu[c] = (fu[c] * nn + du * w) / (nn + w);
            fv[c] = (fv[c] * nn + dv * w) / (nn + w);
        }
    }
    store19<S, LAY, DEV>(L, fB, n, f);
}

/* moments for the coarse->fine interpolation (LR7:1590-1605): post-collision
 * for fluid nodes, the pulled values at bounce-back nodes */
template <class S>
__device__ __forceinline__ void sc_export(const Level& L, const StepParams& p, float* __restrict__ mom_export,
                                          const typename Fmt<S>::T f[19], const int x, const int y, const int z) {
    constexpr bool DEV = LBM_SC_DEV && sizeof(S) == 2;
    const int ex = x - p.exp_x0, ey = y - p.exp_y0;
    if (ex >= 0 && ex < p.exp_nx && ey >= 0 && ey < p.exp_ny) {
        float ff[19], mom[9];
#pragma unroll
        for (int q = 0; q < 19; ++q) ff[q] = DEV ? float(f[q]) + L.off[q] : float(f[q]);
        physical_moments<float>(ff, mom);
        const unsigned ne = unsigned(p.exp_nx * p.exp_ny * L.nz);
        const unsigned ce = (unsigned(z) * p.exp_ny + ey) * p.exp_nx + ex;
#pragma unroll
        for (int i = 0; i < 9; ++i) mom_export[i * ne + ce] = mom[i];
    }
}

/* one node of the step: its addressing, mask byte and coordinates */
template <int LAY> struct ScNode {
    NodeIdx<LAY> n;
    unsigned c;
    int mbyte, type, x, y, z;
};

template <int FEAT, int LAY>
__device__ __forceinline__ ScNode<LAY> sc_setup(const Level& L, const uint8_t* __restrict__ mask, const int x,
                                                const int y, const int z) {
    /* 32-bit element offsets: a level holds fewer than 2^31 elements per
     * buffer (checked at allocation) */
    const unsigned plane = unsigned(L.plane), pitch = unsigned(L.pitch);
    const unsigned c = z * plane + y * pitch + x;
    const int mbyte = mask[c];
    /* periodic neighbours; only boundary nodes, whose pulled values the
     * reference discards or bounces, ever wrap in x or y */
    constexpr bool cl = (FEAT & FEAT_CLAMP) != 0;
    const unsigned xm = (x == 0) ? (cl ? 0 : L.nx - 1) : x - 1;
    const unsigned xp = (x == L.nx - 1) ? (cl ? x : 0) : x + 1;
    const unsigned ym = (y == 0) ? (cl ? 0 : L.ny - 1) : y - 1;
    const unsigned yp = (y == L.ny - 1) ? (cl ? y : 0) : y + 1;
    const unsigned zm = (z == 0) ? (cl ? 0 : L.nz - 1) : z - 1;
    const unsigned zp = (z == L.nz - 1) ? (cl ? z : 0) : z + 1;
    return ScNode<LAY>{NodeIdx<LAY>(L, xm, unsigned(x), xp, ym, unsigned(y), yp, zm, unsigned(z), zp), c, mbyte,
                       mbyte & TYPE_MASK, x, y, z};
}

/* the 19 pulls of a node: populations, or for DEV their stored deviations */
template <class S>
__device__ __forceinline__ constexpr bool sc_dev() { return LBM_SC_DEV && sizeof(S) == 2; }
template <class S, int LAY>
__device__ __forceinline__ void sc_load(const Level& L, const S* __restrict__ fA, const ScNode<LAY>& nd,
                                        typename Fmt<S>::T f[19]) {
    using F = Fmt<S>;
    using T = typename F::T;
#pragma unroll
    for (int q = 0; q < 19; ++q)
        f[q] = sc_dev<S>() ? T(F::ldr(nd.n.pull(fA, q))) : F::ld(nd.n.pull(fA, q), L.off[q]);
}

/* the rest of the node update once its pulls are in f.
 * FP16 / BF16 storage (DEV): the node works on the stored deviations
 * h = f - off and LR7's MRT collides them in that form (collide_mrt_dev),
 * so no population is offset on its way in or out; boundary rebuilds, the
 * lid, the alternate boundaries, the other collision models, the
 * statistics and the moment export see populations f = h + off. */
template <class S, int FEAT, int LAY>
__device__ __forceinline__ void sc_finish(const Level& L, const StepParams& p, const S* __restrict__ fA,
                                          S* __restrict__ fB, float* __restrict__ stats,
                                          float* __restrict__ mom_export, const uint32_t* __restrict__ links,
                                          const ScNode<LAY>& nd, typename Fmt<S>::T f[19]) {
    using F = Fmt<S>;
    using T = typename F::T;
    constexpr bool DEV = sc_dev<S>();
    constexpr bool HALFWAY = (FEAT & FEAT_HALFWAY) != 0;
    const NodeIdx<LAY>& n = nd.n;
    const unsigned c = nd.c, pitch = unsigned(L.pitch);
    const int mbyte = nd.mbyte, type = nd.type, x = nd.x, y = nd.y, z = nd.z;
    /* the neighbours of the inlet / outlet rebuilds (wrapped as the pulls) */
    constexpr bool cl = (FEAT & FEAT_CLAMP) != 0;
    const unsigned xm = (x == 0) ? (cl ? 0 : L.nx - 1) : x - 1;
    const unsigned xp = (x == L.nx - 1) ? (cl ? x : 0) : x + 1;
    const unsigned ym = (y == 0) ? (cl ? 0 : L.ny - 1) : y - 1;
    const unsigned yp = (y == L.ny - 1) ? (cl ? y : 0) : y + 1;
    if (HALFWAY && (mbyte & NEAR_SOLID)) {
        /* a population that would come from a solid node is the node's own
         * post-collision population of the opposite direction, reflected
         * half-way to the solid; links has bit q set for those q */
        const uint32_t lk = links[c];
#pragma unroll
        for (int q = 1; q < 19; ++q)
            if (lk & (1u << q))
                f[q] = DEV ? F::ldr(n.own(fA, opp(q))) + (L.off[opp(q)] - L.off[q])
                           : F::ld(n.own(fA, opp(q)), L.off[opp(q)]);
    }

    if (type == WALL || type == BODY) {
        /* full-way bounce-back (LR7:1493-1526); the momentum exchange of BODY
         * nodes is summed by k_force_list from the same fA */
        T g[19];
#pragma unroll
        for (int q = 0; q < 19; ++q) g[q] = DEV ? f[opp(q)] + (L.off[opp(q)] - L.off[q]) : f[opp(q)];
        store19<S, LAY, DEV>(L, fB, n, g);
        if (p.exp_nx > 0) sc_export<S>(L, p, mom_export, f, x, y, z);
        return;
    } else {
        if (type >= WEST_INLET && type <= NORTH_OUTLET) {
            /* rebuild from the neighbour's stored post-collision state */
            const unsigned cn = type == WEST_INLET ? c - x + xp : type == EAST_OUTLET ? c - x + xm
                              : type == SOUTH_INLET ? c + (yp - y) * pitch : c + (ym - y) * pitch;
#pragma unroll
            for (int q = 0; q < 19; ++q) f[q] = F::ld(n.at(fA, q, cn), L.off[q]);
            T uin = T(p.u_in);
            if (p.noise_amp != 0.f) {
                const uint32_t cell = uint32_t((z * L.ny + y) * L.nx + x);
                const float xi = philox_uniform(p.noise_seed, cell, uint32_t(p.t));
                uin = uin + T(p.u_in) * T(p.noise_amp) * (T(2) * T(xi) - T(1));
            }
            extrap<T>(type, f, T(p.rho_out), uin);
            if (DEV) {
#pragma unroll
                for (int q = 0; q < 19; ++q) f[q] -= L.off[q];
            }
        } else if (((FEAT & FEAT_LID) && type == LID) || ((FEAT & FEAT_XBC) && type >= DIR_WEST)) {
            if (DEV) {
#pragma unroll
                for (int q = 0; q < 19; ++q) f[q] += L.off[q];
            }
            if ((FEAT & FEAT_LID) && type == LID) {
                lid<T>(f, p.lid_face, T(p.lid_u[0]), T(p.lid_u[1]), T(p.lid_u[2]), p.lid_quirk != 0);
            } else if (FEAT & FEAT_XBC) {
                alt_boundary<T>(type, f, x, y, z, L.nx, L.ny, L.nz, T(p.u_in), p.t);
            }
            if (DEV) {
#pragma unroll
                for (int q = 0; q < 19; ++q) f[q] -= L.off[q];
            }
        }
        sc_collide_store<S, LAY, (FEAT & FEAT_DEVMRT) != 0, (FEAT & FEAT_NUBUF) != 0>(L, p, fB, stats, mom_export, n,
                                                                                      f, c, x, y, z);
    }
    if (p.exp_nx > 0) sc_export<S>(L, p, mom_export, f, x, y, z);
}


/* the node update of one node (x, y, z) inside the level */
template <class S, int FEAT, int LAY>
__device__ __forceinline__ void sc_node(const Level& L, const StepParams& p, const S* __restrict__ fA,
                                        S* __restrict__ fB, const uint8_t* __restrict__ mask,
                                        float* __restrict__ stats, float* __restrict__ mom_export,
                                        const uint32_t* __restrict__ links, const int x, const int y, const int z) {
    const ScNode<LAY> nd = sc_setup<FEAT, LAY>(L, mask, x, y, z);
    typename Fmt<S>::T f[19];
    sc_load<S, LAY>(L, fA, nd, f);
    sc_finish<S, FEAT, LAY>(L, p, fA, fB, stats, mom_export, links, nd, f);
}

template <int FEAT> __host__ __device__ constexpr int sc_min_blocks() {
    return (FEAT & FEAT_DEVMRT) && !(FEAT & (FEAT_LID | FEAT_XBC)) ? LBM_SC_MINB : 0;
}

template <class S, int FEAT, int LAY>
__global__ void __launch_bounds__(SC_BX* SC_BY, sc_min_blocks<FEAT>()) k_stream_collide(const Level L, const StepParams p,
                                                                  const S* __restrict__ fA, S* __restrict__ fB,
                                                                  const uint8_t* __restrict__ mask,
                                                                  float* __restrict__ stats,
                                                                  float* __restrict__ mom_export,
                                                                  const uint32_t* __restrict__ links) {
    const int x = blockIdx.x * SC_BX + threadIdx.x;
    const int y = blockIdx.y * SC_BY + threadIdx.y;
    if (x >= L.nx || y >= L.ny) return;
    sc_node<S, FEAT, LAY>(L, p, fA, fB, mask, stats, mom_export, links, x, y, int(blockIdx.z));
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
/* resident blocks per SM the closure kernel is compiled for */
#ifndef LBM_MLP_MINB
#define LBM_MLP_MINB 7
#endif
template <class S, bool HALFWAY, int LAY>
__global__ void __launch_bounds__(SC_BX* MLP_BY, LBM_MLP_MINB) k_stream_collide_mlp(const Level L, const StepParams p,
                                                                      const S* __restrict__ fA, S* __restrict__ fB,
                                                                      const uint8_t* __restrict__ mask,
                                                                      float* __restrict__ stats,
                                                                      const uint32_t* __restrict__ links,
                                                                      const unsigned char* __restrict__ blob,
                                                                      int* __restrict__ err) {
    using F = Fmt<S>;
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
    /* the node of this thread in tile g */
    auto node_of = [&](int g, int& x, int& y, int& z) {
        z = g / (tiles_x * tiles_y);
        const int r = g - z * tiles_x * tiles_y;
        x = (r % tiles_x) * SC_BX + int(threadIdx.x);
        y = (r / tiles_x) * MLP_BY + int(threadIdx.y);
    };
    auto node_idx = [&](int x, int y, int z) {
        const unsigned xm = (x == 0) ? L.nx - 1 : x - 1, xp = (x == L.nx - 1) ? 0 : x + 1;
        const unsigned ym = (y == 0) ? L.ny - 1 : y - 1, yp = (y == L.ny - 1) ? 0 : y + 1;
        const unsigned zm = (z == 0) ? L.nz - 1 : z - 1, zp = (z == L.nz - 1) ? 0 : z + 1;
        return NodeIdx<LAY>(L, xm, unsigned(x), xp, ym, unsigned(y), yp, zm, unsigned(z), zp);
    };
    for (int g = blockIdx.x; g < ntiles; g += gridDim.x) {
        int x, y, z;
        node_of(g, x, y, z);
        const bool live = x < L.nx && y < L.ny;
        float f[19];
        int type = FLUID;
        unsigned c = 0;
        const unsigned xm = (x == 0) ? L.nx - 1 : x - 1, xp = (x == L.nx - 1) ? 0 : x + 1;
        const unsigned ym = (y == 0) ? L.ny - 1 : y - 1, yp = (y == L.ny - 1) ? 0 : y + 1;
        const NodeIdx<LAY> n = node_idx(x, y, z);
        if (live) {
            c = unsigned(z) * plane + unsigned(y) * pitch + unsigned(x);
            const int mbyte = mask[c];
            type = mbyte & TYPE_MASK;
#pragma unroll
            for (int q = 0; q < 19; ++q) f[q] = F::ld(n.pull(fA, q), L.off[q]);
            if (HALFWAY && (mbyte & NEAR_SOLID)) {
                const uint32_t lk = links[c];
#pragma unroll
                for (int q = 1; q < 19; ++q)
                    if (lk & (1u << q)) f[q] = F::ld(n.own(fA, opp(q)), L.off[opp(q)]);
            }
            if (type >= WEST_INLET && type <= NORTH_OUTLET) {
                const unsigned cn = type == WEST_INLET ? c - x + xp : type == EAST_OUTLET ? c - x + xm
                                  : type == SOUTH_INLET ? c + (yp - y) * pitch : c + (ym - y) * pitch;
#pragma unroll
                for (int q = 0; q < 19; ++q) f[q] = F::ld(n.at(fA, q, cn), L.off[q]);
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
        /* bounce-back nodes are done before the closure, so that only the
         * moments stay live across its tensor-core round trips */
        const bool solid = live && (type == WALL || type == BODY);
        if (solid) {
            float gb[19];
#pragma unroll
            for (int q = 0; q < 19; ++q) gb[q] = f[opp(q)];
            store19<S, LAY, false>(L, fB, n, gb);
        }
        /* the closure for the whole tile; the collision's moments give
         * Pi_neq (the projected MRT collision on full populations) */
        const MrtDev<float> mo = mrt_dev_moments<float>(f, 0.f);
        float p6[6], xf[sgs::NIN];
        mrt_dev_pi(mo, p6);
        const float sc = -1.5f / mo.rho;
#pragma unroll
        for (int k = 0; k < 6; ++k) p6[k] *= sc;
        sgs::features_fast(p6, tau0, inv_t0, xf);
        /* across the tensor-core round trips only rho, j and the five
         * stresses stay live; the products are formed again afterwards */
        float keep[10] = {mo.rho, mo.jx, mo.jy, mo.jz, mo.n9, mo.n11, mo.n13, mo.n14, mo.n15,
                          sgs::strain_gain(xf, inv_t0)};
        const float o = sgs::infer_nu<ROWS>(sm, xf, err);
        if (o < 0.f) break; /* a tensor-core wait ran out (block-uniform) */
        if (!live || solid) continue;
#pragma unroll
        for (int k = 0; k < 10; ++k) asm volatile("" : "+f"(keep[k]));
        const float nu = o * keep[9];
        if (p.nu) p.nu[c] = nu;
        MrtDev<float> mr;
        mr.rho = keep[0], mr.jx = keep[1], mr.jy = keep[2], mr.jz = keep[3], mr.n9 = keep[4], mr.n11 = keep[5];
        mr.n13 = keep[6], mr.n14 = keep[7], mr.n15 = keep[8], mr.n1 = 0.f;
        mrt_dev_complete(mr, 0.f);
        mrt_dev_relax(f, mr, 1.f / (tau0 + 3.f * nu));
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
                const float nn = float(p.t - p.start_av);
                au[c] = (au[c] * nn + u * w) / (nn + w);
                av[c] = (av[c] * nn + v * w) / (nn + w);
            } else {
                float* fu = stats + 2 * (size_t)qs;
                float* fv = stats + 3 * (size_t)qs;
                const float nn = float(p.t - p.start_fluc);
                fu[c] = (fu[c] * nn + (u - au[c]) * (u - au[c]) * w) / (nn + w);
                fv[c] = (fv[c] * nn + (v - av[c]) * (v - av[c]) * w) / (nn + w);
            }
        }
        store19<S, LAY, false>(L, fB, n, f);
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
template <int LAY>
inline cudaError_t launch_sc_layout(const Level& L, const StepParams& p, const void* fA, void* fB,
                                    const uint8_t* mask, float* stats, float* mom_export, cudaStream_t s,
                                    const uint32_t* links) {
    const dim3 block(SC_BX, SC_BY), grid(L.pitch / SC_BX, (L.ny + SC_BY - 1) / SC_BY, L.nz);
    const bool reduced = L.storage == STORE_F16 || L.storage == STORE_BF16;
    const int feat = (p.halfway ? FEAT_HALFWAY : 0) | (p.has_lid ? FEAT_LID : 0) | (p.pull_clamp ? FEAT_CLAMP : 0) |
                     (p.has_xbc ? FEAT_XBC : 0) |
                     (reduced && p.model == MRT && p.dpdy == 0.f && !p.dpdy_dev ? FEAT_DEVMRT : 0) |
                     (p.nu_reuse ? FEAT_NUBUF : 0);
#define LBM_SC_CALL(FT)                                                                                          \
    (k_stream_collide<S, FT, LAY><<<grid, block, 0, s>>>(L, p, (const S*)fA, (S*)fB, mask, stats, mom_export, \
                                                          links))
#define LBM_SC(FT)                                                                   \
    if constexpr (LAY != 0) {                                                        \
        LBM_DISPATCH3(L.storage, LBM_SC_CALL(FT))                                    \
    } else {                                                                         \
        if (L.storage == STORE_F64) {                                                \
            using S = double;                                                        \
            LBM_SC_CALL(FT);                                                         \
        } else {                                                                     \
            LBM_DISPATCH3(L.storage, LBM_SC_CALL(FT))                                \
        }                                                                            \
    }
#define LBM_SC_DEV(FT)                                                               \
    if (L.storage == STORE_F16) {                                                    \
        using S = __half;                                                            \
        LBM_SC_CALL(FT);                                                             \
    } else {                                                                         \
        using S = __nv_bfloat16;                                                     \
        LBM_SC_CALL(FT);                                                             \
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
        /* FP16 / BF16 with the deviation MRT collision */
        case 16: LBM_SC_DEV(16); break;
        case 17: LBM_SC_DEV(17); break;
        case 18: LBM_SC_DEV(18); break;
        case 19: LBM_SC_DEV(19); break;
        case 20: LBM_SC_DEV(20); break;
        case 21: LBM_SC_DEV(21); break;
        case 22: LBM_SC_DEV(22); break;
        case 23: LBM_SC_DEV(23); break;
        case 24: LBM_SC_DEV(24); break;
        case 25: LBM_SC_DEV(25); break;
        case 26: LBM_SC_DEV(26); break;
        case 27: LBM_SC_DEV(27); break;
        case 28: LBM_SC_DEV(28); break;
        case 29: LBM_SC_DEV(29); break;
        case 30: LBM_SC_DEV(30); break;
        case 31: LBM_SC_DEV(31); break;
        /* the steps between refreshes of the learned closure (channels:
         * no lid, no alternate boundaries, no clamped pulls) */
        case 32: LBM_SC(32); break;
        case 33: LBM_SC(33); break;
        case 48: LBM_SC_DEV(48); break;
        case 49: LBM_SC_DEV(49); break;
        default: return cudaErrorInvalidValue;
    }
#undef LBM_SC
#undef LBM_SC_DEV
#undef LBM_SC_CALL
    return cudaGetLastError();
}

template <class S, bool HW, int LAY>
static cudaError_t sc_mlp_t(const Level& L, const StepParams& p, const void* fA, void* fB, const uint8_t* mask,
                            float* stats, const uint32_t* links, const void* blob, int* err, cudaStream_t s) {
    const size_t smem = sgs::infer_dyn_smem<SC_BX * MLP_BY>();
    static cudaError_t attr = cudaErrorNotReady;
    static int grid = 0;
    if (attr == cudaErrorNotReady) {
        attr = cudaFuncSetAttribute(k_stream_collide_mlp<S, HW, LAY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    int(smem));
        /* all of the unified L1 / shared array as shared memory, so that the
         * register limit (6 blocks of 128 threads at 80 registers) decides */
        if (attr == cudaSuccess)
            attr = cudaFuncSetAttribute(k_stream_collide_mlp<S, HW, LAY>,
                                        cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        /* resident blocks per SM from the kernel's own limits: registers,
         * shared memory, threads, and TMEM (64 columns of 512 per block) */
        cudaFuncAttributes fa{};
        int dev = 0, sms = 0, regs_sm = 0, smem_sm = 0;
        if (attr == cudaSuccess) attr = cudaFuncGetAttributes(&fa, k_stream_collide_mlp<S, HW, LAY>);
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
    k_stream_collide_mlp<S, HW, LAY><<<grid < ntiles ? grid : ntiles, dim3(SC_BX, MLP_BY), smem, s>>>(
        L, p, (const S*)fA, (S*)fB, mask, stats, links, (const unsigned char*)blob, err);
    return cudaGetLastError();
}

/* the closure's stream-collide launch of one layout (FP32, FP16, BF16) */
template <int LAY>
inline cudaError_t launch_sc_mlp_layout(const Level& L, const StepParams& p, const void* fA, void* fB,
                                        const uint8_t* mask, float* stats, const uint32_t* links, const void* blob,
                                        int* err, cudaStream_t s) {
    switch (L.storage) {
        case STORE_F32:
            return p.halfway ? sc_mlp_t<float, true, LAY>(L, p, fA, fB, mask, stats, links, blob, err, s)
                             : sc_mlp_t<float, false, LAY>(L, p, fA, fB, mask, stats, links, blob, err, s);
        case STORE_F16:
            return p.halfway ? sc_mlp_t<__half, true, LAY>(L, p, fA, fB, mask, stats, links, blob, err, s)
                             : sc_mlp_t<__half, false, LAY>(L, p, fA, fB, mask, stats, links, blob, err, s);
        case STORE_BF16:
            return p.halfway ? sc_mlp_t<__nv_bfloat16, true, LAY>(L, p, fA, fB, mask, stats, links, blob, err, s)
                             : sc_mlp_t<__nv_bfloat16, false, LAY>(L, p, fA, fB, mask, stats, links, blob, err, s);
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
