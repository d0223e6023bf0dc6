/*
 * lbm_kernels.cu -- CUDA kernels of the D3Q19 stream-collide path for sm_103a:
 * the structure-of-arrays instances of the stream-collide kernels
 * (sc_kernels.cuh), and every other kernel of a level in either population
 * layout (pidx): the body-force sums, init, field and population read-outs,
 * the FP64 audit, DI3's inlet control and the refinement exchange.
 */
#include <algorithm>
#include <mutex>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "sc_kernels.cuh"

namespace lbm {

/* DI3's AverageV (DI3:2561-2598) and the P-control update of the body force
 * (DI3:3150-3170) in one block on the device, so the loop needs no host
 * round trip: the y momentum of every node of the plane y1 (all x, all z)
 * summed in FP64 in a fixed order, divided by (nx - 2) nz as the reference
 * does, then dpdy += (mean - umax) / umax * kp * |dpdy0| */
template <class S>
__global__ void __launch_bounds__(256) k_dyn_control(const Level L, const S* __restrict__ f, int y1, float umax,
                                                     float kp, float dpdy0_abs, float* __restrict__ dpdy,
                                                     float* __restrict__ hist3, int t) {
    using F = Fmt<S>;
    __shared__ double red[256];
    double s = 0;
    const int n = L.nx * L.nz;
    for (int i = threadIdx.x; i < n; i += 256) {
        const int x = i % L.nx, z = i / L.nx;
        const size_t c = size_t(z) * L.plane + size_t(y1) * L.pitch + x;
        float v = 0;
#pragma unroll
        for (int q = 0; q < 19; ++q)
            if (cy(q)) v += float(cy(q)) * float(F::ld(f + pidx(L, q, unsigned(c)), L.off[q]));
        s += double(v);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (int(threadIdx.x) < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const float av = float(red[0]) / float((L.nx - 2) * L.nz);
        const float diff = (av - umax) / umax;
        const float d = *dpdy + diff * kp * dpdy0_abs;
        *dpdy = d;
        hist3[0] = float(t);
        hist3[1] = av;
        hist3[2] = d;
    }
}

/* Momentum exchange at BODY nodes (LR7:1494-1502, reduced per block at
 * LR7:1607-1626): F += 2 sum_q c_q f_q over the populations a body node pulls
 * from fA.  Runs over a compact list of body nodes (pitched indices) instead
 * of inside the stream-collide kernel, so the hot kernel carries no FP64 and no
 * block barrier.  Per node the sum is FP32 (as in the reference); across nodes
 * it is FP64: per-block partials, and the last block to finish adds them in
 * block order, so the result does not depend on scheduling. */
constexpr int FORCE_BLOCKS = 152, FORCE_THREADS = 256;
template <class S>
__global__ void __launch_bounds__(FORCE_THREADS) k_force_list(const Level L, const S* __restrict__ fA,
                                                              const unsigned* __restrict__ body, int nbody,
                                                              double* __restrict__ part, unsigned* __restrict__ done,
                                                              double* __restrict__ out3,
                                                              const uint8_t* __restrict__ mask, int halfway) {
    using F = Fmt<S>;
    using T = typename F::T;
    double s[3] = {0.0, 0.0, 0.0};
    const unsigned plane = unsigned(L.plane), pitch = unsigned(L.pitch);
    for (int i = blockIdx.x * FORCE_THREADS + threadIdx.x; i < nbody; i += FORCE_BLOCKS * FORCE_THREADS) {
        const unsigned c = body[i];
        const unsigned z = c / plane, r = c - z * plane;
        const unsigned y = r / pitch, x = r - y * pitch;
        const unsigned xm = (x == 0) ? L.nx - 1 : x - 1, xp = (x == unsigned(L.nx) - 1) ? 0 : x + 1;
        const unsigned ym = (y == 0) ? L.ny - 1 : y - 1, yp = (y == unsigned(L.ny) - 1) ? 0 : y + 1;
        const unsigned zm = (z == 0) ? L.nz - 1 : z - 1, zp = (z == unsigned(L.nz) - 1) ? 0 : z + 1;
        const unsigned zb[3] = {zm * plane, z * plane, zp * plane};
        const unsigned yb[3] = {ym * pitch, y * pitch, yp * pitch};
        const unsigned xs[3] = {xm, x, xp};
        T a[3] = {0, 0, 0};
        if (halfway) {
            /* link-wise exchange at a fluid node next to the body: each
             * population heading into a BODY node (opp(q), arriving back as q)
             * hands over 2 c_opp(q) f*_opp(q) */
#pragma unroll
            for (int q = 1; q < 19; ++q) {
                if ((mask[zb[1 - cz(q)] + yb[1 - cy(q)] + xs[1 - cx(q)]] & TYPE_MASK) != BODY) continue;
                const T v = T(2) * F::ld(fA + pidx(L, opp(q), c), L.off[opp(q)]);
                if (cx(q)) a[0] -= T(cx(q)) * v;
                if (cy(q)) a[1] -= T(cy(q)) * v;
                if (cz(q)) a[2] -= T(cz(q)) * v;
            }
        } else {
#pragma unroll
            for (int q = 1; q < 19; ++q) {
                const T v = T(2) * F::ld(fA + pidx(L, q, zb[1 - cz(q)] + yb[1 - cy(q)] + xs[1 - cx(q)]), L.off[q]);
                if (cx(q)) a[0] += T(cx(q)) * v;
                if (cy(q)) a[1] += T(cy(q)) * v;
                if (cz(q)) a[2] += T(cz(q)) * v;
            }
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) s[k] += double(a[k]);
    }
    __shared__ double red[3][FORCE_THREADS / 32];
    __shared__ bool last;
    for (int k = 0; k < 3; ++k) {
        double v = s[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double v = 0.0;
#pragma unroll
        for (int w = 0; w < FORCE_THREADS / 32; ++w) v += red[threadIdx.x][w];
        part[3 * blockIdx.x + threadIdx.x] = v;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(done, 1u) == gridDim.x - 1);
    __syncthreads();
    if (last) {
        /* warp k sums component k: lane-strided partials, then a fixed shuffle tree */
        const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
        if (k < 3) {
            double v = 0.0;
            for (int b = lane; b < int(gridDim.x); b += 32) v += __ldcg(part + 3 * b + k);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) out3[k] += v;
        }
        if (threadIdx.x == 0) *done = 0u;
    }
}

/* sum n block partials (3 doubles each) in a fixed order; one block */
__global__ void k_reduce3(const double* __restrict__ part, int n, double* __restrict__ out) {
    __shared__ double red[3][32];
    double s[3] = {0.0, 0.0, 0.0};
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        s[0] += part[3LL * i];
        s[1] += part[3LL * i + 1];
        s[2] += part[3LL * i + 2];
    }
    for (int k = 0; k < 3; ++k) {
        double v = s[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double v = 0.0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) v += red[threadIdx.x][w];
        out[threadIdx.x] += v;
    }
}

/* initialize / initializeLR (LR7:1060-1125): rest state at rho = 1 with the
 * x velocity u0 (zero at bounce-back nodes).  kind 0: the MRT equilibrium
 * moments (mrt_meq + InvertMoments); kind 1: the BGK equilibrium; kind 2: the
 * BGK equilibrium at u0 on every node, solids included (CPU:1226-1308). */
template <class S>
__global__ void k_init(const Level L, const uint8_t* __restrict__ mask, S* __restrict__ f, int kind, float u0,
                       int axis) {
    using F = Fmt<S>;
    using T = typename F::T;
    const int x = blockIdx.x * SC_BX + threadIdx.x, y = blockIdx.y * SC_BY + threadIdx.y, z = blockIdx.z;
    if (x >= L.nx || y >= L.ny) return;
    const long long c = z * L.plane + (long long)y * L.pitch + x;
    const int type = mask[c] & TYPE_MASK;
    const T u = (kind != 2 && (type == WALL || type == BODY)) ? T(0) : T(u0);
    T g[19];
    if (kind == 0) {
        T mom[9] = {T(1), T(0), T(0), T(0), T(0), T(0), T(0), T(0), T(0)};
        mom[1 + axis] = u;
        invert_scaled<T>(mom, T(0), g);
    } else {
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            const T cu = T(axis == 0 ? cx(q) : axis == 1 ? cy(q) : cz(q)) * u;
            g[q] = T(wq(q)) * (T(1) + T(3) * cu + T(4.5) * cu * cu - T(1.5) * u * u);
        }
    }
#pragma unroll
    for (int q = 0; q < 19; ++q) F::st(f + pidx(L, q, unsigned(c)), g[q], L.off[q]);
}

/* density and momentum (the reference's u, v, w are momenta) into compact arrays */
template <class S>
__global__ void k_fields(const Level L, const S* __restrict__ f, float* rho, float* u, float* v, float* w) {
    using F = Fmt<S>;
    using T = typename F::T;
    const int x = blockIdx.x * SC_BX + threadIdx.x, y = blockIdx.y * SC_BY + threadIdx.y, z = blockIdx.z;
    if (x >= L.nx || y >= L.ny) return;
    const long long c = z * L.plane + (long long)y * L.pitch + x;
    T r = 0, a = 0, b = 0, d = 0;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const T g = F::ld(f + pidx(L, q, unsigned(c)), L.off[q]);
        r += g;
        if (cx(q)) a += T(cx(q)) * g;
        if (cy(q)) b += T(cy(q)) * g;
        if (cz(q)) d += T(cz(q)) * g;
    }
    const long long o = ((long long)z * L.ny + y) * L.nx + x;
    if (rho) rho[o] = float(r);
    if (u) u[o] = float(a);
    if (v) v[o] = float(b);
    if (w) w[o] = float(d);
}

template <class S> __global__ void k_pack(const Level L, const S* __restrict__ f, float* __restrict__ out) {
    using F = Fmt<S>;
    const int x = blockIdx.x * SC_BX + threadIdx.x, y = blockIdx.y * SC_BY + threadIdx.y, z = blockIdx.z;
    if (x >= L.nx || y >= L.ny) return;
    const long long c = z * L.plane + (long long)y * L.pitch + x;
    const long long n = (long long)L.nx * L.ny * L.nz, o = ((long long)z * L.ny + y) * L.nx + x;
#pragma unroll
    for (int q = 0; q < 19; ++q) out[q * n + o] = float(F::ld(f + pidx(L, q, unsigned(c)), L.off[q]));
}

template <class S> __global__ void k_unpack(const Level L, const float* __restrict__ in, S* __restrict__ f) {
    using F = Fmt<S>;
    const int x = blockIdx.x * SC_BX + threadIdx.x, y = blockIdx.y * SC_BY + threadIdx.y, z = blockIdx.z;
    if (x >= L.nx || y >= L.ny) return;
    const long long c = z * L.plane + (long long)y * L.pitch + x;
    const long long n = (long long)L.nx * L.ny * L.nz, o = ((long long)z * L.ny + y) * L.nx + x;
#pragma unroll
    for (int q = 0; q < 19; ++q) F::st(f + pidx(L, q, unsigned(c)), in[q * n + o], L.off[q]);
}

/* FP64 mass and momentum of the non-solid nodes; grid-stride over rows so the
 * number of block partials is fixed (audit_partials) */
constexpr int AUDIT_BLOCKS = 1216; /* 8 blocks per SM on a 152-SM GB300 */
template <class S>
__global__ void __launch_bounds__(256) k_audit(const Level L, const S* __restrict__ f, const uint8_t* __restrict__ mask,
                                               double* __restrict__ part) {
    using F = Fmt<S>;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const long long rows = (long long)L.ny * L.nz;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (long long r = (long long)blockIdx.x * 8 + warp; r < rows; r += (long long)gridDim.x * 8) {
        const int y = int(r % L.ny), z = int(r / L.ny);
        for (int x = lane; x < L.nx; x += 32) {
            const long long c = z * L.plane + (long long)y * L.pitch + x;
            const int t = mask[c] & TYPE_MASK;
            if (t == WALL || t == BODY) continue;
            typename F::T m[4] = {0, 0, 0, 0};
#pragma unroll
            for (int q = 0; q < 19; ++q) {
                const typename F::T g = F::ld(f + pidx(L, q, unsigned(c)), L.off[q]);
                m[0] += g;
                if (cx(q)) m[1] += cx(q) * g;
                if (cy(q)) m[2] += cy(q) * g;
                if (cz(q)) m[3] += cz(q) * g;
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[k] += double(m[k]);
        }
    }
    __shared__ double red[4][8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        double v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double v = 0.0;
#pragma unroll
        for (int w = 0; w < 8; ++w) v += red[threadIdx.x][w];
        part[4LL * blockIdx.x + threadIdx.x] = v;
    }
}

__global__ void k_audit_final(const double* __restrict__ part, int n, double* __restrict__ out) {
    __shared__ double red[4][8];
    double s[4] = {0, 0, 0, 0};
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        for (int k = 0; k < 4; ++k) s[k] += part[4LL * i + k];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = 0; k < 4; ++k) {
        double v = s[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double v = 0.0;
        for (int w = 0; w < 8; ++w) v += red[threadIdx.x][w];
        out[threadIdx.x] = v;
    }
}

/* ---- refinement exchange ---- */

template <class S>
__device__ __forceinline__ void load19(const Level& L, const S* f, long long c, float g[19]) {
#pragma unroll
    for (int q = 0; q < 19; ++q) g[q] = float(Fmt<S>::ld(f + pidx(L, q, unsigned(c)), L.off[q]));
}

/* second-order correction of the interpolated momentum from the 8 corner
 * strain rates and momenta (LR7:2101-2144, 2270-2316); corner i = x + 2y + 4z.
 * Accumulated one corner at a time as the corners are read (a starts at 0),
 * so that no thread holds all eight corners' moments at once */
__device__ __forceinline__ void second_order_add(float a[9], int i, const float mc[9], const float S[6]) {
    const float sx = (i & 1) ? 1.f : -1.f, sy = (i & 2) ? 1.f : -1.f, sz = (i & 4) ? 1.f : -1.f;
    a[0] += sx * S[0];
    a[1] += sy * S[3] - sx * sy * mc[2];
    a[2] += sz * S[5] - sx * sz * mc[3];
    a[3] += sx * S[3] - sx * sy * mc[1];
    a[4] += sy * S[1];
    a[5] += sz * S[4] - sy * sz * mc[3];
    a[6] += sx * S[5] - sx * sz * mc[1];
    a[7] += sy * S[4] - sy * sz * mc[2];
    a[8] += sz * S[2];
}
__device__ __forceinline__ void second_order_scale(float a[9]) {
#pragma unroll
    for (int j = 0; j < 9; ++j) a[j] *= (j % 4 == 0) ? -0.03125f : -0.0625f;
}

/* InterpCF (LR7:1991-2170): fine nodes of the LRLEVEL-wide x/y band get the
 * coarse moments interpolated (trilinear + second-order velocity correction)
 * and rebuilt with the LES-aware non-equilibrium rescale (LR7:524-579).  One
 * thread per band node; mom_c is [9][cnz][eny][enx] (coarse footprint).
 * With mom_prev (the previous coarse step's export) the corner moments are
 * first interpolated in time, (1 - theta) prev + theta cur. */
/* band nodes of the coarse-to-fine fill */
inline long long cf_nodes(const RefineParams& r) {
    const int L = r.lrlevel;
    return (long long)(r.fny * 2 * L + (r.fnx - 2 * L) * 2 * L) * r.fnz +
           (r.zbounded ? 2LL * L * (r.fnx - 2 * L) * (r.fny - 2 * L) : 0LL);
}

/* the band node idx of the coarse-to-fine fill */
template <class S>
__device__ __forceinline__ void interp_cf_node(const RefineParams& r, const Level& F, const float* __restrict__ mom_c,
                                               const float* __restrict__ mom_prev, float theta, S* __restrict__ f_f,
                                               const uint8_t* __restrict__ mask_f, const long long idx) {
    const int L = r.lrlevel;
    const int nb_x = r.fny * 2 * L;                /* x-band nodes per plane */
    const int nb_y = (r.fnx - 2 * L) * 2 * L;      /* y-band nodes per plane (x-band excluded) */
    const int per_plane = nb_x + nb_y;
    const int inner = (r.fnx - 2 * L) * (r.fny - 2 * L);  /* z-band nodes per plane (bounded patch) */
    const long long nxy = (long long)per_plane * r.fnz;
    if (idx >= nxy + (r.zbounded ? 2LL * L * inner : 0LL)) return;
    int k, xf, yf;
    if (idx < nxy) {
        k = int(idx / per_plane);
        int i = int(idx % per_plane);
        if (i < nb_x) {
            yf = i / (2 * L);
            const int b = i % (2 * L);
            xf = b < L ? b : r.fnx - 2 * L + b;
        } else {
            i -= nb_x;
            xf = L + i / (2 * L);
            const int b = i % (2 * L);
            yf = b < L ? b : r.fny - 2 * L + b;
        }
    } else {
        /* the L bottom and L top planes of a bounded patch, x/y band excluded */
        const int j = int(idx - nxy), b = j / inner, rem = j % inner;
        k = b < L ? b : r.fnz - 2 * L + b;
        xf = L + rem % (r.fnx - 2 * L);
        yf = L + rem / (r.fnx - 2 * L);
    }
    const long long cf = k * F.plane + (long long)yf * F.pitch + xf;
    const int t = mask_f[cf] & TYPE_MASK;
    if (t == WALL || t == BODY) return;
    const float xr = xf * r.lrfactor + r.lrfactor * 0.5f, yr = yf * r.lrfactor + r.lrfactor * 0.5f;
    const int xm = int(xr), ym = int(yr);
    const float fx = xr - xm, fy = yr - ym;
    /* z: periodic full-depth patch (fine plane k at coarse z k / L - 1 +
     * ...), or, bounded, as x and y from the coarse plane cz0 */
    int zb;
    float fz;
    if (r.zbounded) {
        const float zr = k * r.lrfactor + r.lrfactor * 0.5f;
        zb = r.cz0 + int(zr);
        fz = zr - int(zr);
    } else {
        zb = k / L - 1;
        fz = (k % L) * r.lrfactor + r.lrfactor * 0.5f;
    }
    const long long ne = (long long)r.enx * r.eny * r.cnz;
    /* trilinear moments and the second-order terms, one corner at a time */
    float mom[9], a[9];
#pragma unroll
    for (int m = 0; m < 9; ++m) mom[m] = a[m] = 0.f;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        int zc = zb + ((c >> 2) & 1);
        zc = zc < 0 ? zc + r.cnz : (zc >= r.cnz ? zc - r.cnz : zc);
        const long long ce = ((long long)zc * r.eny + (ym + ((c >> 1) & 1))) * r.enx + (xm + (c & 1));
        float mc[9], Sc[6];
#pragma unroll
        for (int m = 0; m < 9; ++m) mc[m] = __ldg(mom_c + m * ne + ce);
        if (mom_prev) {
#pragma unroll
            for (int m = 0; m < 9; ++m) mc[m] = (1.f - theta) * __ldg(mom_prev + m * ne + ce) + theta * mc[m];
        }
        const float wx = (c & 1) ? fx : 1.f - fx, wy = (c & 2) ? fy : 1.f - fy, wz = (c & 4) ? fz : 1.f - fz;
#pragma unroll
        for (int m = 0; m < 9; ++m) mom[m] += mc[m] * wx * wy * wz;
        if (r.order == 2) {
            strain_rate<float>(mc, Sc);
            second_order_add(a, c, mc, Sc);
        }
    }
    if (r.order == 2) {
        second_order_scale(a);
        const float wx = 1.f - (4.f * fx * fx - 4.f * fx + 1.f);
        const float wy = 1.f - (4.f * fy * fy - 4.f * fy + 1.f);
        const float wz = 1.f - (4.f * fz * fz - 4.f * fz + 1.f);
        mom[1] += a[0] * wx + a[1] * wy + a[2] * wz;
        mom[2] += a[3] * wx + a[4] * wy + a[5] * wz;
        mom[3] += a[6] * wx + a[7] * wy + a[8] * wz;
    }
    /* InvertPhysicalMoments_LES_cf: rescale factor from the local eddy viscosity */
    float Sm[6];
    strain_rate<float>(mom, Sm);
    const float smag = strain_mag<float>(Sm);
    float tau_c = 1.f / r.omega_c;
    const float tau_f = 2.f * tau_c - 0.5f + 1.5f * smag * r.cs;
    const float omega_f = 1.f / tau_f;
    tau_c = tau_c + smag * r.cs;
    const float omega_c = 1.f / tau_c;
    const float SF = (r.lrfactor * omega_c * (1.f - omega_f)) / ((1.f - omega_c) * omega_f);
    float g[19];
    invert_scaled<float>(mom, SF, g);
#pragma unroll
    for (int q = 0; q < 19; ++q) Fmt<S>::st(f_f + pidx(F, q, unsigned(cf)), g[q], F.off[q]);
}

template <class S>
__global__ void k_interp_cf(const RefineParams r, const Level F, const float* __restrict__ mom_c,
                            const float* __restrict__ mom_prev, float theta, S* __restrict__ f_f,
                            const uint8_t* __restrict__ mask_f) {
    interp_cf_node<S>(r, F, mom_c, mom_prev, theta, f_f, mask_f, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

/* the coarse nodes strictly inside the patch that the restriction replaces:
 * x0 .. x0 + nxi - 1 and likewise in y and z */
struct FcBox {
    int x0, y0, z0, nxi, nyi, nzi;
};

/* InterpFC (LR7:2172-2348): coarse nodes strictly inside the patch (2-node
 * margin) are replaced by the restriction of their 8 fine children. */
template <class S>
__device__ __forceinline__ void interp_fc_node(const RefineParams& r, const Level& C, const Level& F,
                                               const S* __restrict__ f_f, S* __restrict__ f_c,
                                               const uint8_t* __restrict__ mask_c, const int x, const int y,
                                               const int z) {
    const long long cc = z * C.plane + (long long)y * C.pitch + x;
    const int t = mask_c[cc] & TYPE_MASK;
    if (t == WALL || t == BODY) return;
    const int L = r.lrlevel;
    const int xm = int(L * (x - r.lrx0)), ym = int(L * (y - r.lry0));
    int kl = int(L * (z - r.lrz0)), kh = kl + 1;
    const bool top = kh >= r.fnz;
    kl = kl >= r.fnz ? kl - r.fnz : kl;
    kh = kh >= r.fnz ? kh - r.fnz : kh;
    int k0 = kl, k1 = kh;
    if (top && r.quirk_fc_top_zflip) {
        /* the reference reads the top plane's corners upper plane first */
        k0 = kh;
        k1 = kl;
    }
    /* the children's mean moments and the second-order terms, one child at
     * a time */
    float sum[9], a[9];
#pragma unroll
    for (int m = 0; m < 9; ++m) sum[m] = a[m] = 0.f;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int kk = (c & 4) ? k1 : k0;
        const long long cf = kk * F.plane + (long long)(ym + ((c >> 1) & 1)) * F.pitch + (xm + (c & 1));
        float g[19], mc[9], Sc[6];
        load19<S>(F, f_f, cf, g);
        physical_moments<float>(g, mc);
#pragma unroll
        for (int m = 0; m < 9; ++m) sum[m] += mc[m];
        if (r.order == 2) {
            strain_rate<float>(mc, Sc);
            second_order_add(a, c, mc, Sc);
        }
    }
    float mom[9];
#pragma unroll
    for (int m = 0; m < 9; ++m) mom[m] = 0.125f * sum[m];
    if (r.order == 2) {
        second_order_scale(a);
        mom[1] += a[0] + a[1] + a[2];
        mom[2] += a[3] + a[4] + a[5];
        mom[3] += a[6] + a[7] + a[8];
    }
    /* InvertPhysicalMoments_LES_fc */
    float Sm[6];
    strain_rate<float>(mom, Sm);
    const float smag = strain_mag<float>(Sm);
    float tau_f = 1.f / r.omega_f;
    float tau_c = tau_f + 0.5f + 12.f * smag * r.cs;
    tau_c *= 0.5f;
    const float omega_c = 1.f / tau_c;
    tau_f = tau_f + smag * r.cs;
    const float omega_f = 1.f / tau_f;
    const float SF = (1.f - omega_c) * omega_f / (r.lrfactor * omega_c * (1.f - omega_f));
    float g[19];
    invert_scaled<float>(mom, SF, g);
#pragma unroll
    for (int q = 0; q < 19; ++q) Fmt<S>::st(f_c + pidx(C, q, unsigned(cc)), g[q], C.off[q]);
}

template <class S>
__global__ void k_interp_fc(const RefineParams r, const Level C, const Level F, const S* __restrict__ f_f,
                            S* __restrict__ f_c, const uint8_t* __restrict__ mask_c, const FcBox b) {
    const int xi = blockIdx.x * blockDim.x + threadIdx.x, yi = blockIdx.y * blockDim.y + threadIdx.y;
    if (xi >= b.nxi || yi >= b.nyi) return;
    interp_fc_node<S>(r, C, F, f_f, f_c, mask_c, b.x0 + xi, b.y0 + yi, b.z0 + int(blockIdx.z));
}

/* the final band fill of a coarse step and the restriction in one launch:
 * they touch disjoint nodes (the band, and the coarse nodes over the
 * patch's interior with its 2-node margin), so the first cf_blocks blocks
 * fill the band and the others restrict, one coarse node per thread */
constexpr int IFACE_THREADS = 128;
template <class S>
__global__ void __launch_bounds__(IFACE_THREADS) k_interface(const RefineParams r, const Level C, const Level F,
                                                             const float* __restrict__ mom_c, S* __restrict__ f_f,
                                                             const uint8_t* __restrict__ mask_f, S* __restrict__ f_c,
                                                             const uint8_t* __restrict__ mask_c, const FcBox b,
                                                             int cf_blocks) {
    if (int(blockIdx.x) < cf_blocks) {
        interp_cf_node<S>(r, F, mom_c, nullptr, 1.f, f_f, mask_f,
                          (long long)blockIdx.x * IFACE_THREADS + threadIdx.x);
        return;
    }
    const long long i = (long long)(blockIdx.x - cf_blocks) * IFACE_THREADS + threadIdx.x;
    const long long per_plane = (long long)b.nxi * b.nyi;
    if (i >= per_plane * b.nzi) return;
    const int zi = int(i / per_plane), rem = int(i - zi * per_plane);
    interp_fc_node<S>(r, C, F, f_f, f_c, mask_c, b.x0 + rem % b.nxi, b.y0 + rem / b.nxi, b.z0 + zi);
}

/* ---- launchers ---- */

#define LBM_DISPATCH(storage, KERNEL_CALL)                   \
    switch (storage) {                                        \
        case STORE_F32: { using S = float; KERNEL_CALL; } break;            \
        case STORE_F16: { using S = __half; KERNEL_CALL; } break;           \
        case STORE_BF16: { using S = __nv_bfloat16; KERNEL_CALL; } break;   \
        case STORE_F64: { using S = double; KERNEL_CALL; } break;           \
        default: return cudaErrorInvalidValue;                \
    }

/* ---- the tensor-memory lane: one stream and two events per device,
 * created on first use and kept for the life of the process */
namespace {
constexpr int LANE_DEVICES = 64;
std::mutex g_lane_mu[LANE_DEVICES];
cudaStream_t g_lane[LANE_DEVICES] = {};
cudaEvent_t g_lane_in[LANE_DEVICES] = {}, g_lane_out[LANE_DEVICES] = {};
}  // namespace

TmemLane::TmemLane(cudaStream_t caller) : caller_(caller) {
    if ((err_ = cudaGetDevice(&dev_)) != cudaSuccess) return;
    if (dev_ < 0 || dev_ >= LANE_DEVICES) {
        err_ = cudaErrorInvalidDevice;
        dev_ = -1;
        return;
    }
    g_lane_mu[dev_].lock();
    if (!g_lane[dev_]) {
        if ((err_ = cudaStreamCreateWithFlags(&g_lane[dev_], cudaStreamNonBlocking)) != cudaSuccess ||
            (err_ = cudaEventCreateWithFlags(&g_lane_in[dev_], cudaEventDisableTiming)) != cudaSuccess ||
            (err_ = cudaEventCreateWithFlags(&g_lane_out[dev_], cudaEventDisableTiming)) != cudaSuccess)
            return;
    }
    lane_ = g_lane[dev_];
    done_ = g_lane_out[dev_];
    if ((err_ = cudaEventRecord(g_lane_in[dev_], caller_)) == cudaSuccess)
        err_ = cudaStreamWaitEvent(lane_, g_lane_in[dev_], 0);
}

cudaError_t TmemLane::prepare() {
    TmemLane lane(nullptr);
    return lane.status();
}

TmemLane::~TmemLane() {
    if (dev_ < 0) return;
    if (lane_ && cudaEventRecord(done_, lane_) == cudaSuccess) cudaStreamWaitEvent(caller_, done_, 0);
    g_lane_mu[dev_].unlock();
}

cudaError_t launch_stream_collide(const Level& L, const StepParams& p, const void* fA, void* fB, const uint8_t* mask,
                                  float* stats, float* mom_export, cudaStream_t s, const uint32_t* links) {
    if (p.halfway && !links) return cudaErrorInvalidValue;
    StepParams q = p;
    q.tau0 = 1.f / p.omega;
    q.smag_k = 18.f * 1.41421356f * p.cs;
    if (L.blocked) return launch_sc_blocked(L, q, fA, fB, mask, stats, mom_export, s, links);
    return launch_sc_layout<0>(L, q, fA, fB, mask, stats, mom_export, s, links);
}

cudaError_t launch_stream_collide_mlp(const Level& L, const StepParams& p, const void* fA, void* fB,
                                      const uint8_t* mask, float* stats, const uint32_t* links, const void* blob,
                                      int* err, cudaStream_t s) {
    if ((p.halfway && !links) || !blob || !err || p.has_lid || p.has_xbc || p.pull_clamp || p.exp_nx > 0)
        return cudaErrorInvalidValue;
    TmemLane lane(s);
    if (lane.status() != cudaSuccess) return lane.status();
    if (L.blocked) return launch_sc_mlp_blocked(L, p, fA, fB, mask, stats, links, blob, err, lane.stream());
    return launch_sc_mlp_layout<0>(L, p, fA, fB, mask, stats, links, blob, err, lane.stream());
}

cudaError_t launch_dyn_control(const Level& L, const void* f, int y1, float umax, float kp, float dpdy0_abs,
                               float* dpdy_dev, float* hist3, int t, cudaStream_t s) {
    if (y1 < 0 || y1 >= L.ny) return cudaErrorInvalidValue;
    LBM_DISPATCH(L.storage, (k_dyn_control<S><<<1, 256, 0, s>>>(L, (const S*)f, y1, umax, kp, dpdy0_abs, dpdy_dev,
                                                                  hist3, t)));
    return cudaGetLastError();
}

int force_partials() { return FORCE_BLOCKS; }

cudaError_t launch_force(const Level& L, const void* fA, const unsigned* body, int nbody, double* partials,
                         unsigned* done, double* out3, cudaStream_t s, const uint8_t* mask, int halfway) {
    if (nbody <= 0) return cudaSuccess;
    LBM_DISPATCH(L.storage, (k_force_list<S><<<FORCE_BLOCKS, FORCE_THREADS, 0, s>>>(L, (const S*)fA, body, nbody,
                                                                                    partials, done, out3, mask,
                                                                                    halfway)));
    return cudaGetLastError();
}

/* momentum exchange by scanning the mask (the kernel-level API has no body
 * list): grid-stride over rows, FP64 per-block partials, fixed-order sum */
constexpr int SCAN_BLOCKS = 1216; /* 8 blocks per SM on a 152-SM GB300 */
template <class S>
__global__ void __launch_bounds__(256) k_force_scan(const Level L, const S* __restrict__ fA,
                                                    const uint8_t* __restrict__ mask, double* __restrict__ part) {
    using F = Fmt<S>;
    double s[3] = {0.0, 0.0, 0.0};
    const long long rows = (long long)L.ny * L.nz;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (long long r = (long long)blockIdx.x * 8 + warp; r < rows; r += (long long)gridDim.x * 8) {
        const int y = int(r % L.ny), z = int(r / L.ny);
        for (int x = lane; x < L.nx; x += 32) {
            if ((mask[z * L.plane + (long long)y * L.pitch + x] & TYPE_MASK) != BODY) continue;
            const int xm = (x == 0) ? L.nx - 1 : x - 1, xp = (x == L.nx - 1) ? 0 : x + 1;
            const int ym = (y == 0) ? L.ny - 1 : y - 1, yp = (y == L.ny - 1) ? 0 : y + 1;
            const int zm = (z == 0) ? L.nz - 1 : z - 1, zp = (z == L.nz - 1) ? 0 : z + 1;
            const long long zb[3] = {zm * L.plane, z * L.plane, zp * L.plane};
            const long long yb[3] = {(long long)ym * L.pitch, (long long)y * L.pitch, (long long)yp * L.pitch};
            const int xs[3] = {xm, x, xp};
            /* per node in the storage's arithmetic (as k_force_list), across nodes FP64 */
            typename F::T a[3] = {0, 0, 0};
#pragma unroll
            for (int q = 1; q < 19; ++q) {
                const typename F::T v = typename F::T(2) *
                    F::ld(fA + pidx(L, q, unsigned(zb[1 - cz(q)] + yb[1 - cy(q)] + xs[1 - cx(q)])), L.off[q]);
                if (cx(q)) a[0] += cx(q) * v;
                if (cy(q)) a[1] += cy(q) * v;
                if (cz(q)) a[2] += cz(q) * v;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) s[k] += double(a[k]);
        }
    }
    __shared__ double red[3][8];
    for (int k = 0; k < 3; ++k) {
        double v = s[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double v = 0.0;
#pragma unroll
        for (int w = 0; w < 8; ++w) v += red[threadIdx.x][w];
        part[3 * blockIdx.x + threadIdx.x] = v;
    }
}

int force_scan_partials() { return SCAN_BLOCKS; }

cudaError_t launch_force_scan(const Level& L, const void* fA, const uint8_t* mask, double* partials, double* out3,
                              cudaStream_t s) {
    LBM_DISPATCH(L.storage, (k_force_scan<S><<<SCAN_BLOCKS, 256, 0, s>>>(L, (const S*)fA, mask, partials)));
    k_reduce3<<<1, 1024, 0, s>>>(partials, SCAN_BLOCKS, out3);
    return cudaGetLastError();
}

cudaError_t launch_init(const Level& L, const uint8_t* mask, void* f, int kind, float u0, cudaStream_t s, int axis) {
    const dim3 block(SC_BX, SC_BY), grid = sc_grid(L);
    LBM_DISPATCH(L.storage, (k_init<S><<<grid, block, 0, s>>>(L, mask, (S*)f, kind, u0, axis)));
    return cudaGetLastError();
}

cudaError_t launch_fields(const Level& L, const void* f, float* rho, float* u, float* v, float* w, cudaStream_t s) {
    const dim3 block(SC_BX, SC_BY), grid = sc_grid(L);
    LBM_DISPATCH(L.storage, (k_fields<S><<<grid, block, 0, s>>>(L, (const S*)f, rho, u, v, w)));
    return cudaGetLastError();
}

cudaError_t launch_pack(const Level& L, const void* f, float* compact, cudaStream_t s) {
    const dim3 block(SC_BX, SC_BY), grid = sc_grid(L);
    LBM_DISPATCH(L.storage, (k_pack<S><<<grid, block, 0, s>>>(L, (const S*)f, compact)));
    return cudaGetLastError();
}

cudaError_t launch_unpack(const Level& L, const float* compact, void* f, cudaStream_t s) {
    const dim3 block(SC_BX, SC_BY), grid = sc_grid(L);
    LBM_DISPATCH(L.storage, (k_unpack<S><<<grid, block, 0, s>>>(L, compact, (S*)f)));
    return cudaGetLastError();
}

int audit_partials(const Level&) { return AUDIT_BLOCKS; }

cudaError_t launch_audit(const Level& L, const void* f, const uint8_t* mask, double* partials, int npart, double* out4,
                         cudaStream_t s) {
    if (npart < AUDIT_BLOCKS) return cudaErrorInvalidValue;
    LBM_DISPATCH(L.storage, (k_audit<S><<<AUDIT_BLOCKS, 256, 0, s>>>(L, (const S*)f, mask, partials)));
    k_audit_final<<<1, 256, 0, s>>>(partials, AUDIT_BLOCKS, out4);
    return cudaGetLastError();
}

cudaError_t launch_interp_cf(const RefineParams& r, const Level& F, const float* mom_c, void* f_f,
                             const uint8_t* mask_f, cudaStream_t s, const float* mom_prev, float theta) {
    const long long n = cf_nodes(r);
    const int threads = 128;
    const unsigned blocks = unsigned((n + threads - 1) / threads);
    LBM_DISPATCH(F.storage,
                 (k_interp_cf<S><<<blocks, threads, 0, s>>>(r, F, mom_c, mom_prev, theta, (S*)f_f, mask_f)));
    return cudaGetLastError();
}

/* the coarse nodes the restriction replaces: x with x > lrx0 + 1 and
 * x < lrx0 + fnx lrfactor - 2, the same in y, and in z every plane of a
 * full-depth patch or, for a bounded one, as in x and y */
static FcBox fc_box(const RefineParams& r, const Level& C) {
    int x0 = 0, x1 = -1, y0 = 0, y1 = -1;
    for (int x = 0; x < C.nx; ++x)
        if (x > r.lrx0 + 1 && x < r.lrx0 + r.fnx * r.lrfactor - 2) {
            if (x1 < x0) x0 = x;
            x1 = x;
        }
    for (int y = 0; y < C.ny; ++y)
        if (y > r.lry0 + 1 && y < r.lry0 + r.fny * r.lrfactor - 2) {
            if (y1 < y0) y0 = y;
            y1 = y;
        }
    int z0 = 0, z1 = C.nz - 1;
    if (r.zbounded) {
        z1 = -1;
        for (int z = 0; z < C.nz; ++z)
            if (z > r.lrz0 + 1 && z < r.lrz0 + r.fnz * r.lrfactor - 2) {
                if (z1 < z0) z0 = z;
                z1 = z;
            }
    }
    FcBox b{x0, y0, z0, x1 - x0 + 1, y1 - y0 + 1, z1 - z0 + 1};
    if (b.nxi <= 0 || b.nyi <= 0 || b.nzi <= 0) b.nxi = b.nyi = b.nzi = 0;
    return b;
}

cudaError_t launch_interp_fc(const RefineParams& r, const Level& C, const Level& F, const void* f_f, void* f_c,
                             const uint8_t* mask_c, cudaStream_t s) {
    const FcBox b = fc_box(r, C);
    if (b.nxi == 0) return cudaSuccess;
    const dim3 block(32, 4), grid((b.nxi + 31) / 32, (b.nyi + 3) / 4, b.nzi);
    LBM_DISPATCH(C.storage, (k_interp_fc<S><<<grid, block, 0, s>>>(r, C, F, (const S*)f_f, (S*)f_c, mask_c, b)));
    return cudaGetLastError();
}

cudaError_t launch_interface(const RefineParams& r, const Level& C, const Level& F, const float* mom_c, void* f_f,
                             const uint8_t* mask_f, void* f_c, const uint8_t* mask_c, cudaStream_t s) {
    if (C.storage != F.storage) return cudaErrorInvalidValue;
    const FcBox b = fc_box(r, C);
    const int cf_blocks = int((cf_nodes(r) + IFACE_THREADS - 1) / IFACE_THREADS);
    const long long nfc = (long long)b.nxi * b.nyi * b.nzi;
    const unsigned blocks = unsigned(cf_blocks + (nfc + IFACE_THREADS - 1) / IFACE_THREADS);
    LBM_DISPATCH(C.storage, (k_interface<S><<<blocks, IFACE_THREADS, 0, s>>>(r, C, F, mom_c, (S*)f_f, mask_f, (S*)f_c,
                                                                             mask_c, b, cf_blocks)));
    return cudaGetLastError();
}

}  // namespace lbm
