/* Ensemble kernels: many periodic D3Q19 boxes of uneven sizes advanced
 * together by one launch per step.
 *
 * Every member is a compact SoA level f[q][z][y][pitch] (pitch = n rounded up
 * to 32) inside one A and one B buffer; a block of 32 x TY threads updates a
 * 32 x TY tile of one z plane of one member.  The launch is persistent: a
 * grid sized by the autotuner walks the global tile list, so the per-member
 * work is balanced across the SMs whatever the mix of sizes, and a CUDA graph
 * of several steps replays the whole sequence with one host call.
 *
 * The collision is the LR7 MRT (LRTurbTest/LRMultiGPU7.cu:583-711) with
 *   SGS_NONE   molecular viscosity only (the 2x-resolution "truth" runs),
 *   SGS_SMAG   the constant-Cs Smagorinsky model of LR7:683-685,
 *   SGS_MLP    the learned closure: Pi_neq -> features -> tensor-core MLP ->
 *              nu_t -> tau_eff = tau0 + 3 nu_t.
 * Also: the random-phase turbulence initialisation, velocity and energy
 * read-outs, and the 2x2x2 box filter that turns fine members into training
 * samples for the closure.
 */
#include <cuda_runtime.h>

#include <type_traits>

#include "d3q19.cuh"
#include "ensemble.cuh"
#include "sgs_infer.cuh"

namespace lbm {
namespace ens {

__device__ __forceinline__ int find_member(const Table& T, int g) {
    int m = 0;
    while (m + 1 < T.count && g >= T.m[m + 1].tile0) ++m;
    return m;
}

template <int TY, int SGS>
__global__ void __launch_bounds__(32 * TY) k_ens_step(const Table T, const float* __restrict__ fA,
                                                      float* __restrict__ fB, const unsigned char* __restrict__ blob,
                                                      float cs, int* __restrict__ err) {
    constexpr int ROWS = 32 * TY;
    /* the MLP variant's operands live in dynamic shared memory (over 48 KB
     * for 256 rows), aligned up to 1 KB inside the allocation */
    extern __shared__ unsigned char dsm[];
    sgs::InferSmem<ROWS>& smem = *reinterpret_cast<sgs::InferSmem<ROWS>*>(
        (reinterpret_cast<uintptr_t>(dsm) + 1023) & ~uintptr_t(1023));
#if defined(__CUDA_ARCH__)
    if constexpr (SGS == SGS_MLP) sgs::infer_setup<ROWS>(smem, blob);
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int g = blockIdx.x; g < T.ntiles; g += gridDim.x) {
        const int mi = find_member(T, g);
        const Member& M = T.m[mi];
        const int local = g - M.tile0;
        const int per_z = M.tiles_x * M.tiles_y;
        const int z = local / per_z, r = local - z * per_z;
        const int y = (r / M.tiles_x) * TY + ty, x = (r % M.tiles_x) * 32 + tx;
        const int n = M.n;
        const bool live = x < n && y < n;
        const unsigned pitch = unsigned(M.pitch), plane = unsigned(n) * pitch, qs = plane * unsigned(n);
        const float* a = fA + M.off;
        float* b = fB + M.off;
        float f[19];
        unsigned c = 0;
        if (live) {
            c = unsigned(z) * plane + unsigned(y) * pitch + unsigned(x);
            const unsigned xs[3] = {unsigned(x == 0 ? n - 1 : x - 1), unsigned(x), unsigned(x == n - 1 ? 0 : x + 1)};
            const unsigned yb[3] = {(y == 0 ? n - 1 : y - 1) * pitch, y * pitch, (y == n - 1 ? 0 : y + 1) * pitch};
            const unsigned zb[3] = {(z == 0 ? n - 1 : z - 1) * plane, z * plane, (z == n - 1 ? 0 : z + 1) * plane};
#pragma unroll
            for (int q = 0; q < 19; ++q)
                f[q] = __ldg(a + q * qs + zb[1 - cz(q)] + yb[1 - cy(q)] + xs[1 - cx(q)]);
        } else {
#pragma unroll
            for (int q = 0; q < 19; ++q) f[q] = wq(q);
        }
        float omega = M.omega;
        if constexpr (SGS == SGS_MLP) {
            float rho, p6[6], xf[sgs::NIN];
            pi_neq<float>(f, rho, p6);
            const float s = -1.5f / rho;
#pragma unroll
            for (int k = 0; k < 6; ++k) p6[k] *= s;
            sgs::features_fast(p6, M.tau0, M.omega, xf); /* omega = 1 / tau0 */
            const float o = sgs::infer_nu<ROWS>(smem, xf, err);
            if (o < 0.f) break; /* a tensor-core wait ran out (block-uniform) */
            omega = 1.f / (M.tau0 + 3.f * o * sgs::strain_gain(xf, M.omega));
        }
        collide_mrt<MRT>(f, omega, SGS == SGS_SMAG, cs, 0.f);
        if (live) {
#pragma unroll
            for (int q = 0; q < 19; ++q) b[q * qs + c] = f[q];
        }
    }
    if constexpr (SGS == SGS_MLP) sgs::infer_teardown<ROWS>(smem);
#endif
}

/* random-phase solenoidal field: u = sum_m a_m e_m cos(2 pi k_m.x / n + phi_m);
 * the equilibrium at rho = 1 and u into both buffers */
__global__ void k_ens_init(const Table T, const Mode* __restrict__ modes, float* __restrict__ fA,
                           float* __restrict__ fB, float* __restrict__ u_out) {
    const int g = blockIdx.x;
    if (g >= T.ntiles) return;
    const int mi = find_member(T, g);
    const Member& M = T.m[mi];
    const int local = g - M.tile0, per_z = M.tiles_x * M.tiles_y;
    const int z = local / per_z, r = local - z * per_z;
    const int y = (r / M.tiles_x) * T.ty + (threadIdx.x >> 5), x = (r % M.tiles_x) * 32 + (threadIdx.x & 31);
    const int n = M.n;
    if (x >= n || y >= n) return;
    double u[3] = {0, 0, 0};
    for (int k = M.mode0; k < M.mode0 + M.nmodes; ++k) {
        const Mode md = modes[k];
        long long ph = (long long)md.k[0] * x + (long long)md.k[1] * y + (long long)md.k[2] * z;
        ph %= n;
        if (ph < 0) ph += n;
        const double c = cospi(2.0 * double(ph) / n + md.phase);
        u[0] += md.a[0] * c;
        u[1] += md.a[1] * c;
        u[2] += md.a[2] * c;
    }
    const unsigned pitch = unsigned(M.pitch), plane = unsigned(n) * pitch, qs = plane * unsigned(n);
    const unsigned c = unsigned(z) * plane + unsigned(y) * pitch + unsigned(x);
    const float ux = float(u[0]), uy = float(u[1]), uz = float(u[2]);
    const float usq = ux * ux + uy * uy + uz * uz;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const float cu = float(cx(q)) * ux + float(cy(q)) * uy + float(cz(q)) * uz;
        const float fe = wq(q) * (1.f + 3.f * cu + 4.5f * cu * cu - 1.5f * usq);
        fA[M.off + q * qs + c] = fe;
        fB[M.off + q * qs + c] = fe;
    }
    if (u_out) {
        const size_t o = M.uoff + (size_t(z) * n + y) * n + x, nn = size_t(n) * n * n;
        u_out[o] = ux;
        u_out[o + nn] = uy;
        u_out[o + 2 * nn] = uz;
    }
}

/* equilibrium at rho = 1 and the given velocity field (compact, per member
 * at Member::uoff) */
__global__ void k_ens_init_from(const Table T, const float* __restrict__ u, float* __restrict__ fA,
                                float* __restrict__ fB) {
    const int g = blockIdx.x;
    if (g >= T.ntiles) return;
    const int mi = find_member(T, g);
    const Member& M = T.m[mi];
    const int local = g - M.tile0, per_z = M.tiles_x * M.tiles_y;
    const int z = local / per_z, r = local - z * per_z;
    const int y = (r / M.tiles_x) * T.ty + (threadIdx.x >> 5), x = (r % M.tiles_x) * 32 + (threadIdx.x & 31);
    const int n = M.n;
    if (x >= n || y >= n) return;
    const size_t o = M.uoff + (size_t(z) * n + y) * n + x, nn = size_t(n) * n * n;
    const float ux = u[o], uy = u[o + nn], uz = u[o + 2 * nn];
    const unsigned pitch = unsigned(M.pitch), plane = unsigned(n) * pitch, qs = plane * unsigned(n);
    const unsigned c = unsigned(z) * plane + unsigned(y) * pitch + unsigned(x);
    const float usq = ux * ux + uy * uy + uz * uz;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const float cu = float(cx(q)) * ux + float(cy(q)) * uy + float(cz(q)) * uz;
        const float fe = wq(q) * (1.f + 3.f * cu + 4.5f * cu * cu - 1.5f * usq);
        fA[M.off + q * qs + c] = fe;
        fB[M.off + q * qs + c] = fe;
    }
}

/* velocity j / rho of every member into the compact buffer at Member::uoff */
__global__ void k_ens_velocity(const Table T, const float* __restrict__ f, float* __restrict__ u) {
    const int g = blockIdx.x;
    if (g >= T.ntiles) return;
    const int mi = find_member(T, g);
    const Member& M = T.m[mi];
    const int local = g - M.tile0, per_z = M.tiles_x * M.tiles_y;
    const int z = local / per_z, r = local - z * per_z;
    const int y = (r / M.tiles_x) * T.ty + (threadIdx.x >> 5), x = (r % M.tiles_x) * 32 + (threadIdx.x & 31);
    const int n = M.n;
    if (x >= n || y >= n) return;
    const unsigned pitch = unsigned(M.pitch), plane = unsigned(n) * pitch, qs = plane * unsigned(n);
    const unsigned c = unsigned(z) * plane + unsigned(y) * pitch + unsigned(x);
    float rho = 0, jx = 0, jy = 0, jz = 0;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const float v = f[M.off + q * qs + c];
        rho += v;
        if (cx(q)) jx += float(cx(q)) * v;
        if (cy(q)) jy += float(cy(q)) * v;
        if (cz(q)) jz += float(cz(q)) * v;
    }
    const size_t o = M.uoff + (size_t(z) * n + y) * n + x, nn = size_t(n) * n * n;
    u[o] = jx / rho;
    u[o + nn] = jy / rho;
    u[o + 2 * nn] = jz / rho;
}

/* per-member kinetic energy 1/2 <|u|^2> over the nodes, FP64, from the
 * compact velocities: one block per member, fixed order */
__global__ void k_ens_energy(const Table T, const float* __restrict__ u, double* __restrict__ out) {
    const int mi = blockIdx.x;
    if (mi >= T.count) return;
    const Member& M = T.m[mi];
    const size_t nn = size_t(M.n) * M.n * M.n;
    double s = 0;
    for (size_t i = threadIdx.x; i < nn; i += blockDim.x) {
        const double a = u[M.uoff + i], b = u[M.uoff + nn + i], c = u[M.uoff + 2 * nn + i];
        s += a * a + b * b + c * c;
    }
    __shared__ double red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (int(threadIdx.x) < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[mi] = 0.5 * red[0] / double(nn);
}

/* 2x2x2 box filter of one fine member's velocity (compact [3][n][n][n]) onto
 * the coarse grid: ubar[3][nc^3], uu[6][nc^3] (xx, yy, zz, xy, xz, yz) */
__global__ void k_box_filter(const float* __restrict__ u, int n, double* __restrict__ ubar, double* __restrict__ uu) {
    const int nc = n / 2;
    const size_t cn = size_t(nc) * nc * nc, fn = size_t(n) * n * n;
    const size_t o = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (o >= cn) return;
    const int x = int(o % nc), y = int((o / nc) % nc), z = int(o / (size_t(nc) * nc));
    double s[3] = {0, 0, 0}, p[6] = {0, 0, 0, 0, 0, 0};
    for (int c = 0; c < 8; ++c) {
        const size_t i = (size_t(2 * z + (c >> 2)) * n + 2 * y + ((c >> 1) & 1)) * n + 2 * x + (c & 1);
        const double a = u[i], b = u[fn + i], d = u[2 * fn + i];
        s[0] += a, s[1] += b, s[2] += d;
        p[0] += a * a, p[1] += b * b, p[2] += d * d, p[3] += a * b, p[4] += a * d, p[5] += b * d;
    }
    for (int k = 0; k < 3; ++k) ubar[k * cn + o] = s[k] / 8;
    for (int k = 0; k < 6; ++k) uu[k * cn + o] = p[k] / 8;
}

/* training samples of the filtered member, pass 1 per coarse cell: the
 * filtered strain S (central differences, periodic) and the two
 * contractions of the least-squares eddy viscosity, tau^d : S and S : S,
 * with tau = uu - ubar ubar the filtered subgrid stress */
__global__ void k_sgs_contract(const double* __restrict__ ubar, const double* __restrict__ uu, int nc,
                               double* __restrict__ s8) {
    const size_t cn = size_t(nc) * nc * nc;
    const size_t o = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (o >= cn) return;
    const int x = int(o % nc), y = int((o / nc) % nc), z = int(o / (size_t(nc) * nc));
    auto at = [&](int k, int xx, int yy, int zz) {
        xx = (xx + nc) % nc, yy = (yy + nc) % nc, zz = (zz + nc) % nc;
        return ubar[k * cn + (size_t(zz) * nc + yy) * nc + xx];
    };
    double g[3][3];
    for (int k = 0; k < 3; ++k) {
        g[k][0] = 0.5 * (at(k, x + 1, y, z) - at(k, x - 1, y, z));
        g[k][1] = 0.5 * (at(k, x, y + 1, z) - at(k, x, y - 1, z));
        g[k][2] = 0.5 * (at(k, x, y, z + 1) - at(k, x, y, z - 1));
    }
    const double S[6] = {g[0][0], g[1][1], g[2][2], 0.5 * (g[0][1] + g[1][0]), 0.5 * (g[0][2] + g[2][0]),
                         0.5 * (g[1][2] + g[2][1])};
    const double u0 = ubar[o], u1 = ubar[cn + o], u2 = ubar[2 * cn + o];
    double tau[6] = {uu[o] - u0 * u0,          uu[cn + o] - u1 * u1,     uu[2 * cn + o] - u2 * u2,
                     uu[3 * cn + o] - u0 * u1, uu[4 * cn + o] - u0 * u2, uu[5 * cn + o] - u1 * u2};
    const double tr = (tau[0] + tau[1] + tau[2]) / 3;
    for (int k = 0; k < 3; ++k) tau[k] -= tr;
    double ts = 0, ss = 0;
    for (int k = 0; k < 6; ++k) {
        const double w = k < 3 ? 1 : 2;
        ts += w * tau[k] * S[k];
        ss += w * S[k] * S[k];
    }
    for (int k = 0; k < 6; ++k) s8[k * cn + o] = S[k];
    s8[6 * cn + o] = ts;
    s8[7 * cn + o] = ss;
}

/* pass 2: nu = max(0, -<tau^d:S> / (2 <S:S>)) with <> the 3x3x3 box average
 * (periodic), the features of p = (tau0 + 3 nu) S, and the target nu */
__global__ void k_sgs_targets(const double* __restrict__ s8, int nc, double tau0, float* __restrict__ X,
                              float* __restrict__ T) {
    const size_t cn = size_t(nc) * nc * nc;
    const size_t o = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (o >= cn) return;
    const int x = int(o % nc), y = int((o / nc) % nc), z = int(o / (size_t(nc) * nc));
    double ts = 0, ss = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const size_t i = (size_t((z + dz + nc) % nc) * nc + (y + dy + nc) % nc) * nc + (x + dx + nc) % nc;
                ts += s8[6 * cn + i];
                ss += s8[7 * cn + i];
            }
    double nu = ss > 1e-30 ? -ts / (2 * ss) : 0;
    if (nu < 0) nu = 0;
    double p[6], xf[sgs::NIN];
    for (int k = 0; k < 6; ++k) p[k] = (tau0 + 3 * nu) * s8[k * cn + o];
    sgs::features<double>(p, tau0, xf);
    for (int k = 0; k < sgs::NIN; ++k) X[o * sgs::NIN + k] = float(xf[k]);
    T[o] = float(nu);
}

__global__ void k_d2f(const double* __restrict__ a, float* __restrict__ b, size_t n) {
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i < n) b[i] = float(a[i]);
}

}  // namespace ens

/* ---- launchers */
template <int TY, int SGS> static size_t step_smem() {
    return SGS == ens::SGS_MLP ? sgs::infer_dyn_smem<32 * TY>() : 0;
}

template <int TY, int SGS> static cudaError_t step_attr() {
    static cudaError_t done = cudaErrorNotReady;
    if (done == cudaErrorNotReady)
        done = cudaFuncSetAttribute(ens::k_ens_step<TY, SGS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    int(step_smem<TY, SGS>()));
    return done;
}

template <int TY, int SGS> static cudaError_t step_t(const ens::Table& T, const float* fA, float* fB,
                                                    const void* blob, float cs, int* err, int grid, cudaStream_t s) {
    if (cudaError_t e = step_attr<TY, SGS>()) return e;
    if (SGS == ens::SGS_MLP) {
        TmemLane lane(s);
        if (lane.status() != cudaSuccess) return lane.status();
        ens::k_ens_step<TY, SGS><<<grid, 32 * TY, step_smem<TY, SGS>(), lane.stream()>>>(
            T, fA, fB, (const unsigned char*)blob, cs, err);
        return cudaGetLastError();
    }
    ens::k_ens_step<TY, SGS><<<grid, 32 * TY, step_smem<TY, SGS>(), s>>>(T, fA, fB, (const unsigned char*)blob, cs,
                                                                         err);
    return cudaGetLastError();
}

cudaError_t launch_ens_step(const ens::Table& T, const float* fA, float* fB, int sgs, const void* blob, float cs,
                            int* err, int grid, cudaStream_t s) {
    if (T.ty == 4) {
        if (sgs == ens::SGS_NONE) return step_t<4, ens::SGS_NONE>(T, fA, fB, blob, cs, err, grid, s);
        if (sgs == ens::SGS_SMAG) return step_t<4, ens::SGS_SMAG>(T, fA, fB, blob, cs, err, grid, s);
        return step_t<4, ens::SGS_MLP>(T, fA, fB, blob, cs, err, grid, s);
    }
    if (T.ty == 8) {
        if (sgs == ens::SGS_NONE) return step_t<8, ens::SGS_NONE>(T, fA, fB, blob, cs, err, grid, s);
        if (sgs == ens::SGS_SMAG) return step_t<8, ens::SGS_SMAG>(T, fA, fB, blob, cs, err, grid, s);
        return step_t<8, ens::SGS_MLP>(T, fA, fB, blob, cs, err, grid, s);
    }
    return cudaErrorInvalidValue;
}

int ens_step_occupancy(int ty, int sgs) {
    int nb = 0;
    cudaError_t e = cudaSuccess;
    if (ty == 4) {
        if (sgs == ens::SGS_NONE)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, ens::k_ens_step<4, ens::SGS_NONE>, 128, 0);
        else if (sgs == ens::SGS_SMAG)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, ens::k_ens_step<4, ens::SGS_SMAG>, 128, 0);
        else if ((e = step_attr<4, ens::SGS_MLP>()) == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, ens::k_ens_step<4, ens::SGS_MLP>, 128,
                                                              step_smem<4, ens::SGS_MLP>());
    } else {
        if (sgs == ens::SGS_NONE)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, ens::k_ens_step<8, ens::SGS_NONE>, 256, 0);
        else if (sgs == ens::SGS_SMAG)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, ens::k_ens_step<8, ens::SGS_SMAG>, 256, 0);
        else if ((e = step_attr<8, ens::SGS_MLP>()) == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, ens::k_ens_step<8, ens::SGS_MLP>, 256,
                                                              step_smem<8, ens::SGS_MLP>());
    }
    if (e != cudaSuccess) return 1;
    return nb < 1 ? 1 : nb;
}

cudaError_t launch_ens_init(const ens::Table& T, const ens::Mode* modes, float* fA, float* fB, float* u_out,
                            cudaStream_t s) {
    ens::k_ens_init<<<T.ntiles, 32 * T.ty, 0, s>>>(T, modes, fA, fB, u_out);
    return cudaGetLastError();
}
cudaError_t launch_ens_init_from(const ens::Table& T, const float* u, float* fA, float* fB, cudaStream_t s) {
    ens::k_ens_init_from<<<T.ntiles, 32 * T.ty, 0, s>>>(T, u, fA, fB);
    return cudaGetLastError();
}
cudaError_t launch_ens_velocity(const ens::Table& T, const float* f, float* u, cudaStream_t s) {
    ens::k_ens_velocity<<<T.ntiles, 32 * T.ty, 0, s>>>(T, f, u);
    return cudaGetLastError();
}
cudaError_t launch_ens_energy(const ens::Table& T, const float* u, double* out, cudaStream_t s) {
    ens::k_ens_energy<<<T.count, 256, 0, s>>>(T, u, out);
    return cudaGetLastError();
}
cudaError_t launch_box_filter(const float* u, int n, double* ubar, double* uu, cudaStream_t s) {
    const size_t cn = size_t(n / 2) * (n / 2) * (n / 2);
    ens::k_box_filter<<<unsigned((cn + 255) / 256), 256, 0, s>>>(u, n, ubar, uu);
    return cudaGetLastError();
}
cudaError_t launch_d2f(const double* a, float* b, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ens::k_d2f<<<unsigned((n + 255) / 256), 256, 0, s>>>(a, b, n);
    return cudaGetLastError();
}
cudaError_t launch_sgs_targets(const double* ubar, const double* uu, int nc, double tau0, double* s8, float* X,
                               float* T, cudaStream_t s) {
    const size_t cn = size_t(nc) * nc * nc;
    const unsigned nb = unsigned((cn + 255) / 256);
    ens::k_sgs_contract<<<nb, 256, 0, s>>>(ubar, uu, nc, s8);
    ens::k_sgs_targets<<<nb, 256, 0, s>>>(s8, nc, tau0, X, T);
    return cudaGetLastError();
}

}  // namespace lbm
