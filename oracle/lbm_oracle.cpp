/*
 * lbm_oracle.cpp -- CPU restatement of the reference's D3Q19 hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see lbm_oracle.h).  Every function names the
 * reference lines it restates.  Arithmetic is FP32 like the reference (a
 * double-precision twin exists for the FP64 error audits); the moment basis and
 * its inverse are built from the basis table (the inverse of an orthogonal basis
 * is its transpose scaled by the row norms), which is the same linear map the
 * reference spells out term by term in LR7:393-419.
 *
 * Built with -ffp-contract=off so x86 and aarch64 hosts give identical results.
 */
#include "lbm_oracle.h"

#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {



constexpr int Q = 19;
constexpr int CX[Q] = {0, 1, 0, -1, 0, 1, -1, -1, 1, 0, 1, 0, -1, 0, 0, 1, 0, -1, 0};
constexpr int CY[Q] = {0, 0, 1, 0, -1, 1, 1, -1, -1, 0, 0, 1, 0, -1, 0, 0, 1, 0, -1};
constexpr int CZ[Q] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, -1, -1, -1, -1, -1};
constexpr int OPP[Q] = {0, 3, 4, 1, 2, 7, 8, 5, 6, 14, 17, 18, 15, 16, 9, 12, 13, 10, 11};

/* The reference's 19x19 moment basis, one row per moment (LR7:258-279).  Each
 * row is a polynomial in the lattice velocity c; writing the polynomial keeps
 * the table readable and makes it the same integers row for row. */
struct Basis {
    int M[Q][Q];
    double norm2[Q];
    Basis() {
        for (int q = 0; q < Q; ++q) {
            int cx = CX[q], cy = CY[q], cz = CZ[q];
            int c2 = cx * cx + cy * cy + cz * cz;
            M[0][q] = 1;
            M[1][q] = 19 * c2 - 30;
            M[2][q] = (21 * c2 * c2 - 53 * c2 + 24) / 2;
            M[3][q] = cx;
            M[4][q] = (5 * c2 - 9) * cx;
            M[5][q] = cy;
            M[6][q] = (5 * c2 - 9) * cy;
            M[7][q] = cz;
            M[8][q] = (5 * c2 - 9) * cz;
            M[9][q] = 3 * cx * cx - c2;
            M[10][q] = (3 * c2 - 5) * (3 * cx * cx - c2);
            M[11][q] = cy * cy - cz * cz;
            M[12][q] = (3 * c2 - 5) * (cy * cy - cz * cz);
            M[13][q] = cx * cy;
            M[14][q] = cy * cz;
            M[15][q] = cx * cz;
            M[16][q] = (cy * cy - cz * cz) * cx;
            M[17][q] = (cz * cz - cx * cx) * cy;
            M[18][q] = (cx * cx - cy * cy) * cz;
        }
        for (int k = 0; k < Q; ++k) {
            double s = 0;
            for (int q = 0; q < Q; ++q) s += double(M[k][q]) * M[k][q];
            norm2[k] = s;
        }
    }
};
const Basis B;

template <class T> inline void moments(const T* f, T* m) {
    for (int k = 0; k < Q; ++k) {
        T s = 0;
        for (int q = 0; q < Q; ++q)
            if (B.M[k][q] != 0) s += T(B.M[k][q]) * f[q];
        m[k] = s;
    }
}

/* f = M^-1 m with M^-1 = M^T diag(1/|row|^2) (LR7:393-419 spells it out) */
template <class T> inline void invert(const T* m, T* f) {
    for (int q = 0; q < Q; ++q) {
        T s = 0;
        for (int k = 0; k < Q; ++k)
            if (B.M[k][q] != 0) s += T(double(B.M[k][q]) / B.norm2[k]) * m[k];
        f[q] = s;
    }
}

/* mrt_meq (LR7:332-348) with its meq2 = 7.53968254*|j|^2 */
template <class T> inline void meq_lr7(T* meq, T rho, T u, T v, T w) {
    for (int k = 0; k < Q; ++k) meq[k] = 0;
    T usq = u * u + v * v + w * w;
    meq[0] = rho;
    meq[1] = T(-11) * rho + T(19) * usq;
    meq[2] = T(7.53968254) * usq;
    meq[3] = u;
    meq[4] = T(-0.666666667) * u;
    meq[5] = v;
    meq[6] = T(-0.666666667) * v;
    meq[7] = w;
    meq[8] = T(-0.666666667) * w;
    meq[9] = T(2) * u * u - (v * v + w * w);
    meq[11] = v * v - w * w;
    meq[13] = u * v;
    meq[14] = v * w;
    meq[15] = u * w;
}

/* bgk_meq (MRTtest/DynInlet3.cu:347-366) */
template <class T> inline void meq_di3(T* meq, T rho, T u, T v, T w) {
    for (int k = 0; k < Q; ++k) meq[k] = 0;
    T usq = u * u + v * v + w * w;
    meq[0] = rho;
    meq[1] = T(-11) * rho + T(19) * usq;
    meq[2] = T(3) * rho - T(5.5) * usq;
    meq[3] = u;
    meq[4] = T(-0.666666667) * u;
    meq[5] = v;
    meq[6] = T(-0.666666667) * v;
    meq[7] = w;
    meq[8] = T(-0.666666667) * w;
    meq[9] = T(2) * u * u - (v * v + w * w);
    meq[10] = T(-0.5) * meq[9] * T(0.333333333333);
    meq[11] = v * v - w * w;
    meq[12] = T(-0.5) * meq[11];
    meq[13] = u * v;
    meq[14] = v * w;
    meq[15] = u * w;
}

template <class T> inline T wq(int q) {
    return q == 0 ? T(1) / T(3) : (q <= 4 || q == 9 || q == 14) ? T(1) / T(18) : T(1) / T(36);
}

/* incompressible BGK equilibrium used by the reference (DI3:806-827, CPU:135-153):
 * feq_q = w_q (rho + 3 c.u + 4.5 (c.u)^2 - 1.5 |u|^2) */
template <class T> inline T feq_bgk(int q, T rho, T u, T v, T w) {
    T cu = T(CX[q]) * u + T(CY[q]) * v + T(CZ[q]) * w;
    T usq = u * u + v * v + w * w;
    return wq<T>(q) * (rho + T(3) * cu + T(4.5) * cu * cu - T(1.5) * usq);
}

/* Smagorinsky tau_eff (LR7:672-685): Q = |Pi_neq|, Pi_neq = sum c c (f - feq).
 * For both reference equilibria Pi_neq = sum c c f - rho/3 I - j j. */
template <class T> inline T les_omega(const T* f, T omega, T cs) {
    T rho = 0, jx = 0, jy = 0, jz = 0, pxx = 0, pyy = 0, pzz = 0, pxy = 0, pyz = 0, pxz = 0;
    for (int q = 0; q < Q; ++q) {
        T cx = T(CX[q]), cy = T(CY[q]), cz = T(CZ[q]);
        rho += f[q];
        jx += cx * f[q];
        jy += cy * f[q];
        jz += cz * f[q];
        pxx += cx * cx * f[q];
        pyy += cy * cy * f[q];
        pzz += cz * cz * f[q];
        pxy += cx * cy * f[q];
        pyz += cy * cz * f[q];
        pxz += cx * cz * f[q];
    }
    T third = rho / T(3);
    T nxx = pxx - third - jx * jx, nyy = pyy - third - jy * jy, nzz = pzz - third - jz * jz;
    T nxy = pxy - jx * jy, nyz = pyz - jy * jz, nxz = pxz - jx * jz;
    T qn = std::sqrt(nxx * nxx + nyy * nyy + nzz * nzz + T(2) * nxy * nxy + T(2) * nyz * nyz +
                     T(2) * nxz * nxz);
    T tau0 = T(1) / omega;
    T tau = T(0.5) * tau0 + T(0.5) * std::sqrt(tau0 * tau0 + T(18) * cs * std::sqrt(T(2)) * qn);
    return T(1) / tau;
}

/* AddForce (DI3:229-252): constant dp/dy forcing on the y-moving populations */
template <class T> inline void add_force(T* f, T dpdy) {
    T a = T(0.0555555556) * T(3) * dpdy, b = T(0.0277777778) * T(3) * dpdy;
    f[2] -= a;
    f[4] += a;
    f[5] -= b;
    f[6] -= b;
    f[7] += b;
    f[8] += b;
    f[11] -= b;
    f[13] += b;
    f[16] -= b;
    f[18] += b;
}

/* LR7 mrt_collide (LR7:583-711): non-equilibrium moments relaxed at rate 1,
 * except the stress moments 9, 11, 13, 14, 15 which relax with omega (tau_eff
 * when LES is on). */
template <class T> inline void collide_mrt(T* f, T omega, int les, T cs, bool cpu3d = false) {
    if (les) omega = les_omega(f, omega, cs);
    T m[Q], meq[Q], n[Q];
    moments(f, m);
    meq_lr7(meq, m[0], m[3], m[5], m[7]);
    /* CPU_3D's mrt_collide: meq2 = -7.53968254 |j|^2 (CPU:222) and m13, m14
     * relaxed at rate 1 (CPU:246-248) */
    if (cpu3d) meq[2] = -meq[2];
    for (int k = 0; k < Q; ++k) n[k] = m[k] - meq[k];
    n[0] = n[3] = n[5] = n[7] = 0;
    n[9] *= omega;
    n[11] *= omega;
    if (!cpu3d) {
        n[13] *= omega;
        n[14] *= omega;
    }
    n[15] *= omega;
    T df[Q];
    invert(n, df);
    for (int q = 0; q < Q; ++q) f[q] -= df[q];
}

/* DynInlet3 MRT branch (DI3:770-789): moments relaxed to bgk_meq; the stress
 * moments with omega.  Followed by AddForce (DI3:830). */
template <class T> inline void collide_mrt_di3(T* f, T omega, int les, T cs, T dpdy) {
    if (les) omega = les_omega(f, omega, cs);
    T m[Q], meq[Q];
    moments(f, m);
    meq_di3(meq, m[0], m[3], m[5], m[7]);
    for (int k : {9, 11, 13, 14, 15}) meq[k] = m[k] - omega * (m[k] - meq[k]);
    invert(meq, f);
    add_force(f, dpdy);
}

/* BGK branch (DI3:806-830, CPU:116-162) */
template <class T> inline void collide_bgk(T* f, T omega, int les, T cs, T dpdy) {
    if (les) omega = les_omega(f, omega, cs);
    T rho = 0, u = 0, v = 0, w = 0;
    for (int q = 0; q < Q; ++q) {
        rho += f[q];
        u += T(CX[q]) * f[q];
        v += T(CY[q]) * f[q];
        w += T(CZ[q]) * f[q];
    }
    for (int q = 0; q < Q; ++q) f[q] -= omega * (f[q] - feq_bgk<T>(q, rho, u, v, w));
    add_force(f, dpdy);
}

template <class T> inline void collide(int model, T* f, T omega, int les, T cs, T dpdy) {
    if (model == ORC_MRT) collide_mrt(f, omega, les, cs);
    else if (model == ORC_MRT_CPU3D) collide_mrt(f, omega, les, cs, true);
    else if (model == ORC_MRT_DI3) collide_mrt_di3(f, omega, les, cs, dpdy);
    else collide_bgk(f, omega, les, cs, dpdy);
}

/* *_Extrap rebuilds (LR7:713-897): every moment of the neighbour's populations
 * is kept except density (outlets, density prescribed) or momentum (inlets,
 * momentum prescribed).  The linear map reduces to
 *   f_q += (rho_new - rho)/19 + (c_q . (j_new - j))/10. */
template <class T> inline void extrap(int kind, T* f, T rho_bc, T u_in) {
    T rho = 0, jx = 0, jy = 0, jz = 0;
    for (int q = 0; q < Q; ++q) {
        rho += f[q];
        jx += T(CX[q]) * f[q];
        jy += T(CY[q]) * f[q];
        jz += T(CZ[q]) * f[q];
    }
    T m[Q];
    moments(f, m);
    if (kind == ORC_EAST_OUTLET || kind == ORC_NORTH_OUTLET) {
        m[0] = rho_bc;
    } else if (kind == ORC_WEST_INLET) {
        m[3] = u_in;
        m[5] = 0;
        m[7] = 0;
    } else if (kind == ORC_SOUTH_INLET) {
        m[3] = 0;
        m[5] = u_in;
        m[7] = 0;
    }
    (void)jx;
    (void)jy;
    (void)jz;
    invert(m, f);
}

/* Regularised velocity (Dirichlet) boundary, the reference's
 * DirichletWest_Regularized (CPU:974-1054) written for any face: density from
 * the known populations, unknown populations by non-equilibrium bounce-back,
 * then f = feq + w_q 4.5 (c_q c_q - I/3) : Pi_neq. */
/* ---- alternate boundaries, restated from CPU_3D/CPU_3D.cpp:411-1140,
 * LRTurbTest/LRMultiGPU7.cu:899-1016 and BC1/LRMultiGPU7.cu:789-870 ---- */

/* the y/z edge assignments at a west face (CPU:417-470; LR7:901-945):
 * each entry {dst, src}; corners first, else the y edges */
template <class T> void alt_west_edges(T* f, int y, int z, int ny, int nz) {
    const bool y0 = y == 0, y1 = y == ny - 1, z0 = z == 0, z1 = z == nz - 1;
    if (y0 && z0) { f[2] = f[4]; f[13] = f[18]; f[11] = f[18]; f[16] = f[18]; f[6] = f[7]; f[9] = f[14]; f[12] = f[17]; }
    else if (y0 && z1) { f[4] = f[2]; f[11] = f[13]; f[18] = f[13]; f[16] = f[13]; f[6] = f[7]; f[14] = f[9]; f[17] = f[12]; }
    else if (y1 && z0) { f[4] = f[2]; f[11] = f[16]; f[18] = f[16]; f[13] = f[16]; f[7] = f[6]; f[9] = f[14]; f[12] = f[17]; }
    else if (y1 && z1) { f[4] = f[2]; f[16] = f[11]; f[18] = f[11]; f[13] = f[11]; f[7] = f[6]; f[14] = f[9]; f[17] = f[12]; }
    else if (y0) { f[2] = f[4]; f[11] = f[13]; f[16] = f[18]; f[8] = f[5]; }
    else if (y1) { f[4] = f[2]; f[13] = f[11]; f[18] = f[16]; f[5] = f[8]; }
}
/* at an east face (CPU:590-644; LR7:958-1006) */
template <class T> void alt_east_edges(T* f, int y, int z, int ny, int nz) {
    const bool y0 = y == 0, y1 = y == ny - 1, z0 = z == 0, z1 = z == nz - 1;
    if (y0 && z0) { f[2] = f[4]; f[13] = f[18]; f[11] = f[18]; f[16] = f[18]; f[5] = f[8]; f[9] = f[14]; f[10] = f[15]; }
    else if (y0 && z1) { f[2] = f[4]; f[11] = f[13]; f[18] = f[13]; f[16] = f[13]; f[5] = f[8]; f[14] = f[9]; f[15] = f[10]; }
    else if (y1 && z0) { f[4] = f[2]; f[18] = f[16]; f[11] = f[16]; f[13] = f[16]; f[8] = f[5]; f[9] = f[14]; f[10] = f[15]; }
    else if (y1 && z1) { f[4] = f[2]; f[13] = f[11]; f[16] = f[11]; f[18] = f[11]; f[8] = f[5]; f[14] = f[9]; f[15] = f[10]; }
    else if (y0) { f[2] = f[4]; f[11] = f[13]; f[16] = f[18]; f[5] = f[8]; }
    else if (y1) { f[4] = f[2]; f[13] = f[11]; f[18] = f[16]; f[8] = f[5]; }
}
/* the z edge copies of a non-corner west / east node (CPU:471-482, 633-644) */
template <class T> void alt_z_edges(T* f, int y, int z, int ny, int nz) {
    if ((y == 0 || y == ny - 1) && (z == 0 || z == nz - 1)) return;
    if (z == 0) { f[9] = f[14]; f[10] = f[15]; f[11] = f[16]; f[13] = f[18]; }
    else if (z == nz - 1) { f[14] = f[9]; f[15] = f[10]; f[16] = f[11]; f[18] = f[13]; }
}

template <class T> void alt_boundary(int type, T* f, int y, int z, int ny, int nz, T u, int t) {
    if (type == ORC_DIR_WEST) {
        alt_west_edges(f, y, z, ny, nz);
        alt_z_edges(f, y, z, ny, nz);
        /* CPU:484-488 with v = w = 0 */
        f[1] = std::fma(T(0.0555555556), T(6) * u, f[3]);
        f[5] = std::fma(T(0.0277777778), T(6) * u, f[7]);
        f[8] = std::fma(T(0.0277777778), T(6) * u, f[6]);
        f[10] = std::fma(T(0.0277777778), T(6) * u, f[17]);
        f[15] = std::fma(T(0.0277777778), T(6) * u, f[12]);
    } else if (type == ORC_NEU_EAST || type == ORC_NEU_EAST_REG) {
        if (type == ORC_NEU_EAST) {
            alt_east_edges(f, y, z, ny, nz);
            alt_z_edges(f, y, z, ny, nz);
        }
        const T rho = 1;
        const T ux = -rho + (f[0] + f[2] + f[4] + f[9] + f[11] + f[13] + f[14] + f[16] + f[18] +
                             T(2) * (f[1] + f[8] + f[5] + f[10] + f[15]));
        if (type == ORC_NEU_EAST) {
            /* CPU:651-655 with v = w = 0 */
            f[3] = f[1] - T(0.333333333) * ux;
            f[7] = f[5] - T(0.166666667) * ux;
            f[6] = f[8] - T(0.166666667) * ux;
            f[17] = f[10] - T(0.166666667) * ux;
            f[12] = f[15] - T(0.166666667) * ux;
        } else {
            /* CPU:1080-1137 as written */
            T fe[19];
            const T usq = ux * ux;
            for (int q = 0; q < 19; ++q) {
                const T cu = T(CX[q]) * ux;
                const T w = q == 0 ? T(0.3333333333) : (q <= 4 || q == 9 || q == 14) ? T(0.0555555556) : T(0.0277777778);
                fe[q] = q == 0 ? w * (rho - T(1.5) * usq) : w * (rho + T(3) * cu + T(4.5) * cu * cu - T(1.5) * usq);
            }
            f[3] = fe[1] + f[1] - fe[1];
            f[7] = fe[5] + f[5] - fe[5];
            f[6] = fe[6] + f[8] - fe[8];
            f[17] = fe[10] + f[10] - fe[10];
            f[12] = fe[15] + f[15] - fe[15];
            T d[19];
            for (int q = 0; q < 19; ++q) d[q] = f[q] - fe[q];
            const T P11 = d[1] + d[3] + d[5] + d[6] + d[7] + d[8] + d[10] + d[12] + d[15] + d[17];
            const T P22 = d[2] + d[4] + d[5] + d[6] + d[7] + d[8] + d[11] + d[13] + d[16] + d[18];
            const T P33 = d[9] + d[14] + d[10] + d[12] + d[15] + d[17] + d[11] + d[13] + d[16] + d[18];
            const T P12 = d[5] + d[7] - d[6] - d[8];
            const T P13 = d[10] + d[17] - d[12] - d[15];
            const T P23 = d[11] + d[18] - d[13] - d[16];
            const T A = T(0.666666667), B = T(-0.333333333);
            /* f_q = feq_q + w'_q (Q_q : Pi), Q_q = c c - I/3 scaled as CPU:1119-1137 */
            for (int q = 0; q < 19; ++q) {
                const int ax = CX[q] * CX[q], ay = CY[q] * CY[q], az = CZ[q] * CZ[q];
                const T pre = q == 0 ? T(1.5) : (q <= 4 || q == 9 || q == 14) ? T(0.25) : T(0.125);
                T s = (ax ? A : B) * P11;
                if (CX[q] * CY[q]) s = s + T(2) * (T(CX[q] * CY[q]) * P12);
                if (CX[q] * CZ[q]) s = s + T(2) * (T(CX[q] * CZ[q]) * P13);
                if (CY[q] * CZ[q]) s = s + T(2) * (T(CY[q] * CZ[q]) * P23);
                s = s + (ay ? A : B) * P22;
                s = s + (az ? A : B) * P33;
                f[q] = fe[q] + pre * s;
            }
        }
    } else if (type == ORC_XSYM_BOT) {
        alt_west_edges(f, y, z, ny, nz);
        f[1] = f[3]; f[5] = f[6]; f[8] = f[7]; f[10] = f[12]; f[15] = f[17];
    } else if (type == ORC_XSYM_TOP) {
        alt_east_edges(f, y, z, ny, nz);
        f[3] = f[1]; f[6] = f[5]; f[7] = f[8]; f[12] = f[10]; f[17] = f[15];
    } else if (type == ORC_YSYM_TOP || type == ORC_YSYM_BOT) {
        if (z == 0) { f[9] = f[14]; f[10] = f[15]; f[11] = f[16]; f[12] = f[17]; f[13] = f[18]; }
        if (z == nz - 1) { f[14] = f[9]; f[15] = f[10]; f[16] = f[11]; f[17] = f[12]; f[18] = f[13]; }
        if (type == ORC_YSYM_TOP) { f[4] = f[2]; f[7] = f[6]; f[8] = f[5]; f[13] = f[11]; f[18] = f[16]; }
        else { f[2] = f[4]; f[6] = f[7]; f[5] = f[8]; f[11] = f[13]; f[16] = f[18]; }
    } else if (type == ORC_ZSYM_TOP || type == ORC_ZSYM_BOT) {
        if (y == 0) { f[2] = f[4]; f[6] = f[7]; f[5] = f[8]; f[11] = f[13]; f[16] = f[18]; }
        if (y == ny - 1) { f[4] = f[2]; f[7] = f[6]; f[8] = f[5]; f[13] = f[11]; f[18] = f[16]; }
        if (type == ORC_ZSYM_TOP) { f[14] = f[9]; f[15] = f[10]; f[16] = f[11]; f[17] = f[12]; f[18] = f[13]; }
        else { f[9] = f[14]; f[10] = f[15]; f[11] = f[16]; f[12] = f[17]; f[13] = f[18]; }
    } else if (type == ORC_WEST_REG) {
        /* BC1:789-870: momentum replaced by (u, 0, w), everything else kept;
         * w = 0.01 at t = 1000, 2000, 3000 */
        const T w = (t == 1000 || t == 2000 || t == 3000) ? T(0.01) : T(0);
        T j[3] = {0, 0, 0};
        for (int q = 0; q < 19; ++q) j[0] += CX[q] * f[q], j[1] += CY[q] * f[q], j[2] += CZ[q] * f[q];
        const T d[3] = {(u - j[0]) / T(10), (T(0) - j[1]) / T(10), (w - j[2]) / T(10)};
        for (int q = 0; q < 19; ++q) f[q] += CX[q] * d[0] + CY[q] * d[1] + CZ[q] * d[2];
    } else if (type == ORC_DIR_WEST_V || type == ORC_DIR_NORTH || type == ORC_DIR_SOUTH) {
        /* CPU:379-453 (west, velocity (0, u, 0), its y edges first) and
         * CPU:578-745 (north / south walls moving with (u, 0, 0)): the z
         * face copies, then each unknown from its opposite plus
         * 6 w_q rho c_q . u at rho = 1 */
        if (type == ORC_DIR_WEST_V) {
            if (y == 0) { f[2] = f[4]; f[6] = f[7]; f[11] = f[13]; f[16] = f[18]; }
            else if (y == ny - 1) { f[4] = f[2]; f[7] = f[6]; f[13] = f[11]; f[18] = f[16]; }
        }
        if (z == 0) { f[9] = f[14]; f[10] = f[15]; f[11] = f[16]; f[12] = f[17]; f[13] = f[18]; }
        else if (z == nz - 1) { f[14] = f[9]; f[15] = f[10]; f[16] = f[11]; f[17] = f[12]; f[18] = f[13]; }
        const T ux = type == ORC_DIR_WEST_V ? T(0) : u, uy = type == ORC_DIR_WEST_V ? u : T(0), uz = 0;
        const T a = T(0.33333333), b = T(0.166666667);
        if (type == ORC_DIR_WEST_V) {
            f[1] = f[3] + a * ux;
            f[5] = f[7] + b * (ux + uy);
            f[8] = f[6] + b * (ux - uy);
            f[10] = f[17] + b * (ux + uz);
            f[15] = f[12] + b * (ux - uz);
        } else if (type == ORC_DIR_NORTH) {
            f[4] = f[2] - a * uy;
            f[7] = f[5] - b * (ux + uy);
            f[8] = f[6] + b * (ux - uy);
            f[13] = f[16] - b * (uy - uz);
            f[18] = f[11] - b * (uy + uz);
        } else {
            f[2] = f[4] + a * uy;
            f[5] = f[7] + b * (ux + uy);
            f[6] = f[8] - b * (ux - uy);
            f[16] = f[13] + b * (uy - uz);
            f[11] = f[18] + b * (uy + uz);
        }
    }
}

template <class T> inline void lid(T* f, int face, T ux, T uy, T uz, int quirk) {
    int axis = face / 2;
    int sgn = (face % 2 == 0) ? 1 : -1; /* inward normal component */
    const int* C[3] = {CX, CY, CZ};
    T un = (axis == 0 ? ux : axis == 1 ? uy : uz) * T(sgn);
    T s0 = 0, s1 = 0;
    for (int q = 0; q < Q; ++q) {
        int cn = C[axis][q] * sgn;
        if (cn == 0) s0 += f[q];
        else if (cn < 0) s1 += f[q];
    }
    T rho = un + (s0 + T(2) * s1);
    T feq[Q];
    for (int q = 0; q < Q; ++q) feq[q] = feq_bgk<T>(q, rho, ux, uy, uz);
    T usq = ux * ux + uy * uy + uz * uz;
    if (quirk) {
        /* CPU:1012, 1014: (v+w)*(u+w) and (-v+w)*(u+w) in place of the squares */
        feq[11] = wq<T>(11) * (rho + T(3) * (uy + uz) + T(4.5) * (uy + uz) * (ux + uz) - T(1.5) * usq);
        feq[13] = wq<T>(13) * (rho + T(3) * (-uy + uz) + T(4.5) * (-uy + uz) * (ux + uz) - T(1.5) * usq);
    }
    T f6 = f[6];
    for (int q = 0; q < Q; ++q)
        if (C[axis][q] * sgn > 0) f[q] = feq[q] + f[OPP[q]] - feq[OPP[q]];
    if (quirk && face == 0) f[8] = feq[6] + f6 - feq[6]; /* CPU:1023 */
    T P[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int q = 0; q < Q; ++q) {
        T g = f[q] - feq[q];
        int c[3] = {CX[q], CY[q], CZ[q]};
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) P[a][b] += T(c[a] * c[b]) * g;
    }
    for (int q = 0; q < Q; ++q) {
        int c[3] = {CX[q], CY[q], CZ[q]};
        T s = 0;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) s += (T(c[a] * c[b]) - (a == b ? T(1) / T(3) : T(0))) * P[a][b];
        f[q] = feq[q] + wq<T>(q) * T(4.5) * s;
    }
}

/* PhysicalMoments (LR7:380-391): rho, j, and the second-order moments m9,
 * m11, m13, m14, m15 of f */
template <class T> inline void physical_moments(const T* f, T* mom) {
    T m[Q];
    moments(f, m);
    mom[0] = m[0];
    mom[1] = m[3];
    mom[2] = m[5];
    mom[3] = m[7];
    mom[4] = m[9];
    mom[5] = m[11];
    mom[6] = m[13];
    mom[7] = m[14];
    mom[8] = m[15];
}

/* StrainRate (LR7:351-377) with omega = 1, m1 = 0, dx = 1 */
template <class T> inline void strain_rate(const T* mom, T* S) {
    T u = mom[1], v = mom[2], w = mom[3];
    T n9 = mom[4] - (T(2) * u * u - (v * v + w * w));
    T n11 = mom[5] - (v * v - w * w);
    T n13 = mom[6] - u * v;
    T n14 = mom[7] - v * w;
    T n15 = mom[8] - u * w;
    S[0] = T(-0.5) * n9;
    S[1] = T(0.25) * (n9 - T(3) * n11);
    S[2] = T(0.25) * (n9 + T(3) * n11);
    S[3] = T(-1.5) * n13;
    S[4] = T(-1.5) * n14;
    S[5] = T(-1.5) * n15;
}

template <class T> inline T strain_mag(const T* S) {
    return std::sqrt(T(2) * (S[0] * S[0] + S[1] * S[1] + S[2] * S[2] + T(2) * S[3] * S[3] +
                             T(2) * S[4] * S[4] + T(2) * S[5] * S[5]));
}

/* moments -> populations with the non-equilibrium stress scaled by SF
 * (InvertPhysicalMoments, LR7:421-465) */
template <class T> inline void invert_scaled(const T* mom, T SF, T* f) {
    T m[Q];
    for (int k = 0; k < Q; ++k) m[k] = 0;
    T rho = mom[0], u = mom[1], v = mom[2], w = mom[3];
    T usq = u * u + v * v + w * w;
    m[0] = rho;
    m[1] = T(-11) * rho + T(19) * usq;
    m[2] = T(7.53968254) * usq;
    m[3] = u;
    m[4] = T(-0.666666667) * u;
    m[5] = v;
    m[6] = T(-0.666666667) * v;
    m[7] = w;
    m[8] = T(-0.666666667) * w;
    m[9] = mom[4] * SF + (T(1) - SF) * (T(2) * u * u - (v * v + w * w));
    m[11] = mom[5] * SF + (T(1) - SF) * (v * v - w * w);
    m[13] = mom[6] * SF + (T(1) - SF) * u * v;
    m[14] = mom[7] * SF + (T(1) - SF) * v * w;
    m[15] = mom[8] * SF + (T(1) - SF) * u * w;
    invert(m, f);
}

/* InvertPhysicalMoments_LES_cf (LR7:524-579): coarse -> fine rescale factor
 * with the eddy viscosity of the interpolated strain */
template <class T> inline void invert_les_cf(const T* mom, T omega_c, T cs, T lrf, T* f) {
    T S[6];
    strain_rate(mom, S);
    T smag = strain_mag(S);
    T tau_c = T(1) / omega_c;
    T tau_f = T(2) * tau_c - T(0.5) + T(1.5) * smag * cs;
    T omega_f = T(1) / tau_f;
    tau_c = tau_c + smag * cs;
    omega_c = T(1) / tau_c;
    T SF = (lrf * omega_c * (T(1) - omega_f)) / ((T(1) - omega_c) * omega_f);
    invert_scaled(mom, SF, f);
}

/* InvertPhysicalMoments_LES_fc (LR7:467-522) */
template <class T> inline void invert_les_fc(const T* mom, T omega_f, T cs, T lrf, T* f) {
    T S[6];
    strain_rate(mom, S);
    T smag = strain_mag(S);
    T tau_f = T(1) / omega_f;
    T tau_c = tau_f + T(0.5) + T(12) * smag * cs;
    tau_c *= T(0.5);
    T omega_c = T(1) / tau_c;
    tau_f = tau_f + smag * cs;
    omega_f = T(1) / tau_f;
    T SF = (T(1) - omega_c) * omega_f / (lrf * omega_c * (T(1) - omega_f));
    invert_scaled(mom, SF, f);
}

inline int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
inline int edge(int i, int n, int clamp) { return clamp ? (i < 0 ? 0 : (i >= n ? n - 1 : i)) : wrap(i, n); }

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter (cell, step, 0, 0),
 * key (seed, 0): the seeded inlet noise stream (extension, not in the reference). */
inline void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = uint64_t(0xD2511F53u) * c[0];
        uint64_t p1 = uint64_t(0xCD9E8D57u) * c[2];
        uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
        uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
        uint32_t n0 = hi1 ^ c[1] ^ k0, n1 = lo1, n2 = hi0 ^ c[3] ^ k1, n3 = lo0;
        c[0] = n0;
        c[1] = n1;
        c[2] = n2;
        c[3] = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

template <class T>
void step_impl(const orc_params* p, const uint8_t* mask, const T* fA, T* fB, double* force3,
               float* av_u, float* av_v, float* fl_u, float* fl_v, float* mom_export) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const long N = long(nx) * ny * nz;
    double fx = 0, fy = 0, fz = 0;
#pragma omp parallel for reduction(+ : fx, fy, fz) schedule(static)
    for (int z = 0; z < nz; ++z) {
        for (int y = 0; y < ny; ++y) {
            for (int x = 0; x < nx; ++x) {
                const long c = (long(z) * ny + y) * nx + x;
                const int im = mask[c];
                /* half-way bounce-back: solid nodes keep the full-way update
                 * (their values are never pulled by a fluid node) */
                const bool hw = p->halfway && im != ORC_WALL && im != ORC_BODY;
                T f[Q];
                /* pull (LR7:1445-1491); the reference's z halo planes become a
                 * periodic wrap, x/y wrap only reaches boundary nodes whose
                 * pulled values the reference discards */
                for (int q = 0; q < Q; ++q) {
                    const int cl = p->pull_clamp;
                    int xs = edge(x - CX[q], nx, cl), ys = edge(y - CY[q], ny, cl), zs = edge(z - CZ[q], nz, cl);
                    f[q] = fA[q * N + (long(zs) * ny + ys) * nx + xs];
                    if (hw && q > 0) {
                        const int nt = mask[(long(zs) * ny + ys) * nx + xs];
                        if (nt == ORC_WALL || nt == ORC_BODY) {
                            /* the node's own opposite population, reflected half-way */
                            f[q] = fA[OPP[q] * N + c];
                            if (nt == ORC_BODY && p->force_on) {
                                /* link-wise momentum exchange: 2 c_opp(q) f*_opp(q) */
                                const double v = 2.0 * double(f[q]);
                                fx -= CX[q] * v;
                                fy -= CY[q] * v;
                                fz -= CZ[q] * v;
                            }
                        }
                    }
                }
                if (im == ORC_WALL || im == ORC_BODY) {
                    /* full-way bounce-back + momentum exchange (LR7:1493-1526) */
                    if (im == ORC_BODY && p->force_on && !p->halfway) {
                        double sx = 0, sy = 0, sz = 0;
                        for (int q = 1; q < Q; ++q) {
                            sx += 2.0 * CX[q] * double(f[q]);
                            sy += 2.0 * CY[q] * double(f[q]);
                            sz += 2.0 * CZ[q] * double(f[q]);
                        }
                        fx += sx;
                        fy += sy;
                        fz += sz;
                    }
                    for (int q = 0; q < Q; ++q) fB[q * N + c] = f[OPP[q]];
                } else {
                    if (im == ORC_WEST_INLET || im == ORC_EAST_OUTLET || im == ORC_SOUTH_INLET ||
                        im == ORC_NORTH_OUTLET) {
                        /* the rebuild starts from the neighbour's stored
                         * (post-collision) populations, LR7:1531-1557 */
                        int xs = x, ys = y;
                        if (im == ORC_WEST_INLET) xs = wrap(x + 1, nx);
                        if (im == ORC_EAST_OUTLET) xs = wrap(x - 1, nx);
                        if (im == ORC_SOUTH_INLET) ys = wrap(y + 1, ny);
                        if (im == ORC_NORTH_OUTLET) ys = wrap(y - 1, ny);
                        long cs_ = (long(z) * ny + ys) * nx + xs;
                        for (int q = 0; q < Q; ++q) f[q] = fA[q * N + cs_];
                        T uin = T(p->u_in);
                        if (p->noise_amp != 0.f)
                            uin = uin + T(p->u_in) * T(p->noise_amp) *
                                            (T(2) * T(orc_noise_uniform(p->noise_seed, uint32_t(c),
                                                                        uint32_t(p->t))) -
                                             T(1));
                        extrap<T>(im, f, T(p->rho_out), uin);
                    } else if (im == ORC_LID) {
                        lid<T>(f, p->lid_face, T(p->lid_u[0]), T(p->lid_u[1]), T(p->lid_u[2]), p->lid_quirk);
                    } else if (im >= ORC_DIR_WEST) {
                        alt_boundary<T>(im, f, y, z, ny, nz, T(p->u_in), p->t);
                    }
                    if (p->mlp) {
                        double g[Q];
                        for (int q = 0; q < Q; ++q) g[q] = double(f[q]);
                        const double tau0 = 1.0 / double(p->omega);
                        if (p->mlp_every <= 1 || !p->mlp_nu || p->t % p->mlp_every == 0) {
                            double nu = 0;
                            orc_collide_mlp(p->mlp, tau0, g, 1, &nu);
                            if (p->mlp_nu) p->mlp_nu[c] = nu;
                        } else {
                            orc_collide_d(0, 0, 1.0 / (tau0 + 3.0 * p->mlp_nu[c]), 0, 0, g, 1);
                        }
                        for (int q = 0; q < Q; ++q) f[q] = T(g[q]);
                    } else {
                        /* DI3:1358: the body force acts only up to DYNY1 */
                        const T dp = (p->dyn_y1 > 0 && y > p->dyn_y1) ? T(0) : T(p->dpdy);
                        collide<T>(p->model, f, T(p->omega), p->les, T(p->cs), dp);
                    }
                    if (p->stats_on && av_u) {
                        /* vel_av / vel_fluc (LR7:1018-1058) */
                        float u = 0, v = 0;
                        for (int q = 0; q < Q; ++q) {
                            u += float(CX[q]) * float(f[q]);
                            v += float(CY[q]) * float(f[q]);
                        }
                        float wgt = p->stats_weight;
                        if (p->t >= p->start_av && p->t < p->start_fluc) {
                            float n = float(p->t - p->start_av);
                            av_u[c] = (av_u[c] * n + u * wgt) / (n + wgt);
                            av_v[c] = (av_v[c] * n + v * wgt) / (n + wgt);
                        } else if (p->t >= p->start_fluc) {
                            float n = float(p->t - p->start_fluc);
                            float du = (u - av_u[c]) * (u - av_u[c]);
                            float dv = (v - av_v[c]) * (v - av_v[c]);
                            fl_u[c] = (fl_u[c] * n + du * wgt) / (n + wgt);
                            fl_v[c] = (fl_v[c] * n + dv * wgt) / (n + wgt);
                        }
                    }
                    for (int q = 0; q < Q; ++q) fB[q * N + c] = f[q];
                }
                if (mom_export && p->exp_nx > 0) {
                    /* moments for the coarse->fine interpolation (LR7:1590-1605):
                     * post-collision for fluid nodes, the pulled values at
                     * bounce-back nodes */
                    int ex = x - p->exp_x0, ey = y - p->exp_y0;
                    if (ex >= 0 && ex < p->exp_nx && ey >= 0 && ey < p->exp_ny) {
                        float ff[Q], mom[9];
                        for (int q = 0; q < Q; ++q) ff[q] = float(f[q]);
                        physical_moments(ff, mom);
                        long ne = long(p->exp_nx) * p->exp_ny * nz;
                        long ce = (long(z) * p->exp_ny + ey) * p->exp_nx + ex;
                        for (int i = 0; i < 9; ++i) mom_export[i * ne + ce] = mom[i];
                    }
                }
            }
        }
    }
    if (force3) {
        force3[0] += fx;
        force3[1] += fy;
        force3[2] += fz;
    }
}

}  // namespace

extern "C" {

void orc_collide(int model, int les, float omega, float cs, float dpdy, float* f, int n) {
    for (int i = 0; i < n; ++i) collide<float>(model, f + 19L * i, omega, les, cs, dpdy);
}

void orc_collide_d(int model, int les, double omega, double cs, double dpdy, double* f, int n) {
    for (int i = 0; i < n; ++i) collide<double>(model, f + 19L * i, omega, les, cs, dpdy);
}

void orc_extrap(int kind, float* f, int n, float rho, float u_in) {
    for (int i = 0; i < n; ++i) extrap<float>(kind, f + 19L * i, rho, u_in);
}

void orc_moments(const float* f, float* m, int n) {
    for (int i = 0; i < n; ++i) moments(f + 19L * i, m + 19L * i);
}

void orc_physical_moments(const float* f, float* mom, int n) {
    for (int i = 0; i < n; ++i) physical_moments(f + 19L * i, mom + 9L * i);
}

void orc_strain_rate(const float* mom, float* s, int n) {
    for (int i = 0; i < n; ++i) strain_rate(mom + 9L * i, s + 6L * i);
}

void orc_invert_les_cf(const float* mom, float* f, int n, float omega_c, float cs, float lrf) {
    for (int i = 0; i < n; ++i) invert_les_cf(mom + 9L * i, omega_c, cs, lrf, f + 19L * i);
}

void orc_invert_les_fc(const float* mom, float* f, int n, float omega_f, float cs, float lrf) {
    for (int i = 0; i < n; ++i) invert_les_fc(mom + 9L * i, omega_f, cs, lrf, f + 19L * i);
}

void orc_alt_boundary(int type, float* f, int n, const int* yz, int ny, int nz, float u, int t) {
    for (int i = 0; i < n; ++i) alt_boundary<float>(type, f + 19L * i, yz[2 * i], yz[2 * i + 1], ny, nz, u, t);
}

void orc_lid(float* f, int n, int face, float ux, float uy, float uz, int quirk) {
    for (int i = 0; i < n; ++i) lid<float>(f + 19L * i, face, ux, uy, uz, quirk);
}

/* initialize / initializeLR (LR7:1060-1125): equilibrium at rho = 1, u = u0
 * (zero at bounce-back nodes).  kind 0: mrt_meq + InvertMoments (LR7);
 * kind 1: BGK equilibrium (DI3); kind 2: BGK equilibrium on every node,
 * solids included (CPU_3D/CPU_3D.cpp:1226-1308). */
void orc_init_axis(const orc_params* p, const uint8_t* mask, float* f, int kind, float u0, int axis) {
    const long N = long(p->nx) * p->ny * p->nz;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < N; ++c) {
        /* kind 2: CPU_3D initialises every node, solids included, at u0 */
        float u = (kind != 2 && (mask[c] == ORC_WALL || mask[c] == ORC_BODY)) ? 0.f : u0;
        float v3[3] = {0.f, 0.f, 0.f};
        v3[axis] = u;
        float ff[Q];
        if (kind == 0) {
            float meq[Q];
            meq_lr7<float>(meq, 1.f, v3[0], v3[1], v3[2]);
            invert(meq, ff);
        } else {
            for (int q = 0; q < Q; ++q) ff[q] = feq_bgk<float>(q, 1.f, v3[0], v3[1], v3[2]);
        }
        for (int q = 0; q < Q; ++q) f[q * N + c] = ff[q];
    }
}

void orc_init(const orc_params* p, const uint8_t* mask, float* f, int kind, float u0) {
    orc_init_axis(p, mask, f, kind, u0, 0);
}

void orc_step(const orc_params* p, const uint8_t* mask, const float* fA, float* fB, double* force3,
              float* av_u, float* av_v, float* fl_u, float* fl_v, float* mom_export) {
    step_impl<float>(p, mask, fA, fB, force3, av_u, av_v, fl_u, fl_v, mom_export);
}

void orc_step_d(const orc_params* p, const uint8_t* mask, const double* fA, double* fB,
                double* force3) {
    step_impl<double>(p, mask, fA, fB, force3, nullptr, nullptr, nullptr, nullptr, nullptr);
}

/* InterpCF (LR7:1991-2170): fill the fine patch's 2-wide x/y band from the
 * coarse moments exported after the coarse step.  mom_c is [9][cnz][eny][enx]
 * with enx = fnx*lrfactor + 1, origin (int(lrx0), int(lry0)).  The fine patch
 * spans the periodic z extent: fine plane k sits at lrz0 + k*lrfactor. */
void orc_interp_cf(const orc_refine* r, const float* mom_c, float* f_f, const uint8_t* mask_f) {
    const int enx = int(r->fnx * r->lrfactor) + 1, eny = int(r->fny * r->lrfactor) + 1;
    const long ne = long(enx) * eny * r->cnz;
    const long NF = long(r->fnx) * r->fny * r->fnz;
    const int L = r->lrlevel;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < r->fnz; ++k) {
        for (int yf = 0; yf < r->fny; ++yf) {
            for (int xf = 0; xf < r->fnx; ++xf) {
                if (!(xf < L || xf > r->fnx - L - 1 || yf < L || yf > r->fny - L - 1 ||
                      (r->zbounded && (k < L || k > r->fnz - L - 1))))
                    continue;
                long cf = (long(k) * r->fny + yf) * r->fnx + xf;
                if (mask_f[cf] == ORC_WALL || mask_f[cf] == ORC_BODY) continue;
                /* coarse cell containing the fine node: base corner and offsets
                 * (LR7:2004-2005, 2082-2088); z base is plane k/L - 1 (periodic) */
                float xr = xf * r->lrfactor + r->lrfactor * 0.5f;
                float yr = yf * r->lrfactor + r->lrfactor * 0.5f;
                int xm = int(xr), ym = int(yr);
                float fx_ = xr - xm, fy_ = yr - ym;
                int zb = k / L - 1;
                float fz_ = (k % L) * r->lrfactor + r->lrfactor * 0.5f;
                if (r->zbounded) {
                    /* as x and y, from the coarse plane cz0 */
                    const float zr = k * r->lrfactor + r->lrfactor * 0.5f;
                    zb = r->cz0 + int(zr);
                    fz_ = zr - int(zr);
                }
                float mc[8][9], S[8][6];
                for (int cz = 0; cz < 2; ++cz)
                    for (int cy = 0; cy < 2; ++cy)
                        for (int cx = 0; cx < 2; ++cx) {
                            int i = cx + 2 * cy + 4 * cz;
                            int zc = wrap(zb + cz, r->cnz);
                            long ce = (long(zc) * eny + (ym + cy)) * enx + (xm + cx);
                            for (int m = 0; m < 9; ++m) mc[i][m] = mom_c[m * ne + ce];
                            strain_rate(mc[i], S[i]);
                        }
                float mom[9];
                for (int m = 0; m < 9; ++m) {
                    mom[m] = mc[0][m] * (1.f - fx_) * (1.f - fy_) * (1.f - fz_) +
                             mc[1][m] * fx_ * (1.f - fy_) * (1.f - fz_) +
                             mc[2][m] * (1.f - fx_) * fy_ * (1.f - fz_) +
                             mc[3][m] * fx_ * fy_ * (1.f - fz_) +
                             mc[4][m] * (1.f - fx_) * (1.f - fy_) * fz_ +
                             mc[5][m] * fx_ * (1.f - fy_) * fz_ +
                             mc[6][m] * (1.f - fx_) * fy_ * fz_ + mc[7][m] * fx_ * fy_ * fz_;
                }
                if (r->order == 2) {
                    /* second-order velocity correction from the corner strain
                     * rates and momenta (LR7:2101-2144) */
                    float sx[8], sy[8], sz[8];
                    for (int i = 0; i < 8; ++i) {
                        sx[i] = (i & 1) ? 1.f : -1.f;
                        sy[i] = (i & 2) ? 1.f : -1.f;
                        sz[i] = (i & 4) ? 1.f : -1.f;
                    }
                    float a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                    /* a: cx cy cz dx dy dz ex ey ez */
                    for (int i = 0; i < 8; ++i) {
                        a[0] += sx[i] * S[i][0];
                        a[1] += sy[i] * S[i][3] - sx[i] * sy[i] * mc[i][2];
                        a[2] += sz[i] * S[i][5] - sx[i] * sz[i] * mc[i][3];
                        a[3] += sx[i] * S[i][3] - sx[i] * sy[i] * mc[i][1];
                        a[4] += sy[i] * S[i][1];
                        a[5] += sz[i] * S[i][4] - sy[i] * sz[i] * mc[i][3];
                        a[6] += sx[i] * S[i][5] - sx[i] * sz[i] * mc[i][1];
                        a[7] += sy[i] * S[i][4] - sy[i] * sz[i] * mc[i][2];
                        a[8] += sz[i] * S[i][2];
                    }
                    for (int j = 0; j < 9; ++j) a[j] *= (j % 4 == 0) ? -0.03125f : -0.0625f;
                    float wx = 1.f - (4.f * fx_ * fx_ - 4.f * fx_ + 1.f);
                    float wy = 1.f - (4.f * fy_ * fy_ - 4.f * fy_ + 1.f);
                    float wz = 1.f - (4.f * fz_ * fz_ - 4.f * fz_ + 1.f);
                    mom[1] += a[0] * wx + a[1] * wy + a[2] * wz;
                    mom[2] += a[3] * wx + a[4] * wy + a[5] * wz;
                    mom[3] += a[6] * wx + a[7] * wy + a[8] * wz;
                }
                float ff[Q];
                invert_les_cf(mom, r->omega_c, r->cs, r->lrfactor, ff);
                for (int q = 0; q < Q; ++q) f_f[q * NF + cf] = ff[q];
            }
        }
    }
}

/* InterpFC (LR7:2172-2348): overwrite coarse nodes strictly inside the patch
 * (2-node margin) with the restriction of their 8 fine children. */
void orc_interp_fc(const orc_refine* r, const float* f_f, float* f_c, const uint8_t* mask_c) {
    const long NF = long(r->fnx) * r->fny * r->fnz;
    const long NC = long(r->cnx) * r->cny * r->cnz;
    const int L = r->lrlevel;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < r->cnz; ++z) {
        for (int y = 0; y < r->cny; ++y) {
            for (int x = 0; x < r->cnx; ++x) {
                if (!(x > r->lrx0 + 1 && x < r->lrx0 + r->fnx * r->lrfactor - 2 && y > r->lry0 + 1 &&
                      y < r->lry0 + r->fny * r->lrfactor - 2))
                    continue;
                if (r->zbounded && !(z > r->lrz0 + 1 && z < r->lrz0 + r->fnz * r->lrfactor - 2)) continue;
                long cc = (long(z) * r->cny + y) * r->cnx + x;
                if (mask_c[cc] == ORC_WALL || mask_c[cc] == ORC_BODY) continue;
                int xm = int(L * (x - r->lrx0)), ym = int(L * (y - r->lry0));
                /* fine planes at z -/+ lrfactor/2: global fine index 2z+1, 2z+2 */
                int kl = int(L * (z - r->lrz0)), kh = kl + 1;
                bool top = (kh >= r->fnz);
                kl = wrap(kl, r->fnz);
                kh = wrap(kh, r->fnz);
                /* the reference reads the top plane's corners upper-plane first
                 * (LR7:2195-2229) */
                int k0 = kl, k1 = kh;
                if (top && r->quirk_fc_top_zflip) {
                    k0 = kh;
                    k1 = kl;
                }
                float mc[8][9], S[8][6];
                for (int cz = 0; cz < 2; ++cz)
                    for (int cy = 0; cy < 2; ++cy)
                        for (int cx = 0; cx < 2; ++cx) {
                            int i = cx + 2 * cy + 4 * cz;
                            int kk = cz ? k1 : k0;
                            long cf = (long(kk) * r->fny + (ym + cy)) * r->fnx + (xm + cx);
                            float ff[Q];
                            for (int q = 0; q < Q; ++q) ff[q] = f_f[q * NF + cf];
                            physical_moments(ff, mc[i]);
                            strain_rate(mc[i], S[i]);
                        }
                float mom[9];
                for (int m = 0; m < 9; ++m) {
                    float s = 0;
                    for (int i = 0; i < 8; ++i) s += mc[i][m];
                    mom[m] = 0.125f * s;
                }
                if (r->order == 2) {
                    float sx[8], sy[8], sz[8];
                    for (int i = 0; i < 8; ++i) {
                        sx[i] = (i & 1) ? 1.f : -1.f;
                        sy[i] = (i & 2) ? 1.f : -1.f;
                        sz[i] = (i & 4) ? 1.f : -1.f;
                    }
                    float a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                    for (int i = 0; i < 8; ++i) {
                        a[0] += sx[i] * S[i][0];
                        a[1] += sy[i] * S[i][3] - sx[i] * sy[i] * mc[i][2];
                        a[2] += sz[i] * S[i][5] - sx[i] * sz[i] * mc[i][3];
                        a[3] += sx[i] * S[i][3] - sx[i] * sy[i] * mc[i][1];
                        a[4] += sy[i] * S[i][1];
                        a[5] += sz[i] * S[i][4] - sy[i] * sz[i] * mc[i][3];
                        a[6] += sx[i] * S[i][5] - sx[i] * sz[i] * mc[i][1];
                        a[7] += sy[i] * S[i][4] - sy[i] * sz[i] * mc[i][2];
                        a[8] += sz[i] * S[i][2];
                    }
                    for (int j = 0; j < 9; ++j) a[j] *= (j % 4 == 0) ? -0.03125f : -0.0625f;
                    /* the reference sets xpr = ypr = zpr = 0 here (LR7:2310-2312) */
                    mom[1] += a[0] + a[1] + a[2];
                    mom[2] += a[3] + a[4] + a[5];
                    mom[3] += a[6] + a[7] + a[8];
                }
                float ff[Q];
                invert_les_fc(mom, r->omega_f, r->cs, r->lrfactor, ff);
                for (int q = 0; q < Q; ++q) f_c[q * NC + cc] = ff[q];
            }
        }
    }
}

/* ImageFcn of the channel programs (LR7:88-127): body (square |dx|,|dy| < r or
 * circle dx^2 + dy^2 < r^2), walls at y = 0 and y = ny-1, inlet x = 0, outlet
 * x = nx-1; walls take precedence over the inlet/outlet, which take precedence
 * over the body. */
void orc_mask_channel(uint8_t* mask, int nx, int ny, int nz, int body_shape, float ox, float oy,
                      float r) {
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                int v = ORC_FLUID;
                if (body_shape == 1) {
                    if (std::fabs(float(x) - ox) < r && std::fabs(float(y) - oy) < r) v = ORC_BODY;
                } else if (body_shape == 2) {
                    float dx = float(x) - ox, dy = float(y) - oy;
                    if (dx * dx + dy * dy < r * r) v = ORC_BODY;
                }
                if (y == 0 || y == ny - 1) v = ORC_WALL;
                else if (x == 0) v = ORC_WEST_INLET;
                else if (x == nx - 1) v = ORC_EAST_OUTLET;
                mask[(long(z) * ny + y) * nx + x] = uint8_t(v);
            }
}

/* ImageFcnLR (LR7:68-86) on fine-node coordinates */
void orc_mask_fine(uint8_t* mask, int nx, int ny, int nz, float x0, float y0, float z0, float h,
                   int body_shape, float ox, float oy, float r) {
    (void)z0;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                float xc = x0 + float(x) * h, yc = y0 + float(y) * h;
                int v = ORC_FLUID;
                if (body_shape == 1) {
                    if (std::fabs(xc - ox) < r && std::fabs(yc - oy) < r) v = ORC_BODY;
                } else if (body_shape == 2) {
                    float dx = xc - ox, dy = yc - oy;
                    if (dx * dx + dy * dy < r * r) v = ORC_BODY;
                }
                mask[(long(z) * ny + y) * nx + x] = uint8_t(v);
            }
}

/* lid-driven cavity: the lid face is ORC_LID, every other face ORC_WALL
 * (CPU_3D/CPU_3D.cpp:67-73 has the lid at x = 0) */
void orc_mask_cavity(uint8_t* mask, int nx, int ny, int nz, int lid_face) {
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                int c[3] = {x, y, z}, n[3] = {nx, ny, nz};
                int a = lid_face / 2;
                bool on_lid = (lid_face % 2 == 0) ? c[a] == 0 : c[a] == n[a] - 1;
                int v = ORC_FLUID;
                if (on_lid) v = ORC_LID;
                else if (x == 0 || x == nx - 1 || y == 0 || y == ny - 1 || z == 0 || z == nz - 1)
                    v = ORC_WALL;
                mask[(long(z) * ny + y) * nx + x] = uint8_t(v);
            }
}

void orc_mask_dyninlet(uint8_t* mask, int nx, int ny, int nz, float ox, float oy, float r, int trip) {
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                int v = ORC_FLUID;
                if (trip) {
                    if (std::fabs(float(x) - ox) < r && std::fabs(float(y) - oy) < r) v = ORC_BODY;
                    if (std::fabs(float(x) - ox - 3.f) < r && std::fabs(float(y) - oy - 3.f) < r && z == 10)
                        v = ORC_BODY;
                }
                if (x == 0 || x == nx - 1) v = ORC_WALL;
                mask[(long(z) * ny + y) * nx + x] = uint8_t(v);
            }
}

double orc_mass(const float* f, const uint8_t* mask, int ncell) {
    double s = 0;
    for (long c = 0; c < ncell; ++c) {
        if (mask && (mask[c] == ORC_WALL || mask[c] == ORC_BODY)) continue;
        for (int q = 0; q < Q; ++q) s += double(f[q * long(ncell) + c]);
    }
    return s;
}

uint32_t orc_noise_hash(uint32_t seed, uint32_t cell, uint32_t step) {
    uint32_t c[4] = {cell, step, 0u, 0u};
    philox(c, seed, 0u);
    return c[0];
}

float orc_noise_uniform(uint32_t seed, uint32_t cell, uint32_t step) {
    return float(orc_noise_hash(seed, cell, step) >> 8) * (1.0f / 16777216.0f);
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}

}  // extern "C"
