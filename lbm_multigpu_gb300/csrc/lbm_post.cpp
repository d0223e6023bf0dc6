/*
 * lbm_post.cpp -- the post-processing of the reference's outputs behind the
 * C ABI, host only:
 *   ForceCalcs (bgk_channel1/Re3000_Cyl2/ForceCalcs.cpp, TandemCylinderTest1/
 *   ForceCalcs.cpp): mean and RMS of each force component of a `.force`
 *   history between two line indices, with that program's FP32 running
 *   updates (ForceCalcs.cpp:60-95);
 *   drag and lift coefficients and the Strouhal number of the lift;
 *   VelProf (bgk_channel1/Re3000/VelProf.cpp, MRTtest/bgk/VelProf.cpp,
 *   TurbChannel4/VelProf.cpp): a wall-normal line of mean and fluctuation
 *   statistics in wall units (VelProf.cpp:94-100);
 *   velplus (TurbChannel3/Re500/velplus.cpp): centre-line mean and RMS
 *   profiles of the middle z plane, in units of uMax;
 *   mean/fluctuation profiles along y from a level's statistics arrays,
 *   averaged over z (the `_slice.dat` columns velAv / velFluc, LR7:2350-2420).
 */
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "lbm_kernels.cuh"

using namespace lbm;

namespace {

/* in-place radix-2 FFT (n a power of two) */
void fft(std::vector<std::complex<double>>& a) {
    const size_t n = a.size();
    for (size_t i = 1, j = 0; i < n; ++i) {
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[i], a[j]);
    }
    for (size_t len = 2; len <= n; len <<= 1) {
        const double ang = -2 * M_PI / double(len);
        const std::complex<double> wl(std::cos(ang), std::sin(ang));
        for (size_t i = 0; i < n; i += len) {
            std::complex<double> w(1);
            for (size_t j = 0; j < len / 2; ++j) {
                const std::complex<double> u = a[i + j], v = a[i + j + len / 2] * w;
                a[i + j] = u + v;
                a[i + j + len / 2] = u - v;
                w *= wl;
            }
        }
    }
}

}  // namespace

extern "C" {

int lbm_force_stats(const float* fxyz, int n, int t_start, int t_end, float* mean3, float* rms3) {
    if (!fxyz || !mean3 || !rms3 || t_start < 0 || t_end > n || t_end <= t_start)
        return set_error(LBM_ERR_ARG, "force stats: bad range", cudaSuccess);
    float av[3] = {0, 0, 0}, fl[3] = {0, 0, 0};
    /* running mean in FP32 over the lines t_start .. t_end - 1 */
    for (int i = t_start; i < t_end; ++i) {
        const int j = i - t_start;
        for (int k = 0; k < 3; ++k) av[k] = av[k] * j / (j + 1) + fxyz[3 * i + k] / (j + 1);
    }
    /* then the running variance about that mean */
    for (int i = t_start; i < t_end; ++i) {
        const int j = i - t_start;
        for (int k = 0; k < 3; ++k) {
            const float d = fxyz[3 * i + k] - av[k];
            fl[k] = fl[k] * j / (j + 1) + d * d / (j + 1);
        }
    }
    for (int k = 0; k < 3; ++k) {
        mean3[k] = av[k];
        rms3[k] = std::sqrt(fl[k]);
    }
    return LBM_OK;
}

int lbm_force_coefficients(const double* fxyz, int n, int t_start, double u, double d, double lz, double rho,
                           double* cd, double* cl_rms, double* st) {
    if (!fxyz || t_start < 0 || n - t_start < 4 || !(u > 0) || !(d > 0) || !(lz > 0) || !(rho > 0))
        return set_error(LBM_ERR_ARG, "force coefficients: bad arguments", cudaSuccess);
    const int m = n - t_start;
    double sx = 0, sy = 0;
    for (int i = t_start; i < n; ++i) sx += fxyz[3 * i], sy += fxyz[3 * i + 1];
    const double mx = sx / m, my = sy / m;
    double vy = 0;
    for (int i = t_start; i < n; ++i) vy += (fxyz[3 * i + 1] - my) * (fxyz[3 * i + 1] - my);
    const double q = 0.5 * rho * u * u * d * lz;
    if (cd) *cd = mx / q;
    if (cl_rms) *cl_rms = std::sqrt(vy / m) / q;
    if (st) {
        /* dominant frequency of the lift: the periodogram peak of the
         * mean-removed signal (Hann window, zero padded), refined by a
         * parabola through the peak bin and its neighbours */
        size_t np = 1;
        while (np < size_t(2 * m)) np <<= 1;
        std::vector<std::complex<double>> a(np, 0.0);
        for (int i = 0; i < m; ++i) {
            const double w = 0.5 - 0.5 * std::cos(2 * M_PI * i / (m - 1));
            a[i] = w * (fxyz[3 * (t_start + i) + 1] - my);
        }
        fft(a);
        size_t kb = 1;
        double pb = 0;
        for (size_t k = 1; k < np / 2; ++k)
            if (std::norm(a[k]) > pb) pb = std::norm(a[k]), kb = k;
        double kf = double(kb);
        if (kb > 1 && kb + 1 < np / 2) {
            const double l = std::log(std::norm(a[kb - 1]) + 1e-300), c = std::log(pb + 1e-300),
                         r = std::log(std::norm(a[kb + 1]) + 1e-300);
            const double den = l - 2 * c + r;
            if (den < 0) kf += 0.5 * (l - r) / den;
        }
        *st = pb > 0 ? (kf / double(np)) * d / u : 0.0;
    }
    return LBM_OK;
}

int lbm_wall_profile(const float* v_mean, const float* u_fluc, const float* v_fluc, const float* w_fluc, int n,
                     float u_tau, float nu, float* yplus, float* vplus, float* urms, float* vrms, float* wrms) {
    if (!v_mean || !u_fluc || !v_fluc || !w_fluc || n <= 0 || !(u_tau > 0) || !(nu > 0))
        return set_error(LBM_ERR_ARG, "wall profile: bad arguments", cudaSuccess);
    for (int i = 0; i < n; ++i) {
        /* first fluid node half a spacing off the wall (VelProf.cpp:96) */
        if (yplus) yplus[i] = (i - 0.5f) * u_tau / nu;
        if (vplus) vplus[i] = v_mean[i] / u_tau;
        if (urms) urms[i] = std::sqrt(u_fluc[i]) / u_tau;
        if (vrms) vrms[i] = std::sqrt(v_fluc[i]) / u_tau;
        if (wrms) wrms[i] = std::sqrt(w_fluc[i]) / u_tau;
    }
    return LBM_OK;
}

int lbm_centerline_profiles(const float* stats4, int nx, int ny, int nz, double umax, float* uave, float* urms,
                            float* vave, float* vrms) {
    if (!stats4 || nx <= 0 || ny <= 0 || nz <= 0 || !(umax > 0))
        return set_error(LBM_ERR_ARG, "centerline profiles: bad arguments", cudaSuccess);
    const size_t n = size_t(nx) * ny * nz;
    const size_t plane = size_t(nz / 2) * ny * nx;
    const float* au = stats4;
    const float* av = stats4 + n;
    const float* fu = stats4 + 2 * n;
    const float* fv = stats4 + 3 * n;
    /* u along y on x = nx / 2, v along x on y = ny / 2 (velplus.cpp:94-101);
     * the division by uMax in double, stored as float as that program does */
    for (int y = 0; y < ny; ++y) {
        const size_t c = plane + size_t(y) * nx + nx / 2;
        if (uave) uave[y] = float(au[c] / umax);
        if (urms) urms[y] = float(std::sqrt(fu[c]) / umax);
    }
    for (int x = 0; x < nx; ++x) {
        const size_t c = plane + size_t(ny / 2) * nx + x;
        if (vave) vave[x] = float(av[c] / umax);
        if (vrms) vrms[x] = float(std::sqrt(fv[c]) / umax);
    }
    return LBM_OK;
}

int lbm_stats_profiles(const float* stats4, int nx, int ny, int nz, int x, float* prof4) {
    if (!stats4 || !prof4 || nx <= 0 || ny <= 0 || nz <= 0 || x < 0 || x >= nx)
        return set_error(LBM_ERR_ARG, "stats profiles: bad arguments", cudaSuccess);
    const size_t n = size_t(nx) * ny * nz;
    for (int k = 0; k < 4; ++k)
        for (int y = 0; y < ny; ++y) {
            double s = 0;
            for (int z = 0; z < nz; ++z) s += stats4[k * n + (size_t(z) * ny + y) * nx + x];
            prof4[k * ny + y] = float(s / nz);
        }
    return LBM_OK;
}

}  // extern "C"
