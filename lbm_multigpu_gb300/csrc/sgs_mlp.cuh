/* The learned subgrid closure: a per-cell MLP 16 -> 64 -> 64 -> 1 (ReLU,
 * softplus output) giving a local Smagorinsky coefficient, whose eddy
 * viscosity nu_t replaces the constant-Cs Smagorinsky model in the
 * collision.
 *
 * Hidden unit HC = 63 of the first layer is the constant 1 (whatever row 63
 * of W1 holds; that row takes no part).  It carries the second layer's bias
 * on the tensor cores: the weight blob stores W2[j][HC] + b2[j] in column HC
 * and W1 row HC = e15, so that the MMA itself makes h1[HC] = relu(x15) = 1.
 *
 * Inputs, all local to a node (what the collide kernel has in registers):
 * with the non-equilibrium stress Pi_neq of the pulled populations,
 *   p_ij = -3/2 Pi_neq_ij / rho  (= tau_eff S_ij by Chapman-Enskog),
 *   x0..x11  0 (reserved)
 *   x12      |p| = sqrt(2 p:p)                              (/ P_REF)
 *   x13      tr(p^3) / (p:p)^(3/2), 0 for p = 0
 *   x14      (tau0 - 1/2) * 100, the molecular viscosity
 *   x15      1 (carries the first layer's bias)
 * The inputs are invariants of p only.  Its components (frame-dependent)
 * are left out: near tau0 = 1/2 the non-equilibrium stress carries a mode
 * that changes sign every step (factor 1 - omega per collision), and a
 * network that responds to the signed components modulates the relaxation
 * at that rate and pumps the mode (in the 512 x 128 x 128 channel at
 * tau0 = 0.52 it raised the wake's u_rms by 65 %; without them, 0.1 %).
 * Output: the coefficient o = NU_SCALE * softplus(y) and the eddy viscosity
 *   nu_t = o * x12 / tau0 = o * G |S|,  |S| = sqrt(2 S:S) = sqrt(2 p:p) / tau0,
 * with G = 1 / P_REF = 100: o = 1e-4 is Smagorinsky's Cs = 0.1 (Cs^2 = o G),
 * and nu_t goes to zero with the strain whatever the network makes of the
 * other inputs; tau_eff = tau0 + 3 nu_t.
 *
 * Parameter vector (FP32 master copy, PyTorch Linear order [out][in]):
 *   W1[64][16] (column 15 = b1, row HC unused) | W2[64][64] | b2[64] | w3[64] | b3
 */
#pragma once
#include <cstdint>

namespace lbm {
namespace sgs {

constexpr int NIN = 16, NH = 64, HC = NH - 1;
constexpr int OFF_W1 = 0, OFF_W2 = OFF_W1 + NH * NIN, OFF_B2 = OFF_W2 + NH * NH, OFF_W3 = OFF_B2 + NH,
              OFF_B3 = OFF_W3 + NH, NPARAM = OFF_B3 + 1;
constexpr float P_REF = 0.01f, NU_SCALE = 1e-4f;

/* features of one node from p_ij (xx, yy, zz, xy, xz, yz), tau0 and
 * inv_t0 = 1 / tau0 (a kernel computes it once) */
template <class T> __host__ __device__ inline void features(const T p[6], T tau0, T inv_t0, T x[NIN]) {
    const T pp = p[0] * p[0] + p[1] * p[1] + p[2] * p[2] + T(2) * (p[3] * p[3] + p[4] * p[4] + p[5] * p[5]);
    /* tr(p^3) of the symmetric tensor */
    const T xx = p[0], yy = p[1], zz = p[2], xy = p[3], xz = p[4], yz = p[5];
    const T tr3 = xx * xx * xx + yy * yy * yy + zz * zz * zz + T(3) * xx * (xy * xy + xz * xz) +
                  T(3) * yy * (xy * xy + yz * yz) + T(3) * zz * (xz * xz + yz * yz) + T(6) * xy * xz * yz;
    (void)inv_t0;
    for (int i = 0; i < 12; ++i) x[i] = T(0);
    x[12] = sqrt(T(2) * pp) * T(1.0 / P_REF);
    x[13] = pp > T(1e-30) ? tr3 / (pp * sqrt(pp)) : T(0);
    x[14] = (tau0 - T(0.5)) * T(100);
    x[15] = T(1);
}

#if defined(__CUDACC__)
/* the same features in FP32 with one rsqrt for |p| and the invariant (the
 * inference rounds them to bf16, far above the rsqrt's 2 ulp) */
__device__ __forceinline__ void features_fast(const float p[6], float tau0, float inv_t0, float x[NIN]) {
    const float pp = p[0] * p[0] + p[1] * p[1] + p[2] * p[2] + 2.f * (p[3] * p[3] + p[4] * p[4] + p[5] * p[5]);
    const float xx = p[0], yy = p[1], zz = p[2], xy = p[3], xz = p[4], yz = p[5];
    const float tr3 = xx * xx * xx + yy * yy * yy + zz * zz * zz + 3.f * xx * (xy * xy + xz * xz) +
                      3.f * yy * (xy * xy + yz * yz) + 3.f * zz * (xz * xz + yz * yz) + 6.f * xy * xz * yz;
    (void)inv_t0;
    for (int i = 0; i < 12; ++i) x[i] = 0.f;
    const float r = pp > 1e-30f ? rsqrtf(pp) : 0.f;
    x[12] = pp * r * (1.41421356f / P_REF);
    x[13] = tr3 * (r * r * r);
    x[14] = (tau0 - 0.5f) * 100.f;
    x[15] = 1.f;
}
#endif

template <class T> __host__ __device__ inline void features(const T p[6], T tau0, T x[NIN]) {
    features<T>(p, tau0, T(1) / tau0, x);
}

/* nu_t / o of a node with features x: G |S| = x12 / tau0 */
template <class T> __host__ __device__ inline T strain_gain(const T x[NIN], T inv_t0) { return x[12] * inv_t0; }

}  // namespace sgs
}  // namespace lbm
