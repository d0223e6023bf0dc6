/*
 * cell_ops_shim.cu -- test-only host build of the product's per-cell operators
 * (lbm_multigpu_gb300/csrc/d3q19.cuh) so their arithmetic can be compared with
 * the oracle on a machine without a GPU.  Not part of the product library.
 */
#include <stdint.h>

#include "../../lbm_multigpu_gb300/csrc/d3q19.cuh"

using namespace lbm;

extern "C" {

void cell_collide(int model, int les, float omega, float cs, float dpdy, float* f, int n) {
    for (int i = 0; i < n; ++i) collide<float>(model, f + 19L * i, omega, les != 0, cs, dpdy);
}
void cell_collide_d(int model, int les, double omega, double cs, double dpdy, double* f, int n) {
    for (int i = 0; i < n; ++i) collide<double>(model, f + 19L * i, omega, les != 0, cs, dpdy);
}
void cell_extrap(int type, float* f, int n, float rho, float u_in) {
    for (int i = 0; i < n; ++i) extrap<float>(type, f + 19L * i, rho, u_in);
}
void cell_lid(float* f, int n, int face, float ux, float uy, float uz, int quirk) {
    for (int i = 0; i < n; ++i) lid<float>(f + 19L * i, face, ux, uy, uz, quirk != 0);
}
void cell_physical_moments(const float* f, float* mom, int n) {
    for (int i = 0; i < n; ++i) physical_moments<float>(f + 19L * i, mom + 9L * i);
}
void cell_strain_rate(const float* mom, float* s, int n) {
    for (int i = 0; i < n; ++i) strain_rate<float>(mom + 9L * i, s + 6L * i);
}
void cell_invert_scaled(const float* mom, float sf, float* f, int n) {
    for (int i = 0; i < n; ++i) invert_scaled<float>(mom + 9L * i, sf, f + 19L * i);
}
void cell_collide_mrt_dev_d(int les, double omega, double cs, double u, double* h, int n) {
    const double k = 18.0 * 1.4142135623730951 * cs;
    for (int i = 0; i < n; ++i) collide_mrt_dev<double>(h + 19L * i, omega, les != 0, 1.0 / omega, k, u);
}
void cell_collide_mrt_dev(int les, float omega, float cs, float u, float* h, int n) {
    const float k = 18.f * 1.41421356f * cs;
    for (int i = 0; i < n; ++i) collide_mrt_dev<float>(h + 19L * i, omega, les != 0, 1.f / omega, k, u);
}
void cell_pi_neq_d(const double* f, double* rho, double* p6, int n) {
    for (int i = 0; i < n; ++i) pi_neq<double>(f + 19L * i, rho[i], p6 + 6L * i);
}
void cell_mrt_dev_pi_d(const double* f, double* rho, double* p6, int n) {
    for (int i = 0; i < n; ++i) {
        const MrtDev<double> m = mrt_dev_moments<double>(f + 19L * i, 0.0);
        rho[i] = m.rho;
        mrt_dev_pi(m, p6 + 6L * i);
    }
}
float cell_philox_uniform(uint32_t seed, uint32_t cell, uint32_t step) { return philox_uniform(seed, cell, step); }
void cell_alt_boundary(int type, float* f, int n, const int* yz, int ny, int nz, float u, int t) {
    for (int i = 0; i < n; ++i) alt_boundary<float>(type, f + 19L * i, 0, yz[2 * i], yz[2 * i + 1], 0, ny, nz, u, t);
}

}  // extern "C"
