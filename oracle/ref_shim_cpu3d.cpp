/*
 * ref_shim_cpu3d.cpp -- host build of the reference CPU code's per-cell
 * functions (CPU_3D/CPU_3D.cpp from bgk_collide up to main(), CPU:116-1209),
 * staged by oracle/ref_recipe.py into oracle/_ref/cpu3d_body.inc.
 *
 * TEST INFRASTRUCTURE ONLY.  Exposes bgk_collide, mrt_collide, the
 * regularised lid boundary DirichletWest_Regularized and the boundaries()
 * dispatch on n cells (cell-major).
 */
#include <sys/time.h>

#include <cmath>
#include <cstdlib>
#include <iostream>

using namespace std;

#include "cpu3d_body.inc"

#define F19(g) g[0], g[1], g[2], g[3], g[4], g[5], g[6], g[7], g[8], g[9], g[10], g[11], g[12], g[13], g[14], g[15], g[16], g[17], g[18]

extern "C" {

void ref_cpu3d_bgk(float* f, int n, float omega) {
    for (int i = 0; i < n; ++i) {
        float* g = f + 19L * i;
        bgk_collide(F19(g), omega);
    }
}

void ref_cpu3d_mrt(float* f, int n, float omega) {
    for (int i = 0; i < n; ++i) {
        float* g = f + 19L * i;
        mrt_collide(F19(g), omega);
    }
}

void ref_cpu3d_lid_west(float* f, int n) {
    for (int i = 0; i < n; ++i) {
        float* g = f + 19L * i;
        DirichletWest_Regularized(F19(g), 1, 1);
    }
}

/* CPU_3D's boundaries() dispatch (CPU:1142-1196) for node code im on n
 * cells at (y, z) = yz[2 i], yz[2 i + 1] of its YDIM x ZDIM domain */
void ref_cpu3d_boundary(float* f, int n, const int* yz, int im) {
    for (int i = 0; i < n; ++i) {
        float* g = f + 19L * i;
        boundaries(F19(g), yz[2 * i], yz[2 * i + 1], im);
    }
}

/* DirichletNorth_Reg / DirichletSouth_Reg (CPU:578-745; written, but the
 * dispatch's lines for them are commented out) on n cells at (y, z) */
void ref_cpu3d_dirichlet_ns(float* f, int n, const int* yz, int north) {
    for (int i = 0; i < n; ++i) {
        float* g = f + 19L * i;
        if (north) DirichletNorth_Reg(F19(g), yz[2 * i], yz[2 * i + 1]);
        else DirichletSouth_Reg(F19(g), yz[2 * i], yz[2 * i + 1]);
    }
}

/* the domain the staged functions were compiled for */
int ref_cpu3d_ydim(void) { return YDIM; }
int ref_cpu3d_zdim(void) { return ZDIM; }
float ref_cpu3d_umax(void) { return UMAX; }

}  // extern "C"
