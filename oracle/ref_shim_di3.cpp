/*
 * ref_shim_di3.cpp -- host build of the reference's DynInlet3 per-cell device
 * functions (MRTtest/DynInlet3.cu, from ImageFcnLR up to the first kernel),
 * staged by oracle/ref_recipe.py into oracle/_ref/di3_body.inc.
 *
 * TEST INFRASTRUCTURE ONLY.  Exposes the MRT (bgk_meq) and BGK collide
 * branches with their Smagorinsky block and AddForce (DI3:599-832).  MODEL is
 * a pointer to a string literal of this translation unit, so the reference's
 * MODEL == "MRT" pointer comparison (DI3:609) behaves as in the original.
 */
#include <cmath>
#include <cstring>
#include <iostream>

using namespace std;

#define __global__
#define __device__

static const char* g_model = "MRT";
#define MODEL g_model

#include "di3_body.inc"

extern "C" {

void ref_di3_collide(float* f, int n, float omega, float dpdy, int use_mrt) {
    g_model = use_mrt ? "MRT" : "BGK";
    for (int i = 0; i < n; ++i) mrt_collide(f + 19L * i, omega, dpdy);
}

}  // extern "C"
