/*
 * ref_shim_bc1.cpp -- host build of BC1's West_Reg (BC1/LRMultiGPU7.cu:789,
 * defined there and not called), staged by oracle/ref_recipe.py into
 * oracle/_ref/bc1_westreg.inc.  TEST INFRASTRUCTURE ONLY.
 */
#include <cmath>

#define __device__

#include "bc1_westreg.inc"

extern "C" {

void ref_west_reg(float* f, int n, float u, int t) {
    for (int i = 0; i < n; ++i) West_Reg(f + 19L * i, u, t);
}

}  // extern "C"
