/*
 * lbm_blocked.cu -- the stream-collide kernels (sc_kernels.cuh) in the blocked
 * population layout (Level::blocked: the 19 populations of 32 x-consecutive
 * nodes stored together, each opposite pair interleaved), for FP32, FP16 and
 * BF16 storage.  A separate translation unit, so that it compiles in
 * parallel with the structure-of-arrays instances in lbm_kernels.cu.
 */
#include "sc_kernels.cuh"

namespace lbm {

cudaError_t launch_sc_blocked(const Level& L, const StepParams& p, const void* fA, void* fB, const uint8_t* mask,
                              float* stats, float* mom_export, cudaStream_t s, const uint32_t* links) {
    return launch_sc_layout<1>(L, p, fA, fB, mask, stats, mom_export, s, links);
}

cudaError_t launch_sc_mlp_blocked(const Level& L, const StepParams& p, const void* fA, void* fB,
                                  const uint8_t* mask, float* stats, const uint32_t* links, const void* blob, int* err,
                                  cudaStream_t s) {
    return launch_sc_mlp_layout<1>(L, p, fA, fB, mask, stats, links, blob, err, s);
}

}  // namespace lbm
