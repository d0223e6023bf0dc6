/*
 * lbm_pairs.cu -- the stream-collide kernels (sc_kernels.cuh) in the blocked
 * pair layout (Level::blocked = 2: the 19 populations of 32 x-consecutive
 * nodes stored together, each opposite pair interleaved so that a node
 * stores it with one wide store), for FP32, FP16 and BF16 storage.  A
 * separate translation unit, compiled in parallel with the others.
 */
#include "sc_kernels.cuh"

namespace lbm {

cudaError_t launch_sc_pairs(const Level& L, const StepParams& p, const void* fA, void* fB, const uint8_t* mask,
                              float* stats, float* mom_export, cudaStream_t s, const uint32_t* links) {
    return launch_sc_layout<2>(L, p, fA, fB, mask, stats, mom_export, s, links);
}

cudaError_t launch_sc_mlp_pairs(const Level& L, const StepParams& p, const void* fA, void* fB,
                                  const uint8_t* mask, float* stats, const uint32_t* links, const void* blob, int* err,
                                  cudaStream_t s) {
    return launch_sc_mlp_layout<2>(L, p, fA, fB, mask, stats, links, blob, err, s);
}

}  // namespace lbm
