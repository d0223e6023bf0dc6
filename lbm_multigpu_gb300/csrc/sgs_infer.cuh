/* Tensor-core inference of the learned subgrid closure, for use inside a
 * kernel whose block of ROWS threads (ROWS = 128 or 256) each holds one
 * node's 16 features.  One call evaluates the MLP for the whole block:
 *
 *   features -> bf16 -> shared memory (A operand, core-matrix layout)
 *   layer 1:  tcgen05.mma  Z1[ROWS][64] = X[ROWS][16] W1^T   (TMEM, FP32)
 *   tcgen05.ld -> GELU -> bf16 -> shared memory (A operand of layer 2)
 *   layer 2:  tcgen05.mma  Z2[ROWS][64] = H1[ROWS][64] W2^T, 4 K-steps
 *   tcgen05.ld -> + b2 -> GELU -> dot w3 + b3 -> softplus -> nu_t
 *
 * Thread t of the block owns row t: MMA h = t / 128 covers rows 128 h ..
 * 128 h + 127 in TMEM lanes 0..127 of columns 64 h .. 64 h + 63, and warp w
 * reads lanes 32 (w % 4) .. + 31, which are exactly its threads' rows.
 * One elected thread issues the MMAs; completion arrives on an mbarrier whose
 * wait is bounded (on a timeout the block reports an error code and returns
 * nu_t = 0 so that the caller's state stays finite).
 */
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "sgs_mlp.cuh"
#include "tc_sm103.cuh"

namespace lbm {
namespace sgs {

/* shared-memory byte layout of the operands (no swizzle, K-major) */
constexpr uint32_t W1_LBO = 128, W1_SBO = 256;    /* K = 16: two core matrices per row group */
constexpr uint32_t W2_LBO = 128, W2_SBO = 1024;   /* K = 64: eight */
constexpr uint32_t W1_BYTES = NH * NIN * 2, W2_BYTES = NH * NH * 2;
/* device weight blob: W1 and W2 already in the core-matrix layout as bf16,
 * then b2[64], w3[64], b3 as FP32 */
constexpr uint32_t BLOB_BYTES = W1_BYTES + W2_BYTES + (2 * NH + 4) * 4;
constexpr int SM_SMEM_BYTES = 228 * 1024; /* shared memory per SM */

template <int ROWS> struct InferSmem;

/* dynamic shared memory for a block of ROWS rows that holds InferSmem (plus
 * 1 KB of alignment slack) and is large enough that no more blocks than TMEM
 * can serve (512 columns) fit on one SM */
template <int ROWS> inline size_t infer_dyn_smem();

template <int ROWS> struct InferSmem {
    alignas(1024) unsigned char w1[W1_BYTES];
    alignas(1024) unsigned char w2[W2_BYTES];
    alignas(1024) unsigned char a1[ROWS * NIN * 2];
    alignas(1024) unsigned char a2[ROWS * NH * 2];
    float b2[NH], w3[NH], b3;
    alignas(8) uint64_t mbar;
    uint32_t tmem;
    uint32_t phase;
};

/* TMEM columns a block holds: 64 per 128 rows */
template <int ROWS> __host__ __device__ constexpr int tmem_cols() { return ROWS / 2 < 32 ? 32 : ROWS / 2; }

template <int ROWS> inline size_t infer_dyn_smem() {
    static size_t v = 0;
    if (!v) {
        int dev = 0, per_sm = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
            per_sm <= 0)
            per_sm = SM_SMEM_BYTES;
        const int max_blocks = 512 / tmem_cols<ROWS>();
        const size_t need = sizeof(InferSmem<ROWS>) + 1024;
        const size_t floor = size_t(per_sm) / size_t(max_blocks + 1) + 1;
        v = need > floor ? need : floor;
    }
    return v;
}

#if defined(__CUDA_ARCH__)

/* linear thread index (blocks may be 1-D or 2-D): row of the block's tile */
__device__ __forceinline__ int row_index() {
    return int(threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z));
}

/* once per block: weights into shared memory, the mbarrier, TMEM columns.
 * tcgen05.alloc waits until the columns are free, so a launch must never
 * make more blocks resident on an SM than 512 / tmem_cols<ROWS>() (the
 * launchers size dynamic shared memory to guarantee it) */
template <int ROWS> __device__ __forceinline__ void infer_setup(InferSmem<ROWS>& s, const unsigned char* blob) {
    const int t = row_index();
    const uint4* src = reinterpret_cast<const uint4*>(blob);
    for (int i = t; i < int(W1_BYTES / 16); i += ROWS) reinterpret_cast<uint4*>(s.w1)[i] = src[i];
    for (int i = t; i < int(W2_BYTES / 16); i += ROWS)
        reinterpret_cast<uint4*>(s.w2)[i] = src[W1_BYTES / 16 + i];
    const float* fp = reinterpret_cast<const float*>(blob + W1_BYTES + W2_BYTES);
    if (t < NH) {
        s.b2[t] = fp[t];
        s.w3[t] = fp[NH + t];
    }
    if (t == 0) {
        s.b3 = fp[2 * NH];
        tc::mbar_init(&s.mbar, 1);
        s.phase = 0;
    }
    if (t < 32) tc::tmem_alloc(&s.tmem, tmem_cols<ROWS>());
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

template <int ROWS> __device__ __forceinline__ void infer_teardown(InferSmem<ROWS>& s) {
    tc::fence_before_sync();
    __syncthreads();
    if (row_index() < 32) tc::tmem_dealloc(s.tmem, tmem_cols<ROWS>());
}

__device__ __forceinline__ float gelu_fast(float z) {
    float t;
    const float u = GELU_A * fmaf(GELU_B * z, z * z, z);
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
    const float h = 0.5f * z;
    return fmaf(h, t, h);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

/* the block's MMA pair; every thread of the block must call it (uniformly);
 * returns false when a completion wait ran out */
template <int ROWS> __device__ __forceinline__ bool infer_mma_wait(InferSmem<ROWS>& s) {
    /* block-uniform verdict: tcgen05.ld below is warp-collective */
    const bool ok = __syncthreads_and(tc::mbar_wait(&s.mbar, s.phase, 1u << 20));
    tc::fence_after_sync();
    return ok;
}

/* nu_t of this thread's row; x[16] are its features (FP32) */
template <int ROWS> __device__ __forceinline__ float infer_nu(InferSmem<ROWS>& s, const float x[NIN], int* err) {
    static_assert(ROWS == 128 || ROWS == 256, "one or two M=128 MMAs per block");
    const int t = row_index(), warp = t >> 5;
    /* A of layer 1 */
    {
        uint4 v0, v1;
        v0.x = pack_bf16(x[0], x[1]), v0.y = pack_bf16(x[2], x[3]), v0.z = pack_bf16(x[4], x[5]),
        v0.w = pack_bf16(x[6], x[7]);
        v1.x = pack_bf16(x[8], x[9]), v1.y = pack_bf16(x[10], x[11]), v1.z = pack_bf16(x[12], x[13]),
        v1.w = pack_bf16(x[14], x[15]);
        *reinterpret_cast<uint4*>(s.a1 + tc::core_off(t, 0, W1_LBO, W1_SBO)) = v0;
        *reinterpret_cast<uint4*>(s.a1 + tc::core_off(t, 8, W1_LBO, W1_SBO)) = v1;
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t id = tc::idesc_bf16_f32(128, NH);
    if (t == 0) {
#pragma unroll
        for (int h = 0; h < ROWS / 128; ++h)
            tc::mma_bf16(s.tmem + 64 * h, tc::sdesc(tc::smem_u32(s.a1) + h * 16 * W1_SBO, W1_LBO, W1_SBO),
                         tc::sdesc(tc::smem_u32(s.w1), W1_LBO, W1_SBO), id, 0);
        tc::mma_commit(&s.mbar);
    }
    bool ok = infer_mma_wait(s);
    const uint32_t ta = s.tmem + (uint32_t((warp & 3) * 32) << 16) + uint32_t(warp >> 2) * 64;
    /* accumulator columns in chunks of 16 (few live registers):
     * GELU -> bf16 -> A of layer 2 */
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        uint32_t r[16];
        if (ok) {
            tc::tmem_ld16(ta + 16 * c, r);
            tc::tmem_wait_ld();
            tc::tmem_fence_regs<16>(r);
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            float g[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) g[k] = ok ? gelu_fast(__uint_as_float(r[8 * h + k])) : 0.f;
            uint4 v;
            v.x = pack_bf16(g[0], g[1]), v.y = pack_bf16(g[2], g[3]), v.z = pack_bf16(g[4], g[5]),
            v.w = pack_bf16(g[6], g[7]);
            *reinterpret_cast<uint4*>(s.a2 + tc::core_off(t, 16 * c + 8 * h, W2_LBO, W2_SBO)) = v;
        }
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (t == 0) {
        s.phase ^= 1;
#pragma unroll
        for (int h = 0; h < ROWS / 128; ++h)
#pragma unroll
            for (int kc = 0; kc < NH / 16; ++kc)
                tc::mma_bf16(s.tmem + 64 * h,
                             tc::sdesc(tc::smem_u32(s.a2) + h * 16 * W2_SBO + kc * 2 * W2_LBO, W2_LBO, W2_SBO),
                             tc::sdesc(tc::smem_u32(s.w2) + kc * 2 * W2_LBO, W2_LBO, W2_SBO), id, kc > 0);
        tc::mma_commit(&s.mbar);
    }
    __syncthreads(); /* every thread sees the flipped phase */
    ok = infer_mma_wait(s) && ok;
    float y = s.b3;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        uint32_t r[16];
        if (ok) {
            tc::tmem_ld16(ta + 16 * c, r);
            tc::tmem_wait_ld();
            tc::tmem_fence_regs<16>(r);
        }
#pragma unroll
        for (int k = 0; k < 16; ++k)
            y = ok ? fmaf(s.w3[16 * c + k], gelu_fast(__uint_as_float(r[k]) + s.b2[16 * c + k]), y) : y;
    }
    tc::fence_before_sync();
    __syncthreads();
    if (t == 0) s.phase ^= 1;
    if (!ok) {
        if (t == 0) atomicExch(err, 2);
        return 0.f;
    }
    const float sp = y > 20.f ? y : log1pf(__expf(y));
    return NU_SCALE * sp;
}

#endif /* __CUDA_ARCH__ */

}  // namespace sgs
}  // namespace lbm
