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
/* device weight blob: W1 and W2 in the core-matrix layout as bf16, then
 * b2[64], b3 (+ 3 pad) and w3[64] as FP32 */
constexpr uint32_t BLOB_B2 = W1_BYTES + W2_BYTES;
constexpr uint32_t BLOB_BYTES = BLOB_B2 + NH * 4 + 16 + NH * 4;
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
    alignas(1024) unsigned char a2[ROWS * NH * 2]; /* h1, then h2 */
    float b2[NH], b3;
    alignas(16) float w3[NH];
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
    if (t < NH) {
        s.b2[t] = reinterpret_cast<const float*>(blob + BLOB_B2)[t];
        s.w3[t] = reinterpret_cast<const float*>(blob + BLOB_B2 + NH * 4 + 16)[t];
    }
    if (t == 0) {
        s.b3 = *reinterpret_cast<const float*>(blob + BLOB_B2 + NH * 4);
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

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

/* GELU (tanh form) of two FP32 accumulator values in packed FP32 pair
 * arithmetic (f32x2, one instruction per pair), one MUFU tanh per value:
 *   u = z (a + a b z^2),  gelu = h + h tanh(u),  h = z / 2
 * returned as a bf16 pair for the next layer's A operand */
__device__ __forceinline__ uint32_t gelu2(float z0, float z1) {
    uint64_t z, z2, t, u, h, th, g;
    const uint64_t ca = 0x3F4C422A3F4C422Aull;  /* a   = 0.7978846 */
    const uint64_t cab = 0x3D12226A3D12226Aull; /* a b = 0.0356774 */
    const uint64_t half = 0x3F0000003F000000ull;
    asm("mov.b64 %0, {%1, %2};" : "=l"(z) : "f"(z0), "f"(z1));
    asm("mul.rn.f32x2 %0, %1, %1;" : "=l"(z2) : "l"(z));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(t) : "l"(z2), "l"(cab), "l"(ca));
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(u) : "l"(t), "l"(z));
    float u0, u1, t0, t1;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(u0), "=f"(u1) : "l"(u));
    asm("tanh.approx.f32 %0, %1;" : "=f"(t0) : "f"(u0));
    asm("tanh.approx.f32 %0, %1;" : "=f"(t1) : "f"(u1));
    asm("mov.b64 %0, {%1, %2};" : "=l"(th) : "f"(t0), "f"(t1));
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(h) : "l"(z), "l"(half));
    asm("fma.rn.f32x2 %0, %1, %2, %1;" : "=l"(g) : "l"(h), "l"(th));
    float g0, g1;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(g0), "=f"(g1) : "l"(g));
    return pack_bf16(g0, g1);
}

/* the same GELU pair kept in FP32, accumulated into acc += gelu(z) * w
 * (packed pair arithmetic): the output layer on the CUDA cores */
__device__ __forceinline__ uint64_t gelu2_dot(float z0, float z1, uint64_t w, uint64_t acc) {
    uint64_t z, z2, t, u, h, th, g, r;
    const uint64_t ca = 0x3F4C422A3F4C422Aull;
    const uint64_t cab = 0x3D12226A3D12226Aull;
    const uint64_t half = 0x3F0000003F000000ull;
    asm("mov.b64 %0, {%1, %2};" : "=l"(z) : "f"(z0), "f"(z1));
    asm("mul.rn.f32x2 %0, %1, %1;" : "=l"(z2) : "l"(z));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(t) : "l"(z2), "l"(cab), "l"(ca));
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(u) : "l"(t), "l"(z));
    float u0, u1, t0, t1;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(u0), "=f"(u1) : "l"(u));
    asm("tanh.approx.f32 %0, %1;" : "=f"(t0) : "f"(u0));
    asm("tanh.approx.f32 %0, %1;" : "=f"(t1) : "f"(u1));
    asm("mov.b64 %0, {%1, %2};" : "=l"(th) : "f"(t0), "f"(t1));
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(h) : "l"(z), "l"(half));
    asm("fma.rn.f32x2 %0, %1, %2, %1;" : "=l"(g) : "l"(h), "l"(th));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(g), "l"(w), "l"(acc));
    return r;
}

/* every thread of the block must call it (uniformly); returns false when a
 * completion wait ran out.  Flips the expected phase for the next wait. */
template <int ROWS> __device__ __forceinline__ bool infer_mma_wait(InferSmem<ROWS>& s) {
    /* one warp polls the mbarrier; the others wait at the block barrier
     * without taking issue slots.  The verdict is block-uniform (tcgen05.ld
     * below is warp-collective) */
    bool w = true;
    if (row_index() < 32) w = tc::mbar_wait(&s.mbar, s.phase, 1u << 20);
    const bool ok = __syncthreads_and(w);
    tc::fence_after_sync();
    return ok;
}

/* make this thread's shared-memory operand rows visible to the tensor core
 * and line the block up behind the MMA issue */
__device__ __forceinline__ void infer_publish() {
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

/* the accumulator (16 columns at a time) of this thread's row through the
 * epilogue: (+ b2) -> GELU -> bf16 -> A operand rows in a2.  The loads run
 * even after a failed wait (they are valid TMEM reads); the caller then
 * discards the row's result */
template <int ROWS, bool BIAS> __device__ __forceinline__ void infer_epilogue(InferSmem<ROWS>& s, uint32_t ta, int t) {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        uint32_t r[16];
        tc::tmem_ld16(ta + 16 * c, r);
        tc::tmem_wait_ld();
        tc::tmem_fence_regs<16>(r);
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
            uint32_t g[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int j = 16 * c + 8 * hh + 2 * k;
                float z0 = __uint_as_float(r[8 * hh + 2 * k]), z1 = __uint_as_float(r[8 * hh + 2 * k + 1]);
                if (BIAS) z0 += s.b2[j], z1 += s.b2[j + 1];
                g[k] = gelu2(z0, z1);
            }
            *reinterpret_cast<uint4*>(s.a2 + tc::core_off(t, 16 * c + 8 * hh, W2_LBO, W2_SBO)) =
                make_uint4(g[0], g[1], g[2], g[3]);
        }
    }
}

/* nu_t of this thread's row; x[16] are its features (FP32) */
template <int ROWS> __device__ __forceinline__ float infer_nu(InferSmem<ROWS>& s, const float x[NIN], int* err) {
    static_assert(ROWS == 128 || ROWS == 256, "one or two M=128 MMAs per block");
    const int t = row_index(), warp = t >> 5;
    /* A of layer 1 */
    *reinterpret_cast<uint4*>(s.a1 + tc::core_off(t, 0, W1_LBO, W1_SBO)) =
        make_uint4(pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(x[4], x[5]), pack_bf16(x[6], x[7]));
    *reinterpret_cast<uint4*>(s.a1 + tc::core_off(t, 8, W1_LBO, W1_SBO)) = make_uint4(
        pack_bf16(x[8], x[9]), pack_bf16(x[10], x[11]), pack_bf16(x[12], x[13]), pack_bf16(x[14], x[15]));
    infer_publish();
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
    /* layer 1 epilogue: GELU -> h1 */
    infer_epilogue<ROWS, false>(s, ta, t);
    infer_publish();
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
    /* layer 2 epilogue and the output layer: y = b3 + sum_j w3_j GELU(z2_j + b2_j) */
    uint64_t acc = 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        uint32_t r[16];
        tc::tmem_ld16(ta + 16 * c, r);
        tc::tmem_wait_ld();
        tc::tmem_fence_regs<16>(r);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int j = 16 * c + 2 * k;
            const uint64_t w = *reinterpret_cast<const uint64_t*>(&s.w3[j]);
            acc = gelu2_dot(__uint_as_float(r[2 * k]) + s.b2[j], __uint_as_float(r[2 * k + 1]) + s.b2[j + 1], w, acc);
        }
    }
    float a0, a1;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a0), "=f"(a1) : "l"(acc));
    const float y = s.b3 + a0 + a1;
    tc::fence_before_sync();
    __syncthreads();
    if (t == 0) s.phase ^= 1; /* one flip per completion: phase names the next one */
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
