/* Tensor-core inference of the learned subgrid closure, for use inside a
 * kernel whose block of ROWS threads (ROWS = 128 or 256) each holds one
 * node's 16 features.  One call evaluates the MLP for the whole block, the
 * two hidden layers on the tensor core:
 *
 *   features -> bf16 -> shared memory (A operand, core-matrix layout)
 *   layer 1:  tcgen05.mma  Z1[ROWS][64] = X[ROWS][16] W1^T       (TMEM, FP32)
 *   tcgen05.ld -> ReLU + bf16 pack (one cvt per pair) -> shared memory
 *   layer 2:  tcgen05.mma  Z2[ROWS][64] = H1[ROWS][64] W2^T, 4 K-steps
 *             (b2 rides in column HC against the constant unit h1[HC] = 1)
 *   tcgen05.ld -> y = b3 + w3 . ReLU(z2) in FP32 on the CUDA cores (one
 *             tensor-core round trip fewer than an N = 16 output MMA,
 *             measured faster)
 *   -> softplus -> the coefficient o (nu_t = o * strain_gain in the caller)
 *
 * Thread t of the block owns row t: MMA h = t / 128 covers rows 128 h ..
 * 128 h + 127 in TMEM lanes 0..127 of columns 64 h .. 64 h + 63, and warp w
 * reads lanes 32 (w % 4) .. + 31, which are exactly its threads' rows.
 * One elected thread issues the MMAs; completion arrives on an mbarrier that
 * every warp polls with a bounded wait (on a timeout the warp reports an
 * error code and returns o = 0 so that the caller's state stays finite).
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
constexpr uint32_t W2_LBO = 128, W2_SBO = 1024;   /* K = 64: eight (also W3 and the hidden rows) */
constexpr int N3 = 16;                            /* the smallest N of an M = 128 MMA */
constexpr uint32_t W1_BYTES = NH * NIN * 2, W2_BYTES = NH * NH * 2, W3_BYTES = N3 * NH * 2;
/* device weight blob: W1 (row HC = e15), W2 (b2 folded into column HC) and
 * W3 (row 0 = w3, rows 1..15 zero) in the core-matrix layout as bf16, then
 * b3 (+ 3 pad) as FP32 */
constexpr uint32_t BLOB_W2 = W1_BYTES, BLOB_W3 = BLOB_W2 + W2_BYTES, BLOB_B3 = BLOB_W3 + W3_BYTES;
constexpr uint32_t BLOB_BYTES = BLOB_B3 + 16;
constexpr int SM_SMEM_BYTES = 228 * 1024; /* shared memory per SM */

template <int ROWS> struct InferSmem;

/* dynamic shared memory for a block of ROWS rows that holds InferSmem (plus
 * 1 KB of alignment slack) and is large enough that no more blocks than TMEM
 * can serve (512 columns) fit on one SM */
template <int ROWS> inline size_t infer_dyn_smem();

template <int ROWS> struct InferSmem {
    alignas(1024) unsigned char w1[W1_BYTES];
    alignas(1024) unsigned char w2[W2_BYTES];
    /* the layer-1 A operand (features, ROWS x 16 bf16) at the start, then
     * h1 over it (written only after the layer-1 MMA has read x) */
    alignas(1024) unsigned char a2[ROWS * NH * 2];
    alignas(16) float w3f[NH];
    float b3;
    alignas(8) uint64_t mbar;
    uint32_t tmem;
    uint32_t phase;
    /* a completion wait ran out: no further MMA is issued by this block,
     * and failed_parity is the completion still outstanding */
    uint32_t failed, failed_parity;
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
        reinterpret_cast<uint4*>(s.w2)[i] = src[BLOB_W2 / 16 + i];
    /* w3 = row 0 of the blob's output-layer B operand, as FP32 */
    if (t < NH) {
        const __nv_bfloat16 w = *reinterpret_cast<const __nv_bfloat16*>(blob + BLOB_W3 + tc::core_off(0, t, W2_LBO,
                                                                                                      W2_SBO));
        s.w3f[t] = __bfloat162float(w);
    }
    if (t == 0) {
        s.b3 = *reinterpret_cast<const float*>(blob + BLOB_B3);
        tc::mbar_init(&s.mbar, 1);
        s.phase = 0;
        s.failed = 0;
    }
    if (t < 32) tc::tmem_alloc(&s.tmem, tmem_cols<ROWS>());
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

/* After a wait that ran out, the MMA it waited for may still be running:
 * one thread waits for it once more (bounded) before the columns are freed */
template <int ROWS> __device__ __forceinline__ void infer_teardown(InferSmem<ROWS>& s) {
    tc::fence_before_sync();
    __syncthreads();
    if (s.failed && row_index() == 0) tc::mbar_wait(&s.mbar, s.failed_parity, 1u << 20);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (row_index() < 32) tc::tmem_dealloc(s.tmem, tmem_cols<ROWS>());
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

/* relu(z0), relu(z1) rounded to bf16 and packed (z0 in the low half): one
 * instruction per pair */
__device__ __forceinline__ uint32_t relu_bf16x2(uint32_t z0, uint32_t z1) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(__uint_as_float(z1)), "f"(__uint_as_float(z0)));
    return d;
}

/* every warp polls the mbarrier for the completion of the given parity
 * (no block barrier: a warp goes on to its TMEM reads as soon as it sees the
 * MMA done); returns false when the wait ran out.  The verdict is
 * warp-uniform, as the warp-collective tcgen05.ld after it needs.  No
 * parity is reused before every warp has passed its wait: the next MMA is
 * issued only behind the block barrier of infer_publish */
template <int ROWS> __device__ __forceinline__ bool infer_mma_wait(InferSmem<ROWS>& s, uint32_t parity) {
    const bool w = tc::mbar_wait(&s.mbar, parity, 1u << 20);
    const bool ok = __all_sync(0xffffffffu, w);
    tc::fence_after_sync();
    if (!ok && (threadIdx.x & 31) == 0) {
        s.failed = 1;
        s.failed_parity = parity;
    }
    return ok;
}

/* make this thread's shared-memory operand rows visible to the tensor core,
 * order its TMEM reads before the next MMA, and line the block up behind
 * the MMA issue */
__device__ __forceinline__ void infer_publish() {
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

/* the 64 accumulator columns of this thread's row through ReLU into bf16
 * A-operand rows of a2.  The loads run even after a failed wait (they are
 * valid TMEM reads); the caller then discards the row's result */
template <int ROWS> __device__ __forceinline__ void infer_epilogue(InferSmem<ROWS>& s, uint32_t ta, int t) {
    const uint32_t a2 = tc::smem_u32(s.a2);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        uint32_t r[16];
        tc::tmem_ld16(ta + 16 * c, r);
        tc::tmem_wait_ld();
        tc::tmem_fence_regs<16>(r);
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
            const uint32_t* v = r + 8 * hh;
            tc::sts128(a2 + tc::core_off(t, 16 * c + 8 * hh, W2_LBO, W2_SBO),
                       make_uint4(relu_bf16x2(v[0], v[1]), relu_bf16x2(v[2], v[3]), relu_bf16x2(v[4], v[5]),
                                  relu_bf16x2(v[6], v[7])));
        }
    }
}

/* D (+)= A B^T over K = 64 in four K-steps of 16, for each 128-row half */
template <int ROWS>
__device__ __forceinline__ void infer_mma_k64(uint32_t tmem, uint32_t a, const unsigned char* b, uint32_t id) {
#pragma unroll
    for (int h = 0; h < ROWS / 128; ++h)
#pragma unroll
        for (int kc = 0; kc < NH / 16; ++kc)
            tc::mma_bf16(tmem + 64 * h, tc::sdesc(a + h * 16 * W2_SBO + kc * 2 * W2_LBO, W2_LBO, W2_SBO),
                         tc::sdesc(tc::smem_u32(b) + kc * 2 * W2_LBO, W2_LBO, W2_SBO), id, kc > 0);
}

/* nu_t of this thread's row; x[16] are its features (FP32, x[15] = 1).
 * Returns -1 (block-uniform) once a completion wait of this block has run
 * out: the caller then leaves its loop and tears down */
template <int ROWS> __device__ __forceinline__ float infer_nu(InferSmem<ROWS>& s, const float x[NIN], int* err) {
    static_assert(ROWS == 128 || ROWS == 256, "one or two M=128 MMAs per block");
    const int t = row_index(), warp = t >> 5;
    /* A of layer 1 (at the start of a2) */
    const uint32_t a1 = tc::smem_u32(s.a2);
    tc::sts128(a1 + tc::core_off(t, 0, W1_LBO, W1_SBO),
               make_uint4(pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(x[4], x[5]), pack_bf16(x[6], x[7])));
    tc::sts128(a1 + tc::core_off(t, 8, W1_LBO, W1_SBO), make_uint4(pack_bf16(x[8], x[9]), pack_bf16(x[10], x[11]),
                                                                   pack_bf16(x[12], x[13]), pack_bf16(x[14], x[15])));
    infer_publish();
    if (s.failed) return -1.f;
    /* the two completions of a call have parities ph, ph ^ 1, so every
     * call starts at the parity set up by infer_setup */
    const uint32_t ph = s.phase;
    const uint32_t id = tc::idesc_bf16_f32(128, NH);
    if (t == 0) {
#pragma unroll
        for (int h = 0; h < ROWS / 128; ++h)
            tc::mma_bf16(s.tmem + 64 * h, tc::sdesc(a1 + h * 16 * W1_SBO, W1_LBO, W1_SBO),
                         tc::sdesc(tc::smem_u32(s.w1), W1_LBO, W1_SBO), id, 0);
        tc::mma_commit(&s.mbar);
    }
    bool ok = infer_mma_wait(s, ph);
    const uint32_t ta = s.tmem + (uint32_t((warp & 3) * 32) << 16) + uint32_t(warp >> 2) * 64;
    /* layer 1 epilogue: relu -> h1 */
    infer_epilogue<ROWS>(s, ta, t);
    infer_publish();
    if (s.failed) return -1.f;
    if (t == 0) {
        infer_mma_k64<ROWS>(s.tmem, tc::smem_u32(s.a2), s.w2, id);
        tc::mma_commit(&s.mbar);
    }
    ok = infer_mma_wait(s, ph ^ 1u) && ok;
    /* output layer: y = b3 + w3 . relu(z2) in FP32, from the layer-2
     * accumulators (two completions per call: parities ph, ph ^ 1) */
    float y = s.b3;
    const uint32_t w3 = tc::smem_u32(s.w3f);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        uint32_t r[16];
        tc::tmem_ld16(ta + 16 * c, r);
        tc::tmem_wait_ld();
        tc::tmem_fence_regs<16>(r);
#pragma unroll
        for (int j = 0; j < 16; j += 4) {
            const float4 w = tc::lds128f(w3 + 4 * (16 * c + j));
            y = fmaf(w.x, fmaxf(__uint_as_float(r[j]), 0.f), y);
            y = fmaf(w.y, fmaxf(__uint_as_float(r[j + 1]), 0.f), y);
            y = fmaf(w.z, fmaxf(__uint_as_float(r[j + 2]), 0.f), y);
            y = fmaf(w.w, fmaxf(__uint_as_float(r[j + 3]), 0.f), y);
        }
    }
    /* two completions per call leave the parity of the next one at ph */
    if (!ok) {
        if ((t & 31) == 0) atomicExch(err, 2);
        return 0.f;
    }
    const float sp = y > 20.f ? y : log1pf(__expf(y));
    return NU_SCALE * sp;
}

#endif /* __CUDA_ARCH__ */

}  // namespace sgs
}  // namespace lbm
