/* Blackwell (sm_103a) tensor-core building blocks in inline PTX: tensor
 * memory allocation, tcgen05.mma of kind::f16 (BF16 operands, FP32
 * accumulator) with both operands in shared memory, completion through an
 * mbarrier, and tcgen05.ld of the accumulator back to registers.
 *
 * Operand layout (no swizzle, K-major): the tensor core reads a matrix of R
 * rows by K bf16 as "core matrices" of 8 rows x 16 bytes (8 x 8 bf16, 128
 * contiguous bytes, row r at byte 16 r).  Core matrix (i, j) -- rows 8i..8i+7,
 * columns 8j..8j+7 -- sits at byte  i * SBO + j * LBO  from the start address:
 * LBO steps along K, SBO along the rows.  core_off() gives the byte offset of
 * element (row, k) in that layout.
 *
 * Every wait is bounded: a wait that runs out reports failure to the caller,
 * which records an error code and skips the dependent work.
 */
#pragma once
#include <cstdint>

namespace lbm {
namespace tc {

__host__ __device__ constexpr uint32_t core_off(uint32_t row, uint32_t k, uint32_t lbo, uint32_t sbo) {
    return (row >> 3) * sbo + (k >> 3) * lbo + (row & 7) * 16 + (k & 7) * 2;
}

/* instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator, BF16 A
 * and B, both K-major, dense, M x N tile */
__host__ __device__ constexpr uint32_t idesc_bf16_f32(uint32_t M, uint32_t N) {
    return (1u << 4)                /* D format: F32 */
           | (1u << 7)              /* A format: BF16 */
           | (1u << 10)             /* B format: BF16 */
           | ((N >> 3) << 17)       /* N / 8 */
           | ((M >> 4) << 24);      /* M / 16 */
}

#if defined(__CUDA_ARCH__)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

/* shared-memory matrix descriptor: start, leading (K) and stride (row-group)
 * byte offsets, no swizzle */
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= uint64_t((saddr & 0x3FFFFu) >> 4);
    d |= uint64_t((lbo >> 4) & 0x3FFFu) << 16;
    d |= uint64_t((sbo >> 4) & 0x3FFFu) << 32;
    d |= uint64_t(1) << 46; /* descriptor version of tcgen05 */
    return d;
}

/* 16 bytes to a shared-memory address (32-bit shared window) */
__device__ __forceinline__ void sts128(uint32_t saddr, uint4 v) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(saddr), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
                 : "memory");
}

/* 16 bytes from a shared-memory address as four floats */
__device__ __forceinline__ float4 lds128f(uint32_t saddr) {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(saddr));
    return v;
}

/* one warp allocates ncols (power of two >= 32) TMEM columns; the base
 * address lands in *slot (shared memory) */
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
/* generic-proxy shared-memory stores become visible to the tensor core */
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

/* D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread */
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

/* the mbarrier completes once every tcgen05.mma issued so far by this thread
 * has finished */
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

/* wait for the phase with the given parity to complete; false after
 * max_iter polls */
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t max_iter) {
    const uint32_t a = smem_u32(mbar);
    for (uint32_t i = 0; i < max_iter; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

/* 16 consecutive 32-bit accumulator columns of this thread's TMEM lane; the
 * registers are valid only after tmem_wait_ld() and tmem_fence_regs() */
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
/* one 32-bit accumulator column of this thread's TMEM lane */
__device__ __forceinline__ void tmem_ld1(uint32_t taddr, uint32_t* r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(r[0]) : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
/* ties each register to a point after the wait, so no use moves above it */
template <int N> __device__ __forceinline__ void tmem_fence_regs(uint32_t* r) {
#pragma unroll
    for (int i = 0; i < N; ++i) asm volatile("" : "+r"(r[i]));
}

#endif /* __CUDA_ARCH__ */

}  // namespace tc
}  // namespace lbm
