/* Training and evaluation kernels of the learned subgrid closure, and the
 * self-check of the tensor-core path.
 *
 * k_mlp_grad fuses forward, loss and backward for a tile of 128 samples per
 * block: every thread carries one sample through both layers (weights in
 * shared memory), the per-sample activations and deltas go to shared memory,
 * and the weight gradients are then accumulated over the tile as small
 * shared-memory GEMMs into per-thread registers.  Each block writes its
 * partial gradient; k_mlp_adam sums the partials in a fixed order (so runs
 * are reproducible) and applies one Adam step.  Loss: mean squared error of
 * o / NU_SCALE, o the network's coefficient (the eddy viscosity is
 * o * strain_gain in the collision).
 */
#include <cstdint>
#include <cuda_bf16.h>

#include "lbm_kernels.cuh"
#include "sgs_infer.cuh"
#include "sgs_mlp.cuh"
#include "tc_sm103.cuh"

namespace lbm {
namespace sgs {

constexpr int GT = 128;        /* samples (threads) per block */
constexpr int RS = NH + 1;     /* padded row stride of the per-sample arrays */

/* ReLU and its slope (0 at z = 0) */
__device__ __forceinline__ float relu(float z, float& dg) {
    dg = z > 0.f ? 1.f : 0.f;
    return z > 0.f ? z : 0.f;
}
__device__ __forceinline__ float softplus(float y) { return y > 20.f ? y : log1pf(expf(y)); }
__device__ __forceinline__ float sigmoid(float y) { return 1.f / (1.f + expf(-y)); }

struct GradSmem {
    float W1[NH * NIN], W2[NH * NH], b2[NH], w3[NH], b3;
    float X[GT * NIN];
    float H1[GT * RS], Z2[GT * RS], Z1[GT * RS], H2[GT * RS];
    float DY[GT];
};

/* grad_part[block][NPARAM + 1]: the block's gradient sum and loss sum over
 * its samples (idx[i] selects sample i of the batch, or i itself when idx is
 * null); the loss is scaled by 1/n_total */
__global__ void __launch_bounds__(GT) k_mlp_grad(const float* __restrict__ params, const float* __restrict__ X,
                                                 const float* __restrict__ T, const int* __restrict__ idx, int n,
                                                 float inv_n, float* __restrict__ grad_part) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    GradSmem& s = *reinterpret_cast<GradSmem*>(smem_raw);
    const int t = threadIdx.x;
    for (int i = t; i < NH * NIN; i += GT) s.W1[i] = params[OFF_W1 + i];
    for (int i = t; i < NH * NH; i += GT) s.W2[i] = params[OFF_W2 + i];
    if (t < NH) {
        s.b2[t] = params[OFF_B2 + t];
        s.w3[t] = params[OFF_W3 + t];
    }
    if (t == 0) s.b3 = params[OFF_B3];
    /* register accumulators: dW2 rows j = t/2, columns (t&1)*32 .. +32;
     * dW1 row t/2, columns (t&1)*8 .. +8; db2 / dw3 by thread */
    float gW2[32], gW1[8], gb = 0.f, gl = 0.f, gd3 = 0.f;
#pragma unroll
    for (int i = 0; i < 32; ++i) gW2[i] = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) gW1[i] = 0.f;
    const int jr = t >> 1, c2 = (t & 1) * 32, c1 = (t & 1) * 8;
    __syncthreads();

    for (int base = blockIdx.x * GT; base < n; base += gridDim.x * GT) {
        const int i = base + t;
        const bool live = i < n;
        const int si = live ? (idx ? idx[i] : i) : 0;
        float x[NIN];
#pragma unroll
        for (int k = 0; k < NIN; ++k) x[k] = live ? X[size_t(si) * NIN + k] : 0.f;
#pragma unroll
        for (int k = 0; k < NIN; ++k) s.X[t * NIN + k] = x[k];
        /* layer 1 */
        float* h1 = s.H1 + t * RS;
        float* z1 = s.Z1 + t * RS;
        for (int j = 0; j < NH; ++j) {
            float z = 0.f;
#pragma unroll
            for (int k = 0; k < NIN; ++k) z = fmaf(s.W1[j * NIN + k], x[k], z);
            float dg;
            h1[j] = relu(z, dg);
            z1[j] = dg; /* keep relu'(z1) */
        }
        h1[HC] = 1.f; /* the constant unit */
        z1[HC] = 0.f;
        /* layer 2 + output */
        float* z2 = s.Z2 + t * RS;
        float* h2 = s.H2 + t * RS;
        float y = s.b3;
        for (int j = 0; j < NH; ++j) {
            float z = s.b2[j];
            for (int k = 0; k < NH; ++k) z = fmaf(s.W2[j * NH + k], h1[k], z);
            float dg;
            h2[j] = relu(z, dg);
            z2[j] = dg;
            y = fmaf(s.w3[j], h2[j], y);
        }
        const float out = softplus(y);
        const float tgt = live ? T[si] * (1.f / NU_SCALE) : 0.f;
        const float err = live ? out - tgt : 0.f;
        gl += err * err * inv_n;
        const float dy = 2.f * err * inv_n * sigmoid(y);
        s.DY[t] = dy;
        gd3 += dy;
        /* dz2 = dy w3 * relu'(z2), in place */
        for (int j = 0; j < NH; ++j) z2[j] = dy * s.w3[j] * z2[j];
        /* dz1 = (W2^T dz2) * relu'(z1), in place */
        for (int k = 0; k < NH; ++k) {
            float a = 0.f;
            for (int j = 0; j < NH; ++j) a = fmaf(s.W2[j * NH + k], z2[j], a);
            z1[k] = a * z1[k];
        }
        __syncthreads();
        /* weight gradients over the tile */
        for (int q = 0; q < GT; ++q) {
            const float d2 = s.Z2[q * RS + jr];
            const float* hq = s.H1 + q * RS + c2;
#pragma unroll
            for (int k = 0; k < 32; ++k) gW2[k] = fmaf(d2, hq[k], gW2[k]);
            const float d1 = s.Z1[q * RS + jr];
            const float* xq = s.X + q * NIN + c1;
#pragma unroll
            for (int k = 0; k < 8; ++k) gW1[k] = fmaf(d1, xq[k], gW1[k]);
            if (t < NH) gb += s.Z2[q * RS + t];
            else gb += s.DY[q] * s.H2[q * RS + (t - NH)];
        }
        __syncthreads();
    }
    /* loss and db3: block sums through shared memory (DY and H2 are free now) */
    s.DY[t] = gl;
    s.H2[t] = gd3;
    __syncthreads();
    float* out = grad_part + size_t(blockIdx.x) * (NPARAM + 1);
#pragma unroll
    for (int k = 0; k < 32; ++k) out[OFF_W2 + jr * NH + c2 + k] = gW2[k];
#pragma unroll
    for (int k = 0; k < 8; ++k) out[OFF_W1 + jr * NIN + c1 + k] = gW1[k];
    if (t < NH) out[OFF_B2 + t] = gb;
    else out[OFF_W3 + (t - NH)] = gb;
    if (t == 0) {
        float l = 0.f, d = 0.f;
        for (int q = 0; q < GT; ++q) {
            l += s.DY[q];
            d += s.H2[q];
        }
        out[NPARAM] = l;
        out[OFF_B3] = d;
    }
}

/* sum the block partials in block order; optionally one Adam step */
__global__ void k_mlp_adam(const float* __restrict__ grad_part, int nblocks, float* __restrict__ params,
                           float* __restrict__ m, float* __restrict__ v, float* __restrict__ grad_out,
                           float* __restrict__ loss_out, float lr, float b1, float b2, float eps, int step) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > NPARAM) return;
    float g = 0.f;
    for (int b = 0; b < nblocks; ++b) g += grad_part[size_t(b) * (NPARAM + 1) + p];
    if (p == NPARAM) {
        if (loss_out) *loss_out = g;
        return;
    }
    if (grad_out) grad_out[p] = g;
    if (step > 0) {
        const float mm = b1 * m[p] + (1.f - b1) * g;
        const float vv = b2 * v[p] + (1.f - b2) * g * g;
        m[p] = mm;
        v[p] = vv;
        const float mh = mm / (1.f - powf(b1, float(step)));
        const float vh = vv / (1.f - powf(b2, float(step)));
        params[p] -= lr * mh / (sqrtf(vh) + eps);
    }
}

/* nu_t for n samples (FP32, CUDA cores): the training-side forward */
__global__ void __launch_bounds__(GT) k_mlp_predict(const float* __restrict__ params, const float* __restrict__ X,
                                                    int n, float* __restrict__ nu) {
    __shared__ float W1[NH * NIN], W2[NH * NH], b2[NH], w3[NH];
    const int t = threadIdx.x;
    for (int i = t; i < NH * NIN; i += GT) W1[i] = params[OFF_W1 + i];
    for (int i = t; i < NH * NH; i += GT) W2[i] = params[OFF_W2 + i];
    if (t < NH) {
        b2[t] = params[OFF_B2 + t];
        w3[t] = params[OFF_W3 + t];
    }
    const float b3 = params[OFF_B3];
    __syncthreads();
    for (int i = blockIdx.x * GT + t; i < n; i += gridDim.x * GT) {
        float x[NIN], h1[NH];
#pragma unroll
        for (int k = 0; k < NIN; ++k) x[k] = X[size_t(i) * NIN + k];
        for (int j = 0; j < NH; ++j) {
            float z = 0.f;
#pragma unroll
            for (int k = 0; k < NIN; ++k) z = fmaf(W1[j * NIN + k], x[k], z);
            h1[j] = fmaxf(z, 0.f);
        }
        h1[HC] = 1.f;
        float y = b3;
        for (int j = 0; j < NH; ++j) {
            float z = b2[j];
            for (int k = 0; k < NH; ++k) z = fmaf(W2[j * NH + k], h1[k], z);
            y = fmaf(w3[j], fmaxf(z, 0.f), y);
        }
        nu[i] = NU_SCALE * softplus(y);
    }
}

/* ---- tensor-core self-check: D[128][64] = A[128][K] B[64][K]^T, K = 16 * kc */
__global__ void __launch_bounds__(128) k_tc_selftest(const __nv_bfloat16* __restrict__ A,
                                                     const __nv_bfloat16* __restrict__ B, int kc,
                                                     float* __restrict__ D, int* __restrict__ err) {
    __shared__ __align__(1024) unsigned char sa[128 * 64 * 2];
    __shared__ __align__(1024) unsigned char sb[64 * 64 * 2];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tslot;
    const int t = threadIdx.x, warp = t >> 5;
    const int K = 16 * kc;
    const uint32_t lbo = 128, sbo = uint32_t(K / 8) * 128;
    /* operands into the core-matrix layout, 16 bytes (8 bf16) at a time */
    for (int k8 = 0; k8 < K / 8; ++k8) {
        *reinterpret_cast<uint4*>(sa + tc::core_off(t, k8 * 8, lbo, sbo)) =
            *reinterpret_cast<const uint4*>(A + size_t(t) * K + k8 * 8);
        if (t < 64)
            *reinterpret_cast<uint4*>(sb + tc::core_off(t, k8 * 8, lbo, sbo)) =
                *reinterpret_cast<const uint4*>(B + size_t(t) * K + k8 * 8);
    }
#if defined(__CUDA_ARCH__)
    if (t == 0) tc::mbar_init(&mbar, 1);
    if (warp == 0) tc::tmem_alloc(&tslot, 64);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tm = tslot;
    if (t == 0) {
        const uint32_t id = tc::idesc_bf16_f32(128, 64);
        for (int c = 0; c < kc; ++c)
            tc::mma_bf16(tm, tc::sdesc(tc::smem_u32(sa) + c * 2 * lbo, lbo, sbo),
                         tc::sdesc(tc::smem_u32(sb) + c * 2 * lbo, lbo, sbo), id, c > 0);
        tc::mma_commit(&mbar);
    }
    const bool ok = __syncthreads_and(tc::mbar_wait(&mbar, 0, 1u << 22));
    tc::fence_after_sync();
    if (ok) {
        uint32_t r[64];
        const uint32_t ta = tm + (uint32_t(warp * 32) << 16);
#pragma unroll
        for (int c = 0; c < 4; ++c) tc::tmem_ld16(ta + 16 * c, r + 16 * c);
        tc::tmem_wait_ld();
        tc::tmem_fence_regs<64>(r);
#pragma unroll
        for (int c = 0; c < 64; ++c) D[size_t(t) * 64 + c] = __uint_as_float(r[c]);
    } else if (t == 0) {
        atomicExch(err, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tm, 64);
#endif
}

/* nu_t of n samples through the tensor-core inference path (the one the
 * collide kernels use): persistent blocks of 128 rows */
__global__ void __launch_bounds__(128) k_mlp_predict_tc(const unsigned char* __restrict__ blob,
                                                        const float* __restrict__ X, int n, float* __restrict__ nu,
                                                        int* __restrict__ err) {
    extern __shared__ unsigned char dsm[];
    InferSmem<128>& s =
        *reinterpret_cast<InferSmem<128>*>((reinterpret_cast<uintptr_t>(dsm) + 1023) & ~uintptr_t(1023));
#if defined(__CUDA_ARCH__)
    infer_setup<128>(s, blob);
    for (int base = blockIdx.x * 128; base < n; base += gridDim.x * 128) {
        const int i = base + threadIdx.x;
        float x[NIN];
#pragma unroll
        for (int k = 0; k < NIN; ++k) x[k] = i < n ? X[size_t(i) * NIN + k] : 0.f;
        const float v = infer_nu<128>(s, x, err);
        if (v < 0.f) break; /* a tensor-core wait ran out (block-uniform) */
        if (i < n) nu[i] = v;
    }
    infer_teardown<128>(s);
#endif
}

}  // namespace sgs

/* ---- launchers */
int mlp_grad_blocks(int n) {
    int b = (n + sgs::GT - 1) / sgs::GT;
    return b < 1 ? 1 : (b > 152 * 2 ? 152 * 2 : b);
}

cudaError_t launch_mlp_grad(const float* params, const float* X, const float* T, const int* idx, int n,
                            float* grad_part, int nblocks, cudaStream_t s) {
    const size_t sm = sizeof(sgs::GradSmem);
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(sgs::k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const float inv_n = 1.f / float(n > 0 ? n : 1);
    sgs::k_mlp_grad<<<nblocks, sgs::GT, sm, s>>>(params, X, T, idx, n, inv_n, grad_part);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(const float* grad_part, int nblocks, float* params, float* m, float* v, float* grad_out,
                            float* loss_out, float lr, int step, cudaStream_t s) {
    const int n = sgs::NPARAM + 1;
    sgs::k_mlp_adam<<<(n + 255) / 256, 256, 0, s>>>(grad_part, nblocks, params, m, v, grad_out, loss_out, lr, 0.9f,
                                                    0.999f, 1e-8f, step);
    return cudaGetLastError();
}

cudaError_t launch_mlp_predict(const float* params, const float* X, int n, float* nu, cudaStream_t s) {
    int b = (n + sgs::GT - 1) / sgs::GT;
    if (b > 152 * 8) b = 152 * 8;
    if (b < 1) b = 1;
    sgs::k_mlp_predict<<<b, sgs::GT, 0, s>>>(params, X, n, nu);
    return cudaGetLastError();
}

cudaError_t launch_mlp_predict_tc(const void* blob, const float* X, int n, float* nu, int* err, cudaStream_t s) {
    int b = (n + 127) / 128;
    if (b > 152 * 4) b = 152 * 4;
    if (b < 1) b = 1;
    const size_t smem = sgs::infer_dyn_smem<128>();
    static cudaError_t attr = cudaErrorNotReady;
    if (attr == cudaErrorNotReady)
        attr = cudaFuncSetAttribute(sgs::k_mlp_predict_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (attr != cudaSuccess) return attr;
    TmemLane lane(s);
    if (lane.status() != cudaSuccess) return lane.status();
    sgs::k_mlp_predict_tc<<<b, 128, smem, lane.stream()>>>((const unsigned char*)blob, X, n, nu, err);
    return cudaGetLastError();
}

cudaError_t launch_tc_selftest(const void* A, const void* B, int kc, float* D, int* err, cudaStream_t s) {
    if (kc < 1 || kc > 4) return cudaErrorInvalidValue;
    TmemLane lane(s);
    if (lane.status() != cudaSuccess) return lane.status();
    sgs::k_tc_selftest<<<1, 128, 0, lane.stream()>>>((const __nv_bfloat16*)A, (const __nv_bfloat16*)B, kc, D, err);
    return cudaGetLastError();
}

}  // namespace lbm
