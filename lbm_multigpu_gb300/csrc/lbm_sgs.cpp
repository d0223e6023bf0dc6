/*
 * lbm_sgs.cpp -- host side of the learned subgrid closure behind the C ABI:
 * parameter initialisation, the training loop (fused gradient kernel + Adam
 * kernel per mini-batch), evaluation and the tensor-core self-check.
 *
 * None of this has a counterpart in the reference, whose LES is the
 * constant-Cs Smagorinsky model (LRTurbTest/LRMultiGPU7.cu:683-685); the
 * closure it trains replaces that model in the collision.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "lbm_kernels.cuh"
#include "sgs_infer.cuh"
#include "sgs_mlp.cuh"
#include "tc_sm103.cuh"

using namespace lbm;

namespace {

#define SGS_TRY(call, what)                                                  \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) return set_error(LBM_ERR_CUDA, what, e_);     \
    } while (0)

/* splitmix64: a small, portable, seedable generator for initialisation and
 * mini-batch shuffles (identical on every host) */
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return double(next() >> 11) * (1.0 / 9007199254740992.0); }
};

/* device scratch that frees itself */
template <class T> struct DevBuf {
    T* p = nullptr;
    ~DevBuf() { cudaFree(p); }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, n * sizeof(T)); }
};

uint16_t bf16_rne(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7F800000u) == 0x7F800000u) return uint16_t(u >> 16); /* inf / nan kept */
    u += 0x7FFFu + ((u >> 16) & 1u);
    return uint16_t(u >> 16);
}

}  // namespace

namespace lbm {
void mlp_make_blob(const float* P, unsigned char* blob) {
    std::memset(blob, 0, sgs::BLOB_BYTES);
    auto put = [&](unsigned char* base, uint32_t off, float v) {
        const uint16_t b = bf16_rne(v);
        std::memcpy(base + off, &b, 2);
    };
    /* W1 with row HC = e15: the MMA makes the constant unit relu(x15) = 1 */
    for (int j = 0; j < sgs::NH; ++j)
        for (int k = 0; k < sgs::NIN; ++k)
            put(blob, tc::core_off(j, k, sgs::W1_LBO, sgs::W1_SBO),
                j == sgs::HC ? float(k == sgs::NIN - 1) : P[sgs::OFF_W1 + j * sgs::NIN + k]);
    /* W2 with b2 folded into column HC */
    for (int j = 0; j < sgs::NH; ++j)
        for (int k = 0; k < sgs::NH; ++k)
            put(blob + sgs::BLOB_W2, tc::core_off(j, k, sgs::W2_LBO, sgs::W2_SBO),
                P[sgs::OFF_W2 + j * sgs::NH + k] + (k == sgs::HC ? P[sgs::OFF_B2 + j] : 0.f));
    /* the output layer as the B operand of an N = 16 MMA: row 0 = w3 */
    for (int k = 0; k < sgs::NH; ++k)
        put(blob + sgs::BLOB_W3, tc::core_off(0, k, sgs::W2_LBO, sgs::W2_SBO), P[sgs::OFF_W3 + k]);
    std::memcpy(blob + sgs::BLOB_B3, &P[sgs::OFF_B3], 4);
}
}  // namespace lbm

extern "C" {

int lbm_mlp_param_count(void) { return sgs::NPARAM; }

size_t lbm_mlp_blob_bytes(void) { return sgs::BLOB_BYTES; }

int lbm_mlp_make_blob(const float* params, unsigned char* blob) {
    if (!params || !blob) return set_error(LBM_ERR_ARG, "null argument", cudaSuccess);
    mlp_make_blob(params, blob);
    return LBM_OK;
}

int lbm_mlp_init_params(uint32_t seed, float* params) {
    if (!params) return set_error(LBM_ERR_ARG, "params is null", cudaSuccess);
    Rng r(seed);
    /* uniform(-a, a): He (a = sqrt(6 / fan_in)) for the ReLU layers,
     * Glorot for the output */
    auto uniform = [&](int off, int rows, int ncols, double a) {
        for (int j = 0; j < rows; ++j)
            for (int k = 0; k < ncols; ++k) params[off + j * ncols + k] = float((2 * r.uniform() - 1) * a);
    };
    uniform(sgs::OFF_W1, sgs::NH, sgs::NIN, std::sqrt(6.0 / (sgs::NIN - 1)));
    for (int j = 0; j < sgs::NH; ++j) params[sgs::OFF_W1 + j * sgs::NIN + sgs::NIN - 1] = 0.f; /* b1 */
    for (int k = 0; k < sgs::NIN; ++k) params[sgs::OFF_W1 + sgs::HC * sgs::NIN + k] = k == sgs::NIN - 1; /* unused */
    uniform(sgs::OFF_W2, sgs::NH, sgs::NH, std::sqrt(6.0 / sgs::NH));
    for (int j = 0; j < sgs::NH; ++j) params[sgs::OFF_B2 + j] = 0.f;
    uniform(sgs::OFF_W3, 1, sgs::NH, std::sqrt(6.0 / (sgs::NH + 1)));
    params[sgs::OFF_B3] = 0.f;
    return LBM_OK;
}

int lbm_mlp_grad(const float* d_params, const float* d_X, const float* d_T, int n, float* d_grad, float* d_loss,
                 void* stream) {
    if (!d_params || !d_X || !d_T || !d_grad || n <= 0) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = mlp_grad_blocks(n);
    DevBuf<float> part;
    SGS_TRY(part.alloc(size_t(nb) * (sgs::NPARAM + 1)), "cudaMalloc(gradient partials)");
    SGS_TRY(launch_mlp_grad(d_params, d_X, d_T, nullptr, n, part.p, nb, s), "gradient launch");
    SGS_TRY(launch_mlp_adam(part.p, nb, nullptr, nullptr, nullptr, d_grad, d_loss, 0.f, 0, s), "reduce launch");
    SGS_TRY(cudaStreamSynchronize(s), "gradient");
    return LBM_OK;
}

int lbm_mlp_predict(const float* d_params, const float* d_X, int n, float* d_nu, void* stream) {
    if (!d_params || !d_X || !d_nu || n < 0) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    if (n == 0) return LBM_OK;
    SGS_TRY(launch_mlp_predict(d_params, d_X, n, d_nu, (cudaStream_t)stream), "predict launch");
    return LBM_OK;
}

int lbm_mlp_train(const float* d_X, const float* d_T, int n, int batch, int steps, float lr, uint32_t seed,
                  float* params, float* loss_hist, void* stream) {
    if (!d_X || !d_T || !params || n <= 0 || batch <= 0 || steps < 0 || !(lr > 0))
        return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    if (batch > n) batch = n;
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = mlp_grad_blocks(batch);
    DevBuf<float> P, M, V, part, loss;
    DevBuf<int> idx;
    SGS_TRY(P.alloc(sgs::NPARAM), "cudaMalloc");
    SGS_TRY(M.alloc(sgs::NPARAM), "cudaMalloc");
    SGS_TRY(V.alloc(sgs::NPARAM), "cudaMalloc");
    SGS_TRY(part.alloc(size_t(nb) * (sgs::NPARAM + 1)), "cudaMalloc");
    SGS_TRY(loss.alloc(size_t(steps > 0 ? steps : 1)), "cudaMalloc");
    SGS_TRY(idx.alloc(size_t(n)), "cudaMalloc");
    SGS_TRY(cudaMemcpyAsync(P.p, params, sgs::NPARAM * sizeof(float), cudaMemcpyHostToDevice, s), "params upload");
    SGS_TRY(cudaMemsetAsync(M.p, 0, sgs::NPARAM * sizeof(float), s), "memset");
    SGS_TRY(cudaMemsetAsync(V.p, 0, sgs::NPARAM * sizeof(float), s), "memset");
    /* epochs over a seeded permutation; one pinned-free upload per epoch */
    Rng r(seed);
    std::vector<int> perm(n);
    for (int i = 0; i < n; ++i) perm[i] = i;
    int pos = n;
    for (int st = 0; st < steps; ++st) {
        if (pos + batch > n) {
            for (int i = n - 1; i > 0; --i) std::swap(perm[i], perm[int(r.next() % uint64_t(i + 1))]);
            SGS_TRY(cudaMemcpyAsync(idx.p, perm.data(), size_t(n) * sizeof(int), cudaMemcpyHostToDevice, s),
                    "index upload");
            SGS_TRY(cudaStreamSynchronize(s), "index upload");
            pos = 0;
        }
        SGS_TRY(launch_mlp_grad(P.p, d_X, d_T, idx.p + pos, batch, part.p, nb, s), "gradient launch");
        SGS_TRY(launch_mlp_adam(part.p, nb, P.p, M.p, V.p, nullptr, loss.p + st, lr, st + 1, s), "Adam launch");
        pos += batch;
    }
    SGS_TRY(cudaMemcpyAsync(params, P.p, sgs::NPARAM * sizeof(float), cudaMemcpyDeviceToHost, s), "params read");
    if (loss_hist && steps > 0)
        SGS_TRY(cudaMemcpyAsync(loss_hist, loss.p, size_t(steps) * sizeof(float), cudaMemcpyDeviceToHost, s),
                "loss read");
    SGS_TRY(cudaStreamSynchronize(s), "training");
    return LBM_OK;
}

int lbm_mlp_predict_tc(const float* params, const float* d_X, int n, float* d_nu, void* stream) {
    if (!params || !d_X || !d_nu || n < 0) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    if (n == 0) return LBM_OK;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<unsigned char> blob(sgs::BLOB_BYTES);
    mlp_make_blob(params, blob.data());
    DevBuf<unsigned char> d;
    DevBuf<int> err;
    SGS_TRY(d.alloc(blob.size()), "cudaMalloc");
    SGS_TRY(err.alloc(1), "cudaMalloc");
    SGS_TRY(cudaMemcpyAsync(d.p, blob.data(), blob.size(), cudaMemcpyHostToDevice, s), "blob upload");
    SGS_TRY(cudaMemsetAsync(err.p, 0, sizeof(int), s), "memset");
    SGS_TRY(launch_mlp_predict_tc(d.p, d_X, n, d_nu, err.p, s), "tensor-core predict launch");
    int e = 0;
    SGS_TRY(cudaMemcpyAsync(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost, s), "read");
    SGS_TRY(cudaStreamSynchronize(s), "tensor-core predict");
    if (e) return set_error(LBM_ERR_CUDA, "tensor-core inference: an MMA completion wait ran out", cudaSuccess);
    return LBM_OK;
}

int lbm_tc_selftest(int kc, const uint16_t* A, const uint16_t* B, float* D) {
    if (kc < 1 || kc > 4 || !A || !B || !D) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    const int K = 16 * kc;
    DevBuf<uint16_t> dA, dB;
    DevBuf<float> dD;
    DevBuf<int> err;
    SGS_TRY(dA.alloc(size_t(128) * K), "cudaMalloc");
    SGS_TRY(dB.alloc(size_t(64) * K), "cudaMalloc");
    SGS_TRY(dD.alloc(size_t(128) * 64), "cudaMalloc");
    SGS_TRY(err.alloc(1), "cudaMalloc");
    SGS_TRY(cudaMemcpy(dA.p, A, size_t(128) * K * 2, cudaMemcpyHostToDevice), "upload");
    SGS_TRY(cudaMemcpy(dB.p, B, size_t(64) * K * 2, cudaMemcpyHostToDevice), "upload");
    SGS_TRY(cudaMemset(err.p, 0, sizeof(int)), "memset");
    SGS_TRY(cudaMemset(dD.p, 0, size_t(128) * 64 * 4), "memset");
    SGS_TRY(launch_tc_selftest(dA.p, dB.p, kc, dD.p, err.p, 0), "self-test launch");
    SGS_TRY(cudaDeviceSynchronize(), "self-test");
    int e = 0;
    SGS_TRY(cudaMemcpy(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost), "read");
    SGS_TRY(cudaMemcpy(D, dD.p, size_t(128) * 64 * 4, cudaMemcpyDeviceToHost), "read");
    if (e) return set_error(LBM_ERR_CUDA, "tensor-core self-test: the MMA completion wait ran out", cudaSuccess);
    return LBM_OK;
}

}  // extern "C"
