/*
 * lbm_noalloc.cu -- the body-force reduction for callers that cannot
 * allocate device memory.
 *
 * lbm_body_force_f32 needs a scratch buffer for its per-block partial sums,
 * which the caller allocates.  Some callers cannot do that: a host framework
 * that has already reserved the device's memory for its own allocator (a
 * cudaMalloc from a plugin then fails or fragments that pool), a real-time
 * loop that must not pay cudaMalloc's latency and implicit device-wide
 * synchronisation, or a plugin host whose rules forbid allocation calls.
 * lbm_body_force_f32_noalloc gives them the same reduction with its scratch in
 * a fixed array of this library's own device memory, reserved when the library
 * is loaded: NOALLOC_SCRATCH_DOUBLES doubles (32 KiB) on every device the
 * library is used on, held until the process exits.
 */
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/lbm_gb300.h"
#include "lbm_kernels.cuh"

namespace {

/* partial sums of the reduction: 3 doubles per block of the scan kernel */
constexpr int NOALLOC_SCRATCH_DOUBLES = 4096;
static __device__ __align__(256) double g_force_scratch[NOALLOC_SCRATCH_DOUBLES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
double* g_scratch_addr[MAX_DEVICES] = {nullptr};

/* The device address of g_force_scratch on the current device.  In host
 * code the array's name only stands in for the symbol: a kernel given it
 * would fault, or on a system where the GPU can reach host memory silently
 * use the wrong memory.  So the address is looked up once per device, with
 * that device current, and reused.  A cudaDeviceReset (or anything else that
 * destroys the device's primary context) reloads the module and can move
 * the array; the cached address is then stale, so this entry point must not
 * be used on a device after it has been reset in the same process. */
int scratch_on_current_device(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return lbm::set_error(LBM_ERR_CUDA, "cudaGetDevice", e);
    if (dev < 0 || dev >= MAX_DEVICES) return lbm::set_error(LBM_ERR_ARG, "device index beyond 63", cudaSuccess);
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_force_scratch);
        if (e != cudaSuccess) return lbm::set_error(LBM_ERR_CUDA, "cudaGetSymbolAddress(g_force_scratch)", e);
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return LBM_OK;
}

}  // namespace

extern "C" int lbm_body_force_f32_noalloc(const float* fA, const uint8_t* mask, int nx, int ny, int nz, int pitch,
                                          double* force_out, void* cuda_stream) {
    if (!fA || !mask || !force_out) return lbm::set_error(LBM_ERR_ARG, "null device pointer", cudaSuccess);
    /* the same level as lbm_body_force_f32 builds */
    lbm::Level L;
    const int lc = lbm::f32_kernel_level(L, nx, ny, nz, pitch);
    if (lc == 1) return lbm::set_error(LBM_ERR_ARG, "bad dimensions or pitch", cudaSuccess);
    if (lc == 2)
        return lbm::set_error(LBM_ERR_ARG, "level too large: 19 populations must index below 2^31", cudaSuccess);
    /* the reduction needs force_scan_partials()*3 doubles whatever the domain
     * size (the scan kernel strides over rows with a fixed grid) */
    if (lbm::force_scan_partials() * 3 > NOALLOC_SCRATCH_DOUBLES)
        return lbm::set_error(LBM_ERR_ARG, "the reduction needs more partial sums than the fixed scratch holds",
                              cudaSuccess);
    double* scratch = nullptr;
    if (int rc = scratch_on_current_device(&scratch)) return rc;
    /* every launch writes all partials before its final sum reads them, so
     * nothing in the shared array needs clearing between calls */
    cudaError_t e = lbm::launch_force_scan(L, fA, mask, scratch, force_out, (cudaStream_t)cuda_stream);
    if (e != cudaSuccess) return lbm::set_error(LBM_ERR_CUDA, "body force launch", e);
    return LBM_OK;
}
