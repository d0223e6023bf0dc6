/*
 * lbm_ensemble.cpp -- host side of the ensemble of periodic decaying-
 * turbulence boxes behind the C ABI: member layout, the seeded random-phase
 * initial fields, stepping through a captured CUDA graph of a persistent
 * kernel, the autotuner of tile height and grid size, read-outs, and the
 * filtered training samples of the learned subgrid closure.
 *
 * No counterpart in the reference: it runs one domain per program.  The
 * update rule of each member is the reference's MRT collision
 * (LRTurbTest/LRMultiGPU7.cu:583-711) with periodic streaming in x, y, z.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "ensemble.cuh"
#include "lbm_kernels.cuh"
#include "sgs_infer.cuh"

using namespace lbm;

struct lbm_ensemble {
    ens::Table T{};
    int sgs = ens::SGS_NONE;
    float cs = 0.01f;
    std::vector<int> sizes;
    std::vector<float> tau0;
    float* f[2] = {nullptr, nullptr};
    size_t nelem = 0; /* per buffer */
    float* u = nullptr;
    size_t nu = 0;
    double* ubar = nullptr; /* filter scratch, sized for the largest member */
    double* uu = nullptr;
    double* s8 = nullptr;
    ens::Mode* modes = nullptr;
    unsigned char* blob = nullptr;
    int* err = nullptr;
    double* energy = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int cur = 0;
    long long steps = 0;
    int grid = 0;
    cudaGraphExec_t gexec = nullptr;
    int gsteps = 8;
    float tuned_ms = 0;
    long long cells = 0;
};

namespace {

#define ENS_TRY(call, what)                                                 \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) return set_error(LBM_ERR_CUDA, what, e_);    \
    } while (0)

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0xD1B54A32D192ED03ull) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return double(next() >> 11) * (1.0 / 9007199254740992.0); }
};

int sm_count() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 152;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 152;
    return n;
}

/* tile bookkeeping for tile height ty (offsets do not depend on it) */
void layout(lbm_ensemble* e, int ty) {
    ens::Table& T = e->T;
    T.ty = ty;
    int tile = 0;
    for (int m = 0; m < T.count; ++m) {
        ens::Member& M = T.m[m];
        M.tiles_x = M.pitch / 32;
        M.tiles_y = (M.n + ty - 1) / ty;
        M.tile0 = tile;
        tile += M.tiles_x * M.tiles_y * M.n;
    }
    T.ntiles = tile;
}

void drop_graph(lbm_ensemble* e) {
    if (e->gexec) cudaGraphExecDestroy(e->gexec);
    e->gexec = nullptr;
}

cudaError_t one_step(lbm_ensemble* e) {
    cudaError_t r = launch_ens_step(e->T, e->f[e->cur], e->f[1 - e->cur], e->sgs, e->blob, e->cs, e->err, e->grid,
                                    e->stream);
    e->cur = 1 - e->cur;
    return r;
}

/* the graph runs gsteps (even) steps starting from buffer 0 */
cudaError_t build_graph(lbm_ensemble* e) {
    drop_graph(e);
    cudaGraph_t g = nullptr;
    if (cudaError_t r0 = lbm::TmemLane::prepare()) return r0;
    cudaError_t r = cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal);
    if (r != cudaSuccess) return r;
    const int saved = e->cur;
    e->cur = 0;
    for (int i = 0; i < e->gsteps && r == cudaSuccess; ++i) r = one_step(e);
    e->cur = saved;
    cudaError_t r2 = cudaStreamEndCapture(e->stream, &g);
    if (r == cudaSuccess) r = r2;
    if (r == cudaSuccess) r = cudaGraphInstantiate(&e->gexec, g, 0);
    if (g) cudaGraphDestroy(g);
    return r;
}

std::mutex g_tune_mu;
std::map<std::string, std::pair<int, int>> g_tune_cache;

std::string tune_key(const lbm_ensemble* e) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::string k = std::to_string(dev) + ":" + std::to_string(e->sgs);
    for (int n : e->sizes) k += "," + std::to_string(n);
    return k;
}

/* seeded random-phase solenoidal modes with E(k) ~ k^-5/3 for k = 1..kmax,
 * up to `per_shell` wavevectors per shell (one of each +-k pair), scaled so
 * that the per-component rms velocity is u_rms */
void make_modes(int n, int kmax, int per_shell, uint64_t seed, double u_rms, std::vector<ens::Mode>& out) {
    Rng r(seed);
    std::vector<ens::Mode> mm;
    for (int k = 1; k <= kmax; ++k) {
        std::vector<std::array<int, 3>> shell;
        for (int a = -k - 1; a <= k + 1; ++a)
            for (int b = -k - 1; b <= k + 1; ++b)
                for (int c = -k - 1; c <= k + 1; ++c) {
                    const double km = std::sqrt(double(a * a + b * b + c * c));
                    if (km < k - 0.5 || km >= k + 0.5) continue;
                    /* one representative of each +-k pair */
                    if (a < 0 || (a == 0 && (b < 0 || (b == 0 && c <= 0)))) continue;
                    shell.push_back({a, b, c});
                }
        for (int i = int(shell.size()) - 1; i > 0; --i) std::swap(shell[i], shell[size_t(r.next() % uint64_t(i + 1))]);
        const int take = std::min<int>(per_shell, int(shell.size()));
        const double Ek = std::pow(double(k), -5.0 / 3.0);
        const double amp = std::sqrt(4 * Ek / take);
        for (int i = 0; i < take; ++i) {
            ens::Mode md{};
            md.k[0] = shell[i][0], md.k[1] = shell[i][1], md.k[2] = shell[i][2];
            const double kk = std::sqrt(double(md.k[0] * md.k[0] + md.k[1] * md.k[1] + md.k[2] * md.k[2]));
            /* a random direction orthogonal to k */
            double v[3], dot;
            do {
                for (double& x : v) x = 2 * r.uniform() - 1;
                dot = (v[0] * md.k[0] + v[1] * md.k[1] + v[2] * md.k[2]) / kk;
                for (int j = 0; j < 3; ++j) v[j] -= dot * md.k[j] / kk;
            } while (v[0] * v[0] + v[1] * v[1] + v[2] * v[2] < 1e-6);
            const double vn = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            for (int j = 0; j < 3; ++j) md.a[j] = amp * v[j] / vn;
            md.phase = 2 * r.uniform();
            mm.push_back(md);
        }
    }
    /* <|u|^2> = sum a^2 / 2 for distinct wavevectors; rms per component */
    double s2 = 0;
    for (const auto& md : mm) s2 += md.a[0] * md.a[0] + md.a[1] * md.a[1] + md.a[2] * md.a[2];
    const double scale = s2 > 0 ? u_rms / std::sqrt(s2 / 6) : 0;
    for (auto& md : mm)
        for (double& a : md.a) a *= scale;
    (void)n;
    out.insert(out.end(), mm.begin(), mm.end());
}

int sync_check(lbm_ensemble* e) {
    ENS_TRY(cudaStreamSynchronize(e->stream), "ensemble");
    int v = 0;
    ENS_TRY(cudaMemcpy(&v, e->err, sizeof(int), cudaMemcpyDeviceToHost), "error flag");
    if (v) {
        cudaMemset(e->err, 0, sizeof(int));
        return set_error(LBM_ERR_CUDA, "ensemble: a tensor-core completion wait ran out", cudaSuccess);
    }
    return LBM_OK;
}

}  // namespace

extern "C" {

int lbm_ensemble_create(int count, const int* sizes, const float* tau0, int sgs, float cs, lbm_ensemble** out) {
    if (!out || !sizes || !tau0 || count < 1 || count > ens::MAXM || sgs < 0 || sgs > 2)
        return set_error(LBM_ERR_ARG, "ensemble: bad argument (1..32 members, sgs 0..2)", cudaSuccess);
    *out = nullptr;
    for (int m = 0; m < count; ++m)
        if (sizes[m] < 8 || sizes[m] > 1024 || (sizes[m] & 1) || !(tau0[m] > 0.5f))
            return set_error(LBM_ERR_ARG, "ensemble: member sides must be even, 8..1024, tau0 > 1/2", cudaSuccess);
    lbm_ensemble* e = new lbm_ensemble();
    auto bail = [&](int rc) {
        lbm_ensemble_destroy(e);
        return rc;
    };
    e->sgs = sgs;
    e->cs = cs;
    e->sizes.assign(sizes, sizes + count);
    e->tau0.assign(tau0, tau0 + count);
    ens::Table& T = e->T;
    T.count = count;
    unsigned long long off = 0, uoff = 0;
    size_t maxc = 0;
    for (int m = 0; m < count; ++m) {
        ens::Member& M = T.m[m];
        M.n = sizes[m];
        M.pitch = (M.n + 31) / 32 * 32;
        M.off = off;
        M.uoff = uoff;
        M.tau0 = tau0[m];
        M.omega = 1.f / tau0[m];
        const unsigned long long qs = (unsigned long long)M.n * M.n * M.pitch;
        if (qs * 19 >= (1ull << 31))
            return bail(set_error(LBM_ERR_ARG, "ensemble: a member must index below 2^31", cudaSuccess));
        off += 19 * qs;
        uoff += 3ull * M.n * M.n * M.n;
        e->cells += (long long)M.n * M.n * M.n;
        maxc = std::max(maxc, size_t(M.n / 2) * (M.n / 2) * (M.n / 2));
    }
    e->nelem = off;
    e->nu = uoff;
    layout(e, 8);
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(set_error(LBM_ERR_CUDA, "ensemble: stream", cudaSuccess));
    cudaEventCreate(&e->e0);
    cudaEventCreate(&e->e1);
    for (int i = 0; i < 2; ++i)
        if (cudaMalloc(&e->f[i], e->nelem * sizeof(float)) != cudaSuccess)
            return bail(set_error(LBM_ERR_CUDA, "ensemble: population buffers", cudaGetLastError()));
    if (cudaMalloc(&e->u, e->nu * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&e->ubar, maxc * 3 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&e->uu, maxc * 6 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&e->s8, maxc * 8 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&e->err, sizeof(int)) != cudaSuccess || cudaMalloc(&e->energy, ens::MAXM * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&e->blob, sgs::BLOB_BYTES) != cudaSuccess)
        return bail(set_error(LBM_ERR_CUDA, "ensemble: buffers", cudaGetLastError()));
    cudaMemset(e->err, 0, sizeof(int));
    cudaMemset(e->blob, 0, sgs::BLOB_BYTES);
    /* at rest until an initialiser runs */
    cudaMemset(e->u, 0, e->nu * sizeof(float));
    if (launch_ens_init_from(e->T, e->u, e->f[0], e->f[1], e->stream) != cudaSuccess)
        return bail(set_error(LBM_ERR_CUDA, "ensemble: init", cudaGetLastError()));
    e->grid = std::min(e->T.ntiles, sm_count() * ens_step_occupancy(e->T.ty, sgs));
    if (int rc = sync_check(e)) return bail(rc);
    *out = e;
    return LBM_OK;
}

int lbm_ensemble_destroy(lbm_ensemble* e) {
    if (!e) return LBM_OK;
    if (e->stream) cudaStreamSynchronize(e->stream);
    drop_graph(e);
    cudaFree(e->f[0]);
    cudaFree(e->f[1]);
    cudaFree(e->u);
    cudaFree(e->ubar);
    cudaFree(e->uu);
    cudaFree(e->s8);
    cudaFree(e->modes);
    cudaFree(e->blob);
    cudaFree(e->err);
    cudaFree(e->energy);
    if (e->e0) cudaEventDestroy(e->e0);
    if (e->e1) cudaEventDestroy(e->e1);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
    return LBM_OK;
}

int lbm_ensemble_init_turbulence(lbm_ensemble* e, uint32_t seed, float u_rms, int kmax_div, int per_shell) {
    if (!e || !(u_rms >= 0) || kmax_div < 2 || per_shell < 1) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    std::vector<ens::Mode> all;
    for (int m = 0; m < e->T.count; ++m) {
        ens::Member& M = e->T.m[m];
        M.mode0 = int(all.size());
        make_modes(M.n, std::max(1, M.n / kmax_div), per_shell, (uint64_t(seed) << 8) + uint64_t(m), u_rms, all);
        M.nmodes = int(all.size()) - M.mode0;
    }
    cudaFree(e->modes);
    e->modes = nullptr;
    ENS_TRY(cudaMalloc(&e->modes, std::max<size_t>(1, all.size()) * sizeof(ens::Mode)), "modes");
    ENS_TRY(cudaMemcpy(e->modes, all.data(), all.size() * sizeof(ens::Mode), cudaMemcpyHostToDevice), "modes");
    ENS_TRY(launch_ens_init(e->T, e->modes, e->f[0], e->f[1], e->u, e->stream), "turbulence init");
    e->cur = 0;
    e->steps = 0;
    return sync_check(e);
}

int lbm_ensemble_modes(const lbm_ensemble* e, int member, int* k3, double* phase, double* a3, int cap, int* n) {
    if (!e || member < 0 || member >= e->T.count || !n) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    const ens::Member& M = e->T.m[member];
    *n = M.nmodes;
    if (!e->modes || M.nmodes == 0) return LBM_OK;
    std::vector<ens::Mode> mm(M.nmodes);
    ENS_TRY(cudaMemcpy(mm.data(), e->modes + M.mode0, M.nmodes * sizeof(ens::Mode), cudaMemcpyDeviceToHost), "modes");
    for (int i = 0; i < M.nmodes && i < cap; ++i) {
        for (int j = 0; j < 3; ++j) {
            if (k3) k3[3 * i + j] = mm[i].k[j];
            if (a3) a3[3 * i + j] = mm[i].a[j];
        }
        if (phase) phase[i] = mm[i].phase;
    }
    return LBM_OK;
}

int lbm_ensemble_init_filtered(lbm_ensemble* coarse, lbm_ensemble* fine) {
    if (!coarse || !fine || coarse->T.count != fine->T.count)
        return set_error(LBM_ERR_ARG, "ensembles do not match", cudaSuccess);
    for (int m = 0; m < fine->T.count; ++m)
        if (coarse->T.m[m].n * 2 != fine->T.m[m].n)
            return set_error(LBM_ERR_ARG, "coarse members must be half the fine sides", cudaSuccess);
    ENS_TRY(launch_ens_velocity(fine->T, fine->f[fine->cur], fine->u, fine->stream), "velocity");
    for (int m = 0; m < fine->T.count; ++m) {
        const ens::Member& F = fine->T.m[m];
        const size_t cn = size_t(F.n / 2) * (F.n / 2) * (F.n / 2);
        ENS_TRY(launch_box_filter(fine->u + F.uoff, F.n, fine->ubar, fine->uu, fine->stream), "filter");
        ENS_TRY(launch_d2f(fine->ubar, coarse->u + coarse->T.m[m].uoff, 3 * cn, fine->stream), "copy");
    }
    ENS_TRY(cudaStreamSynchronize(fine->stream), "filter");
    ENS_TRY(launch_ens_init_from(coarse->T, coarse->u, coarse->f[0], coarse->f[1], coarse->stream), "init");
    coarse->cur = 0;
    coarse->steps = 0;
    return sync_check(coarse);
}

int lbm_ensemble_set_mlp(lbm_ensemble* e, const float* params) {
    if (!e || !params) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    std::vector<unsigned char> blob(sgs::BLOB_BYTES);
    mlp_make_blob(params, blob.data());
    ENS_TRY(cudaMemcpyAsync(e->blob, blob.data(), blob.size(), cudaMemcpyHostToDevice, e->stream), "weights");
    return sync_check(e);
}

int lbm_ensemble_step(lbm_ensemble* e, int nsteps) {
    if (!e || nsteps < 0) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    while (nsteps > 0 && e->cur != 0) {
        ENS_TRY(one_step(e), "ensemble step");
        --nsteps, ++e->steps;
    }
    if (nsteps >= e->gsteps) {
        if (!e->gexec) ENS_TRY(build_graph(e), "graph capture");
        for (; nsteps >= e->gsteps; nsteps -= e->gsteps, e->steps += e->gsteps)
            ENS_TRY(cudaGraphLaunch(e->gexec, e->stream), "graph launch");
    }
    for (; nsteps > 0; --nsteps, ++e->steps) ENS_TRY(one_step(e), "ensemble step");
    return LBM_OK;
}

int lbm_ensemble_step_timed(lbm_ensemble* e, int nsteps, float* ms) {
    if (!e || !ms) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    ENS_TRY(cudaEventRecord(e->e0, e->stream), "event");
    if (int rc = lbm_ensemble_step(e, nsteps)) return rc;
    ENS_TRY(cudaEventRecord(e->e1, e->stream), "event");
    ENS_TRY(cudaEventSynchronize(e->e1), "event");
    ENS_TRY(cudaEventElapsedTime(ms, e->e0, e->e1), "event");
    return sync_check(e);
}

int lbm_ensemble_autotune(lbm_ensemble* e, int* ty_out, int* grid_out, float* ms_out) {
    if (!e) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    const std::string key = tune_key(e);
    int best_ty = 0, best_grid = 0;
    float best = 1e30f;
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) best_ty = it->second.first, best_grid = it->second.second;
    }
    if (!best_ty) {
        /* trial steps run from a copy of the state, which is put back */
        float* backup = nullptr;
        ENS_TRY(cudaMalloc(&backup, e->nelem * sizeof(float)), "autotune backup");
        cudaMemcpyAsync(backup, e->f[e->cur], e->nelem * sizeof(float), cudaMemcpyDeviceToDevice, e->stream);
        const int sms = sm_count();
        cudaError_t r = cudaSuccess;
        for (int ty : {4, 8}) {
            layout(e, ty);
            const int occ = ens_step_occupancy(ty, e->sgs);
            std::vector<int> grids;
            for (int b = 1; b <= occ; ++b) grids.push_back(std::min(e->T.ntiles, sms * b));
            grids.push_back(e->T.ntiles); /* one tile per block */
            for (int gsz : grids) {
                e->grid = gsz;
                for (int i = 0; i < 2 && r == cudaSuccess; ++i) r = one_step(e);
                cudaEventRecord(e->e0, e->stream);
                for (int i = 0; i < 6 && r == cudaSuccess; ++i) r = one_step(e);
                cudaEventRecord(e->e1, e->stream);
                if (r == cudaSuccess) r = cudaEventSynchronize(e->e1);
                float ms = 0;
                if (r == cudaSuccess) cudaEventElapsedTime(&ms, e->e0, e->e1);
                if (r == cudaSuccess && ms / 6 < best) best = ms / 6, best_ty = ty, best_grid = gsz;
            }
        }
        cudaMemcpyAsync(e->f[0], backup, e->nelem * sizeof(float), cudaMemcpyDeviceToDevice, e->stream);
        cudaStreamSynchronize(e->stream);
        cudaFree(backup);
        e->cur = 0;
        ENS_TRY(r, "autotune trial");
        std::lock_guard<std::mutex> g(g_tune_mu);
        g_tune_cache[key] = {best_ty, best_grid};
    }
    layout(e, best_ty);
    e->grid = best_grid;
    e->tuned_ms = best < 1e29f ? best : 0.f;
    drop_graph(e);
    if (ty_out) *ty_out = best_ty;
    if (grid_out) *grid_out = best_grid;
    if (ms_out) *ms_out = e->tuned_ms;
    return sync_check(e);
}

int lbm_ensemble_info(const lbm_ensemble* e, int* ty, int* grid, long long* cells, long long* steps) {
    if (!e) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    if (ty) *ty = e->T.ty;
    if (grid) *grid = e->grid;
    if (cells) *cells = e->cells;
    if (steps) *steps = e->steps;
    return LBM_OK;
}

int lbm_ensemble_energy(lbm_ensemble* e, double* E) {
    if (!e || !E) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    ENS_TRY(launch_ens_velocity(e->T, e->f[e->cur], e->u, e->stream), "velocity");
    ENS_TRY(launch_ens_energy(e->T, e->u, e->energy, e->stream), "energy");
    ENS_TRY(cudaMemcpyAsync(E, e->energy, e->T.count * sizeof(double), cudaMemcpyDeviceToHost, e->stream), "read");
    return sync_check(e);
}

int lbm_ensemble_velocity(lbm_ensemble* e, int member, float* u3) {
    if (!e || !u3 || member < 0 || member >= e->T.count) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    const ens::Member& M = e->T.m[member];
    ENS_TRY(launch_ens_velocity(e->T, e->f[e->cur], e->u, e->stream), "velocity");
    ENS_TRY(cudaMemcpyAsync(u3, e->u + M.uoff, 3ull * M.n * M.n * M.n * sizeof(float), cudaMemcpyDeviceToHost,
                            e->stream),
            "read");
    return sync_check(e);
}

/* compact f[19][n][n][n] in and out */
int lbm_ensemble_populations(lbm_ensemble* e, int member, float* f) {
    if (!e || !f || member < 0 || member >= e->T.count) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    const ens::Member& M = e->T.m[member];
    ENS_TRY(cudaStreamSynchronize(e->stream), "sync");
    ENS_TRY(cudaMemcpy2D(f, M.n * sizeof(float), e->f[e->cur] + M.off, M.pitch * sizeof(float), M.n * sizeof(float),
                         size_t(19) * M.n * M.n, cudaMemcpyDeviceToHost),
            "read");
    return LBM_OK;
}

int lbm_ensemble_set_populations(lbm_ensemble* e, int member, const float* f) {
    if (!e || !f || member < 0 || member >= e->T.count) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    const ens::Member& M = e->T.m[member];
    ENS_TRY(cudaStreamSynchronize(e->stream), "sync");
    for (int i = 0; i < 2; ++i)
        ENS_TRY(cudaMemcpy2D(e->f[i] + M.off, M.pitch * sizeof(float), f, M.n * sizeof(float), M.n * sizeof(float),
                             size_t(19) * M.n * M.n, cudaMemcpyHostToDevice),
                "write");
    return LBM_OK;
}

/* training samples of every (fine) member filtered 2x2x2 onto its coarse
 * grid: X[n][16] features, T[n] target eddy viscosities, appended from *n
 * (device pointers; cap = capacity in samples) */
int lbm_ensemble_samples(lbm_ensemble* e, float tau0_coarse, float* d_X, float* d_T, long long cap, long long* n) {
    if (!e || !d_X || !d_T || !n || *n < 0) return set_error(LBM_ERR_ARG, "bad argument", cudaSuccess);
    ENS_TRY(launch_ens_velocity(e->T, e->f[e->cur], e->u, e->stream), "velocity");
    long long pos = *n;
    for (int m = 0; m < e->T.count; ++m) {
        const ens::Member& M = e->T.m[m];
        const int nc = M.n / 2;
        const long long cn = (long long)nc * nc * nc;
        if (pos + cn > cap) return set_error(LBM_ERR_ARG, "sample buffer full", cudaSuccess);
        ENS_TRY(launch_box_filter(e->u + M.uoff, M.n, e->ubar, e->uu, e->stream), "filter");
        /* acoustic scaling: half the lattice viscosity on the 2x coarser grid */
        const double t0 = tau0_coarse > 0.5f ? double(tau0_coarse) : 0.5 + (double(M.tau0) - 0.5) / 2;
        ENS_TRY(launch_sgs_targets(e->ubar, e->uu, nc, t0, e->s8, d_X + pos * sgs::NIN, d_T + pos, e->stream),
                "targets");
        pos += cn;
    }
    *n = pos;
    return sync_check(e);
}

}  // extern "C"
