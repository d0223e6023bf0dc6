/*
 * ref_shim_lr7.cpp -- host harness that runs the reference's own LR7 code.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/ref_recipe.py copies the device functions,
 * kernels and writers of LRTurbTest/LRMultiGPU7.cu (lines 68 up to main(),
 * i.e. LR7:68-2573) into oracle/_ref/lr7_body.inc and compiles this file once
 * per configuration with the reference's #define block given as -D flags.
 *
 * CUDA constructs are emulated on the host: a kernel launch runs each thread
 * block as blockDim coroutines that share the block's __shared__ arrays
 * (function statics, one block in flight at a time) and meet at a barrier in
 * syncthreads(); atomicAdd is a plain add (a single host thread runs).  The host loop restates the
 * single-GPU schedule of LR7:2849-2950 (the peer copies become memcpy).
 */
#include <sys/time.h>
#include <unistd.h>

#include <ucontext.h>

#include <functional>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <ostream>
#include <sstream>
#include <string>
#include <vector>

using namespace std;

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
static dim3 threadIdx, blockIdx, blockDim, gridDim;

/* One CUDA thread = one coroutine on the calling host thread.  syncthreads()
 * yields to the scheduler, which resumes every thread of the block once per
 * round, so no thread passes the k-th barrier before all threads reach it. */
static ucontext_t g_sched;
static std::vector<ucontext_t> g_ctx;
static std::vector<std::vector<char>> g_stack;
static std::vector<int> g_done;
static int g_cur = 0;
static std::function<void()>* g_body = nullptr;
static inline void syncthreads() { swapcontext(&g_ctx[g_cur], &g_sched); }
static inline float atomicAdd(float* a, float v) {
    float o = *a;
    *a = o + v;
    return o;
}
static void trampoline() {
    (*g_body)();
    g_done[g_cur] = 1;
}

#define __global__
#define __device__
#define __shared__ static

#include "lr7_body.inc"

/* run every block of a launch, one block at a time */
template <class F> static void launch(dim3 grid, dim3 block, F&& body) {
    gridDim = grid;
    blockDim = block;
    const int nthr = int(block.x * block.y * block.z);
    std::function<void()> fn(body);
    g_body = &fn;
    if (int(g_ctx.size()) < nthr) {
        g_ctx.resize(nthr);
        g_stack.resize(nthr);
        g_done.resize(nthr);
    }
    for (int t = 0; t < nthr; ++t)
        if (g_stack[t].empty()) g_stack[t].resize(256 * 1024);
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx) {
                blockIdx = dim3(bx, by, bz);
                for (int t = 0; t < nthr; ++t) {
                    getcontext(&g_ctx[t]);
                    g_ctx[t].uc_stack.ss_sp = g_stack[t].data();
                    g_ctx[t].uc_stack.ss_size = g_stack[t].size();
                    g_ctx[t].uc_link = &g_sched;
                    makecontext(&g_ctx[t], trampoline, 0);
                    g_done[t] = 0;
                }
                bool left = true;
                while (left) {
                    left = false;
                    for (int t = 0; t < nthr; ++t) {
                        if (g_done[t]) continue;
                        g_cur = t;
                        threadIdx = dim3(t % block.x, (t / block.x) % block.y, t / (block.x * block.y));
                        swapcontext(&g_sched, &g_ctx[t]);
                        if (!g_done[t]) left = true;
                    }
                }
            }
}

static size_t next_pow2(size_t n) {
    size_t p = 2;
    while (p < n) p *= 2;
    return p;
}

struct RefState {
    size_t pitch_e, pitchLR_e, pitchInterp_e;
    int zInner, zLRInner;
    float omega, omegaLR, SF_cf, SF_fc;
    vector<float> f[2], g[2], h[2], g_temp, h_temp;
    vector<float> F[3];
    vector<float> velAv[3], velFluc[3];
    vector<float> fLR[2], gLR[2], hLR[2], gLR_temp, hLR_temp;
    vector<float> velAvLR[3], velFlucLR[3];
    vector<float> f_interp, g_interp, h_interp, g_interp_temp, h_interp_temp;
    int A = 0, B = 1, C = 0, D = 1;
};

static RefState S;

/* compact [19][ZDIM][YDIM][XDIM] <-> (g, inner f, h) with pitch */
static void gather_level(const vector<float>& fin, const vector<float>& gin, const vector<float>& hin,
                         size_t pitch, int X, int Y, int Z, int zInner, float* out) {
    long N = long(X) * Y * Z;
    for (int q = 0; q < 19; ++q)
        for (int z = 0; z < Z; ++z)
            for (int y = 0; y < Y; ++y)
                for (int x = 0; x < X; ++x) {
                    float v;
                    if (z == 0) v = gin[x + y * pitch + q * pitch * Y];
                    else if (z == Z - 1) v = hin[x + y * pitch + q * pitch * Y];
                    else v = fin[x + y * pitch + (z - 1) * Y * pitch + q * pitch * Y * zInner];
                    out[q * N + (long(z) * Y + y) * X + x] = v;
                }
}

static void scatter_level(vector<float>& fin, vector<float>& gin, vector<float>& hin, size_t pitch,
                          int X, int Y, int Z, int zInner, const float* src) {
    long N = long(X) * Y * Z;
    for (int q = 0; q < 19; ++q)
        for (int z = 0; z < Z; ++z)
            for (int y = 0; y < Y; ++y)
                for (int x = 0; x < X; ++x) {
                    float v = src[q * N + (long(z) * Y + y) * X + x];
                    if (z == 0) gin[x + y * pitch + q * pitch * Y] = v;
                    else if (z == Z - 1) hin[x + y * pitch + q * pitch * Y] = v;
                    else fin[x + y * pitch + (z - 1) * Y * pitch + q * pitch * Y * zInner] = v;
                }
}

extern "C" {

/* allocation and initialisation, LR7:2599-2827 for GPU_N = 1 */
int ref_setup(const float* init_coarse, const float* init_fine) {
    const int GPU_N = 1;
    S = RefState();
    S.pitch_e = next_pow2(XDIM);
    S.zInner = ZDIM / GPU_N - 2;
    float CharLength = OBSTR1 * 2.f;
    S.omega = 1.0f / (3.0f * (UMAX * CharLength / RE) + 0.5f);
    S.omegaLR = 2.0f / (1.0f + 2.0f * (2.0f / S.omega - 1.0f));
    if (LRFACTOR == 0.25f) S.omegaLR = 2.0f / (1.0f + 2.0f * (2.0f / S.omegaLR - 1.0f));
    S.SF_cf = S.omega * (1.0f - S.omegaLR) / ((1.0f - S.omega) * S.omegaLR / LRFACTOR);
    S.SF_fc = 1.f / S.SF_cf;
    const size_t P = S.pitch_e;
    for (int i = 0; i < 2; ++i) {
        S.f[i].assign(P * YDIM * S.zInner * 19, 0.f);
        S.g[i].assign(P * YDIM * 19, 0.f);
        S.h[i].assign(P * YDIM * 19, 0.f);
    }
    S.g_temp.assign(P * YDIM * 19, 0.f);
    S.h_temp.assign(P * YDIM * 19, 0.f);
    for (int i = 0; i < 3; ++i) {
        S.F[i].assign(TMAX > STARTF ? TMAX - STARTF : 1, 0.f);
        S.velAv[i].assign(P * YDIM * ZDIM, 0.f);
        S.velFluc[i].assign(P * YDIM * ZDIM, 0.f);
    }
    dim3 threads(BLOCKSIZEX, BLOCKSIZEY, BLOCKSIZEZ);
    dim3 grid((XDIM + BLOCKSIZEX - 1) / BLOCKSIZEX, (YDIM + BLOCKSIZEY - 1) / BLOCKSIZEY, S.zInner / BLOCKSIZEZ);
    dim3 g_grid((XDIM + BLOCKSIZEX - 1) / BLOCKSIZEX, (YDIM + BLOCKSIZEY - 1) / BLOCKSIZEY, 1);
    for (int i = 0; i < 2; ++i) {
        launch(grid, threads, [&] { initialize(S.f[i].data(), P, S.zInner, GPU_N); });
        launch(g_grid, threads, [&] { initialize(S.g[i].data(), P, 1, GPU_N); });
        launch(g_grid, threads, [&] { initialize(S.h[i].data(), P, 1, GPU_N); });
    }
    launch(g_grid, threads, [&] { initialize(S.g_temp.data(), P, 1, GPU_N); });
    launch(g_grid, threads, [&] { initialize(S.h_temp.data(), P, 1, GPU_N); });
    if (init_coarse)
        for (int i = 0; i < 2; ++i)
            scatter_level(S.f[i], S.g[i], S.h[i], P, XDIM, YDIM, ZDIM, S.zInner, init_coarse);

    if (REFINEMENT == 1) {
        S.pitchLR_e = next_pow2(XLRDIM);
        S.pitchInterp_e = next_pow2(size_t(XLRDIM * LRFACTOR + 1));
        S.zLRInner = ZLRDIM / GPU_N - 2;
        const size_t PL = S.pitchLR_e, PI = S.pitchInterp_e;
        const size_t ymax = size_t(YLRDIM * LRFACTOR + 1);
        for (int i = 0; i < 2; ++i) {
            S.fLR[i].assign(PL * YLRDIM * S.zLRInner * 19, 0.f);
            S.gLR[i].assign(PL * YLRDIM * 19, 0.f);
            S.hLR[i].assign(PL * YLRDIM * 19, 0.f);
        }
        S.gLR_temp.assign(PL * YLRDIM * 19, 0.f);
        S.hLR_temp.assign(PL * YLRDIM * 19, 0.f);
        for (int i = 0; i < 3; ++i) {
            S.velAvLR[i].assign(PL * YLRDIM * ZLRDIM, 0.f);
            S.velFlucLR[i].assign(PL * YLRDIM * ZLRDIM, 0.f);
        }
        S.f_interp.assign(PI * ymax * S.zInner * 9, 0.f);
        S.g_interp.assign(PI * ymax * 9, 0.f);
        S.h_interp.assign(PI * ymax * 9, 0.f);
        S.g_interp_temp.assign(PI * ymax * 9, 0.f);
        S.h_interp_temp.assign(PI * ymax * 9, 0.f);
        dim3 LR_threads(BLOCKSIZELRX, BLOCKSIZELRY, BLOCKSIZELRZ);
        dim3 LR_grid((XLRDIM + BLOCKSIZELRX - 1) / BLOCKSIZELRX, (YLRDIM + BLOCKSIZELRY - 1) / BLOCKSIZELRY,
                     S.zLRInner / BLOCKSIZELRZ);
        dim3 g_LR_grid((XLRDIM + BLOCKSIZELRX - 1) / BLOCKSIZELRX, (YLRDIM + BLOCKSIZELRY - 1) / BLOCKSIZELRY, 1);
        for (int i = 0; i < 2; ++i) {
            launch(LR_grid, LR_threads, [&] { initializeLR(S.fLR[i].data(), PL, S.zLRInner, GPU_N); });
            launch(g_LR_grid, LR_threads, [&] { initializeLR(S.gLR[i].data(), PL, 1, GPU_N); });
            launch(g_LR_grid, LR_threads, [&] { initializeLR(S.hLR[i].data(), PL, 1, GPU_N); });
        }
        launch(g_LR_grid, LR_threads, [&] { initializeLR(S.gLR_temp.data(), PL, 1, GPU_N); });
        launch(g_LR_grid, LR_threads, [&] { initializeLR(S.hLR_temp.data(), PL, 1, GPU_N); });
        if (init_fine)
            for (int i = 0; i < 2; ++i)
                scatter_level(S.fLR[i], S.gLR[i], S.hLR[i], PL, XLRDIM, YLRDIM, ZLRDIM, S.zLRInner, init_fine);
    }
    return 0;
}

/* time loop, LR7:2849-2950 with GPU_N = 1 */
int ref_run(int t0, int nsteps) {
    const int GPU_N = 1;
    const size_t P = S.pitch_e;
    dim3 threads(BLOCKSIZEX, BLOCKSIZEY, BLOCKSIZEZ);
    dim3 grid((XDIM + BLOCKSIZEX - 1) / BLOCKSIZEX, (YDIM + BLOCKSIZEY - 1) / BLOCKSIZEY, S.zInner / BLOCKSIZEZ);
    dim3 g_grid((XDIM + BLOCKSIZEX - 1) / BLOCKSIZEX, (YDIM + BLOCKSIZEY - 1) / BLOCKSIZEY, 1);
    for (int t = t0; t < t0 + nsteps; ++t) {
        int &A = S.A, &B = S.B;
        memcpy(&S.h_temp[P * YDIM * 14], &S.g[A][P * YDIM * 14], P * YDIM * sizeof(float) * 5);
        memcpy(&S.g_temp[P * YDIM * 9], &S.h[A][P * YDIM * 9], P * YDIM * sizeof(float) * 5);
        int flag = (!REFINEMENT && t > STARTF);
        launch(grid, threads, [&] {
            update_inn(S.f[B].data(), S.f[A].data(), S.g[A].data(), S.h[A].data(), S.omega, P, 0, S.zInner,
                       S.velAv[0].data(), S.velAv[1].data(), S.velFluc[0].data(), S.velFluc[1].data(),
                       S.F[0].data(), S.F[1].data(), S.F[2].data(), t, flag, S.f_interp.data(), S.pitchInterp_e);
        });
        launch(g_grid, threads, [&] {
            update_top(S.h[B].data(), S.h[A].data(), S.f[A].data(), S.h_temp.data(), S.omega, P, 0, S.zInner,
                       S.F[0].data(), S.F[1].data(), S.F[2].data(), t, flag, S.h_interp.data(), S.pitchInterp_e);
        });
        launch(g_grid, threads, [&] {
            update_bot(S.g[B].data(), S.g[A].data(), S.f[A].data(), S.g_temp.data(), S.omega, P, 0, S.zInner,
                       S.F[0].data(), S.F[1].data(), S.F[2].data(), t, flag, S.g_interp.data(), S.pitchInterp_e);
        });
        std::swap(A, B);
        if (REFINEMENT == 1) {
            const size_t PL = S.pitchLR_e, PI = S.pitchInterp_e;
            const size_t ymax = size_t(YLRDIM * LRFACTOR + 1);
            dim3 LR_threads(BLOCKSIZELRX, BLOCKSIZELRY, BLOCKSIZELRZ);
            dim3 LR_grid((XLRDIM + BLOCKSIZELRX - 1) / BLOCKSIZELRX, (YLRDIM + BLOCKSIZELRY - 1) / BLOCKSIZELRY,
                         S.zLRInner / BLOCKSIZELRZ);
            dim3 g_LR_grid((XLRDIM + BLOCKSIZELRX - 1) / BLOCKSIZELRX, (YLRDIM + BLOCKSIZELRY - 1) / BLOCKSIZELRY,
                           1);
            int &C = S.C, &D = S.D;
            for (int i = 0; i < LRLEVEL; ++i) {
                int flag_F = (t > STARTF && i == 0) ? 1 : 0;
                memcpy(&S.hLR_temp[PL * YLRDIM * 14], &S.gLR[C][PL * YLRDIM * 14], PL * YLRDIM * sizeof(float) * 5);
                memcpy(&S.gLR_temp[PL * YLRDIM * 9], &S.hLR[C][PL * YLRDIM * 9], PL * YLRDIM * sizeof(float) * 5);
                launch(LR_grid, LR_threads, [&] {
                    update_inn_LR(S.fLR[D].data(), S.fLR[C].data(), S.gLR[C].data(), S.hLR[C].data(), S.omegaLR, PL,
                                  0, S.zLRInner, S.velAvLR[0].data(), S.velAvLR[1].data(), S.velFlucLR[0].data(),
                                  S.velFlucLR[1].data(), S.F[0].data(), S.F[1].data(), S.F[2].data(), t, flag_F);
                });
                launch(g_LR_grid, LR_threads, [&] {
                    update_top_LR(S.hLR[D].data(), S.hLR[C].data(), S.fLR[C].data(), S.hLR_temp.data(), S.omegaLR,
                                  PL, 0, S.zLRInner, S.F[0].data(), S.F[1].data(), S.F[2].data(), t, flag_F);
                });
                launch(g_LR_grid, LR_threads, [&] {
                    update_bot_LR(S.gLR[D].data(), S.gLR[C].data(), S.fLR[C].data(), S.gLR_temp.data(), S.omegaLR,
                                  PL, 0, S.zLRInner, S.F[0].data(), S.F[1].data(), S.F[2].data(), t, flag_F);
                });
                if (i == LRLEVEL - 1)
                    memcpy(S.g_interp_temp.data(), S.h_interp.data(), PI * ymax * sizeof(float) * 9);
                std::swap(C, D);
            }
            dim3 Interp_threads(BLOCKSIZEINTERP, LRLEVEL, LRLEVEL);
            dim3 Interp_grid((XLRDIM + BLOCKSIZEINTERP - 1) / BLOCKSIZEINTERP, (YLRDIM + LRLEVEL - 1) / LRLEVEL,
                             ZLRDIM / LRLEVEL / GPU_N);
            launch(Interp_grid, Interp_threads, [&] {
                InterpCF(S.fLR[C].data(), S.gLR[C].data(), S.hLR[C].data(), PL, S.f_interp.data(), S.g_interp.data(),
                         S.h_interp.data(), S.g_interp_temp.data(), PI, S.SF_cf, S.omega, 0, S.zInner, S.zLRInner);
            });
            memcpy(S.hLR_temp.data(), S.gLR[C].data(), PL * YLRDIM * sizeof(float) * 19);
            dim3 Interp_grid_c((XDIM + BLOCKSIZEX - 1) / BLOCKSIZEX, (YDIM + BLOCKSIZEY - 1) / BLOCKSIZEY,
                               (ZDIM / GPU_N) / BLOCKSIZEZ);
            launch(Interp_grid_c, threads, [&] {
                InterpFC(S.f[A].data(), S.g[A].data(), S.h[A].data(), S.fLR[C].data(), S.hLR[C].data(),
                         S.hLR_temp.data(), P, PL, S.SF_fc, S.omegaLR, 0, S.zInner, S.zLRInner);
            });
        }
    }
    return 0;
}

void ref_get_coarse(float* out) { gather_level(S.f[S.A], S.g[S.A], S.h[S.A], S.pitch_e, XDIM, YDIM, ZDIM, S.zInner, out); }

void ref_get_fine(float* out) {
    if (REFINEMENT == 1)
        gather_level(S.fLR[S.C], S.gLR[S.C], S.hLR[S.C], S.pitchLR_e, XLRDIM, YLRDIM, ZLRDIM, S.zLRInner, out);
}

/* compact coarse moments [9][ZDIM][ymax][xmax] exported by the last coarse step */
void ref_get_moments(float* out) {
    if (REFINEMENT != 1) return;
    const int xm = int(XLRDIM * LRFACTOR + 1), ym = int(YLRDIM * LRFACTOR + 1);
    const size_t PI = S.pitchInterp_e;
    long N = long(xm) * ym * ZDIM;
    for (int i = 0; i < 9; ++i)
        for (int z = 0; z < ZDIM; ++z)
            for (int y = 0; y < ym; ++y)
                for (int x = 0; x < xm; ++x) {
                    float v;
                    if (z == 0) v = S.g_interp[x + y * PI + i * ym * PI];
                    else if (z == ZDIM - 1) v = S.h_interp[x + y * PI + i * ym * PI];
                    else v = S.f_interp[x + y * PI + (z - 1) * ym * PI + i * ym * PI * S.zInner];
                    out[i * N + (long(z) * ym + y) * xm + x] = v;
                }
}

/* velAv u, velAv v, velFluc u, velFluc v as compact [4][ZDIM][YDIM][XDIM] */
void ref_get_stats(float* out) {
    const long N = long(XDIM) * YDIM * ZDIM;
    const size_t P = S.pitch_e;
    const vector<float>* src[4] = {&S.velAv[0], &S.velAv[1], &S.velFluc[0], &S.velFluc[1]};
    for (int k = 0; k < 4; ++k)
        for (int z = 0; z < ZDIM; ++z)
            for (int y = 0; y < YDIM; ++y)
                for (int x = 0; x < XDIM; ++x)
                    out[k * N + (long(z) * YDIM + y) * XDIM + x] = (*src[k])[x + y * P + z * P * YDIM];
}

void ref_get_forces(float* out, int n) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < n && j < int(S.F[i].size()); ++j) out[i * n + j] = S.F[i][j];
}

void ref_get_params(float* out) {
    out[0] = S.omega;
    out[1] = S.omegaLR;
    out[2] = S.SF_cf;
    out[3] = S.SF_fc;
}

/* the reference's ImageFcn / ImageFcnLR on every node (node-type codes of LR7:88-127) */
void ref_image(int* out) {
    for (int z = 0; z < ZDIM; ++z)
        for (int y = 0; y < YDIM; ++y)
            for (int x = 0; x < XDIM; ++x) out[(long(z) * YDIM + y) * XDIM + x] = ImageFcn(x, y, z);
}

void ref_image_lr(int* out) {
    for (int z = 0; z < ZLRDIM; ++z)
        for (int y = 0; y < YLRDIM; ++y)
            for (int x = 0; x < XLRDIM; ++x)
                out[(long(z) * YLRDIM + y) * XLRDIM + x] =
                    ImageFcnLR(LRX0 + x * LRFACTOR, LRY0 + y * LRFACTOR, LRZ0 + LRFACTOR * z);
}

/* per-cell device functions on n cells stored cell-major */
void ref_mrt_collide(float* f, int n, float omega) {
    for (int i = 0; i < n; ++i) mrt_collide(f + 19L * i, omega, 0.f);
}
void ref_extrap(int kind, float* f, int n, float val) {
    for (int i = 0; i < n; ++i) {
        float* g = f + 19L * i;
        if (kind == 3) West_Extrap(g, val, 0);
        else if (kind == 4) East_Extrap(g, val);
        else if (kind == 5) South_Extrap(g, val);
        else if (kind == 6) North_Extrap(g, val);
    }
}
void ref_init_meq(float* f, float u) {
    float m[19] = {0};
    mrt_meq(m, 1.f, u, 0.f, 0.f);
    InvertMoments(f, m);
}
void ref_physical_moments(const float* f, float* mom, int n) {
    for (int i = 0; i < n; ++i) PhysicalMoments(mom + 9L * i, const_cast<float*>(f + 19L * i));
}
void ref_strain_rate(const float* mom, float* s, int n) {
    for (int i = 0; i < n; ++i) StrainRate(s + 6L * i, const_cast<float*>(mom + 9L * i), 1.f);
}
void ref_invert_les_cf(const float* mom, float* f, int n, float omega_c) {
    for (int i = 0; i < n; ++i) InvertPhysicalMoments_LES_cf(f + 19L * i, const_cast<float*>(mom + 9L * i), 0.f, omega_c);
}
void ref_invert_les_fc(const float* mom, float* f, int n, float omega_f) {
    for (int i = 0; i < n; ++i) InvertPhysicalMoments_LES_fc(f + 19L * i, const_cast<float*>(mom + 9L * i), 0.f, omega_f);
}

/* the reference's run-record and output writers (LR7:2350-2573) */
int ref_write_inputs(char* buf, int len) {
    std::ostringstream os;
    WriteInputs(os, S.omega, S.omegaLR, 1);
    std::string s = os.str();
    if (int(s.size()) + 1 > len) return -1;
    memcpy(buf, s.c_str(), s.size() + 1);
    return int(s.size());
}

int ref_write_results(char* buf, int len, char* slice, int slen) {
    const int Z = ZDIM;
    vector<float> fin(size_t(XDIM) * YDIM * (Z - 2) * 19), gin(size_t(XDIM) * YDIM * 19), hin(size_t(XDIM) * YDIM * 19);
    const size_t P = S.pitch_e;
    for (int q = 0; q < 19; ++q)
        for (int y = 0; y < YDIM; ++y)
            for (int x = 0; x < XDIM; ++x) {
                gin[x + y * XDIM + q * XDIM * YDIM] = S.g[S.A][x + y * P + q * P * YDIM];
                hin[x + y * XDIM + q * XDIM * YDIM] = S.h[S.A][x + y * P + q * P * YDIM];
                for (int z = 0; z < Z - 2; ++z)
                    fin[x + y * XDIM + z * XDIM * YDIM + q * XDIM * YDIM * (Z - 2)] =
                        S.f[S.A][x + y * P + z * YDIM * P + q * P * YDIM * S.zInner];
            }
    vector<float> av[3], fl[3];
    float* avp[3];
    float* flp[3];
    for (int i = 0; i < 3; ++i) {
        av[i].assign(size_t(XDIM) * YDIM * Z, 0.f);
        fl[i].assign(size_t(XDIM) * YDIM * Z, 0.f);
        for (int z = 0; z < Z; ++z)
            for (int y = 0; y < YDIM; ++y)
                for (int x = 0; x < XDIM; ++x) {
                    av[i][x + y * XDIM + z * XDIM * YDIM] = S.velAv[i][x + y * P + z * P * YDIM];
                    fl[i][x + y * XDIM + z * XDIM * YDIM] = S.velFluc[i][x + y * P + z * P * YDIM];
                }
        avp[i] = av[i].data();
        flp[i] = fl[i].data();
    }
    std::ostringstream os, ss;
    WriteResults(os, ss, fin.data(), gin.data(), hin.data(), avp, flp, S.omega, 1, 0);
    std::string a = os.str(), b = ss.str();
    if (int(a.size()) + 1 > len || int(b.size()) + 1 > slen) return -1;
    memcpy(buf, a.c_str(), a.size() + 1);
    memcpy(slice, b.c_str(), b.size() + 1);
    return 0;
}

int ref_write_forces(char* buf, int len, int level) {
    int n = int(S.F[0].size());
    float* Fp[3] = {S.F[0].data(), S.F[1].data(), S.F[2].data()};
    std::string path = std::string("/tmp/ref_forces_") + std::to_string(getpid()) + ".force";
    {
        std::ofstream o(path.c_str());
        WriteForces(Fp, o, n, level);
    }
    std::ifstream i(path.c_str());
    std::stringstream ss;
    ss << i.rdbuf();
    std::remove(path.c_str());
    std::string s = ss.str();
    if (int(s.size()) + 1 > len) return -1;
    memcpy(buf, s.c_str(), s.size() + 1);
    return int(s.size());
}

/* xsymmetry_top / xsymmetry_bot (LR7:899-1016) on n cells at (y, z) */
void ref_xsymmetry(float* f, int n, const int* yz, int top) {
    for (int i = 0; i < n; ++i) {
        if (top) xsymmetry_top(f + 19L * i, yz[2 * i], yz[2 * i + 1]);
        else xsymmetry_bot(f + 19L * i, yz[2 * i], yz[2 * i + 1]);
    }
}
int ref_ydim(void) { return YDIM; }
int ref_zdim(void) { return ZDIM; }

}  // extern "C"
