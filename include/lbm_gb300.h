/*
 * lbm_gb300.h -- C ABI of the GB300 D3Q19 stream-collide engine.
 *
 * The reference (gladyslol/LBM_MultiGPU) has no library API: its programs are
 * configured by #define blocks, record their parameters in a ".inputs" file,
 * drive the kernels from main() and write tecplot/.force files.  This header
 * replaces that boundary with functions a host program (or an FFI binding)
 * calls; each entry point names the reference code it stands in for.
 *
 * Conventions: every function returns 0 (LBM_OK) or an LBM_ERR_* code and
 * lbm_last_error() gives the message of the last failure on the calling
 * thread.  A handle is driven by one host thread at a time and owns one CUDA
 * stream.  Population arrays crossing the ABI are compact structure-of-arrays
 * float[19][nz][ny][nx] in the reference's velocity order; fields are
 * float[nz][ny][nx]; "velocity" is the momentum sum c_q f_q, as in the
 * reference's output (LRTurbTest/LRMultiGPU7.cu:2368-2370).
 * Level 0 is the base grid, level 1 the refinement patch.
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum lbm_status {
    LBM_OK = 0,
    LBM_ERR_ARG = 1,        /* bad argument or size */
    LBM_ERR_CUDA = 2,       /* a CUDA call failed (message has the CUDA error) */
    LBM_ERR_PARSE = 3,      /* malformed .inputs record */
    LBM_ERR_CONFIG = 4,     /* inconsistent configuration (e.g. LRLEVEL vs LRFACTOR) */
    LBM_ERR_NOMEM = 5,
    LBM_ERR_STATE = 6       /* call not valid in the handle's state */
};

/* node types of the solid/boundary mask (the reference's ImageFcn codes in
 * brackets, LRTurbTest/LRMultiGPU7.cu:88-127) */
enum lbm_node {
    LBM_FLUID = 0,          /* [0] */
    LBM_WALL = 1,           /* [1]   full-way bounce-back */
    LBM_BODY = 2,           /* [10]  full-way bounce-back + momentum-exchange force */
    LBM_WEST_INLET = 3,     /* [400] West_Extrap, LR7:852-897 */
    LBM_EAST_OUTLET = 4,    /* [300] East_Extrap, LR7:805-850 */
    LBM_SOUTH_INLET = 5,    /* [200] South_Extrap, LR7:760-803 */
    LBM_NORTH_OUTLET = 6,   /* [100] North_Extrap, LR7:713-758 */
    LBM_LID = 7             /* [53 in CPU_3D] regularised moving lid, CPU_3D/CPU_3D.cpp:974-1054 */
};

typedef struct lbm_handle lbm_handle;

const char* lbm_last_error(void);
const char* lbm_version(void);

/* ---- host-only helpers (no CUDA device needed) ---- */

/* Parse a .inputs record and write it back in WriteInputs' format
 * (LR7:2547-2573) with the derived omega / omegaLR lines recomputed
 * (LR7:2607-2619).  Same length/capacity convention as lbm_write_inputs. */
int lbm_inputs_normalize(const char* inputs_text, char* buf, size_t cap, size_t* len);
/* Node mask a record describes (ImageFcn for level 0, ImageFcnLR for level
 * 1, LR7:68-127), uint8[nz][ny][nx] of lbm_node values; *n = node count */
int lbm_inputs_mask(const char* inputs_text, int level, uint8_t* mask, size_t cap, size_t* n);
/* Tecplot POINT zone of one level in WriteResults' layout (LR7:2350-2442;
 * WriteResultsLR, LR7:2444-2535, for level 1) from compact populations f and
 * optional statistics stats4 (float[4][nz][ny][nx] or NULL for zeros).  The
 * zone goes to buf, the slice rows (k == 1 on level 0, k == 3 on level 1) to
 * slice; length/capacity convention as lbm_write_inputs for both. */
int lbm_format_tecplot(const char* inputs_text, int level, const float* f, const float* stats4, char* buf,
                       size_t cap, size_t* len, char* slice, size_t slice_cap, size_t* slice_len);

/* The .force file text (WriteForces, LR7:2537-2545) of a force history
 * fxyz[3*i + k], i = 0..n-1 for steps STARTF + i, for the record's UMAX,
 * ZDIM, Obst1 radius and refinement level. */
int lbm_format_forces(const char* inputs_text, const double* fxyz, int n, char* buf, size_t cap, size_t* len);

/* ---- handle API: the reference program's main() (LR7:2575-3029) ---- */

/* Parse a .inputs record (the text WriteInputs produces, LR7:2547-2573, plus
 * the DPDY line of MRTtest/DynInlet3.cu and this library's extension keys:
 * GEOMETRY, PRECISION, LAYOUT, TAU, BOUNCEBACK, SGS, CF TIME, ...),
 * allocate both grid levels on the current CUDA device,
 * build the node masks from the configured geometry (ImageFcn / ImageFcnLR)
 * and initialise at equilibrium (initialize / initializeLR, LR7:1060-1125). */
int lbm_create(const char* inputs_text, lbm_handle** out);
int lbm_destroy(lbm_handle* h);

/* nx, ny, nz of a level; nlevels is 2 with refinement, else 1 */
int lbm_get_dims(const lbm_handle* h, int level, int* nx, int* ny, int* nz);
int lbm_get_nlevels(const lbm_handle* h, int* nlevels);
/* relaxation rates (LR7:2607-2619): omega, omegaLR, SF_cf, SF_fc */
int lbm_get_params(const lbm_handle* h, float* omega4);
/* the 19 offsets a level's FP16 / BF16 storage subtracts before rounding
 * (the collision model's equilibrium at density 1 and the reference
 * velocity); zeros for FP32 / FP64.  No counterpart in the reference, which
 * stores FP32 populations (LR7:2676-2678). */
int lbm_get_storage_offsets(const lbm_handle* h, int level, float* off19);
/* steps taken so far */
int lbm_get_time(const lbm_handle* h, int* t);

/* node mask of a level, uint8[nz][ny][nx] of lbm_node values */
int lbm_get_mask(const lbm_handle* h, int level, uint8_t* mask);
int lbm_set_mask(lbm_handle* h, int level, const uint8_t* mask);
/* the base level's geometry (ImageFcn, LR7:88-127): mask as lbm_set_mask on
 * level 0, or NULL for the record's analytic geometry on every level (at
 * the handle's time, for the dynamic inlet's timed trip blocks) */
int lbm_set_geometry(lbm_handle* h, const uint8_t* mask);

/* equilibrium at rho = 1 and the configured initial velocity */
int lbm_init_equilibrium(lbm_handle* h);
int lbm_get_populations(lbm_handle* h, int level, float* f);
int lbm_set_populations(lbm_handle* h, int level, const float* f);

/* Advance n base-grid steps; with refinement every base step runs LRLEVEL
 * patch sub-steps and the two interpolations (the loop of LR7:2849-2950).
 * Steps are captured in batches of 16 into a CUDA graph and replayed
 * (except with the learned closure); the results equal those of single
 * steps bit for bit. */
int lbm_step(lbm_handle* h, int nsteps);
/* Same, timed on the handle's stream with CUDA events; *ms = elapsed time */
int lbm_step_timed(lbm_handle* h, int nsteps, float* ms);
int lbm_synchronize(lbm_handle* h);

/* density and momentum of a level (any pointer may be NULL) */
int lbm_get_fields(lbm_handle* h, int level, float* rho, float* u, float* v, float* w);
/* running statistics (velAv u/v, velFluc u/v: LR7:1018-1058), float[4][nz][ny][nx] */
int lbm_get_stats(lbm_handle* h, int level, float* stats4);

/* momentum-exchange force per step, FP64, fxyz[3*i + k] for step STARTF + i
 * (the reference's FX/FY/FZ arrays, LR7:1607-1626); *n = entries written */
int lbm_get_forces(lbm_handle* h, double* fxyz, int max_steps, int* n);

/* the force of the last step (3 doubles; zeros before STARTF) */
int lbm_get_last_force(lbm_handle* h, double* f3);

/* the same copy queued without waiting, behind the force reduction on the
 * handle's force stream (the step stream does not wait for it): f3 (pinned
 * host memory for a truly asynchronous copy) holds the force once
 * lbm_synchronize returns; lets a monitor read every step's drag without
 * stalling the step loop.  No reference counterpart (the reference copies its
 * force arrays once, after the loop, LR7:2970-2980) */
int lbm_get_last_force_async(lbm_handle* h, double* f3);

/* dynamic inlet (DI3, records with DYNY1): the P-control history, one
 * entry {t, mean v of the plane DYNY1, dpdy after the update} per control
 * step (DI3:3150-3170, its outputAvV file); *n = entries so far, up to
 * max_entries written */
int lbm_get_dyn_history(lbm_handle* h, float* hist3, int max_entries, int* n);

/* number of kernels the handle has launched since lbm_create (all levels,
 * every entry point that takes the handle); instrumentation with no
 * counterpart in the reference */
int lbm_get_launch_count(const lbm_handle* h, long long* n);

/* FP64 mass and momentum of the non-solid nodes of a level: out4 = {M, Jx, Jy, Jz} */
int lbm_audit(lbm_handle* h, int level, double* out4);

/* Profiling: n back-to-back launches of the stream-collide kernel alone on a
 * level (no force, statistics or refinement work; the populations advance n
 * steps but the step counter does not), timed with CUDA events on the
 * handle's stream; *ms = mean duration of one launch. */
int lbm_time_stream_collide(lbm_handle* h, int level, int n, float* ms);

/* ---- run record and outputs (LR7:2350-2573) ---- */

/* the .inputs record of this handle (WriteInputs); returns the length in
 * *len, writes at most cap bytes including the terminating NUL */
int lbm_write_inputs(const lbm_handle* h, char* buf, size_t cap, size_t* len);
/* CASENAME.dat (empty), CASENAME_part<n>.dat, CASENAME_slice.dat,
 * CASENAME.force, CASENAME.inputs (WriteResults, WriteResultsLR,
 * WriteForces, WriteInputs) */
int lbm_write_outputs(lbm_handle* h, const char* casename);
/* the tecplot files alone: CASENAME_part<n>.dat and CASENAME_slice.dat
 * (WriteResults, WriteResultsLR, LR7:2350-2535) */
int lbm_write_tecplot(lbm_handle* h, const char* casename);

/* ---- kernel-level API on caller-owned device buffers ---- */

/* One stream-collide step of a level from device buffer fA into fB: the work
 * of update_inn/update_top/update_bot (LR7:1127-1628) over a single domain
 * with periodic z.  Buffers are float[19][nz][ny][pitch] (pitch a multiple of
 * 32, >= nx, 19*nz*ny*pitch < 2^31), mask uint8[nz][ny][pitch] of lbm_node
 * values.  model: 0 MRT (LR7 mrt_collide), 1 MRT with bgk_meq (DynInlet3),
 * 2 BGK, 3 CPU_3D MRT.  les != 0 folds the Smagorinsky eddy viscosity into
 * tau (cs is the reference's CS).  Enqueued on cuda_stream (NULL: default). */
int lbm_stream_collide_f32(const float* fA, float* fB, const uint8_t* mask, int nx, int ny, int nz, int pitch,
                           int model, int les, float omega, float cs, float u_in, float rho_out, int t,
                           void* cuda_stream);
/* FP64 momentum-exchange force 2 sum_q c_q f_q over the BODY nodes of mask,
 * pulled from fA (the force the reference sums at LR7:1494-1502 and
 * 1607-1626 during the step that reads fA).  The three sums are ADDED to
 * force_out[0..2] (device memory); scratch is device memory of
 * lbm_body_force_scratch_doubles() doubles; the sum order is fixed, so the
 * result is reproducible. */
int lbm_body_force_f32(const float* fA, const uint8_t* mask, int nx, int ny, int nz, int pitch, double* force_out,
                       double* scratch, void* cuda_stream);
size_t lbm_body_force_scratch_doubles(void);

/* lbm_body_force_f32 for callers that cannot allocate device memory (a host
 * framework that has reserved the device memory for its own allocator, a
 * real-time loop that cannot afford cudaMalloc's latency and device-wide
 * synchronisation, a plugin host that forbids allocation calls).  No
 * counterpart in the reference.  Same inputs and output (the three sums are
 * ADDED to force_out), no scratch argument: the partial sums live in a fixed
 * 32 KiB array of the library's own device memory, one per device, held until
 * the process exits.  It never allocates.  The first call on a device looks
 * up that array's address (make the first call before capturing work into a
 * stream).  All calls share the array: calls that overlap on the GPU (other
 * streams, other threads) race and must be serialised by the caller.  The
 * looked-up address is kept for the life of the process, so a device that
 * has been reset (cudaDeviceReset) must not be used with this call again.  Domains
 * whose 19 populations need 2^31 or more elements are rejected (LBM_ERR_ARG),
 * as by lbm_body_force_f32. */
int lbm_body_force_f32_noalloc(const float* fA, const uint8_t* mask, int nx, int ny, int nz, int pitch,
                               double* force_out, void* cuda_stream);

/* ------------------------------------------------------------------------
 * Learned subgrid closure.  No counterpart in the reference (its LES is the
 * constant-Cs Smagorinsky model, LR7:683-685): a per-node MLP
 * 16 -> 64 -> 64 -> 1 (ReLU, softplus output) gives a local Smagorinsky
 * coefficient o = 1e-4 softplus(y) from the node's non-equilibrium stress;
 * the collision's eddy viscosity is nu_t = o * x12 / tau0 = o * 100 |S|
 * (o = 1e-4 is Cs = 0.1).  Parameters are a float vector of
 * lbm_mlp_param_count() entries: W1[64][16] (column 15 = bias), W2[64][64],
 * b2[64], w3[64], b3.  Hidden unit 63 of the first layer is the constant 1
 * (row 63 of W1 takes no part).  Samples are X[n][16] features (x15 = 1) and
 * T[n] target coefficients.
 * ------------------------------------------------------------------------ */
int lbm_mlp_param_count(void);
/* He-uniform hidden weights, Glorot-uniform output weights, zero biases,
 * from a seed (host memory) */
int lbm_mlp_init_params(uint32_t seed, float* params);
/* gradient of the mean squared error of o / 1e-4 over n samples, and the
 * loss; device pointers, synchronous on stream */
int lbm_mlp_grad(const float* d_params, const float* d_X, const float* d_T, int n, float* d_grad, float* d_loss,
                 void* stream);
/* the coefficient o of n samples (FP32 forward on CUDA cores); device
 * pointers, async */
int lbm_mlp_predict(const float* d_params, const float* d_X, int n, float* d_nu, void* stream);
/* Adam (beta 0.9 / 0.999) over seeded shuffled mini-batches of device
 * samples; params (host) in and out, loss_hist[steps] (host, may be NULL) */
int lbm_mlp_train(const float* d_X, const float* d_T, int n, int batch, int steps, float lr, uint32_t seed,
                  float* params, float* loss_hist, void* stream);
/* the coefficient o of n samples through the tensor-core path the collide
 * kernels use:
 * BF16 weights and activations, FP32 accumulation (tcgen05.mma for the two
 * hidden layers, the output layer in FP32), b2 folded into W2 against the
 * constant unit; params in host memory, samples and output on the device;
 * synchronous on stream.
 * Every kernel of this library that uses tensor memory (this call,
 * lbm_tc_selftest, steps of a handle with the learned closure, ensemble steps
 * with it) runs on one internal stream per device, ordered after the
 * caller's stream and before its later work, so such kernels never run side
 * by side: two of them sharing an SM could ask for more than its 512 tensor-
 * memory columns.  Calls from several threads are serialised by a lock. */
int lbm_mlp_predict_tc(const float* params, const float* d_X, int n, float* d_nu, void* stream);
/* the weight blob the tensor-core inference stages in shared memory, from
 * a parameter vector (host memory, lbm_mlp_blob_bytes() bytes):
 * W1 [64][16] with row 63 = e15 (the constant unit), W2 [64][64] with
 * column 63 = W2[:,63] + b2, W3 [16][64] with row 0 = w3 and the rest zero,
 * all bf16 (round to nearest even) in the K-major core-matrix layout (core
 * matrix (i, j), rows 8i..8i+7 and columns 8j..8j+7, at i * SBO + j * 128
 * bytes with SBO 256 for W1 and 1024 for W2 and W3, row r of a core matrix
 * at 16 r), then b3 as FP32 and 12 zero bytes */
size_t lbm_mlp_blob_bytes(void);
int lbm_mlp_make_blob(const float* params, unsigned char* blob);
/* tensor-core self-check: D[128][64] = A[128][16 kc] * B[64][16 kc]^T with
 * BF16 operands (raw 16-bit patterns) and an FP32 accumulator, through
 * tcgen05.mma; kc = 1..4; host pointers */
int lbm_tc_selftest(int kc, const uint16_t* A, const uint16_t* B, float* D);

/* weights of the learned closure for a handle whose record selects
 * "SGS: mlp" (the record may instead name a float32 file in "SGS weights:");
 * the stream-collide then takes its eddy viscosity from the MLP on the
 * tensor cores instead of the Smagorinsky model ("SGS every: k" evaluates it
 * on the steps t % k == 0 and on the first step after weights, populations
 * or a checkpoint were set, and reuses each node's value in between).
 * n = lbm_mlp_param_count() */
int lbm_set_sgs_mlp(lbm_handle* h, const float* params, int n);

/* Checkpoint and restart (no counterpart in the reference, which always
 * starts from the equilibrium).  A checkpoint holds the run record, the time,
 * every level's stored populations as they are (so FP16 / BF16 restart
 * bit-exactly), the statistics, the force history and the closure weights.
 * lbm_restore_state loads one into a handle made from an equivalent record;
 * lbm_create_from_state makes the handle from the record inside the file.
 * Continuing a restored run gives the same bits as never stopping. */
int lbm_save_state(lbm_handle* h, const char* path);
int lbm_restore_state(lbm_handle* h, const char* path);
int lbm_create_from_state(const char* path, lbm_handle** out);

/* ------------------------------------------------------------------------
 * Ensemble of periodic D3Q19 boxes (decaying turbulence), the data source of
 * the learned closure.  No counterpart in the reference, which runs one
 * domain per program; each member uses the reference's MRT collision
 * (LR7:583-711) with periodic streaming.  All members advance together: one
 * persistent kernel launch per step over the tiles of every member, replayed
 * from a captured CUDA graph.  sgs: 0 none, 1 Smagorinsky (cs = Cs^2, as the
 * reference's CS), 2 the learned MLP (lbm_ensemble_set_mlp).
 * ------------------------------------------------------------------------ */
typedef struct lbm_ensemble lbm_ensemble;
/* count members of side sizes[m] (even, 8..1024) and relaxation time tau0[m] */
int lbm_ensemble_create(int count, const int* sizes, const float* tau0, int sgs, float cs, lbm_ensemble** out);
int lbm_ensemble_destroy(lbm_ensemble* e);
/* seeded random-phase solenoidal velocity, E(k) ~ k^-5/3 for k = 1..n/kmax_div
 * with up to per_shell wavevectors per shell, rms u_rms per component;
 * populations at the rho = 1 equilibrium */
int lbm_ensemble_init_turbulence(lbm_ensemble* e, uint32_t seed, float u_rms, int kmax_div, int per_shell);
/* the modes of a member: k3[3n] integer wavevectors, phase[n] (in units of
 * pi), a3[3n] amplitude vectors; *n = count (up to cap written) */
int lbm_ensemble_modes(const lbm_ensemble* e, int member, int* k3, double* phase, double* a3, int cap, int* n);
/* coarse members (half the fine sides) start from the 2x2x2 box filter of
 * the fine members' current velocity */
int lbm_ensemble_init_filtered(lbm_ensemble* coarse, lbm_ensemble* fine);
int lbm_ensemble_set_mlp(lbm_ensemble* e, const float* params);
/* picks tile height and grid size by timing candidates on a copy of the
 * state (the state is unchanged); results are cached per device and shape */
int lbm_ensemble_autotune(lbm_ensemble* e, int* ty, int* grid, float* ms_per_step);
int lbm_ensemble_step(lbm_ensemble* e, int nsteps);
int lbm_ensemble_step_timed(lbm_ensemble* e, int nsteps, float* ms);
int lbm_ensemble_info(const lbm_ensemble* e, int* ty, int* grid, long long* cells, long long* steps);
/* kinetic energy 1/2 <|u|^2> per member (FP64) */
int lbm_ensemble_energy(lbm_ensemble* e, double* E);
/* velocity u[3][n][n][n] of a member */
int lbm_ensemble_velocity(lbm_ensemble* e, int member, float* u3);
/* compact populations f[19][n][n][n] of a member, out and in */
int lbm_ensemble_populations(lbm_ensemble* e, int member, float* f);
int lbm_ensemble_set_populations(lbm_ensemble* e, int member, const float* f);
/* training samples of every member filtered 2x2x2 (features X[.][16] and
 * target nu T[.] on the device, appended at *n, capacity cap); tau0_coarse
 * <= 1/2 takes each member's coarse relaxation time by acoustic scaling */
int lbm_ensemble_samples(lbm_ensemble* e, float tau0_coarse, float* d_X, float* d_T, long long cap, long long* n);

/* ------------------------------------------------------------------------
 * Post-processing of the outputs (host only, no device)
 * ------------------------------------------------------------------------ */
/* ForceCalcs (bgk_channel1/Re3000_Cyl2/ForceCalcs.cpp): mean and RMS of each
 * component of a force history fxyz[3 n] (the values of a .force file) over
 * the lines t_start .. t_end - 1, with that program's FP32 running updates */
int lbm_force_stats(const float* fxyz, int n, int t_start, int t_end, float* mean3, float* rms3);
/* drag coefficient 2 <Fx> / (rho u^2 d lz), RMS lift coefficient, and the
 * Strouhal number f d / u of the lift's dominant frequency, over lines
 * t_start .. n - 1 of raw forces (not normalised); cd, cl_rms, st may be NULL */
int lbm_force_coefficients(const double* fxyz, int n, int t_start, double u, double d, double lz, double rho,
                           double* cd, double* cl_rms, double* st);
/* VelProf (bgk_channel1/Re3000/VelProf.cpp): wall units of a wall-normal
 * line of n nodes: y+ = (i - 1/2) u_tau / nu, v+ = v / u_tau, rms+ =
 * sqrt(fluctuation) / u_tau; any output may be NULL */
int lbm_wall_profile(const float* v_mean, const float* u_fluc, const float* v_fluc, const float* w_fluc, int n,
                     float u_tau, float nu, float* yplus, float* vplus, float* urms, float* vrms, float* wrms);
/* velplus (TurbChannel3/Re500/velplus.cpp:60-112): on the plane z = nz / 2
 * of a level's statistics (lbm_get_stats layout), uave[y] = velAv_u / umax
 * and urms[y] = sqrt(velFluc_u) / umax on x = nx / 2, vave[x], vrms[x] the
 * same of v on y = ny / 2; any output may be NULL */
int lbm_centerline_profiles(const float* stats4, int nx, int ny, int nz, double umax, float* uave, float* urms,
                            float* vave, float* vrms);
/* profiles along y at x of a level's statistics (lbm_get_stats layout
 * float[4][nz][ny][nx]: velAv u, v, velFluc u, v), averaged over z:
 * prof4[4][ny] */
int lbm_stats_profiles(const float* stats4, int nx, int ny, int nz, int x, float* prof4);

#ifdef __cplusplus
}
#endif
#endif
