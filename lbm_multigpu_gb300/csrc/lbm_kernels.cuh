/*
 * lbm_kernels.cuh -- level descriptor and kernel launchers shared by the host
 * library and the kernels (one compilation unit: lbm_kernels.cu).
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lbm {

/* node types of the one-byte mask; numbering shared with include/lbm_gb300.h.
 * In the device copy bit 7 (NEAR_SOLID) marks non-solid nodes with a solid
 * neighbour; the type is mask & TYPE_MASK. */
constexpr uint8_t NEAR_SOLID = 0x80, TYPE_MASK = 0x7F;
enum NodeType : uint8_t {
    FLUID = 0,
    WALL = 1,
    BODY = 2,
    WEST_INLET = 3,
    EAST_OUTLET = 4,
    SOUTH_INLET = 5,
    NORTH_OUTLET = 6,
    LID = 7,
    /* the alternate boundaries of CPU_3D (CPU:411-1140), LR7's x symmetry
     * planes (LR7:899-1016) and BC1's West_Reg (BC1/LRMultiGPU7.cu:789):
     * applied to the pulled populations before the collision */
    DIR_WEST = 8,       /* DirichletWest, CPU_3D im 3 */
    NEU_EAST = 9,       /* NeumannEast_Reg, im 14 */
    NEU_EAST_REG = 10,  /* NeumannEast_Regularized, im 54 */
    XSYM_TOP = 11,      /* xsymmetry_top, x = nx - 1 */
    XSYM_BOT = 12,      /* xsymmetry_bot, x = 0 */
    YSYM_TOP = 13,      /* ysymmetry_top, im 21 */
    YSYM_BOT = 14,      /* ysymmetry_bot, im 22 */
    ZSYM_TOP = 15,      /* zsymmetry_top, im 23 */
    ZSYM_BOT = 16,      /* zsymmetry_bot, im 24 */
    WEST_REG = 17,      /* BC1 West_Reg */
    DIR_WEST_V = 18,    /* DirichletWest_Reg, im 13: tangential v on x = 0 */
    DIR_NORTH = 19,     /* DirichletNorth_Reg: y = ny - 1 moving in x */
    DIR_SOUTH = 20,     /* DirichletSouth_Reg: y = 0 moving in x */
    NODE_TYPES = 21
};

/* collision models: LR7 mrt_collide, DynInlet3's MRT (bgk_meq + AddForce),
 * BGK, CPU_3D's MRT */
enum Model : int { MRT = 0, MRT_DI3 = 1, BGK = 2, MRT_CPU3D = 3 };

enum Storage : int { STORE_F32 = 0, STORE_F16 = 1, STORE_BF16 = 2, STORE_F64 = 3 };

/* One grid level in HBM.  Nodes are numbered c = z plane + y pitch + x with
 * a padded x pitch (a multiple of 32).  Populations are stored either
 *   0, structure-of-arrays: f[q][z][y][x], q-planes qstride elements apart
 *     (the reference's layout, LR7:210-216), or
 *   1, blocked: the 32 nodes x = 32 b .. 32 b + 31 of a row keep their 19
 *     populations together in 19 x 32 elements, population 0 of lane l at
 *     l, then the nine opposite pairs (q, opp(q)) interleaved, pair k at
 *     32 + 64 k + 2 l (+1 for the second member), so that a node stores a
 *     pair with one wide store and the offset of a population from the
 *     node's block position is a compile-time constant. */
struct Level {
    int nx, ny, nz;
    int pitch;            /* elements per row, a multiple of 32 */
    long long plane;      /* pitch * ny */
    long long qstride;    /* plane * nz */
    int storage;          /* Storage */
    int blocked;          /* 0: structure-of-arrays, 1: blocked */
    float off[19];        /* FP16/BF16 store f - off[q] (equilibrium at the reference velocity) */
    float u_ref;          /* that reference velocity (along x) */
};

/* elements of one 32-node block of the blocked layout */
constexpr unsigned BLOCK_ELEMS = 19u * 32u;

/* The FP32 structure-of-arrays level of the kernel-level API (caller-owned
 * buffers in the reference's layout, no storage offsets).  Returns 1 for bad
 * dimensions or pitch, 2 when 19 populations would not index below 2^31,
 * else 0 with L filled in. */
inline int f32_kernel_level(Level& L, int nx, int ny, int nz, int pitch) {
    if (nx < 1 || ny < 1 || nz < 1 || pitch < nx || pitch % 32) return 1;
    if ((long long)pitch * ny * nz * 19 >= (1LL << 31)) return 2;
    L = Level{};
    L.nx = nx;
    L.ny = ny;
    L.nz = nz;
    L.pitch = pitch;
    L.plane = (long long)pitch * ny;
    L.qstride = L.plane * nz;
    L.storage = STORE_F32;
    L.blocked = 0;
    return 0;
}

/* the pairs of the blocked layout: (q, opp(q)) for the first members
 * 1, 2, 9, 5, 6, 10, 12, 11, 13 */
__host__ __device__ constexpr int pair_first(int k) {
    return k == 0 ? 1 : k == 1 ? 2 : k == 2 ? 9 : k == 3 ? 5 : k == 4 ? 6 : k == 5 ? 10 : k == 6 ? 12 : k == 7 ? 11 : 13;
}
__host__ __device__ constexpr int pair_of(int q) {
    return (q == 1 || q == 3) ? 0 : (q == 2 || q == 4) ? 1 : (q == 9 || q == 14) ? 2 : (q == 5 || q == 7) ? 3 :
           (q == 6 || q == 8) ? 4 : (q == 10 || q == 17) ? 5 : (q == 12 || q == 15) ? 6 : (q == 11 || q == 18) ? 7 : 8;
}
__host__ __device__ constexpr int pair_slot(int q) {
    return (q == 3 || q == 4 || q == 14 || q == 7 || q == 8 || q == 17 || q == 15 || q == 18 || q == 16) ? 1 : 0;
}
/* offset of population q from its block's start, lane 0 */
__host__ __device__ constexpr unsigned pair_qoff(int q) {
    return q == 0 ? 0u : 32u + 64u * unsigned(pair_of(q)) + unsigned(pair_slot(q));
}

/* element offset of population q of node c in either layout */
__host__ __device__ __forceinline__ unsigned pidx(const Level& L, int q, unsigned c) {
    if (L.blocked) return (c >> 5) * BLOCK_ELEMS + pair_qoff(q) + (q == 0 ? 1u : 2u) * (c & 31u);
    return unsigned(q) * unsigned(L.qstride) + c;
}

struct StepParams {
    int model;
    int les;
    float omega, cs, dpdy;
    /* derived by launch_stream_collide: 1 / omega and 18 sqrt(2) cs, the
     * constants of the Smagorinsky relaxation (LR7:683-685) */
    float tau0, smag_k;
    /* dynamic inlet (DI3): when dpdy_dev is set the body force is read from
     * the device (the P-control updates it there); nodes with y > dyn_y1 get
     * no body force (DI3:1358) */
    const float* dpdy_dev;
    int dyn_y1;
    int has_xbc; /* the level holds alternate-boundary nodes (DIR_WEST ..) */
    float u_in, rho_out;
    float lid_u[3];
    int lid_face;
    int lid_quirk;         /* CPU_3D's regularised lid as written (CPU:1010-1023) */
    int pull_clamp;        /* pulls from outside the domain clamp to the edge (CPU:1369-1388) instead of wrapping */
    int halfway;           /* half-way bounce-back: a pull from a solid node returns the node's own
                            * opposite post-collision population; solids are not updated */
    int has_lid;           /* the level's mask contains LID nodes */
    int force_on;          /* accumulate momentum exchange at BODY nodes */
    int t;                 /* time step index (stats, noise) */
    int stats_on, start_av, start_fluc;
    float stats_weight;
    float noise_amp;
    uint32_t noise_seed;
    /* coarse-moment export for the coarse->fine interpolation */
    int exp_x0, exp_y0, exp_nx, exp_ny;
    /* the learned closure refreshed every k steps: its stream-collide writes
     * each node's eddy viscosity here (when non-null), and the steps between
     * refreshes (nu_reuse) relax at tau0 + 3 nu[c] in the plain kernel */
    float* nu;
    int nu_reuse;
};

/* launch configuration of the stream-collide kernel: a warp per row, 4 rows
 * per block (measured on 512x128x128 against 32 x {1, 2, 8, 16}: fastest
 * for FP32 and FP16 storage) */
constexpr int SC_BX = 32, SC_BY = 4;

inline dim3 sc_grid(const Level& L) { return dim3(L.pitch / SC_BX, (L.ny + SC_BY - 1) / SC_BY, L.nz); }
inline int sc_blocks(const Level& L) {
    dim3 g = sc_grid(L);
    return int(g.x * g.y * g.z);
}

/* kernel launchers (lbm_kernels.cu) */
/* links: per node, bit q set when the pull source of population q is a solid
 * node (read only by NEAR_SOLID nodes; needed for half-way bounce-back) */
cudaError_t launch_stream_collide(const Level& L, const StepParams& p, const void* fA, void* fB,
                                  const uint8_t* mask, float* stats, float* mom_export, cudaStream_t s,
                                  const uint32_t* links = nullptr);
/* the same step with the learned closure (tensor-core MLP) in place of the
 * Smagorinsky model; blob = weights (sgs::BLOB_BYTES), err = device flag set
 * to 2 when an MMA completion wait ran out.  Channel features only: no lid,
 * no clamped edges, no refinement export; FP32 / FP16 / BF16 storage */
cudaError_t launch_stream_collide_mlp(const Level& L, const StepParams& p, const void* fA, void* fB,
                                      const uint8_t* mask, float* stats, const uint32_t* links, const void* blob,
                                      int* err, cudaStream_t s);
/* FP64 momentum exchange over a list of BODY nodes (pitched indices), ADDED to out3 */
cudaError_t launch_force(const Level& L, const void* fA, const unsigned* body, int nbody, double* partials,
                         unsigned* done, double* out3, cudaStream_t s, const uint8_t* mask = nullptr,
                         int halfway = 0);
int force_partials();
/* the same sum found by scanning the mask; partials holds force_scan_partials()*3 doubles */
cudaError_t launch_force_scan(const Level& L, const void* fA, const uint8_t* mask, double* partials, double* out3,
                              cudaStream_t s);
int force_scan_partials();

/* The tensor-memory lane of the current device.  Every kernel of this
 * library that allocates tensor memory (TMEM) is launched on one stream per
 * device, ordered after the caller's stream and before the caller's later
 * work by events, so that no two of them run at the same time on a device.
 * Each such kernel sizes its shared memory so that its own resident blocks
 * never ask an SM for more than its 512 TMEM columns; two different ones
 * side by side could, and tcgen05.alloc would then wait for columns.  The
 * lane is held (a host mutex) from construction to destruction. */
class TmemLane {
public:
    explicit TmemLane(cudaStream_t caller);
    ~TmemLane();
    TmemLane(const TmemLane&) = delete;
    TmemLane& operator=(const TmemLane&) = delete;
    cudaStream_t stream() const { return lane_; }
    cudaError_t status() const { return err_; }
    /* creates the current device's lane, before any stream capture that
     * will use it */
    static cudaError_t prepare();

private:
    cudaStream_t caller_ = nullptr, lane_ = nullptr;
    cudaEvent_t done_ = nullptr;
    int dev_ = -1;
    cudaError_t err_ = cudaSuccess;
};

/* record an error for lbm_last_error(); returns code (lbm_host.cpp) */
int set_error(int code, const char* what, cudaError_t e);
/* axis: direction of the initial velocity u0 (0 x, 1 y, 2 z) */
cudaError_t launch_init(const Level& L, const uint8_t* mask, void* f, int kind, float u0, cudaStream_t s,
                        int axis = 0);
/* DI3 P-control (DI3:2561-2598, 3150-3170), on the device: the mean y
 * momentum of the plane y1 over (nx - 2) nz nodes, then
 * dpdy += (mean - umax) / umax * kp * |dpdy0|; hist3 gets {t, mean, dpdy} */
cudaError_t launch_dyn_control(const Level& L, const void* f, int y1, float umax, float kp, float dpdy0_abs,
                               float* dpdy_dev, float* hist3, int t, cudaStream_t s);
cudaError_t launch_fields(const Level& L, const void* f, float* rho, float* u, float* v, float* w, cudaStream_t s);
cudaError_t launch_pack(const Level& L, const void* f, float* compact, cudaStream_t s);
cudaError_t launch_unpack(const Level& L, const float* compact, void* f, cudaStream_t s);
cudaError_t launch_audit(const Level& L, const void* f, const uint8_t* mask, double* partials, int npart,
                         double* out4, cudaStream_t s);
int audit_partials(const Level& L);

struct RefineParams {
    int cnx, cny, cnz;
    int fnx, fny, fnz;
    float lrx0, lry0, lrz0;
    float lrfactor;
    int lrlevel;
    int order;
    float cs;
    float omega_c, omega_f;
    int quirk_fc_top_zflip;
    int enx, eny;          /* exported coarse-moment footprint */
    /* a patch bounded in z (an extension; the reference's spans the
     * periodic z extent): z is treated like x and y, the fine node k at
     * coarse z lrz0 + k lrfactor with cz0 = int(lrz0) */
    int zbounded, cz0;
};

/* mom_prev: the previous coarse export, blended in time with weight theta
 * on mom_c (linear temporal interpolation); null: mom_c alone */
cudaError_t launch_interp_cf(const RefineParams& r, const Level& F, const float* mom_c, void* f_f,
                             const uint8_t* mask_f, cudaStream_t s, const float* mom_prev = nullptr,
                             float theta = 1.f);
cudaError_t launch_interp_fc(const RefineParams& r, const Level& C, const Level& F, const void* f_f, void* f_c,
                             const uint8_t* mask_c, cudaStream_t s);
/* the final band fill of a coarse step (from mom_c alone) and the
 * restriction in one launch (they touch disjoint nodes) */
cudaError_t launch_interface(const RefineParams& r, const Level& C, const Level& F, const float* mom_c, void* f_f,
                             const uint8_t* mask_f, void* f_c, const uint8_t* mask_c, cudaStream_t s);

/* learned subgrid closure (sgs_mlp.cu) */
int mlp_grad_blocks(int n);
/* per-block partial gradients (+ loss) of the mean loss over n samples */
cudaError_t launch_mlp_grad(const float* params, const float* X, const float* T, const int* idx, int n,
                            float* grad_part, int nblocks, cudaStream_t s);
/* sums the partials; with step > 0 also one Adam step on params (m, v state) */
cudaError_t launch_mlp_adam(const float* grad_part, int nblocks, float* params, float* m, float* v, float* grad_out,
                            float* loss_out, float lr, int step, cudaStream_t s);
cudaError_t launch_mlp_predict(const float* params, const float* X, int n, float* nu, cudaStream_t s);
cudaError_t launch_tc_selftest(const void* A, const void* B, int kc, float* D, int* err, cudaStream_t s);
/* tensor-core inference of n samples from a weight blob (sgs::BLOB_BYTES, see
 * mlp_make_blob); err gets 2 when an MMA completion wait ran out */
cudaError_t launch_mlp_predict_tc(const void* blob, const float* X, int n, float* nu, int* err, cudaStream_t s);
/* host: the device weight blob of a parameter vector (lbm_sgs.cpp) */
void mlp_make_blob(const float* params, unsigned char* blob);

}  // namespace lbm
