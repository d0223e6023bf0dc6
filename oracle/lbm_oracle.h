/*
 * lbm_oracle.h -- CPU restatement of the reference's D3Q19 stream-collide path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path is
 * compared against.  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg may load it.  The product (liblbm_gb300.so) never links or
 * calls it.
 *
 * Parity status: pinned.  The per-cell functions are checked against the
 * reference's own device math compiled for the host (oracle/ref_recipe.py
 * stages LRTurbTest/LRMultiGPU7.cu and MRTtest/DynInlet3.cu into oracle/_ref),
 * through the committed golden vectors in tests/golden/, and the whole-step
 * loop against the reference's GPU program output fixtures.
 *
 * Layout: populations are compact structure-of-arrays, f[q][z][y][x], no pitch.
 * Lattice: D3Q19 in the reference's ordering (LRTurbTest/LRMultiGPU7.cu:258-279):
 *   0:(0,0,0) 1:(1,0,0) 2:(0,1,0) 3:(-1,0,0) 4:(0,-1,0) 5:(1,1,0) 6:(-1,1,0)
 *   7:(-1,-1,0) 8:(1,-1,0) 9:(0,0,1) 10:(1,0,1) 11:(0,1,1) 12:(-1,0,1)
 *   13:(0,-1,1) 14:(0,0,-1) 15:(1,0,-1) 16:(0,1,-1) 17:(-1,0,-1) 18:(0,-1,-1)
 */
#ifndef LBM_ORACLE_H
#define LBM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* node types: shared numbering with the product (include/lbm_gb300.h) */
enum {
    ORC_FLUID = 0,        /* ImageFcn 0 */
    ORC_WALL = 1,         /* ImageFcn 1: full-way bounce-back, no force */
    ORC_BODY = 2,         /* ImageFcn 10: full-way bounce-back + momentum exchange */
    ORC_WEST_INLET = 3,   /* ImageFcn 400: West_Extrap, LR7:852-897 */
    ORC_EAST_OUTLET = 4,  /* ImageFcn 300: East_Extrap, LR7:805-850 */
    ORC_SOUTH_INLET = 5,  /* ImageFcn 200: South_Extrap, LR7:760-803 */
    ORC_NORTH_OUTLET = 6, /* ImageFcn 100: North_Extrap, LR7:713-758 */
    ORC_LID = 7,          /* moving lid, regularised Dirichlet (CPU_3D/CPU_3D.cpp:974-1054) */
    /* alternate boundaries (CPU_3D/CPU_3D.cpp:411-1140, LRTurbTest/LRMultiGPU7.cu:899-1016,
     * BC1/LRMultiGPU7.cu:789), applied to the pulled populations before the collision */
    ORC_DIR_WEST = 8,     /* DirichletWest, CPU_3D im 3 */
    ORC_NEU_EAST = 9,     /* NeumannEast_Reg, im 14 */
    ORC_NEU_EAST_REG = 10,/* NeumannEast_Regularized, im 54 */
    ORC_XSYM_TOP = 11,    /* xsymmetry_top (LR7) */
    ORC_XSYM_BOT = 12,    /* xsymmetry_bot (LR7) */
    ORC_YSYM_TOP = 13,    /* ysymmetry_top, im 21 */
    ORC_YSYM_BOT = 14,    /* ysymmetry_bot, im 22 */
    ORC_ZSYM_TOP = 15,    /* zsymmetry_top, im 23 */
    ORC_ZSYM_BOT = 16,    /* zsymmetry_bot, im 24 */
    ORC_WEST_REG = 17,    /* BC1 West_Reg */
    ORC_DIR_WEST_V = 18,  /* DirichletWest_Reg, im 13 (x = 0, velocity (0, u, 0)) */
    ORC_DIR_NORTH = 19,   /* DirichletNorth_Reg (y = ny - 1, velocity (u, 0, 0)) */
    ORC_DIR_SOUTH = 20    /* DirichletSouth_Reg (y = 0, velocity (u, 0, 0)) */
};

/* collision models */
enum {
    ORC_MRT = 0,      /* LR7 mrt_collide, LR7:583-711 */
    ORC_MRT_DI3 = 1,  /* DynInlet3 MRT branch with bgk_meq, MRTtest/DynInlet3.cu:770-789 */
    ORC_BGK = 2,      /* DynInlet3 / CPU_3D BGK, MRTtest/DynInlet3.cu:806-827 */
    ORC_MRT_CPU3D = 3 /* CPU_3D mrt_collide, CPU_3D/CPU_3D.cpp:164-409 */
};

typedef struct {
    int nx, ny, nz;        /* level dimensions (compact arrays) */
    int model;             /* ORC_MRT / ORC_MRT_DI3 / ORC_BGK */
    int les;               /* Smagorinsky folded into tau_eff (LR7:610-686) */
    float omega;           /* 1/tau0 of this level */
    float cs;              /* the reference's CS (it enters as Cs^2, LR7:684) */
    float dpdy;            /* body force of the dynamic-inlet variant (DI3:229-252) */
    float u_in;            /* inlet velocity (PoisProf3D returns UMAX, LR7:135-143) */
    float rho_out;         /* outlet density (1.0 in the reference) */
    float lid_u[3];        /* lid velocity for ORC_LID nodes */
    int lid_face;          /* 0:-x 1:+x 2:-y 3:+y 4:-z 5:+z */
    int force_on;          /* accumulate momentum exchange at ORC_BODY nodes */
    /* statistics (LR7:1018-1058, 1567-1584) */
    int stats_on;
    int t;
    int start_av, start_fluc;
    float stats_weight;    /* 1 on the coarse level, LRFACTOR on the fine level */
    /* moment export footprint for the coarse->fine interpolation (LR7:1590-1605) */
    int exp_x0, exp_y0, exp_nx, exp_ny;   /* exp_nx == 0: off */
    /* inlet noise (extension, off in parity runs) */
    float noise_amp;
    uint32_t noise_seed;
    /* CPU_3D semantics: pulls from outside the domain clamp to the edge
     * (dmin/dmax, CPU:1369-1388); the lid as written (CPU:1010-1023) */
    int pull_clamp;
    int lid_quirk;
    /* half-way bounce-back (extension; the reference is full-way) */
    int halfway;
    /* learned subgrid closure (sgs_oracle.cpp): when non-null, the collision
     * of fluid and boundary nodes takes nu_t from this MLP parameter vector
     * (MRT at tau0 + 3 nu_t) instead of the model / LES settings */
    const float* mlp;
    /* dynamic inlet (DI3:1358): no body force for y > dyn_y1; a large value
     * switches the cut off */
    int dyn_y1;
    /* the closure refreshed every mlp_every steps: on steps t with
     * t % mlp_every == 0 the MLP's nu_t of each node goes to mlp_nu[node]
     * (compact index), the other steps relax at tau0 + 3 mlp_nu[node];
     * mlp_every <= 1 or mlp_nu null: the MLP on every step */
    int mlp_every;
    double* mlp_nu;
} orc_params;

typedef struct {
    /* coarse and fine dimensions */
    int cnx, cny, cnz;
    int fnx, fny, fnz;
    float lrx0, lry0, lrz0;   /* fine origin in coarse coordinates */
    float lrfactor;           /* fine spacing / coarse spacing (0.5) */
    int lrlevel;              /* 1/lrfactor */
    int order;                /* 1 or 2 (LR7: ORDER) */
    float cs;
    float omega_c, omega_f;
    int quirk_fc_top_zflip;   /* reproduce LR7:2195-2229 corner order on the top plane */
    /* a patch bounded in z (an extension): z as x and y from coarse plane
     * cz0 = int(lrz0); 0 for the reference's periodic full-depth patch */
    int zbounded, cz0;
} orc_refine;

/* per-cell kernels on arrays of n cells stored cell-major (n x 19) */
void orc_collide(int model, int les, float omega, float cs, float dpdy, float* f, int n);
void orc_collide_d(int model, int les, double omega, double cs, double dpdy, double* f, int n);
void orc_extrap(int kind, float* f, int n, float rho, float u_in);
void orc_moments(const float* f, float* m, int n);
void orc_physical_moments(const float* f, float* mom, int n);
void orc_strain_rate(const float* mom, float* s, int n);
void orc_invert_les_cf(const float* mom, float* f, int n, float omega_c, float cs, float lrfactor);
void orc_invert_les_fc(const float* mom, float* f, int n, float omega_f, float cs, float lrfactor);
void orc_lid(float* f, int n, int face, float ux, float uy, float uz, int quirk);
/* an alternate boundary of node type on n cells at (y, z) = yz[2i], yz[2i+1]
 * of an ny x nz domain; u the inlet velocity, t the step */
void orc_alt_boundary(int type, float* f, int n, const int* yz, int ny, int nz, float u, int t);

/* whole-level operations on compact SoA arrays */
void orc_init(const orc_params* p, const uint8_t* mask, float* f, int kind, float u0);
void orc_step(const orc_params* p, const uint8_t* mask, const float* fA, float* fB,
              double* force3, float* av_u, float* av_v, float* fl_u, float* fl_v,
              float* mom_export);
void orc_step_d(const orc_params* p, const uint8_t* mask, const double* fA, double* fB,
                double* force3);
void orc_interp_cf(const orc_refine* r, const float* mom_c, float* f_f, const uint8_t* mask_f);
void orc_interp_fc(const orc_refine* r, const float* f_f, float* f_c, const uint8_t* mask_c);

/* geometry (restatement of ImageFcn variants, LR7:68-127, CPU_3D/CPU_3D.cpp:39-74) */
void orc_mask_channel(uint8_t* mask, int nx, int ny, int nz, int body_shape,
                      float ox, float oy, float r);
void orc_mask_fine(uint8_t* mask, int nx, int ny, int nz, float x0, float y0, float z0,
                   float h, int body_shape, float ox, float oy, float r);
void orc_mask_cavity(uint8_t* mask, int nx, int ny, int nz, int lid_face);
/* DI3's ImageFcn (DI3:72-90): trip blocks around (ox, oy) of half-width r,
 * the second shifted by 3 and only in z = 10, while trip != 0; walls at
 * x = 0 and nx - 1 */
void orc_mask_dyninlet(uint8_t* mask, int nx, int ny, int nz, float ox, float oy, float r, int trip);
/* orc_init with the initial velocity along axis (0 x, 1 y, 2 z) */
void orc_init_axis(const orc_params* p, const uint8_t* mask, float* f, int kind, float u0, int axis);

/* helpers */
double orc_mass(const float* f, const uint8_t* mask, int ncell);
uint32_t orc_noise_hash(uint32_t seed, uint32_t cell, uint32_t step);
float orc_noise_uniform(uint32_t seed, uint32_t cell, uint32_t step);
int orc_num_threads(void);
/* learned subgrid closure (sgs_oracle.cpp) */
void orc_collide_mlp(const float* params, double tau0, double* f, int n, double* nu_out);
void orc_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
