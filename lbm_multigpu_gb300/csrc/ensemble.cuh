/* Ensemble of periodic D3Q19 boxes: member table and launchers
 * (ensemble.cu; host side in lbm_ensemble.cpp). */
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace lbm {
namespace ens {

constexpr int MAXM = 32;
constexpr int SGS_NONE = 0, SGS_SMAG = 1, SGS_MLP = 2;

struct Member {
    int n;                  /* cube side */
    int pitch;              /* x row length in the buffers, a multiple of 32 */
    unsigned long long off; /* element offset of the member's f[0][0][0][0] in A and B */
    unsigned long long uoff;/* element offset in the compact velocity buffer [3][n][n][n] */
    int tile0;              /* first global tile index */
    int tiles_x, tiles_y;   /* tiles per z plane */
    int mode0, nmodes;      /* the member's rows of the mode table */
    float tau0, omega;
};

struct Table {
    int count;
    int ntiles;
    int ty; /* tile height: a block is 32 x ty threads */
    Member m[MAXM];
};

/* one Fourier mode of the initial field: integer wavevector, phase / pi,
 * amplitude vector orthogonal to k */
struct Mode {
    int k[3];
    double phase;
    double a[3];
};

}  // namespace ens

cudaError_t launch_ens_step(const ens::Table& T, const float* fA, float* fB, int sgs, const void* blob, float cs,
                            int* err, int grid, cudaStream_t s);
int ens_step_occupancy(int ty, int sgs);
cudaError_t launch_ens_init(const ens::Table& T, const ens::Mode* modes, float* fA, float* fB, float* u_out,
                            cudaStream_t s);
cudaError_t launch_ens_init_from(const ens::Table& T, const float* u, float* fA, float* fB, cudaStream_t s);
cudaError_t launch_ens_velocity(const ens::Table& T, const float* f, float* u, cudaStream_t s);
cudaError_t launch_ens_energy(const ens::Table& T, const float* u, double* out, cudaStream_t s);
cudaError_t launch_box_filter(const float* u, int n, double* ubar, double* uu, cudaStream_t s);
cudaError_t launch_d2f(const double* a, float* b, size_t n, cudaStream_t s);
/* two passes: per-cell strain and contractions into s8 (8 * nc^3 doubles),
 * then the 3x3x3-averaged least-squares eddy viscosity and the features */
cudaError_t launch_sgs_targets(const double* ubar, const double* uu, int nc, double tau0, double* s8, float* X,
                               float* T, cudaStream_t s);

}  // namespace lbm
