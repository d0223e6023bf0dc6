/* CPU oracle of the learned subgrid closure (test infrastructure only: the
 * checker of the GPU training, inference and data-generation kernels, never
 * a product path).  Double precision throughout, plain loops.
 *
 * The closure is not part of the reference (its LES is the constant-Cs
 * Smagorinsky model of LRTurbTest/LRMultiGPU7.cu:683-685); this file restates
 * the definitions the GPU code implements:
 *   MLP 16 -> 64 -> 64 -> 1, ReLU, softplus output, hidden unit 63 of
 *   the first layer the constant 1 (row 63 of W1 takes no part),
 *   coefficient o = 1e-4 * softplus(y), eddy viscosity in the collision
 *   nu_t = o * x12 / tau0 (o * 100 |S|); loss = mean over samples of
 *   (softplus(y) - o_target / 1e-4)^2;
 *   features of p_ij = -3/2 Pi_neq_ij / rho and tau0 (x0..x15: x0..x11 = 0,
 *   x12 = |p|, x13 = tr(p^3) / |p|^3, x14 = (tau0 - 1/2) 100, x15 = 1);
 *   box filter of a fine velocity field onto the coarse grid and the
 *   least-squares eddy viscosity of the filtered subgrid stress, its
 *   contractions averaged over 3x3x3 coarse cells.
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {
constexpr int NIN = 16, NH = 64, HC = NH - 1;
constexpr int OFF_W1 = 0, OFF_W2 = OFF_W1 + NH * NIN, OFF_B2 = OFF_W2 + NH * NH, OFF_W3 = OFF_B2 + NH,
              OFF_B3 = OFF_W3 + NH, NPARAM = OFF_B3 + 1;
constexpr double P_REF = 0.01, NU_SCALE = 1e-4;
double relu(double z, double* dg) {
    if (dg) *dg = z > 0 ? 1 : 0;
    return z > 0 ? z : 0;
}
double softplus(double y) { return y > 30 ? y : std::log1p(std::exp(y)); }
double sigmoid(double y) { return 1 / (1 + std::exp(-y)); }

struct Fwd {
    double z1[NH], h1[NH], g1[NH], z2[NH], h2[NH], g2[NH], y;
};

void forward(const float* P, const float* x, Fwd& a) {
    for (int j = 0; j < NH; ++j) {
        double z = 0;
        for (int k = 0; k < NIN; ++k) z += double(P[OFF_W1 + j * NIN + k]) * x[k];
        a.z1[j] = z;
        a.h1[j] = relu(z, &a.g1[j]);
    }
    a.h1[HC] = 1, a.g1[HC] = 0;
    a.y = P[OFF_B3];
    for (int j = 0; j < NH; ++j) {
        double z = P[OFF_B2 + j];
        for (int k = 0; k < NH; ++k) z += double(P[OFF_W2 + j * NH + k]) * a.h1[k];
        a.z2[j] = z;
        a.h2[j] = relu(z, &a.g2[j]);
        a.y += double(P[OFF_W3 + j]) * a.h2[j];
    }
}
/* the GPU inference's rounding (orc_mlp_set_bf16): features, W1, W2 (with
 * b2 added to its column HC, the constant hidden unit) and w3 rounded to
 * bf16 (nearest even), the first hidden layer rounded to bf16 after the
 * ReLU, the layers summed in FP64 and read as FP32, the output layer
 * y = b3 + sum_j w3_j relu(z2_j) as a chain of FP32 fused multiply-adds in
 * j order */
bool g_bf16 = false;
float bf16(float v) {
    uint32_t u;
    std::memcpy(&u, &v, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

double forward_bf16(const float* P, const float* x) {
    double h1[NH];
    for (int j = 0; j < NH; ++j) {
        double z = 0;
        for (int k = 0; k < NIN; ++k) z += double(bf16(P[OFF_W1 + j * NIN + k])) * double(bf16(x[k]));
        h1[j] = double(bf16(float(z > 0 ? z : 0)));
    }
    h1[HC] = 1;
    float y = P[OFF_B3];
    for (int j = 0; j < NH; ++j) {
        double z = 0;
        for (int k = 0; k < NH; ++k) {
            const float w = k == HC ? P[OFF_W2 + j * NH + k] + P[OFF_B2 + j] : P[OFF_W2 + j * NH + k];
            z += double(bf16(w)) * h1[k];
        }
        const float z2 = float(z);
        y = std::fma(bf16(P[OFF_W3 + j]), z2 > 0 ? z2 : 0.f, y);
    }
    return y;
}
}  // namespace

extern "C" {

int orc_mlp_nparam(void) { return NPARAM; }

/* 1: the closure's forward follows the GPU inference's bf16 rounding
 * (forward_bf16), 0: FP64 */
void orc_mlp_set_bf16(int on) { g_bf16 = on != 0; }

void orc_sgs_features(const double* p, double tau0, double* x) {
    double pp = 0;
    for (int i = 0; i < 3; ++i) pp += p[i] * p[i];
    for (int i = 3; i < 6; ++i) pp += 2 * p[i] * p[i];
    /* full symmetric tensor, trace of its cube */
    const double m[3][3] = {{p[0], p[3], p[4]}, {p[3], p[1], p[5]}, {p[4], p[5], p[2]}};
    double tr3 = 0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) tr3 += m[i][j] * m[j][k] * m[k][i];
    for (int i = 0; i < 12; ++i) x[i] = 0; /* reserved: the inputs are invariants of p only */
    x[12] = std::sqrt(2 * pp) / P_REF;
    x[13] = pp > 1e-30 ? tr3 / std::pow(pp, 1.5) : 0;
    x[14] = (tau0 - 0.5) * 100;
    x[15] = 1;
}

/* the network's coefficient o of n samples X[n][16] (the collision's eddy
 * viscosity is o * x12 / tau0) */
void orc_mlp_forward(const float* params, const float* X, int n, double* nu) {
    Fwd a;
    for (int i = 0; i < n; ++i) {
        if (g_bf16) {
            nu[i] = NU_SCALE * softplus(forward_bf16(params, X + size_t(i) * NIN));
            continue;
        }
        forward(params, X + size_t(i) * NIN, a);
        nu[i] = NU_SCALE * softplus(a.y);
    }
}

/* gradient of the mean loss over the n samples (grad[NPARAM]) and the loss */
void orc_mlp_grad(const float* params, const float* X, const float* T, int n, double* grad, double* loss) {
    std::memset(grad, 0, sizeof(double) * NPARAM);
    double L = 0;
    Fwd a;
    for (int i = 0; i < n; ++i) {
        const float* x = X + size_t(i) * NIN;
        forward(params, x, a);
        const double err = softplus(a.y) - double(T[i]) / NU_SCALE;
        L += err * err / n;
        const double dy = 2 * err / n * sigmoid(a.y);
        grad[OFF_B3] += dy;
        double dz2[NH];
        for (int j = 0; j < NH; ++j) {
            grad[OFF_W3 + j] += dy * a.h2[j];
            dz2[j] = dy * double(params[OFF_W3 + j]) * a.g2[j];
            grad[OFF_B2 + j] += dz2[j];
            for (int k = 0; k < NH; ++k) grad[OFF_W2 + j * NH + k] += dz2[j] * a.h1[k];
        }
        for (int k = 0; k < NH; ++k) {
            double d = 0;
            for (int j = 0; j < NH; ++j) d += double(params[OFF_W2 + j * NH + k]) * dz2[j];
            const double dz1 = d * a.g1[k];
            for (int c = 0; c < NIN; ++c) grad[OFF_W1 + k * NIN + c] += dz1 * x[c];
        }
    }
    *loss = L;
}

void orc_collide_d(int model, int les, double omega, double cs, double dpdy, double* f, int n);

/* density and Pi_neq = sum c c f - rho/3 I - j j (xx, yy, zz, xy, xz, yz) */
void orc_pi_neq(const double* f, double* rho, double* p) {
    static const int CX[19] = {0, 1, 0, -1, 0, 1, -1, -1, 1, 0, 1, 0, -1, 0, 0, 1, 0, -1, 0};
    static const int CY[19] = {0, 0, 1, 0, -1, 1, 1, -1, -1, 0, 0, 1, 0, -1, 0, 0, 1, 0, -1};
    static const int CZ[19] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, -1, -1, -1, -1, -1};
    double r = 0, j[3] = {0, 0, 0}, m[6] = {0, 0, 0, 0, 0, 0};
    for (int q = 0; q < 19; ++q) {
        const double c[3] = {double(CX[q]), double(CY[q]), double(CZ[q])};
        r += f[q];
        for (int a = 0; a < 3; ++a) j[a] += c[a] * f[q];
        m[0] += c[0] * c[0] * f[q], m[1] += c[1] * c[1] * f[q], m[2] += c[2] * c[2] * f[q];
        m[3] += c[0] * c[1] * f[q], m[4] += c[0] * c[2] * f[q], m[5] += c[1] * c[2] * f[q];
    }
    *rho = r;
    p[0] = m[0] - r / 3 - j[0] * j[0];
    p[1] = m[1] - r / 3 - j[1] * j[1];
    p[2] = m[2] - r / 3 - j[2] * j[2];
    p[3] = m[3] - j[0] * j[1];
    p[4] = m[4] - j[0] * j[2];
    p[5] = m[5] - j[1] * j[2];
}

/* the learned closure in the collision: per node (AoS f[n][19]) Pi_neq ->
 * p = -3/2 Pi_neq / rho -> features -> MLP -> coefficient o, eddy viscosity
 * nu_t = o * x12 / tau0 (o G |S|, G = 1 / P_REF), then the LR7 MRT collision
 * (model 0, no Smagorinsky) at 1 / (tau0 + 3 nu_t); nu_out[n] = nu_t */
void orc_collide_mlp(const float* params, double tau0, double* f, int n, double* nu_out) {
    for (int i = 0; i < n; ++i) {
        double* g = f + 19L * i;
        double rho, p[6], x[16];
        orc_pi_neq(g, &rho, p);
        for (double& v : p) v *= -1.5 / rho;
        orc_sgs_features(p, tau0, x);
        float xf[16];
        for (int k = 0; k < 16; ++k) xf[k] = float(x[k]);
        double y;
        if (g_bf16) {
            y = forward_bf16(params, xf);
        } else {
            Fwd a;
            forward(params, xf, a);
            y = a.y;
        }
        const double nu = NU_SCALE * softplus(y) * x[12] / tau0;
        if (nu_out) nu_out[i] = nu;
        orc_collide_d(0, 0, 1 / (tau0 + 3 * nu), 0, 0, g, 1);
    }
}

/* 2x2x2 box filter of a fine periodic velocity field (u[3][fz][fy][fx]) onto
 * the coarse grid: ubar[3][cz][cy][cx], and the filtered products
 * uu[6][...] (xx, yy, zz, xy, xz, yz) */
void orc_box_filter(const float* u, int fx, int fy, int fz, double* ubar, double* uu) {
    const int cx = fx / 2, cy = fy / 2, cz = fz / 2;
    const size_t fn = size_t(fx) * fy * fz, cn = size_t(cx) * cy * cz;
    for (int z = 0; z < cz; ++z)
        for (int y = 0; y < cy; ++y)
            for (int x = 0; x < cx; ++x) {
                double s[3] = {0, 0, 0}, p[6] = {0, 0, 0, 0, 0, 0};
                for (int c = 0; c < 8; ++c) {
                    const size_t i = (size_t(2 * z + (c >> 2)) * fy + 2 * y + ((c >> 1) & 1)) * fx + 2 * x + (c & 1);
                    const double a = u[i], b = u[fn + i], d = u[2 * fn + i];
                    s[0] += a, s[1] += b, s[2] += d;
                    p[0] += a * a, p[1] += b * b, p[2] += d * d, p[3] += a * b, p[4] += a * d, p[5] += b * d;
                }
                const size_t o = (size_t(z) * cy + y) * cx + x;
                for (int k = 0; k < 3; ++k) ubar[k * cn + o] = s[k] / 8;
                for (int k = 0; k < 6; ++k) uu[k * cn + o] = p[k] / 8;
            }
}

/* per coarse cell: filtered strain S (central differences, periodic), the
 * contractions tau^d:S and S:S of the subgrid stress tau = uu - ubar ubar,
 * their 3x3x3 box averages (periodic), the least-squares eddy viscosity
 * nu = max(0, -<tau^d:S> / (2 <S:S>)), the features of p = (tau0 + 3 nu) S
 * (X[n][16]) and the target nu (T[n]) */
void orc_sgs_targets(const double* ubar, const double* uu, int cx, int cy, int cz, double tau0, float* X, float* T) {
    const size_t cn = size_t(cx) * cy * cz;
    auto at = [&](int k, int x, int y, int z) {
        x = (x + cx) % cx, y = (y + cy) % cy, z = (z + cz) % cz;
        return ubar[k * cn + (size_t(z) * cy + y) * cx + x];
    };
    std::vector<double> S6(6 * cn), TS(cn), SS(cn);
    for (int z = 0; z < cz; ++z)
        for (int y = 0; y < cy; ++y)
            for (int x = 0; x < cx; ++x) {
                double g[3][3];
                for (int k = 0; k < 3; ++k) {
                    g[k][0] = 0.5 * (at(k, x + 1, y, z) - at(k, x - 1, y, z));
                    g[k][1] = 0.5 * (at(k, x, y + 1, z) - at(k, x, y - 1, z));
                    g[k][2] = 0.5 * (at(k, x, y, z + 1) - at(k, x, y, z - 1));
                }
                const double S[6] = {g[0][0], g[1][1], g[2][2], 0.5 * (g[0][1] + g[1][0]), 0.5 * (g[0][2] + g[2][0]),
                                     0.5 * (g[1][2] + g[2][1])};
                const size_t o = (size_t(z) * cy + y) * cx + x;
                const double u0 = ubar[o], u1 = ubar[cn + o], u2 = ubar[2 * cn + o];
                double tau[6] = {uu[o] - u0 * u0,          uu[cn + o] - u1 * u1,     uu[2 * cn + o] - u2 * u2,
                                 uu[3 * cn + o] - u0 * u1, uu[4 * cn + o] - u0 * u2, uu[5 * cn + o] - u1 * u2};
                const double tr = (tau[0] + tau[1] + tau[2]) / 3;
                for (int k = 0; k < 3; ++k) tau[k] -= tr;
                double ts = 0, ss = 0;
                for (int k = 0; k < 6; ++k) {
                    const double w = k < 3 ? 1 : 2;
                    ts += w * tau[k] * S[k];
                    ss += w * S[k] * S[k];
                }
                for (int k = 0; k < 6; ++k) S6[k * cn + o] = S[k];
                TS[o] = ts;
                SS[o] = ss;
            }
    for (int z = 0; z < cz; ++z)
        for (int y = 0; y < cy; ++y)
            for (int x = 0; x < cx; ++x) {
                double ts = 0, ss = 0;
                for (int dz = -1; dz <= 1; ++dz)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dx = -1; dx <= 1; ++dx) {
                            const size_t i = (size_t((z + dz + cz) % cz) * cy + (y + dy + cy) % cy) * cx +
                                             (x + dx + cx) % cx;
                            ts += TS[i];
                            ss += SS[i];
                        }
                double nu = ss > 1e-30 ? -ts / (2 * ss) : 0;
                if (nu < 0) nu = 0;
                const size_t o = (size_t(z) * cy + y) * cx + x;
                double p[6], x16[16];
                for (int k = 0; k < 6; ++k) p[k] = (tau0 + 3 * nu) * S6[k * cn + o];
                orc_sgs_features(p, tau0, x16);
                for (int k = 0; k < 16; ++k) X[o * 16 + k] = float(x16[k]);
                T[o] = float(nu);
            }
}

}  // extern "C"
