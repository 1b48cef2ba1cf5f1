/*
 * CPU oracle for the P0 mollified-triangle kernels (TEST INFRASTRUCTURE).
 *
 * This file checks the CUDA path and is not the product: only tests/, the smoke check of
 * __graft_entry__ and the cpu_baseline / reference leg of bench.py load it.
 * It restates, in plain C with OpenMP, the algorithm of the reference's
 * numba kernels in src/mbem/kernels/tri_kernels.py, function by function and
 * in the same order of operations where that is cheap, so that it can be
 * pinned against golden vectors produced by the reference itself
 * (tests/golden/) and then serve as the full-size oracle for the CUDA path.
 *
 * Layouts follow the reference: x_field (Nf,3), tri_verts (Ns,3,3) vertex
 * major, normals (Ns,3), eps (Ns,), density (Ns,3); matrices row-major
 * (3Nf, 3Ns) with block (3f+i, 3s+j); basis stacks (nb, 3Nf, 3Ns); stress
 * (Nf,3,3).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define PI 3.14159265358979323846

/* ---- edge antiderivatives: tri_kernels.py:54-76 and :606-619 ---------- */
static inline double J1(double u, double rho2) {
    return log(u + sqrt(u * u + rho2) + 1e-300);
}
static inline double J3(double u, double rho2) {
    if (rho2 < 1e-60) return 0.0;
    return u / (rho2 * sqrt(u * u + rho2));
}
static inline double K1(double u, double rho2) { return sqrt(u * u + rho2); }
static inline double K3(double u, double rho2) {
    double R = sqrt(u * u + rho2);
    if (R < 1e-30) R = 1e-30;
    return -1.0 / R;
}
static inline double J5(double u, double rho2) {
    if (rho2 < 1e-60) return 0.0;
    double R = sqrt(u * u + rho2);
    return u * (3.0 * rho2 + 2.0 * u * u) / (3.0 * rho2 * rho2 * R * R * R);
}
static inline double K5(double u, double rho2) {
    double R = sqrt(u * u + rho2);
    if (R < 1e-30) return 0.0;
    return -1.0 / (3.0 * R * R * R);
}

/* van Oosterom signed solid angle: tri_kernels.py:80-96 */
static double solid_angle(const double *tv, double ox, double oy, double oz) {
    double r1x = tv[0] - ox, r1y = tv[1] - oy, r1z = tv[2] - oz;
    double r2x = tv[3] - ox, r2y = tv[4] - oy, r2z = tv[5] - oz;
    double r3x = tv[6] - ox, r3y = tv[7] - oy, r3z = tv[8] - oz;
    double R1 = sqrt(r1x * r1x + r1y * r1y + r1z * r1z);
    double R2 = sqrt(r2x * r2x + r2y * r2y + r2z * r2z);
    double R3 = sqrt(r3x * r3x + r3y * r3y + r3z * r3z);
    double cx = r2y * r3z - r2z * r3y;
    double cy = r2z * r3x - r2x * r3z;
    double cz = r2x * r3y - r2y * r3x;
    double numer = r1x * cx + r1y * cy + r1z * cz;
    double d12 = r1x * r2x + r1y * r2y + r1z * r2z;
    double d23 = r2x * r3x + r2y * r3y + r2z * r3z;
    double d13 = r1x * r3x + r1y * r3y + r1z * r3z;
    double denom = R1 * R2 * R3 + R3 * d12 + R1 * d23 + R2 * d13;
    return 2.0 * atan2(numer, denom);
}

static inline double ipow(double x, int n) {
    double r = 1.0;
    for (int i = 0; i < n; i++) r *= x;
    return r;
}

/* Edge integral of xi1^a xi2^b / R^m, a+b <= 2: tri_kernels.py:100-129 */
static double edge_int(int a, int b, double dp, double nx, double ny,
                       double tx, double ty, double dJ, double dK, double dL) {
    double total = 0.0;
    for (int i = 0; i <= a; i++)
        for (int j = 0; j <= b; j++) {
            double ca = (a == 2 && i == 1) ? 2.0 : 1.0;
            double cb = (b == 2 && j == 1) ? 2.0 : 1.0;
            double coeff = ca * cb * ipow(dp, a + b - i - j) * ipow(nx, a - i) *
                           ipow(tx, i) * ipow(ny, b - j) * ipow(ty, j);
            int k = i + j;
            double delta = (k == 0) ? dJ : ((k == 1) ? dK : dL);
            total += coeff * delta;
        }
    return total;
}

/* binomial for n,k <= 3: tri_kernels.py:622-629 */
static inline double binom3(int n, int k) {
    if (k <= 0 || k >= n) return 1.0;
    if (n == 2) return 2.0;
    return 3.0;
}

/* Edge integral with a+b <= 3: tri_kernels.py:632-652 */
static double edge_int3(int a, int b, double dp, double nx, double ny,
                        double tx, double ty, double dJ, double dK, double dL,
                        double dM) {
    double total = 0.0;
    for (int i = 0; i <= a; i++)
        for (int j = 0; j <= b; j++) {
            double coeff = binom3(a, i) * binom3(b, j) *
                           ipow(dp, a + b - i - j) * ipow(nx, a - i) *
                           ipow(tx, i) * ipow(ny, b - j) * ipow(ty, j);
            int k = i + j;
            double delta = (k == 0) ? dJ : (k == 1) ? dK : (k == 2) ? dL : dM;
            total += coeff * delta;
        }
    return total;
}

/* In-plane frame of a source triangle: tri_kernels.py:137-153 */
static int tri_frame(const double *tv, double *ex, double *ey, double *nh) {
    double e1x = tv[3] - tv[0], e1y = tv[4] - tv[1], e1z = tv[5] - tv[2];
    double e2x = tv[6] - tv[0], e2y = tv[7] - tv[1], e2z = tv[8] - tv[2];
    double nx = e1y * e2z - e1z * e2y;
    double ny = e1z * e2x - e1x * e2z;
    double nz = e1x * e2y - e1y * e2x;
    double area2 = sqrt(nx * nx + ny * ny + nz * nz);
    if (area2 < 1e-30) return 0;
    nh[0] = nx / area2; nh[1] = ny / area2; nh[2] = nz / area2;
    double e1n = sqrt(e1x * e1x + e1y * e1y + e1z * e1z);
    ex[0] = e1x / e1n; ex[1] = e1y / e1n; ex[2] = e1z / e1n;
    ey[0] = nh[1] * ex[2] - nh[2] * ex[1];
    ey[1] = nh[2] * ex[0] - nh[0] * ex[2];
    ey[2] = nh[0] * ex[1] - nh[1] * ex[0];
    return 1;
}

/* Common pair geometry: the lift of the observer and the projected
 * vertices, as at the top of every pair function (tri_kernels.py:164-182,
 * :257-273, :663-679). */
typedef struct {
    double z, h2, h, I3;
    double px[3], py[3];
} PairGeo;

static void pair_geo(const double *tv, const double *ex, const double *ey,
                     const double *nh, const double *obs, double eps,
                     PairGeo *g) {
    double dx = obs[0] - tv[0], dy = obs[1] - tv[1], dz = obs[2] - tv[2];
    double z = dx * nh[0] + dy * nh[1] + dz * nh[2];
    double h2 = z * z + eps * eps;
    double h = sqrt(h2);
    double opx = obs[0] - z * nh[0];
    double opy = obs[1] - z * nh[1];
    double opz = obs[2] - z * nh[2];
    for (int k = 0; k < 3; k++) {
        double wx = tv[3 * k] - opx, wy = tv[3 * k + 1] - opy, wz = tv[3 * k + 2] - opz;
        g->px[k] = wx * ex[0] + wy * ex[1] + wz * ex[2];
        g->py[k] = wx * ey[0] + wy * ey[1] + wz * ey[2];
    }
    double oex = opx + h * nh[0], oey = opy + h * nh[1], oez = opz + h * nh[2];
    double Omega = solid_angle(tv, oex, oey, oez);
    g->z = z; g->h2 = h2; g->h = h; g->I3 = -Omega / h;
}

/* Edge frame (tri_kernels.py:190-201); returns 0 for a degenerate edge. */
static int edge_setup(const PairGeo *g, int e, double *nx, double *ny,
                      double *tx, double *ty, double *dp, double *ua,
                      double *ub, double *rho2) {
    double ax = g->px[e], ay = g->py[e];
    double bx = g->px[(e + 1) % 3], by = g->py[(e + 1) % 3];
    double evx = bx - ax, evy = by - ay;
    double L = sqrt(evx * evx + evy * evy);
    if (L <= 1e-30) return 0;
    *tx = evx / L; *ty = evy / L;
    *nx = *ty; *ny = -*tx;
    *dp = ax * *nx + ay * *ny;
    *ua = ax * *tx + ay * *ty;
    *ub = bx * *tx + by * *ty;
    *rho2 = *dp * *dp + g->h2;
    return 1;
}

/* U-kernel basis blocks out[3][3][3] ([b][i][j]): tri_kernels.py:161-243 */
static void u_basis_pair(const double *tv, const double *ex, const double *ey,
                         const double *nh, const double *obs, double eps,
                         double out[3][3][3]) {
    PairGeo g;
    pair_geo(tv, ex, ey, nh, obs, eps, &g);
    double BD001 = 0, BN1_001 = 0, BN2_001 = 0, BN1_101 = 0, BN2_101 = 0,
           BN1_011 = 0, BN2_011 = 0;
    (void)BN2_101;
    for (int e = 0; e < 3; e++) {
        double nx, ny, tx, ty, dp, ua, ub, rho2;
        if (!edge_setup(&g, e, &nx, &ny, &tx, &ty, &dp, &ua, &ub, &rho2)) continue;
        double dJ1 = J1(ub, rho2) - J1(ua, rho2);
        double dK1 = K1(ub, rho2) - K1(ua, rho2);
        double v00 = edge_int(0, 0, dp, nx, ny, tx, ty, dJ1, dK1, 0.0);
        double v10 = edge_int(1, 0, dp, nx, ny, tx, ty, dJ1, dK1, 0.0);
        double v01 = edge_int(0, 1, dp, nx, ny, tx, ty, dJ1, dK1, 0.0);
        BD001 += dp * v00;
        BN1_001 += nx * v00; BN2_001 += ny * v00;
        BN1_101 += nx * v10; BN2_101 += ny * v10;
        BN1_011 += nx * v01; BN2_011 += ny * v01;
    }
    double I3 = g.I3, z = g.z;
    double I1 = BD001 - g.h2 * I3;
    double m10 = -BN1_001, m01 = -BN2_001;
    double m20 = I1 - BN1_101, m11 = -BN1_011, m02 = I1 - BN2_011;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            out[0][i][j] = (i == j) ? I1 : 0.0;
            out[1][i][j] = (i == j) ? eps * eps * I3 : 0.0;
            out[2][i][j] = ex[i] * ex[j] * m20 + (ex[i] * ey[j] + ey[i] * ex[j]) * m11 +
                           ey[i] * ey[j] * m02 - z * (ex[i] * nh[j] + nh[i] * ex[j]) * m10 -
                           z * (ey[i] * nh[j] + nh[i] * ey[j]) * m01 +
                           z * z * nh[i] * nh[j] * I3;
        }
}

/* N (lam-slot) / R (mu-slot) contractions: tri_kernels.py:431-444 */
static void contract_NR(double P[3][3][3], const double *n, double out[6][3][3],
                        int iN, int iR) {
    for (int i = 0; i < 3; i++) {
        double tr = P[i][0][0] + P[i][1][1] + P[i][2][2];
        for (int j = 0; j < 3; j++) {
            out[iN][i][j] = n[j] * tr;
            out[iR][i][j] = P[i][j][0] * n[0] + P[i][j][1] * n[1] + P[i][j][2] * n[2] +
                            n[0] * P[i][0][j] + n[1] * P[i][1][j] + n[2] * P[i][2][j];
        }
    }
}

/* T-kernel basis blocks out[6][3][3]: tri_kernels.py:251-427 */
static void t_basis_pair(const double *tv, const double *ex, const double *ey,
                         const double *nh, const double *nsrc, const double *obs,
                         double eps, double out[6][3][3]) {
    PairGeo g;
    pair_geo(tv, ex, ey, nh, obs, eps, &g);
    double BN1_001 = 0, BN2_001 = 0, BD003 = 0, BN1_003 = 0, BN2_003 = 0,
           BN1_103 = 0, BN1_013 = 0, BN2_013 = 0, BN1_203 = 0, BN1_113 = 0,
           BN1_023 = 0, BN2_023 = 0;
    for (int e = 0; e < 3; e++) {
        double nx, ny, tx, ty, dp, ua, ub, rho2;
        if (!edge_setup(&g, e, &nx, &ny, &tx, &ty, &dp, &ua, &ub, &rho2)) continue;
        double dJ1 = J1(ub, rho2) - J1(ua, rho2);
        double dK1 = K1(ub, rho2) - K1(ua, rho2);
        double dJ3 = J3(ub, rho2) - J3(ua, rho2);
        double dK3 = K3(ub, rho2) - K3(ua, rho2);
        double dL3 = dJ1 - rho2 * dJ3;
        double v00m1 = edge_int(0, 0, dp, nx, ny, tx, ty, dJ1, dK1, 0.0);
        double v00 = edge_int(0, 0, dp, nx, ny, tx, ty, dJ3, dK3, dL3);
        double v10 = edge_int(1, 0, dp, nx, ny, tx, ty, dJ3, dK3, dL3);
        double v01 = edge_int(0, 1, dp, nx, ny, tx, ty, dJ3, dK3, dL3);
        double v20 = edge_int(2, 0, dp, nx, ny, tx, ty, dJ3, dK3, dL3);
        double v11 = edge_int(1, 1, dp, nx, ny, tx, ty, dJ3, dK3, dL3);
        double v02 = edge_int(0, 2, dp, nx, ny, tx, ty, dJ3, dK3, dL3);
        BN1_001 += nx * v00m1; BN2_001 += ny * v00m1;
        BD003 += dp * v00;
        BN1_003 += nx * v00; BN2_003 += ny * v00;
        BN1_103 += nx * v10;
        BN1_013 += nx * v01; BN2_013 += ny * v01;
        BN1_203 += nx * v20;
        BN1_113 += nx * v11;
        BN1_023 += nx * v02; BN2_023 += ny * v02;
    }
    double I3 = g.I3, z = g.z;
    double I5 = (BD003 + I3) / (3.0 * g.h2);
    double m10_3 = -BN1_001, m01_3 = -BN2_001;
    double m10_5 = -BN1_003 / 3.0, m01_5 = -BN2_003 / 3.0;
    double m20_5 = (I3 - BN1_103) / 3.0, m11_5 = -BN1_013 / 3.0,
           m02_5 = (I3 - BN2_013) / 3.0;
    double m30_5 = (2.0 * m10_3 - BN1_203) / 3.0, m21_5 = (m01_3 - BN1_113) / 3.0,
           m12_5 = -BN1_023 / 3.0, m03_5 = (2.0 * m01_3 - BN2_023) / 3.0;
    double V3[3], V5[3];
    for (int i = 0; i < 3; i++) {
        V3[i] = -ex[i] * m10_3 - ey[i] * m01_3 + nh[i] * z * I3;
        V5[i] = -ex[i] * m10_5 - ey[i] * m01_5 + nh[i] * z * I5;
    }
    /* T3[5] by the 27 frame triples: tri_kernels.py:350-394 */
    double T35[3][3][3];
    memset(T35, 0, sizeof(T35));
    const double *bas[3] = {ex, ey, nh};
    for (int c1 = 0; c1 < 3; c1++)
        for (int c2 = 0; c2 < 3; c2++)
            for (int c3 = 0; c3 < 3; c3++) {
                int a = (c1 == 0) + (c2 == 0) + (c3 == 0);
                int b = (c1 == 1) + (c2 == 1) + (c3 == 1);
                int nz = 3 - a - b;
                double mom;
                if (a == 3) mom = m30_5;
                else if (a == 2 && b == 1) mom = m21_5;
                else if (a == 2 && b == 0) mom = m20_5;
                else if (a == 1 && b == 2) mom = m12_5;
                else if (a == 1 && b == 1) mom = m11_5;
                else if (a == 1 && b == 0) mom = m10_5;
                else if (a == 0 && b == 3) mom = m03_5;
                else if (a == 0 && b == 2) mom = m02_5;
                else if (a == 0 && b == 1) mom = m01_5;
                else mom = I5;
                double sign = ((a + b) % 2 == 1) ? -1.0 : 1.0;
                double coeff = sign * ipow(z, nz) * mom;
                if (coeff == 0.0) continue;
                for (int i = 0; i < 3; i++) {
                    double ci = coeff * bas[c1][i];
                    for (int j = 0; j < 3; j++) {
                        double cij = ci * bas[c2][j];
                        for (int k = 0; k < 3; k++) T35[i][j][k] += cij * bas[c3][k];
                    }
                }
            }
    double e2 = eps * eps;
    double P[3][3][3];
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++)
            for (int m = 0; m < 3; m++) P[i][k][m] = (i == k) ? V3[m] : 0.0;
    contract_NR(P, nsrc, out, 0, 3);
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++)
            for (int m = 0; m < 3; m++) {
                double val = -3.0 * T35[i][k][m];
                if (i == m) val += V3[k];
                if (k == m) val += V3[i];
                P[i][k][m] = val;
            }
    contract_NR(P, nsrc, out, 1, 4);
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++)
            for (int m = 0; m < 3; m++) P[i][k][m] = (i == k) ? e2 * V5[m] : 0.0;
    contract_NR(P, nsrc, out, 2, 5);
}

/* 2-D area moments for the stress kernels: tri_kernels.py:656-769.
 * M3 is 3x3, M5 4x4, M7 5x5 (row-major, index [a][b]). */
static void stress_2d_moments(const double *tv, const double *ex, const double *ey,
                              const double *nh, const double *obs, double eps,
                              double M3[3][3], double M5[4][4], double M7[5][5],
                              int need7, double *I3o, double *I5o, double *I7o,
                              double *zo) {
    PairGeo g;
    pair_geo(tv, ex, ey, nh, obs, eps, &g);
    double BN1m1 = 0, BN2m1 = 0, BD003 = 0, BD005 = 0;
    double bn1_3[3][3] = {{0}}, bn2_3[3][3] = {{0}};
    double bn1_5[4][4] = {{0}}, bn2_5[4][4] = {{0}};
    for (int e = 0; e < 3; e++) {
        double nx, ny, tx, ty, dp, ua, ub, rho2;
        if (!edge_setup(&g, e, &nx, &ny, &tx, &ty, &dp, &ua, &ub, &rho2)) continue;
        double dJ1 = J1(ub, rho2) - J1(ua, rho2);
        double dK1 = K1(ub, rho2) - K1(ua, rho2);
        double dJ3 = J3(ub, rho2) - J3(ua, rho2);
        double dK3 = K3(ub, rho2) - K3(ua, rho2);
        double dL3 = dJ1 - rho2 * dJ3;
        double v = edge_int3(0, 0, dp, nx, ny, tx, ty, dJ1, dK1, 0.0, 0.0);
        BN1m1 += nx * v; BN2m1 += ny * v;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3 - a; b++) {
                v = edge_int3(a, b, dp, nx, ny, tx, ty, dJ3, dK3, dL3, 0.0);
                bn1_3[a][b] += nx * v;
                bn2_3[a][b] += ny * v;
                if (a == 0 && b == 0) BD003 += dp * v;
            }
        if (need7) {
            double dJ5 = J5(ub, rho2) - J5(ua, rho2);
            double dK5 = K5(ub, rho2) - K5(ua, rho2);
            double dL5 = dJ3 - rho2 * dJ5;
            double dM5 = dK3 - rho2 * dK5;
            for (int a = 0; a < 4; a++)
                for (int b = 0; b < 4 - a; b++) {
                    v = edge_int3(a, b, dp, nx, ny, tx, ty, dJ5, dK5, dL5, dM5);
                    bn1_5[a][b] += nx * v;
                    bn2_5[a][b] += ny * v;
                    if (a == 0 && b == 0) BD005 += dp * v;
                }
        }
    }
    double I3 = g.I3, h2 = g.h2;
    double I5 = (h2 > 1e-60) ? (BD003 + I3) / (3.0 * h2) : 0.0;
    M3[0][0] = I3;
    M3[1][0] = -BN1m1;
    M3[0][1] = -BN2m1;
    M5[0][0] = I5;
    M5[1][0] = -bn1_3[0][0] / 3.0;
    M5[0][1] = -bn2_3[0][0] / 3.0;
    M5[2][0] = (I3 - bn1_3[1][0]) / 3.0;
    M5[1][1] = -bn1_3[0][1] / 3.0;
    M5[0][2] = (I3 - bn2_3[0][1]) / 3.0;
    M5[3][0] = (2.0 * M3[1][0] - bn1_3[2][0]) / 3.0;
    M5[2][1] = (M3[0][1] - bn1_3[1][1]) / 3.0;
    M5[1][2] = -bn1_3[0][2] / 3.0;
    M5[0][3] = (2.0 * M3[0][1] - bn2_3[0][2]) / 3.0;
    double I7 = 0.0;
    if (need7) {
        I7 = (h2 > 1e-60) ? (BD005 + 3.0 * I5) / (5.0 * h2) : 0.0;
        M7[0][0] = I7;
        M7[1][0] = -bn1_5[0][0] / 5.0;
        M7[0][1] = -bn2_5[0][0] / 5.0;
        M7[2][0] = (I5 - bn1_5[1][0]) / 5.0;
        M7[1][1] = -bn1_5[0][1] / 5.0;
        M7[0][2] = (I5 - bn2_5[0][1]) / 5.0;
        M7[3][0] = (2.0 * M5[1][0] - bn1_5[2][0]) / 5.0;
        M7[2][1] = (M5[0][1] - bn1_5[1][1]) / 5.0;
        M7[1][2] = -bn1_5[0][2] / 5.0;
        M7[0][3] = (2.0 * M5[0][1] - bn2_5[0][2]) / 5.0;
        M7[4][0] = (3.0 * M5[2][0] - bn1_5[3][0]) / 5.0;
        M7[3][1] = (2.0 * M5[1][1] - bn1_5[2][1]) / 5.0;
        M7[2][2] = (M5[0][2] - bn1_5[1][2]) / 5.0;
        M7[1][3] = -bn1_5[0][3] / 5.0;
        M7[0][4] = (3.0 * M5[0][2] - bn2_5[0][3]) / 5.0;
    }
    *I3o = I3; *I5o = I5; *I7o = I7; *zo = g.z;
}

/* moment lookup for an (a,b) count: the M arrays have different strides */
#define MOM(M, a, b) ((M)[(a)][(b)])

/* T2[n][i,j] from 2-D moments: tri_kernels.py:773-784 (Mab(a,b) accessor) */
static void build_T2_5(double M[4][4], const double *ex, const double *ey,
                       const double *nh, double z, double out[3][3]) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            out[i][j] = ex[i] * ex[j] * M[2][0] + (ex[i] * ey[j] + ey[i] * ex[j]) * M[1][1] +
                        ey[i] * ey[j] * M[0][2] - z * (ex[i] * nh[j] + nh[i] * ex[j]) * M[1][0] -
                        z * (ey[i] * nh[j] + nh[i] * ey[j]) * M[0][1] +
                        z * z * nh[i] * nh[j] * M[0][0];
}
static void build_T2_7(double M[5][5], const double *ex, const double *ey,
                       const double *nh, double z, double out[3][3]) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            out[i][j] = ex[i] * ex[j] * M[2][0] + (ex[i] * ey[j] + ey[i] * ex[j]) * M[1][1] +
                        ey[i] * ey[j] * M[0][2] - z * (ex[i] * nh[j] + nh[i] * ex[j]) * M[1][0] -
                        z * (ey[i] * nh[j] + nh[i] * ey[j]) * M[0][1] +
                        z * z * nh[i] * nh[j] * M[0][0];
}

/* T3 from M5: tri_kernels.py:787-820 */
static void build_T3(double M[4][4], const double *bas[3], double z, double out[3][3][3]) {
    memset(out, 0, sizeof(double) * 27);
    for (int c1 = 0; c1 < 3; c1++)
        for (int c2 = 0; c2 < 3; c2++)
            for (int c3 = 0; c3 < 3; c3++) {
                int a = (c1 == 0) + (c2 == 0) + (c3 == 0);
                int b = (c1 == 1) + (c2 == 1) + (c3 == 1);
                int nz = 3 - a - b;
                double sign = ((a + b) % 2 == 1) ? -1.0 : 1.0;
                double coeff = sign * ipow(z, nz) * M[a][b];
                if (coeff == 0.0) continue;
                for (int i = 0; i < 3; i++) {
                    double ci = coeff * bas[c1][i];
                    for (int j = 0; j < 3; j++) {
                        double cij = ci * bas[c2][j];
                        for (int k = 0; k < 3; k++) out[i][j][k] += cij * bas[c3][k];
                    }
                }
            }
}

/* T4 from M7: tri_kernels.py:823-853 */
static void build_T4(double M[5][5], const double *bas[3], double z,
                     double out[3][3][3][3]) {
    memset(out, 0, sizeof(double) * 81);
    for (int c1 = 0; c1 < 3; c1++)
        for (int c2 = 0; c2 < 3; c2++)
            for (int c3 = 0; c3 < 3; c3++)
                for (int c4 = 0; c4 < 3; c4++) {
                    int cs[4] = {c1, c2, c3, c4};
                    int a = 0, b = 0;
                    for (int t = 0; t < 4; t++) {
                        if (cs[t] == 0) a++;
                        else if (cs[t] == 1) b++;
                    }
                    int nz = 4 - a - b;
                    double sign = ((a + b) % 2 == 1) ? -1.0 : 1.0;
                    double coeff = sign * ipow(z, nz) * M[a][b];
                    if (coeff == 0.0) continue;
                    for (int i = 0; i < 3; i++) {
                        double ci = coeff * bas[c1][i];
                        for (int j = 0; j < 3; j++) {
                            double cij = ci * bas[c2][j];
                            for (int k = 0; k < 3; k++) {
                                double cijk = cij * bas[c3][k];
                                for (int l = 0; l < 3; l++) out[i][j][k][l] += cijk * bas[c4][l];
                            }
                        }
                    }
                }
}

/* Force -> stress S[i][j][k]: tri_kernels.py:857-897 */
static void kelvin_stress_pair(const double *tv, const double *ex, const double *ey,
                               const double *nh, const double *obs, double eps,
                               double mu, double nu, double lam, double S[3][3][3]) {
    double M3[3][3] = {{0}}, M5[4][4] = {{0}}, M7[5][5] = {{0}};
    double I3, I5, I7, z;
    stress_2d_moments(tv, ex, ey, nh, obs, eps, M3, M5, M7, 0, &I3, &I5, &I7, &z);
    double V3[3], V5[3];
    for (int i = 0; i < 3; i++) {
        V3[i] = -ex[i] * M3[1][0] - ey[i] * M3[0][1] + z * nh[i] * M3[0][0];
        V5[i] = -ex[i] * M5[1][0] - ey[i] * M5[0][1] + z * nh[i] * M5[0][0];
    }
    const double *bas[3] = {ex, ey, nh};
    double T35[3][3][3];
    build_T3(M5, bas, z, T35);
    double C1 = 1.0 / (16.0 * PI * mu * (1.0 - nu));
    double c34 = 3.0 - 4.0 * nu;
    double cbdg = 6.0 * (1.0 - nu) * eps * eps;
    double G1[3][3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double dij = (i == j) ? 1.0 : 0.0;
            for (int m = 0; m < 3; m++) {
                double dim = (i == m) ? 1.0 : 0.0, djm = (j == m) ? 1.0 : 0.0;
                G1[i][j][m] = C1 * (-c34 * dij * V3[m] + dim * V3[j] + djm * V3[i] -
                                    3.0 * T35[i][j][m] - cbdg * dij * V5[m]);
            }
        }
    for (int k = 0; k < 3; k++) {
        double trace_k = G1[0][k][0] + G1[1][k][1] + G1[2][k][2];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double dij = (i == j) ? 1.0 : 0.0;
                S[i][j][k] = lam * dij * trace_k + mu * G1[i][k][j] + mu * G1[j][k][i];
            }
    }
}

/* Slip -> total stress H[m][n][k]: tri_kernels.py:900-964 */
static void dd_stress_pair(const double *tv, const double *ex, const double *ey,
                           const double *nh, const double *nrm, const double *obs,
                           double eps, double mu, double nu, double lam,
                           double H[3][3][3]) {
    double M3[3][3] = {{0}}, M5[4][4] = {{0}}, M7[5][5] = {{0}};
    double I3, I5, I7, z;
    stress_2d_moments(tv, ex, ey, nh, obs, eps, M3, M5, M7, 1, &I3, &I5, &I7, &z);
    const double *bas[3] = {ex, ey, nh};
    double T2_5[3][3], T2_7[3][3], T4_7[3][3][3][3];
    build_T2_5(M5, ex, ey, nh, z, T2_5);
    build_T2_7(M7, ex, ey, nh, z, T2_7);
    build_T4(M7, bas, z, T4_7);
    double C1 = 1.0 / (16.0 * PI * mu * (1.0 - nu));
    double c34 = 3.0 - 4.0 * nu;
    double cblob = 2.0 * (1.0 - nu) * eps * eps;
    double ID2G[3][3][3][3];
    for (int r = 0; r < 3; r++)
        for (int p = 0; p < 3; p++) {
            double drp = (r == p);
            for (int s = 0; s < 3; s++) {
                double drs = (r == s), dps = (p == s);
                for (int q = 0; q < 3; q++) {
                    double dsq = (s == q), dpq = (p == q), drq = (r == q);
                    double val = -c34 * drp * dsq * I3 + drs * dpq * I3 + dps * drq * I3 +
                                 c34 * drp * 3.0 * T2_5[s][q] - drs * 3.0 * T2_5[p][q] -
                                 dps * 3.0 * T2_5[r][q] - 3.0 * drq * T2_5[p][s] -
                                 3.0 * dpq * T2_5[r][s] - 3.0 * dsq * T2_5[r][p] +
                                 15.0 * T4_7[r][p][s][q] +
                                 cblob * drp * (-3.0 * dsq * I5 + 15.0 * T2_7[s][q]);
                    ID2G[r][p][s][q] = C1 * val;
                }
            }
        }
    double B[3][3][3];
    for (int r = 0; r < 3; r++)
        for (int s = 0; s < 3; s++) {
            double tr = 0.0;
            for (int p = 0; p < 3; p++) tr += ID2G[r][p][s][p];
            for (int k = 0; k < 3; k++) {
                double nq = 0.0, npd = 0.0;
                for (int q = 0; q < 3; q++) nq += nrm[q] * ID2G[r][k][s][q];
                for (int p = 0; p < 3; p++) npd += nrm[p] * ID2G[r][p][s][k];
                B[r][s][k] = lam * nrm[k] * tr + mu * nq + mu * npd;
            }
        }
    for (int k = 0; k < 3; k++) {
        double trB = B[0][0][k] + B[1][1][k] + B[2][2][k];
        for (int m = 0; m < 3; m++)
            for (int n = 0; n < 3; n++) {
                double dmn = (m == n);
                H[m][n][k] = -(lam * dmn * trB + mu * (B[m][n][k] + B[n][m][k]));
            }
    }
}

/* Exact eigenstress H*[m][n][k]: tri_kernels.py:1194-1214 */
static void eigenstress_pair(const double *tv, const double *ex, const double *ey,
                             const double *nh, const double *nrm, const double *obs,
                             double eps, double mu, double lam, double H[3][3][3]) {
    if (eps <= 0.0) {
        memset(H, 0, sizeof(double) * 27);
        return;
    }
    double M3[3][3] = {{0}}, M5[4][4] = {{0}}, M7[5][5] = {{0}};
    double I3, I5, I7, z;
    stress_2d_moments(tv, ex, ey, nh, obs, eps, M3, M5, M7, 1, &I3, &I5, &I7, &z);
    double phi = (15.0 * eps * eps * eps * eps / (8.0 * PI)) * I7;
    for (int m = 0; m < 3; m++)
        for (int n = 0; n < 3; n++) {
            double dmn = (m == n);
            for (int k = 0; k < 3; k++) {
                double dmk = (m == k), dnk = (n == k);
                H[m][n][k] = phi * (lam * dmn * nrm[k] + mu * (dmk * nrm[n] + dnk * nrm[m]));
            }
        }
}

/* ====================================================================== */
/* Drivers (tri_kernels.py:451-591, :976-1260)                             */
/* ====================================================================== */

int oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* out (3Nf, 3Ns) or basis stacks; kind 0 = T direct (c[6]), 1 = U direct
 * (c[3]), 2 = T basis (6 stacked), 3 = U basis (3 stacked).
 * Source rows [s0, s1) only, so a bounded sample can be timed; the output
 * is still indexed by the global source index. */
void oracle_matrix(int kind, const double *x_field, int64_t Nf,
                   const double *tri_verts, const double *normals,
                   const double *eps_arr, int64_t Ns, const double *c,
                   int64_t s0, int64_t s1, double *out) {
    int64_t ncol = 3 * Ns, nrow = 3 * Nf;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t s = s0; s < s1; s++) {
        const double *tv = tri_verts + 9 * s;
        double ex[3], ey[3], nh[3];
        if (!tri_frame(tv, ex, ey, nh)) continue;
        double eps = eps_arr[s];
        for (int64_t f = 0; f < Nf; f++) {
            const double *obs = x_field + 3 * f;
            if (kind == 0 || kind == 2) {
                double blk[6][3][3];
                t_basis_pair(tv, ex, ey, nh, normals + 3 * s, obs, eps, blk);
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) {
                        int64_t idx = (3 * f + i) * ncol + 3 * s + j;
                        if (kind == 0)
                            out[idx] = c[0] * blk[0][i][j] + c[1] * blk[1][i][j] +
                                       c[2] * blk[2][i][j] + c[3] * blk[3][i][j] +
                                       c[4] * blk[4][i][j] + c[5] * blk[5][i][j];
                        else
                            for (int b = 0; b < 6; b++) out[b * nrow * ncol + idx] = blk[b][i][j];
                    }
            } else {
                double blk[3][3][3];
                u_basis_pair(tv, ex, ey, nh, obs, eps, blk);
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) {
                        int64_t idx = (3 * f + i) * ncol + 3 * s + j;
                        if (kind == 1)
                            out[idx] = c[0] * blk[0][i][j] + c[1] * blk[1][i][j] +
                                       c[2] * blk[2][i][j];
                        else
                            for (int b = 0; b < 3; b++) out[b * nrow * ncol + idx] = blk[b][i][j];
                    }
            }
        }
    }
}

/* Contractions over sources, parallel over observers [f0, f1).
 * kind 0 = t_disp (out (Nf,3), c[6]), 1 = u_disp (out (Nf,3), c[3]),
 * 2 = dd stress, 3 = kelvin stress, 4 = eigenstress (out (Nf,3,3), c = {mu, lam}).
 * Zero-density sources are skipped, as the reference does. */
void oracle_contract(int kind, const double *x_field, int64_t Nf,
                     const double *tri_verts, const double *normals,
                     const double *eps_arr, int64_t Ns, const double *density,
                     const double *c, int64_t f0, int64_t f1, double *out) {
    double mu = c[0], lam = c[1];
    double nu = lam / (2.0 * (lam + mu));
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t f = f0; f < f1; f++) {
        const double *obs = x_field + 3 * f;
        double acc[9] = {0};
        for (int64_t s = 0; s < Ns; s++) {
            const double *tv = tri_verts + 9 * s;
            double ex[3], ey[3], nh[3];
            if (!tri_frame(tv, ex, ey, nh)) continue;
            const double *d = density + 3 * s;
            if (d[0] == 0.0 && d[1] == 0.0 && d[2] == 0.0) continue;
            double eps = eps_arr[s];
            if (kind == 0 || kind == 1) {
                double m[3][3];
                if (kind == 0) {
                    double blk[6][3][3];
                    t_basis_pair(tv, ex, ey, nh, normals + 3 * s, obs, eps, blk);
                    for (int i = 0; i < 3; i++)
                        for (int j = 0; j < 3; j++)
                            m[i][j] = c[0] * blk[0][i][j] + c[1] * blk[1][i][j] +
                                      c[2] * blk[2][i][j] + c[3] * blk[3][i][j] +
                                      c[4] * blk[4][i][j] + c[5] * blk[5][i][j];
                } else {
                    double blk[3][3][3];
                    u_basis_pair(tv, ex, ey, nh, obs, eps, blk);
                    for (int i = 0; i < 3; i++)
                        for (int j = 0; j < 3; j++)
                            m[i][j] = c[0] * blk[0][i][j] + c[1] * blk[1][i][j] +
                                      c[2] * blk[2][i][j];
                }
                for (int j = 0; j < 3; j++) {
                    if (d[j] == 0.0) continue;
                    for (int i = 0; i < 3; i++) acc[i] += m[i][j] * d[j];
                }
            } else {
                double H[3][3][3];
                if (kind == 2)
                    dd_stress_pair(tv, ex, ey, nh, normals + 3 * s, obs, eps, mu, nu, lam, H);
                else if (kind == 3)
                    kelvin_stress_pair(tv, ex, ey, nh, obs, eps, mu, nu, lam, H);
                else
                    eigenstress_pair(tv, ex, ey, nh, normals + 3 * s, obs, eps, mu, lam, H);
                for (int m = 0; m < 3; m++)
                    for (int n = 0; n < 3; n++)
                        acc[3 * m + n] += H[m][n][0] * d[0] + H[m][n][1] * d[1] + H[m][n][2] * d[2];
            }
        }
        if (kind <= 1)
            for (int i = 0; i < 3; i++) out[3 * f + i] = acc[i];
        else
            for (int i = 0; i < 9; i++) out[9 * f + i] = acc[i];
    }
}

/* Dense FP64 y = A x over rows [r0, r1) (the CPU side of the solve). */
void oracle_dgemv(const double *A, int64_t n_rows, int64_t n_cols, const double *x,
                  int64_t r0, int64_t r1, double *y) {
    (void)n_rows;
#pragma omp parallel for schedule(static)
    for (int64_t r = r0; r < r1; r++) {
        const double *a = A + r * n_cols;
        double acc = 0.0;
        for (int64_t c = 0; c < n_cols; c++) acc += a[c] * x[c];
        y[r] = acc;
    }
}

/* ====================================================================== */
/* Flat compressed product (flatview.py FlatView.matvec, _flat_matvec)     */
/* ====================================================================== */
/* y = A x for the flat layout of one material view: low-rank block i with
 * U^T (rank rows of pad4(3 nr) floats) at U + lr_u[i] and V^T likewise at
 * V + lr_v[i]; dense block d transposed, D^T (3 nc rows of pad4(3 nr)), at
 * D + d_off[d];
 * element ranges in the tree order (field_order / src_order map positions to
 * elements). Phase 1 forms w_i = V_i^T x per block; phase 2 owns rows: strip
 * s adds the blocks strip_items[strip_ptr[s] .. strip_ptr[s+1]) in order.
 * FP32 storage, FP64 arithmetic (as the reference). */
static inline int64_t pad4_64(int64_t n) { return (n + 3) / 4 * 4; }

void oracle_flat_matvec(int64_t n_field, int64_t n_src, const int64_t *field_order,
                        const int64_t *src_order, int64_t n_lr, const int32_t *lr_r0,
                        const int32_t *lr_nr, const int32_t *lr_c0, const int32_t *lr_nc,
                        const int32_t *lr_rank, const int64_t *lr_u, const int64_t *lr_v,
                        const int64_t *lr_w, const float *U, const float *V, int64_t n_w,
                        const int32_t *d_r0, const int32_t *d_nr, const int32_t *d_nc, const int32_t *d_c0,
                        const int64_t *d_off, const float *D, int64_t n_strips,
                        const int32_t *strip_r0, const int32_t *strip_nr, const int64_t *strip_ptr,
                        const int32_t *strip_items, const double *x, double *y) {
    double *xs = (double *)malloc(sizeof(double) * (size_t)(3 * n_src + 1));
    double *w = (double *)malloc(sizeof(double) * (size_t)(n_w + 1));
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n_src; p++)
        for (int a = 0; a < 3; a++) xs[3 * p + a] = x[3 * src_order[p] + a];
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < n_lr; i++) {
        const int64_t nc3 = 3 * (int64_t)lr_nc[i], ldv = pad4_64(nc3);
        const double *xc = xs + 3 * (int64_t)lr_c0[i];
        for (int k = 0; k < lr_rank[i]; k++) {
            const float *row = V + lr_v[i] + k * ldv;
            double acc = 0.0;
            for (int64_t c = 0; c < nc3; c++) acc += (double)row[c] * xc[c];
            w[lr_w[i] + k] = acc;
        }
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t s = 0; s < n_strips; s++) {
        const int64_t R = 3 * (int64_t)strip_nr[s], sr0 = strip_r0[s];
        double acc[3 * 1024];
        double *a = R <= 3 * 1024 ? acc : (double *)malloc(sizeof(double) * (size_t)R);
        for (int64_t r = 0; r < R; r++) a[r] = 0.0;
        for (int64_t q = strip_ptr[s]; q < strip_ptr[s + 1]; q++) {
            const int64_t id = strip_items[q];
            if (id < n_lr) {
                const int64_t ldu = pad4_64(3 * (int64_t)lr_nr[id]);
                const float *Ub = U + lr_u[id] + 3 * (sr0 - lr_r0[id]);
                const double *wi = w + lr_w[id];
                for (int k = 0; k < lr_rank[id]; k++) {
                    const float *u = Ub + k * ldu;
                    for (int64_t r = 0; r < R; r++) a[r] += (double)u[r] * wi[k];
                }
            } else {
                const int64_t d = id - n_lr;
                const int64_t nc3 = 3 * (int64_t)d_nc[d], ld = pad4_64(3 * (int64_t)d_nr[d]);
                const float *Db = D + d_off[d] + 3 * (sr0 - d_r0[d]);
                const double *xc = xs + 3 * (int64_t)d_c0[d];
                for (int64_t c = 0; c < nc3; c++) {
                    const float *col = Db + c * ld;
                    for (int64_t r = 0; r < R; r++) a[r] += (double)col[r] * xc[c];
                }
            }
        }
        for (int64_t r = 0; r < R; r++) y[3 * field_order[sr0 + r / 3] + r % 3] = a[r];
        if (a != acc) free(a);
    }
    (void)n_field;
    free(xs);
    free(w);
}
