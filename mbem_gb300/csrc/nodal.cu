// Nodal (Lagrange P0/P1/P2) kernels and traction rows, FP64 (sm_103a).
//
// Per (field point, source triangle) pair the per-node weighted moment
// tables W_k[n][a,b] = int_T N_k xi1^a xi2^b / R^n dS (n = 1, 3, 5, 7; xi
// about the foot point of the observer in the source's centroid frame) come
// from (src/mbem/kernels/tri_nodal.py):
//   * within D <= NODAL_D_STAR * L (D = sqrt(|x - c|^2 + eps^2), L the
//     longest edge): the divergence-theorem recursion of the raw moments
//     M[n][a,b] (n = -1 .. 7) over cancellation-free edge primitives
//     int u^k / R^m du (m = -1, 1, 3, 5), each evaluated in one of three
//     regimes (small-|u| series, large-|u| series, closed form; :262-410),
//     weighted by the Lagrange shape coefficients about the foot (:473-637);
//   * beyond: a collapsed Gauss-Legendre product rule (12 x 12, or 8 x 8
//     beyond NODAL_D_STAR_DISTANT * L) of the smooth integrand (:641-708).
// Every kernel is then the P0 contraction of p0_pair.cuh applied to W_k
// (:732-888). Traction rows (:1176-1227) take the stress per unit nodal
// density dotted with the field point's normal, columns scattered through an
// ids table; one thread owns a field point's three rows (no atomics).
//
// The tables live in per-thread local memory (~10 KB); these are the
// near-field / readout kernels, not the dense far field.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>

#include "p0_pair.cuh"

namespace mbem {

constexpr int ND_MAXK = 6;          // nodes per triangle (P2)
constexpr int ND_EDGE = 5;          // max edge-primitive degree (P2)
constexpr int ND_TAB = 6;           // max raw-moment degree (P2: n = 7 at degree 4 + 2)
constexpr int ND_TERMS = 32;        // series terms (NODAL_SERIES_TERMS)
constexpr int ND_SER = 2 * ND_TERMS + 2 + ND_EDGE + 3;   // series table length
constexpr int ND_Q = 144 + 64;      // far rules: 12 x 12 then 8 x 8

enum { KF_T = 1, KF_U = 2, KF_H = 4, KF_S = 8, KF_E = 16 };

struct NodalSpec {
    int order, K, q_split;
    bool valid;
    int lattice[ND_MAXK][3];
    int degn[5];        // raw-moment degree for n = -1, 1, 3, 5, 7 (-1: not needed)
    int ekmax[4];       // edge-primitive degree for m = -1, 1, 3, 5
    int need0[4];       // weighted-table degree for n = 1, 3, 5, 7
    double d_star, d_star_distant, small_u, series_u;
    double binom[4][ND_TERMS];   // C(-m/2, j) for m = -1, 1, 3, 5
};

// far rules: barycentric coordinates and weights (sum 1/2 per rule)
__constant__ double c_rule_lam[ND_Q][3];
__constant__ double c_rule_w[ND_Q];

// ---------------------------------------------------------------------------
// host: degrees and series coefficients (tri_nodal.py:72-140)
// ---------------------------------------------------------------------------
static NodalSpec make_spec(int order, int flags) {
    NodalSpec sp;
    memset(&sp, 0, sizeof(sp));
    sp.order = order;
    sp.K = (order + 1) * (order + 2) / 2;
    sp.q_split = 144;
    // lattice: vertices, then edges 12, 23, 31 (interior nodes appear only above P2)
    const int p = order;
    int k = 0;
    if (p == 0) {
        sp.lattice[0][0] = sp.lattice[0][1] = sp.lattice[0][2] = 0;
        k = 1;
    } else {
        for (int v = 0; v < 3; v++) {
            sp.lattice[k][0] = sp.lattice[k][1] = sp.lattice[k][2] = 0;
            sp.lattice[k][v] = p;
            k++;
        }
        const int ij[3][2] = {{0, 1}, {1, 2}, {2, 0}};
        for (int e = 0; e < 3; e++)
            for (int s = 1; s < p; s++) {
                sp.lattice[k][0] = sp.lattice[k][1] = sp.lattice[k][2] = 0;
                sp.lattice[k][ij[e][0]] = p - s;
                sp.lattice[k][ij[e][1]] = s;
                k++;
            }
    }
    auto kernel_degrees = [&](int ord, std::map<int, int>& need) {
        auto add = [&](int n, int d) {
            auto it = need.find(n);
            need[n] = (it == need.end()) ? d : std::max(it->second, d);
        };
        if (flags & KF_T) { add(3, 1 + ord); add(5, 3 + ord); }
        if (flags & KF_H) { add(3, 0 + ord); add(5, 2 + ord); add(7, 4 + ord); }
        if (flags & KF_E) { add(7, 0 + ord); }
        if (flags & KF_U) { add(1, 0 + ord); add(3, 2 + ord); }
        if (flags & KF_S) { add(3, 1 + ord); add(5, 3 + ord); }
    };
    std::map<int, int> need0, deg;
    kernel_degrees(0, need0);
    kernel_degrees(order, deg);
    auto get = [](const std::map<int, int>& m, int n) {
        auto it = m.find(n);
        return it == m.end() ? -1 : it->second;
    };
    auto raise = [&](std::map<int, int>& m, int n, int d) { m[n] = std::max(get(m, n), d); };
    // lower-n degrees the recursion consumes, and the vertical seeds (:98-116)
    int n = deg.rbegin()->first;
    while (true) {
        const int d = get(deg, n);
        if (d >= 2) raise(deg, n - 2, d - 2);
        if (n - 2 < deg.begin()->first) break;
        n -= 2;
    }
    raise(deg, 3, 0);
    std::map<int, int> snapshot = deg;
    for (auto& kv : snapshot) {
        if (kv.first >= 5)
            for (int m = 3; m < kv.first; m += 2) raise(deg, m, 0);
        if (kv.first <= 1)
            for (int m = kv.first; m < 4; m += 2) raise(deg, m, 0);
    }
    // edge degrees (:119-128)
    std::map<int, int> edge;
    for (auto& kv : deg) {
        if (kv.second < 0) continue;
        if (kv.second >= 1) raise(edge, kv.first - 2, kv.second - 1);
    }
    for (auto& kv : deg) {
        if (kv.second < 0) continue;
        if (kv.first >= 5) raise(edge, kv.first - 2, 0);
        if (kv.first <= 1) raise(edge, kv.first, 0);
    }
    // the P2 spec bounds (tri_nodal.py:197-203): no recursion below n = -1,
    // edge degrees within the tables, closure of the edge recursion
    sp.valid = get(deg, -1) < 1 && edge.begin()->first >= -1 && deg.begin()->first >= -1 &&
               deg.rbegin()->first <= 7 && edge.rbegin()->first <= 5;
    for (auto& kv : edge) {
        sp.valid = sp.valid && kv.second <= ND_EDGE;
        for (int kk = 2; kk <= kv.second; kk++) sp.valid = sp.valid && get(edge, kv.first - 2) >= kk - 2;
    }
    for (auto& kv : deg) sp.valid = sp.valid && kv.second <= ND_TAB;
    for (int i = 0; i < 5; i++) sp.degn[i] = get(deg, 2 * i - 1);
    for (int i = 0; i < 4; i++) sp.ekmax[i] = get(edge, 2 * i - 1);
    for (int i = 0; i < 4; i++) sp.need0[i] = get(need0, 2 * i + 1);
    sp.d_star = 10.0;
    sp.d_star_distant = 40.0;
    sp.small_u = 0.5;
    sp.series_u = 2.0;
    // C(-m/2, j) as an exact fraction p / q (q a power of two once reduced),
    // rounded once to double
    for (int mi = 0; mi < 4; mi++) {
        const int num_a = -(2 * mi - 1);                 // -m/2 = num_a / 2
        __int128 bp = 1, bq = 1;
        for (int j = 0; j < ND_TERMS; j++) {
            sp.binom[mi][j] = (double)bp / (double)bq;
            bp *= (num_a - 2 * j);
            bq *= 2 * (j + 1);
            __int128 x = bp < 0 ? -bp : bp, y = bq;
            while (y != 0) {
                const __int128 t = x % y;
                x = y;
                y = t;
            }
            if (x > 1) {
                bp /= x;
                bq /= x;
            }
        }
    }
    return sp;
}

static void gauss_legendre_nodal(int n, double* x, double* w) {
    for (int i = 0; i < n; i++) {
        double z = cos(MBEM_PI * (i + 0.75) / (n + 0.5));
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; k++) {
                const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            const double dp = n * (z * p1 - p0) / (z * z - 1.0);
            const double dz = p1 / dp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        double p0 = 1.0, p1 = z;
        for (int k = 2; k <= n; k++) {
            const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
            p0 = p1;
            p1 = p2;
        }
        const double dp = n * (z * p1 - p0) / (z * z - 1.0);
        x[i] = z;
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

static std::mutex g_rule_mutex;
static bool g_rule_ready[64] = {false};

// The far rules in constant memory of the current device, once per device.
static int ensure_rules() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return set_error(MBEM_ERR_CUDA, "no current CUDA device for the nodal rules");
    std::lock_guard<std::mutex> lock(g_rule_mutex);
    if (g_rule_ready[dev]) return MBEM_OK;
    static double lam[ND_Q][3], w[ND_Q];
    int q = 0;
    for (int n : {12, 8}) {
        double g[12], gw[12];
        gauss_legendre_nodal(n, g, gw);
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                const double gi = 0.5 * (g[i] + 1.0), gj = 0.5 * (g[j] + 1.0);
                const double x1 = gi, x2 = gj * (1.0 - gi);
                lam[q][0] = 1.0 - x1 - x2;
                lam[q][1] = x1;
                lam[q][2] = x2;
                w[q] = (0.5 * gw[i]) * (0.5 * gw[j]) * (1.0 - gi);
                q++;
            }
    }
    cudaError_t e = cudaMemcpyToSymbol(c_rule_lam, lam, sizeof(lam));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_rule_w, w, sizeof(w));
    if (e != cudaSuccess) return set_error(MBEM_ERR_CUDA, "nodal rules: %s", cudaGetErrorString(e));
    g_rule_ready[dev] = true;
    return MBEM_OK;
}

// ---------------------------------------------------------------------------
// device: per-source record (tri_nodal.py:418-455)
// ---------------------------------------------------------------------------
struct NodalSrc {
    double ex[3], ey[3], nh[3], c[3];
    double p2d[3][2];     // vertices in the centroid frame
    double abc[3][3];     // lam_k(eta) = A_k + B_k eta1 + C_k eta2
    double L, area2;
    bool ok;
};

__device__ bool nodal_frame(const double* __restrict__ tv, NodalSrc& g) {
    SrcP0 s;
    src_setup(tv, 1.0, s);
    g.ok = s.ok;
    if (!s.ok) return false;
    for (int k = 0; k < 3; k++) {
        g.ex[k] = s.ex[k]; g.ey[k] = s.ey[k]; g.nh[k] = s.nh[k];
        g.c[k] = ((tv[k] + tv[3 + k]) + tv[6 + k]) / 3.0;
    }
    for (int k = 0; k < 3; k++) {
        const double dx = tv[3 * k] - g.c[0], dy = tv[3 * k + 1] - g.c[1], dz = tv[3 * k + 2] - g.c[2];
        g.p2d[k][0] = dx * g.ex[0] + dy * g.ex[1] + dz * g.ex[2];
        g.p2d[k][1] = dx * g.ey[0] + dy * g.ey[1] + dz * g.ey[2];
    }
    double L = 0.0;
    for (int k = 0; k < 3; k++) {
        const int k2 = (k + 1) % 3;
        const double dx = tv[3 * k2] - tv[3 * k], dy = tv[3 * k2 + 1] - tv[3 * k + 1],
                     dz = tv[3 * k2 + 2] - tv[3 * k + 2];
        L = fmax(L, sqrt(dx * dx + dy * dy + dz * dz));
    }
    g.L = L;
    const double e1x = tv[3] - tv[0], e1y = tv[4] - tv[1], e1z = tv[5] - tv[2];
    const double e2x = tv[6] - tv[0], e2y = tv[7] - tv[1], e2z = tv[8] - tv[2];
    const double nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
    g.area2 = sqrt(nx * nx + ny * ny + nz * nz);
    const double den = (g.p2d[1][0] - g.p2d[0][0]) * (g.p2d[2][1] - g.p2d[0][1]) -
                       (g.p2d[1][1] - g.p2d[0][1]) * (g.p2d[2][0] - g.p2d[0][0]);
    for (int k = 0; k < 3; k++) {
        const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
        const double x1 = g.p2d[k1][0], y1 = g.p2d[k1][1], x2 = g.p2d[k2][0], y2 = g.p2d[k2][1];
        g.abc[k][0] = (x1 * y2 - y1 * x2) / den;
        g.abc[k][1] = (y1 - y2) / den;
        g.abc[k][2] = (x2 - x1) / den;
    }
    return true;
}

// ---------------------------------------------------------------------------
// edge primitives: P[mi][k] = int_ua^ub u^k / R^m du, m = 2 mi - 1
// ---------------------------------------------------------------------------
__device__ __forceinline__ double ipow(double x, int n) {
    double r = 1.0;
    if (n >= 0) {
        for (int i = 0; i < n; i++) r *= x;
    } else {
        const double xi = 1.0 / x;
        for (int i = 0; i < -n; i++) r *= xi;
    }
    return r;
}

// large-|u| series, 0 < a < b, rho^2 / a^2 <= 1/4: one-sign chains for
// r^q - 1 (tri_nodal.py:262-298)
__device__ void series_large_row(int mi, int kmax, double a, double b, double rho2, const NodalSpec& sp,
                                 double P[4][ND_EDGE + 1], double* T) {
    const int m = 2 * mi - 1;
    const double x = rho2 / (a * a);
    const double r = b / a;
    const double log_r = log1p((b - a) / a);
    const double up = (b - a) / a;
    const double dn = -(b - a) / b;
    const double rinv = 1.0 / r;
    const int off = 2 * ND_TERMS + 2;
    T[off] = 0.0;
    const int qmax = kmax - m + 1;
    for (int q = 1; q <= qmax; q++) T[off + q] = T[off + q - 1] * r + up;
    const int qmin = 1 - m - 2 * (ND_TERMS - 1);
    for (int q = -1; q >= qmin; q--) T[off + q] = T[off + q + 1] * rinv + dn;
    double base = ipow(a, 1 - m);
    for (int k = 0; k <= kmax; k++) {
        double out = 0.0, xj = 1.0;
        for (int j = 0; j < ND_TERMS; j++) {
            const int q = k - m + 1 - 2 * j;
            const double term = (q == 0) ? log_r : T[off + q] / q;
            out = out + sp.binom[mi][j] * xj * term;
            xj = xj * x;
        }
        P[mi][k] = base * out;
        base = base * a;
    }
}

// small-|u| series, max(|ua|, |ub|) <= rho / 2 (tri_nodal.py:302-342)
__device__ void series_small_row(int mi, int kmax, double ua, double ub, double rho2, const NodalSpec& sp,
                                 double P[4][ND_EDGE + 1], double* YA, double* YB, double* E) {
    const int m = 2 * mi - 1;
    const double rho = sqrt(rho2);
    const double ya = ua / rho, yb = ub / rho;
    const int pmax = kmax + 2 * (ND_TERMS - 1) + 1;
    YA[0] = 1.0;
    YB[0] = 1.0;
    for (int p = 1; p <= pmax; p++) {
        YA[p] = YA[p - 1] * ya;
        YB[p] = YB[p - 1] * yb;
    }
    bool close = false;
    if (ua * ub > 0.0) {
        const double ratio = ub / ua;
        close = (ratio < 2.0) && (ratio > 0.5);
        if (close) {
            const double up = (ub - ua) / ua;
            E[0] = 0.0;
            for (int p = 1; p <= pmax; p++) E[p] = E[p - 1] * ratio + up;
        }
    }
    double scale = ipow(rho, 1 - m);
    for (int k = 0; k <= kmax; k++) {
        double out = 0.0;
        for (int j = 0; j < ND_TERMS; j++) {
            const int pw = k + 2 * j + 1;
            const double dpow = close ? YA[pw] * E[pw] : YB[pw] - YA[pw];
            out = out + sp.binom[mi][j] * dpow / pw;
        }
        P[mi][k] = scale * out;
        scale = scale * rho;
    }
}

// conjugate closed-form differences (tri_nodal.py:346-382)
__device__ void closed_form(double ua, double ub, double rho2, const int ekmax[4], double P[4][ND_EDGE + 1]) {
    const double Ra = sqrt(ua * ua + rho2), Rb = sqrt(ub * ub + rho2);
    const double dR = (ub - ua) * (ub + ua) / (Ra + Rb);
    double dJ1;
    if (ua >= 0.0) dJ1 = log1p(((ub - ua) + dR) / (ua + Ra));
    else if (ub <= 0.0) dJ1 = log1p(((ub - ua) - dR) / (Rb - ub));
    else dJ1 = log(((ub + Rb) * (Ra - ua)) / rho2);
    double dJ3;
    if (ua * ub > 0.0) dJ3 = ((ub - ua) * (ub + ua)) / (Ra * Rb * (ub * Ra + ua * Rb));
    else dJ3 = (ub / Rb - ua / Ra) / rho2;
    // the endpoint terms of dJ5 nearly cancel: pow keeps each one to an ulp
    const double duRm = ub * pow(Rb, -3.0) - ua * pow(Ra, -3.0);
    const double dJ5 = (duRm + 2.0 * dJ3) / (3.0 * rho2);
    const double duR = 0.5 * (ub - ua) * (Ra + Rb) + 0.5 * (ua + ub) * dR;
    const double dJm1 = 0.5 * (duR + rho2 * dJ1);
    const double RaRb = Ra * Rb;
    const double S3 = (Rb * Rb + Ra * Rb) + Ra * Ra;
    const double dK[4] = {dR * S3 / 3.0, dR, dR / RaRb, dR * S3 / (3.0 * pow(RaRb, 3.0))};
    const double dJ[4] = {dJm1, dJ1, dJ3, dJ5};
    for (int mi = 0; mi < 4; mi++) {
        if (ekmax[mi] < 0) continue;
        P[mi][0] = dJ[mi];
        if (ekmax[mi] >= 1) P[mi][1] = dK[mi];
    }
    for (int k = 2; k <= ND_EDGE; k++)
        for (int mi = 1; mi < 4; mi++)
            if (ekmax[mi] >= k) P[mi][k] = P[mi - 1][k - 2] - rho2 * P[mi][k - 2];
}

__device__ void edge_primitives(double ua, double ub, double rho2, const NodalSpec& sp,
                                double P[4][ND_EDGE + 1], double* SER) {
    const double rho = sqrt(rho2);
    const double aua = fabs(ua), aub = fabs(ub);
    const double umax = fmax(aua, aub), umin = fmin(aua, aub);
    if (umax <= sp.small_u * rho) {
        for (int mi = 0; mi < 4; mi++)
            if (sp.ekmax[mi] >= 0)
                series_small_row(mi, sp.ekmax[mi], ua, ub, rho2, sp, P, SER, SER + ND_SER, SER + 2 * ND_SER);
    } else if ((ua * ub > 0.0) && umin >= sp.series_u * rho) {
        const bool negative = ua < 0.0;
        const double a = negative ? -ub : ua, b = negative ? -ua : ub;
        for (int mi = 0; mi < 4; mi++)
            if (sp.ekmax[mi] >= 0) {
                series_large_row(mi, sp.ekmax[mi], a, b, rho2, sp, P, SER);
                if (negative)
                    for (int k = 1; k <= sp.ekmax[mi]; k += 2) P[mi][k] = -P[mi][k];
            }
    } else {
        closed_form(ua, ub, rho2, sp.ekmax, P);
    }
}

__device__ __forceinline__ double comb(int a, int i) {
    // C(a, i) for a <= 5
    const double f[6] = {1.0, 1.0, 2.0, 6.0, 24.0, 120.0};
    return f[a] / (f[i] * f[a - i]);
}

// ---------------------------------------------------------------------------
// one pair: the weighted tables W[ni2][k][a][b] (n = 2 ni2 + 1)
// ---------------------------------------------------------------------------
struct NodalScratch {
    double M[5][ND_TAB + 1][ND_TAB + 1];
    double BN1[4][ND_EDGE + 1][ND_EDGE + 1];
    double BN2[4][ND_EDGE + 1][ND_EDGE + 1];
    double BD[4];
    double P[4][ND_EDGE + 1];
    double C[ND_MAXK][3][3];
    double SER[3 * ND_SER];
};

// shape coefficients C[k][a][b] of N_k about the foot X (tri_nodal.py:473-515)
__device__ void shape_coeffs(const NodalSpec& sp, const NodalSrc& g, double X1, double X2, double C[ND_MAXK][3][3]) {
    const int order = sp.order, D = order + 1;
    for (int k = 0; k < sp.K; k++)
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) C[k][a][b] = 0.0;
    if (order == 0) {
        C[0][0][0] = 1.0;
        return;
    }
    for (int k = 0; k < sp.K; k++) {
        double poly[3][3] = {{1.0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int i = 0; i < 3; i++) {
            const double l0 = (g.abc[i][0] + X1 * g.abc[i][1]) + X2 * g.abc[i][2];
            for (int j = 0; j < sp.lattice[k][i]; j++) {
                const double f00 = (order * l0) / (j + 1) - (double)j / (j + 1);
                const double f10 = (order * g.abc[i][1]) / (j + 1);
                const double f01 = (order * g.abc[i][2]) / (j + 1);
                double out[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                for (int a = 0; a < D; a++)
                    for (int b = 0; a + b < D; b++) {
                        const double pab = poly[a][b];
                        if (pab == 0.0) continue;
                        out[a][b] += pab * f00;
                        if (a + b + 1 < D) {
                            out[a + 1][b] += pab * f10;
                            out[a][b + 1] += pab * f01;
                        }
                    }
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) poly[a][b] = out[a][b];
            }
        }
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) C[k][a][b] = poly[a][b];
    }
}

// raw moments M[ni][a][b], n = 2 ni - 1 (tri_nodal.py:519-619)
__device__ void moment_table(const NodalSpec& sp, const NodalSrc& g, double X1, double X2, double h2,
                             NodalScratch& S) {
    const double h = sqrt(h2);
    // I3 from the solid angle of the lifted point, in the centroid frame
    double px[3], py[3], R[3];
    for (int k = 0; k < 3; k++) {
        px[k] = g.p2d[k][0] - X1;
        py[k] = g.p2d[k][1] - X2;
        R[k] = sqrt(px[k] * px[k] + py[k] * py[k] + h2);
    }
    const double area2s = (g.p2d[1][0] - g.p2d[0][0]) * (g.p2d[2][1] - g.p2d[0][1]) -
                          (g.p2d[2][0] - g.p2d[0][0]) * (g.p2d[1][1] - g.p2d[0][1]);
    const double d01 = px[0] * px[1] + py[0] * py[1] + h2;
    const double d12 = px[1] * px[2] + py[1] * py[2] + h2;
    const double d02 = px[0] * px[2] + py[0] * py[2] + h2;
    const double omega = 2.0 * atan2(-h * area2s, R[0] * R[1] * R[2] + R[2] * d01 + R[0] * d12 + R[1] * d02);
    const double I3 = -omega / h;

    int kall = 0;
    for (int mi = 0; mi < 4; mi++) kall = max(kall, sp.ekmax[mi]);
    for (int mi = 0; mi < 4; mi++) {
        S.BD[mi] = 0.0;
        for (int a = 0; a <= ND_EDGE; a++)
            for (int b = 0; b <= ND_EDGE; b++) S.BN1[mi][a][b] = S.BN2[mi][a][b] = 0.0;
    }
    for (int e = 0; e < 3; e++) {
        const int e2 = (e + 1) % 3;
        const double pax = px[e], pay = py[e], pbx = px[e2], pby = py[e2];
        const double evx = pbx - pax, evy = pby - pay;
        const double Le = sqrt(evx * evx + evy * evy);
        const double tx = evx / Le, ty = evy / Le;
        const double c1 = ty, c2 = -tx;
        const double dp = pax * c1 + pay * c2;
        const double ua = pax * tx + pay * ty, ub = pbx * tx + pby * ty;
        const double rho2 = dp * dp + h2;
        edge_primitives(ua, ub, rho2, sp, S.P, S.SER);
        double dpP[ND_EDGE + 1], c1P[ND_EDGE + 1], s1P[ND_EDGE + 1], c2P[ND_EDGE + 1], s2P[ND_EDGE + 1];
        dpP[0] = c1P[0] = s1P[0] = c2P[0] = s2P[0] = 1.0;
        for (int q = 1; q <= kall; q++) {
            dpP[q] = dpP[q - 1] * dp;
            c1P[q] = c1P[q - 1] * c1;
            s1P[q] = s1P[q - 1] * tx;
            c2P[q] = c2P[q - 1] * c2;
            s2P[q] = s2P[q - 1] * ty;
        }
        for (int mi = 0; mi < 4; mi++) {
            const int kmax = sp.ekmax[mi];
            if (kmax < 0) continue;
            S.BD[mi] += dp * S.P[mi][0];
            for (int a = 0; a <= kmax; a++)
                for (int b = 0; a + b <= kmax; b++) {
                    double val = 0.0;
                    for (int i = 0; i <= a; i++)
                        for (int j = 0; j <= b; j++) {
                            const int pw = a + b - i - j;
                            double coeff = (comb(a, i) * comb(b, j)) * dpP[pw];
                            coeff = coeff * c1P[a - i];
                            coeff = coeff * s1P[i];
                            coeff = coeff * c2P[b - j];
                            coeff = coeff * s2P[j];
                            val = val + coeff * S.P[mi][i + j];
                        }
                    S.BN1[mi][a][b] += c1 * val;
                    S.BN2[mi][a][b] += c2 * val;
                }
        }
    }
    const int* degn = sp.degn;
    S.M[2][0][0] = I3;
    if (degn[3] >= 0) S.M[3][0][0] = (S.BD[2] + I3) / (3.0 * h2);
    if (degn[4] >= 0) S.M[4][0][0] = (S.BD[3] + 3.0 * S.M[3][0][0]) / (5.0 * h2);
    if (degn[1] >= 0) S.M[1][0][0] = S.BD[1] - h2 * S.M[2][0][0];
    if (degn[0] >= 0) S.M[0][0][0] = (S.BD[0] + h2 * S.M[1][0][0]) / 3.0;
    for (int ni = 0; ni < 5; ni++) {
        const int d = degn[ni];
        if (d < 1 || ni < 1) continue;   // n = -1 never recurses at P2 (checked on the host)
        const int n = 2 * ni - 1;
        const int mi = ni - 1;
        for (int q = 1; q <= d; q++)
            for (int a = q; a >= 0; a--) {
                const int b = q - a;
                double val;
                if (a >= 1) {
                    val = -S.BN1[mi][a - 1][b];
                    if (a >= 2) val += (a - 1) * S.M[mi][a - 2][b];
                } else {
                    val = -S.BN2[mi][0][b - 1];
                    if (b >= 2) val += (b - 1) * S.M[mi][0][b - 2];
                }
                S.M[ni][a][b] = val / (n - 2);
            }
    }
}

// N_k at barycentric lam by the lattice product formula
__device__ __forceinline__ double lagrange_value(const NodalSpec& sp, int k, const double lam[3]) {
    double v = 1.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < sp.lattice[k][i]; j++) v *= (sp.order * lam[i] - j) / (j + 1);
    return v;
}

// Fills W; returns the signed height z (tri_nodal.py:683-708).
__device__ double nodal_pair_tables(const NodalSpec& sp, const NodalSrc& g, const double obs[3], double eps,
                                    double W[4][ND_MAXK][5][5], NodalScratch& S) {
    const double dx = obs[0] - g.c[0], dy = obs[1] - g.c[1], dz = obs[2] - g.c[2];
    const double z = dx * g.nh[0] + dy * g.nh[1] + dz * g.nh[2];
    const double X1 = dx * g.ex[0] + dy * g.ex[1] + dz * g.ex[2];
    const double X2 = dx * g.ey[0] + dy * g.ey[1] + dz * g.ey[2];
    const double h2 = z * z + eps * eps;
    const double D = sqrt((dx * dx + dy * dy + dz * dz) + eps * eps);
    const int K = sp.K;
    if (D <= sp.d_star * g.L) {
        shape_coeffs(sp, g, X1, X2, S.C);
        moment_table(sp, g, X1, X2, h2, S);
        for (int ni2 = 0; ni2 < 4; ni2++) {
            const int d = sp.need0[ni2];
            if (d < 0) continue;
            for (int k = 0; k < K; k++)
                for (int a = 0; a <= d; a++)
                    for (int b = 0; a + b <= d; b++) {
                        double acc = 0.0;
                        for (int ap = 0; ap <= sp.order; ap++)
                            for (int bp = 0; ap + bp <= sp.order; bp++)
                                acc += S.C[k][ap][bp] * S.M[ni2 + 1][a + ap][b + bp];
                        W[ni2][k][a][b] = acc;
                    }
        }
    } else {
        const int q0 = (D > sp.d_star_distant * g.L) ? sp.q_split : 0;
        const int q1 = (D > sp.d_star_distant * g.L) ? ND_Q : sp.q_split;
        int dmax = 0;
        for (int ni2 = 0; ni2 < 4; ni2++) {
            const int d = sp.need0[ni2];
            dmax = max(dmax, d);
            if (d < 0) continue;
            for (int k = 0; k < K; k++)
                for (int a = 0; a <= d; a++)
                    for (int b = 0; a + b <= d; b++) W[ni2][k][a][b] = 0.0;
        }
        for (int q = q0; q < q1; q++) {
            const double lam[3] = {c_rule_lam[q][0], c_rule_lam[q][1], c_rule_lam[q][2]};
            const double eta1 = lam[0] * g.p2d[0][0] + lam[1] * g.p2d[1][0] + lam[2] * g.p2d[2][0];
            const double eta2 = lam[0] * g.p2d[0][1] + lam[1] * g.p2d[1][1] + lam[2] * g.p2d[2][1];
            const double xi1 = eta1 - X1, xi2 = eta2 - X2;
            const double R2 = xi1 * xi1 + xi2 * xi2 + h2;
            const double wq = c_rule_w[q] * g.area2;
            const double r2i = 1.0 / R2;
            double Nk[ND_MAXK];
            for (int k = 0; k < K; k++) Nk[k] = lagrange_value(sp, k, lam);
            double x1p[6], x2p[6];
            x1p[0] = x2p[0] = 1.0;
            for (int a = 1; a <= dmax; a++) {
                x1p[a] = x1p[a - 1] * xi1;
                x2p[a] = x2p[a - 1] * xi2;
            }
            double Rn = sqrt(r2i);
            for (int ni2 = 0; ni2 < 4; ni2++) {
                const int d = sp.need0[ni2];
                if (d >= 0)
                    for (int a = 0; a <= d; a++)
                        for (int b = 0; a + b <= d; b++) {
                            const double f = wq * x1p[a] * x2p[b] * Rn;
                            for (int k = 0; k < K; k++) W[ni2][k][a][b] += f * Nk[k];
                        }
                Rn = Rn * r2i;
            }
        }
    }
    return z;
}

// moments of node k in the layouts of p0_pair.cuh
__device__ __forceinline__ void node_tscal(const double W[4][ND_MAXK][5][5], int k, double z, TScal& q) {
    q.z = z;
    q.I3 = W[1][k][0][0]; q.m10_3 = W[1][k][1][0]; q.m01_3 = W[1][k][0][1];
    q.I5 = W[2][k][0][0]; q.m10_5 = W[2][k][1][0]; q.m01_5 = W[2][k][0][1];
    q.m20_5 = W[2][k][2][0]; q.m11_5 = W[2][k][1][1]; q.m02_5 = W[2][k][0][2];
    q.m30_5 = W[2][k][3][0]; q.m21_5 = W[2][k][2][1]; q.m12_5 = W[2][k][1][2]; q.m03_5 = W[2][k][0][3];
}

__device__ __forceinline__ void node_smoments(const double W[4][ND_MAXK][5][5], int k, double z,
                                              StressMoments& M) {
    M.z = z;
    M.I3 = W[1][k][0][0];
    M.m3_10 = W[1][k][1][0];
    M.m3_01 = W[1][k][0][1];
    for (int a = 0; a < 4; a++)
        for (int b = 0; a + b < 4; b++) M.M5[a][b] = W[2][k][a][b];
    for (int a = 0; a < 5; a++)
        for (int b = 0; a + b < 5; b++) M.M7[a][b] = W[3][k][a][b];
}

// U basis of node k: I1, I3 and T2[3] (global)
__device__ void node_u(const NodalSrc& g, const double W[4][ND_MAXK][5][5], int k, double z, double& I1,
                       double& I3, double T2[3][3]) {
    I1 = W[0][k][0][0];
    I3 = W[1][k][0][0];
    const double L[3][3] = {{W[1][k][2][0], W[1][k][1][1], -z * W[1][k][1][0]},
                            {W[1][k][1][1], W[1][k][0][2], -z * W[1][k][0][1]},
                            {-z * W[1][k][1][0], -z * W[1][k][0][1], z * z * W[1][k][0][0]}};
    double Y[3][3];
    for (int a = 0; a < 3; a++)
        for (int j = 0; j < 3; j++) Y[a][j] = L[a][0] * g.ex[j] + L[a][1] * g.ey[j] + L[a][2] * g.nh[j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) T2[i][j] = g.ex[i] * Y[0][j] + g.ey[i] * Y[1][j] + g.nh[i] * Y[2][j];
}

__device__ __forceinline__ void frame_local(const NodalSrc& g, const double* v, double l[3]) {
    l[0] = v[0] * g.ex[0] + v[1] * g.ex[1] + v[2] * g.ex[2];
    l[1] = v[0] * g.ey[0] + v[1] * g.ey[1] + v[2] * g.ey[2];
    l[2] = v[0] * g.nh[0] + v[1] * g.nh[1] + v[2] * g.nh[2];
}

__device__ __forceinline__ void frame_rotate_sym(const NodalSrc& g, const double L[3][3], double G[3][3]) {
    double Y[3][3];
    for (int a = 0; a < 3; a++)
        for (int j = 0; j < 3; j++) Y[a][j] = L[a][0] * g.ex[j] + L[a][1] * g.ey[j] + L[a][2] * g.nh[j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) G[i][j] = g.ex[i] * Y[0][j] + g.ey[i] * Y[1][j] + g.nh[i] * Y[2][j];
}

// stress (global, symmetric) per density d of node k: which 0 dd, 1 kelvin,
// 2 eigen, 3 dd - eigen
// stress (global, symmetric) per density d from a node's stress moments M
// (I7 = M.M7[0][0]): which 0 dd, 1 kelvin, 2 eigen, 3 dd - eigen
__device__ void moments_stress(const NodalSrc& g, const StressMoments& M, const double* nrm, const double* d,
                               double eps, double mu, double lam, int which, double out[3][3]) {
    const double nu = lam / (2.0 * (lam + mu));
    const double C1 = 1.0 / (16.0 * MBEM_PI * mu * (1.0 - nu));
    const double c34 = 3.0 - 4.0 * nu;
    double loc[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    if (which != 2) {
        double dl[3];
        frame_local(g, d, dl);
        if (which == 1) {
            kelvin_stress_local(M, dl, mu, lam, C1, c34, 6.0 * (1.0 - nu) * eps * eps, loc);
        } else {
            double nl[3];
            frame_local(g, nrm, nl);
            dd_stress_local(M, nl, dl, mu, lam, C1, c34, 2.0 * (1.0 - nu) * eps * eps, loc);
        }
    }
    frame_rotate_sym(g, loc, out);
    if (which >= 2) {
        const double phi = (15.0 * eps * eps * eps * eps / (8.0 * MBEM_PI)) * M.M7[0][0];
        const double sgn = (which == 3) ? -1.0 : 1.0;
        const double nd = nrm[0] * d[0] + nrm[1] * d[1] + nrm[2] * d[2];
        for (int m = 0; m < 3; m++)
            for (int n = 0; n < 3; n++)
                out[m][n] += sgn * phi * ((m == n ? lam * nd : 0.0) + mu * (d[m] * nrm[n] + d[n] * nrm[m]));
    }
}

__device__ void node_stress(const NodalSrc& g, const double W[4][ND_MAXK][5][5], int k, double z,
                            const double* nrm, const double* d, double eps, double mu, double lam, int which,
                            double out[3][3]) {
    StressMoments M;
    node_smoments(W, k, z, M);
    moments_stress(g, M, nrm, d, eps, mu, lam, which, out);
}

// Far pairs of a P0 (one-node) density: the Gauss tables of the stress
// moments held in registers (I3; M5 and M7 to the degrees the kernel needs),
// the same sums as the general tables (tri_nodal.py:641-679) with N = 1.
template <bool KELVIN>
__device__ void far_moments_p0(const NodalSrc& g, double X1, double X2, double h2, int q0, int q1,
                               StressMoments& M) {
    constexpr int D5 = KELVIN ? 3 : 2;      // n = 5 degree: kelvin 3, dd 2
    double I3 = 0.0, m3_10 = 0.0, m3_01 = 0.0;
    double m5[D5 + 1][D5 + 1], m7[5][5];
#pragma unroll
    for (int a = 0; a <= D5; a++)
#pragma unroll
        for (int b = 0; b <= D5; b++) m5[a][b] = 0.0;
#pragma unroll
    for (int a = 0; a < 5; a++)
#pragma unroll
        for (int b = 0; b < 5; b++) m7[a][b] = 0.0;
    for (int q = q0; q < q1; q++) {
        const double l0 = c_rule_lam[q][0], l1 = c_rule_lam[q][1], l2 = c_rule_lam[q][2];
        const double eta1 = l0 * g.p2d[0][0] + l1 * g.p2d[1][0] + l2 * g.p2d[2][0];
        const double eta2 = l0 * g.p2d[0][1] + l1 * g.p2d[1][1] + l2 * g.p2d[2][1];
        const double xi1 = eta1 - X1, xi2 = eta2 - X2;
        const double R2 = xi1 * xi1 + xi2 * xi2 + h2;
        const double wq = c_rule_w[q] * g.area2;
        const double r2i = 1.0 / R2;
        const double Rn1 = sqrt(r2i);
        const double Rn3 = Rn1 * r2i, Rn5 = Rn3 * r2i, Rn7 = Rn5 * r2i;
        double x1p[5], x2p[5];
        x1p[0] = x2p[0] = 1.0;
#pragma unroll
        for (int a = 1; a < 5; a++) {
            x1p[a] = x1p[a - 1] * xi1;
            x2p[a] = x2p[a - 1] * xi2;
        }
        I3 += wq * Rn3;
        if (KELVIN) {
            m3_10 += wq * x1p[1] * x2p[0] * Rn3;
            m3_01 += wq * x1p[0] * x2p[1] * Rn3;
        }
#pragma unroll
        for (int a = 0; a <= D5; a++)
#pragma unroll
            for (int b = 0; a + b <= D5; b++) m5[a][b] += wq * x1p[a] * x2p[b] * Rn5;
        if (!KELVIN) {
#pragma unroll
            for (int a = 0; a < 5; a++)
#pragma unroll
                for (int b = 0; a + b < 5; b++) m7[a][b] += wq * x1p[a] * x2p[b] * Rn7;
        }
    }
    M.I3 = I3;
    M.m3_10 = m3_10;
    M.m3_01 = m3_01;
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) M.M5[a][b] = (a <= D5 && b <= D5) ? m5[a < D5 + 1 ? a : 0][b < D5 + 1 ? b : 0] : 0.0;
#pragma unroll
    for (int a = 0; a < 5; a++)
#pragma unroll
        for (int b = 0; b < 5; b++) M.M7[a][b] = m7[a][b];
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
struct NodalArgs {
    const double* x_field;
    const double* n_field;
    int64_t n_field_pts;
    const double* tri_verts;
    const double* normals;
    const double* eps;
    int64_t n_src;
    const double* density;
    const int64_t* ids;
    int64_t n_cols;
    double c[6];
    double mu, lam, alpha;
    int accumulate, which;
    double* out;
    int64_t ld;
    int64_t plane;
    const int64_t* pair_rowptr;   // listed pairs (traction rows of the mixed operator): field point f's
    const int64_t* pair_cols;     // sources at pair_cols[pair_rowptr[f] .. pair_rowptr[f+1]); NULL: all pairs
    int64_t n_pairs;
};

constexpr int ND_THREADS = 64;

// matrices: one thread per (field point, source); kind 0 T, 1 U, 2 T basis, 3 U basis
__global__ void __launch_bounds__(ND_THREADS)
nodal_matrix_kernel(NodalArgs a, NodalSpec sp, int kind) {
    const int64_t idx = (int64_t)blockIdx.x * ND_THREADS + threadIdx.x;
    const int64_t total = a.n_field_pts * a.n_src;
    if (idx >= total) return;
    const int64_t f = idx / a.n_src, s = idx % a.n_src;
    const int K = sp.K;
    NodalSrc g;
    const bool ok = nodal_frame(a.tri_verts + 9 * s, g);
    double W[4][ND_MAXK][5][5];
    NodalScratch S;
    double z = 0.0;
    if (ok) z = nodal_pair_tables(sp, g, a.x_field + 3 * f, a.eps[s], W, S);
    const double eps2 = a.eps[s] * a.eps[s];
    const double* nrm = a.normals ? a.normals + 3 * s : nullptr;
    for (int k = 0; k < K; k++) {
        const int64_t col = 3 * (K * s + k);
        if (kind == 0 || kind == 2) {
            double blk6[6][3][3];
            if (ok) {
                TScal q;
                node_tscal(W, k, z, q);
                TMoments m;
                t_from_scal(g.ex, g.ey, g.nh, nrm, q, m);
                t_basis_blocks(m, nrm, eps2, blk6);
            } else {
                for (int b = 0; b < 6; b++)
                    for (int i = 0; i < 3; i++)
                        for (int j = 0; j < 3; j++) blk6[b][i][j] = 0.0;
            }
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    const int64_t o = (3 * f + i) * a.ld + col + j;
                    if (kind == 0) {
                        double v = 0.0;
                        for (int b = 0; b < 6; b++) v += a.c[b] * blk6[b][i][j];
                        v *= a.alpha;
                        a.out[o] = a.accumulate ? a.out[o] + v : v;
                    } else {
                        for (int b = 0; b < 6; b++) a.out[b * a.plane + o] = blk6[b][i][j];
                    }
                }
        } else {
            double I1 = 0.0, I3 = 0.0, T2[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            if (ok) node_u(g, W, k, z, I1, I3, T2);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    const int64_t o = (3 * f + i) * a.ld + col + j;
                    const double b0 = (i == j) ? I1 : 0.0, b1 = (i == j) ? eps2 * I3 : 0.0, b2 = T2[i][j];
                    if (kind == 1) {
                        const double v = a.alpha * (a.c[0] * b0 + a.c[1] * b1 + a.c[2] * b2);
                        a.out[o] = a.accumulate ? a.out[o] + v : v;
                    } else {
                        a.out[o] = b0;
                        a.out[a.plane + o] = b1;
                        a.out[2 * a.plane + o] = b2;
                    }
                }
        }
    }
}

// contractions: one thread per field point; kind 0 T disp, 1 U disp, 2+w stress
__global__ void __launch_bounds__(ND_THREADS)
nodal_contract_kernel(NodalArgs a, NodalSpec sp, int kind, int split) {
    // split threads per observer take interleaved sources; their partial sums
    // are added in slice order (deterministic)
    __shared__ double red[ND_THREADS][9];
    const int obs_per_block = ND_THREADS / split;
    const int lane = threadIdx.x % obs_per_block, slice = threadIdx.x / obs_per_block;
    const int64_t f = (int64_t)blockIdx.x * obs_per_block + lane;
    const bool active = f < a.n_field_pts;
    const int K = sp.K;
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double W[4][ND_MAXK][5][5];
    NodalScratch S;
    for (int64_t s = slice; active && s < a.n_src; s += split) {
        bool zero = true;
        for (int k = 0; k < K * 3 && zero; k++) zero = a.density[3 * K * s + k] == 0.0;
        if (zero) continue;
        NodalSrc g;
        if (!nodal_frame(a.tri_verts + 9 * s, g)) continue;
        const double eps = a.eps[s];
        const double z = nodal_pair_tables(sp, g, a.x_field + 3 * f, eps, W, S);
        const double* nrm = a.normals ? a.normals + 3 * s : nullptr;
        for (int k = 0; k < K; k++) {
            const double* d = a.density + 3 * (K * s + k);
            if (kind == 0) {
                TScal q;
                node_tscal(W, k, z, q);
                TMoments m;
                t_from_scal(g.ex, g.ey, g.nh, nrm, q, m);
                double blk[3][3];
                t_block(m, nrm, a.c, eps * eps, blk);
                for (int i = 0; i < 3; i++) acc[i] += blk[i][0] * d[0] + blk[i][1] * d[1] + blk[i][2] * d[2];
            } else if (kind == 1) {
                double I1, I3, T2[3][3];
                node_u(g, W, k, z, I1, I3, T2);
                const double dg = a.c[0] * I1 + a.c[1] * eps * eps * I3;
                for (int i = 0; i < 3; i++)
                    acc[i] += dg * d[i] + a.c[2] * (T2[i][0] * d[0] + T2[i][1] * d[1] + T2[i][2] * d[2]);
            } else {
                double sg[3][3];
                node_stress(g, W, k, z, nrm, d, eps, a.mu, a.lam, kind - 2, sg);
                for (int m = 0; m < 3; m++)
                    for (int n = 0; n < 3; n++) acc[3 * m + n] += sg[m][n];
            }
        }
    }
    const int nout = kind <= 1 ? 3 : 9;
    if (split > 1) {
        for (int i = 0; i < nout; i++) red[threadIdx.x][i] = acc[i];
        __syncthreads();
        if (slice != 0) return;
        for (int k = 1; k < split; k++)
            for (int i = 0; i < nout; i++) acc[i] += red[k * obs_per_block + lane][i];
    }
    if (!active) return;
    double* o = a.out + nout * f;
    for (int i = 0; i < nout; i++) {
        const double v = a.alpha * acc[i];
        o[i] = a.accumulate ? o[i] + v : v;
    }
}

// traction rows: out[3f+i, 3 ids[s,k] + j] += alpha * n_f . sigma(e_j density of node k).
// One thread per (field point, source), sources fastest so that a warp
// writes neighbouring columns of the same rows. Entries are added
// atomically: a shared-node ids table maps several sources onto one column
// (the element-major table maps each entry once, so its result does not
// depend on the order of the adds).
__global__ void __launch_bounds__(ND_THREADS)
nodal_traction_kernel(NodalArgs a, NodalSpec sp) {
    const int64_t idx = (int64_t)blockIdx.x * ND_THREADS + threadIdx.x;
    int64_t f, s;
    if (a.pair_cols) {
        if (idx >= a.n_pairs) return;
        int64_t lo = 0, hi = a.n_field_pts;
        while (hi - lo > 1) {
            const int64_t mid = (lo + hi) >> 1;
            if (a.pair_rowptr[mid] <= idx) lo = mid;
            else hi = mid;
        }
        f = lo;
        s = a.pair_cols[idx];
    } else {
        if (idx >= a.n_field_pts * a.n_src) return;
        f = idx / a.n_src;
        s = idx % a.n_src;
    }
    const int K = sp.K;
    const double* nf = a.n_field + 3 * f;
    double W[4][ND_MAXK][5][5];
    NodalScratch S;
    // which: 0 slip (dd - eigen), 1 force, 2 eigen, 3 total (dd)
    const int sw = a.which == 0 ? 3 : (a.which == 1 ? 1 : (a.which == 2 ? 2 : 0));
    NodalSrc g;
    if (!nodal_frame(a.tri_verts + 9 * s, g)) return;
    const double eps = a.eps[s];
    const double zero_n[3] = {0.0, 0.0, 0.0};
    const double* nrm = a.normals ? a.normals + 3 * s : zero_n;
    if (K == 1) {
        // one-node density: far pairs through the register tables
        const double* x = a.x_field + 3 * f;
        const double dx = x[0] - g.c[0], dy = x[1] - g.c[1], dz = x[2] - g.c[2];
        const double D = sqrt((dx * dx + dy * dy + dz * dz) + eps * eps);
        if (D > sp.d_star * g.L) {
            const double z = dx * g.nh[0] + dy * g.nh[1] + dz * g.nh[2];
            const double X1 = dx * g.ex[0] + dy * g.ex[1] + dz * g.ex[2];
            const double X2 = dx * g.ey[0] + dy * g.ey[1] + dz * g.ey[2];
            const double h2 = z * z + eps * eps;
            const bool distant = D > sp.d_star_distant * g.L;
            const int q0 = distant ? sp.q_split : 0, q1 = distant ? ND_Q : sp.q_split;
            StressMoments M;
            M.z = z;
            if (sw == 1) far_moments_p0<true>(g, X1, X2, h2, q0, q1, M);
            else far_moments_p0<false>(g, X1, X2, h2, q0, q1, M);
            const int64_t id = a.ids ? a.ids[s] : s;
            if (id < 0 || id >= a.n_cols) return;
            for (int j = 0; j < 3; j++) {
                const double d[3] = {j == 0 ? 1.0 : 0.0, j == 1 ? 1.0 : 0.0, j == 2 ? 1.0 : 0.0};
                double sg[3][3];
                moments_stress(g, M, nrm, d, eps, a.mu, a.lam, sw, sg);
                for (int i = 0; i < 3; i++) {
                    const double t = nf[0] * sg[i][0] + nf[1] * sg[i][1] + nf[2] * sg[i][2];
                    atomicAdd(&a.out[(3 * f + i) * a.ld + 3 * id + j], a.alpha * t);
                }
            }
            return;
        }
    }
    const double z = nodal_pair_tables(sp, g, a.x_field + 3 * f, eps, W, S);
    for (int k = 0; k < K; k++) {
        const int64_t id = a.ids ? a.ids[s * K + k] : s * K + k;
        if (id < 0 || id >= a.n_cols) continue;        // outside the block: never written
        const int64_t col = 3 * id;
        for (int j = 0; j < 3; j++) {
            const double d[3] = {j == 0 ? 1.0 : 0.0, j == 1 ? 1.0 : 0.0, j == 2 ? 1.0 : 0.0};
            double sg[3][3];
            node_stress(g, W, k, z, nrm, d, eps, a.mu, a.lam, sw, sg);
            for (int i = 0; i < 3; i++) {
                const double t = nf[0] * sg[i][0] + nf[1] * sg[i][1] + nf[2] * sg[i][2];
                atomicAdd(&a.out[(3 * f + i) * a.ld + col + j], a.alpha * t);
            }
        }
    }
}

// Listed (observer, source) pairs of a readout: the FP64 elastic stress
// (DD minus eigen) of the source's nodal slip density at the observer, nine
// components per pair; the mixed-precision readout sends its near pairs here.
__global__ void __launch_bounds__(ND_THREADS)
nodal_pairs_stress_kernel(NodalArgs a, NodalSpec sp, const int64_t* __restrict__ pair_obs,
                          const int32_t* __restrict__ pair_src, int64_t n_pairs, double* __restrict__ out,
                          double* __restrict__ out_eig) {
    const int64_t p = (int64_t)blockIdx.x * ND_THREADS + threadIdx.x;
    if (p >= n_pairs) return;
    const int64_t f = pair_obs[p], s = pair_src[p];
    double acc[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double acc_e[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    NodalSrc g;
    if (nodal_frame(a.tri_verts + 9 * s, g)) {
        double W[4][ND_MAXK][5][5];
        NodalScratch S;
        const double eps = a.eps[s];
        const double z = nodal_pair_tables(sp, g, a.x_field + 3 * f, eps, W, S);
        const double* nrm = a.normals + 3 * s;
        for (int k = 0; k < sp.K; k++) {
            const double* d = a.density + 3 * (sp.K * s + k);
            if (d[0] == 0.0 && d[1] == 0.0 && d[2] == 0.0) continue;
            double sg[3][3];
            node_stress(g, W, k, z, nrm, d, eps, a.mu, a.lam, 3, sg);
            for (int m = 0; m < 3; m++)
                for (int n = 0; n < 3; n++) acc[m][n] += sg[m][n];
            if (out_eig) {
                node_stress(g, W, k, z, nrm, d, eps, a.mu, a.lam, 2, sg);
                for (int m = 0; m < 3; m++)
                    for (int n = 0; n < 3; n++) acc_e[m][n] += sg[m][n];
            }
        }
    }
    for (int m = 0; m < 3; m++)
        for (int n = 0; n < 3; n++) out[9 * p + 3 * m + n] = acc[m][n];
    if (out_eig)
        for (int m = 0; m < 3; m++)
            for (int n = 0; n < 3; n++) out_eig[9 * p + 3 * m + n] = acc_e[m][n];
}

int nodal_pairs_stress(const double* x, const double* tv, const double* normals, const double* eps,
                       const double* density, double mu, double lam, int order, const int64_t* pair_obs,
                       const int32_t* pair_src, int64_t n_pairs, double* out, cudaStream_t st, double* out_eig) {
    MBEM_REQUIRE(order >= 0 && order <= 2, MBEM_ERR_ARG, "order must be 0, 1 or 2");
    int e = ensure_rules();
    if (e) return e;
    const NodalSpec sp = make_spec(order, KF_H);
    MBEM_REQUIRE(sp.valid, MBEM_ERR_UNSUPPORTED, "nodal degrees beyond the P2 tables");
    if (n_pairs == 0) return MBEM_OK;
    NodalArgs a;
    memset(&a, 0, sizeof(a));
    a.x_field = x; a.tri_verts = tv; a.normals = normals; a.eps = eps; a.density = density;
    a.mu = mu; a.lam = lam;
    nodal_pairs_stress_kernel<<<(unsigned)ceil_div(n_pairs, ND_THREADS), ND_THREADS, 0, st>>>(a, sp, pair_obs, pair_src,
                                                                                          n_pairs, out, out_eig);
    return launch_status("nodal_pairs_stress_kernel");
}

static int flags_for_matrix(int kind) { return (kind == 0 || kind == 2) ? KF_T : KF_U; }

// The FP64 nodal blocks of listed near pairs (the mixed operator's near
// field at order 1/2): pair q = (field point f, source s) from a CSR by field
// point; node k's 3x3 block goes to vals[(K q + k) * 9], the layout of the
// node-level near list (columns K s + k).
__global__ void __launch_bounds__(ND_THREADS)
nodal_near_eval_kernel(NodalArgs a, NodalSpec sp, int kind, const int64_t* __restrict__ rowptr,
                       const int64_t* __restrict__ cols, int64_t nnz, double* __restrict__ vals) {
    const int64_t q = (int64_t)blockIdx.x * ND_THREADS + threadIdx.x;
    if (q >= nnz) return;
    int64_t lo = 0, hi = a.n_field_pts;
    while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (rowptr[mid] <= q) lo = mid;
        else hi = mid;
    }
    const int64_t f = lo, s = cols[q];
    const int K = sp.K;
    NodalSrc g;
    const bool ok = nodal_frame(a.tri_verts + 9 * s, g);
    double W[4][ND_MAXK][5][5];
    NodalScratch S;
    double z = 0.0;
    if (ok) z = nodal_pair_tables(sp, g, a.x_field + 3 * f, a.eps[s], W, S);
    const double eps2 = a.eps[s] * a.eps[s];
    const double* nrm = a.normals ? a.normals + 3 * s : nullptr;
    for (int k = 0; k < K; k++) {
        double* out = vals + 9 * (K * q + k);
        if (!ok) {
            for (int e = 0; e < 9; e++) out[e] = 0.0;
            continue;
        }
        if (kind == 0) {
            TScal ts;
            node_tscal(W, k, z, ts);
            TMoments m;
            t_from_scal(g.ex, g.ey, g.nh, nrm, ts, m);
            double blk[3][3];
            t_block(m, nrm, a.c, eps2, blk);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) out[3 * i + j] = a.alpha * blk[i][j];
        } else {
            double I1 = 0.0, I3 = 0.0, T2[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            node_u(g, W, k, z, I1, I3, T2);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    out[3 * i + j] =
                        a.alpha * (a.c[0] * (i == j ? I1 : 0.0) + a.c[1] * (i == j ? eps2 * I3 : 0.0) + a.c[2] * T2[i][j]);
        }
    }
}

int nodal_matrix(int kind, const double* x, int64_t nf, const double* tv, const double* normals,
                 const double* eps, int64_t ns, const double* coeffs, int order, double alpha, int accumulate,
                 double* out, int64_t ld, void* stream) {
    MBEM_REQUIRE(order == 1 || order == 2, MBEM_ERR_ARG, "nodal order must be 1 or 2");
    int e = ensure_rules();
    if (e) return e;
    const NodalSpec sp = make_spec(order, flags_for_matrix(kind));
    MBEM_REQUIRE(sp.valid, MBEM_ERR_UNSUPPORTED, "nodal degrees beyond the P2 tables");
    NodalArgs a;
    memset(&a, 0, sizeof(a));
    a.x_field = x; a.n_field_pts = nf; a.tri_verts = tv; a.normals = normals; a.eps = eps; a.n_src = ns;
    const int nc = (kind == 0) ? 6 : (kind == 1 ? 3 : 0);
    for (int i = 0; i < 6; i++) a.c[i] = (coeffs && i < nc) ? coeffs[i] : 0.0;
    a.alpha = alpha; a.accumulate = accumulate; a.out = out;
    a.ld = (kind >= 2) ? 3 * sp.K * ns : ld;
    a.plane = 3 * nf * 3 * sp.K * ns;
    MBEM_REQUIRE(kind >= 2 || ld >= 3 * sp.K * ns, MBEM_ERR_ARG, "ld_out %lld < 3*K*n_src", (long long)ld);
    const int64_t total = nf * ns;
    if (total == 0) return MBEM_OK;
    nodal_matrix_kernel<<<(unsigned)ceil_div(total, ND_THREADS), ND_THREADS, 0, (cudaStream_t)stream>>>(a, sp,
                                                                                                      kind);
    return launch_status("nodal_matrix_kernel");
}

int nodal_contract(int kind, const double* x, int64_t nf, const double* tv, const double* normals,
                   const double* eps, int64_t ns, const double* density, const double* coeffs, double mu,
                   double lam, int order, double alpha, int accumulate, double* out, void* stream) {
    MBEM_REQUIRE(order == 1 || order == 2, MBEM_ERR_ARG, "nodal order must be 1 or 2");
    int e = ensure_rules();
    if (e) return e;
    int flags = KF_T;
    if (kind == 1) flags = KF_U;
    else if (kind == 2 + MBEM_STRESS_DD) flags = KF_H;
    else if (kind == 2 + MBEM_STRESS_KELVIN) flags = KF_S;
    else if (kind == 2 + MBEM_STRESS_EIGEN) flags = KF_E;
    else if (kind == 2 + MBEM_STRESS_ELASTIC) flags = KF_H | KF_E;
    const NodalSpec sp = make_spec(order, flags);
    MBEM_REQUIRE(sp.valid, MBEM_ERR_UNSUPPORTED, "nodal degrees beyond the P2 tables");
    NodalArgs a;
    memset(&a, 0, sizeof(a));
    a.x_field = x; a.n_field_pts = nf; a.tri_verts = tv; a.normals = normals; a.eps = eps; a.n_src = ns;
    a.density = density;
    for (int i = 0; i < 6; i++) a.c[i] = (coeffs && i < (kind == 0 ? 6 : 3)) ? coeffs[i] : 0.0;
    a.mu = mu; a.lam = lam; a.alpha = alpha; a.accumulate = accumulate; a.out = out;
    if (nf == 0) return MBEM_OK;
    int split = 1;      // about eight 64-thread blocks per SM (152 SMs)
    while (split < 16 && nf * split < (int64_t)152 * 8 * ND_THREADS) split *= 2;
    nodal_contract_kernel<<<(unsigned)ceil_div(nf, ND_THREADS / split), ND_THREADS, 0, (cudaStream_t)stream>>>(
        a, sp, kind, split);
    return launch_status("nodal_contract_kernel");
}

}  // namespace mbem

extern "C" int mbem_near_eval_nodal(int kernel, int order, const double* x_field, int64_t n_field,
                                    const double* tri_verts, const double* normals, const double* eps,
                                    const int64_t* rowptr, const int64_t* cols, int64_t nnz, const double* coeffs,
                                    double alpha, double* vals, void* stream) {
    using namespace mbem;
    MBEM_REQUIRE(kernel == 0 || kernel == 1, MBEM_ERR_ARG, "kernel must be 0 (T) or 1 (U)");
    MBEM_REQUIRE(order == 1 || order == 2, MBEM_ERR_ARG, "nodal order must be 1 or 2 (order 0: mbem_near_eval)");
    MBEM_REQUIRE(kernel == 1 || normals, MBEM_ERR_ARG, "normals is NULL");
    MBEM_REQUIRE(coeffs && n_field >= 0 && nnz >= 0 && (nnz == 0 || (rowptr && cols && vals)), MBEM_ERR_ARG,
                 "bad nodal near-eval args");
    if (nnz == 0) return MBEM_OK;
    int e = ensure_rules();
    if (e) return e;
    const NodalSpec sp = make_spec(order, kernel == 0 ? KF_T : KF_U);
    MBEM_REQUIRE(sp.valid, MBEM_ERR_UNSUPPORTED, "nodal degrees beyond the P2 tables");
    NodalArgs a;
    memset(&a, 0, sizeof(a));
    a.x_field = x_field; a.n_field_pts = n_field; a.tri_verts = tri_verts; a.normals = normals; a.eps = eps;
    const int nc = kernel == 0 ? 6 : 3;
    for (int i = 0; i < 6; i++) a.c[i] = i < nc ? coeffs[i] : 0.0;
    a.alpha = alpha;
    nodal_near_eval_kernel<<<(unsigned)ceil_div(nnz, ND_THREADS), ND_THREADS, 0, (cudaStream_t)stream>>>(
        a, sp, kernel, rowptr, cols, nnz, vals);
    return launch_status("nodal_near_eval_kernel");
}

namespace mbem {
// FP64 traction blocks of listed (field point, source) pairs of an order-0
// source patch (the near pairs of the mixed operator's traction rows), added
// into out at column 3 s + j: the per-pair code of mbem_traction_matrix.
int traction_pairs(const double* x_field, const double* n_field, int64_t n_pts, const double* tri_verts,
                   const double* normals, const double* eps, int64_t n_src, double mu, double lam, int which,
                   double alpha, const int64_t* rowptr, const int64_t* cols, int64_t nnz, double* out, int64_t ld,
                   cudaStream_t st) {
    int e = ensure_rules();
    if (e) return e;
    const int flags = (which == 1) ? KF_S : (which == 2 ? KF_E : KF_H);
    const NodalSpec sp = make_spec(0, flags);
    MBEM_REQUIRE(sp.valid, MBEM_ERR_UNSUPPORTED, "nodal degrees beyond the P2 tables");
    NodalArgs a;
    memset(&a, 0, sizeof(a));
    a.x_field = x_field; a.n_field = n_field; a.n_field_pts = n_pts; a.tri_verts = tri_verts;
    a.normals = normals; a.eps = eps; a.n_src = n_src; a.n_cols = n_src;
    a.mu = mu; a.lam = lam; a.alpha = alpha; a.which = which; a.out = out; a.ld = ld;
    a.pair_rowptr = rowptr; a.pair_cols = cols; a.n_pairs = nnz;
    a.ids = nullptr;
    if (nnz == 0) return MBEM_OK;
    nodal_traction_kernel<<<(unsigned)ceil_div(nnz, ND_THREADS), ND_THREADS, 0, st>>>(a, sp);
    return launch_status("nodal_traction_kernel");
}
}  // namespace mbem

extern "C" int mbem_traction_matrix(const double* x_field, const double* n_field, int64_t n_pts,
                                    const double* tri_verts, const double* normals, const double* eps,
                                    int64_t n_src, const int64_t* ids, int64_t n_cols, double mu, double lam,
                                    int order, int which, double alpha, double* out, int64_t ld_out,
                                    void* stream) {
    using namespace mbem;
    MBEM_REQUIRE(order >= 0 && order <= 2, MBEM_ERR_ARG, "order must be 0, 1 or 2 (got %d)", order);
    MBEM_REQUIRE(which >= 0 && which <= 3, MBEM_ERR_ARG, "which must be 0..3 (got %d)", which);
    MBEM_REQUIRE(n_pts >= 0 && n_src >= 0 && n_cols >= 0 && ld_out >= 3 * n_cols, MBEM_ERR_ARG,
                 "bad traction shape");
    MBEM_REQUIRE(n_src == 0 || (tri_verts && (normals || which == 1) && eps && ids), MBEM_ERR_ARG,
                 "NULL source arrays");
    MBEM_REQUIRE(n_pts == 0 || (x_field && n_field && out), MBEM_ERR_ARG, "NULL field arrays");
    MBEM_REQUIRE(mu > 0.0 && lam + mu > 0.0, MBEM_ERR_ARG, "material (mu=%g, lam=%g)", mu, lam);
    int e = ensure_rules();
    if (e) return e;
    // tri_nodal.py:1367 _TRACTION_KINDS: slip and total share the H tables
    const int flags = (which == 1) ? KF_S : (which == 2 ? KF_E : KF_H);
    const NodalSpec sp = make_spec(order, flags);
    MBEM_REQUIRE(sp.valid, MBEM_ERR_UNSUPPORTED, "nodal degrees beyond the P2 tables");
    NodalArgs a;
    memset(&a, 0, sizeof(a));
    a.x_field = x_field; a.n_field = n_field; a.n_field_pts = n_pts; a.tri_verts = tri_verts;
    a.normals = normals; a.eps = eps; a.n_src = n_src; a.ids = ids; a.n_cols = n_cols;
    a.mu = mu; a.lam = lam; a.alpha = alpha; a.which = which; a.out = out; a.ld = ld_out;
    if (n_pts == 0 || n_src == 0) return MBEM_OK;
    nodal_traction_kernel<<<(unsigned)ceil_div(n_pts * n_src, ND_THREADS), ND_THREADS, 0, (cudaStream_t)stream>>>(
        a, sp);
    return launch_status("nodal_traction_kernel");
}
