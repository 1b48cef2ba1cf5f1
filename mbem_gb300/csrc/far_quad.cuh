// The far-field quadrature of the P0 pair kernels in FP32, shared by the mixed
// operator (mixed.cu) and the compressed pair operator (aca.cu): collapsed
// Gauss-Legendre rules on the source triangle, per-source constants, the
// near / far decision and the T (double layer) and U (single layer) blocks.
#pragma once
#include <math.h>

#include "common.cuh"
#include "dfloat.cuh"

namespace mbem {

// ---------------------------------------------------------------------------
// quadrature rules on (0,0),(1,0),(0,1): collapsed Gauss-Legendre n x n
// (code n, n^2 points, exact to total degree 2n - 2), and Radon's symmetric
// 7-point rule (code QR_RADON, exact to degree 5: the centroid and two orbits
// of three points, from Radon (1948) / Stroud's table T2:5-1)
// ---------------------------------------------------------------------------
constexpr int QR_MIN = 3, QR_MAX = 8;      // P0 uses n = 4..6; nodal densities up to 8
constexpr int QR_RADON = 2;                // the code of the 7-point rule
constexpr int QR_POINTS = 9 + 16 + 25 + 36 + 49 + 64 + 7;

__host__ __device__ __forceinline__ int rule_points(int code) { return code == QR_RADON ? 7 : code * code; }

struct QuadRules {
    float a[QR_POINTS];    // xi1 - 1/3
    float b[QR_POINTS];    // xi2 - 1/3
    float w[QR_POINTS];    // weights, sum 1/2 per rule
    int off[QR_MAX + 1];
};

// Gauss-Legendre nodes/weights on [-1, 1] by Newton iteration on P_n.
static void gauss_legendre(int n, double* x, double* w) {
    for (int i = 0; i < n; i++) {
        double z = cos(MBEM_PI * (i + 0.75) / (n + 0.5));
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; k++) {
                double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            double dp = n * (z * p1 - p0) / (z * z - 1.0);
            double dz = p1 / dp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        double p0 = 1.0, p1 = z;
        for (int k = 2; k <= n; k++) {
            double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
            p0 = p1;
            p1 = p2;
        }
        double dp = n * (z * p1 - p0) / (z * z - 1.0);
        x[i] = z;
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

static QuadRules make_rules() {
    QuadRules r;
    int k = 0;
    for (int n = 0; n <= QR_MAX; n++) r.off[n] = 0;
    for (int n = QR_MIN; n <= QR_MAX; n++) {
        r.off[n] = k;
        double g[QR_MAX], gw[QR_MAX];
        gauss_legendre(n, g, gw);
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                const double gi = 0.5 * (g[i] + 1.0), gj = 0.5 * (g[j] + 1.0);
                const double wi = 0.5 * gw[i], wj = 0.5 * gw[j];
                const double x1 = gi, x2 = gj * (1.0 - gi);
                r.a[k] = (float)(x1 - 1.0 / 3.0);
                r.b[k] = (float)(x2 - 1.0 / 3.0);
                r.w[k] = (float)(wi * wj * (1.0 - gi));
                k++;
            }
    }
    // Radon: weights for the triangle of area 1/2
    r.off[QR_RADON] = k;
    const double s15 = sqrt(15.0);
    const double orbit[2][3] = {{(6.0 - s15) / 21.0, (9.0 + 2.0 * s15) / 21.0, (155.0 - s15) / 2400.0},
                                {(6.0 + s15) / 21.0, (9.0 - 2.0 * s15) / 21.0, (155.0 + s15) / 2400.0}};
    r.a[k] = 0.0f;
    r.b[k] = 0.0f;
    r.w[k] = (float)(9.0 / 80.0);
    k++;
    for (int o = 0; o < 2; o++) {
        const double p = orbit[o][0], q = orbit[o][1];
        const double pts[3][2] = {{p, p}, {p, q}, {q, p}};
        for (int t = 0; t < 3; t++) {
            r.a[k] = (float)(pts[t][0] - 1.0 / 3.0);
            r.b[k] = (float)(pts[t][1] - 1.0 / 3.0);
            r.w[k] = (float)orbit[o][2];
            k++;
        }
    }
    return r;
}

static const QuadRules& rules() {
    static const QuadRules r = make_rules();
    return r;
}

// ---------------------------------------------------------------------------
// double-float helpers
// ---------------------------------------------------------------------------
// (a_hi + a_lo) - (b_hi + b_lo) rounded to FP32 with the hi difference exact
// (Knuth's TwoSum; the _rn intrinsics keep the compiler from contracting or
// reassociating the error-free steps)
__device__ __forceinline__ float df_diff(F2 a, F2 b) {
    const float s = __fsub_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(-b.hi, bb));
    return __fadd_rn(s, __fadd_rn(err, __fsub_rn(a.lo, b.lo)));
}

// ---------------------------------------------------------------------------
// per-source far-field constants
// ---------------------------------------------------------------------------
struct SrcFar {
    F2 c[3];            // centroid
    float e1[3], e2[3]; // edges from vertex 0
    float n[3];         // normal as passed (T kernel)
    float area2, eps2;
    float L2;           // longest edge squared
    float rnear2;       // near radius squared
    bool ok;
};

// Edges as exact FP64 differences rounded to FP32, the centroid in
// double-float, twice the area in FP64 (it scales every entry of the source:
// an FP32 cross product would bias each source's column by ~1e-7); the
// lengths and radii, which only choose rules and near pairs, in FP32 (the FP64
// pipe runs 1/64 of FP32 here, and every CTA of the far-field kernels sets up
// its sources).
__device__ __forceinline__ void far_setup(const double* __restrict__ tv, const double* __restrict__ nrm,
                                          double eps, double near_factor, SrcFar& s) {
    const double d1x = tv[3] - tv[0], d1y = tv[4] - tv[1], d1z = tv[5] - tv[2];
    const double d2x = tv[6] - tv[0], d2y = tv[7] - tv[1], d2z = tv[8] - tv[2];
    const double cx = d1y * d2z - d1z * d2y, cy = d1z * d2x - d1x * d2z, cz = d1x * d2y - d1y * d2x;
    const float a2 = (float)sqrt(cx * cx + cy * cy + cz * cz);
    const float e1x = (float)d1x, e1y = (float)d1y, e1z = (float)d1z;
    const float e2x = (float)d2x, e2y = (float)d2y, e2z = (float)d2z;
    const float e3x = (float)(tv[6] - tv[3]), e3y = (float)(tv[7] - tv[4]), e3z = (float)(tv[8] - tv[5]);
    s.ok = a2 >= 1e-30f;
    const float l1 = sqrtf(e1x * e1x + e1y * e1y + e1z * e1z);
    const float l2 = sqrtf(e2x * e2x + e2y * e2y + e2z * e2z);
    const float l3 = sqrtf(e3x * e3x + e3y * e3y + e3z * e3z);
    const float Lm = fmaxf(fmaxf(l1, l2), l3);
    const float h = (l1 + l2 + l3) * (1.0f / 3.0f);    // mean edge length
    const float rn = (float)near_factor * fmaxf((float)eps, h);
    for (int k = 0; k < 3; k++) s.c[k] = split_d((tv[k] + tv[3 + k] + tv[6 + k]) * (1.0 / 3.0));
    s.e1[0] = e1x; s.e1[1] = e1y; s.e1[2] = e1z;
    s.e2[0] = e2x; s.e2[1] = e2y; s.e2[2] = e2z;
    if (nrm) {
        s.n[0] = (float)nrm[0]; s.n[1] = (float)nrm[1]; s.n[2] = (float)nrm[2];
    } else {
        s.n[0] = s.n[1] = s.n[2] = 0.0f;
    }
    s.area2 = a2;
    s.eps2 = (float)(eps * eps);
    s.L2 = Lm * Lm;
    s.rnear2 = fmaxf(rn * rn, 2.25f * Lm * Lm);
}

// The one near/far decision, shared by every kernel that needs it.
__device__ __forceinline__ bool is_near(const F2 x[3], const SrcFar& s, float d[3], float& D2) {
    d[0] = df_diff(x[0], s.c[0]);
    d[1] = df_diff(x[1], s.c[1]);
    d[2] = df_diff(x[2], s.c[2]);
    D2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    return D2 < s.rnear2;
}

// the collapsed rule n by D / L_max (measured against the FP64 closed form:
// <= ~1.7e-7); the nodal far blocks add their order to it
__device__ __forceinline__ int far_rule_collapsed(float D2, float L2) {
    if (D2 >= 50.0f * L2) return 3;        // D/L >= 7.07
    if (D2 >= 8.0f * L2) return 4;         // D/L >= 2.83
    if (D2 >= 3.125f * L2) return 5;       // D/L >= 1.77
    return 6;
}

// the P0 rule: Radon's 7 points from D/L >= 5 (<= 8.8e-8 of the closed form
// there, 1.1e-8 at D/L = 7.07 where the collapsed 3 x 3 rule's 9 points give
// 1.7e-7), else the collapsed rules
__device__ __forceinline__ int far_rule(float D2, float L2) {
    if (D2 >= 25.0f * L2) return QR_RADON;
    return far_rule_collapsed(D2, L2);
}

// Far T block (FP32): out_ij = n_j alpha_i + n_i beta_j + d_ij gamma - 6 c5 W_ij
// from the quadrature sums V3 = int d/R^3, V5 = int d/R^5,
// t = int d |d|^2/R^5, W = int d d (d.n)/R^5 (d = x - y).
// U block: out_ij = c2 W_ij + d_ij (c0 I1 + c1 eps^2 I3), W = int d d / R^3.
struct FarSums {
    float V3[3], V5[3], t[3];
    float W00, W01, W02, W11, W12, W22;
    float I1, I3;
};

template <bool TKERNEL>
__device__ __forceinline__ void far_epilogue(const SrcFar& s, const FarSums& m, const float c[6], float out[3][3]) {
    const float A = s.area2;
    const float W[3][3] = {{m.W00, m.W01, m.W02}, {m.W01, m.W11, m.W12}, {m.W02, m.W12, m.W22}};
    if (TKERNEL) {
        const float* n = s.n;
        const float nV3 = n[0] * m.V3[0] + n[1] * m.V3[1] + n[2] * m.V3[2];
        const float nV5 = n[0] * m.V5[0] + n[1] * m.V5[1] + n[2] * m.V5[2];
        const float ca = c[0] + 4.0f * c[1] + 2.0f * c[4];
        const float cb = c[3] + c[4];
        const float ce3 = c[2] * s.eps2, ce6 = c[5] * s.eps2;
        const float gam = cb * nV3 + ce6 * nV5;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const float al = ca * m.V3[i] - 3.0f * c[1] * m.t[i] + ce3 * m.V5[i];
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const float be = cb * m.V3[j] + ce6 * m.V5[j];
                out[i][j] = A * (n[j] * al + n[i] * be - 6.0f * c[4] * W[i][j] + (i == j ? gam : 0.0f));
            }
        }
    } else {
        const float dg = c[0] * m.I1 + c[1] * s.eps2 * m.I3;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) out[i][j] = A * (c[2] * W[i][j] + (i == j ? dg : 0.0f));
    }
}

template <bool TKERNEL>
__device__ __forceinline__ void far_block(const QuadRules& Q, const SrcFar& s, const float dc[3], float D2,
                                          const float c[6], float out[3][3]) {
    const int nq = far_rule(D2, s.L2);
    const int q0 = Q.off[nq], q1 = q0 + rule_points(nq);
    FarSums m = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int q = q0; q < q1; q++) {
        const float a = Q.a[q], b = Q.b[q];
        const float dx = dc[0] - (a * s.e1[0] + b * s.e2[0]);
        const float dy = dc[1] - (a * s.e1[1] + b * s.e2[1]);
        const float dz = dc[2] - (a * s.e1[2] + b * s.e2[2]);
        const float r2 = dx * dx + dy * dy + dz * dz;
        const float iR = rsqrtf(r2 + s.eps2);
        const float w = Q.w[q];
        const float iR2 = iR * iR;
        const float w3 = w * iR2 * iR;
        if (TKERNEL) {
            const float w5 = w3 * iR2;
            m.V3[0] += w3 * dx; m.V3[1] += w3 * dy; m.V3[2] += w3 * dz;
            m.V5[0] += w5 * dx; m.V5[1] += w5 * dy; m.V5[2] += w5 * dz;
            const float wt = w5 * r2;
            m.t[0] += wt * dx; m.t[1] += wt * dy; m.t[2] += wt * dz;
            const float wn = w5 * (dx * s.n[0] + dy * s.n[1] + dz * s.n[2]);
            const float ux = wn * dx, uy = wn * dy, uz = wn * dz;
            m.W00 += ux * dx; m.W01 += ux * dy; m.W02 += ux * dz;
            m.W11 += uy * dy; m.W12 += uy * dz; m.W22 += uz * dz;
        } else {
            m.I1 += w * iR;
            m.I3 += w3;
            const float ux = w3 * dx, uy = w3 * dy, uz = w3 * dz;   // T2[3] = int d d / R^3
            m.W00 += ux * dx; m.W01 += ux * dy; m.W02 += ux * dz;
            m.W11 += uy * dy; m.W12 += uy * dz; m.W22 += uz * dz;
        }
    }
    far_epilogue<TKERNEL>(s, m, c, out);
}

// Two field points of one source at once (both far), in packed FP32
// (FFMA2 / FMUL2 / FADD2 on float2 lanes): the quadrature point offsets are
// shared, every per-point quantity is a pair. Both points take the rule of
// the nearer one (a rule at least as accurate as its own for the farther).
__device__ __forceinline__ float2 f2s(float v) { return make_float2(v, v); }

template <bool TKERNEL>
__device__ __forceinline__ void far_block2(const QuadRules& Q, const SrcFar& s, const float da[3], const float db[3],
                                           float D2a, float D2b, const float c[6], float outa[3][3],
                                           float outb[3][3]) {
    const int nq = far_rule(fminf(D2a, D2b), s.L2);
    const int q0 = Q.off[nq], q1 = q0 + rule_points(nq);
    const float2 dc0 = make_float2(da[0], db[0]), dc1 = make_float2(da[1], db[1]), dc2 = make_float2(da[2], db[2]);
    const float2 e2 = f2s(s.eps2);
    const float2 n0 = f2s(s.n[0]), n1 = f2s(s.n[1]), n2 = f2s(s.n[2]);
    const float2 z = f2s(0.0f);
    float2 V30 = z, V31 = z, V32 = z, V50 = z, V51 = z, V52 = z, t0 = z, t1 = z, t2 = z;
    float2 W00 = z, W01 = z, W02 = z, W11 = z, W12 = z, W22 = z, I1 = z, I3 = z;
    for (int q = q0; q < q1; q++) {
        const float a = Q.a[q], b = Q.b[q];
        const float ox = a * s.e1[0] + b * s.e2[0];
        const float oy = a * s.e1[1] + b * s.e2[1];
        const float oz = a * s.e1[2] + b * s.e2[2];
        const float2 dx = __fadd2_rn(dc0, f2s(-ox));
        const float2 dy = __fadd2_rn(dc1, f2s(-oy));
        const float2 dz = __fadd2_rn(dc2, f2s(-oz));
        const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
        const float2 re = __fadd2_rn(r2, e2);
        const float2 iR = make_float2(rsqrtf(re.x), rsqrtf(re.y));
        const float2 w = f2s(Q.w[q]);
        const float2 iR2 = __fmul2_rn(iR, iR);
        const float2 w3 = __fmul2_rn(__fmul2_rn(w, iR2), iR);
        if (TKERNEL) {
            const float2 w5 = __fmul2_rn(w3, iR2);
            V30 = __ffma2_rn(w3, dx, V30); V31 = __ffma2_rn(w3, dy, V31); V32 = __ffma2_rn(w3, dz, V32);
            V50 = __ffma2_rn(w5, dx, V50); V51 = __ffma2_rn(w5, dy, V51); V52 = __ffma2_rn(w5, dz, V52);
            const float2 wt = __fmul2_rn(w5, r2);
            t0 = __ffma2_rn(wt, dx, t0); t1 = __ffma2_rn(wt, dy, t1); t2 = __ffma2_rn(wt, dz, t2);
            const float2 dn = __ffma2_rn(dx, n0, __ffma2_rn(dy, n1, __fmul2_rn(dz, n2)));
            const float2 wn = __fmul2_rn(w5, dn);
            const float2 ux = __fmul2_rn(wn, dx), uy = __fmul2_rn(wn, dy), uz = __fmul2_rn(wn, dz);
            W00 = __ffma2_rn(ux, dx, W00); W01 = __ffma2_rn(ux, dy, W01); W02 = __ffma2_rn(ux, dz, W02);
            W11 = __ffma2_rn(uy, dy, W11); W12 = __ffma2_rn(uy, dz, W12); W22 = __ffma2_rn(uz, dz, W22);
        } else {
            I1 = __ffma2_rn(w, iR, I1);
            I3 = __fadd2_rn(I3, w3);
            const float2 ux = __fmul2_rn(w3, dx), uy = __fmul2_rn(w3, dy), uz = __fmul2_rn(w3, dz);
            W00 = __ffma2_rn(ux, dx, W00); W01 = __ffma2_rn(ux, dy, W01); W02 = __ffma2_rn(ux, dz, W02);
            W11 = __ffma2_rn(uy, dy, W11); W12 = __ffma2_rn(uy, dz, W12); W22 = __ffma2_rn(uz, dz, W22);
        }
    }
    const FarSums ma = {{V30.x, V31.x, V32.x}, {V50.x, V51.x, V52.x}, {t0.x, t1.x, t2.x}, W00.x, W01.x, W02.x,
                        W11.x, W12.x, W22.x, I1.x, I3.x};
    const FarSums mb = {{V30.y, V31.y, V32.y}, {V50.y, V51.y, V52.y}, {t0.y, t1.y, t2.y}, W00.y, W01.y, W02.y,
                        W11.y, W12.y, W22.y, I1.y, I3.y};
    far_epilogue<TKERNEL>(s, ma, c, outa);
    far_epilogue<TKERNEL>(s, mb, c, outb);
}


}  // namespace mbem
