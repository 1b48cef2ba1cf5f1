// FP64 device code for one (observer, P0 source triangle) pair of the
// mollified Kelvin kernels.
//
// The mathematics is the reference's (src/mbem/kernels/tri_kernels.py): the
// observer is lifted to h = sqrt(z^2 + eps^2) over the source plane, the 2-D
// area moments M_n[a,b] = int xi1^a xi2^b / R^n come from the solid angle
// (I3 = -Omega/h) and the divergence-theorem recursion over the three edges,
// and every kernel is a contraction of those moments. The GPU formulation
// differs in what it materialises:
//
//  * all per-source quantities (frame, in-plane vertices, edge tangents,
//    twice the area) are computed once per source and kept in registers;
//  * the lifted-point solid angle uses the in-plane triple product
//    r1.(r2 x r3) = -h * (twice the signed area), exact for the lifted point;
//  * the vertex distances R_k = sqrt(|p_k|^2 + h^2) are shared by the solid
//    angle and the six edge endpoints (the reference recomputes them);
//  * the T-kernel block needs only V3, V5, the trace t_i = T3[i,m,m] and
//    W = T3 . n, so the rank-3 tensor is never built; the stress kernels are
//    contracted with the density in the source frame before rotating back.
// All of these are exact rewrites; results agree with the reference to a
// few ulps of the moments involved.
#pragma once

#include "common.cuh"

namespace mbem {

struct SrcP0 {
    double v0[3];
    double ex[3], ey[3], nh[3];
    double Px1, Px2, Py1, Py2;   // in-plane coordinates of vertices 1, 2 (vertex 0 at origin)
    double tx[3], ty[3];         // unit in-plane edge tangents, edge e = (e, e+1)
    double area2;                // twice the signed in-plane area
    double eps, eps2;
    bool ok;                     // false for a degenerate triangle (zero block)
    bool edge_ok[3];
};

// Frame of a source triangle (tri_kernels.py:137-153) and its per-source
// constants. `tv` points at 9 doubles (vertex-major).
__device__ __forceinline__ void src_setup(const double* __restrict__ tv, double eps, SrcP0& s) {
    double e1x = tv[3] - tv[0], e1y = tv[4] - tv[1], e1z = tv[5] - tv[2];
    double e2x = tv[6] - tv[0], e2y = tv[7] - tv[1], e2z = tv[8] - tv[2];
    double cx = e1y * e2z - e1z * e2y;
    double cy = e1z * e2x - e1x * e2z;
    double cz = e1x * e2y - e1y * e2x;
    double a2 = sqrt(cx * cx + cy * cy + cz * cz);
    s.ok = a2 >= 1e-30;
    s.eps = eps;
    s.eps2 = eps * eps;
    s.v0[0] = tv[0]; s.v0[1] = tv[1]; s.v0[2] = tv[2];
    if (!s.ok) {
        // never used: the caller writes a zero block
        for (int k = 0; k < 3; k++) {
            s.ex[k] = s.ey[k] = s.nh[k] = 0.0;
            s.tx[k] = s.ty[k] = 0.0;
            s.edge_ok[k] = false;
        }
        s.Px1 = s.Px2 = s.Py1 = s.Py2 = s.area2 = 0.0;
        return;
    }
    double ia = 1.0 / a2;
    s.nh[0] = cx * ia; s.nh[1] = cy * ia; s.nh[2] = cz * ia;
    double e1n = sqrt(e1x * e1x + e1y * e1y + e1z * e1z);
    double ie = 1.0 / e1n;
    s.ex[0] = e1x * ie; s.ex[1] = e1y * ie; s.ex[2] = e1z * ie;
    s.ey[0] = s.nh[1] * s.ex[2] - s.nh[2] * s.ex[1];
    s.ey[1] = s.nh[2] * s.ex[0] - s.nh[0] * s.ex[2];
    s.ey[2] = s.nh[0] * s.ex[1] - s.nh[1] * s.ex[0];
    s.Px1 = e1x * s.ex[0] + e1y * s.ex[1] + e1z * s.ex[2];
    s.Py1 = e1x * s.ey[0] + e1y * s.ey[1] + e1z * s.ey[2];
    s.Px2 = e2x * s.ex[0] + e2y * s.ex[1] + e2z * s.ex[2];
    s.Py2 = e2x * s.ey[0] + e2y * s.ey[1] + e2z * s.ey[2];
    s.area2 = s.Px1 * s.Py2 - s.Px2 * s.Py1;
    const double Px[3] = {0.0, s.Px1, s.Px2};
    const double Py[3] = {0.0, s.Py1, s.Py2};
#pragma unroll
    for (int e = 0; e < 3; e++) {
        int b = (e + 1) % 3;
        double evx = Px[b] - Px[e], evy = Py[b] - Py[e];
        double L = sqrt(evx * evx + evy * evy);
        s.edge_ok[e] = L > 1e-30;
        double iL = s.edge_ok[e] ? 1.0 / L : 0.0;
        s.tx[e] = evx * iL;
        s.ty[e] = evy * iL;
    }
}

// Pair geometry shared by all kernels: height, lift, projected vertices,
// vertex distances and I3 = -Omega / h (tri_kernels.py:257-273).
struct PairP0 {
    double z, h2, h, ih2;        // ih2 = 1 / h^2
    double px[3], py[3];
    double R[3], iR[3];
    double I3;
};

// FP64 work is the cost of every pair (the FP64 pipe is 1/64 of FP32 on
// this part), so reciprocals come from rsqrt (R and 1/R from one call) and
// from shared divisions.
__device__ __forceinline__ void pair_setup(const SrcP0& s, double ox, double oy, double oz, PairP0& p) {
    double dx = ox - s.v0[0], dy = oy - s.v0[1], dz = oz - s.v0[2];
    p.z = dx * s.nh[0] + dy * s.nh[1] + dz * s.nh[2];
    double qx = dx * s.ex[0] + dy * s.ex[1] + dz * s.ex[2];
    double qy = dx * s.ey[0] + dy * s.ey[1] + dz * s.ey[2];
    p.h2 = p.z * p.z + s.eps2;
    const double ih = rsqrt(p.h2);
    p.h = p.h2 * ih;
    p.ih2 = ih * ih;
    p.px[0] = -qx;          p.py[0] = -qy;
    p.px[1] = s.Px1 - qx;   p.py[1] = s.Py1 - qy;
    p.px[2] = s.Px2 - qx;   p.py[2] = s.Py2 - qy;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const double r2 = p.px[k] * p.px[k] + p.py[k] * p.py[k] + p.h2;
        p.iR[k] = rsqrt(r2);
        p.R[k] = r2 * p.iR[k];
    }
    // van Oosterom at the lifted point, in the source frame: r_k = (px, py, -h)
    double d01 = p.px[0] * p.px[1] + p.py[0] * p.py[1] + p.h2;
    double d12 = p.px[1] * p.px[2] + p.py[1] * p.py[2] + p.h2;
    double d02 = p.px[0] * p.px[2] + p.py[0] * p.py[2] + p.h2;
    double numer = -p.h * s.area2;
    double denom = p.R[0] * p.R[1] * p.R[2] + p.R[2] * d01 + p.R[0] * d12 + p.R[1] * d02;
    double omega = 2.0 * atan2(numer, denom);
    p.I3 = -omega * ih;
}

// Per-edge primitive differences at orders 1 and 3 (tri_kernels.py:54-76,
// :298-302): J1 = log(u + R), K1 = R, J3 = u / (rho^2 R), K3 = -1/R.
struct EdgeP0 {
    double nx, ny, tx, ty, dp, ua, ub, rho2, ir2;
    double dJ1, dK1, dJ3, dK3, dL3;
};

// All three edges at once: dJ1 = log((u_b + R_b) / (u_a + R_a)) takes one
// log per edge, and the three quotients and the three 1/rho^2 share one
// division each through the product of their denominators.
__device__ __forceinline__ void edges_setup(const SrcP0& s, const PairP0& p, EdgeP0 g[3]) {
    double num[3], den[3];
#pragma unroll
    for (int e = 0; e < 3; e++) {
        const int a = e, b = (e + 1) % 3;
        g[e].tx = s.tx[e]; g[e].ty = s.ty[e];
        g[e].nx = g[e].ty; g[e].ny = -g[e].tx;
        g[e].dp = p.px[a] * g[e].nx + p.py[a] * g[e].ny;
        g[e].ua = p.px[a] * g[e].tx + p.py[a] * g[e].ty;
        g[e].ub = p.px[b] * g[e].tx + p.py[b] * g[e].ty;
        g[e].rho2 = s.edge_ok[e] ? g[e].dp * g[e].dp + p.h2 : 1.0;
        num[e] = s.edge_ok[e] ? g[e].ub + p.R[b] + 1e-300 : 1.0;
        den[e] = s.edge_ok[e] ? g[e].ua + p.R[a] + 1e-300 : 1.0;
        g[e].dK1 = p.R[b] - p.R[a];
        g[e].dK3 = p.iR[a] - p.iR[b];
    }
    const double r01 = g[0].rho2 * g[1].rho2;
    const double d01 = den[0] * den[1];
    const bool tiny = fmin(fmin(g[0].rho2, g[1].rho2), g[2].rho2) < 1e-60;
    const double ir = tiny ? 0.0 : 1.0 / (r01 * g[2].rho2);
    const double id = 1.0 / (d01 * den[2]);
    g[0].ir2 = g[1].rho2 * g[2].rho2 * ir;
    g[1].ir2 = g[0].rho2 * g[2].rho2 * ir;
    g[2].ir2 = r01 * ir;
    if (tiny) {
#pragma unroll
        for (int e = 0; e < 3; e++) g[e].ir2 = (g[e].rho2 < 1e-60) ? 0.0 : 1.0 / g[e].rho2;
    }
    const double q[3] = {num[0] * den[1] * den[2] * id, num[1] * den[0] * den[2] * id, num[2] * d01 * id};
#pragma unroll
    for (int e = 0; e < 3; e++) {
        const int a = e, b = (e + 1) % 3;
        g[e].dJ1 = log(q[e]);
        g[e].dJ3 = (g[e].ub * p.iR[b] - g[e].ua * p.iR[a]) * g[e].ir2;
        g[e].dL3 = g[e].dJ1 - g[e].rho2 * g[e].dJ3;
    }
}

// ---------------------------------------------------------------------------
// T kernel (slip -> displacement): the combined 3x3 block
//   out_ij = sum_b c_b B_b,ij,  B = [N[P1], N[P2], N[P3], R[P1], R[P2], R[P3]]
// (tri_kernels.py:251-427 with the coefficients of basis.py:58-72).
// With V3, V5 (first moments), t_i = sum_m T3[i,m,m] and W_ij = T3[i,j,.].n:
//   N1 = n_j V3_i          R1 = d_ij n.V3 + n_i V3_j
//   N2 = n_j (4 V3_i - 3 t_i)
//   R2 = n_i V3_j + 2 n_j V3_i + d_ij n.V3 - 6 W_ij
//   N3 = eps^2 n_j V5_i    R3 = eps^2 (d_ij n.V5 + n_i V5_j)
// ---------------------------------------------------------------------------
struct TMoments {
    double V3[3], V5[3], t[3], W[3][3];   // global frame
};

// T-kernel moments V3, V5, t, W (global frame) from the 2-D moments of the
// source frame (ex, ey, nh); shared by the P0 pair and the nodal tables.
struct TScal {
    double z, I3, I5, m10_3, m01_3, m10_5, m01_5, m20_5, m11_5, m02_5, m30_5, m21_5, m12_5, m03_5;
};

__device__ __forceinline__ void t_from_scal(const double* ex, const double* ey, const double* nh,
                                            const double* __restrict__ nrm, const TScal& q, TMoments& m) {
    const double z = q.z, I3 = q.I3, I5 = q.I5;
    const double m10_3 = q.m10_3, m01_3 = q.m01_3, m10_5 = q.m10_5, m01_5 = q.m01_5;
    const double m20_5 = q.m20_5, m11_5 = q.m11_5, m02_5 = q.m02_5;
    const double m30_5 = q.m30_5, m21_5 = q.m21_5, m12_5 = q.m12_5, m03_5 = q.m03_5;
    // local frame (ex, ey, nh): d = (-xi1, -xi2, z)
    const double V3l[3] = {-m10_3, -m01_3, z * I3};
    const double V5l[3] = {-m10_5, -m01_5, z * I5};
    const double z2 = z * z;
    // T3 in the local frame, T[a][b][c] = (-1)^(#0+#1) z^(#2) M5(#0,#1)
    const double T000 = -m30_5, T001 = -m21_5, T002 = z * m20_5, T011 = -m12_5,
                 T012 = z * m11_5, T022 = -z2 * m10_5, T111 = -m03_5, T112 = z * m02_5,
                 T122 = -z2 * m01_5, T222 = z2 * z * I5;
    const double tl[3] = {T000 + T011 + T022, T001 + T111 + T122, T002 + T112 + T222};
    // local normal of the source normal passed in (may differ from nh)
    const double nl0 = nrm[0] * ex[0] + nrm[1] * ex[1] + nrm[2] * ex[2];
    const double nl1 = nrm[0] * ey[0] + nrm[1] * ey[1] + nrm[2] * ey[2];
    const double nl2 = nrm[0] * nh[0] + nrm[1] * nh[1] + nrm[2] * nh[2];
    double Wl[3][3];
    Wl[0][0] = T000 * nl0 + T001 * nl1 + T002 * nl2;
    Wl[0][1] = T001 * nl0 + T011 * nl1 + T012 * nl2;
    Wl[0][2] = T002 * nl0 + T012 * nl1 + T022 * nl2;
    Wl[1][1] = T011 * nl0 + T111 * nl1 + T112 * nl2;
    Wl[1][2] = T012 * nl0 + T112 * nl1 + T122 * nl2;
    Wl[2][2] = T022 * nl0 + T122 * nl1 + T222 * nl2;
    Wl[1][0] = Wl[0][1]; Wl[2][0] = Wl[0][2]; Wl[2][1] = Wl[1][2];
    // rotate to the global frame: v = Q^T v_l, W = Q^T W_l Q (Q rows ex, ey, nh)
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const double qi[3] = {ex[i], ey[i], nh[i]};
        m.V3[i] = qi[0] * V3l[0] + qi[1] * V3l[1] + qi[2] * V3l[2];
        m.V5[i] = qi[0] * V5l[0] + qi[1] * V5l[1] + qi[2] * V5l[2];
        m.t[i] = qi[0] * tl[0] + qi[1] * tl[1] + qi[2] * tl[2];
    }
    double Y[3][3];  // Y = W_l Q  (3x3 local-by-global)
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            Y[a][j] = Wl[a][0] * ex[j] + Wl[a][1] * ey[j] + Wl[a][2] * nh[j];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
            double w = ex[i] * Y[0][j] + ey[i] * Y[1][j] + nh[i] * Y[2][j];
            m.W[i][j] = w;
            m.W[j][i] = w;
        }
}


__device__ __forceinline__ void t_moments(const SrcP0& s, const double* __restrict__ nrm,
                                          const PairP0& p, TMoments& m) {
    double BN1_001 = 0, BN2_001 = 0, BD003 = 0, BN1_003 = 0, BN2_003 = 0, BN1_103 = 0,
           BN1_013 = 0, BN2_013 = 0, BN1_203 = 0, BN1_113 = 0, BN1_023 = 0, BN2_023 = 0;
    EdgeP0 G[3];
    edges_setup(s, p, G);
#pragma unroll
    for (int e = 0; e < 3; e++) {
        if (!s.edge_ok[e]) continue;
        const EdgeP0& g = G[e];
        double A = g.dp * g.nx, B = g.dp * g.ny;
        double v10 = A * g.dJ3 + g.tx * g.dK3;
        double v01 = B * g.dJ3 + g.ty * g.dK3;
        double v20 = A * A * g.dJ3 + 2.0 * A * g.tx * g.dK3 + g.tx * g.tx * g.dL3;
        double v11 = A * B * g.dJ3 + (A * g.ty + B * g.tx) * g.dK3 + g.tx * g.ty * g.dL3;
        double v02 = B * B * g.dJ3 + 2.0 * B * g.ty * g.dK3 + g.ty * g.ty * g.dL3;
        BN1_001 += g.nx * g.dJ1; BN2_001 += g.ny * g.dJ1;
        BD003 += g.dp * g.dJ3;
        BN1_003 += g.nx * g.dJ3; BN2_003 += g.ny * g.dJ3;
        BN1_103 += g.nx * v10;
        BN1_013 += g.nx * v01; BN2_013 += g.ny * v01;
        BN1_203 += g.nx * v20;
        BN1_113 += g.nx * v11;
        BN1_023 += g.nx * v02; BN2_023 += g.ny * v02;
    }
    const double I3 = p.I3, z = p.z;
    const double I5 = (BD003 + I3) * p.ih2 * (1.0 / 3.0);
    const double third = 1.0 / 3.0;
    const double m10_3 = -BN1_001, m01_3 = -BN2_001;
    const double m10_5 = -BN1_003 * third, m01_5 = -BN2_003 * third;
    const double m20_5 = (I3 - BN1_103) * third, m11_5 = -BN1_013 * third;
    const double m02_5 = (I3 - BN2_013) * third;
    const double m30_5 = (2.0 * m10_3 - BN1_203) * third, m21_5 = (m01_3 - BN1_113) * third;
    const double m12_5 = -BN1_023 * third, m03_5 = (2.0 * m01_3 - BN2_023) * third;
    TScal q{z, I3, I5, m10_3, m01_3, m10_5, m01_5, m20_5, m11_5, m02_5, m30_5, m21_5, m12_5, m03_5};
    t_from_scal(s.ex, s.ey, s.nh, nrm, q, m);
}

// Combined T block with six coefficients.
__device__ __forceinline__ void t_block(const TMoments& m, const double* __restrict__ n,
                                        const double c[6], double eps2, double out[3][3]) {
    const double nV3 = n[0] * m.V3[0] + n[1] * m.V3[1] + n[2] * m.V3[2];
    const double nV5 = n[0] * m.V5[0] + n[1] * m.V5[1] + n[2] * m.V5[2];
    const double ca = c[0] + 4.0 * c[1] + 2.0 * c[4];
    const double cb = c[3] + c[4];
    const double ce3 = c[2] * eps2, ce6 = c[5] * eps2;
    const double gam = cb * nV3 + ce6 * nV5;
    const double w6 = -6.0 * c[4];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const double al = ca * m.V3[i] - 3.0 * c[1] * m.t[i] + ce3 * m.V5[i];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const double bej = cb * m.V3[j] + ce6 * m.V5[j];
            out[i][j] = n[j] * al + n[i] * bej + w6 * m.W[i][j] + (i == j ? gam : 0.0);
        }
    }
}

// The six basis blocks separately (t_basis_matrices, tri_kernels.py:473-492).
__device__ __forceinline__ void t_basis_blocks(const TMoments& m, const double* __restrict__ n,
                                               double eps2, double out[6][3][3]) {
    const double nV3 = n[0] * m.V3[0] + n[1] * m.V3[1] + n[2] * m.V3[2];
    const double nV5 = n[0] * m.V5[0] + n[1] * m.V5[1] + n[2] * m.V5[2];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const double d = (i == j) ? 1.0 : 0.0;
            out[0][i][j] = n[j] * m.V3[i];
            out[1][i][j] = n[j] * (4.0 * m.V3[i] - 3.0 * m.t[i]);
            out[2][i][j] = eps2 * n[j] * m.V5[i];
            out[3][i][j] = d * nV3 + n[i] * m.V3[j];
            out[4][i][j] = n[i] * m.V3[j] + 2.0 * n[j] * m.V3[i] + d * nV3 - 6.0 * m.W[i][j];
            out[5][i][j] = eps2 * (d * nV5 + n[i] * m.V5[j]);
        }
}

// ---------------------------------------------------------------------------
// U kernel (force -> displacement) basis [I1 d, eps^2 I3 d, T2[3]]
// (tri_kernels.py:161-243).
// ---------------------------------------------------------------------------
struct UMoments {
    double I1, I3, T2[3][3];   // T2 in the global frame
};

__device__ __forceinline__ void u_moments(const SrcP0& s, const PairP0& p, UMoments& m) {
    double BD001 = 0, BN1_001 = 0, BN2_001 = 0, BN1_101 = 0, BN1_011 = 0, BN2_011 = 0;
    EdgeP0 G[3];
    edges_setup(s, p, G);
#pragma unroll
    for (int e = 0; e < 3; e++) {
        if (!s.edge_ok[e]) continue;
        const double tx = G[e].tx, ty = G[e].ty, nx = G[e].nx, ny = G[e].ny;
        const double dp = G[e].dp;
        const double dJ1 = G[e].dJ1;
        const double dK1 = G[e].dK1;
        const double v10 = dp * nx * dJ1 + tx * dK1;
        const double v01 = dp * ny * dJ1 + ty * dK1;
        BD001 += dp * dJ1;
        BN1_001 += nx * dJ1; BN2_001 += ny * dJ1;
        BN1_101 += nx * v10;
        BN1_011 += nx * v01; BN2_011 += ny * v01;
    }
    const double I3 = p.I3, z = p.z;
    const double I1 = BD001 - p.h2 * I3;
    const double m10 = -BN1_001, m01 = -BN2_001;
    const double m20 = I1 - BN1_101, m11 = -BN1_011, m02 = I1 - BN2_011;
    // local T2: [0][0]=m20 [0][1]=m11 [1][1]=m02 [0][2]=-z m10 [1][2]=-z m01 [2][2]=z^2 I3
    const double L00 = m20, L01 = m11, L11 = m02, L02 = -z * m10, L12 = -z * m01, L22 = z * z * I3;
    double Y[3][3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
        Y[0][j] = L00 * s.ex[j] + L01 * s.ey[j] + L02 * s.nh[j];
        Y[1][j] = L01 * s.ex[j] + L11 * s.ey[j] + L12 * s.nh[j];
        Y[2][j] = L02 * s.ex[j] + L12 * s.ey[j] + L22 * s.nh[j];
    }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
            double w = s.ex[i] * Y[0][j] + s.ey[i] * Y[1][j] + s.nh[i] * Y[2][j];
            m.T2[i][j] = w;
            m.T2[j][i] = w;
        }
    m.I1 = I1;
    m.I3 = I3;
}

// ---------------------------------------------------------------------------
// Stress moments up to n = 7 (tri_kernels.py:656-769), in the source frame.
// M3: I3, m10, m01.  M5: a+b <= 3.  M7: a+b <= 4 (only when NEED7).
// ---------------------------------------------------------------------------
struct StressMoments {
    double z;
    double I3, m3_10, m3_01;
    double M5[4][4];   // [a][b], a+b <= 3
    double M7[5][5];   // [a][b], a+b <= 4
};

// polynomial coefficients in u of (A + tx u)^a (B + ty u)^b, a+b <= 3
template <int a, int b>
__device__ __forceinline__ void edge_poly(double A, double B, double tx, double ty, double c[4]) {
    double pa[4] = {1.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int i = 0; i < a; i++) {
        double q[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int k = 0; k < 3; k++) {
            q[k] += pa[k] * A;
            q[k + 1] += pa[k] * tx;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) pa[k] = q[k];
    }
#pragma unroll
    for (int i = 0; i < b; i++) {
        double q[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int k = 0; k < 3; k++) {
            q[k] += pa[k] * B;
            q[k + 1] += pa[k] * ty;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) pa[k] = q[k];
    }
#pragma unroll
    for (int k = 0; k < 4; k++) c[k] = pa[k];
}

template <int a, int b>
__device__ __forceinline__ double edge_int(double A, double B, double tx, double ty,
                                           double D0, double D1, double D2, double D3) {
    double c[4];
    edge_poly<a, b>(A, B, tx, ty, c);
    double r = c[0] * D0;
    if (a + b >= 1) r += c[1] * D1;
    if (a + b >= 2) r += c[2] * D2;
    if (a + b >= 3) r += c[3] * D3;
    return r;
}

template <bool NEED7>
__device__ __forceinline__ void stress_moments(const SrcP0& s, const PairP0& p, StressMoments& M) {
    double BN1m1 = 0, BN2m1 = 0, BD003 = 0, BD005 = 0;
    // m = 3 edge sums (a+b <= 2): bn1 for 00,10,01,20,11,02 ; bn2 for 00,01,02
    double b3_1_00 = 0, b3_1_10 = 0, b3_1_01 = 0, b3_1_20 = 0, b3_1_11 = 0, b3_1_02 = 0;
    double b3_2_00 = 0, b3_2_01 = 0, b3_2_02 = 0;
    // m = 5 edge sums (a+b <= 3)
    double b5_1_00 = 0, b5_1_10 = 0, b5_1_01 = 0, b5_1_20 = 0, b5_1_11 = 0, b5_1_02 = 0,
           b5_1_30 = 0, b5_1_21 = 0, b5_1_12 = 0, b5_1_03 = 0;
    double b5_2_00 = 0, b5_2_01 = 0, b5_2_02 = 0, b5_2_03 = 0;
    EdgeP0 G[3];
    edges_setup(s, p, G);
#pragma unroll
    for (int e = 0; e < 3; e++) {
        if (!s.edge_ok[e]) continue;
        const EdgeP0& g = G[e];
        const double A = g.dp * g.nx, B = g.dp * g.ny;
        BN1m1 += g.nx * g.dJ1; BN2m1 += g.ny * g.dJ1;
        double v;
        v = g.dJ3;                                                            // (0,0)
        b3_1_00 += g.nx * v; b3_2_00 += g.ny * v; BD003 += g.dp * v;
        v = edge_int<1, 0>(A, B, g.tx, g.ty, g.dJ3, g.dK3, g.dL3, 0.0); b3_1_10 += g.nx * v;
        v = edge_int<0, 1>(A, B, g.tx, g.ty, g.dJ3, g.dK3, g.dL3, 0.0);
        b3_1_01 += g.nx * v; b3_2_01 += g.ny * v;
        v = edge_int<2, 0>(A, B, g.tx, g.ty, g.dJ3, g.dK3, g.dL3, 0.0); b3_1_20 += g.nx * v;
        v = edge_int<1, 1>(A, B, g.tx, g.ty, g.dJ3, g.dK3, g.dL3, 0.0); b3_1_11 += g.nx * v;
        v = edge_int<0, 2>(A, B, g.tx, g.ty, g.dJ3, g.dK3, g.dL3, 0.0);
        b3_1_02 += g.nx * v; b3_2_02 += g.ny * v;
        if (NEED7) {
            const int a = e, b = (e + 1) % 3;
            const double ua = g.ua, ub = g.ub;
            // J5 = u (3 rho^2 + 2 u^2) / (3 rho^4 R^3), K5 = -1 / (3 R^3)
            double dJ5 = 0.0;
            if (g.rho2 >= 1e-60) {
                const double ir2 = g.ir2;
                const double ia3 = p.iR[a] * p.iR[a] * p.iR[a];
                const double ib3 = p.iR[b] * p.iR[b] * p.iR[b];
                dJ5 = (ub * (3.0 * g.rho2 + 2.0 * ub * ub) * ib3 -
                       ua * (3.0 * g.rho2 + 2.0 * ua * ua) * ia3) * (ir2 * ir2 * (1.0 / 3.0));
            }
            const double dK5 = (p.iR[a] * p.iR[a] * p.iR[a] - p.iR[b] * p.iR[b] * p.iR[b]) * (1.0 / 3.0);
            const double dL5 = g.dJ3 - g.rho2 * dJ5;
            const double dM5 = g.dK3 - g.rho2 * dK5;
            v = dJ5;
            b5_1_00 += g.nx * v; b5_2_00 += g.ny * v; BD005 += g.dp * v;
            v = edge_int<1, 0>(A, B, g.tx, g.ty, dJ5, dK5, dL5, dM5); b5_1_10 += g.nx * v;
            v = edge_int<0, 1>(A, B, g.tx, g.ty, dJ5, dK5, dL5, dM5);
            b5_1_01 += g.nx * v; b5_2_01 += g.ny * v;
            v = edge_int<2, 0>(A, B, g.tx, g.ty, dJ5, dK5, dL5, dM5); b5_1_20 += g.nx * v;
            v = edge_int<1, 1>(A, B, g.tx, g.ty, dJ5, dK5, dL5, dM5); b5_1_11 += g.nx * v;
            v = edge_int<0, 2>(A, B, g.tx, g.ty, dJ5, dK5, dL5, dM5);
            b5_1_02 += g.nx * v; b5_2_02 += g.ny * v;
            v = edge_int<3, 0>(A, B, g.tx, g.ty, dJ5, dK5, dL5, dM5); b5_1_30 += g.nx * v;
            v = edge_int<2, 1>(A, B, g.tx, g.ty, dJ5, dK5, dL5, dM5); b5_1_21 += g.nx * v;
            v = edge_int<1, 2>(A, B, g.tx, g.ty, dJ5, dK5, dL5, dM5); b5_1_12 += g.nx * v;
            v = edge_int<0, 3>(A, B, g.tx, g.ty, dJ5, dK5, dL5, dM5);
            b5_1_03 += g.nx * v; b5_2_03 += g.ny * v;
        }
    }
    const double I3 = p.I3, h2 = p.h2;
    const double third = 1.0 / 3.0, fifth = 0.2;
    const double I5 = (h2 > 1e-60) ? (BD003 + I3) * p.ih2 * third : 0.0;
    M.z = p.z;
    M.I3 = I3;
    M.m3_10 = -BN1m1;
    M.m3_01 = -BN2m1;
    M.M5[0][0] = I5;
    M.M5[1][0] = -b3_1_00 * third;
    M.M5[0][1] = -b3_2_00 * third;
    M.M5[2][0] = (I3 - b3_1_10) * third;
    M.M5[1][1] = -b3_1_01 * third;
    M.M5[0][2] = (I3 - b3_2_01) * third;
    M.M5[3][0] = (2.0 * M.m3_10 - b3_1_20) * third;
    M.M5[2][1] = (M.m3_01 - b3_1_11) * third;
    M.M5[1][2] = -b3_1_02 * third;
    M.M5[0][3] = (2.0 * M.m3_01 - b3_2_02) * third;
    if (NEED7) {
        const double I7 = (h2 > 1e-60) ? (BD005 + 3.0 * I5) * p.ih2 * fifth : 0.0;
        M.M7[0][0] = I7;
        M.M7[1][0] = -b5_1_00 * fifth;
        M.M7[0][1] = -b5_2_00 * fifth;
        M.M7[2][0] = (I5 - b5_1_10) * fifth;
        M.M7[1][1] = -b5_1_01 * fifth;
        M.M7[0][2] = (I5 - b5_2_01) * fifth;
        M.M7[3][0] = (2.0 * M.M5[1][0] - b5_1_20) * fifth;
        M.M7[2][1] = (M.M5[0][1] - b5_1_11) * fifth;
        M.M7[1][2] = -b5_1_02 * fifth;
        M.M7[0][3] = (2.0 * M.M5[0][1] - b5_2_02) * fifth;
        M.M7[4][0] = (3.0 * M.M5[2][0] - b5_1_30) * fifth;
        M.M7[3][1] = (2.0 * M.M5[1][1] - b5_1_21) * fifth;
        M.M7[2][2] = (M.M5[0][2] - b5_1_12) * fifth;
        M.M7[1][3] = -b5_1_03 * fifth;
        M.M7[0][4] = (3.0 * M.M5[0][2] - b5_2_03) * fifth;
    }
}

// Local-frame moment tensors of d = (-xi1, -xi2, z): component c counts
// toward a (c = 0), b (c = 1) or the z power (c = 2).
template <int N>
__device__ __forceinline__ double sgnz(double z) {
    double r = 1.0;
#pragma unroll
    for (int i = 0; i < N; i++) r *= z;
    return r;
}

__device__ __forceinline__ void cnt2(int i, int j, int& a, int& b) {
    a = (i == 0) + (j == 0);
    b = (i == 1) + (j == 1);
}

// Rotation of a symmetric local tensor to the global frame.
__device__ __forceinline__ void rotate_sym(const SrcP0& s, const double L[3][3], double G[3][3]) {
    double Y[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int j = 0; j < 3; j++) Y[a][j] = L[a][0] * s.ex[j] + L[a][1] * s.ey[j] + L[a][2] * s.nh[j];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
            double w = s.ex[i] * Y[0][j] + s.ey[i] * Y[1][j] + s.nh[i] * Y[2][j];
            G[i][j] = w;
            G[j][i] = w;
        }
}

__device__ __forceinline__ void to_local(const SrcP0& s, const double* v, double l[3]) {
    l[0] = v[0] * s.ex[0] + v[1] * s.ex[1] + v[2] * s.ex[2];
    l[1] = v[0] * s.ey[0] + v[1] * s.ey[1] + v[2] * s.ey[2];
    l[2] = v[0] * s.nh[0] + v[1] * s.nh[1] + v[2] * s.nh[2];
}

// Local moment value for index counts (a of xi1, b of xi2, c of z) with sign
// (-1)^(a+b) and z^c.
#define MBEM_T2L(M, a, b, c, z) (((((a) + (b)) & 1) ? -1.0 : 1.0) * sgnz<(c)>(z) * (M)[(a)][(b)])

// Slip -> total stress contracted with a density (local frame in, local
// frame symmetric out): sigma_l[m][n] = H[m,n,k] s_k for the source frame
// (tri_kernels.py:900-964, contracted analytically).
__device__ __forceinline__ void dd_stress_local(const StressMoments& M, const double nl[3],
                                                const double sl[3], double mu, double lam,
                                                double C1, double c34, double cblob,
                                                double out[3][3]) {
    const double z = M.z;
    const double I3 = M.I3, I5 = M.M5[0][0];
    // T2_5, T2_7 local
    double T5[3][3], T7[3][3];
    T5[0][0] = MBEM_T2L(M.M5, 2, 0, 0, z); T5[0][1] = MBEM_T2L(M.M5, 1, 1, 0, z);
    T5[1][1] = MBEM_T2L(M.M5, 0, 2, 0, z); T5[0][2] = MBEM_T2L(M.M5, 1, 0, 1, z);
    T5[1][2] = MBEM_T2L(M.M5, 0, 1, 1, z); T5[2][2] = MBEM_T2L(M.M5, 0, 0, 2, z);
    T7[0][0] = MBEM_T2L(M.M7, 2, 0, 0, z); T7[0][1] = MBEM_T2L(M.M7, 1, 1, 0, z);
    T7[1][1] = MBEM_T2L(M.M7, 0, 2, 0, z); T7[0][2] = MBEM_T2L(M.M7, 1, 0, 1, z);
    T7[1][2] = MBEM_T2L(M.M7, 0, 1, 1, z); T7[2][2] = MBEM_T2L(M.M7, 0, 0, 2, z);
    T5[1][0] = T5[0][1]; T5[2][0] = T5[0][2]; T5[2][1] = T5[1][2];
    T7[1][0] = T7[0][1]; T7[2][0] = T7[0][2]; T7[2][1] = T7[1][2];
    // T4_7 distinct values by (a, b) counts, c = 4 - a - b
    double T4v[5][5];
#pragma unroll
    for (int a = 0; a <= 4; a++)
#pragma unroll
        for (int b = 0; a + b <= 4; b++) {
            const int c = 4 - a - b;
            double zc = 1.0;
            for (int i = 0; i < c; i++) zc *= z;
            T4v[a][b] = (((a + b) & 1) ? -1.0 : 1.0) * zc * M.M7[a][b];
        }
    const double ns = nl[0] * sl[0] + nl[1] * sl[1] + nl[2] * sl[2];
    double u[3], w[3], u7[3], w7[3];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        u[r] = T5[r][0] * nl[0] + T5[r][1] * nl[1] + T5[r][2] * nl[2];
        w[r] = T5[r][0] * sl[0] + T5[r][1] * sl[1] + T5[r][2] * sl[2];
        u7[r] = T7[r][0] * nl[0] + T7[r][1] * nl[1] + T7[r][2] * nl[2];
        w7[r] = T7[r][0] * sl[0] + T7[r][1] * sl[1] + T7[r][2] * sl[2];
    }
    const double su = sl[0] * u[0] + sl[1] * u[1] + sl[2] * u[2];
    const double trT5 = T5[0][0] + T5[1][1] + T5[2][2];
    // symmetric products S_pq = sl_p n_q + n_p sl_q
    double S[3][3];
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
        for (int q = 0; q < 3; q++) S[p][q] = sl[p] * nl[q] + nl[p] * sl[q];
    double Bs[3][3];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int t = 0; t < 3; t++) {
            // T4 contractions: sum_pq T4[r,t,p,q] S_pq / 2 * 2 (= Q4(sl,n)+Q4(n,sl))
            double q4 = 0.0, t4c = 0.0;
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    const int a = (r == 0) + (t == 0) + (p == 0) + (q == 0);
                    const int b = (r == 1) + (t == 1) + (p == 1) + (q == 1);
                    const double tv = T4v[a][b];
                    q4 += tv * S[p][q];
                    if (p == q) t4c += tv;
                }
            const double drt = (r == t) ? 1.0 : 0.0;
            const double X = (4.0 - c34) * I3 * drt + (3.0 * c34 - 18.0) * T5[r][t] -
                             3.0 * trT5 * drt + 15.0 * t4c + cblob * (15.0 * T7[r][t] - 3.0 * I5 * drt);
            const double Ysum = I3 * (1.0 - c34) * S[r][t] + 2.0 * drt * ns * I3 +
                                3.0 * (c34 - 1.0) * (sl[r] * u[t] + nl[r] * w[t]) -
                                6.0 * (sl[t] * u[r] + nl[t] * w[r]) - 6.0 * drt * su -
                                6.0 * ns * T5[r][t] + 15.0 * q4 +
                                cblob * (-3.0 * I5 * S[r][t] + 15.0 * (sl[r] * u7[t] + nl[r] * w7[t]));
            Bs[r][t] = C1 * (lam * ns * X + mu * Ysum);
        }
    const double trB = Bs[0][0] + Bs[1][1] + Bs[2][2];
#pragma unroll
    for (int m = 0; m < 3; m++)
#pragma unroll
        for (int n = m; n < 3; n++) {
            const double v = -((m == n ? lam * trB : 0.0) + mu * (Bs[m][n] + Bs[n][m]));
            out[m][n] = v;
            out[n][m] = v;
        }
}

// Force -> stress contracted with a force density, local frame
// (tri_kernels.py:857-897 contracted analytically).
__device__ __forceinline__ void kelvin_stress_local(const StressMoments& M, const double fl[3],
                                                    double mu, double lam, double C1, double c34,
                                                    double cbdg, double out[3][3]) {
    const double z = M.z;
    const double V3[3] = {-M.m3_10, -M.m3_01, z * M.I3};
    const double V5[3] = {-M.M5[1][0], -M.M5[0][1], z * M.M5[0][0]};
    // T3 local from M5: T[a][b][c] by counts
    double T3v[4][4];
#pragma unroll
    for (int a = 0; a <= 3; a++)
#pragma unroll
        for (int b = 0; a + b <= 3; b++) {
            const int c = 3 - a - b;
            double zc = 1.0;
            for (int i = 0; i < c; i++) zc *= z;
            T3v[a][b] = (((a + b) & 1) ? -1.0 : 1.0) * zc * M.M5[a][b];
        }
    double Tf[3][3];   // (T3 f)_ij
    double tvec[3];    // t_k = sum_i T3[i,k,i]
#pragma unroll
    for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int j = 0; j < 3; j++) {
            double acc = 0.0;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const int a = (i == 0) + (j == 0) + (k == 0);
                const int b = (i == 1) + (j == 1) + (k == 1);
                acc += T3v[a][b] * fl[k];
            }
            Tf[i][j] = acc;
        }
        double acc = 0.0;
#pragma unroll
        for (int m = 0; m < 3; m++) {
            const int a = 2 * (m == 0) + (i == 0);
            const int b = 2 * (m == 1) + (i == 1);
            acc += T3v[a][b];
        }
        tvec[i] = acc;
    }
    const double fV3 = fl[0] * V3[0] + fl[1] * V3[1] + fl[2] * V3[2];
    const double fV5 = fl[0] * V5[0] + fl[1] * V5[1] + fl[2] * V5[2];
    const double ft = fl[0] * tvec[0] + fl[1] * tvec[1] + fl[2] * tvec[2];
    const double tau = C1 * ((4.0 - c34) * fV3 - 3.0 * ft - cbdg * fV5);
    double Gf[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            Gf[i][j] = C1 * (-c34 * fl[i] * V3[j] + (i == j ? fV3 : 0.0) + fl[j] * V3[i] -
                             3.0 * Tf[i][j] - cbdg * fl[i] * V5[j]);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
            const double v = (i == j ? lam * tau : 0.0) + mu * (Gf[i][j] + Gf[j][i]);
            out[i][j] = v;
            out[j][i] = v;
        }
}

}  // namespace mbem
