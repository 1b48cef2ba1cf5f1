// The elastic stress (DD stress minus the exact eigenstress) of a mollified
// point dislocation in FP32: the integrand of the far-field quadratures of the
// mixed readout (readout.cu) and of the mixed operator's traction rows
// (traction_mixed.cu). tri_kernels.py:901-964 with every moment replaced by its
// integrand, minus (15 eps^4 / 8 pi) / R^7 C:sym(s n) (tri_kernels.py:1206-1214).
#pragma once

#include "common.cuh"

namespace mbem {

struct RoMat {
    float lam, mu, C1, c34, cblob_per_eps2, phi_per_eps4;
};

// elastic stress of one quadrature point (d = x - y, slip u, normal v),
// weight folded in; sym holds xx, yy, zz, xy, xz, yz; with EIG the
// eigenstress integrand goes to sym_e as well
template <bool EIG>
__device__ __forceinline__ void point_stress(const float d[3], const float u[3], const float v[3], float w,
                                             float eps2, const RoMat& m, float sym[6], float sym_e[6]) {
    const float dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const float ir = rsqrtf(dd + eps2);
    const float ir2 = ir * ir;
    const float a = ir * ir2, b = a * ir2, c = b * ir2;       // 1/R^3, 1/R^5, 1/R^7
    const float du = d[0] * u[0] + d[1] * u[1] + d[2] * u[2];
    const float dv = d[0] * v[0] + d[1] * v[1] + d[2] * v[2];
    const float uv = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
    const float cblob = m.cblob_per_eps2 * eps2;
    // X = C1 (delta X0 + X1 d d); S = C1 (A1 sym(u, v) + delta S0 + G w d^T - 6 b d w^T + E d d^T), w = dv u + du v
    const float X0 = (4.0f - m.c34) * a - 3.0f * (dd + cblob) * b;
    const float X1 = (3.0f * m.c34 - 18.0f) * b + 15.0f * (dd + cblob) * c;
    const float A1 = (1.0f - m.c34) * a - 3.0f * cblob * b;
    const float S0 = 2.0f * uv * a - 6.0f * du * dv * b;
    const float G = (3.0f * m.c34 - 3.0f) * b + 15.0f * cblob * c;
    const float E = 30.0f * du * dv * c - 6.0f * uv * b;
    const float wv[3] = {dv * u[0] + du * v[0], dv * u[1] + du * v[1], dv * u[2] + du * v[2]};
    const float trX = 3.0f * X0 + X1 * dd;
    const float trS = 2.0f * A1 * uv + 3.0f * S0 + (G - 6.0f * b) * (2.0f * du * dv) + E * dd;
    const float lam = m.lam, mu = m.mu;
    // tr(Bs) = lam uv trX + mu trS; Bs + Bs^T = 2 lam uv X + mu (S + S^T); all times C1
    const float trB = m.C1 * (lam * uv * trX + mu * trS);
    const float phi = m.phi_per_eps4 * eps2 * eps2 * c;
    const int ia[6] = {0, 1, 2, 0, 0, 1}, ib[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int t = 0; t < 6; t++) {
        const int i = ia[t], j = ib[t];
        const float delta = (i == j) ? 1.0f : 0.0f;
        const float symuv = u[i] * v[j] + v[i] * u[j];
        const float X = delta * X0 + X1 * d[i] * d[j];
        const float SS = 2.0f * A1 * symuv + 2.0f * delta * S0 + (G - 6.0f * b) * (wv[i] * d[j] + d[i] * wv[j]) +
                         2.0f * E * d[i] * d[j];
        const float BB = m.C1 * (2.0f * lam * uv * X + mu * SS);
        const float sig = -(lam * delta * trB + mu * BB);
        const float eig = phi * (lam * delta * uv + mu * symuv);
        sym[t] = fmaf(w, sig - eig, sym[t]);
        if (EIG) sym_e[t] = fmaf(w, eig, sym_e[t]);
    }
}


// the material constants of point_stress from (mu, lam)
inline RoMat make_romat(double mu, double lam) {
    const double nu = lam / (2.0 * (lam + mu));
    RoMat m;
    m.lam = (float)lam;
    m.mu = (float)mu;
    m.C1 = (float)(1.0 / (16.0 * MBEM_PI * mu * (1.0 - nu)));
    m.c34 = (float)(3.0 - 4.0 * nu);
    m.cblob_per_eps2 = (float)(2.0 * (1.0 - nu));
    m.phi_per_eps4 = (float)(15.0 / (8.0 * MBEM_PI));
    return m;
}

}  // namespace mbem
