// Traction rows of the mixed operator (FAULT_TRACTION faults): the elastic
// traction (DD stress minus eigenstress, contracted with the field point's
// normal) of unit slips of order-0 source triangles, FP32 quadrature for the
// far pairs and the FP64 closed form (nodal.cu) for the near ones, written
// into an FP64 block so that the fault-row transformation applies to it as to
// the FP64 system's rows (tri_nodal.py:1176-1227, 1370-1404 traction_matrix
// with which = "slip"; basis.py:406-427).
//
// Far pair (f, s): T[i][k] = sum_q w_q 2A sigma(x_f - y_q; u = e_k, n_s)_ij n_f,j,
// sigma the mollified point integrand of point_stress.cuh; collapsed Gauss
// rules of 3 x 3, 5 x 5 and 8 x 8 points for D / L above 12, above 6 and below
// (D^2 = |x - c|^2 + eps^2, L the longest edge), the readout's choice; the
// offset x - c in double-float. The near rule is the mixed operator's
// (far_quad.cuh is_near), the same one the near list of the pairs uses.
#include <math.h>

#include "common.cuh"
#include "dfloat.cuh"
#include "far_quad.cuh"
#include "point_stress.cuh"

namespace mbem {
namespace {

constexpr int TM_THREADS = 128;
constexpr int TM_FIELD_TILE = 64;

struct TracArgs {
    const double* x;      // (n_pts, 3)
    const double* nf;     // (n_pts, 3)
    int64_t n_pts;
    const double* tv;
    const double* nrm;
    const double* eps;
    int64_t n_src;
    double near_factor;
    double alpha;
    double* out;
    int64_t ld;
};

// a thread per source, the field points of one tile (blockIdx.y) in turn
__global__ void __launch_bounds__(TM_THREADS) traction_far_kernel(TracArgs a, RoMat mat, QuadRules Q) {
    __shared__ F2 xs[TM_FIELD_TILE][3];
    __shared__ float ns_[TM_FIELD_TILE][3];
    const int64_t s = (int64_t)blockIdx.x * TM_THREADS + threadIdx.x;
    const bool active = s < a.n_src;
    const int64_t f0 = (int64_t)blockIdx.y * TM_FIELD_TILE;
    const int nf = (int)lmin(TM_FIELD_TILE, a.n_pts - f0);
    for (int t = threadIdx.x; t < 3 * nf; t += TM_THREADS) {
        xs[t / 3][t % 3] = split_d(a.x[3 * f0 + t]);
        ns_[t / 3][t % 3] = (float)a.nf[3 * f0 + t];
    }
    __syncthreads();
    if (!active) return;
    SrcFar src;
    far_setup(a.tv + 9 * s, a.nrm + 3 * s, a.eps[s], a.near_factor, src);
    if (!src.ok) return;
    const float eps2 = src.eps2;
    const float A2 = src.area2;
    for (int ff = 0; ff < nf; ff++) {
        float dc[3], D2;
        if (is_near(xs[ff], src, dc, D2)) continue;       // the FP64 pass adds this pair
        const float R2 = D2 + eps2;
        int nq = 8;
        if (R2 > 144.0f * src.L2) nq = 3;
        else if (R2 > 36.0f * src.L2) nq = 5;
        const int q0 = Q.off[nq], q1 = q0 + nq * nq;
        float sym[3][6];
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int t = 0; t < 6; t++) sym[k][t] = 0.0f;
        for (int q = q0; q < q1; q++) {
            const float qa = Q.a[q], qb = Q.b[q];
            const float d[3] = {dc[0] - (qa * src.e1[0] + qb * src.e2[0]), dc[1] - (qa * src.e1[1] + qb * src.e2[1]),
                                dc[2] - (qa * src.e1[2] + qb * src.e2[2])};
            const float w = Q.w[q] * A2;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const float u[3] = {k == 0 ? 1.0f : 0.0f, k == 1 ? 1.0f : 0.0f, k == 2 ? 1.0f : 0.0f};
                point_stress<false>(d, u, src.n, w, eps2, mat, sym[k], nullptr);
            }
        }
        const float* n = ns_[ff];
        double* o = a.out + 3 * (f0 + ff) * a.ld + 3 * s;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            // sym: xx, yy, zz, xy, xz, yz
            const float* m = sym[k];
            const float t0 = m[0] * n[0] + m[3] * n[1] + m[4] * n[2];
            const float t1 = m[3] * n[0] + m[1] * n[1] + m[5] * n[2];
            const float t2 = m[4] * n[0] + m[5] * n[1] + m[2] * n[2];
            o[k] += a.alpha * (double)t0;
            o[a.ld + k] += a.alpha * (double)t1;
            o[2 * a.ld + k] += a.alpha * (double)t2;
        }
    }
}

}  // namespace
}  // namespace mbem

using namespace mbem;

extern "C" int mbem_traction_matrix_mixed(const double* x_field, const double* n_field, int64_t n_pts,
                                          const double* tri_verts, const double* normals, const double* eps,
                                          int64_t n_src, double mu, double lam, double near_factor, double alpha,
                                          const int64_t* near_rowptr, const int64_t* near_cols, int64_t nnz,
                                          double* out, int64_t ld_out, void* stream) {
    MBEM_REQUIRE(n_pts >= 0 && n_src >= 0 && nnz >= 0 && ld_out >= 3 * n_src, MBEM_ERR_ARG, "bad traction shape");
    MBEM_REQUIRE(n_src == 0 || (tri_verts && normals && eps), MBEM_ERR_ARG, "NULL source arrays");
    MBEM_REQUIRE(n_pts == 0 || (x_field && n_field && out && near_rowptr), MBEM_ERR_ARG, "NULL field arrays");
    MBEM_REQUIRE(nnz == 0 || near_cols, MBEM_ERR_ARG, "NULL near-pair columns");
    MBEM_REQUIRE(mu > 0.0 && lam + mu > 0.0, MBEM_ERR_ARG, "material (mu=%g, lam=%g)", mu, lam);
    MBEM_REQUIRE(n_pts / TM_FIELD_TILE < 65535, MBEM_ERR_SIZE, "too many field points (%lld)", (long long)n_pts);
    if (n_pts == 0 || n_src == 0) return MBEM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    TracArgs a;
    a.x = x_field;
    a.nf = n_field;
    a.n_pts = n_pts;
    a.tv = tri_verts;
    a.nrm = normals;
    a.eps = eps;
    a.n_src = n_src;
    a.near_factor = near_factor;
    a.alpha = alpha;
    a.out = out;
    a.ld = ld_out;
    const dim3 grid((unsigned)ceil_div(n_src, TM_THREADS), (unsigned)ceil_div(n_pts, TM_FIELD_TILE));
    traction_far_kernel<<<grid, TM_THREADS, 0, st>>>(a, make_romat(mu, lam), rules());
    int e = launch_status("traction_far_kernel");
    if (e) return e;
    return traction_pairs(x_field, n_field, n_pts, tri_verts, normals, eps, n_src, mu, lam, 0, alpha, near_rowptr,
                          near_cols, nnz, out, ld_out, st);
}
