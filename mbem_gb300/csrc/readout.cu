// Mixed-precision stress readout of a nodal (P0/P1/P2) slip density at many
// points: the elastic stress (DD minus the exact eigenstress,
// evaluate.py:383-407 with subtract_anelastic) of every source at every
// observer, FP32 quadrature for the far pairs and the FP64 nodal machinery
// (nodal.cu) for the near ones.
//
// Far pairs: sum_q w_q H(x - y_q) s(y_q), s(y_q) = sum_k N_k(y_q) d_k, H the
// mollified point kernel of the DD stress (tri_kernels.py:901-964 with every
// moment replaced by its integrand) minus the eigenstress integrand
// (15 eps^4 / 8 pi) / R^7 C:sym(s n) (tri_kernels.py:1206-1214). Collapsed
// Gauss rules of 3 x 3, 5 x 5 and 8 x 8 points for D / L above 12, above 6
// and below (D = sqrt(|x - c|^2 + eps^2), L the longest edge). The offset
// x - c is formed in double-float and each point adds its FP32 offset from
// the centroid, so FP32 sees lengths of the size of the pair, not of the
// coordinates; a source's quadrature sum is FP32, the sum over sources FP64.
// Near pairs: D below near_factor * max(eps, L); listed per observer in
// source order (a count pass, a scan, a fill), evaluated in FP64, and added
// per observer in list order. Every sum runs in a fixed order.
#include <math.h>

#include <mutex>

#include "common.cuh"
#include "point_stress.cuh"

namespace mbem {

constexpr int RO_Q0 = 9, RO_Q1 = 25, RO_Q2 = 64;
constexpr int RO_Q = RO_Q0 + RO_Q1 + RO_Q2;
constexpr int RO_HDR = 16;                    // c_hi[3], c_lo[3], n[3], eps, L, rnear2, pad
constexpr int RO_REC = RO_HDR + 7 * RO_Q;     // + per point: offset[3], weight, slip[3]
constexpr int RO_REC_PAD = (RO_REC + 3) / 4 * 4;
constexpr int RO_THREADS = 128;
constexpr int RO_TILE = 16;                   // sources staged in shared memory at a time

__constant__ double c_ro_lam[RO_Q][3];
__constant__ double c_ro_w[RO_Q];

static std::mutex g_ro_mutex;
static bool g_ro_ready[64] = {false};

static void gauss_legendre_ro(int n, double* x, double* w) {
    for (int i = 0; i < n; i++) {
        double z = cos(MBEM_PI * (i + 0.75) / (n + 0.5));
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; k++) {
                const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            const double dz = p1 / (n * (z * p1 - p0) / (z * z - 1.0));
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

static int ro_rules() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return set_error(MBEM_ERR_CUDA, "no current CUDA device for the readout rules");
    std::lock_guard<std::mutex> lock(g_ro_mutex);
    if (g_ro_ready[dev]) return MBEM_OK;
    static double lam[RO_Q][3], w[RO_Q];
    int q = 0;
    for (int n : {3, 5, 8}) {
        double g[8], gw[8];
        gauss_legendre_ro(n, g, gw);
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                const double gi = 0.5 * (g[i] + 1.0), gj = 0.5 * (g[j] + 1.0);
                lam[q][0] = 1.0 - gi - gj * (1.0 - gi);
                lam[q][1] = gi;
                lam[q][2] = gj * (1.0 - gi);
                w[q] = (0.5 * gw[i]) * (0.5 * gw[j]) * (1.0 - gi);
                q++;
            }
    }
    cudaError_t e = cudaMemcpyToSymbol(c_ro_lam, lam, sizeof(lam));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ro_w, w, sizeof(w));
    if (e != cudaSuccess) return set_error(MBEM_ERR_CUDA, "readout rules: %s", cudaGetErrorString(e));
    g_ro_ready[dev] = true;
    return MBEM_OK;
}

struct Lattice {
    int order, K;
    int a[6][3];
};

// per-source record: centroid (double-float), normal, eps, L, near radius^2,
// and the three rules' points (offset from the centroid, weight x 2 area,
// interpolated slip)
__global__ void readout_prep_kernel(const double* __restrict__ tv, const double* __restrict__ normals,
                                    const double* __restrict__ eps, const double* __restrict__ density,
                                    int64_t n_src, Lattice lat, double near_factor, float* __restrict__ rec) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_src) return;
    const double* v = tv + 9 * s;
    float* r = rec + s * RO_REC_PAD;
    double c[3];
    for (int k = 0; k < 3; k++) {
        c[k] = ((v[k] + v[3 + k]) + v[6 + k]) / 3.0;
        const float hi = (float)c[k];
        r[k] = hi;
        r[3 + k] = (float)(c[k] - (double)hi);
        r[6 + k] = (float)normals[3 * s + k];
    }
    double L = 0.0;
    for (int e = 0; e < 3; e++) {
        const int e2 = (e + 1) % 3;
        const double dx = v[3 * e2] - v[3 * e], dy = v[3 * e2 + 1] - v[3 * e + 1], dz = v[3 * e2 + 2] - v[3 * e + 2];
        L = fmax(L, sqrt(dx * dx + dy * dy + dz * dz));
    }
    const double e1x = v[3] - v[0], e1y = v[4] - v[1], e1z = v[5] - v[2];
    const double e2x = v[6] - v[0], e2y = v[7] - v[1], e2z = v[8] - v[2];
    const double cx = e1y * e2z - e1z * e2y, cy = e1z * e2x - e1x * e2z, cz = e1x * e2y - e1y * e2x;
    const double area2 = sqrt(cx * cx + cy * cy + cz * cz);
    const double ep = eps[s];
    const double rn = near_factor * fmax(ep, L);
    r[9] = (float)ep;
    r[10] = (float)L;
    r[11] = (float)(rn * rn);
    for (int k = 12; k < RO_HDR; k++) r[k] = 0.0f;
    for (int q = 0; q < RO_Q; q++) {
        const double l0 = c_ro_lam[q][0], l1 = c_ro_lam[q][1], l2 = c_ro_lam[q][2];
        const double lam3[3] = {l0, l1, l2};
        float* pq = r + RO_HDR + 7 * q;
        for (int k = 0; k < 3; k++) pq[k] = (float)(((l0 * v[k] + l1 * v[3 + k]) + l2 * v[6 + k]) - c[k]);
        pq[3] = (float)(c_ro_w[q] * area2);
        double sl[3] = {0.0, 0.0, 0.0};
        for (int kk = 0; kk < lat.K; kk++) {
            double N = 1.0;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < lat.a[kk][i]; j++) N *= (lat.order * lam3[i] - j) / (j + 1);
            const double* d = density + 3 * (lat.K * s + kk);
            sl[0] += N * d[0];
            sl[1] += N * d[1];
            sl[2] += N * d[2];
        }
        pq[4] = (float)sl[0];
        pq[5] = (float)sl[1];
        pq[6] = (float)sl[2];
    }
}

// |x - c| in double-float, as FP32 components
__device__ __forceinline__ void df_offset(const double* x, const float* r, float d[3]) {
    for (int k = 0; k < 3; k++) {
        const float xh = (float)x[k];
        const float xl = (float)(x[k] - (double)xh);
        d[k] = __fadd_rn(__fsub_rn(xh, r[k]), __fsub_rn(xl, r[3 + k]));
    }
}

// the one near test (count and fill must agree exactly: no contraction)
__device__ __forceinline__ float pair_d2(const float d[3], float eps) {
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2])),
                     __fmul_rn(eps, eps));
}

__global__ void __launch_bounds__(RO_THREADS)
readout_count_kernel(const double* __restrict__ x, int64_t n_obs, const float* __restrict__ rec, int64_t n_src,
                     int64_t* __restrict__ counts) {
    const int64_t f = (int64_t)blockIdx.x * RO_THREADS + threadIdx.x;
    if (f >= n_obs) return;
    int64_t cnt = 0;
    for (int64_t s = 0; s < n_src; s++) {
        const float* r = rec + s * RO_REC_PAD;
        float d[3];
        df_offset(x + 3 * f, r, d);
        cnt += pair_d2(d, r[9]) <= r[11];
    }
    counts[f] = cnt;
}

__global__ void ro_scan_kernel(const int64_t* __restrict__ counts, int64_t n, int64_t* __restrict__ rowptr) {
    __shared__ int64_t part[1024];
    const int t = threadIdx.x;
    const int64_t chunk = (n + 1023) / 1024;
    const int64_t b0 = t * chunk, b1 = lmin(n, b0 + chunk);
    int64_t s = 0;
    for (int64_t i = b0; i < b1; i++) s += counts[i];
    part[t] = s;
    __syncthreads();
    if (t == 0) {
        int64_t run = 0;
        for (int i = 0; i < 1024; i++) {
            const int64_t v = part[i];
            part[i] = run;
            run += v;
        }
        rowptr[n] = run;
    }
    __syncthreads();
    int64_t run = part[t];
    for (int64_t i = b0; i < b1; i++) {
        rowptr[i] = run;
        run += counts[i];
    }
}

// far pairs by quadrature, near pairs listed; a thread per observer, sources
// staged RO_TILE at a time in shared memory; with EIG the eigenstress of the
// far pairs goes to eig_out as well
template <bool EIG>
__global__ void __launch_bounds__(RO_THREADS)
readout_far_kernel(const double* __restrict__ x, int64_t n_obs, const float* __restrict__ rec, int64_t n_src,
                   RoMat mat, const int64_t* __restrict__ rowptr, int64_t* __restrict__ pair_obs,
                   int32_t* __restrict__ pair_src, double alpha, int accumulate, double* __restrict__ out,
                   double* __restrict__ eig_out) {
    extern __shared__ __align__(16) float tile[];
    const int64_t f = (int64_t)blockIdx.x * RO_THREADS + threadIdx.x;
    const bool live = f < n_obs;
    double xo[3] = {0.0, 0.0, 0.0};
    if (live)
        for (int k = 0; k < 3; k++) xo[k] = x[3 * f + k];
    double acc[6] = {0, 0, 0, 0, 0, 0};
    double acc_e[6] = {0, 0, 0, 0, 0, 0};
    int64_t slot = live ? rowptr[f] : 0;
    const int64_t slot_end = live ? rowptr[f + 1] : 0;
    for (int64_t s0 = 0; s0 < n_src; s0 += RO_TILE) {
        const int ns = (int)lmin(RO_TILE, n_src - s0);
        __syncthreads();
        const float4* src4 = reinterpret_cast<const float4*>(rec + s0 * RO_REC_PAD);
        float4* dst4 = reinterpret_cast<float4*>(tile);
        for (int t = threadIdx.x; t < ns * RO_REC_PAD / 4; t += RO_THREADS) dst4[t] = src4[t];
        __syncthreads();
        if (!live) continue;
        for (int t = 0; t < ns; t++) {
            const float* r = tile + t * RO_REC_PAD;
            float dc[3];
            df_offset(xo, r, dc);
            const float eps2 = r[9] * r[9];
            const float D2 = pair_d2(dc, r[9]);
            if (D2 <= r[11]) {
                if (slot < slot_end) {
                    pair_obs[slot] = f;
                    pair_src[slot] = (int32_t)(s0 + t);
                }
                slot++;
                continue;
            }
            const float L2 = r[10] * r[10];
            int q0, q1;
            if (D2 > 144.0f * L2) { q0 = 0; q1 = RO_Q0; }
            else if (D2 > 36.0f * L2) { q0 = RO_Q0; q1 = RO_Q0 + RO_Q1; }
            else { q0 = RO_Q0 + RO_Q1; q1 = RO_Q; }
            const float nv[3] = {r[6], r[7], r[8]};
            float sym[6] = {0, 0, 0, 0, 0, 0};
            float sym_e[6] = {0, 0, 0, 0, 0, 0};
            for (int q = q0; q < q1; q++) {
                const float* pq = r + RO_HDR + 7 * q;
                const float d[3] = {dc[0] - pq[0], dc[1] - pq[1], dc[2] - pq[2]};
                const float u[3] = {pq[4], pq[5], pq[6]};
                point_stress<EIG>(d, u, nv, pq[3], eps2, mat, sym, sym_e);
            }
#pragma unroll
            for (int k = 0; k < 6; k++) acc[k] += (double)sym[k];
            if (EIG) {
#pragma unroll
                for (int k = 0; k < 6; k++) acc_e[k] += (double)sym_e[k];
            }
        }
    }
    if (!live) return;
    double* o = out + 9 * f;
    const double v9[9] = {acc[0], acc[3], acc[4], acc[3], acc[1], acc[5], acc[4], acc[5], acc[2]};
    for (int k = 0; k < 9; k++) o[k] = accumulate ? o[k] + alpha * v9[k] : alpha * v9[k];
    if (EIG) {
        double* oe = eig_out + 9 * f;
        const double e9[9] = {acc_e[0], acc_e[3], acc_e[4], acc_e[3], acc_e[1], acc_e[5], acc_e[4], acc_e[5], acc_e[2]};
        for (int k = 0; k < 9; k++) oe[k] = accumulate ? oe[k] + alpha * e9[k] : alpha * e9[k];
    }
}

// out[f] += alpha * sum of its near pairs' stresses, in list order
__global__ void readout_near_add_kernel(const int64_t* __restrict__ rowptr, int64_t n_obs,
                                        const double* __restrict__ pair_out, double alpha, double* __restrict__ out) {
    const int64_t f = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (f >= n_obs) return;
    double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t p = rowptr[f]; p < rowptr[f + 1]; p++)
        for (int k = 0; k < 9; k++) s[k] += pair_out[9 * p + k];
    for (int k = 0; k < 9; k++) out[9 * f + k] += alpha * s[k];
}

static Lattice lattice_of(int order) {
    Lattice L;
    memset(&L, 0, sizeof(L));
    L.order = order;
    L.K = (order + 1) * (order + 2) / 2;
    if (order == 0) return L;
    int k = 0;
    for (int v = 0; v < 3; v++) {
        L.a[k][v] = order;
        k++;
    }
    const int ij[3][2] = {{0, 1}, {1, 2}, {2, 0}};
    for (int e = 0; e < 3; e++)
        for (int s = 1; s < order; s++) {
            L.a[k][ij[e][0]] = order - s;
            L.a[k][ij[e][1]] = s;
            k++;
        }
    return L;
}

}  // namespace mbem

using namespace mbem;

extern "C" {

size_t mbem_readout_record_bytes(int64_t n_src) { return (size_t)n_src * RO_REC_PAD * sizeof(float); }

int mbem_readout_prepare(const double* x, int64_t n_obs, const double* tri_verts, const double* normals,
                         const double* eps, int64_t n_src, const double* density, int order, double near_factor,
                         float* records, int64_t* counts, int64_t* rowptr, int64_t* n_near, void* stream) {
    MBEM_REQUIRE(n_obs >= 0 && n_src >= 0 && order >= 0 && order <= 2 && near_factor > 0.0, MBEM_ERR_ARG,
                 "bad readout sizes");
    MBEM_REQUIRE((n_obs == 0 || (x && rowptr)) && (n_src == 0 || (tri_verts && normals && eps && density && records)) &&
                     n_near,
                 MBEM_ERR_ARG, "NULL readout arrays");
    MBEM_REQUIRE(n_src < INT32_MAX, MBEM_ERR_SIZE, "too many sources");
    int e = ro_rules();
    if (e) return e;
    cudaStream_t st = (cudaStream_t)stream;
    if (n_src > 0) {
        readout_prep_kernel<<<(unsigned)ceil_div(n_src, 128), 128, 0, st>>>(tri_verts, normals, eps, density, n_src,
                                                                            lattice_of(order), near_factor, records);
        if ((e = launch_status("readout_prep_kernel"))) return e;
    }
    if (n_obs == 0) {
        cudaMemsetAsync(rowptr, 0, sizeof(int64_t), st);
        *n_near = 0;
        return launch_status("readout memset", 0);
    }
    MBEM_REQUIRE(counts != nullptr, MBEM_ERR_ARG, "NULL counts");
    readout_count_kernel<<<(unsigned)ceil_div(n_obs, RO_THREADS), RO_THREADS, 0, st>>>(x, n_obs, records, n_src,
                                                                                       counts);
    if ((e = launch_status("readout_count_kernel"))) return e;
    ro_scan_kernel<<<1, 1024, 0, st>>>(counts, n_obs, rowptr);
    if ((e = launch_status("ro_scan_kernel"))) return e;
    cudaMemcpyAsync(n_near, rowptr + n_obs, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("readout sync", 0);
    return MBEM_OK;
}

int mbem_readout_evaluate(const double* x, int64_t n_obs, const double* tri_verts, const double* normals,
                          const double* eps, int64_t n_src, const double* density, double mu, double lam, int order,
                          const float* records, const int64_t* rowptr, int64_t n_near, int64_t* pair_obs,
                          int32_t* pair_src, double* pair_out, double alpha, int accumulate, double* out,
                          void* stream) {
    return mbem_readout_evaluate_parts(x, n_obs, tri_verts, normals, eps, n_src, density, mu, lam, order, records,
                                       rowptr, n_near, pair_obs, pair_src, pair_out, nullptr, alpha, accumulate, out,
                                       nullptr, stream);
}

int mbem_readout_evaluate_parts(const double* x, int64_t n_obs, const double* tri_verts, const double* normals,
                                const double* eps, int64_t n_src, const double* density, double mu, double lam,
                                int order, const float* records, const int64_t* rowptr, int64_t n_near,
                                int64_t* pair_obs, int32_t* pair_src, double* pair_out, double* pair_eig,
                                double alpha, int accumulate, double* out, double* eig_out, void* stream) {
    MBEM_REQUIRE(n_obs >= 0 && n_src >= 0 && n_near >= 0 && mu > 0.0 && lam + mu > 0.0, MBEM_ERR_ARG,
                 "bad readout arguments");
    MBEM_REQUIRE(n_obs == 0 || (x && rowptr && out), MBEM_ERR_ARG, "NULL readout arrays");
    MBEM_REQUIRE(n_near == 0 || (pair_obs && pair_src && pair_out), MBEM_ERR_ARG, "NULL near-pair arrays");
    MBEM_REQUIRE(!eig_out || n_near == 0 || pair_eig, MBEM_ERR_ARG, "the eigenstress needs its near-pair array");
    if (n_obs == 0) return MBEM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const RoMat m = make_romat(mu, lam);
    const size_t smem = (size_t)RO_TILE * RO_REC_PAD * sizeof(float);
    const unsigned grid = (unsigned)ceil_div(n_obs, RO_THREADS);
    if (eig_out) {
        cudaFuncSetAttribute(readout_far_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        readout_far_kernel<true><<<grid, RO_THREADS, smem, st>>>(x, n_obs, records, n_src, m, rowptr, pair_obs,
                                                                 pair_src, alpha, accumulate, out, eig_out);
    } else {
        cudaFuncSetAttribute(readout_far_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        readout_far_kernel<false><<<grid, RO_THREADS, smem, st>>>(x, n_obs, records, n_src, m, rowptr, pair_obs,
                                                                  pair_src, alpha, accumulate, out, nullptr);
    }
    int e = launch_status("readout_far_kernel");
    if (e) return e;
    if (n_near == 0) return MBEM_OK;
    if ((e = nodal_pairs_stress(x, tri_verts, normals, eps, density, mu, lam, order, pair_obs, pair_src, n_near,
                                pair_out, st, eig_out ? pair_eig : nullptr)))
        return e;
    readout_near_add_kernel<<<(unsigned)ceil_div(n_obs, 256), 256, 0, st>>>(rowptr, n_obs, pair_out, alpha, out);
    if ((e = launch_status("readout_near_add_kernel"))) return e;
    if (!eig_out) return MBEM_OK;
    readout_near_add_kernel<<<(unsigned)ceil_div(n_obs, 256), 256, 0, st>>>(rowptr, n_obs, pair_eig, alpha, eig_out);
    return launch_status("readout_near_add_kernel");
}

}  // extern "C"
