// P0 kernel matrices and matrix-free contractions, FP64 (sm_103a).
//
// Matrices: one thread per source triangle, FIELD_TILE observers per block
// staged in shared memory (broadcast reads), the source frame kept in
// registers across the tile; each warp writes 32 consecutive 3-column
// blocks of a row, i.e. 768 contiguous bytes per output row.
// Contractions: one thread per observer, source tiles prepared once per
// block in shared memory (frame and constants) and read as broadcasts.
#include "p0_pair.cuh"

namespace mbem {

constexpr int MAT_THREADS = 128;
constexpr int FIELD_TILE = 16;
constexpr int CON_THREADS = 128;
constexpr int SRC_TILE = 64;

enum MatKind { MAT_T_DIRECT = 0, MAT_U_DIRECT = 1, MAT_T_BASIS = 2, MAT_U_BASIS = 3 };

struct MatArgs {
    const double* x_field;
    int64_t n_field;
    const double* tri_verts;
    const double* normals;
    const double* eps;
    int64_t n_src;
    double c[6];
    double alpha;
    int accumulate;
    double* out;
    int64_t ld;          // leading dimension (row stride) of `out`
    int64_t plane;       // stride between basis planes (basis kinds)
};

template <int KIND>
__global__ void __launch_bounds__(MAT_THREADS)
p0_matrix_kernel(MatArgs a) {
    __shared__ double xs[FIELD_TILE][3];
    const int64_t s = (int64_t)blockIdx.x * MAT_THREADS + threadIdx.x;
    const bool active = s < a.n_src;
    SrcP0 src;
    double nrm[3] = {0.0, 0.0, 0.0};
    if (active) {
        src_setup(a.tri_verts + 9 * s, a.eps[s], src);
        if (KIND == MAT_T_DIRECT || KIND == MAT_T_BASIS) {
            nrm[0] = a.normals[3 * s]; nrm[1] = a.normals[3 * s + 1]; nrm[2] = a.normals[3 * s + 2];
        }
    }
    for (int64_t f0 = (int64_t)blockIdx.y * FIELD_TILE; f0 < a.n_field;
         f0 += (int64_t)gridDim.y * FIELD_TILE) {
        __syncthreads();
        for (int t = threadIdx.x; t < FIELD_TILE * 3; t += MAT_THREADS) {
            int64_t f = f0 + t / 3;
            xs[t / 3][t % 3] = (f < a.n_field) ? a.x_field[3 * f0 + t] : 0.0;
        }
        __syncthreads();
        if (!active) continue;
        const int nf = (int)lmin(FIELD_TILE, a.n_field - f0);
        for (int ff = 0; ff < nf; ff++) {
            const int64_t f = f0 + ff;
            if (KIND == MAT_T_DIRECT || KIND == MAT_U_DIRECT) {
                double blk[3][3];
                if (src.ok) {
                    PairP0 p;
                    pair_setup(src, xs[ff][0], xs[ff][1], xs[ff][2], p);
                    if (KIND == MAT_T_DIRECT) {
                        TMoments m;
                        t_moments(src, nrm, p, m);
                        t_block(m, nrm, a.c, src.eps2, blk);
                    } else {
                        UMoments m;
                        u_moments(src, p, m);
#pragma unroll
                        for (int i = 0; i < 3; i++)
#pragma unroll
                            for (int j = 0; j < 3; j++)
                                blk[i][j] = a.c[2] * m.T2[i][j] +
                                            (i == j ? a.c[0] * m.I1 + a.c[1] * src.eps2 * m.I3 : 0.0);
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 3; i++)
#pragma unroll
                        for (int j = 0; j < 3; j++) blk[i][j] = 0.0;
                }
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    double* row = a.out + (3 * f + i) * a.ld + 3 * s;
#pragma unroll
                    for (int j = 0; j < 3; j++) {
                        double v = a.alpha * blk[i][j];
                        row[j] = a.accumulate ? row[j] + v : v;
                    }
                }
            } else if (KIND == MAT_T_BASIS) {
                double blk[6][3][3];
                if (src.ok) {
                    PairP0 p;
                    pair_setup(src, xs[ff][0], xs[ff][1], xs[ff][2], p);
                    TMoments m;
                    t_moments(src, nrm, p, m);
                    t_basis_blocks(m, nrm, src.eps2, blk);
                } else {
                    for (int b = 0; b < 6; b++)
                        for (int i = 0; i < 3; i++)
                            for (int j = 0; j < 3; j++) blk[b][i][j] = 0.0;
                }
#pragma unroll
                for (int b = 0; b < 6; b++)
#pragma unroll
                    for (int i = 0; i < 3; i++)
#pragma unroll
                        for (int j = 0; j < 3; j++)
                            a.out[b * a.plane + (3 * f + i) * a.ld + 3 * s + j] = blk[b][i][j];
            } else {  // MAT_U_BASIS
                double I1 = 0.0, I3 = 0.0, T2[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                if (src.ok) {
                    PairP0 p;
                    pair_setup(src, xs[ff][0], xs[ff][1], xs[ff][2], p);
                    UMoments m;
                    u_moments(src, p, m);
                    I1 = m.I1;
                    I3 = m.I3;
#pragma unroll
                    for (int i = 0; i < 3; i++)
#pragma unroll
                        for (int j = 0; j < 3; j++) T2[i][j] = m.T2[i][j];
                }
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) {
                        const int64_t idx = (3 * f + i) * a.ld + 3 * s + j;
                        a.out[idx] = (i == j) ? I1 : 0.0;
                        a.out[a.plane + idx] = (i == j) ? src.eps2 * I3 : 0.0;
                        a.out[2 * a.plane + idx] = T2[i][j];
                    }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Contractions: out[f] (+)= alpha * sum_s K(x_f, s) density_s
// ---------------------------------------------------------------------------
enum ConKind {
    CON_T_DISP = 0,
    CON_U_DISP = 1,
    CON_DD_STRESS = 2,
    CON_KELVIN_STRESS = 3,
    CON_EIGENSTRESS = 4,
    CON_ELASTIC_STRESS = 5,   // dd stress minus eigenstress, one pass
};

struct ConArgs {
    const double* x_field;
    int64_t n_field;
    const double* tri_verts;
    const double* normals;
    const double* eps;
    const double* density;
    int64_t n_src;
    double c[6];
    double mu, lam;
    double alpha;
    int accumulate;
    double* out;
    int split;       // source slices per observer (1, 2, 4, 8 or 16)
};

struct SrcTile {
    SrcP0 g;
    double n[3];     // source normal as passed
    double d[3];     // density
    bool live;       // non-degenerate and non-zero density
};

template <int KIND>
__global__ void __launch_bounds__(CON_THREADS)
p0_contract_kernel(ConArgs a) {
    // A block holds CON_THREADS / split observers; the split threads of an
    // observer take interleaved sources of each tile and their partial sums
    // are added in slice order at the end (deterministic).
    __shared__ SrcTile tile[SRC_TILE];
    __shared__ double red[CON_THREADS][9];
    const int split = a.split;
    const int obs_per_block = CON_THREADS / split;
    const int lane = threadIdx.x % obs_per_block;
    const int slice = threadIdx.x / obs_per_block;
    const int64_t f = (int64_t)blockIdx.x * obs_per_block + lane;
    const bool active = f < a.n_field;
    double ox = 0, oy = 0, oz = 0;
    if (active) {
        ox = a.x_field[3 * f]; oy = a.x_field[3 * f + 1]; oz = a.x_field[3 * f + 2];
    }
    constexpr bool STRESS = KIND >= CON_DD_STRESS;
    double acc[9];
#pragma unroll
    for (int i = 0; i < 9; i++) acc[i] = 0.0;
    const double nu = a.lam / (2.0 * (a.lam + a.mu));
    const double C1 = 1.0 / (16.0 * MBEM_PI * a.mu * (1.0 - nu));
    const double c34 = 3.0 - 4.0 * nu;

    for (int64_t s0 = 0; s0 < a.n_src; s0 += SRC_TILE) {
        __syncthreads();
        for (int t = threadIdx.x; t < SRC_TILE; t += CON_THREADS) {
            const int64_t s = s0 + t;
            SrcTile& T = tile[t];
            if (s < a.n_src) {
                src_setup(a.tri_verts + 9 * s, a.eps[s], T.g);
                for (int k = 0; k < 3; k++) {
                    T.n[k] = (KIND == CON_U_DISP || KIND == CON_KELVIN_STRESS) ? 0.0 : a.normals[3 * s + k];
                    T.d[k] = a.density[3 * s + k];
                }
                T.live = T.g.ok && !(T.d[0] == 0.0 && T.d[1] == 0.0 && T.d[2] == 0.0);
                if (KIND == CON_EIGENSTRESS && !(T.g.eps > 0.0)) T.live = false;
            } else {
                T.live = false;
            }
        }
        __syncthreads();
        if (!active) continue;
        const int ns = (int)lmin(SRC_TILE, a.n_src - s0);
        for (int t = slice; t < ns; t += split) {
            const SrcTile& T = tile[t];
            if (!T.live) continue;
            const SrcP0& sg = T.g;
            PairP0 p;
            pair_setup(sg, ox, oy, oz, p);
            if (KIND == CON_T_DISP) {
                TMoments m;
                t_moments(sg, T.n, p, m);
                double blk[3][3];
                t_block(m, T.n, a.c, sg.eps2, blk);
#pragma unroll
                for (int i = 0; i < 3; i++)
                    acc[i] += blk[i][0] * T.d[0] + blk[i][1] * T.d[1] + blk[i][2] * T.d[2];
            } else if (KIND == CON_U_DISP) {
                UMoments m;
                u_moments(sg, p, m);
                const double dg = a.c[0] * m.I1 + a.c[1] * sg.eps2 * m.I3;
#pragma unroll
                for (int i = 0; i < 3; i++)
                    acc[i] += dg * T.d[i] +
                              a.c[2] * (m.T2[i][0] * T.d[0] + m.T2[i][1] * T.d[1] + m.T2[i][2] * T.d[2]);
            } else if (STRESS) {
                double sl[3];
                to_local(sg, T.d, sl);
                double loc[3][3];
                if (KIND == CON_KELVIN_STRESS) {
                    StressMoments M;
                    stress_moments<false>(sg, p, M);
                    const double cbdg = 6.0 * (1.0 - nu) * sg.eps2;
                    kelvin_stress_local(M, sl, a.mu, a.lam, C1, c34, cbdg, loc);
                } else {
                    StressMoments M;
                    stress_moments<true>(sg, p, M);
                    double phi = 0.0;
                    if (KIND == CON_EIGENSTRESS || KIND == CON_ELASTIC_STRESS)
                        phi = (sg.eps > 0.0) ? (15.0 * sg.eps2 * sg.eps2 / (8.0 * MBEM_PI)) * M.M7[0][0] : 0.0;
                    if (KIND == CON_DD_STRESS || KIND == CON_ELASTIC_STRESS) {
                        double nl[3];
                        to_local(sg, T.n, nl);
                        const double cblob = 2.0 * (1.0 - nu) * sg.eps2;
                        dd_stress_local(M, nl, sl, a.mu, a.lam, C1, c34, cblob, loc);
                    } else {
#pragma unroll
                        for (int i = 0; i < 3; i++)
#pragma unroll
                            for (int j = 0; j < 3; j++) loc[i][j] = 0.0;
                    }
                    if (KIND == CON_EIGENSTRESS || KIND == CON_ELASTIC_STRESS) {
                        // eigenstress in the global frame, tri_kernels.py:1206-1214
                        const double sgn = (KIND == CON_ELASTIC_STRESS) ? -1.0 : 1.0;
                        const double ns_ = T.n[0] * T.d[0] + T.n[1] * T.d[1] + T.n[2] * T.d[2];
                        double G[3][3];
                        rotate_sym(sg, loc, G);
#pragma unroll
                        for (int m = 0; m < 3; m++)
#pragma unroll
                            for (int n = 0; n < 3; n++)
                                acc[3 * m + n] += G[m][n] + sgn * phi *
                                    ((m == n ? a.lam * ns_ : 0.0) + a.mu * (T.d[m] * T.n[n] + T.d[n] * T.n[m]));
                        continue;
                    }
                }
                double G[3][3];
                rotate_sym(sg, loc, G);
#pragma unroll
                for (int m = 0; m < 3; m++)
#pragma unroll
                    for (int n = 0; n < 3; n++) acc[3 * m + n] += G[m][n];
            }
        }
    }
    const int nout = STRESS ? 9 : 3;
    if (split > 1) {
        __syncthreads();
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

// Slices per observer so that a launch holds about four 128-thread blocks
// per SM (152 SMs) whatever the observer count.
static int contract_split(int64_t nf) {
    int split = 1;
    while (split < 16 && nf * split < (int64_t)152 * 4 * CON_THREADS) split *= 2;
    return split;
}

static int check_common(const double* x, int64_t nf, const double* tv, const double* eps, int64_t ns,
                        int order) {
    MBEM_REQUIRE(nf >= 0 && ns >= 0, MBEM_ERR_ARG, "negative size (n_field=%lld, n_src=%lld)",
                 (long long)nf, (long long)ns);
    MBEM_REQUIRE(order == 0 || order == 1 || order == 2, MBEM_ERR_ARG,
                 "order must be 0, 1 or 2 (got %d)", order);
    MBEM_REQUIRE(nf == 0 || x != nullptr, MBEM_ERR_ARG, "x_field is NULL");
    MBEM_REQUIRE(ns == 0 || (tv != nullptr && eps != nullptr), MBEM_ERR_ARG, "tri_verts/eps is NULL");
    return MBEM_OK;
}

int launch_matrix(int kind, const double* x, int64_t nf, const double* tv, const double* normals,
                  const double* eps, int64_t ns, const double* c, int nc, double alpha, int accumulate,
                  double* out, int64_t ld, int64_t plane, cudaStream_t st) {
    MatArgs a;
    a.x_field = x; a.n_field = nf; a.tri_verts = tv; a.normals = normals; a.eps = eps; a.n_src = ns;
    for (int i = 0; i < 6; i++) a.c[i] = (c && i < nc) ? c[i] : 0.0;
    a.alpha = alpha; a.accumulate = accumulate; a.out = out; a.ld = ld; a.plane = plane;
    if (nf == 0 || ns == 0) return MBEM_OK;
    dim3 grid((unsigned)ceil_div(ns, MAT_THREADS), (unsigned)lmin(ceil_div(nf, FIELD_TILE), 65535));
    switch (kind) {
        case MAT_T_DIRECT: p0_matrix_kernel<MAT_T_DIRECT><<<grid, MAT_THREADS, 0, st>>>(a); break;
        case MAT_U_DIRECT: p0_matrix_kernel<MAT_U_DIRECT><<<grid, MAT_THREADS, 0, st>>>(a); break;
        case MAT_T_BASIS: p0_matrix_kernel<MAT_T_BASIS><<<grid, MAT_THREADS, 0, st>>>(a); break;
        default: p0_matrix_kernel<MAT_U_BASIS><<<grid, MAT_THREADS, 0, st>>>(a); break;
    }
    return launch_status("p0_matrix_kernel");
}

int launch_contract(int kind, const double* x, int64_t nf, const double* tv, const double* normals,
                    const double* eps, int64_t ns, const double* density, const double* c, int nc,
                    double mu, double lam, double alpha, int accumulate, double* out, cudaStream_t st) {
    ConArgs a;
    a.x_field = x; a.n_field = nf; a.tri_verts = tv; a.normals = normals; a.eps = eps;
    a.density = density; a.n_src = ns;
    for (int i = 0; i < 6; i++) a.c[i] = (c && i < nc) ? c[i] : 0.0;
    a.mu = mu; a.lam = lam; a.alpha = alpha; a.accumulate = accumulate; a.out = out;
    if (nf == 0) return MBEM_OK;
    a.split = contract_split(nf);
    dim3 grid((unsigned)ceil_div(nf, CON_THREADS / a.split));
    switch (kind) {
        case CON_T_DISP: p0_contract_kernel<CON_T_DISP><<<grid, CON_THREADS, 0, st>>>(a); break;
        case CON_U_DISP: p0_contract_kernel<CON_U_DISP><<<grid, CON_THREADS, 0, st>>>(a); break;
        case CON_DD_STRESS: p0_contract_kernel<CON_DD_STRESS><<<grid, CON_THREADS, 0, st>>>(a); break;
        case CON_KELVIN_STRESS: p0_contract_kernel<CON_KELVIN_STRESS><<<grid, CON_THREADS, 0, st>>>(a); break;
        case CON_EIGENSTRESS: p0_contract_kernel<CON_EIGENSTRESS><<<grid, CON_THREADS, 0, st>>>(a); break;
        default: p0_contract_kernel<CON_ELASTIC_STRESS><<<grid, CON_THREADS, 0, st>>>(a); break;
    }
    return launch_status("p0_contract_kernel");
}

}  // namespace mbem

using namespace mbem;

extern "C" {

int mbem_t_matrix_direct(const double* x_field, int64_t n_field, const double* tri_verts,
                         const double* normals, const double* eps, int64_t n_src, const double* coeffs,
                         int order, double alpha, int accumulate, double* out, int64_t ld_out,
                         void* stream) {
    int st = check_common(x_field, n_field, tri_verts, eps, n_src, order);
    if (st) return st;
    MBEM_REQUIRE(coeffs != nullptr, MBEM_ERR_ARG, "coeffs is NULL");
    MBEM_REQUIRE(n_src == 0 || normals != nullptr, MBEM_ERR_ARG, "normals is NULL");
    if (order != 0)
        return mbem::nodal_matrix(0, x_field, n_field, tri_verts, normals, eps, n_src, coeffs, order, alpha,
                                 accumulate, out, ld_out, stream);
    MBEM_REQUIRE(ld_out >= 3 * n_src, MBEM_ERR_ARG, "ld_out %lld < 3*n_src", (long long)ld_out);
    return launch_matrix(MAT_T_DIRECT, x_field, n_field, tri_verts, normals, eps, n_src, coeffs, 6, alpha,
                         accumulate, out, ld_out, 0, (cudaStream_t)stream);
}

int mbem_u_matrix_direct(const double* x_field, int64_t n_field, const double* tri_verts, const double* eps,
                         int64_t n_src, const double* coeffs, int order, double alpha, int accumulate,
                         double* out, int64_t ld_out, void* stream) {
    int st = check_common(x_field, n_field, tri_verts, eps, n_src, order);
    if (st) return st;
    MBEM_REQUIRE(coeffs != nullptr, MBEM_ERR_ARG, "coeffs is NULL");
    if (order != 0)
        return mbem::nodal_matrix(1, x_field, n_field, tri_verts, nullptr, eps, n_src, coeffs, order, alpha,
                                 accumulate, out, ld_out, stream);
    MBEM_REQUIRE(ld_out >= 3 * n_src, MBEM_ERR_ARG, "ld_out %lld < 3*n_src", (long long)ld_out);
    return launch_matrix(MAT_U_DIRECT, x_field, n_field, tri_verts, nullptr, eps, n_src, coeffs, 3, alpha,
                         accumulate, out, ld_out, 0, (cudaStream_t)stream);
}

int mbem_t_basis_matrices(const double* x_field, int64_t n_field, const double* tri_verts,
                          const double* normals, const double* eps, int64_t n_src, int order, double* out,
                          void* stream) {
    int st = check_common(x_field, n_field, tri_verts, eps, n_src, order);
    if (st) return st;
    MBEM_REQUIRE(n_src == 0 || normals != nullptr, MBEM_ERR_ARG, "normals is NULL");
    if (order != 0)
        return mbem::nodal_matrix(2, x_field, n_field, tri_verts, normals, eps, n_src, nullptr, order, 1.0, 0,
                                 out, 0, stream);
    return launch_matrix(MAT_T_BASIS, x_field, n_field, tri_verts, normals, eps, n_src, nullptr, 0, 1.0, 0,
                         out, 3 * n_src, 9 * n_field * n_src, (cudaStream_t)stream);
}

int mbem_u_basis_matrices(const double* x_field, int64_t n_field, const double* tri_verts, const double* eps,
                          int64_t n_src, int order, double* out, void* stream) {
    int st = check_common(x_field, n_field, tri_verts, eps, n_src, order);
    if (st) return st;
    if (order != 0)
        return mbem::nodal_matrix(3, x_field, n_field, tri_verts, nullptr, eps, n_src, nullptr, order, 1.0, 0,
                                 out, 0, stream);
    return launch_matrix(MAT_U_BASIS, x_field, n_field, tri_verts, nullptr, eps, n_src, nullptr, 0, 1.0, 0,
                         out, 3 * n_src, 9 * n_field * n_src, (cudaStream_t)stream);
}

int mbem_t_disp_contract(const double* x_field, int64_t n_field, const double* tri_verts,
                         const double* normals, const double* eps, int64_t n_src, const double* density,
                         const double* coeffs, int order, double alpha, int accumulate, double* out,
                         void* stream) {
    int st = check_common(x_field, n_field, tri_verts, eps, n_src, order);
    if (st) return st;
    MBEM_REQUIRE(coeffs != nullptr && (n_src == 0 || (normals && density)), MBEM_ERR_ARG,
                 "coeffs/normals/density is NULL");
    if (order != 0)
        return mbem::nodal_contract(0, x_field, n_field, tri_verts, normals, eps, n_src, density, coeffs, 0.0,
                                   0.0, order, alpha, accumulate, out, stream);
    return launch_contract(CON_T_DISP, x_field, n_field, tri_verts, normals, eps, n_src, density, coeffs, 6,
                           0.0, 0.0, alpha, accumulate, out, (cudaStream_t)stream);
}

int mbem_u_disp_contract(const double* x_field, int64_t n_field, const double* tri_verts, const double* eps,
                         int64_t n_src, const double* density, const double* coeffs, int order, double alpha,
                         int accumulate, double* out, void* stream) {
    int st = check_common(x_field, n_field, tri_verts, eps, n_src, order);
    if (st) return st;
    MBEM_REQUIRE(coeffs != nullptr && (n_src == 0 || density), MBEM_ERR_ARG, "coeffs/density is NULL");
    if (order != 0)
        return mbem::nodal_contract(1, x_field, n_field, tri_verts, nullptr, eps, n_src, density, coeffs, 0.0,
                                   0.0, order, alpha, accumulate, out, stream);
    return launch_contract(CON_U_DISP, x_field, n_field, tri_verts, nullptr, eps, n_src, density, coeffs, 3,
                           0.0, 0.0, alpha, accumulate, out, (cudaStream_t)stream);
}

int mbem_stress_contract(int kind, const double* x_field, int64_t n_field, const double* tri_verts,
                         const double* normals, const double* eps, int64_t n_src, const double* density,
                         double mu, double lam, int order, double alpha, int accumulate, double* out,
                         void* stream) {
    int st = check_common(x_field, n_field, tri_verts, eps, n_src, order);
    if (st) return st;
    MBEM_REQUIRE(kind >= MBEM_STRESS_DD && kind <= MBEM_STRESS_ELASTIC, MBEM_ERR_ARG,
                 "unknown stress kind %d", kind);
    MBEM_REQUIRE(n_src == 0 || density, MBEM_ERR_ARG, "density is NULL");
    MBEM_REQUIRE(kind == MBEM_STRESS_KELVIN || n_src == 0 || normals, MBEM_ERR_ARG, "normals is NULL");
    MBEM_REQUIRE(mu > 0.0 && lam + mu > 0.0, MBEM_ERR_ARG, "material (mu=%g, lam=%g) is not admissible", mu,
                 lam);
    if (order != 0)
        return mbem::nodal_contract(2 + kind, x_field, n_field, tri_verts, normals, eps, n_src, density,
                                   nullptr, mu, lam, order, alpha, accumulate, out, stream);
    return launch_contract(CON_DD_STRESS + kind, x_field, n_field, tri_verts, normals, eps, n_src, density,
                           nullptr, 0, mu, lam, alpha, accumulate, out, (cudaStream_t)stream);
}

}  // extern "C"
