// Compressed pair operator with P0 sources: cross approximation of the
// admissible blocks, exact dense blocks, and the flat product
// (src/mbem/la/hop.py PairCompressed, la/aca.py, la/flatview.py).
//
// Elements are numbered in the cluster-tree order, so a block is a pair of
// contiguous element ranges [r0, r0 + nr) x [c0, c0 + nc). An entry is the
// 3 x 3 pair block of (field point f, source triangle s) for the material's
// coefficients: the FP32 far quadrature of the mixed operator when the pair
// is far, the FP64 closed form otherwise.
//
// Cross approximation (aca.py:334-419 aca_single): one CTA per block. Pivots
// are 3 x 3 element blocks. Step: residual element row of the pivot row
// (exact row minus the factors so far), column pivot = the unused element
// column of largest residual Frobenius norm, residual element column, new
// factors for column pinv(P) row with P the 3 x 3 pivot block, kept at P's
// numerical rank (pivot_factors), then the true residual on a persistent
// 10 x 10 element sample; stop
// when it is below tol/2 of the sample's norm, or when no unused row or
// column has a non-zero residual. The next row pivot is the unused element row
// of largest norm in U_new. A block that reaches its rank cap is applied
// exactly. The finished factors are certified on 3 random element rows and 3
// random element columns evaluated exactly (relative Frobenius error of the
// lines together); a certificate above 3 tol reruns the block at tol/10, and
// a second failure leaves it exact (aca.py:579-658 compress_block).
//
// Differences from the reference, all within its tolerance: entries come
// from the FP32 far quadrature (<= ~1.5e-7 relative per block) and the
// residuals are FP32, so the pivot inverse treats singular values below 1e-6
// of the largest as zero (the reference's 1e-12 suits FP64 entries) and a
// rank-deficient pivot adds only its rank in columns (the reference adds three
// and drops the empty one when it recompresses); the
// sample and certificate lines come from a counter-based generator seeded
// per block instead of numpy's; the optional recompression (rc_kernel) works
// on the K x K core of the factors instead of a QR of each factor, and is
// certified again (the reference certifies the recompressed factors once).
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "common.cuh"
#include "dfloat.cuh"
#include "far_quad.cuh"
#include "p0_pair.cuh"

namespace mbem {
namespace {

constexpr int ACA_THREADS = 256;
constexpr int ACA_WARPS = ACA_THREADS / 32;
constexpr int ACA_SAMPLE = 10;            // sampled element rows / columns (aca.py:565-575 draw_lines)
constexpr int ACA_SLD = 3 * ACA_SAMPLE;   // sample row stride
constexpr int ACA_CERT = 3;               // ACA_CERTIFY_LINES
constexpr double ACA_CERT_FACTOR = 3.0;   // ACA_CERTIFY_FACTOR
constexpr double ACA_RETRY_FACTOR = 10.0; // ACA_RETRY_TOL_FACTOR
constexpr double ACA_PINV_RCOND = 1e-6;   // FP32 entries (see the header comment)
constexpr int CM_THREADS = 256;
constexpr int CM_WARPS = CM_THREADS / 32;
constexpr int CM_UNIT = 32;               // factor rows a work unit of the strip product (MBEM_COMPRESSED_UNIT)

__host__ __device__ __forceinline__ int pad4(int n) { return (n + 3) & ~3; }
inline size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

// prepared arrays of one pair: coefficients, split field points, per-source far constants
struct PrepLayout {
    size_t c64, xf, src, total;
};
inline PrepLayout prep_layout(int64_t nf, int64_t ns) {
    PrepLayout L;
    L.c64 = 0;
    L.xf = 256;
    L.src = L.xf + round256((size_t)nf * 3 * sizeof(F2));
    L.total = L.src + round256((size_t)ns * sizeof(SrcFar));
    return L;
}

// Everything an entry evaluation needs; pointers into device memory.
struct Geo {
    const F2* xf;
    const SrcFar* src;
    const double* x;
    const double* tv;
    const double* nrm;
    const double* eps;
    const double* c64;
    float c32[6];
};

inline Geo make_geo(const mbem_pair_geometry* g) {
    const PrepLayout L = prep_layout(g->n_field, g->n_src);
    char* p = (char*)g->prep;
    Geo G;
    G.c64 = (const double*)(p + L.c64);
    G.xf = (const F2*)(p + L.xf);
    G.src = (const SrcFar*)(p + L.src);
    G.x = g->x_field;
    G.tv = g->tri_verts;
    G.nrm = g->normals;
    G.eps = g->eps;
    for (int k = 0; k < 6; k++) G.c32[k] = (float)g->coeffs[k];
    return G;
}

__global__ void pair_prep_kernel(const double* __restrict__ x, int64_t nf, const double* __restrict__ tv,
                                 const double* __restrict__ nrm, const double* __restrict__ eps, int64_t ns,
                                 double near_factor, int tkernel, F2* __restrict__ xf, SrcFar* __restrict__ src) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 3 * nf; q += stride) xf[q] = split_d(x[q]);
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += stride) {
        SrcFar r;
        far_setup(tv + 9 * s, tkernel ? nrm + 3 * s : nullptr, eps[s], near_factor, r);
        src[s] = r;
    }
}

// FP64 closed form of one near pair, kept out of line so that the far path's
// registers do not carry it.
template <bool TK>
__device__ __noinline__ void near_fp64(const double* __restrict__ x, const double* __restrict__ tv,
                                       const double* __restrict__ nrm, double eps, const double* __restrict__ c,
                                       float* __restrict__ e) {
    SrcP0 s;
    src_setup(tv, eps, s);
    double blk[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    if (s.ok) {
        PairP0 p;
        pair_setup(s, x[0], x[1], x[2], p);
        if (TK) {
            TMoments m;
            t_moments(s, nrm, p, m);
            t_block(m, nrm, c, s.eps2, blk);
        } else {
            UMoments m;
            u_moments(s, p, m);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    blk[i][j] = c[2] * m.T2[i][j] + (i == j ? c[0] * m.I1 + c[1] * s.eps2 * m.I3 : 0.0);
        }
    }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) e[3 * i + j] = (float)blk[i][j];
}

// entry (f, s) with the source's far constants already loaded
template <bool TK>
__device__ __forceinline__ void pair_eval_src(const Geo& g, const QuadRules& Q, const SrcFar& sr, int64_t f,
                                              int64_t s, float e[3][3]) {
    if (!sr.ok) {
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) e[i][j] = 0.0f;
        return;
    }
    const F2 x[3] = {g.xf[3 * f], g.xf[3 * f + 1], g.xf[3 * f + 2]};
    float d[3], D2;
    if (is_near(x, sr, d, D2)) {
        near_fp64<TK>(g.x + 3 * f, g.tv + 9 * s, TK ? g.nrm + 3 * s : nullptr, g.eps[s], g.c64, &e[0][0]);
        return;
    }
    far_block<TK>(Q, sr, d, D2, g.c32, e);
}

template <bool TK>
__device__ __forceinline__ void pair_eval(const Geo& g, const QuadRules& Q, int64_t f, int64_t s, float e[3][3]) {
    const SrcFar sr = g.src[s];
    pair_eval_src<TK>(g, Q, sr, f, s, e);
}

// ---------------------------------------------------------------------------
// small helpers of the cross approximation
// ---------------------------------------------------------------------------
// splitmix64 (Steele, Lea and Flood, 2014)
__device__ __forceinline__ uint64_t splitmix(uint64_t& st) {
    st += 0x9E3779B97F4A7C15ull;
    uint64_t z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// m distinct integers of [0, n) (Floyd's sampling), m <= n
__device__ void draw_distinct(uint64_t& st, int n, int m, int* out) {
    int cnt = 0;
    for (int j = n - m; j < n; j++) {
        const int t = (int)(splitmix(st) % (uint64_t)(j + 1));
        bool dup = false;
        for (int q = 0; q < cnt; q++) dup |= out[q] == t;
        out[cnt++] = dup ? j : t;
    }
}

// The pivot step as factors of its numerical rank r: with P the 3 x 3 pivot
// block, C the residual element column and R the residual element row, the
// update C pinv(P) R is written as (C L)(R^T M)^T with L, M 3 x r (row-major,
// column k of each at [.][k]). When |det P| > rc ||P||_F^3, L = I and
// M = P^-T (r = 3). Otherwise pinv(P) = sum_k w_k (P w_k)^T / lambda_k over
// the eigenpairs of P^T P (cyclic Jacobi) with singular values above rc times
// the largest, and L[:, k] = w_k, M[:, k] = P w_k / lambda_k; a planar pair
// block of the T kernel is rank 2, and its third column is not stored.
// Returns r.
__device__ int pivot_factors(const double P[3][3], double rc, float L[9], float M[9]) {
    const double a = P[0][0], b = P[0][1], c = P[0][2];
    const double d = P[1][0], e = P[1][1], f = P[1][2];
    const double g = P[2][0], h = P[2][1], i = P[2][2];
    const double A = e * i - f * h, B = f * g - d * i, C = d * h - e * g;
    const double det = a * A + b * B + c * C;
    double n2 = 0.0;
    for (int r = 0; r < 3; r++)
        for (int s = 0; s < 3; s++) n2 += P[r][s] * P[r][s];
    const double sc = sqrt(n2);
    if (fabs(det) > rc * sc * sc * sc) {
        // M = P^-T: M[r][s] = inv[s][r]
        const double id = 1.0 / det;
        const double inv[9] = {A * id, (c * h - b * i) * id, (b * f - c * e) * id,
                               B * id, (a * i - c * g) * id, (c * d - a * f) * id,
                               C * id, (b * g - a * h) * id, (a * e - b * d) * id};
        for (int r = 0; r < 3; r++)
            for (int s = 0; s < 3; s++) {
                L[3 * r + s] = r == s ? 1.0f : 0.0f;
                M[3 * r + s] = (float)inv[3 * s + r];
            }
        return 3;
    }
    double G[3][3], W[3][3];
    for (int r = 0; r < 3; r++)
        for (int s = 0; s < 3; s++) {
            double v = 0.0;
            for (int m = 0; m < 3; m++) v += P[m][r] * P[m][s];
            G[r][s] = v;
            W[r][s] = r == s ? 1.0 : 0.0;
        }
    const int pp[3] = {0, 0, 1}, qq[3] = {1, 2, 2};
    for (int sweep = 0; sweep < 32; sweep++) {
        const double off = G[0][1] * G[0][1] + G[0][2] * G[0][2] + G[1][2] * G[1][2];
        const double dia = G[0][0] * G[0][0] + G[1][1] * G[1][1] + G[2][2] * G[2][2];
        if (!(off > 1e-32 * dia)) break;
        for (int r = 0; r < 3; r++) {
            const int p = pp[r], q = qq[r];
            if (G[p][q] == 0.0) continue;
            const double th = (G[q][q] - G[p][p]) / (2.0 * G[p][q]);
            const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
            const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
            for (int k = 0; k < 3; k++) {
                const double gp = G[k][p], gq = G[k][q];
                G[k][p] = cs * gp - sn * gq;
                G[k][q] = sn * gp + cs * gq;
            }
            for (int k = 0; k < 3; k++) {
                const double gp = G[p][k], gq = G[q][k];
                G[p][k] = cs * gp - sn * gq;
                G[q][k] = sn * gp + cs * gq;
            }
            for (int k = 0; k < 3; k++) {
                const double wp = W[k][p], wq = W[k][q];
                W[k][p] = cs * wp - sn * wq;
                W[k][q] = sn * wp + cs * wq;
            }
        }
    }
    const double lmax = fmax(fmax(G[0][0], G[1][1]), G[2][2]);
    int r = 0;
    for (int k = 0; k < 3; k++) {
        if (!(lmax > 0.0 && G[k][k] > rc * rc * lmax)) continue;
        const double il = 1.0 / G[k][k];
        for (int m = 0; m < 3; m++) {
            double pw = 0.0;
            for (int s = 0; s < 3; s++) pw += P[m][s] * W[s][k];
            L[3 * m + r] = (float)W[m][k];
            M[3 * m + r] = (float)(il * pw);
        }
        r++;
    }
    return r;
}

// block-wide sum in a fixed order (every thread gets the result)
__device__ __forceinline__ double block_sum(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    for (int k = 0; k < ACA_WARPS; k++) s += red[k];
    return s;
}

__device__ __forceinline__ void am_merge(float& v, int& i, float v2, int i2) {
    if (v2 > v || (v2 == v && i2 < i)) {
        v = v2;
        i = i2;
    }
}

// block-wide argmax: largest value, lowest index among ties
__device__ __forceinline__ void block_argmax(float& v, int& i, float* rv, int* ri) {
    for (int o = 16; o > 0; o >>= 1) {
        const float v2 = __shfl_xor_sync(0xffffffffu, v, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
        am_merge(v, i, v2, i2);
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        rv[threadIdx.x >> 5] = v;
        ri[threadIdx.x >> 5] = i;
    }
    __syncthreads();
    v = rv[0];
    i = ri[0];
    for (int k = 1; k < ACA_WARPS; k++) am_merge(v, i, rv[k], ri[k]);
}

// ---------------------------------------------------------------------------
// one-sided Jacobi (the recompression's SVD of its K x K core, rc_kernel)
// ---------------------------------------------------------------------------
// Pairs this close to orthogonal are left alone (1e-3 was measured to keep
// more blocks exact: the truncation then misjudges the tail); the certificate
// checks the truncated factors either way.
constexpr float OSJ_ORTH = 1e-5f;
constexpr int OSJ_SWEEPS = 24;

// Rows p and q of round `step` of the circle-method tournament on n (even)
// players: every pair meets once in n - 1 rounds, pairs of a round are disjoint.
__device__ __forceinline__ void osj_pair(int i, int step, int n, int& p, int& q) {
    const int m = n - 1;
    if (i == 0) {
        p = step % m;
        q = m;
    } else {
        p = (step + i) % m;
        q = (step - i + m) % m;
    }
}

// Sweeps of one-sided Jacobi on the K rows of A (length la, stride lda) until
// every pair is orthogonal to OSJ_ORTH; each rotation is applied to the rows
// of B too (length lb, stride ldb), so the product A^T B is unchanged. One
// warp a pair; dot products and rotations in FP32 (the FP64 pipe of this
// part is 1/64 of the FP32 one, and FP32 resolves the orthogonality test).
__device__ int osj_sweeps(float* A, int lda, int la, float* B, int ldb, int lb, int K, int* flag) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = K + (K & 1);
    int sweep = 0;
    for (; sweep < OSJ_SWEEPS; sweep++) {
        if (threadIdx.x == 0) *flag = 0;
        __syncthreads();
        for (int step = 0; step < n - 1; step++) {
            for (int i = warp; i < n / 2; i += ACA_WARPS) {
                int p, q;
                osj_pair(i, step, n, p, q);
                if (p >= K || q >= K) continue;
                float* ap = A + (int64_t)p * lda;
                float* aq = A + (int64_t)q * lda;
                float spp = 0.0f, sqq = 0.0f, spq = 0.0f;
#pragma unroll 4
                for (int c = lane; c < la; c += 32) {
                    const float x = ap[c], y = aq[c];
                    spp += x * x;
                    sqq += y * y;
                    spq += x * y;
                }
                for (int o = 16; o > 0; o >>= 1) {
                    spp += __shfl_xor_sync(0xffffffffu, spp, o);
                    sqq += __shfl_xor_sync(0xffffffffu, sqq, o);
                    spq += __shfl_xor_sync(0xffffffffu, spq, o);
                }
                if (!(fabsf(spq) > OSJ_ORTH * (sqrtf(spp) * sqrtf(sqq)))) continue;
                const float ze = (sqq - spp) / (2.0f * spq);
                const float t = copysignf(1.0f, ze) / (fabsf(ze) + sqrtf(1.0f + ze * ze));
                const float cd = rsqrtf(1.0f + t * t);
                const float c = cd, sn = cd * t;
#pragma unroll 4
                for (int e = lane; e < la; e += 32) {
                    const float x = ap[e], y = aq[e];
                    ap[e] = c * x - sn * y;
                    aq[e] = sn * x + c * y;
                }
                float* bp = B + (int64_t)p * ldb;
                float* bq = B + (int64_t)q * ldb;
#pragma unroll 4
                for (int e = lane; e < lb; e += 32) {
                    const float x = bp[e], y = bq[e];
                    bp[e] = c * x - sn * y;
                    bq[e] = sn * x + c * y;
                }
                if (lane == 0) *flag = 1;
            }
            __syncthreads();
        }
        if (*flag == 0) break;
        __syncthreads();
    }
    __syncthreads();
    return sweep + 1;
}

// squared norm of row k of A over la entries (one warp), in FP64
__device__ __forceinline__ double row_norm2(const float* A, int lda, int la, int k) {
    const int lane = threadIdx.x & 31;
    float s = 0.0f;
    for (int c = lane; c < la; c += 32) {
        const float x = A[(int64_t)k * lda + c];
        s += x * x;
    }
    double d = s;
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    return d;
}

// The sample rows and columns (ACA_SAMPLE each) and the certificate rows and
// columns (ACA_CERT each) of block `index`, from a counter-based stream seeded
// by (seed, index): lines[0..9] rows, [10..19] columns, [20..22] certificate
// rows, [23..25] certificate columns.
__device__ void draw_lines(uint64_t seed, int64_t index, int nr, int nc, int* lines) {
    uint64_t st = seed ^ (0xD1B54A32D192ED03ull * (uint64_t)(index + 1));
    splitmix(st);
    draw_distinct(st, nr, min(ACA_SAMPLE, nr), lines);
    draw_distinct(st, nc, min(ACA_SAMPLE, nc), lines + ACA_SAMPLE);
    draw_distinct(st, nr, min(ACA_CERT, nr), lines + 2 * ACA_SAMPLE);
    draw_distinct(st, nc, min(ACA_CERT, nc), lines + 2 * ACA_SAMPLE + ACA_CERT);
}

struct AcaArgs {
    const int32_t* r0;
    const int32_t* nr;
    const int32_t* c0;
    const int32_t* nc;
    const int32_t* cap;
    const int64_t* u_off;
    const int64_t* v_off;
    float* U;
    float* V;
    int32_t* rank;
    int32_t* status;
    float* err;
    double tol;
    uint64_t seed;
    int64_t first_index;
    int ldr;    // shared row-buffer stride, pad4(3 max_nc)
    int kcap;   // 3 x the largest rank cap
    int max_nr;
};

inline size_t aca_smem_bytes(int max_nr, int max_nc, int max_pivots) {
    const size_t ldr = pad4(3 * max_nc), kcap = 3 * (size_t)max_pivots;
    return sizeof(float) * (3 * ldr + 6 * kcap + 2 * ACA_SLD * ACA_SLD) + (size_t)pad4(max_nr) + (size_t)pad4(max_nc);
}

template <bool TK>
__global__ void __launch_bounds__(ACA_THREADS, 2) aca_kernel(AcaArgs a, Geo g, QuadRules Q) {
    extern __shared__ __align__(16) float sm[];
    __shared__ double red_d[ACA_WARPS];
    __shared__ float red_f[ACA_WARPS];
    __shared__ int red_i[ACA_WARPS];
    __shared__ int lines[2 * ACA_SAMPLE + 2 * ACA_CERT];
    __shared__ float Lp[9], Mp[9];
    __shared__ int rp;

    const int64_t blk = blockIdx.x;
    const int t = threadIdx.x;
    const int r0 = a.r0[blk], nr = a.nr[blk], c0 = a.c0[blk], nc = a.nc[blk];
    const int cap = a.cap[blk];
    const int ldu = pad4(3 * nr), ldv = pad4(3 * nc);
    const int ldr = a.ldr, kcap = a.kcap;
    float* __restrict__ U = a.U + a.u_off[blk];
    float* __restrict__ V = a.V + a.v_off[blk];
    float* R = sm;
    float* Ub = R + 3 * ldr;
    float* Vb = Ub + 3 * kcap;
    float* Sx = Vb + 3 * kcap;
    float* Sr = Sx + ACA_SLD * ACA_SLD;
    uint8_t* used_r = (uint8_t*)(Sr + ACA_SLD * ACA_SLD);
    uint8_t* used_c = used_r + pad4(a.max_nr);

    const int ns_r = min(ACA_SAMPLE, nr), ns_c = min(ACA_SAMPLE, nc);
    const int nc_r = min(ACA_CERT, nr), nc_c = min(ACA_CERT, nc);
    if (t == 0) draw_lines(a.seed, a.first_index + blk, nr, nc, lines);
    __syncthreads();

    // exact sample
    double part = 0.0;
    for (int p = t; p < ns_r * ns_c; p += ACA_THREADS) {
        const int pr = p / ns_c, pc = p - pr * ns_c;
        float e[3][3];
        pair_eval<TK>(g, Q, r0 + lines[pr], c0 + lines[ACA_SAMPLE + pc], e);
        for (int aa = 0; aa < 3; aa++)
            for (int bb = 0; bb < 3; bb++) {
                Sx[(3 * pr + aa) * ACA_SLD + 3 * pc + bb] = e[aa][bb];
                part += (double)e[aa][bb] * e[aa][bb];
            }
    }
    const double snorm2 = block_sum(part, red_d);

    int status = MBEM_ACA_FAILED, rank_out = 0;
    float err_out = 0.0f;
    bool retried = false;
    double tol = a.tol;
    for (int attempt = 0; attempt < 2; attempt++) {
        for (int i = t; i < nr; i += ACA_THREADS) used_r[i] = 0;
        for (int j = t; j < nc; j += ACA_THREADS) used_c[j] = 0;
        for (int p = t; p < ACA_SLD * ACA_SLD; p += ACA_THREADS) Sr[p] = Sx[p];
        __syncthreads();
        const double stop2 = 0.25 * tol * tol * snorm2;
        int K = 0, ip = 0;
        bool conv = false;
        for (int it = 0; it < cap; it++) {
            if (t == 0) used_r[ip] = 1;
            for (int q = t; q < 3 * K; q += ACA_THREADS) {
                const int aa = q / K, k = q - aa * K;
                Ub[aa * kcap + k] = U[(int64_t)k * ldu + 3 * ip + aa];
            }
            __syncthreads();
            // residual element row ip
            float bv = -1.0f;
            int bi = 0x7fffffff;
            for (int j = t; j < nc; j += ACA_THREADS) {
                float e[3][3];
                pair_eval<TK>(g, Q, r0 + ip, c0 + j, e);
                for (int k = 0; k < K; k++) {
                    const float* vk = V + (int64_t)k * ldv + 3 * j;
                    const float v0 = vk[0], v1 = vk[1], v2 = vk[2];
#pragma unroll
                    for (int aa = 0; aa < 3; aa++) {
                        const float u = Ub[aa * kcap + k];
                        e[aa][0] -= u * v0;
                        e[aa][1] -= u * v1;
                        e[aa][2] -= u * v2;
                    }
                }
                float sc = 0.0f;
#pragma unroll
                for (int aa = 0; aa < 3; aa++)
#pragma unroll
                    for (int bb = 0; bb < 3; bb++) {
                        R[aa * ldr + 3 * j + bb] = e[aa][bb];
                        sc += e[aa][bb] * e[aa][bb];
                    }
                if (!used_c[j]) am_merge(bv, bi, sc, j);
            }
            block_argmax(bv, bi, red_f, red_i);
            if (!(bv > 0.0f)) {
                conv = true;
                break;
            }
            const int jp = bi;
            __syncthreads();
            if (t == 0) used_c[jp] = 1;
            for (int q = t; q < 3 * K; q += ACA_THREADS) {
                const int bb = q / K, k = q - bb * K;
                Vb[bb * kcap + k] = V[(int64_t)k * ldv + 3 * jp + bb];
            }
            if (t == 0) {
                double P[3][3];
                for (int aa = 0; aa < 3; aa++)
                    for (int bb = 0; bb < 3; bb++) P[aa][bb] = R[aa * ldr + 3 * jp + bb];
                rp = pivot_factors(P, ACA_PINV_RCOND, Lp, Mp);
            }
            __syncthreads();
            // residual element column jp; new U columns K .. K+r-1 = C L; next row pivot
            const int r = rp;
            float rv = -1.0f;
            int ri = 0x7fffffff;
            for (int i = t; i < nr; i += ACA_THREADS) {
                float e[3][3];
                pair_eval<TK>(g, Q, r0 + i, c0 + jp, e);
                for (int k = 0; k < K; k++) {
                    const float* uk = U + (int64_t)k * ldu + 3 * i;
                    const float u0 = uk[0], u1 = uk[1], u2 = uk[2];
#pragma unroll
                    for (int bb = 0; bb < 3; bb++) {
                        const float v = Vb[bb * kcap + k];
                        e[0][bb] -= u0 * v;
                        e[1][bb] -= u1 * v;
                        e[2][bb] -= u2 * v;
                    }
                }
                float sc = 0.0f;
                for (int k = 0; k < r; k++) {
#pragma unroll
                    for (int aa = 0; aa < 3; aa++) {
                        const float u = e[aa][0] * Lp[k] + e[aa][1] * Lp[3 + k] + e[aa][2] * Lp[6 + k];
                        U[(int64_t)(K + k) * ldu + 3 * i + aa] = u;
                        sc += u * u;
                    }
                }
                if (!used_r[i]) am_merge(rv, ri, sc, i);
            }
            // padding of the new factor rows stays finite (the product reads it)
            for (int q = t; q < r * (ldu - 3 * nr); q += ACA_THREADS) {
                const int k = q / (ldu - 3 * nr), c = 3 * nr + q - k * (ldu - 3 * nr);
                U[(int64_t)(K + k) * ldu + c] = 0.0f;
            }
            // new V columns K .. K+r-1 = R^T M
            for (int c = t; c < ldv; c += ACA_THREADS) {
                const bool in = c < 3 * nc;
                const float x0 = in ? R[c] : 0.0f, x1 = in ? R[ldr + c] : 0.0f, x2 = in ? R[2 * ldr + c] : 0.0f;
                for (int k = 0; k < r; k++)
                    V[(int64_t)(K + k) * ldv + c] = Mp[k] * x0 + Mp[3 + k] * x1 + Mp[6 + k] * x2;
            }
            block_argmax(rv, ri, red_f, red_i);   // its barriers also publish the new factors
            // true residual on the sample
            double res = 0.0;
            for (int p = t; p < 9 * ns_r * ns_c; p += ACA_THREADS) {
                const int ra = p / (3 * ns_c), cb = p - ra * (3 * ns_c);
                const int row = 3 * lines[ra / 3] + ra % 3, col = 3 * lines[ACA_SAMPLE + cb / 3] + cb % 3;
                float v = Sr[ra * ACA_SLD + cb];
                for (int k = 0; k < r; k++)
                    v -= U[(int64_t)(K + k) * ldu + row] * V[(int64_t)(K + k) * ldv + col];
                Sr[ra * ACA_SLD + cb] = v;
                res += (double)v * v;
            }
            const double res2 = block_sum(res, red_d);
            K += r;
            if (snorm2 == 0.0 || res2 < stop2 || !(rv > 0.0f)) {
                conv = true;
                break;
            }
            ip = ri;
        }
        if (!conv) {
            status = MBEM_ACA_CAPPED;
            break;
        }
        // certificate: 3 exact element rows and 3 exact element columns
        float dr = 0.0f, er = 0.0f, dc = 0.0f, ec = 0.0f;   // per thread (FP32); summed in FP64 below
        for (int q = 0; q < nc_r; q++) {
            const int i = lines[2 * ACA_SAMPLE + q];
            __syncthreads();
            for (int z = t; z < 3 * K; z += ACA_THREADS) {
                const int aa = z / K, k = z - aa * K;
                Ub[aa * kcap + k] = U[(int64_t)k * ldu + 3 * i + aa];
            }
            __syncthreads();
            for (int j = t; j < nc; j += ACA_THREADS) {
                float e[3][3], ap[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                pair_eval<TK>(g, Q, r0 + i, c0 + j, e);
                for (int k = 0; k < K; k++) {
                    const float* vk = V + (int64_t)k * ldv + 3 * j;
                    const float v0 = vk[0], v1 = vk[1], v2 = vk[2];
#pragma unroll
                    for (int aa = 0; aa < 3; aa++) {
                        const float u = Ub[aa * kcap + k];
                        ap[aa][0] += u * v0;
                        ap[aa][1] += u * v1;
                        ap[aa][2] += u * v2;
                    }
                }
#pragma unroll
                for (int aa = 0; aa < 3; aa++)
#pragma unroll
                    for (int bb = 0; bb < 3; bb++) {
                        const float df = ap[aa][bb] - e[aa][bb];
                        dr += df * df;
                        er += e[aa][bb] * e[aa][bb];
                    }
            }
        }
        for (int q = 0; q < nc_c; q++) {
            const int j = lines[2 * ACA_SAMPLE + ACA_CERT + q];
            __syncthreads();
            for (int z = t; z < 3 * K; z += ACA_THREADS) {
                const int bb = z / K, k = z - bb * K;
                Vb[bb * kcap + k] = V[(int64_t)k * ldv + 3 * j + bb];
            }
            __syncthreads();
            for (int i = t; i < nr; i += ACA_THREADS) {
                float e[3][3], ap[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                pair_eval<TK>(g, Q, r0 + i, c0 + j, e);
                for (int k = 0; k < K; k++) {
                    const float* uk = U + (int64_t)k * ldu + 3 * i;
                    const float u0 = uk[0], u1 = uk[1], u2 = uk[2];
#pragma unroll
                    for (int bb = 0; bb < 3; bb++) {
                        const float v = Vb[bb * kcap + k];
                        ap[0][bb] += u0 * v;
                        ap[1][bb] += u1 * v;
                        ap[2][bb] += u2 * v;
                    }
                }
#pragma unroll
                for (int aa = 0; aa < 3; aa++)
#pragma unroll
                    for (int bb = 0; bb < 3; bb++) {
                        const float df = ap[aa][bb] - e[aa][bb];
                        dc += df * df;
                        ec += e[aa][bb] * e[aa][bb];
                    }
            }
        }
        const double sdr = block_sum(dr, red_d), ser = block_sum(er, red_d);
        const double sdc = block_sum(dc, red_d), sec = block_sum(ec, red_d);
        const double err = fmax(ser > 0.0 ? sqrt(sdr / ser) : 0.0, sec > 0.0 ? sqrt(sdc / sec) : 0.0);
        if (err <= ACA_CERT_FACTOR * a.tol) {
            status = MBEM_ACA_LOWRANK;
            rank_out = K;
            err_out = (float)err;
            break;
        }
        if (attempt == 0) {
            retried = true;
            tol = a.tol / ACA_RETRY_FACTOR;
            __syncthreads();
            continue;
        }
        status = MBEM_ACA_FAILED;
    }
    if (t == 0) {
        a.rank[blk] = status == MBEM_ACA_LOWRANK ? rank_out : 0;
        a.status[blk] = status | (retried ? MBEM_ACA_RETRIED : 0);
        a.err[blk] = err_out;
    }
}

// ---------------------------------------------------------------------------
// recompression (aca.py:422-438): the SVD of U V^T truncated at tol by its
// K x K core. Grams Gu = U^T U, Gv = V^T V in double-float (exact FP32
// products, compensated sums), Cholesky Gu + d = Ru^T Ru, Gv + d = Rv^T Rv in
// FP64 (d = 1e-12 of the largest diagonal entry), C = Ru Rv^T, one-sided
// Jacobi on C's columns in FP32: C Y = X S. Keeping k singular values,
// U' = U (Rv^T Y_k) and V' = V (Ru^T (C Y)_k S_k^-2), which equal
// Qu X_k S_k and Qv Y_k with no triangular solve. The kept factors are then
// certified on the block's own certificate lines; a block whose certificate
// exceeds 3 tol keeps its cross-approximation factors.
// ---------------------------------------------------------------------------
constexpr int RC_KMAX = 64;

struct RcArgs {
    const int32_t* r0;
    const int32_t* nr;
    const int32_t* c0;
    const int32_t* nc;
    const int32_t* rank;
    const int64_t* u_off;
    const int64_t* v_off;
    const float* U;
    const float* V;
    const int64_t* ur_off;
    const int64_t* vr_off;
    float* Ur;
    float* Vr;
    int32_t* rank_out;
    float* err_out;
    const int64_t* index;
    double tol;
    uint64_t seed;
    int kmax;
};

inline size_t rc_smem_bytes(int kmax) {
    const size_t k2 = (size_t)kmax * kmax;
    return 2 * k2 * sizeof(double) + 4 * k2 * sizeof(float) + 3 * (size_t)kmax * sizeof(float) + 64;
}

// G[i][j] = sum_r A[i][r] A[j][r] (K rows of length len at stride ld), one warp
// a pair, exact products summed in double-float per lane, then in FP64
__device__ void rc_gram(const float* __restrict__ A, int64_t ld, int len, int K, double* G) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int np = K * (K + 1) / 2;
    for (int p = warp; p < np; p += nw) {
        int i = 0, rem = p;
        while (rem >= K - i) {
            rem -= K - i;
            i++;
        }
        const int j = i + rem;
        const float* ai = A + (int64_t)i * ld;
        const float* aj = A + (int64_t)j * ld;
        float sh = 0.0f, sl = 0.0f;
        for (int r = lane; r < len; r += 32) {
            const float x = ai[r], y = aj[r];
            const float pr = __fmul_rn(x, y);
            const float pe = __fmaf_rn(x, y, -pr);
            const float sn = __fadd_rn(sh, pr);
            const float bb = __fsub_rn(sn, sh);
            sl = __fadd_rn(sl, __fadd_rn(__fadd_rn(__fsub_rn(sh, __fsub_rn(sn, bb)), __fsub_rn(pr, bb)), pe));
            sh = sn;
        }
        double v = (double)sh + (double)sl;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) {
            G[i * K + j] = v;
            G[j * K + i] = v;
        }
    }
}

// In place, the upper Cholesky factor R (R^T R = G + d I) of a K x K FP64 matrix
// (row-major; the strict lower part is left undefined)
__device__ void rc_cholesky(double* G, int K) {
    __shared__ double piv;
    double dmax = 0.0;
    for (int i = 0; i < K; i++) dmax = fmax(dmax, G[i * K + i]);
    const double d = 1e-12 * dmax + 1e-300;
    for (int k = 0; k < K; k++) {
        __syncthreads();
        if (threadIdx.x == 0) {
            const double g = G[k * K + k] + d;
            piv = g > 0.0 ? sqrt(g) : sqrt(d);
            G[k * K + k] = piv;
        }
        __syncthreads();
        const double ip = 1.0 / piv;
        for (int j = k + 1 + threadIdx.x; j < K; j += blockDim.x) G[k * K + j] *= ip;
        __syncthreads();
        // trailing update of the upper part: G[i][j] -= R[k][i] R[k][j], k < i <= j
        const int m = K - k - 1;
        for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
            const int i = k + 1 + e / m, j = k + 1 + e % m;
            if (j >= i) G[i * K + j] -= G[k * K + i] * G[k * K + j];
        }
    }
    __syncthreads();
}

template <bool TK>
__global__ void __launch_bounds__(ACA_THREADS) rc_kernel(RcArgs a, Geo g, QuadRules Q) {
    extern __shared__ __align__(16) float rsmf[];
    double* rsm = reinterpret_cast<double*>(rsmf);
    __shared__ int lines[2 * ACA_SAMPLE + 2 * ACA_CERT];
    __shared__ int flag;
    __shared__ double red_d[ACA_WARPS];
    const int64_t blk = blockIdx.x;
    const int t = threadIdx.x;
    const int K = a.rank[blk];
    if (K < 2 || K > a.kmax) {
        if (t == 0) {
            a.rank_out[blk] = 0;
            a.err_out[blk] = 0.0f;
        }
        return;
    }
    const int r0 = a.r0[blk], nr = a.nr[blk], c0 = a.c0[blk], nc = a.nc[blk];
    const int la = 3 * nr, lb = 3 * nc, ldu = pad4(la), ldv = pad4(lb);
    const int KX = a.kmax;
    double* Gu = rsm;
    double* Gv = Gu + KX * KX;
    float* Ct = (float*)(Gv + KX * KX);     // row i: column i of C (then of C Y)
    float* Yt = Ct + KX * KX;               // row i: column i of Y
    float* Cu = Yt + KX * KX;               // K x k, row-major at stride K
    float* Cv = Cu + KX * KX;
    float* sig = Cv + KX * KX;              // 3 K words
    int* rk = (int*)(sig + K);
    const float* U = a.U + a.u_off[blk];
    const float* V = a.V + a.v_off[blk];
    rc_gram(U, ldu, la, K, Gu);
    rc_gram(V, ldv, lb, K, Gv);
    __syncthreads();
    rc_cholesky(Gu, K);
    rc_cholesky(Gv, K);
    // C = Ru Rv^T: C[i][j] = sum_{l >= max(i, j)} Ru[i][l] Rv[j][l]; stored as Ct[j][i]
    for (int e = t; e < K * K; e += blockDim.x) {
        const int i = e / K, j = e % K;
        double v = 0.0;
        for (int l = max(i, j); l < K; l++) v += Gu[i * K + l] * Gv[j * K + l];
        Ct[j * K + i] = (float)v;
        Yt[j * K + i] = i == j ? 1.0f : 0.0f;
    }
    __syncthreads();
    osj_sweeps(Ct, K, K, Yt, K, K, K, &flag);
    for (int k = t >> 5; k < K; k += ACA_WARPS) {
        const double d = sqrt(row_norm2(Ct, K, K, k));
        if ((t & 31) == 0) sig[k] = (float)d;
    }
    __syncthreads();
    for (int j = t; j < K; j += blockDim.x) {
        int r = 0;
        const float sj = sig[j];
        for (int i = 0; i < K; i++) r += (sig[i] > sj || (sig[i] == sj && i < j)) ? 1 : 0;
        rk[j] = r;
    }
    __syncthreads();
    float* srt = sig + 2 * K;
    for (int j = t; j < K; j += blockDim.x) srt[rk[j]] = sig[j];
    __syncthreads();
    if (t == 0) {
        const double s0 = srt[0], tl = 0.5 * a.tol;
        double dropped = 0.0;
        int keep = K;
        for (int r = K - 1; r >= 1; r--) {
            const double sr = srt[r];
            if (dropped + sr * sr > tl * tl * s0 * s0) break;
            dropped += sr * sr;
            keep = r;
        }
        flag = keep;
    }
    __syncthreads();
    const int kk = flag;
    // Cu[:, q] = Rv^T y_j and Cv[:, q] = Ru^T (C y)_j / s_j^2 for the kept j (q its rank)
    for (int e = t; e < K * K; e += blockDim.x) {
        const int i = e / K, j = e % K;
        const int q = rk[j];
        if (q >= kk) continue;
        double cu = 0.0, cv = 0.0;
        for (int l = 0; l <= i; l++) {
            cu += Gv[l * K + i] * (double)Yt[j * K + l];
            cv += Gu[l * K + i] * (double)Ct[j * K + l];
        }
        const double sj = sig[j];
        Cu[i * K + q] = (float)cu;
        Cv[i * K + q] = sj > 0.0 ? (float)(cv / (sj * sj)) : 0.0f;
    }
    __syncthreads();
    // U'^T[q][r] = sum_i U^T[i][r] Cu[i][q]; likewise V'
    float* Ur = a.Ur + a.ur_off[blk];
    float* Vr = a.Vr + a.vr_off[blk];
    for (int r = t; r < ldu; r += blockDim.x) {
        for (int q = 0; q < kk; q++) {
            float acc = 0.0f;
            if (r < la)
                for (int i = 0; i < K; i++) acc += U[(int64_t)i * ldu + r] * Cu[i * K + q];
            Ur[(int64_t)q * ldu + r] = acc;
        }
    }
    for (int r = t; r < ldv; r += blockDim.x) {
        for (int q = 0; q < kk; q++) {
            float acc = 0.0f;
            if (r < lb)
                for (int i = 0; i < K; i++) acc += V[(int64_t)i * ldv + r] * Cv[i * K + q];
            Vr[(int64_t)q * ldv + r] = acc;
        }
    }
    // certificate of the new factors on the block's certificate lines
    if (t == 0) draw_lines(a.seed, a.index[blk], nr, nc, lines);
    __syncthreads();
    float dr = 0.0f, er = 0.0f;
    const int nc_r = min(ACA_CERT, nr), nc_c = min(ACA_CERT, nc);
    for (int q = 0; q < nc_r; q++) {
        const int i = lines[2 * ACA_SAMPLE + q];
        for (int j = t; j < nc; j += blockDim.x) {
            float e[3][3], ap[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            pair_eval<TK>(g, Q, r0 + i, c0 + j, e);
            for (int k = 0; k < kk; k++) {
                const float* vk = Vr + (int64_t)k * ldv + 3 * j;
                const float* uk = Ur + (int64_t)k * ldu + 3 * i;
                for (int aa = 0; aa < 3; aa++)
                    for (int bb = 0; bb < 3; bb++) ap[aa][bb] += uk[aa] * vk[bb];
            }
            for (int aa = 0; aa < 3; aa++)
                for (int bb = 0; bb < 3; bb++) {
                    const float df = ap[aa][bb] - e[aa][bb];
                    dr += df * df;
                    er += e[aa][bb] * e[aa][bb];
                }
        }
    }
    float dc = 0.0f, ec = 0.0f;
    for (int q = 0; q < nc_c; q++) {
        const int j = lines[2 * ACA_SAMPLE + ACA_CERT + q];
        for (int i = t; i < nr; i += blockDim.x) {
            float e[3][3], ap[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            pair_eval<TK>(g, Q, r0 + i, c0 + j, e);
            for (int k = 0; k < kk; k++) {
                const float* vk = Vr + (int64_t)k * ldv + 3 * j;
                const float* uk = Ur + (int64_t)k * ldu + 3 * i;
                for (int aa = 0; aa < 3; aa++)
                    for (int bb = 0; bb < 3; bb++) ap[aa][bb] += uk[aa] * vk[bb];
            }
            for (int aa = 0; aa < 3; aa++)
                for (int bb = 0; bb < 3; bb++) {
                    const float df = ap[aa][bb] - e[aa][bb];
                    dc += df * df;
                    ec += e[aa][bb] * e[aa][bb];
                }
        }
    }
    const double sdr = block_sum(dr, red_d), ser = block_sum(er, red_d);
    const double sdc = block_sum(dc, red_d), sec = block_sum(ec, red_d);
    const double err = fmax(ser > 0.0 ? sqrt(sdr / ser) : 0.0, sec > 0.0 ? sqrt(sdc / sec) : 0.0);
    if (t == 0) {
        const bool ok = err <= ACA_CERT_FACTOR * a.tol;
        a.rank_out[blk] = ok ? kk : 0;
        a.err_out[blk] = (float)err;
    }
}

__global__ void aca_compact_kernel(const int32_t* __restrict__ nr, const int32_t* __restrict__ nc,
                                   const int32_t* __restrict__ rank, const int64_t* __restrict__ u_src,
                                   const int64_t* __restrict__ v_src, const float* __restrict__ U_src,
                                   const float* __restrict__ V_src, const int64_t* __restrict__ u_dst,
                                   const int64_t* __restrict__ v_dst, float* __restrict__ U_dst,
                                   float* __restrict__ V_dst) {
    const int64_t b = blockIdx.x;
    const int K = rank[b];
    const int64_t nu = (int64_t)K * pad4(3 * nr[b]) / 4, nv = (int64_t)K * pad4(3 * nc[b]) / 4;
    const float4* us = (const float4*)(U_src + u_src[b]);
    const float4* vs = (const float4*)(V_src + v_src[b]);
    float4* ud = (float4*)(U_dst + u_dst[b]);
    float4* vd = (float4*)(V_dst + v_dst[b]);
    for (int64_t q = threadIdx.x; q < nu; q += blockDim.x) ud[q] = us[q];
    for (int64_t q = threadIdx.x; q < nv; q += blockDim.x) vd[q] = vs[q];
}

struct DenseArgs {
    int64_t n_blocks, n_items;
    const int32_t* r0;
    const int32_t* nr;
    const int32_t* c0;
    const int32_t* nc;
    const int64_t* d_off;
    const int64_t* col_ptr;
    float* D;
};

// one thread per (block, source column): the source's constants once, every
// row of the block. Blocks are stored transposed: D^T (3 nc rows of
// pad4(3 nr) floats), so that the product streams them like the U^T factors.
template <bool TK>
__global__ void __launch_bounds__(128) pair_dense_kernel(DenseArgs a, Geo g, QuadRules Q) {
    const int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= a.n_items) return;
    int64_t lo = 0, hi = a.n_blocks;
    while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (a.col_ptr[mid] <= it) lo = mid;
        else hi = mid;
    }
    const int64_t j = it - a.col_ptr[lo];
    const int64_t s = a.c0[lo] + j;
    const int nr = a.nr[lo];
    const int64_t ld = pad4(3 * nr);
    const int64_t f0 = a.r0[lo];
    float* out = a.D + a.d_off[lo] + 3 * j * ld;    // rows 3j .. 3j+2 of D^T
    const SrcFar sr = g.src[s];
    for (int i = 0; i < nr; i++) {
        float e[3][3];
        pair_eval_src<TK>(g, Q, sr, f0 + i, s, e);
#pragma unroll
        for (int aa = 0; aa < 3; aa++)
#pragma unroll
            for (int bb = 0; bb < 3; bb++) out[bb * ld + 3 * i + aa] = e[aa][bb];
    }
    // the padding of this column's three rows stays finite (the product reads it)
    for (int bb = 0; bb < 3; bb++)
        for (int c = 3 * nr; c < ld; c++) out[bb * ld + c] = 0.0f;
}

// ---------------------------------------------------------------------------
// the flat product
// ---------------------------------------------------------------------------
__global__ void cm_gather_kernel(const double* __restrict__ x, const int64_t* __restrict__ order, int64_t n,
                                 float* __restrict__ xs) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    if (blockIdx.x == 0 && threadIdx.x < 4) xs[3 * n + threadIdx.x] = 0.0f;   // read by the last padded block
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 3 * n; q += stride) {
        const int64_t p = q / 3;
        xs[q] = (float)x[3 * order[p] + (q - 3 * p)];
    }
}

// w_i = V_i^T x[cols_i] for every low-rank block: one warp a unit of four
// factor rows of one block (proj_block / proj_k0), so that a block of many
// rows is shared among many warps and a small one takes one; 16-byte loads of
// V, x from the gathered vector (L1/L2-resident), the padding columns of V
// (zeros) against zeros
__global__ void __launch_bounds__(CM_THREADS) cm_project_kernel(mbem_compressed_view v, const float* __restrict__ xs,
                                                                float* __restrict__ w) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t u = (int64_t)blockIdx.x * CM_WARPS + warp;
    if (u >= v.n_proj) return;
    const int64_t i = v.proj_block[u];
    const int k0 = v.proj_k0[u];
    const int nc3 = 3 * v.lr_nc[i], ldv = pad4(nc3), K = v.lr_rank[i];
    const float* xsrc = xs + 3 * (int64_t)v.lr_c0[i];
    const float* V = v.V + v.lr_v[i];
    const int n4 = ldv / 4;
    const int nk = min(4, K - k0);
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int q = lane; q < n4; q += 32) {
        const int c = 4 * q;
        const float b0 = xsrc[c], b1 = c + 1 < nc3 ? xsrc[c + 1] : 0.0f;
        const float b2 = c + 2 < nc3 ? xsrc[c + 2] : 0.0f, b3 = c + 3 < nc3 ? xsrc[c + 3] : 0.0f;
#pragma unroll
        for (int m = 0; m < 4; m++) {
            if (m < nk) {
                const float4 a = __ldg((const float4*)(V + (int64_t)(k0 + m) * ldv) + q);
                acc[m] += a.x * b0 + a.y * b1 + a.z * b2 + a.w * b3;
            }
        }
    }
#pragma unroll
    for (int m = 0; m < 4; m++) {
        float t = acc[m];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0 && m < nk) w[v.lr_w[i] + k0 + m] = t;
    }
}

// y rows of one strip. Every block of the strip is the same kind of item: K
// rows of a transposed factor (U^T of a low-rank block with its projection w,
// or D^T of a dense block with the gathered x) times K coefficients. Items are
// cut into units of at most CM_UNIT rows (the strip's unit list, in item
// order), and warps take the units round robin, so that the warps of a strip
// finish together. A lane owns rows lane + 32 m (m < CM_RPL) of the strip,
// sums a unit in FP32 (four factor rows of loads in flight) and adds it to FP64
// accumulators; the warps' sums are added in warp order, so every row has one
// writer and a fixed summation order. Strips of more than 32 CM_RPL rows are
// done in chunks of that many rows.
constexpr int CM_RPL = 9;                // rows a lane: 288 rows = a strip of 96 elements
constexpr int CM_STRIP_WARPS = 8;
__global__ void __launch_bounds__(CM_STRIP_WARPS * 32) cm_strip_kernel(mbem_compressed_view v,
                                                                       const float* __restrict__ xs,
                                                                       const float* __restrict__ w,
                                                                       double* __restrict__ y) {
    __shared__ double part[CM_STRIP_WARPS][32 * CM_RPL];
    const int64_t s = blockIdx.x;
    const int sr0 = v.strip_r0[s], R = 3 * v.strip_nr[s];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t u0 = v.unit_ptr[s], u1 = v.unit_ptr[s + 1];
    for (int rc = 0; rc < R; rc += 32 * CM_RPL) {
        const int Rc = min(32 * CM_RPL, R - rc);
        double acc[CM_RPL];
#pragma unroll
        for (int m = 0; m < CM_RPL; m++) acc[m] = 0.0;
        for (int64_t u = u0 + warp; u < u1; u += CM_STRIP_WARPS) {
            const int id = v.unit_item[u];
            const int k0 = v.unit_k0[u];
            const float* base;
            const float* cf;
            int K;
            int64_t ld;
            if (id < v.n_lr) {
                K = v.lr_rank[id];
                ld = pad4(3 * v.lr_nr[id]);
                base = v.U + v.lr_u[id] + 3 * (int64_t)(sr0 - v.lr_r0[id]) + rc;
                cf = w + v.lr_w[id];
            } else {
                const int d = id - (int)v.n_lr;
                K = 3 * v.d_nc[d];
                ld = pad4(3 * v.d_nr[d]);
                base = v.D + v.d_off[d] + 3 * (int64_t)(sr0 - v.d_r0[d]) + rc;
                cf = xs + 3 * (int64_t)v.d_c0[d];
            }
            const int k1 = min(K, k0 + CM_UNIT);
            float p[CM_RPL];
#pragma unroll
            for (int m = 0; m < CM_RPL; m++) p[m] = 0.0f;
            const float* row = base + lane;
            int k = k0;
            for (; k + 4 <= k1; k += 4) {
                float vv[4][CM_RPL];
#pragma unroll
                for (int j = 0; j < 4; j++)
#pragma unroll
                    for (int m = 0; m < CM_RPL; m++)
                        vv[j][m] = (lane + 32 * m < Rc) ? __ldg(row + (int64_t)(k + j) * ld + 32 * m) : 0.0f;
                const float c0 = cf[k], c1 = cf[k + 1], c2 = cf[k + 2], c3 = cf[k + 3];
#pragma unroll
                for (int m = 0; m < CM_RPL; m++) p[m] += ((vv[0][m] * c0 + vv[1][m] * c1) + (vv[2][m] * c2 + vv[3][m] * c3));
            }
            for (; k < k1; k++) {
                const float c = cf[k];
#pragma unroll
                for (int m = 0; m < CM_RPL; m++)
                    if (lane + 32 * m < Rc) p[m] += __ldg(row + (int64_t)k * ld + 32 * m) * c;
            }
#pragma unroll
            for (int m = 0; m < CM_RPL; m++) acc[m] += (double)p[m];
        }
#pragma unroll
        for (int m = 0; m < CM_RPL; m++) part[warp][lane + 32 * m] = acc[m];
        __syncthreads();
        for (int r = threadIdx.x; r < Rc; r += blockDim.x) {
            double t = 0.0;
            for (int ww = 0; ww < CM_STRIP_WARPS; ww++) t += part[ww][r];
            const int64_t p = sr0 + (rc + r) / 3;
            y[3 * v.field_order[p] + (rc + r) % 3] = t;
        }
        __syncthreads();
    }
}

// every block expanded into a dense FP64 matrix (original order)
__global__ void cm_dense_kernel(mbem_compressed_view v, double* __restrict__ out, int64_t ld) {
    const int64_t b = blockIdx.x;
    const bool lr = b < v.n_lr;
    const int64_t d = b - v.n_lr;
    const int r0 = lr ? v.lr_r0[b] : v.d_r0[d], nr = lr ? v.lr_nr[b] : v.d_nr[d];
    const int c0 = lr ? v.lr_c0[b] : v.d_c0[d], nc = lr ? v.lr_nc[b] : v.d_nc[d];
    const int ldu = pad4(3 * nr), ldc = pad4(3 * nc);
    for (int64_t q = threadIdx.x; q < (int64_t)9 * nr * nc; q += blockDim.x) {
        const int r = (int)(q / (3 * nc)), c = (int)(q - (int64_t)r * 3 * nc);
        double val = 0.0;
        if (lr) {
            const float* U = v.U + v.lr_u[b];
            const float* V = v.V + v.lr_v[b];
            for (int k = 0; k < v.lr_rank[b]; k++) val += (double)U[(int64_t)k * ldu + r] * (double)V[(int64_t)k * ldc + c];
        } else {
            val = v.D[v.d_off[d] + (int64_t)c * ldu + r];     // D^T
        }
        const int64_t row = 3 * v.field_order[r0 + r / 3] + r % 3;
        const int64_t col = 3 * v.src_order[c0 + c / 3] + c % 3;
        out[row * ld + col] = val;
    }
}

int check_geometry(const mbem_pair_geometry* g) {
    MBEM_REQUIRE(g && g->x_field && g->tri_verts && g->eps && g->prep, MBEM_ERR_ARG, "pair geometry: null pointer");
    MBEM_REQUIRE(g->kernel == 0 || g->kernel == 1, MBEM_ERR_ARG, "pair geometry: kernel must be 0 (T) or 1 (U)");
    MBEM_REQUIRE(g->kernel == 1 || g->normals, MBEM_ERR_ARG, "pair geometry: the T kernel needs normals");
    MBEM_REQUIRE(g->n_field >= 0 && g->n_src >= 0 && g->n_field < (1ll << 31) && g->n_src < (1ll << 31),
                 MBEM_ERR_SIZE, "pair geometry: sizes out of range");
    return MBEM_OK;
}

int set_smem(const void* fn, size_t bytes) {
    if (bytes <= 48 * 1024) return MBEM_OK;
    MBEM_REQUIRE(bytes <= 227 * 1024 - 1024, MBEM_ERR_SIZE, "shared memory %zu bytes beyond the limit", bytes);
    const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    MBEM_REQUIRE(e == cudaSuccess, MBEM_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
    return MBEM_OK;
}

}  // namespace
}  // namespace mbem

using namespace mbem;

extern "C" {

size_t mbem_pair_prep_bytes(int64_t n_field, int64_t n_src) {
    if (n_field < 0 || n_src < 0) return 0;
    return prep_layout(n_field, n_src).total;
}

int mbem_pair_prepare(const mbem_pair_geometry* g, void* stream) {
    const int rc = check_geometry(g);
    if (rc) return rc;
    const PrepLayout L = prep_layout(g->n_field, g->n_src);
    cudaStream_t st = (cudaStream_t)stream;
    char* p = (char*)g->prep;
    const cudaError_t e = cudaMemcpyAsync(p + L.c64, g->coeffs, 6 * sizeof(double), cudaMemcpyHostToDevice, st);
    MBEM_REQUIRE(e == cudaSuccess, MBEM_ERR_CUDA, "pair prepare: %s", cudaGetErrorString(e));
    const int64_t n = lmax(3 * g->n_field, g->n_src);
    if (n == 0) return MBEM_OK;
    const unsigned grid = (unsigned)lmin(ceil_div(n, 256), 4096);
    pair_prep_kernel<<<grid, 256, 0, st>>>(g->x_field, g->n_field, g->tri_verts, g->normals, g->eps, g->n_src,
                                           g->near_factor, g->kernel == 0, (F2*)(p + L.xf), (SrcFar*)(p + L.src));
    // the coefficient copy reads host memory: finish it before the caller may reuse it
    const cudaError_t e2 = cudaStreamSynchronize(st);
    MBEM_REQUIRE(e2 == cudaSuccess, MBEM_ERR_CUDA, "pair prepare: %s", cudaGetErrorString(e2));
    return launch_status("pair_prep_kernel");
}

int mbem_aca_compress(const mbem_pair_geometry* g, const mbem_aca_batch* b, void* stream) {
    int rc = check_geometry(g);
    if (rc) return rc;
    MBEM_REQUIRE(b && b->n_blocks >= 0, MBEM_ERR_ARG, "aca: bad batch");
    if (b->n_blocks == 0) return MBEM_OK;
    MBEM_REQUIRE(b->r0 && b->nr && b->c0 && b->nc && b->max_pivots && b->u_off && b->v_off && b->U && b->V &&
                     b->rank && b->status && b->err,
                 MBEM_ERR_ARG, "aca: null pointer");
    MBEM_REQUIRE(b->max_nr >= 1 && b->max_nc >= 1 && b->max_pivots_all >= 1 && b->max_nc <= 16384 &&
                     b->max_nr <= 16384,
                 MBEM_ERR_SIZE, "aca: batch maxima out of range");
    MBEM_REQUIRE(b->tol > 0.0, MBEM_ERR_ARG, "aca: tolerance must be positive");
    const size_t smem = aca_smem_bytes(b->max_nr, b->max_nc, b->max_pivots_all);
    AcaArgs a;
    a.r0 = b->r0;
    a.nr = b->nr;
    a.c0 = b->c0;
    a.nc = b->nc;
    a.cap = b->max_pivots;
    a.u_off = b->u_off;
    a.v_off = b->v_off;
    a.U = b->U;
    a.V = b->V;
    a.rank = b->rank;
    a.status = b->status;
    a.err = b->err;
    a.tol = b->tol;
    a.seed = b->seed;
    a.first_index = b->first_index;
    a.ldr = pad4(3 * b->max_nc);
    a.kcap = 3 * b->max_pivots_all;
    a.max_nr = b->max_nr;
    const Geo G = make_geo(g);
    cudaStream_t st = (cudaStream_t)stream;
    if (g->kernel == 0) {
        rc = set_smem((const void*)aca_kernel<true>, smem);
        if (rc) return rc;
        aca_kernel<true><<<(unsigned)b->n_blocks, ACA_THREADS, smem, st>>>(a, G, rules());
    } else {
        rc = set_smem((const void*)aca_kernel<false>, smem);
        if (rc) return rc;
        aca_kernel<false><<<(unsigned)b->n_blocks, ACA_THREADS, smem, st>>>(a, G, rules());
    }
    return launch_status("aca_kernel");
}

int mbem_aca_recompress(const mbem_pair_geometry* g, const mbem_aca_recompression* r, void* stream) {
    int rc = check_geometry(g);
    if (rc) return rc;
    MBEM_REQUIRE(r && r->n_blocks >= 0, MBEM_ERR_ARG, "recompress: bad arguments");
    if (r->n_blocks == 0) return MBEM_OK;
    MBEM_REQUIRE(r->r0 && r->nr && r->c0 && r->nc && r->rank && r->u_off && r->v_off && r->U && r->V && r->ur_off &&
                     r->vr_off && r->Ur && r->Vr && r->rank_out && r->err_out && r->index,
                 MBEM_ERR_ARG, "recompress: null pointer");
    MBEM_REQUIRE(r->max_rank >= 2 && r->max_rank <= RC_KMAX, MBEM_ERR_SIZE, "recompress: max_rank must be in [2, %d]",
                 RC_KMAX);
    MBEM_REQUIRE(r->tol > 0.0, MBEM_ERR_ARG, "recompress: tolerance must be positive");
    RcArgs a;
    a.r0 = r->r0;
    a.nr = r->nr;
    a.c0 = r->c0;
    a.nc = r->nc;
    a.rank = r->rank;
    a.u_off = r->u_off;
    a.v_off = r->v_off;
    a.U = r->U;
    a.V = r->V;
    a.ur_off = r->ur_off;
    a.vr_off = r->vr_off;
    a.Ur = r->Ur;
    a.Vr = r->Vr;
    a.rank_out = r->rank_out;
    a.err_out = r->err_out;
    a.index = r->index;
    a.tol = r->tol;
    a.seed = r->seed;
    a.kmax = r->max_rank;
    const size_t smem = rc_smem_bytes(r->max_rank);
    const Geo G = make_geo(g);
    cudaStream_t st = (cudaStream_t)stream;
    if (g->kernel == 0) {
        rc = set_smem((const void*)rc_kernel<true>, smem);
        if (rc) return rc;
        rc_kernel<true><<<(unsigned)r->n_blocks, ACA_THREADS, smem, st>>>(a, G, rules());
    } else {
        rc = set_smem((const void*)rc_kernel<false>, smem);
        if (rc) return rc;
        rc_kernel<false><<<(unsigned)r->n_blocks, ACA_THREADS, smem, st>>>(a, G, rules());
    }
    return launch_status("rc_kernel");
}

int mbem_aca_compact(int64_t n_blocks, const int32_t* nr, const int32_t* nc, const int32_t* rank,
                     const int64_t* u_src, const int64_t* v_src, const float* U_src, const float* V_src,
                     const int64_t* u_dst, const int64_t* v_dst, float* U_dst, float* V_dst, void* stream) {
    MBEM_REQUIRE(n_blocks >= 0, MBEM_ERR_ARG, "aca compact: bad block count");
    if (n_blocks == 0) return MBEM_OK;
    MBEM_REQUIRE(nr && nc && rank && u_src && v_src && U_src && V_src && u_dst && v_dst && U_dst && V_dst,
                 MBEM_ERR_ARG, "aca compact: null pointer");
    MBEM_REQUIRE(((uintptr_t)U_src | (uintptr_t)V_src | (uintptr_t)U_dst | (uintptr_t)V_dst) % 16 == 0,
                 MBEM_ERR_ARG, "aca compact: factor arrays must be 16-byte aligned");
    aca_compact_kernel<<<(unsigned)n_blocks, 256, 0, (cudaStream_t)stream>>>(nr, nc, rank, u_src, v_src, U_src,
                                                                           V_src, u_dst, v_dst, U_dst, V_dst);
    return launch_status("aca_compact_kernel");
}

int mbem_pair_dense_blocks(const mbem_pair_geometry* g, int64_t n_blocks, const int32_t* r0, const int32_t* nr,
                           const int32_t* c0, const int32_t* nc, const int64_t* d_off, const int64_t* col_ptr,
                           float* D, void* stream) {
    const int rc = check_geometry(g);
    if (rc) return rc;
    MBEM_REQUIRE(n_blocks >= 0, MBEM_ERR_ARG, "dense blocks: bad block count");
    if (n_blocks == 0) return MBEM_OK;
    MBEM_REQUIRE(r0 && nr && c0 && nc && d_off && col_ptr && D, MBEM_ERR_ARG, "dense blocks: null pointer");
    int64_t n_items = 0;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(&n_items, col_ptr + n_blocks, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    MBEM_REQUIRE(e == cudaSuccess, MBEM_ERR_CUDA, "dense blocks: %s", cudaGetErrorString(e));
    if (n_items == 0) return MBEM_OK;
    DenseArgs a;
    a.n_blocks = n_blocks;
    a.n_items = n_items;
    a.r0 = r0;
    a.nr = nr;
    a.c0 = c0;
    a.nc = nc;
    a.d_off = d_off;
    a.col_ptr = col_ptr;
    a.D = D;
    const Geo G = make_geo(g);
    const unsigned grid = (unsigned)ceil_div(n_items, 128);
    if (g->kernel == 0) pair_dense_kernel<true><<<grid, 128, 0, st>>>(a, G, rules());
    else pair_dense_kernel<false><<<grid, 128, 0, st>>>(a, G, rules());
    return launch_status("pair_dense_kernel");
}

size_t mbem_compressed_matvec_workspace_size(const mbem_compressed_view* v) {
    if (!v) return 0;
    return round256((size_t)(3 * v->n_src + 4) * sizeof(float)) + round256((size_t)v->n_w * sizeof(float));
}

int mbem_compressed_matvec(const mbem_compressed_view* v, const double* x, double* y, void* work,
                           size_t work_bytes, void* stream) {
    MBEM_REQUIRE(v && x && y && work, MBEM_ERR_ARG, "compressed matvec: null pointer");
    MBEM_REQUIRE(work_bytes >= mbem_compressed_matvec_workspace_size(v), MBEM_ERR_SIZE,
                 "compressed matvec: workspace too small");
    MBEM_REQUIRE(((uintptr_t)v->V % 16) == 0 || v->n_lr == 0, MBEM_ERR_ARG,
                 "compressed matvec: V must be 16-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    float* xs = (float*)work;
    float* w = (float*)((char*)work + round256((size_t)(3 * v->n_src + 4) * sizeof(float)));
    int n = 0;
    if (v->n_src > 0) {
        cm_gather_kernel<<<(unsigned)lmin(ceil_div(3 * v->n_src, 256), 8192), 256, 0, st>>>(x, v->src_order,
                                                                                          v->n_src, xs);
        n++;
    }
    if (v->n_proj > 0) {
        MBEM_REQUIRE(v->proj_block && v->proj_k0, MBEM_ERR_ARG, "compressed matvec: no projection units");
        cm_project_kernel<<<(unsigned)ceil_div(v->n_proj, CM_WARPS), CM_THREADS, 0, st>>>(*v, xs, w);
        n++;
    }
    if (v->n_strips > 0) {
        cm_strip_kernel<<<(unsigned)v->n_strips, CM_STRIP_WARPS * 32, 0, st>>>(*v, xs, w, y);
        n++;
    }
    return n ? launch_status("compressed_matvec", n) : MBEM_OK;
}

int mbem_compressed_to_dense(const mbem_compressed_view* v, double* out, int64_t ld, void* stream) {
    MBEM_REQUIRE(v && out && ld >= 3 * v->n_src, MBEM_ERR_ARG, "compressed to_dense: bad arguments");
    const int64_t nb = v->n_lr + v->n_dense;
    if (nb == 0) return MBEM_OK;
    cm_dense_kernel<<<(unsigned)nb, 256, 0, (cudaStream_t)stream>>>(*v, out, ld);
    return launch_status("cm_dense_kernel");
}

}  // extern "C"
