// Mixed-precision operator of the calibrated dense backend (sm_103a).
//
// A = A_far (FP32, dense) + A_near (FP64, 3x3 blocks in CSR by field point).
//
// Near pairs (source centroid within r_s = 3 max(eps_s, h_s) of the field
// point, or closer than 1.5 L_s) are the closed-form FP64 pair of
// p0_pair.cuh, exact to the reference. Far pairs are integrated in FP32 by
// collapsed Gauss-Legendre product rules (n x n points, n = 3..6 chosen by
// D / L) of the smooth mollified point kernel; at these distances the
// quadrature matches the FP64 closed form to ~1.5e-7 of the block (and is
// more accurate than the closed form beyond D/L ~ 40, where the
// divergence-theorem form cancels). The field-to-centroid offset is formed
// in double-float (hi/lo FP32 pairs with an error-free difference), so FP32
// keeps its relative accuracy at every distance; no FP64 instruction runs
// in the far kernel.
//
// The matvec reads the FP32 matrix once from HBM and accumulates each row in
// double-float (error-free products and sums on the FP32 pipes), so the
// operator is applied to ~1e-14 relative accuracy at the HBM roofline; the
// near blocks are applied in FP64.
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "dfloat.cuh"
#include "far_quad.cuh"
#include "p0_pair.cuh"
#include "tma_pipe.cuh"
#include "tune.cuh"

namespace mbem {

constexpr uint32_t TP_WAIT_LIMIT = 1u << 26;

// set by a bulk-copy wait that gave up (matvec ring or assembly tile); read
// (and cleared) by the host
__device__ int g_mixed_wait_error = 0;

// Nodal (P1/P2) far blocks: the moments of far_block weighted by the
// source's Lagrange shape functions at each quadrature point; node k's block
// follows far_block's formula with node k's moments. Barycentric coordinates
// of a point: l2 = a + 1/3, l3 = b + 1/3, l1 = 1 - l2 - l3 (tri_verts vertex
// order); nodes P1 v1 v2 v3, P2 v1 v2 v3 m12 m23 m31.
template <int ORDER>
__device__ __forceinline__ void far_shape(float a, float b, float* N) {
    const float l2 = a + (1.0f / 3.0f), l3 = b + (1.0f / 3.0f), l1 = 1.0f - l2 - l3;
    if (ORDER == 1) {
        N[0] = l1; N[1] = l2; N[2] = l3;
    } else {
        N[0] = l1 * (2.0f * l1 - 1.0f); N[1] = l2 * (2.0f * l2 - 1.0f); N[2] = l3 * (2.0f * l3 - 1.0f);
        N[3] = 4.0f * l1 * l2; N[4] = 4.0f * l2 * l3; N[5] = 4.0f * l3 * l1;
    }
}

template <bool TKERNEL, int ORDER>
__device__ __forceinline__ void far_block_nodal(const QuadRules& Q, const SrcFar& s, const float dc[3], float D2,
                                                const float c[6], float out[][3][3]) {
    constexpr int K = ORDER == 1 ? 3 : 6;
    // the shape functions raise the integrand's degree: ORDER more points a
    // direction than the P0 rule at the same D / L
    const int nq = min(far_rule_collapsed(D2, s.L2) + ORDER, QR_MAX);
    const int q0 = Q.off[nq], q1 = q0 + nq * nq;
    float V3[K][3], V5[K][3], t[K][3], W[K][6], I1[K], I3[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        I1[k] = I3[k] = 0.0f;
#pragma unroll
        for (int i = 0; i < 3; i++) V3[k][i] = V5[k][i] = t[k][i] = 0.0f;
#pragma unroll
        for (int i = 0; i < 6; i++) W[k][i] = 0.0f;
    }
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
        float N[K];
        far_shape<ORDER>(a, b, N);
        if (TKERNEL) {
            const float w5 = w3 * iR2;
            const float wt = w5 * r2;
            const float wn = w5 * (dx * s.n[0] + dy * s.n[1] + dz * s.n[2]);
            const float ux = wn * dx, uy = wn * dy, uz = wn * dz;
            const float base[15] = {w3 * dx, w3 * dy, w3 * dz, w5 * dx, w5 * dy, w5 * dz, wt * dx, wt * dy, wt * dz,
                                    ux * dx, ux * dy, ux * dz, uy * dy, uy * dz, uz * dz};
#pragma unroll
            for (int k = 0; k < K; k++) {
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    V3[k][i] = fmaf(N[k], base[i], V3[k][i]);
                    V5[k][i] = fmaf(N[k], base[3 + i], V5[k][i]);
                    t[k][i] = fmaf(N[k], base[6 + i], t[k][i]);
                }
#pragma unroll
                for (int i = 0; i < 6; i++) W[k][i] = fmaf(N[k], base[9 + i], W[k][i]);
            }
        } else {
            const float ux = w3 * dx, uy = w3 * dy, uz = w3 * dz;
            const float base[8] = {w * iR, w3, ux * dx, ux * dy, ux * dz, uy * dy, uy * dz, uz * dz};
#pragma unroll
            for (int k = 0; k < K; k++) {
                I1[k] = fmaf(N[k], base[0], I1[k]);
                I3[k] = fmaf(N[k], base[1], I3[k]);
#pragma unroll
                for (int i = 0; i < 6; i++) W[k][i] = fmaf(N[k], base[2 + i], W[k][i]);
            }
        }
    }
    const float A = s.area2;
#pragma unroll
    for (int k = 0; k < K; k++) {
        const float Wk[3][3] = {{W[k][0], W[k][1], W[k][2]}, {W[k][1], W[k][3], W[k][4]}, {W[k][2], W[k][4], W[k][5]}};
        if (TKERNEL) {
            const float* n = s.n;
            const float nV3 = n[0] * V3[k][0] + n[1] * V3[k][1] + n[2] * V3[k][2];
            const float nV5 = n[0] * V5[k][0] + n[1] * V5[k][1] + n[2] * V5[k][2];
            const float ca = c[0] + 4.0f * c[1] + 2.0f * c[4];
            const float cb = c[3] + c[4];
            const float ce3 = c[2] * s.eps2, ce6 = c[5] * s.eps2;
            const float gam = cb * nV3 + ce6 * nV5;
#pragma unroll
            for (int i = 0; i < 3; i++) {
                const float al = ca * V3[k][i] - 3.0f * c[1] * t[k][i] + ce3 * V5[k][i];
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    const float be = cb * V3[k][j] + ce6 * V5[k][j];
                    out[k][i][j] = A * (n[j] * al + n[i] * be - 6.0f * c[4] * Wk[i][j] + (i == j ? gam : 0.0f));
                }
            }
        } else {
            const float dg = c[0] * I1[k] + c[1] * s.eps2 * I3[k];
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++) out[k][i][j] = A * (c[2] * Wk[i][j] + (i == j ? dg : 0.0f));
        }
    }
}

// ---------------------------------------------------------------------------
// far assembly: one thread per source, FIELD_TILE field points per block
// ---------------------------------------------------------------------------
constexpr int FAR_THREADS = 128;
constexpr int FAR_FIELD_TILE = 64;

struct FarArgs {
    const double* x_field;
    int64_t n_field;
    const double* tri_verts;
    const double* normals;
    const double* eps;
    int64_t n_src;
    float c[6];
    float alpha;
    double near_factor;
    float* out;
    int64_t ld;
    uint32_t* near_mask;   // optional (n_field, ceil(n_src/32)) bit mask of near pairs
    uint16_t* out16;       // optional BF16 copy of out (round to nearest even)
    int64_t ld16;
};

template <bool TKERNEL, int ORDER>
__global__ void __launch_bounds__(FAR_THREADS)
far_assemble_kernel(FarArgs a, QuadRules Q) {
    constexpr int K = ORDER == 0 ? 1 : (ORDER == 1 ? 3 : 6);
    constexpr uint32_t TILE_BYTES = FAR_FIELD_TILE * 3 * sizeof(double);
    __shared__ F2 xs[FAR_FIELD_TILE][3];
    // the field tile arrives by one bulk copy (cp.async.bulk) while the
    // threads set up their sources; a ragged last tile or an unaligned base
    // falls back to plain loads
    __shared__ __align__(16) double xraw[FAR_FIELD_TILE * 3];
    __shared__ __align__(8) uint64_t tbar;
    const int64_t s = (int64_t)blockIdx.x * FAR_THREADS + threadIdx.x;
    const bool active = s < a.n_src;
    const int64_t n_words = ceil_div(a.n_src, 32);
    bool bulk_ok = ((uintptr_t)a.x_field % 16) == 0;
    if (threadIdx.x == 0) {
        mbar_init(&tbar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    uint32_t phase = 0;
    bool in_flight = false;
    auto issue = [&](int64_t t0) -> bool {
        if (!bulk_ok || t0 + FAR_FIELD_TILE > a.n_field) return false;
        if (threadIdx.x == 0) {
            mbar_arrive_expect_tx(&tbar, TILE_BYTES);
            bulk_g2s(xraw, a.x_field + 3 * t0, TILE_BYTES, &tbar);
        }
        return true;
    };
    const int64_t first = (int64_t)blockIdx.y * FAR_FIELD_TILE;
    bool pending = first < a.n_field && issue(first);
    in_flight = pending;
    SrcFar src;
    if (active) {
        far_setup(a.tri_verts + 9 * s, TKERNEL ? a.normals + 3 * s : nullptr, a.eps[s], a.near_factor, src);
    } else {
        // inactive lanes still vote in the near-mask ballot; they never count as near
        for (int k = 0; k < 3; k++) {
            src.c[k].hi = src.c[k].lo = 0.0f;
            src.e1[k] = src.e2[k] = src.n[k] = 0.0f;
        }
        src.area2 = src.eps2 = src.L2 = 1.0f;
        src.rnear2 = -1.0f;
        src.ok = false;
    }
    for (int64_t f0 = first; f0 < a.n_field; f0 += (int64_t)gridDim.y * FAR_FIELD_TILE) {
        __syncthreads();
        const bool bulk = (f0 == first) ? pending : issue(f0);
        bool got = false;
        if (bulk) {
            if (mbar_wait(&tbar, phase, TP_WAIT_LIMIT)) {
                got = true;
                in_flight = false;
            } else {
                atomicExch(&g_mixed_wait_error, 1);
                bulk_ok = false;                  // plain loads from here on
            }
            phase ^= 1u;
        }
        for (int t = threadIdx.x; t < FAR_FIELD_TILE * 3; t += FAR_THREADS) {
            const int64_t f = f0 + t / 3;
            xs[t / 3][t % 3] = split_d(got ? xraw[t] : (f < a.n_field ? a.x_field[3 * f0 + t] : 0.0));
        }
        __syncthreads();
        const int nf = (int)lmin(FAR_FIELD_TILE, a.n_field - f0);
        // blocks of field point f into the FP32 matrix (and its BF16 copy)
        auto store = [&](int64_t f, const float (*blk)[3][3]) {
            // columns 3 (K s + k) + j
#pragma unroll
            for (int i = 0; i < 3; i++) {
                float* row = a.out + (3 * f + i) * a.ld + 3 * K * s;
#pragma unroll
                for (int k = 0; k < K; k++)
#pragma unroll
                    for (int j = 0; j < 3; j++) row[3 * k + j] = a.alpha * blk[k][i][j];
            }
            if (a.out16) {
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    uint16_t* row = a.out16 + (3 * f + i) * a.ld16 + 3 * K * s;
#pragma unroll
                    for (int k = 0; k < K; k++)
#pragma unroll
                        for (int j = 0; j < 3; j++)
                            row[3 * k + j] = __bfloat16_as_ushort(__float2bfloat16_rn(a.alpha * blk[k][i][j]));
                }
            }
        };
        auto mask = [&](int64_t f, bool near) {
            if (a.near_mask) {
                const unsigned m = __ballot_sync(0xffffffffu, near);
                // lane 0 of a warp with at least one source writes its word
                if ((threadIdx.x & 31) == 0 && (s >> 5) < n_words) a.near_mask[f * n_words + (s >> 5)] = m;
            }
        };
        // P0: field points two at a time in packed FP32 when both are far
        for (int ff = 0; ff < nf; ff += (ORDER == 0 ? 2 : 1)) {
            const int64_t f = f0 + ff;
            const bool two = ORDER == 0 && ff + 1 < nf;
            float d[3], D2, d2[3], D2b = 0.0f;
            float blk[K][3][3], blk2[K][3][3];
            const bool near = is_near(xs[ff], src, d, D2) && active;
            const bool near2 = two && is_near(xs[ff + 1], src, d2, D2b) && active;
            mask(f, near);
            if (two) mask(f + 1, near2);
            if (!active) continue;
            const bool pair = two && src.ok && !near && !near2;
            if (pair) {
                far_block2<TKERNEL>(Q, src, d, d2, D2, D2b, a.c, blk[0], blk2[0]);
            } else if (near || !src.ok) {
#pragma unroll
                for (int k = 0; k < K; k++)
#pragma unroll
                    for (int i = 0; i < 3; i++)
#pragma unroll
                        for (int j = 0; j < 3; j++) blk[k][i][j] = 0.0f;
            } else if (ORDER == 0) {
                far_block<TKERNEL>(Q, src, d, D2, a.c, blk[0]);
            } else {
                far_block_nodal<TKERNEL, ORDER>(Q, src, d, D2, a.c, blk);
            }
            store(f, blk);
            if (two) {
                if (!pair) {
                    if (near2 || !src.ok) {
#pragma unroll
                        for (int k = 0; k < K; k++)
#pragma unroll
                            for (int i = 0; i < 3; i++)
#pragma unroll
                                for (int j = 0; j < 3; j++) blk2[k][i][j] = 0.0f;
                    } else {
                        far_block<TKERNEL>(Q, src, d2, D2b, a.c, blk2[0]);
                    }
                }
                store(f + 1, blk2);
            }
        }
    }
    // a copy whose wait ran out must land before the block's shared memory goes
    if (in_flight && threadIdx.x == 0) mbar_wait(&tbar, phase ^ 1u, TP_WAIT_LIMIT);
}

// ---------------------------------------------------------------------------
// near list: count per field point, scan, fill (deterministic source order)
// ---------------------------------------------------------------------------
constexpr int NL_THREADS = 128;
constexpr int NL_SRC_TILE = 128;

struct NearArgs {
    const double* x_field;
    int64_t n_field;
    const double* tri_verts;
    const double* eps;
    int64_t n_src;
    double near_factor;
    int64_t* counts;       // (n_field,) or rowptr (n_field + 1)
    int64_t* cols;         // fill pass only
};

template <bool FILL>
__global__ void __launch_bounds__(NL_THREADS)
near_list_kernel(NearArgs a) {
    __shared__ SrcFar tile[NL_SRC_TILE];
    const int64_t f = (int64_t)blockIdx.x * NL_THREADS + threadIdx.x;
    const bool active = f < a.n_field;
    F2 x[3];
    for (int k = 0; k < 3; k++) x[k] = split_d(active ? a.x_field[3 * f + k] : 0.0);
    int64_t cnt = 0;
    int64_t pos = (FILL && active) ? a.counts[f] : 0;
    for (int64_t s0 = 0; s0 < a.n_src; s0 += NL_SRC_TILE) {
        __syncthreads();
        for (int t = threadIdx.x; t < NL_SRC_TILE; t += NL_THREADS) {
            const int64_t s = s0 + t;
            if (s < a.n_src) far_setup(a.tri_verts + 9 * s, nullptr, a.eps[s], a.near_factor, tile[t]);
        }
        __syncthreads();
        if (!active) continue;
        const int ns = (int)lmin(NL_SRC_TILE, a.n_src - s0);
        for (int t = 0; t < ns; t++) {
            float d[3], D2;
            if (is_near(x, tile[t], d, D2)) {
                if (FILL) a.cols[pos++] = s0 + t;
                else cnt++;
            }
        }
    }
    if (!FILL && active) a.counts[f] = cnt;
}

// exclusive scan of n counts into rowptr[0..n] (one block, fixed order)
__global__ void scan_kernel(const int64_t* __restrict__ counts, int64_t n, int64_t* __restrict__ rowptr) {
    __shared__ int64_t part[1024];
    const int t = threadIdx.x;
    const int64_t chunk = (n + blockDim.x - 1) / blockDim.x;
    const int64_t b0 = t * chunk, b1 = lmin(n, b0 + chunk);
    int64_t s = 0;
    for (int64_t i = b0; i < b1; i++) s += counts[i];
    part[t] = s;
    __syncthreads();
    if (t == 0) {
        int64_t run = 0;
        for (int i = 0; i < (int)blockDim.x; i++) {
            const int64_t v = part[i];
            part[i] = run;
            run += v;
        }
    }
    __syncthreads();
    int64_t run = part[t];
    for (int64_t i = b0; i < b1; i++) {
        rowptr[i] = run;
        run += counts[i];
    }
    if (b1 == n && b0 < b1) rowptr[n] = run;
    if (n == 0 && t == 0) rowptr[0] = 0;
}

// near list from the far kernel's bit mask: one warp per field point
__global__ void mask_count_kernel(const uint32_t* __restrict__ mask, int64_t n_field, int64_t n_words,
                                  int64_t* __restrict__ counts) {
    const int64_t f = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (f >= n_field) return;
    int64_t c = 0;
    for (int64_t w = lane; w < n_words; w += 32) c += __popc(mask[f * n_words + w]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) counts[f] = c;
}

__global__ void mask_fill_kernel(const uint32_t* __restrict__ mask, int64_t n_field, int64_t n_words,
                                 const int64_t* __restrict__ rowptr, int64_t* __restrict__ cols) {
    const int64_t f = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (f >= n_field) return;
    int64_t pos = rowptr[f];
    for (int64_t w0 = 0; w0 < n_words; w0 += 32) {
        const int64_t w = w0 + lane;
        uint32_t m = (w < n_words) ? mask[f * n_words + w] : 0u;
        const int c = __popc(m);
        int incl = c;   // inclusive warp scan of the counts (lane order = source order)
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        int64_t p = pos + (incl - c);
        while (m) {
            const int b = __ffs(m) - 1;
            cols[p++] = 32 * w + b;
            m &= m - 1;
        }
        pos += __shfl_sync(0xffffffffu, incl, 31);
    }
}

// near T/U blocks in FP64 (closed form), one thread per near pair
struct NearEvalArgs {
    const double* x_field;
    int64_t n_field;
    const double* tri_verts;
    const double* normals;
    const double* eps;
    const int64_t* rowptr;
    const int64_t* cols;
    int64_t nnz;
    double c[6];
    double alpha;
    double* vals;          // (nnz, 3, 3)
};

template <bool TKERNEL>
__global__ void __launch_bounds__(128)
near_eval_kernel(NearEvalArgs a) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.nnz) return;
    // field point of pair k: binary search in rowptr
    int64_t lo = 0, hi = a.n_field;
    while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (a.rowptr[mid] <= k) lo = mid;
        else hi = mid;
    }
    const int64_t f = lo, s = a.cols[k];
    SrcP0 src;
    src_setup(a.tri_verts + 9 * s, a.eps[s], src);
    double blk[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    if (src.ok) {
        PairP0 p;
        pair_setup(src, a.x_field[3 * f], a.x_field[3 * f + 1], a.x_field[3 * f + 2], p);
        if (TKERNEL) {
            const double* nrm = a.normals + 3 * s;
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
                    blk[i][j] = a.c[2] * m.T2[i][j] + (i == j ? a.c[0] * m.I1 + a.c[1] * src.eps2 * m.I3 : 0.0);
        }
    }
    double* v = a.vals + 9 * k;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) v[3 * i + j] = a.alpha * blk[i][j];
}

// near blocks: calibration row sums out[f, i, j] += sum_k vals[k, i, j]
__global__ void near_rowsum_kernel(const int64_t* __restrict__ rowptr, const double* __restrict__ vals,
                                   int64_t n_field, double* __restrict__ out) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_field) return;
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t k = rowptr[f]; k < rowptr[f + 1]; k++)
#pragma unroll
        for (int q = 0; q < 9; q++) acc[q] += vals[9 * k + q];
#pragma unroll
    for (int q = 0; q < 9; q++) out[9 * f + q] += acc[q];
}

// add D[c] to the diagonal (self) block of row c, shape weights at P0 = 1
struct ShapeKxK {
    double w[36];
};

__global__ void near_add_diag_kernel(const int64_t* __restrict__ rowptr, const int64_t* __restrict__ cols,
                                     double* __restrict__ vals, int64_t n_field, const double* __restrict__ D,
                                     int* __restrict__ missing) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_field) return;
    for (int64_t k = rowptr[f]; k < rowptr[f + 1]; k++) {
        if (cols[k] == f) {
#pragma unroll
            for (int q = 0; q < 9; q++) vals[9 * k + q] += D[9 * f + q];
            return;
        }
    }
    atomicAdd(missing, 1);
}

// the calibrated diagonal of collocation point c spread over its element's
// K nodes by the collocation shape: vals of (c, node K s + k) += shape[kc][k] D_c
__global__ void near_add_diag_nodal_kernel(const int64_t* __restrict__ rowptr, const int64_t* __restrict__ cols,
                                           double* __restrict__ vals, int64_t n_field, const double* __restrict__ D,
                                           int K, ShapeKxK shape, int* __restrict__ missing) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_field) return;
    const int64_t s = c / K;
    const int kc = (int)(c % K);
    for (int k = 0; k < K; k++) {
        const double w = shape.w[kc * K + k];
        if (w == 0.0) continue;
        const int64_t node = K * s + k;
        bool found = false;
        for (int64_t q = rowptr[c]; q < rowptr[c + 1]; q++) {
            if (cols[q] == node) {
#pragma unroll
                for (int e = 0; e < 9; e++) vals[9 * q + e] += w * D[9 * c + e];
                found = true;
                break;
            }
        }
        if (!found) atomicAdd(missing, 1);
    }
}

// TwoSum of v into (h, l)
__device__ __forceinline__ void ts_add(float& h, float& l, float v) {
    const float s = __fadd_rn(h, v);
    const float bb = __fsub_rn(s, h);
    l = __fadd_rn(l, __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(v, bb)));
    h = s;
}

// FP32 row sums with double-float accumulation: out[r, j] (+)= sum_c A[r, 3c+j]
__global__ void rowsum3_f32_kernel(const float* __restrict__ A, int64_t ld, int64_t n_rows, int64_t n_cols,
                                   double alpha, int accumulate, double* __restrict__ out) {
    const int64_t r = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (r >= n_rows) return;
    const float* row = A + r * ld;
    // four independent (hi, lo) accumulators per component; a lane reads 12
    // consecutive columns (3 float4) at a time, so element e of the chunk
    // always belongs to component e % 3 and every index is static
    float hi[4][3], lo[4][3];
#pragma unroll
    for (int t = 0; t < 4; t++)
#pragma unroll
        for (int k = 0; k < 3; k++) hi[t][k] = lo[t][k] = 0.0f;
    int64_t c_start = 0;
    if ((reinterpret_cast<uintptr_t>(row) & 15) == 0) {
        const int64_t n12 = n_cols / 12;
        const float4* r4 = reinterpret_cast<const float4*>(row);
        for (int64_t q = lane; q < n12; q += 32) {
            const float4 a = __ldcs(r4 + 3 * q), b = __ldcs(r4 + 3 * q + 1), c = __ldcs(r4 + 3 * q + 2);
            ts_add(hi[0][0], lo[0][0], a.x); ts_add(hi[0][1], lo[0][1], a.y); ts_add(hi[0][2], lo[0][2], a.z);
            ts_add(hi[1][0], lo[1][0], a.w); ts_add(hi[1][1], lo[1][1], b.x); ts_add(hi[1][2], lo[1][2], b.y);
            ts_add(hi[2][0], lo[2][0], b.z); ts_add(hi[2][1], lo[2][1], b.w); ts_add(hi[2][2], lo[2][2], c.x);
            ts_add(hi[3][0], lo[3][0], c.y); ts_add(hi[3][1], lo[3][1], c.z); ts_add(hi[3][2], lo[3][2], c.w);
        }
        c_start = 12 * n12;
    }
    for (int64_t c = c_start + lane; c < n_cols; c += 32) {
        const float v = row[c];
        const int k = (int)(c % 3);
        if (k == 0) ts_add(hi[0][0], lo[0][0], v);
        else if (k == 1) ts_add(hi[0][1], lo[0][1], v);
        else ts_add(hi[0][2], lo[0][2], v);
    }
    double acc[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        acc[k] = 0.0;
#pragma unroll
        for (int t = 0; t < 4; t++) acc[k] += (double)hi[t][k] + (double)lo[t][k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
    }
    if (lane == 0)
        for (int k = 0; k < 3; k++) {
            const double v = alpha * acc[k];
            out[3 * r + k] = accumulate ? out[3 * r + k] + v : v;
        }
}

// ---------------------------------------------------------------------------
// mixed matvec: y = alpha * (A32 x + sum of near blocks x) + beta * y
// ---------------------------------------------------------------------------
__global__ void split_vec_kernel(const double* __restrict__ x, int64_t n, float* __restrict__ xh,
                                 float* __restrict__ xl) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const F2 v = split_d(x[i]);
    xh[i] = v.hi;
    xl[i] = v.lo;
}

constexpr int SGEMV_ROWS = 4;
constexpr int SGEMV_UNROLL = 2;
constexpr int SGEMV_THREADS = 256;

__global__ void __launch_bounds__(SGEMV_THREADS)
sgemv_df_kernel(const float* __restrict__ A, int64_t ld, int64_t n_rows, int64_t n_cols,
                const float* __restrict__ xh, const float* __restrict__ xl, double* __restrict__ y) {
    const int64_t warp = (int64_t)blockIdx.x * (SGEMV_THREADS / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    const int64_t r0 = warp * SGEMV_ROWS;
    if (r0 >= n_rows) return;
    const int nr = (int)lmin(SGEMV_ROWS, n_rows - r0);
    // four independent double-float accumulators per row (one per float4
    // lane): the TwoSum chain, not HBM, bounds a single accumulator
    float sh[SGEMV_ROWS][4], sl[SGEMV_ROWS][4];
#pragma unroll
    for (int i = 0; i < SGEMV_ROWS; i++)
#pragma unroll
        for (int k = 0; k < 4; k++) sh[i][k] = sl[i][k] = 0.0f;
    const int64_t n4 = n_cols / 4;
    const float4* xh4 = reinterpret_cast<const float4*>(xh);
    const float4* xl4 = reinterpret_cast<const float4*>(xl);
    const float4* rows[SGEMV_ROWS];
#pragma unroll
    for (int i = 0; i < SGEMV_ROWS; i++) rows[i] = reinterpret_cast<const float4*>(A + (r0 + min(i, nr - 1)) * ld);
    // full chunks: SGEMV_UNROLL x SGEMV_ROWS independent 16-byte loads per lane
    const int64_t full = (n4 / (32 * SGEMV_UNROLL)) * (32 * SGEMV_UNROLL);
    for (int64_t c0 = lane; c0 < full; c0 += 32 * SGEMV_UNROLL) {
        float4 v[SGEMV_UNROLL][SGEMV_ROWS], h[SGEMV_UNROLL], l[SGEMV_UNROLL];
#pragma unroll
        for (int u = 0; u < SGEMV_UNROLL; u++) {
            const int64_t c = c0 + 32 * u;
            h[u] = __ldg(xh4 + c);
            l[u] = __ldg(xl4 + c);
#pragma unroll
            for (int i = 0; i < SGEMV_ROWS; i++) v[u][i] = __ldcs(rows[i] + c);
        }
#pragma unroll
        for (int u = 0; u < SGEMV_UNROLL; u++)
#pragma unroll
            for (int i = 0; i < SGEMV_ROWS; i++) {
                df_acc(sh[i][0], sl[i][0], v[u][i].x, h[u].x, l[u].x);
                df_acc(sh[i][1], sl[i][1], v[u][i].y, h[u].y, l[u].y);
                df_acc(sh[i][2], sl[i][2], v[u][i].z, h[u].z, l[u].z);
                df_acc(sh[i][3], sl[i][3], v[u][i].w, h[u].w, l[u].w);
            }
    }
    for (int64_t c = full + lane; c < n4; c += 32) {
        const float4 h = __ldg(xh4 + c), l = __ldg(xl4 + c);
#pragma unroll
        for (int i = 0; i < SGEMV_ROWS; i++) {
            const float4 v = __ldcs(rows[i] + c);
            df_acc(sh[i][0], sl[i][0], v.x, h.x, l.x);
            df_acc(sh[i][1], sl[i][1], v.y, h.y, l.y);
            df_acc(sh[i][2], sl[i][2], v.z, h.z, l.z);
            df_acc(sh[i][3], sl[i][3], v.w, h.w, l.w);
        }
    }
    for (int64_t c = 4 * n4 + lane; c < n_cols; c += 32) {
#pragma unroll
        for (int i = 0; i < SGEMV_ROWS; i++)
            df_acc(sh[i][0], sl[i][0], A[(r0 + min(i, nr - 1)) * ld + c], xh[c], xl[c]);
    }
    double acc[SGEMV_ROWS];
#pragma unroll
    for (int i = 0; i < SGEMV_ROWS; i++) {
        acc[i] = ((double)sh[i][0] + (double)sl[i][0]) + ((double)sh[i][1] + (double)sl[i][1]) +
                 ((double)sh[i][2] + (double)sl[i][2]) + ((double)sh[i][3] + (double)sl[i][3]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
    }
    if (lane < nr) {
        double v = acc[0];
#pragma unroll
        for (int i = 1; i < SGEMV_ROWS; i++)
            if (lane == i) v = acc[i];
        y[r0 + lane] = v;
    }
}

// y[3f + i] += sum_k vals[k, i, j] x[3 cols[k] + j]: one warp per row block,
// lanes over its near blocks, fixed-order warp reduction. A set *stop (a
// Krylov step enqueued after its basis ended) makes it return at once.
__global__ void near_matvec_kernel(const int64_t* __restrict__ rowptr, const int64_t* __restrict__ cols,
                                   const double* __restrict__ vals, int64_t n_field, const double* __restrict__ x,
                                   double* __restrict__ y, const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int64_t f = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (f >= n_field) return;
    double a0 = 0, a1 = 0, a2 = 0;
    const int64_t k1 = rowptr[f + 1];
    for (int64_t k = rowptr[f] + lane; k < k1; k += 32) {
        const int64_t s = cols[k];
        const double x0 = x[3 * s], x1 = x[3 * s + 1], x2 = x[3 * s + 2];
        const double* v = vals + 9 * k;
        a0 += v[0] * x0 + v[1] * x1 + v[2] * x2;
        a1 += v[3] * x0 + v[4] * x1 + v[5] * x2;
        a2 += v[6] * x0 + v[7] * x1 + v[8] * x2;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (lane == 0) {
        y[3 * f] += a0;
        y[3 * f + 1] += a1;
        y[3 * f + 2] += a2;
    }
}

// ---------------------------------------------------------------------------
// The same product as a warp-specialised bulk-copy pipeline: one producer
// warp streams TP_ROWS row chunks of A and the matching chunk of x (hi, lo)
// into a TP_STAGES-deep shared-memory ring with cp.async.bulk, completing on
// per-stage mbarriers; TP_WARPS consumer warps (two rows each, so every x
// value read from shared memory serves two rows) accumulate in double-float.
// The ring keeps ~216 KB per SM in flight independent of register pressure.
// ---------------------------------------------------------------------------
// Tile shape (template): TP_ROWS rows per CTA, TP_CH columns per chunk,
// TP_STAGES ring stages; the tuned choice is in tune.cuh.
template <int R, int CH, int S>
constexpr size_t tp_smem() { return (size_t)S * (R + 2) * CH * sizeof(float) + 2 * S * 8; }


template <int TP_ROWS, int TP_CH, int TP_STAGES>
__global__ void __launch_bounds__(32 * (TP_ROWS / 2 + 1))
sgemv_df_tma_kernel(const float* __restrict__ A, int64_t ld, int64_t n_rows, int64_t n_main, int64_t n_cols,
                    const float* __restrict__ xh, const float* __restrict__ xl, double* __restrict__ y) {
    constexpr int TP_WARPS = TP_ROWS / 2;
    extern __shared__ __align__(128) unsigned char smem[];
    float* sA = reinterpret_cast<float*>(smem);                     // [S][ROWS][CH]
    float* sX = sA + TP_STAGES * TP_ROWS * TP_CH;                   // [S][2][CH]
    uint64_t* full = reinterpret_cast<uint64_t*>(sX + TP_STAGES * 2 * TP_CH);
    uint64_t* empty = full + TP_STAGES;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t r0 = (int64_t)blockIdx.x * TP_ROWS;
    const int nrow = (int)lmin(TP_ROWS, n_rows - r0);
    const int64_t nchunks = ceil_div(n_main, TP_CH);
    if (threadIdx.x == 0) {
        for (int s = 0; s < TP_STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], TP_WARPS);
        }
        mbar_init_fence();
    }
    __syncthreads();

    if (warp == TP_WARPS) {
        // producer warp: lane 0 waits for the stage to drain and posts the
        // byte count; the lanes then issue the nrow + 2 copies in parallel
        int64_t issued = 0;
        for (int64_t k = 0; k < nchunks; k++) {
            const int s = (int)(k % TP_STAGES);
            int ok = 1;
            if (lane == 0) {
                if (k >= TP_STAGES && !mbar_wait(&empty[s], (uint32_t)(((k / TP_STAGES) - 1) & 1), TP_WAIT_LIMIT)) {
                    atomicExch(&g_mixed_wait_error, 1);
                    ok = 0;
                }
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) break;
            const int64_t c0 = k * TP_CH;
            const uint32_t bytes = (uint32_t)lmin(TP_CH, n_main - c0) * 4u;
            if (lane == 0) mbar_arrive_expect_tx(&full[s], bytes * (uint32_t)(nrow + 2));
            __syncwarp();
            for (int t = lane; t < TP_ROWS + 2; t += 32) {
                if (t < nrow)
                    bulk_g2s(sA + ((int64_t)s * TP_ROWS + t) * TP_CH, A + (r0 + t) * ld + c0, bytes, &full[s]);
                else if (t == TP_ROWS)
                    bulk_g2s(sX + (int64_t)s * 2 * TP_CH, xh + c0, bytes, &full[s]);
                else if (t == TP_ROWS + 1)
                    bulk_g2s(sX + ((int64_t)s * 2 + 1) * TP_CH, xl + c0, bytes, &full[s]);
            }
            issued = k + 1;
        }
        // do not leave the block while copies into its shared memory are in flight
        if (lane == 0)
            for (int64_t k = (issued > TP_STAGES ? issued - TP_STAGES : 0); k < issued; k++)
                if (!mbar_wait(&full[k % TP_STAGES], (uint32_t)((k / TP_STAGES) & 1), TP_WAIT_LIMIT))
                    atomicExch(&g_mixed_wait_error, 1);
        return;
    }

    // consumers: warp w owns rows r0 + 2w and r0 + 2w + 1; four double-float
    // chains per row (one per float4 component)
    const int ra = 2 * warp, rb = 2 * warp + 1;
    const bool va = ra < nrow, vb = rb < nrow;
    const int rb_eff = vb ? rb : ra;          // an invalid second row re-reads the first
    float ah[4], al[4], bh[4], bl[4];
#pragma unroll
    for (int t = 0; t < 4; t++) ah[t] = al[t] = bh[t] = bl[t] = 0.0f;
    for (int64_t k = 0; k < nchunks; k++) {
        const int s = (int)(k % TP_STAGES);
        if (!mbar_wait(&full[s], (uint32_t)((k / TP_STAGES) & 1), TP_WAIT_LIMIT)) {
            atomicExch(&g_mixed_wait_error, 1);
            break;
        }
        if (va) {
            const int w4 = (int)(lmin(TP_CH, n_main - k * TP_CH) / 4);
            const float4* pa = reinterpret_cast<const float4*>(sA + ((int64_t)s * TP_ROWS + ra) * TP_CH);
            const float4* pb = reinterpret_cast<const float4*>(sA + ((int64_t)s * TP_ROWS + rb_eff) * TP_CH);
            const float4* h4 = reinterpret_cast<const float4*>(sX + (int64_t)s * 2 * TP_CH);
            const float4* l4 = reinterpret_cast<const float4*>(sX + ((int64_t)s * 2 + 1) * TP_CH);
#pragma unroll 2
            for (int q = lane; q < w4; q += 32) {
                const float4 h = h4[q], l = l4[q], a = pa[q], b = pb[q];
                df_acc(ah[0], al[0], a.x, h.x, l.x);
                df_acc(ah[1], al[1], a.y, h.y, l.y);
                df_acc(ah[2], al[2], a.z, h.z, l.z);
                df_acc(ah[3], al[3], a.w, h.w, l.w);
                df_acc(bh[0], bl[0], b.x, h.x, l.x);
                df_acc(bh[1], bl[1], b.y, h.y, l.y);
                df_acc(bh[2], bl[2], b.z, h.z, l.z);
                df_acc(bh[3], bl[3], b.w, h.w, l.w);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
    }
    if (!va) return;
    const int64_t rowa = r0 + ra, rowb = r0 + rb_eff;
    for (int64_t c = n_main + lane; c < n_cols; c += 32) {
        df_acc(ah[0], al[0], A[rowa * ld + c], xh[c], xl[c]);
        df_acc(bh[0], bl[0], A[rowb * ld + c], xh[c], xl[c]);
    }
    double sa = 0.0, sb = 0.0;
#pragma unroll
    for (int t = 0; t < 4; t++) {
        sa += (double)ah[t] + (double)al[t];
        sb += (double)bh[t] + (double)bl[t];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sa += __shfl_xor_sync(0xffffffffu, sa, o);
        sb += __shfl_xor_sync(0xffffffffu, sb, o);
    }
    if (lane == 0) {
        y[rowa] = sa;
        if (vb) y[rowb] = sb;
    }
}

template <int R, int CH, int S>
static int df_tma_launch(const float* A, int64_t ld, int64_t nr, int64_t n_main, int64_t nc, const float* xh,
                         const float* xl, double* y, cudaStream_t st) {
    constexpr size_t smem = tp_smem<R, CH, S>();
    static_assert(smem <= 232448, "ring exceeds 227 KB of shared memory");
    const cudaError_t e = cudaFuncSetAttribute(sgemv_df_tma_kernel<R, CH, S>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return set_error(MBEM_ERR_CUDA, "sgemv smem attribute: %s", cudaGetErrorString(e));
    sgemv_df_tma_kernel<R, CH, S><<<(unsigned)ceil_div(nr, R), 32 * (R / 2 + 1), smem, st>>>(A, ld, nr, n_main, nc,
                                                                                             xh, xl, y);
    return MBEM_OK;
}

// the FP32 double-float matvec with tile configuration `cfg` of kDfTiles
static int launch_df_tma(int cfg, const float* A, int64_t ld, int64_t nr, int64_t n_main, int64_t nc,
                         const float* xh, const float* xl, double* y, cudaStream_t st) {
#define MBEM_DF_CASE(i)                                                                                  \
    case i:                                                                                              \
        return df_tma_launch<kDfTiles[i].rows, kDfTiles[i].ch, kDfTiles[i].stages>(A, ld, nr, n_main, nc, \
                                                                                   xh, xl, y, st);
    static_assert(count_of(kDfTiles) == 6, "one case per configuration");
    switch (cfg) {
        MBEM_DF_CASE(0)
        MBEM_DF_CASE(1)
        MBEM_DF_CASE(2)
        MBEM_DF_CASE(3)
        MBEM_DF_CASE(4)
        MBEM_DF_CASE(5)
        default: break;
    }
#undef MBEM_DF_CASE
    return set_error(MBEM_ERR_ARG, "no FP32 matvec tile configuration %d", cfg);
}

// MBEM_ERR_WAIT if a pipeline wait gave up since the last check (the flag is
// cleared); synchronises the stream.
int mixed_wait_check(cudaStream_t st) {
    int flag = 0;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaMemcpyFromSymbol(&flag, g_mixed_wait_error, sizeof(int));
    if (e != cudaSuccess) return set_error(MBEM_ERR_CUDA, "wait check: %s", cudaGetErrorString(e));
    if (flag) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_mixed_wait_error, &zero, sizeof(int));
        return set_error(MBEM_ERR_WAIT, "a bulk-copy wait expired in a mixed-operator kernel");
    }
    return MBEM_OK;
}

int mixed_matvec(const mbem_mixed_operator* op, const double* x, double* y, float* xh, float* xl,
                 cudaStream_t st) {
    const int64_t nr = op->n_rows, nc = op->n_cols;
    if (nr == 0) return MBEM_OK;
    split_vec_kernel<<<(unsigned)ceil_div(nc > 0 ? nc : 1, 256), 256, 0, st>>>(x, nc, xh, xl);
    const bool vec = ((uintptr_t)op->A32 % 16 == 0) && (op->ld32 % 4 == 0);
    MBEM_REQUIRE(vec, MBEM_ERR_ARG, "the FP32 far matrix must be 16-byte aligned with ld32 %% 4 == 0");
    const bool xal = ((uintptr_t)xh % 16 == 0) && ((uintptr_t)xl % 16 == 0);
    const int64_t n_main = nc & ~(int64_t)3;
    if (xal && n_main > 0) {
        int e = launch_df_tma(tune_get(MBEM_TUNE_MIXED_MATVEC), op->A32, op->ld32, nr, n_main, nc, xh, xl, y, st);
        if (e) return e;
    } else {
        const int64_t warps = ceil_div(nr, SGEMV_ROWS);
        sgemv_df_kernel<<<(unsigned)ceil_div(warps, SGEMV_THREADS / 32), SGEMV_THREADS, 0, st>>>(
            op->A32, op->ld32, nr, nc, xh, xl, y);
    }
    int launches = 2;
    for (int q = 0; q < op->n_near; q++) {
        const mbem_near_blocks& nb = op->near[q];
        near_matvec_kernel<<<(unsigned)ceil_div(nb.n_field, 8), 256, 0, st>>>(
            nb.rowptr, nb.cols, nb.vals, nb.n_field, x + nb.col0, y + nb.row0, nullptr);
        launches++;
    }
    return launch_status("mixed_matvec", launches);
}

// ---------------------------------------------------------------------------
// The inner operator of the mixed solve: y = A16 x + near blocks x, with A16
// the far field rounded to BF16. Rows stream through a warp-specialised
// bulk-copy ring (as sgemv_df_tma_kernel) at half the bytes. Each consumer
// warp owns two rows, so every FP32 x value read from shared memory serves
// two rows; lanes read 8-byte BF16 quads and 16-byte x quads at unit stride
// (no bank conflicts). x is rounded to FP32 once per product; rows sum in
// FP32 over four chains each (the operator is a preconditioner: its 2^-9
// entry rounding, not the summation, sets its accuracy).
// ---------------------------------------------------------------------------
// Tile shape (template): BP_ROWS rows per CTA (BP_ROWS / 2 consumer warps),
// BP_CH columns per chunk, BP_STAGES ring stages; the tuned choice is in
// tune.cuh.
template <int R, int CH, int S>
constexpr size_t bp_smem() { return (size_t)S * (R * CH * 2 + CH * 4) + 2 * S * 8; }

__global__ void d2f_kernel(const double* __restrict__ x, int64_t n, float* __restrict__ xf,
                           const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) xf[i] = (float)x[i];
}

__device__ __forceinline__ float bf16_lo(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t u) { return __uint_as_float(u & 0xffff0000u); }

template <int BP_ROWS, int BP_CH, int BP_STAGES>
__global__ void __launch_bounds__(32 * (BP_ROWS / 2 + 1))
sgemv_bf16_tma_kernel(const uint16_t* __restrict__ A, int64_t ld, int64_t n_rows, int64_t n_main, int64_t n_cols,
                      const float* __restrict__ xf, double* __restrict__ y, const int* __restrict__ stop) {
    constexpr int BP_WARPS = BP_ROWS / 2;
    // the whole CTA leaves before any barrier exists
    if (stop && *stop) return;
    extern __shared__ __align__(128) unsigned char smem[];
    uint16_t* sA = reinterpret_cast<uint16_t*>(smem);                                // [S][ROWS][CH]
    float* sX = reinterpret_cast<float*>(sA + (size_t)BP_STAGES * BP_ROWS * BP_CH);   // [S][CH]
    uint64_t* full = reinterpret_cast<uint64_t*>(sX + BP_STAGES * BP_CH);
    uint64_t* empty = full + BP_STAGES;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t r0 = (int64_t)blockIdx.x * BP_ROWS;
    const int nrow = (int)lmin(BP_ROWS, n_rows - r0);
    const int64_t nchunks = ceil_div(n_main, BP_CH);
    if (threadIdx.x == 0) {
        for (int s = 0; s < BP_STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], BP_WARPS);
        }
        mbar_init_fence();
    }
    __syncthreads();

    if (warp == BP_WARPS) {
        int64_t issued = 0;
        for (int64_t k = 0; k < nchunks; k++) {
            const int s = (int)(k % BP_STAGES);
            int ok = 1;
            if (lane == 0) {
                if (k >= BP_STAGES && !mbar_wait(&empty[s], (uint32_t)(((k / BP_STAGES) - 1) & 1), TP_WAIT_LIMIT)) {
                    atomicExch(&g_mixed_wait_error, 1);
                    ok = 0;
                }
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) break;
            const int64_t c0 = k * BP_CH;
            const uint32_t cols = (uint32_t)lmin(BP_CH, n_main - c0);
            if (lane == 0) mbar_arrive_expect_tx(&full[s], cols * 2u * (uint32_t)nrow + cols * 4u);
            __syncwarp();
            for (int t = lane; t < BP_ROWS + 1; t += 32) {
                if (t < nrow)
                    bulk_g2s(sA + ((int64_t)s * BP_ROWS + t) * BP_CH, A + (r0 + t) * ld + c0, cols * 2u, &full[s]);
                else if (t == BP_ROWS)
                    bulk_g2s(sX + (int64_t)s * BP_CH, xf + c0, cols * 4u, &full[s]);
            }
            issued = k + 1;
        }
        if (lane == 0)
            for (int64_t k = (issued > BP_STAGES ? issued - BP_STAGES : 0); k < issued; k++)
                if (!mbar_wait(&full[k % BP_STAGES], (uint32_t)((k / BP_STAGES) & 1), TP_WAIT_LIMIT))
                    atomicExch(&g_mixed_wait_error, 1);
        return;
    }

    // consumer warp w: rows 2w (always < nrow when the warp has work) and 2w + 1
    const int ra = 2 * warp, rb = 2 * warp + 1;
    const bool va = ra < nrow, vb = rb < nrow;
    const int rb_eff = vb ? rb : ra;          // an invalid second row re-reads the first
    float a[4] = {0.f, 0.f, 0.f, 0.f}, b[4] = {0.f, 0.f, 0.f, 0.f};
    for (int64_t k = 0; k < nchunks; k++) {
        const int s = (int)(k % BP_STAGES);
        if (!mbar_wait(&full[s], (uint32_t)((k / BP_STAGES) & 1), TP_WAIT_LIMIT)) {
            atomicExch(&g_mixed_wait_error, 1);
            break;
        }
        if (va) {
            const int w4 = (int)(lmin(BP_CH, n_main - k * BP_CH) / 4);
            const uint2* pa = reinterpret_cast<const uint2*>(sA + ((int64_t)s * BP_ROWS + ra) * BP_CH);
            const uint2* pb = reinterpret_cast<const uint2*>(sA + ((int64_t)s * BP_ROWS + rb_eff) * BP_CH);
            const float4* x4 = reinterpret_cast<const float4*>(sX + (int64_t)s * BP_CH);
#pragma unroll 4
            for (int q = lane; q < w4; q += 32) {
                const float4 u = x4[q];
                const uint2 p = pa[q], r = pb[q];
                a[0] = fmaf(bf16_lo(p.x), u.x, a[0]);
                a[1] = fmaf(bf16_hi(p.x), u.y, a[1]);
                a[2] = fmaf(bf16_lo(p.y), u.z, a[2]);
                a[3] = fmaf(bf16_hi(p.y), u.w, a[3]);
                b[0] = fmaf(bf16_lo(r.x), u.x, b[0]);
                b[1] = fmaf(bf16_hi(r.x), u.y, b[1]);
                b[2] = fmaf(bf16_lo(r.y), u.z, b[2]);
                b[3] = fmaf(bf16_hi(r.y), u.w, b[3]);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
    }
    if (!va) return;
    const int64_t rowa = r0 + ra, rowb = r0 + rb_eff;
    for (int64_t c = n_main + lane; c < n_cols; c += 32) {
        const float xc = xf[c];
        a[0] = fmaf(__uint_as_float((uint32_t)A[rowa * ld + c] << 16), xc, a[0]);
        b[0] = fmaf(__uint_as_float((uint32_t)A[rowb * ld + c] << 16), xc, b[0]);
    }
    double sa = ((double)a[0] + (double)a[1]) + ((double)a[2] + (double)a[3]);
    double sb = ((double)b[0] + (double)b[1]) + ((double)b[2] + (double)b[3]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sa += __shfl_xor_sync(0xffffffffu, sa, o);
        sb += __shfl_xor_sync(0xffffffffu, sb, o);
    }
    if (lane == 0) {
        y[rowa] = sa;
        if (vb) y[rowb] = sb;
    }
}

template <int R, int CH, int S>
static int bf16_tma_launch(const uint16_t* A, int64_t ld, int64_t nr, int64_t n_main, int64_t nc, const float* xf,
                           double* y, const int* stop, cudaStream_t st) {
    constexpr size_t smem = bp_smem<R, CH, S>();
    static_assert(smem <= 232448, "ring exceeds 227 KB of shared memory");
    const cudaError_t e = cudaFuncSetAttribute(sgemv_bf16_tma_kernel<R, CH, S>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return set_error(MBEM_ERR_CUDA, "bf16 gemv smem attribute: %s", cudaGetErrorString(e));
    sgemv_bf16_tma_kernel<R, CH, S><<<(unsigned)ceil_div(nr, R), 32 * (R / 2 + 1), smem, st>>>(A, ld, nr, n_main,
                                                                                               nc, xf, y, stop);
    return MBEM_OK;
}

// the BF16 matvec with tile configuration `cfg` of kBf16Tiles
static int launch_bf16_tma(int cfg, const uint16_t* A, int64_t ld, int64_t nr, int64_t n_main, int64_t nc,
                           const float* xf, double* y, const int* stop, cudaStream_t st) {
#define MBEM_BF_CASE(i)                                                                                        \
    case i:                                                                                                    \
        return bf16_tma_launch<kBf16Tiles[i].rows, kBf16Tiles[i].ch, kBf16Tiles[i].stages>(A, ld, nr, n_main, nc, \
                                                                                           xf, y, stop, st);
    static_assert(count_of(kBf16Tiles) == 6, "one case per configuration");
    switch (cfg) {
        MBEM_BF_CASE(0)
        MBEM_BF_CASE(1)
        MBEM_BF_CASE(2)
        MBEM_BF_CASE(3)
        MBEM_BF_CASE(4)
        MBEM_BF_CASE(5)
        default: break;
    }
#undef MBEM_BF_CASE
    return set_error(MBEM_ERR_ARG, "no BF16 matvec tile configuration %d", cfg);
}

int bf16_matvec(const uint16_t* A16, int64_t ld16, int64_t n_rows, int64_t n_cols, int n_near,
                const mbem_near_blocks* near, const double* x, double* y, float* xf, cudaStream_t st,
                const int* stop) {
    MBEM_REQUIRE(A16 && x && y && xf && n_rows >= 0 && n_cols >= 0 && ld16 >= n_cols, MBEM_ERR_ARG,
                 "bad BF16 matvec args");
    MBEM_REQUIRE((uintptr_t)A16 % 16 == 0 && ld16 % 8 == 0 && (uintptr_t)xf % 16 == 0, MBEM_ERR_ARG,
                 "the BF16 matrix and the scratch must be 16-byte aligned with ld16 %% 8 == 0");
    MBEM_REQUIRE(n_near >= 0 && (n_near == 0 || near), MBEM_ERR_ARG, "bad near blocks");
    if (n_rows == 0) return MBEM_OK;
    d2f_kernel<<<(unsigned)ceil_div(n_cols > 0 ? n_cols : 1, 256), 256, 0, st>>>(x, n_cols, xf, stop);
    const int64_t n_main = n_cols & ~(int64_t)7;
    int e = launch_bf16_tma(tune_get(MBEM_TUNE_BF16_MATVEC), A16, ld16, n_rows, n_main, n_cols, xf, y, stop, st);
    if (e) return e;
    for (int q = 0; q < n_near; q++) {
        const mbem_near_blocks& nb = near[q];
        near_matvec_kernel<<<(unsigned)ceil_div(nb.n_field, 8), 256, 0, st>>>(
            nb.rowptr, nb.cols, nb.vals, nb.n_field, x + nb.col0, y + nb.row0, stop);
    }
    return launch_status("bf16_matvec", 2 + n_near);
}

// ---------------------------------------------------------------------------
// Mixed P0 displacement readout: out[f] (+)= alpha sum_s T(x_f, s) d_s for a
// slip density d (tri_nodal.py:1310-1319 at order 0). Far pairs by the FP32
// quadrature of the mixed operator (far_block<true>: the T block of the
// mollified point kernel, <= ~1.5e-7 of the closed form by the D / L rule),
// contracted with the density in FP32 and summed over a tile of sources in
// FP32, over tiles in FP64; near pairs (is_near, the operator's own test)
// by the FP64 closed form of p0_pair.cuh, inline. One thread an observer,
// DR_TILE sources staged in shared memory at a time.
// ---------------------------------------------------------------------------
constexpr int DR_THREADS = 128, DR_TILE = 32;

struct DispReadoutArgs {
    const double* x;
    int64_t n_obs;
    const double* tri_verts;
    const double* normals;
    const double* eps;
    const double* density;
    int64_t n_src;
    double c[6];
    float cf[6];
    double near_factor;
    double alpha;
    int accumulate;
    double* out;
};

struct DrSrc {
    SrcFar f;
    float d[3];
    int live;        // non-degenerate, non-zero density
};

__global__ void __launch_bounds__(DR_THREADS) disp_readout_kernel(DispReadoutArgs a, QuadRules Q) {
    __shared__ DrSrc tile[DR_TILE];
    const int64_t i = (int64_t)blockIdx.x * DR_THREADS + threadIdx.x;
    const bool live = i < a.n_obs;
    double ox = 0.0, oy = 0.0, oz = 0.0;
    if (live) {
        ox = a.x[3 * i];
        oy = a.x[3 * i + 1];
        oz = a.x[3 * i + 2];
    }
    const F2 xo[3] = {split_d(ox), split_d(oy), split_d(oz)};
    double acc[3] = {0.0, 0.0, 0.0};
    for (int64_t s0 = 0; s0 < a.n_src; s0 += DR_TILE) {
        __syncthreads();
        for (int t = threadIdx.x; t < DR_TILE; t += DR_THREADS) {
            const int64_t s = s0 + t;
            DrSrc& S = tile[t];
            if (s < a.n_src) {
                far_setup(a.tri_verts + 9 * s, a.normals + 3 * s, a.eps[s], a.near_factor, S.f);
                const double* d = a.density + 3 * s;
                S.d[0] = (float)d[0];
                S.d[1] = (float)d[1];
                S.d[2] = (float)d[2];
                S.live = S.f.ok && !(d[0] == 0.0 && d[1] == 0.0 && d[2] == 0.0);
            } else {
                S.live = 0;
            }
        }
        __syncthreads();
        if (!live) continue;
        const int ns = (int)lmin(DR_TILE, a.n_src - s0);
        float part[3] = {0.0f, 0.0f, 0.0f};
        for (int t = 0; t < ns; t++) {
            const DrSrc& S = tile[t];
            if (!S.live) continue;
            float dc[3], D2;
            if (is_near(xo, S.f, dc, D2)) {
                const int64_t s = s0 + t;
                SrcP0 g;
                src_setup(a.tri_verts + 9 * s, a.eps[s], g);
                if (!g.ok) continue;
                PairP0 p;
                pair_setup(g, ox, oy, oz, p);
                TMoments m;
                const double* n = a.normals + 3 * s;
                t_moments(g, n, p, m);
                double blk[3][3];
                t_block(m, n, a.c, g.eps2, blk);
                const double* d = a.density + 3 * s;
#pragma unroll
                for (int r = 0; r < 3; r++) acc[r] += blk[r][0] * d[0] + blk[r][1] * d[1] + blk[r][2] * d[2];
            } else {
                float blk[3][3];
                far_block<true>(Q, S.f, dc, D2, a.cf, blk);
#pragma unroll
                for (int r = 0; r < 3; r++) part[r] += blk[r][0] * S.d[0] + blk[r][1] * S.d[1] + blk[r][2] * S.d[2];
            }
        }
#pragma unroll
        for (int r = 0; r < 3; r++) acc[r] += (double)part[r];
    }
    if (!live) return;
#pragma unroll
    for (int r = 0; r < 3; r++) a.out[3 * i + r] = (a.accumulate ? a.out[3 * i + r] : 0.0) + a.alpha * acc[r];
}

}  // namespace mbem

using namespace mbem;

extern "C" {

int mbem_far_matrix(int kernel, const double* x_field, int64_t n_field, const double* tri_verts,
                    const double* normals, const double* eps, int64_t n_src, const double* coeffs,
                    double near_factor, double alpha, float* out, int64_t ld_out, uint32_t* near_mask,
                    void* stream) {
    return mbem_far_matrix_bf16(kernel, x_field, n_field, tri_verts, normals, eps, n_src, coeffs, near_factor,
                                alpha, out, ld_out, nullptr, 0, near_mask, stream);
}

int mbem_far_matrix_bf16(int kernel, const double* x_field, int64_t n_field, const double* tri_verts,
                         const double* normals, const double* eps, int64_t n_src, const double* coeffs,
                         double near_factor, double alpha, float* out, int64_t ld_out, uint16_t* out16,
                         int64_t ld16, uint32_t* near_mask, void* stream) {
    return mbem_far_matrix_nodal(kernel, 0, x_field, n_field, tri_verts, normals, eps, n_src, coeffs, near_factor,
                                 alpha, out, ld_out, out16, ld16, near_mask, stream);
}

int mbem_far_matrix_nodal(int kernel, int order, const double* x_field, int64_t n_field, const double* tri_verts,
                          const double* normals, const double* eps, int64_t n_src, const double* coeffs,
                          double near_factor, double alpha, float* out, int64_t ld_out, uint16_t* out16,
                          int64_t ld16, uint32_t* near_mask, void* stream) {
    MBEM_REQUIRE(kernel == 0 || kernel == 1, MBEM_ERR_ARG, "kernel must be 0 (T) or 1 (U)");
    MBEM_REQUIRE(order >= 0 && order <= 2, MBEM_ERR_ARG, "order must be 0, 1 or 2 (got %d)", order);
    const int64_t Kn = order == 0 ? 1 : (order == 1 ? 3 : 6);
    MBEM_REQUIRE(n_field >= 0 && n_src >= 0 && ld_out >= 3 * Kn * n_src, MBEM_ERR_ARG, "bad far matrix shape");
    MBEM_REQUIRE(out16 == nullptr || ld16 >= 3 * Kn * n_src, MBEM_ERR_ARG, "bad BF16 copy stride");
    MBEM_REQUIRE(coeffs != nullptr && near_factor > 0.0, MBEM_ERR_ARG, "coeffs/near_factor");
    MBEM_REQUIRE(kernel == 1 || n_src == 0 || normals, MBEM_ERR_ARG, "normals is NULL");
    if (n_field == 0 || n_src == 0) return MBEM_OK;
    FarArgs a;
    a.x_field = x_field; a.n_field = n_field; a.tri_verts = tri_verts; a.normals = normals; a.eps = eps;
    a.n_src = n_src;
    const int nc = kernel == 0 ? 6 : 3;
    for (int i = 0; i < 6; i++) a.c[i] = i < nc ? (float)coeffs[i] : 0.0f;
    a.alpha = (float)alpha; a.near_factor = near_factor; a.out = out; a.ld = ld_out;
    a.near_mask = near_mask;
    a.out16 = out16; a.ld16 = ld16;
    dim3 grid((unsigned)ceil_div(n_src, FAR_THREADS), (unsigned)lmin(ceil_div(n_field, FAR_FIELD_TILE), 65535));
    const cudaStream_t st = (cudaStream_t)stream;
    const QuadRules& Q = rules();
    switch (kernel * 3 + order) {
        case 0: far_assemble_kernel<true, 0><<<grid, FAR_THREADS, 0, st>>>(a, Q); break;
        case 1: far_assemble_kernel<true, 1><<<grid, FAR_THREADS, 0, st>>>(a, Q); break;
        case 2: far_assemble_kernel<true, 2><<<grid, FAR_THREADS, 0, st>>>(a, Q); break;
        case 3: far_assemble_kernel<false, 0><<<grid, FAR_THREADS, 0, st>>>(a, Q); break;
        case 4: far_assemble_kernel<false, 1><<<grid, FAR_THREADS, 0, st>>>(a, Q); break;
        default: far_assemble_kernel<false, 2><<<grid, FAR_THREADS, 0, st>>>(a, Q); break;
    }
    return launch_status("far_assemble_kernel");
}

size_t mbem_near_list_workspace_size(int64_t n_field) { return (size_t)(n_field + 1) * sizeof(int64_t); }

int mbem_near_mask_count(const uint32_t* mask, int64_t n_field, int64_t n_src, int64_t* rowptr, void* work,
                         size_t work_bytes, int64_t* nnz_host, void* stream) {
    MBEM_REQUIRE(n_field >= 0 && n_src >= 0 && rowptr && nnz_host && (n_field == 0 || mask), MBEM_ERR_ARG,
                 "bad near-mask-count args");
    MBEM_REQUIRE(work && work_bytes >= mbem_near_list_workspace_size(n_field), MBEM_ERR_SIZE,
                 "near-mask-count workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    int64_t* counts = (int64_t*)work;
    const int64_t n_words = ceil_div(n_src, 32);
    if (n_field > 0)
        mask_count_kernel<<<(unsigned)ceil_div(n_field, 8), 256, 0, st>>>(mask, n_field, n_words, counts);
    scan_kernel<<<1, 1024, 0, st>>>(counts, n_field, rowptr);
    cudaMemcpyAsync(nnz_host, rowptr + n_field, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("near_mask_count sync", 2);
    return launch_status("near_mask_count", 2);
}

int mbem_near_mask_fill(const uint32_t* mask, int64_t n_field, int64_t n_src, const int64_t* rowptr, int64_t* cols,
                        void* stream) {
    MBEM_REQUIRE(n_field >= 0 && n_src >= 0 && rowptr && (n_field == 0 || mask), MBEM_ERR_ARG,
                 "bad near-mask-fill args");
    if (n_field == 0) return MBEM_OK;
    mask_fill_kernel<<<(unsigned)ceil_div(n_field, 8), 256, 0, (cudaStream_t)stream>>>(
        mask, n_field, ceil_div(n_src, 32), rowptr, cols);
    return launch_status("mask_fill_kernel");
}

int mbem_near_count(const double* x_field, int64_t n_field, const double* tri_verts, const double* eps,
                    int64_t n_src, double near_factor, int64_t* rowptr, void* work, size_t work_bytes,
                    int64_t* nnz_host, void* stream) {
    MBEM_REQUIRE(n_field >= 0 && n_src >= 0 && rowptr && nnz_host, MBEM_ERR_ARG, "bad near-count args");
    MBEM_REQUIRE(work && work_bytes >= mbem_near_list_workspace_size(n_field), MBEM_ERR_SIZE,
                 "near-count workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    int64_t* counts = (int64_t*)work;
    NearArgs a;
    a.x_field = x_field; a.n_field = n_field; a.tri_verts = tri_verts; a.eps = eps; a.n_src = n_src;
    a.near_factor = near_factor; a.counts = counts; a.cols = nullptr;
    if (n_field > 0)
        near_list_kernel<false><<<(unsigned)ceil_div(n_field, NL_THREADS), NL_THREADS, 0, st>>>(a);
    scan_kernel<<<1, 1024, 0, st>>>(counts, n_field, rowptr);
    cudaMemcpyAsync(nnz_host, rowptr + n_field, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("near_count sync", 2);
    return launch_status("near_count", 2);
}

int mbem_near_fill(const double* x_field, int64_t n_field, const double* tri_verts, const double* eps,
                   int64_t n_src, double near_factor, const int64_t* rowptr, int64_t* cols, void* stream) {
    // cols may be NULL when the list is empty: the kernel writes only near pairs
    MBEM_REQUIRE(n_field >= 0 && rowptr, MBEM_ERR_ARG, "bad near-fill args");
    if (n_field == 0) return MBEM_OK;
    NearArgs a;
    a.x_field = x_field; a.n_field = n_field; a.tri_verts = tri_verts; a.eps = eps; a.n_src = n_src;
    a.near_factor = near_factor; a.counts = const_cast<int64_t*>(rowptr); a.cols = cols;
    near_list_kernel<true><<<(unsigned)ceil_div(n_field, NL_THREADS), NL_THREADS, 0, (cudaStream_t)stream>>>(a);
    return launch_status("near_fill");
}

int mbem_near_eval(int kernel, const double* x_field, int64_t n_field, const double* tri_verts,
                   const double* normals, const double* eps, const int64_t* rowptr, const int64_t* cols,
                   int64_t nnz, const double* coeffs, double alpha, double* vals, void* stream) {
    MBEM_REQUIRE(kernel == 0 || kernel == 1, MBEM_ERR_ARG, "kernel must be 0 (T) or 1 (U)");
    MBEM_REQUIRE(coeffs && nnz >= 0, MBEM_ERR_ARG, "bad near-eval args");
    if (nnz == 0) return MBEM_OK;
    NearEvalArgs a;
    a.x_field = x_field; a.n_field = n_field; a.tri_verts = tri_verts; a.normals = normals; a.eps = eps;
    a.rowptr = rowptr; a.cols = cols; a.nnz = nnz; a.alpha = alpha; a.vals = vals;
    const int nc = kernel == 0 ? 6 : 3;
    for (int i = 0; i < 6; i++) a.c[i] = i < nc ? coeffs[i] : 0.0;
    const unsigned g = (unsigned)ceil_div(nnz, 128);
    if (kernel == 0) near_eval_kernel<true><<<g, 128, 0, (cudaStream_t)stream>>>(a);
    else near_eval_kernel<false><<<g, 128, 0, (cudaStream_t)stream>>>(a);
    return launch_status("near_eval_kernel");
}

int mbem_mixed_rowsum3(const float* A32, int64_t ld, int64_t n_rows, int64_t n_col_nodes,
                       const int64_t* rowptr, const double* vals, double* out, void* stream) {
    MBEM_REQUIRE(n_rows >= 0 && n_rows % 3 == 0 && ld >= 3 * n_col_nodes, MBEM_ERR_ARG, "bad rowsum shape");
    if (n_rows == 0) return MBEM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    rowsum3_f32_kernel<<<(unsigned)ceil_div(n_rows, 8), 256, 0, st>>>(A32, ld, n_rows, 3 * n_col_nodes, 1.0, 0,
                                                                     out);
    near_rowsum_kernel<<<(unsigned)ceil_div(n_rows / 3, 128), 128, 0, st>>>(rowptr, vals, n_rows / 3, out);
    return launch_status("mixed_rowsum3", 2);
}

int mbem_near_add_diagonal(const int64_t* rowptr, const int64_t* cols, double* vals, int64_t n_field,
                           const double* D, int* missing, void* stream) {
    MBEM_REQUIRE(rowptr && D && missing, MBEM_ERR_ARG, "bad near-diag args");
    if (n_field == 0) return MBEM_OK;
    near_add_diag_kernel<<<(unsigned)ceil_div(n_field, 128), 128, 0, (cudaStream_t)stream>>>(rowptr, cols, vals,
                                                                                          n_field, D, missing);
    return launch_status("near_add_diag_kernel");
}

int mbem_near_add_diagonal_nodal(const int64_t* rowptr, const int64_t* cols, double* vals, int64_t n_field,
                                 const double* D, int K, const double* shape, int* missing, void* stream) {
    MBEM_REQUIRE(rowptr && D && missing && shape, MBEM_ERR_ARG, "bad near-diag args");
    MBEM_REQUIRE(K == 1 || K == 3 || K == 6, MBEM_ERR_ARG, "K must be 1, 3 or 6 (got %d)", K);
    MBEM_REQUIRE(n_field % K == 0, MBEM_ERR_ARG, "field points must be whole elements");
    if (n_field == 0) return MBEM_OK;
    ShapeKxK sh;
    memset(&sh, 0, sizeof(sh));
    for (int i = 0; i < K * K; i++) sh.w[i] = shape[i];
    near_add_diag_nodal_kernel<<<(unsigned)ceil_div(n_field, 128), 128, 0, (cudaStream_t)stream>>>(
        rowptr, cols, vals, n_field, D, K, sh, missing);
    return launch_status("near_add_diag_nodal_kernel");
}

int mbem_bf16_matvec(const uint16_t* A16, int64_t ld16, int64_t n_rows, int64_t n_cols, int n_near,
                     const mbem_near_blocks* near, const double* x, double* y, void* work, size_t work_bytes,
                     void* stream) {
    MBEM_REQUIRE(work && work_bytes >= (size_t)n_cols * sizeof(float), MBEM_ERR_SIZE,
                 "BF16 matvec workspace too small (needs %lld bytes)", (long long)(n_cols * sizeof(float)));
    return bf16_matvec(A16, ld16, n_rows, n_cols, n_near, near, x, y, (float*)work, (cudaStream_t)stream);
}

int mbem_t_disp_readout(const double* x, int64_t n_obs, const double* tri_verts, const double* normals,
                        const double* eps, int64_t n_src, const double* density, const double* coeffs,
                        double near_factor, double alpha, int accumulate, double* out, void* stream) {
    MBEM_REQUIRE(n_obs >= 0 && n_src >= 0 && near_factor > 0.0 && coeffs, MBEM_ERR_ARG, "bad readout sizes");
    MBEM_REQUIRE((n_obs == 0 || (x && out)) && (n_src == 0 || (tri_verts && normals && eps && density)),
                 MBEM_ERR_ARG, "NULL readout arrays");
    if (n_obs == 0) return MBEM_OK;
    MBEM_REQUIRE(ceil_div(n_obs, DR_THREADS) < (int64_t)INT32_MAX, MBEM_ERR_SIZE, "too many observers");
    DispReadoutArgs a;
    a.x = x;
    a.n_obs = n_obs;
    a.tri_verts = tri_verts;
    a.normals = normals;
    a.eps = eps;
    a.density = density;
    a.n_src = n_src;
    for (int k = 0; k < 6; k++) {
        a.c[k] = coeffs[k];
        a.cf[k] = (float)coeffs[k];
    }
    a.near_factor = near_factor;
    a.alpha = alpha;
    a.accumulate = accumulate;
    a.out = out;
    disp_readout_kernel<<<(unsigned)ceil_div(n_obs, DR_THREADS), DR_THREADS, 0, (cudaStream_t)stream>>>(a, rules());
    return launch_status("disp_readout_kernel");
}

int mbem_mixed_matvec(const mbem_mixed_operator* op, const double* x, double* y, void* work, size_t work_bytes,
                      void* stream) {
    MBEM_REQUIRE(op && x && y && op->n_rows >= 0 && op->n_cols >= 0 && op->ld32 >= op->n_cols, MBEM_ERR_ARG,
                 "bad mixed matvec args");
    MBEM_REQUIRE(work && work_bytes >= 2 * (size_t)op->n_cols * sizeof(float) + 64, MBEM_ERR_SIZE,
                 "mixed matvec workspace too small");
    float* xh = (float*)work;
    float* xl = xh + ((op->n_cols + 15) / 16) * 16;
    return mixed_matvec(op, x, y, xh, xl, (cudaStream_t)stream);
}

int mbem_mixed_wait_check(void* stream) {
    return mixed_wait_check((cudaStream_t)stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// The mixed matvec for callers that cannot allocate device memory.
//
// Some hosts of this library never call cudaMalloc: a solver embedded in an
// application that hands every byte of device memory to its own pool at
// start-up, a real-time loop that must not take the allocator's locks or its
// synchronisation, or code running where a new allocation would fail the
// memory budget it was given. mbem_mixed_matvec needs 2 n_cols floats of
// scratch (the hi/lo split of x) from such a caller. This variant instead
// keeps that scratch in a fixed array compiled into the library: every GPU
// that loads the library holds it (2 MiB) until the process exits.
// ---------------------------------------------------------------------------
namespace mbem {

constexpr int64_t NOALLOC_MAX_COLS = 262144;          // 2 x 262144 floats = 2 MiB

static __device__ __align__(256) float g_noalloc_split[2 * NOALLOC_MAX_COLS];

static std::mutex g_noalloc_mutex;

// The array's device address differs between CUDA contexts (a driver-API
// context that is not the device's primary one, or the primary context made
// again after cudaDeviceReset), so it is cached per context: the current
// context's handle is read through the driver entry point (no libcuda link).
struct NoallocEntry {
    void* ctx;
    float* ptr;
};
constexpr int NOALLOC_CACHE = 64;
static NoallocEntry g_noalloc_cache[NOALLOC_CACHE];
static int g_noalloc_used = 0;
typedef int (*CtxGetCurrentFn)(void**);
static CtxGetCurrentFn g_ctx_get_current = nullptr;

static void* noalloc_current_context() {
    if (g_ctx_get_current == nullptr) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPoint("cuCtxGetCurrent", &fn, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || fn == nullptr)
            return nullptr;
        g_ctx_get_current = (CtxGetCurrentFn)fn;
    }
    void* ctx = nullptr;
    if (g_ctx_get_current(&ctx) != 0) return nullptr;
    return ctx;
}

// Device address of the scratch array in the current context, looked up once
// per context (the host-side name of a __device__ array is not a device
// address and must never be passed to a kernel). Without a readable context
// handle the address is looked up on every call.
static int noalloc_scratch(float** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(MBEM_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    // makes the device's primary context current on this thread if no
    // context is (it allocates nothing)
    e = cudaSetDevice(dev);
    if (e != cudaSuccess) return set_error(MBEM_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    void* ctx = noalloc_current_context();
    if (ctx != nullptr)
        for (int i = 0; i < g_noalloc_used; i++)
            if (g_noalloc_cache[i].ctx == ctx) {
                *out = g_noalloc_cache[i].ptr;
                return MBEM_OK;
            }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_split);
    if (e != cudaSuccess) return set_error(MBEM_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    if (ctx != nullptr && g_noalloc_used < NOALLOC_CACHE) g_noalloc_cache[g_noalloc_used++] = {ctx, (float*)p};
    *out = static_cast<float*>(p);
    return MBEM_OK;
}

}  // namespace mbem

extern "C" int mbem_mixed_matvec_noalloc(const mbem_mixed_operator* op, const double* x, double* y,
                                         void* stream) {
    MBEM_REQUIRE(op && x && y && op->n_rows >= 0 && op->n_cols >= 0 && op->ld32 >= op->n_cols, MBEM_ERR_ARG,
                 "bad mixed matvec args");
    MBEM_REQUIRE(op->n_cols <= mbem::NOALLOC_MAX_COLS, MBEM_ERR_SIZE,
                 "mbem_mixed_matvec_noalloc: n_cols = %lld exceeds its fixed scratch of %lld columns; use "
                 "mbem_mixed_matvec with a workspace",
                 (long long)op->n_cols, (long long)mbem::NOALLOC_MAX_COLS);
    float* scratch = nullptr;
    int e = mbem::noalloc_scratch(&scratch);
    if (e) return e;
    // Nothing in the scratch has to start at zero: the split kernel writes
    // entries 0 .. n_cols-1 of both halves before the product reads them.
    return mbem::mixed_matvec(op, x, y, scratch, scratch + mbem::NOALLOC_MAX_COLS, (cudaStream_t)stream);
}
