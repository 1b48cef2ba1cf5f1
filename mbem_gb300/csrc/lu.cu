// Dense LU with partial pivoting in FP32 on one GB300 (sm_103a): the
// factorisation behind the reference's la/lu.py `Factor(how="single"|"gpu")`
// (FP32 factors, FP64 iterative refinement by the caller).
//
// Right-looking, in outer blocks of four LU_NB-column panels:
//   1. panel: rows k..n-1 of columns k..k+NB-1 factored by ONE cooperative
//      launch; each CTA holds a contiguous slice of the panel rows in shared
//      memory, and every column takes one grid barrier (bounded spin on a
//      generation counter): local arg-max, candidates published, barrier,
//      every CTA picks the same pivot (largest |value|, then lowest row),
//      swaps and eliminates its own rows;
//   2. the panel's row interchanges applied to the other columns (a later
//      panel of a block is first brought up to date by the earlier ones:
//      their U rows on its columns, each followed by the update of the rows
//      below, left-looking);
//   3. U12 = L11^-1 A12 (unit lower triangle, one column a thread:
//      lu_block_trsm_kernel, also the diagonal blocks of the solves);
//   4. A22 -= L21 U12 on the tensor cores: both operands split into three
//      BF16 pieces, the six piece products of order <= 2 in one tcgen05 GEMM
//      (FP32 accumulation in TMEM) subtracted from A22 in its epilogue.
// Pivots follow LAPACK's getrf convention (0-based): row k was exchanged
// with row piv[k] at step k. A zero pivot column is left unscaled and
// reported in *info (first zero pivot + 1), as getrf does.
//
// Solves: the pivots are turned into a permutation on the host; the
// triangular solves are blocked by LU_NB rows (a small triangle per block,
// then a matrix-vector update of the rows below it).
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "common.cuh"

namespace mbem {

constexpr int LU_NB = 64;                 // panel width
constexpr int LU_OB = 256;                // outer block: four panels, one trailing update
constexpr int LU_PT = 256;                // panel threads
constexpr int LU_LDS = LU_NB + 1;         // padded shared-memory row (no bank conflicts)
constexpr uint32_t LU_WAIT_LIMIT = 1u << 24;

__device__ int g_lu_wait_error = 0;

// optional device time of the factorisation's phases (the panels with their
// interchanges, the U block rows, the trailing updates), in ms
static int g_lu_timing = 0;
static double g_lu_phase_ms[3] = {0, 0, 0};

struct PanelArgs {
    float* A;
    int64_t lda, n, k;
    int32_t* piv;
    float* cand_val;        // [2][G] |pivot candidate|
    int64_t* cand_row;      // [2][G] its global row
    float* cand_rows;       // [2][G][NB] its row values (panel columns)
    float* rowj;            // [2][NB] the current pivot position's old row
    unsigned* bar_count;
    unsigned* bar_gen;
    int* info;
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid barrier of a cooperative launch: arrive on a counter; the last
// arrival resets it and advances the generation; the others poll the
// generation (bounded). Returns false (and flags the error) on a timeout.
__device__ __forceinline__ bool lu_grid_sync(unsigned* count, unsigned* gen, unsigned& my_gen) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        const unsigned g = my_gen;
        __threadfence();
        if (atomicAdd(count, 1u) == gridDim.x - 1) {
            atomicExch(count, 0u);
            __threadfence();
            atomicExch(gen, g + 1u);
        } else {
            uint32_t i = 0;
            while (ld_acquire_u32(gen) == g) {
                if (++i > LU_WAIT_LIMIT) {
                    atomicExch(&g_lu_wait_error, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(20);
            }
        }
        __threadfence();
        my_gen = g + 1u;
    }
    __syncthreads();
    return ok != 0;
}

__global__ void __launch_bounds__(LU_PT)
lu_panel_kernel(PanelArgs a) {
    extern __shared__ float sp[];                 // [rows][LU_LDS]
    __shared__ float prow[LU_NB];
    __shared__ float red_v[LU_PT / 32];
    __shared__ int64_t red_r[LU_PT / 32];
    __shared__ int red_q[LU_PT / 32];
    __shared__ float s_pv;
    __shared__ int64_t s_p;
    __shared__ int s_win;
    const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
    const int lane = tid & 31, wid = tid >> 5;
    const int64_t m = a.n - a.k;
    const int64_t per = ceil_div(m, G);
    const int64_t r0 = a.k + (int64_t)b * per;
    const int64_t r1 = lmin(a.n, r0 + per);
    const int nr = (int)lmax(0, r1 - r0);
    const int nbw = (int)lmin(LU_NB, a.n - a.k);  // panel width (last panel may be narrower)
    for (int64_t e = tid; e < (int64_t)nr * LU_NB; e += LU_PT) {
        const int r = (int)(e / LU_NB), c = (int)(e % LU_NB);
        sp[r * LU_LDS + c] = c < nbw ? a.A[(r0 + r) * a.lda + a.k + c] : 0.0f;
    }
    unsigned my_gen = 0;
    if (tid == 0) my_gen = atomicAdd(a.bar_gen, 0u);
    __syncthreads();
    for (int j = 0; j < nbw; j++) {
        const int64_t gj = a.k + j;
        const int buf = j & 1;
        // a. local candidate: largest |A[r][j]| over own rows r >= gj (lowest row on ties)
        float bv = -1.0f;
        int64_t br = -1;
        for (int r = tid; r < nr; r += LU_PT) {
            if (r0 + r < gj) continue;
            const float v = fabsf(sp[r * LU_LDS + j]);
            if (v > bv) { bv = v; br = r0 + r; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int64_t orow = __shfl_xor_sync(0xffffffffu, br, o);
            if (ov > bv || (ov == bv && orow >= 0 && (br < 0 || orow < br))) { bv = ov; br = orow; }
        }
        if (lane == 0) { red_v[wid] = bv; red_r[wid] = br; }
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < LU_PT / 32; w++)
                if (red_v[w] > red_v[0] || (red_v[w] == red_v[0] && red_r[w] >= 0 && (red_r[0] < 0 || red_r[w] < red_r[0]))) {
                    red_v[0] = red_v[w];
                    red_r[0] = red_r[w];
                }
            a.cand_val[buf * G + b] = red_v[0];
            a.cand_row[buf * G + b] = red_r[0];
        }
        __syncthreads();
        const int64_t mine = red_r[0];
        if (mine >= 0)
            for (int c = tid; c < LU_NB; c += LU_PT) a.cand_rows[((int64_t)buf * G + b) * LU_NB + c] = sp[(mine - r0) * LU_LDS + c];
        if (gj >= r0 && gj < r1)
            for (int c = tid; c < LU_NB; c += LU_PT) a.rowj[buf * LU_NB + c] = sp[(gj - r0) * LU_LDS + c];
        // b. every candidate published
        if (!lu_grid_sync(a.bar_count, a.bar_gen, my_gen)) break;
        // c. the pivot, the same in every CTA: one candidate a thread, then a
        // block reduction (largest value, lowest row on ties)
        {
            float v = -1.0f;
            int64_t r = -1;
            int q = -1;
            if (tid < G) {
                r = __ldcg(a.cand_row + buf * G + tid);
                v = r >= 0 ? __ldcg(a.cand_val + buf * G + tid) : -1.0f;
                q = r >= 0 ? tid : -1;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float ov = __shfl_xor_sync(0xffffffffu, v, o);
                const int64_t orow = __shfl_xor_sync(0xffffffffu, r, o);
                const int oq = __shfl_xor_sync(0xffffffffu, q, o);
                if (orow >= 0 && (r < 0 || ov > v || (ov == v && orow < r))) { v = ov; r = orow; q = oq; }
            }
            if (lane == 0) { red_v[wid] = v; red_r[wid] = r; red_q[wid] = q; }
            __syncthreads();
            if (tid == 0) {
                for (int w = 1; w < LU_PT / 32; w++)
                    if (red_r[w] >= 0 && (red_r[0] < 0 || red_v[w] > red_v[0] || (red_v[w] == red_v[0] && red_r[w] < red_r[0]))) {
                        red_v[0] = red_v[w];
                        red_r[0] = red_r[w];
                        red_q[0] = red_q[w];
                    }
                s_p = red_r[0];
                s_win = red_q[0];
            }
            __syncthreads();
        }
        // no candidate at all: every remaining entry of the column is NaN
        // (|NaN| compares false), e.g. after Inf - Inf in an earlier update.
        // The column is then a zero pivot: row gj stays in place, nothing is
        // eliminated and info reports it.
        const bool none = s_p < 0;
        const int64_t p = none ? gj : s_p;
        const int win = s_win;
        for (int c = tid; c < LU_NB; c += LU_PT)
            prow[c] = none ? __ldcg(a.rowj + buf * LU_NB + c)
                           : __ldcg(a.cand_rows + ((int64_t)buf * G + win) * LU_NB + c);
        __syncthreads();
        if (tid == 0) {
            s_pv = none ? 0.0f : prow[j];
            if (b == 0) a.piv[gj] = (int32_t)p;
            if (b == 0 && s_pv == 0.0f) atomicCAS(a.info, 0, (int)(gj + 1));
        }
        // swap: the pivot row moves to position gj, row gj's old values to position p
        if (p != gj && p >= r0 && p < r1)
            for (int c = tid; c < LU_NB; c += LU_PT) sp[(p - r0) * LU_LDS + c] = __ldcg(a.rowj + buf * LU_NB + c);
        if (gj >= r0 && gj < r1)
            for (int c = tid; c < LU_NB; c += LU_PT) sp[(gj - r0) * LU_LDS + c] = prow[c];
        __syncthreads();
        // eliminate: rows below gj in this slice
        const float pv = s_pv;
        if (pv != 0.0f) {
            const float inv = 1.0f / pv;
            for (int r = tid; r < nr; r += LU_PT) {
                if (r0 + r <= gj) continue;
                float* row = sp + r * LU_LDS;
                const float l = row[j] * inv;
                row[j] = l;
                for (int c = j + 1; c < nbw; c++) row[c] = fmaf(-l, prow[c], row[c]);
            }
        }
        __syncthreads();
    }
    for (int64_t e = tid; e < (int64_t)nr * LU_NB; e += LU_PT) {
        const int r = (int)(e / LU_NB), c = (int)(e % LU_NB);
        if (c < nbw) a.A[(r0 + r) * a.lda + a.k + c] = sp[r * LU_LDS + c];
    }
}

// the panel's interchanges on the columns outside it: one thread a column
__global__ void lu_swap_kernel(float* __restrict__ A, int64_t lda, int64_t n, int64_t k, int nbw,
                               const int32_t* __restrict__ piv) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t ncol = n - nbw;
    if (t >= ncol) return;
    const int64_t c = t < k ? t : t + nbw;     // skip the panel's own columns
    for (int i = 0; i < nbw; i++) {
        const int64_t p = piv[k + i];
        if (p <= k + i || p >= n) continue;      // no interchange (a pivot is never above its row)
        float* x = A + (k + i) * lda + c;
        float* y = A + p * lda + c;
        const float v = *x;
        *x = *y;
        *y = v;
    }
}

// ---- the trailing update on the tensor cores --------------------------------
// FP32 x = hi + mid + lo in three BF16 pieces (24 significant bits); the
// product of two such is taken over the six pieces pairs of order <= 2
// (hi.hi, hi.mid, hi.lo, mid.hi, mid.mid, lo.hi), the dropped ones below
// 2^-24 relative: FP32 accuracy with FP32 accumulation in TMEM.
// The operands: L21 rows as [lo hi mid mid hi hi], U12 columns as
// [hi lo mid hi mid hi], 6 x W BF16 each: along K the products run from the
// smallest (lo.hi, hi.lo, mid.mid ~2^-16) through mid.hi, hi.mid (~2^-8)
// to hi.hi, so the accumulator is small while the corrections are added and
// the rounding of each accumulation step, relative to the running sum,
// falls mostly on the last W terms.
constexpr int LU_K6 = 6 * LU_NB;

__device__ __forceinline__ void bf16_pieces(float x, uint16_t& hi, uint16_t& mid, uint16_t& lo) {
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h);
    const __nv_bfloat16 m = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(m);
    hi = __bfloat16_as_ushort(h);
    mid = __bfloat16_as_ushort(m);
    lo = __bfloat16_as_ushort(__float2bfloat16_rn(r2));
}

// Ls[r][6 x W]: the pieces of rows row0 + r (r < M) of a row-major FP32
// matrix at columns col0 .. col0 + nbw (W = 64, a panel, or 256, an outer
// block; L21 in the factorisation, the L or U panel of a blocked solve)
template <int W>
__global__ void lu_split_rows_kernel(const float* __restrict__ A, int64_t lda, int64_t row0, int64_t col0, int nbw,
                                     int64_t M, uint16_t* __restrict__ Ls) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= M * W) return;
    const int64_t r = e / W;
    const int kk = (int)(e % W);
    const float x = kk < nbw ? A[(row0 + r) * lda + col0 + kk] : 0.0f;
    uint16_t h, m, l;
    bf16_pieces(x, h, m, l);
    uint16_t* o = Ls + r * (6 * W) + kk;
    o[0] = l; o[W] = h; o[2 * W] = m; o[3 * W] = m; o[4 * W] = h; o[5 * W] = h;
}

// Us[j][6 x W]: the pieces of column col0 + j (j < N) of rows row0 ..
// row0 + nbw of a row-major FP32 matrix (U12 in the factorisation, a block of
// right-hand sides in a solve); a W x 32 tile through shared memory keeps
// reads and writes coalesced
template <int W>
__global__ void __launch_bounds__(256)
lu_split_cols_kernel(const float* __restrict__ A, int64_t lda, int64_t row0, int64_t col0, int nbw, int64_t N,
                     uint16_t* __restrict__ Us) {
    __shared__ float T[W][33];
    const int64_t j0 = (int64_t)blockIdx.x * 32;
    for (int e = threadIdx.x; e < W * 32; e += 256) {
        const int kk = e / 32, j = e % 32;
        T[kk][j] = (kk < nbw && j0 + j < N) ? A[(row0 + kk) * lda + col0 + j0 + j] : 0.0f;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < W * 32; e += 256) {
        const int j = e / W, kk = e % W;
        if (j0 + j >= N) continue;
        uint16_t h, m, l;
        bf16_pieces(T[kk][j], h, m, l);
        uint16_t* o = Us + (j0 + j) * (6 * W) + kk;
        o[0] = h; o[W] = l; o[2 * W] = m; o[3 * W] = h; o[4 * W] = m; o[5 * W] = h;
    }
}

// C[M x N] (at ldc) -= rows (row0 .., M) x columns (col0 .., w) of A times
// rows (urow0 .., w) x columns (ucol0 .., N) of A, all in A (at lda): the
// six-piece tensor-core product, panel width W
template <int W>
static int lu_block_update(float* A, int64_t lda, int64_t row0, int64_t col0, int64_t M, int w, int64_t urow0,
                           int64_t ucol0, int64_t N, float* C, int64_t ldc, uint16_t* Ls, uint16_t* Us,
                           cudaStream_t st) {
    if (M <= 0 || N <= 0) return MBEM_OK;
    lu_split_rows_kernel<W><<<(unsigned)ceil_div(M * W, 256), 256, 0, st>>>(A, lda, row0, col0, w, M, Ls);
    lu_split_cols_kernel<W><<<(unsigned)ceil_div(N, 32), 256, 0, st>>>(A, lda, urow0, ucol0, w, N, Us);
    count_launches(2);
    return gemm_bf16_sub(Ls, 6 * W, Us, 6 * W, M, N, 6 * W, C, ldc, st);
}

// The rank-b update of a blocked Gauss-Jordan inverse (FP32 M, n x n at ld),
// in place: M[i, j] -= M[i, K] M[K, j] for i, j outside K = [k0, k0 + b),
// with M[:, K] the block column before its own update and M[K, :] the block
// row after it. The six-piece tensor-core product of lu_block_update, with
// the pieces of the rows K of the column block and of the columns K of the
// row block set to zero, so that those rows and columns are left as they are.
int gj_block_update_tc(float* M, int64_t n, int64_t ld, int64_t k0, int b, uint16_t* Ls, uint16_t* Us,
                       cudaStream_t st) {
    MBEM_REQUIRE(b >= 1 && b <= LU_NB && k0 >= 0 && k0 + b <= n, MBEM_ERR_ARG, "bad Gauss-Jordan block");
    lu_split_rows_kernel<LU_NB><<<(unsigned)ceil_div(n * LU_NB, 256), 256, 0, st>>>(M, ld, 0, k0, b, n, Ls);
    lu_split_cols_kernel<LU_NB><<<(unsigned)ceil_div(n, 32), 256, 0, st>>>(M, ld, k0, 0, b, n, Us);
    cudaMemsetAsync(Ls + k0 * LU_K6, 0, (size_t)b * LU_K6 * sizeof(uint16_t), st);
    cudaMemsetAsync(Us + k0 * LU_K6, 0, (size_t)b * LU_K6 * sizeof(uint16_t), st);
    count_launches(2);
    return gemm_bf16_sub(Ls, LU_K6, Us, LU_K6, n, n, LU_K6, M, ld, st);
}

// X[r0 .. r0 + nb) (ncols columns at ldx) = T^-1 X with T the nb x nb
// diagonal block of LU at (r0, r0): its unit lower triangle (lower) or its
// upper triangle; one thread a column
__global__ void __launch_bounds__(128)
lu_block_trsm_kernel(const float* __restrict__ LU, int64_t lda, float* __restrict__ X, int64_t ldx, int64_t ncols,
                     int64_t r0, int nb, int lower) {
    __shared__ float T[LU_NB][LU_NB + 1];
    for (int e = threadIdx.x; e < LU_NB * LU_NB; e += blockDim.x) {
        const int r = e / LU_NB, c = e % LU_NB;
        T[r][c] = (r < nb && c < nb) ? LU[(r0 + r) * lda + r0 + c] : (r == c ? 1.0f : 0.0f);
    }
    __syncthreads();
    const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= ncols) return;
    float x[LU_NB];
#pragma unroll
    for (int r = 0; r < LU_NB; r++) x[r] = r < nb ? X[(r0 + r) * ldx + col] : 0.0f;
    if (lower) {
#pragma unroll
        for (int r = 1; r < LU_NB; r++) {
            float v = x[r];
#pragma unroll
            for (int c = 0; c < r; c++) v = fmaf(-T[r][c], x[c], v);
            x[r] = v;
        }
    } else {
#pragma unroll
        for (int r = LU_NB - 1; r >= 0; r--) {
            float v = x[r];
#pragma unroll
            for (int c = r + 1; c < LU_NB; c++) v = fmaf(-T[r][c], x[c], v);
            x[r] = v / T[r][r];
        }
    }
#pragma unroll
    for (int r = 0; r < LU_NB; r++)
        if (r < nb) X[(r0 + r) * ldx + col] = x[r];
}

// X32[i][j] = B[perm[i]][j] (FP64 to FP32) and back
__global__ void lu_gather_rows_kernel(const double* __restrict__ B, int64_t ldb, const int32_t* __restrict__ perm,
                                      int64_t n, int64_t k, float* __restrict__ X, int64_t ldx) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * k) return;
    const int64_t i = e / k, j = e % k;
    X[i * ldx + j] = (float)B[(int64_t)perm[i] * ldb + j];
}

__global__ void lu_widen_rows_kernel(const float* __restrict__ X, int64_t ldx, int64_t n, int64_t k,
                                     double* __restrict__ Y, int64_t ldy) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * k) return;
    const int64_t i = e / k, j = e % k;
    Y[i * ldy + j] = (double)X[i * ldx + j];
}

// ---- solves ---------------------------------------------------------------
// x[i] = b[perm[i]] (FP64 in, FP32 working copy)
__global__ void lu_permute_kernel(const double* __restrict__ b, const int32_t* __restrict__ perm, int64_t n,
                                  float* __restrict__ x) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = (float)b[perm[i]];
}

// one diagonal block of a triangular solve (one CTA): x[r0..r0+nb) solved in
// place against the block's triangle; lower = unit lower (L), else upper (U)
__global__ void lu_tri_block_kernel(const float* __restrict__ A, int64_t lda, float* __restrict__ x, int64_t r0,
                                    int nb, int lower) {
    __shared__ float xs[LU_NB];
    __shared__ float T[LU_NB][LU_NB + 1];
    for (int i = threadIdx.x; i < nb; i += blockDim.x) xs[i] = x[r0 + i];
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) T[e / nb][e % nb] = A[(r0 + e / nb) * lda + r0 + e % nb];
    __syncthreads();
    // column sweeps: once x[c] is final every later row subtracts its term
    const int t = threadIdx.x;
    if (lower) {
        for (int c = 0; c < nb - 1; c++) {
            if (t > c && t < nb) xs[t] = fmaf(-T[t][c], xs[c], xs[t]);
            __syncthreads();
        }
    } else {
        for (int c = nb - 1; c >= 0; c--) {
            if (t == c) xs[c] = xs[c] / T[c][c];
            __syncthreads();
            if (t < c) xs[t] = fmaf(-T[t][c], xs[c], xs[t]);
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < nb; i += blockDim.x) x[r0 + i] = xs[i];
}

// rows [i0, i1) of x -= A[rows, c0..c0+nb) x[c0..c0+nb): a warp a row
__global__ void lu_gemv_update_kernel(const float* __restrict__ A, int64_t lda, float* __restrict__ x, int64_t i0,
                                      int64_t i1, int64_t c0, int nb) {
    const int64_t r = i0 + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= i1) return;
    float s = 0.0f;
    for (int c = lane; c < nb; c += 32) s = fmaf(A[r * lda + c0 + c], x[c0 + c], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[r] -= s;
}

__global__ void lu_widen_kernel(const float* __restrict__ x, int64_t n, double* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)x[i];
}

// ---- solves with the transpose: A^T = U^T L^T P ------------------------------
// One diagonal block of U^T w = c (ut = 1: lower, the diagonal of U) or of
// L^T z = w (ut = 0: upper, unit diagonal), x[r0..r0+nb) in place; the
// block's triangle is read transposed from LU
__global__ void lu_tri_block_t_kernel(const float* __restrict__ A, int64_t lda, float* __restrict__ x, int64_t r0,
                                      int nb, int ut) {
    __shared__ float xs[LU_NB];
    __shared__ float T[LU_NB][LU_NB + 1];          // T[r][c] = A[r0 + c][r0 + r]
    for (int i = threadIdx.x; i < nb; i += blockDim.x) xs[i] = x[r0 + i];
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) T[e % nb][e / nb] = A[(r0 + e / nb) * lda + r0 + e % nb];
    __syncthreads();
    const int t = threadIdx.x;
    if (ut) {
        for (int c = 0; c < nb; c++) {
            if (t == c) xs[c] = xs[c] / T[c][c];
            __syncthreads();
            if (t > c && t < nb) xs[t] = fmaf(-T[t][c], xs[c], xs[t]);
            __syncthreads();
        }
    } else {
        for (int c = nb - 1; c > 0; c--) {
            if (t < c) xs[t] = fmaf(-T[t][c], xs[c], xs[t]);
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < nb; i += blockDim.x) x[r0 + i] = xs[i];
}

// x[r] -= sum_c A[c0 + c][r] x[c0 + c] for r in [i0, i1): the transposed
// block's product, one thread a row (a warp reads 32 consecutive columns of
// each row c0 + c)
__global__ void lu_gemv_update_t_kernel(const float* __restrict__ A, int64_t lda, float* __restrict__ x, int64_t i0,
                                        int64_t i1, int64_t c0, int nb) {
    const int64_t r = i0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= i1) return;
    float s = 0.0f;
    for (int c = 0; c < nb; c++) s = fmaf(A[(c0 + c) * lda + r], x[c0 + c], s);
    x[r] -= s;
}

__global__ void lu_narrow_kernel(const double* __restrict__ b, int64_t n, float* __restrict__ x) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = (float)b[i];
}

// out[perm[i]] = x[i]: y = P^T z, widened to FP64
__global__ void lu_scatter_widen_kernel(const float* __restrict__ x, const int32_t* __restrict__ perm, int64_t n,
                                        double* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[perm[i]] = (double)x[i];
}

}  // namespace mbem

using namespace mbem;

extern "C" {

size_t mbem_lu_workspace_size(int64_t n, int sms) {
    const size_t G = (size_t)(sms > 0 ? sms : 1);
    return 2 * G * sizeof(float) + 2 * G * sizeof(int64_t) + 2 * G * LU_NB * sizeof(float) +
           2 * LU_NB * sizeof(float) + 4 * sizeof(unsigned) + 2 * (size_t)n * 6 * LU_OB * sizeof(uint16_t) + 8 * 256;
}

int mbem_lu_factor_f32(float* A, int64_t lda, int64_t n, int32_t* piv, void* work, size_t work_bytes, int* info,
                       void* stream) {
    MBEM_REQUIRE(A && piv && info && n >= 1 && lda >= n, MBEM_ERR_ARG, "bad LU arguments");
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0, coop = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    MBEM_REQUIRE(coop, MBEM_ERR_UNSUPPORTED, "the device cannot launch cooperative kernels");
    // the pivot search reads one CTA's candidate per panel thread
    MBEM_REQUIRE(sms <= LU_PT, MBEM_ERR_UNSUPPORTED, "the LU panel supports at most %d SMs (the device has %d)",
                 LU_PT, sms);
    const size_t need = mbem_lu_workspace_size(n, sms);
    MBEM_REQUIRE(work && work_bytes >= need, MBEM_ERR_SIZE, "LU workspace %zu < %zu bytes", work_bytes, need);
    // the panel slice of each CTA must fit in shared memory
    const int64_t rows_per = ceil_div(n, sms);
    const size_t panel_smem = (size_t)rows_per * LU_LDS * sizeof(float);
    MBEM_REQUIRE(panel_smem <= 200 * 1024, MBEM_ERR_UNSUPPORTED,
                 "n = %lld is beyond the panel's shared memory (at most %lld rows)", (long long)n,
                 (long long)((200 * 1024) / (LU_LDS * sizeof(float)) * sms));
    char* w = (char*)work;
    auto take = [&](size_t bytes) { char* p = w; w += (bytes + 255) & ~(size_t)255; return p; };
    PanelArgs a;
    a.A = A; a.lda = lda; a.n = n; a.piv = piv; a.info = info;
    a.cand_val = (float*)take(2 * (size_t)sms * sizeof(float));
    a.cand_row = (int64_t*)take(2 * (size_t)sms * sizeof(int64_t));
    a.cand_rows = (float*)take(2 * (size_t)sms * LU_NB * sizeof(float));
    a.rowj = (float*)take(2 * LU_NB * sizeof(float));
    unsigned* bar = (unsigned*)take(4 * sizeof(unsigned));
    a.bar_count = bar;
    a.bar_gen = bar + 1;
    uint16_t* Ls = (uint16_t*)take((size_t)n * 6 * LU_OB * sizeof(uint16_t));
    uint16_t* Us = (uint16_t*)take((size_t)n * 6 * LU_OB * sizeof(uint16_t));
    if ((size_t)(w - (char*)work) > work_bytes) return set_error(MBEM_ERR_SIZE, "LU workspace layout");
    cudaMemsetAsync(bar, 0, 4 * sizeof(unsigned), st);
    cudaMemsetAsync(info, 0, sizeof(int), st);
    cudaError_t ce = cudaFuncSetAttribute(lu_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (ce != cudaSuccess) return set_error(MBEM_ERR_CUDA, "LU smem attribute: %s", cudaGetErrorString(ce));
    int64_t launches = 0;
    int e = MBEM_OK;
    std::vector<cudaEvent_t> evs;
    auto mark = [&]() {
        if (!g_lu_timing) return;
        cudaEvent_t e2;
        cudaEventCreate(&e2);
        cudaEventRecord(e2, st);
        evs.push_back(e2);
    };
    // outer blocks of LU_OB columns (four panels): each panel brought up to
    // date and factored (its interchanges applied) in turn, the block's U
    // rows by 64-row triangular solves, then one trailing update with
    // K = 6 x LU_OB
    auto panel = [&](int64_t k, int nbw) -> int {
        a.k = k;
        const int64_t m = n - k;
        const int G = sms;
        const size_t smem = (size_t)ceil_div(m, G) * LU_LDS * sizeof(float);
        void* args[] = {&a};
        cudaError_t le = cudaLaunchCooperativeKernel((const void*)lu_panel_kernel, dim3((unsigned)G), dim3(LU_PT),
                                                     args, smem, st);
        if (le != cudaSuccess) return set_error(MBEM_ERR_CUDA, "LU panel launch: %s", cudaGetErrorString(le));
        const int64_t others = n - nbw;
        if (others > 0) lu_swap_kernel<<<(unsigned)ceil_div(others, 256), 256, 0, st>>>(A, lda, n, k, nbw, piv);
        launches += 2;
        return MBEM_OK;
    };
    auto trsm = [&](int64_t r0, int nb, int64_t col0, int64_t ncols) {
        if (ncols <= 0) return;
        lu_block_trsm_kernel<<<(unsigned)ceil_div(ncols, 128), 128, 0, st>>>(A, lda, A + col0, lda, ncols, r0, nb, 1);
        launches++;
    };
    for (int64_t k = 0; k < n; k += LU_OB) {
        const int ob = (int)lmin(LU_OB, n - k);
        const int np = (int)ceil_div(ob, LU_NB);                 // panels in this block
        mark();
        for (int pnl = 0; pnl < np; pnl++) {
            const int64_t cp = k + (int64_t)pnl * LU_NB;            // the panel's first column (and row)
            const int wp = (int)lmin(LU_NB, k + ob - cp);
            // left-looking within the block: the earlier panels' U rows on
            // this panel's columns, each followed by its update of the rows below
            for (int q = 0; q < pnl; q++) {
                const int64_t cq = k + (int64_t)q * LU_NB;
                trsm(cq, LU_NB, cp, wp);
                if ((e = lu_block_update<LU_NB>(A, lda, cq + LU_NB, cq, n - cq - LU_NB, LU_NB, cq, cp, wp,
                                                A + (cq + LU_NB) * lda + cp, lda, Ls, Us, st)))
                    return e;
            }
            if ((e = panel(cp, wp))) return e;
        }
        mark();
        const int64_t rest = n - k - ob;
        if (rest > 0) {
            // U12 (rows k .. k + ob): panel by panel, each one's rows solved,
            // then its update of the block's later rows
            for (int q = 0; q < np; q++) {
                const int64_t cq = k + (int64_t)q * LU_NB;
                const int wq = (int)lmin(LU_NB, k + ob - cq);
                trsm(cq, wq, k + ob, rest);
                const int64_t below = k + ob - cq - wq;
                if (below > 0 &&
                    (e = lu_block_update<LU_NB>(A, lda, cq + wq, cq, below, wq, cq, k + ob, rest,
                                                A + (cq + wq) * lda + k + ob, lda, Ls, Us, st)))
                    return e;
            }
            mark();
            // A22 -= L21 U12 on the tensor cores (six BF16 piece products, K = 6 x LU_OB)
            if ((e = lu_block_update<LU_OB>(A, lda, k + ob, k, rest, ob, k, k + ob, rest,
                                            A + (k + ob) * lda + k + ob, lda, Ls, Us, st)))
                return e;
        } else {
            mark();
        }
    }
    mark();
    if (g_lu_timing && !evs.empty()) {
        cudaEventSynchronize(evs.back());
        // marks per outer block: start, after its panels, after its U rows; then the next start
        for (size_t i = 0; i + 3 < evs.size(); i += 3)
            for (int ph = 0; ph < 3; ph++) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, evs[i + ph], evs[i + ph + 1]);
                g_lu_phase_ms[ph] += ms;
            }
        for (auto e2 : evs) cudaEventDestroy(e2);
    }
    e = launch_status("lu_factor", (int)launches);
    if (e) return e;
    if ((e = tc_gemm_check(st))) return e;
    int flag = 0;
    ce = cudaStreamSynchronize(st);
    if (ce == cudaSuccess) ce = cudaMemcpyFromSymbol(&flag, g_lu_wait_error, sizeof(int));
    if (ce != cudaSuccess) return set_error(MBEM_ERR_CUDA, "LU sync: %s", cudaGetErrorString(ce));
    if (flag) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_lu_wait_error, &zero, sizeof(int));
        return set_error(MBEM_ERR_WAIT, "an LU panel grid barrier ran out of time");
    }
    return MBEM_OK;
}

void mbem_lu_stats(int timing, double* phase_ms) {
    if (phase_ms)
        for (int i = 0; i < 3; i++) phase_ms[i] = g_lu_phase_ms[i];
    for (int i = 0; i < 3; i++) g_lu_phase_ms[i] = 0.0;
    g_lu_timing = timing != 0;
}

// x = (P L U)^-1 b for one right-hand side: b, x FP64 (n); perm (device,
// n) = the row permutation of the pivots (perm[i] = original row now at i);
// xf: n floats of scratch.
int mbem_lu_solve_f32(const float* LU, int64_t lda, int64_t n, const int32_t* perm, const double* b, double* x,
                      float* xf, void* stream) {
    MBEM_REQUIRE(LU && perm && b && x && xf && n >= 1 && lda >= n, MBEM_ERR_ARG, "bad LU solve arguments");
    cudaStream_t st = (cudaStream_t)stream;
    lu_permute_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(b, perm, n, xf);
    int64_t launches = 1;
    // L y = P b, forward by blocks
    for (int64_t r0 = 0; r0 < n; r0 += LU_NB) {
        const int nb = (int)lmin(LU_NB, n - r0);
        lu_tri_block_kernel<<<1, 256, 0, st>>>(LU, lda, xf, r0, nb, 1);
        if (r0 + nb < n)
            lu_gemv_update_kernel<<<(unsigned)ceil_div((n - r0 - nb) * 32, 256), 256, 0, st>>>(LU, lda, xf, r0 + nb,
                                                                                             n, r0, nb);
        launches += 2;
    }
    // U x = y, backward by blocks
    for (int64_t r0 = ((n - 1) / LU_NB) * LU_NB; r0 >= 0; r0 -= LU_NB) {
        const int nb = (int)lmin(LU_NB, n - r0);
        lu_tri_block_kernel<<<1, 256, 0, st>>>(LU, lda, xf, r0, nb, 0);
        if (r0 > 0)
            lu_gemv_update_kernel<<<(unsigned)ceil_div(r0 * 32, 256), 256, 0, st>>>(LU, lda, xf, 0, r0, r0, nb);
        launches += 2;
    }
    lu_widen_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(xf, n, x);
    return launch_status("lu_solve", (int)launches + 1);
}

// x = (P L U)^-T b = P^T L^-T U^-T b for one right-hand side (the
// condition estimator's second product); arguments as mbem_lu_solve_f32.
int mbem_lu_solve_t_f32(const float* LU, int64_t lda, int64_t n, const int32_t* perm, const double* b, double* x,
                        float* xf, void* stream) {
    MBEM_REQUIRE(LU && perm && b && x && xf && n >= 1 && lda >= n, MBEM_ERR_ARG, "bad LU solve arguments");
    cudaStream_t st = (cudaStream_t)stream;
    lu_narrow_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(b, n, xf);
    int64_t launches = 1;
    // U^T w = b, forward by blocks
    for (int64_t r0 = 0; r0 < n; r0 += LU_NB) {
        const int nb = (int)lmin(LU_NB, n - r0);
        lu_tri_block_t_kernel<<<1, LU_NB, 0, st>>>(LU, lda, xf, r0, nb, 1);
        if (r0 + nb < n)
            lu_gemv_update_t_kernel<<<(unsigned)ceil_div(n - r0 - nb, 256), 256, 0, st>>>(LU, lda, xf, r0 + nb, n,
                                                                                          r0, nb);
        launches += 2;
    }
    // L^T z = w, backward by blocks
    for (int64_t r0 = ((n - 1) / LU_NB) * LU_NB; r0 >= 0; r0 -= LU_NB) {
        const int nb = (int)lmin(LU_NB, n - r0);
        lu_tri_block_t_kernel<<<1, LU_NB, 0, st>>>(LU, lda, xf, r0, nb, 0);
        if (r0 > 0)
            lu_gemv_update_t_kernel<<<(unsigned)ceil_div(r0, 256), 256, 0, st>>>(LU, lda, xf, 0, r0, r0, nb);
        launches += 2;
    }
    lu_scatter_widen_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(xf, perm, n, x);
    return launch_status("lu_solve_t", (int)launches + 1);
}

size_t mbem_lu_solve_many_workspace_size(int64_t n, int64_t k) {
    return ((size_t)n * k * sizeof(float) + 255) / 256 * 256 + ((size_t)n * LU_K6 * 2 + 255) / 256 * 256 +
           ((size_t)k * LU_K6 * 2 + 255) / 256 * 256;
}

// X = (P L U)^-1 B for k right-hand sides (B, X row-major FP64 n x k at ldb,
// ldx): blocked triangular solves, each 64-row block's triangle by
// lu_block_trsm_kernel and the update of the rows below (forward) or above
// (backward) as a tensor-core GEMM of six BF16 piece products.
int mbem_lu_solve_many_f32(const float* LU, int64_t lda, int64_t n, const int32_t* perm, const double* B,
                           int64_t ldb, int64_t k, double* X, int64_t ldx, void* work, size_t work_bytes,
                           void* stream) {
    MBEM_REQUIRE(LU && perm && B && X && n >= 1 && k >= 1 && lda >= n && ldb >= k && ldx >= k, MBEM_ERR_ARG,
                 "bad LU multi-solve arguments");
    const size_t need = mbem_lu_solve_many_workspace_size(n, k);
    MBEM_REQUIRE(work && work_bytes >= need, MBEM_ERR_SIZE, "LU multi-solve workspace %zu < %zu bytes", work_bytes,
                 need);
    cudaStream_t st = (cudaStream_t)stream;
    char* w = (char*)work;
    float* X32 = (float*)w;
    w += ((size_t)n * k * sizeof(float) + 255) / 256 * 256;
    uint16_t* Lp = (uint16_t*)w;
    w += ((size_t)n * LU_K6 * 2 + 255) / 256 * 256;
    uint16_t* Xp = (uint16_t*)w;
    const unsigned g_nk = (unsigned)ceil_div(n * k, 256);
    lu_gather_rows_kernel<<<g_nk, 256, 0, st>>>(B, ldb, perm, n, k, X32, k);
    int64_t launches = 1;
    int e;
    for (int64_t r0 = 0; r0 < n; r0 += LU_NB) {
        const int nb = (int)lmin(LU_NB, n - r0);
        lu_block_trsm_kernel<<<(unsigned)ceil_div(k, 128), 128, 0, st>>>(LU, lda, X32, k, k, r0, nb, 1);
        launches++;
        const int64_t below = n - r0 - nb;
        if (below > 0) {
            lu_split_rows_kernel<LU_NB><<<(unsigned)ceil_div(below * LU_NB, 256), 256, 0, st>>>(LU, lda, r0 + nb, r0,
                                                                                               nb, below, Lp);
            lu_split_cols_kernel<LU_NB><<<(unsigned)ceil_div(k, 32), 256, 0, st>>>(X32, k, r0, 0, nb, k, Xp);
            launches += 2;
            if ((e = gemm_bf16_sub(Lp, LU_K6, Xp, LU_K6, below, k, LU_K6, X32 + (r0 + nb) * k, k, st))) return e;
        }
    }
    for (int64_t r0 = ((n - 1) / LU_NB) * LU_NB; r0 >= 0; r0 -= LU_NB) {
        const int nb = (int)lmin(LU_NB, n - r0);
        lu_block_trsm_kernel<<<(unsigned)ceil_div(k, 128), 128, 0, st>>>(LU, lda, X32, k, k, r0, nb, 0);
        launches++;
        if (r0 > 0) {
            lu_split_rows_kernel<LU_NB><<<(unsigned)ceil_div(r0 * LU_NB, 256), 256, 0, st>>>(LU, lda, 0, r0, nb, r0,
                                                                                            Lp);
            lu_split_cols_kernel<LU_NB><<<(unsigned)ceil_div(k, 32), 256, 0, st>>>(X32, k, r0, 0, nb, k, Xp);
            launches += 2;
            if ((e = gemm_bf16_sub(Lp, LU_K6, Xp, LU_K6, r0, k, LU_K6, X32, k, st))) return e;
        }
    }
    lu_widen_rows_kernel<<<g_nk, 256, 0, st>>>(X32, k, n, k, X, ldx);
    if ((e = launch_status("lu_solve_many", (int)launches + 1))) return e;
    return tc_gemm_check(st);
}

}  // extern "C"
