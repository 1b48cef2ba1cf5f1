// Many right-hand sides at once: the vector kernels of batched GMRES (k
// independent Krylov iterations that share one tensor-core GEMM per step),
// the BF16 copy of the operator that GEMM reads, and the FP64-accurate
// residual R = B - A X of the mixed operator for a block of right-hand sides
// (FP32 far field with double-float accumulation, FP64 near blocks).
//
// Vectors of a block are RHS-major: (k, n) row-major, one row per right-hand
// side, so a row is one solve's vector and the GEMM's K-major operand is a
// row block. Every reduction runs in a fixed order.
#include <math.h>
#include <string.h>

#include <cuda_bf16.h>

#include "common.cuh"

namespace mbem {

constexpr int BT = 256;

__device__ __forceinline__ double block_sum256(double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < BT / 32; w++) s += red[w];
    return s;
}

// ---------------------------------------------------------------------------
// BF16 copies of the operator
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint16_t to_bf16(float x) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}

__global__ void f32_to_bf16_kernel(const float* __restrict__ A, int64_t lda, int64_t rows, int64_t cols,
                                   uint16_t* __restrict__ out, int64_t ldo) {
    const int64_t r = blockIdx.y;
    for (int64_t c = (int64_t)blockIdx.x * BT + threadIdx.x; c < cols; c += (int64_t)gridDim.x * BT)
        out[r * ldo + c] = to_bf16(A[r * lda + c]);
}

__global__ void f64_to_bf16_kernel(const double* __restrict__ A, int64_t lda, int64_t rows, int64_t cols,
                                   uint16_t* __restrict__ out, int64_t ldo) {
    const int64_t r = blockIdx.y;
    for (int64_t c = (int64_t)blockIdx.x * BT + threadIdx.x; c < cols; c += (int64_t)gridDim.x * BT)
        out[r * ldo + c] = to_bf16((float)A[r * lda + c]);
}

// hi = bf16(A), lo = bf16(A - hi): A = hi + lo to about 2^-16
__global__ void f32_to_bf16x2_kernel(const float* __restrict__ A, int64_t lda, int64_t cols,
                                     uint16_t* __restrict__ hi, uint16_t* __restrict__ lo, int64_t ldo) {
    const int64_t r = blockIdx.y;
    for (int64_t c = (int64_t)blockIdx.x * BT + threadIdx.x; c < cols; c += (int64_t)gridDim.x * BT) {
        const float v = A[r * lda + c];
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        hi[r * ldo + c] = __bfloat16_as_ushort(h);
        lo[r * ldo + c] = to_bf16(v - __bfloat162float(h));
    }
}

__global__ void f64_to_bf16x2_kernel(const double* __restrict__ A, int64_t lda, int64_t cols,
                                     uint16_t* __restrict__ hi, uint16_t* __restrict__ lo, int64_t ldo) {
    const int64_t r = blockIdx.y;
    for (int64_t c = (int64_t)blockIdx.x * BT + threadIdx.x; c < cols; c += (int64_t)gridDim.x * BT) {
        const double v = A[r * lda + c];
        const __nv_bfloat16 h = __float2bfloat16_rn((float)v);
        hi[r * ldo + c] = __bfloat16_as_ushort(h);
        lo[r * ldo + c] = to_bf16((float)(v - (double)__bfloat162float(h)));
    }
}

// the near 3x3 blocks of a mixed operator: hi (and lo, when given) of
// A32 + near on their entries; one thread per field point
__global__ void near_to_bf16x2_kernel(const float* __restrict__ A32, int64_t lda, mbem_near_blocks nb,
                                      uint16_t* __restrict__ hi, uint16_t* __restrict__ lo, int64_t ldo) {
    const int64_t f = (int64_t)blockIdx.x * BT + threadIdx.x;
    if (f >= nb.n_field) return;
    for (int64_t q = nb.rowptr[f]; q < nb.rowptr[f + 1]; q++) {
        const int64_t c0 = nb.col0 + 3 * nb.cols[q];
        for (int a = 0; a < 3; a++) {
            const int64_t r = nb.row0 + 3 * f + a;
            for (int b = 0; b < 3; b++) {
                const double v = (double)A32[r * lda + c0 + b] + nb.vals[9 * q + 3 * a + b];
                const __nv_bfloat16 h = __float2bfloat16_rn((float)v);
                hi[r * ldo + c0 + b] = __bfloat16_as_ushort(h);
                if (lo) lo[r * ldo + c0 + b] = to_bf16((float)(v - (double)__bfloat162float(h)));
            }
        }
    }
}

// the near 3x3 blocks: out = bf16(A32 + near) on their entries; one thread
// per (field point, near block)
__global__ void near_to_bf16_kernel(const float* __restrict__ A32, int64_t lda, mbem_near_blocks nb,
                                    uint16_t* __restrict__ out, int64_t ldo) {
    const int64_t f = (int64_t)blockIdx.x * BT + threadIdx.x;
    if (f >= nb.n_field) return;
    for (int64_t q = nb.rowptr[f]; q < nb.rowptr[f + 1]; q++) {
        const int64_t c0 = nb.col0 + 3 * nb.cols[q];
        for (int a = 0; a < 3; a++) {
            const int64_t r = nb.row0 + 3 * f + a;
            for (int b = 0; b < 3; b++)
                out[r * ldo + c0 + b] = to_bf16((float)((double)A32[r * lda + c0 + b] + nb.vals[9 * q + 3 * a + b]));
        }
    }
}

// ---------------------------------------------------------------------------
// batched Arnoldi vector kernels (FP32 vectors, FP64 reductions)
// ---------------------------------------------------------------------------
// H[i, r] = V[i, r, :] . W[r, :]; a block per (i, r)
__global__ void __launch_bounds__(BT)
batch_dots_kernel(const float* __restrict__ V, int64_t k, int64_t n, const float* __restrict__ W,
                  double* __restrict__ H) {
    __shared__ double red[BT / 32];
    const int64_t i = blockIdx.y, r = blockIdx.x;
    const float* v = V + (i * k + r) * n;
    const float* w = W + r * n;
    float s = 0.0f;
    for (int64_t t = threadIdx.x; t < n; t += BT) s = fmaf(v[t], w[t], s);
    const double tot = block_sum256((double)s, red);
    if (threadIdx.x == 0) H[i * k + r] = tot;
}

// W[r, :] += alpha sum_i H[i, r] V[i, r, :]
__global__ void __launch_bounds__(BT)
batch_axpy_kernel(float* __restrict__ W, const float* __restrict__ V, int n_vec, const double* __restrict__ H,
                  double alpha, int64_t k, int64_t n) {
    const int64_t r = blockIdx.y;
    const int64_t t = (int64_t)blockIdx.x * BT + threadIdx.x;
    if (t >= n) return;
    double s = 0.0;
    for (int i = 0; i < n_vec; i++) s += H[(int64_t)i * k + r] * (double)V[((int64_t)i * k + r) * n + t];
    W[r * n + t] = (float)((double)W[r * n + t] + alpha * s);
}

// norms[r] = |W[r]|, V[r] = W[r] / norms[r] (zero rows stay zero), Vbf its BF16 copy
template <typename TIN>
__global__ void __launch_bounds__(BT)
batch_normalize_kernel(const TIN* __restrict__ W, int64_t n, double* __restrict__ norms, float* __restrict__ V,
                       uint16_t* __restrict__ Vbf) {
    __shared__ double red[BT / 32];
    const int64_t r = blockIdx.x;
    const TIN* w = W + r * n;
    double s = 0.0;
    for (int64_t t = threadIdx.x; t < n; t += BT) s += (double)w[t] * (double)w[t];
    const double nrm = sqrt(block_sum256(s, red));
    if (threadIdx.x == 0) norms[r] = nrm;
    const double inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
    for (int64_t t = threadIdx.x; t < n; t += BT) {
        const float v = (float)((double)w[t] * inv);
        V[r * n + t] = v;
        if (Vbf) Vbf[r * n + t] = to_bf16(v);
    }
}

// X[r, :] += sum_i Y[i, r] V[i, r, :]  (X FP64)
__global__ void __launch_bounds__(BT)
batch_update_kernel(double* __restrict__ X, const float* __restrict__ V, int n_vec, const double* __restrict__ Y,
                    int64_t k, int64_t n) {
    const int64_t r = blockIdx.y;
    const int64_t t = (int64_t)blockIdx.x * BT + threadIdx.x;
    if (t >= n) return;
    double s = 0.0;
    for (int i = 0; i < n_vec; i++) s += Y[(int64_t)i * k + r] * (double)V[((int64_t)i * k + r) * n + t];
    X[r * n + t] += s;
}

// X[r] -= Z Z^T X[r] for the rigid translations of the u-ranges (per
// component: the mean over the range's nodes, every range together)
template <typename T>
__global__ void __launch_bounds__(BT)
batch_project_kernel(T* __restrict__ X, int64_t n, URanges ur) {
    __shared__ double red[BT / 32];
    __shared__ double mean[3];
    const int64_t r = blockIdx.x;
    T* x = X + r * n;
    int64_t count = 0;
    for (int q = 0; q < ur.n; q++) count += ur.len[q] / 3;
    for (int c = 0; c < 3; c++) {
        double s = 0.0;
        for (int q = 0; q < ur.n; q++)
            for (int64_t t = threadIdx.x; 3 * t < ur.len[q]; t += BT) s += (double)x[ur.off[q] + 3 * t + c];
        const double tot = block_sum256(s, red);
        if (threadIdx.x == 0) mean[c] = count > 0 ? tot / (double)count : 0.0;
    }
    __syncthreads();
    for (int q = 0; q < ur.n; q++)
        for (int64_t t = threadIdx.x; t < ur.len[q]; t += BT) {
            const int c = (int)(t % 3);
            x[ur.off[q] + t] = (T)((double)x[ur.off[q] + t] - mean[c]);
        }
}

// ---------------------------------------------------------------------------
// R = B - A X for a block: FP32 far field with double-float accumulation,
// FP64 near blocks
// ---------------------------------------------------------------------------
constexpr int DF_ROWS = 64, DF_RHS = 64, DF_K = 16;

__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float p) {
    const float t = __fadd_rn(hi, p);
    const float bp = __fsub_rn(t, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    hi = t;
    lo = __fadd_rn(lo, e);
}

// Y[r, row] = sum_j A32[row, j] X[r, j]: a block per (64 rows, 64 RHS), a
// thread per (4 rows, 4 RHS); every product a x_hi exact (TwoProd), a x_lo
// rounded, sums in hi/lo pairs
__global__ void __launch_bounds__(BT)
df_gemm_kernel(const float* __restrict__ A, int64_t lda, int64_t n_rows, int64_t n_cols,
               const double* __restrict__ X, int64_t k, double* __restrict__ Y) {
    __shared__ float As[DF_K][DF_ROWS + 4];
    __shared__ float Xh[DF_K][DF_RHS + 4], Xl[DF_K][DF_RHS + 4];
    const int64_t row0 = (int64_t)blockIdx.x * DF_ROWS, rhs0 = (int64_t)blockIdx.y * DF_RHS;
    const int tr = threadIdx.x % 16, tc = threadIdx.x / 16;    // rows tr + 16a, RHS tc + 16b
    float hi[4][4], lo[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) hi[a][b] = lo[a][b] = 0.0f;
    for (int64_t j0 = 0; j0 < n_cols; j0 += DF_K) {
        for (int e = threadIdx.x; e < DF_ROWS * DF_K; e += BT) {
            const int i = e / DF_K, j = e % DF_K;      // i: row (and RHS) within the tile, j: column
            const int64_t gr = row0 + i, gc = j0 + j;
            As[j][i] = (gr < n_rows && gc < n_cols) ? A[gr * lda + gc] : 0.0f;
            const int64_t rr = rhs0 + i;
            const double xv = (rr < k && gc < n_cols) ? X[rr * n_cols + gc] : 0.0;
            const float xh = (float)xv;
            Xh[j][i] = xh;
            Xl[j][i] = (float)(xv - (double)xh);
        }
        __syncthreads();
#pragma unroll 4
        for (int j = 0; j < DF_K; j++) {
            float av[4], xh[4], xl[4];
#pragma unroll
            for (int a = 0; a < 4; a++) av[a] = As[j][tr + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; b++) {
                xh[b] = Xh[j][tc + 16 * b];
                xl[b] = Xl[j][tc + 16 * b];
            }
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    const float p = __fmul_rn(av[a], xh[b]);
                    const float err = __fmaf_rn(av[a], xh[b], -p);
                    two_sum_acc(hi[a][b], lo[a][b], p);
                    lo[a][b] = __fadd_rn(lo[a][b], __fmaf_rn(av[a], xl[b], err));
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int64_t gr = row0 + tr + 16 * a, rr = rhs0 + tc + 16 * b;
            if (gr < n_rows && rr < k) Y[rr * n_rows + gr] = (double)hi[a][b] + (double)lo[a][b];
        }
}

// R[r, row] = B[r, row] - Y[r, row] - (near X[r])[row]; a thread per (r, row)
__global__ void __launch_bounds__(BT)
residual_near_kernel(const double* __restrict__ B, const double* __restrict__ Yfar, const double* __restrict__ X,
                     int64_t k, int64_t n, mbem_near_blocks nb, int first, double* __restrict__ R) {
    const int64_t r = blockIdx.y;
    const int64_t row = (int64_t)blockIdx.x * BT + threadIdx.x;
    if (row >= n) return;
    double v = first ? B[r * n + row] - Yfar[r * n + row] : R[r * n + row];
    const int64_t lr = row - nb.row0;
    if (lr >= 0 && lr < 3 * nb.n_field) {
        const int64_t f = lr / 3;
        const int a = (int)(lr % 3);
        const double* x = X + r * n;
        for (int64_t q = nb.rowptr[f]; q < nb.rowptr[f + 1]; q++) {
            const int64_t c0 = nb.col0 + 3 * nb.cols[q];
            const double* blk = nb.vals + 9 * q + 3 * a;
            v -= blk[0] * x[c0] + blk[1] * x[c0 + 1] + blk[2] * x[c0 + 2];
        }
    }
    R[r * n + row] = v;
}

static int ranges_of(const int64_t* u_ranges, int n_u, URanges& ur) { return make_ranges(u_ranges, n_u, ur); }

}  // namespace mbem

using namespace mbem;

extern "C" {

int mbem_to_bf16(const void* A, int is_f64, int64_t lda, int64_t rows, int64_t cols, uint16_t* out, int64_t ldo,
                 void* stream) {
    MBEM_REQUIRE(rows >= 0 && cols >= 0 && lda >= cols && ldo >= cols && rows <= 65535 * 64, MBEM_ERR_ARG,
                 "bad BF16 conversion shape");
    MBEM_REQUIRE(rows * cols == 0 || (A && out), MBEM_ERR_ARG, "NULL conversion pointers");
    if (rows * cols == 0) return MBEM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    for (int64_t r0 = 0; r0 < rows; r0 += 65535) {
        const int64_t nr = lmin(65535, rows - r0);
        const dim3 grid((unsigned)lmin(ceil_div(cols, BT), 64), (unsigned)nr);
        if (is_f64)
            f64_to_bf16_kernel<<<grid, BT, 0, st>>>((const double*)A + r0 * lda, lda, nr, cols, out + r0 * ldo, ldo);
        else
            f32_to_bf16_kernel<<<grid, BT, 0, st>>>((const float*)A + r0 * lda, lda, nr, cols, out + r0 * ldo, ldo);
        count_launches(1);
    }
    return launch_status("to_bf16", 0);
}

int mbem_to_bf16x2(const void* A, int is_f64, int64_t lda, int64_t rows, int64_t cols, uint16_t* hi, uint16_t* lo,
                   int64_t ldo, void* stream) {
    MBEM_REQUIRE(rows >= 0 && cols >= 0 && lda >= cols && ldo >= cols, MBEM_ERR_ARG, "bad BF16 split shape");
    MBEM_REQUIRE(rows * cols == 0 || (A && hi && lo), MBEM_ERR_ARG, "NULL split pointers");
    cudaStream_t st = (cudaStream_t)stream;
    for (int64_t r0 = 0; r0 < rows; r0 += 65535) {
        const int64_t nr = lmin(65535, rows - r0);
        const dim3 grid((unsigned)lmin(ceil_div(cols, BT), 64), (unsigned)nr);
        if (is_f64)
            f64_to_bf16x2_kernel<<<grid, BT, 0, st>>>((const double*)A + r0 * lda, lda, cols, hi + r0 * ldo,
                                                     lo + r0 * ldo, ldo);
        else
            f32_to_bf16x2_kernel<<<grid, BT, 0, st>>>((const float*)A + r0 * lda, lda, cols, hi + r0 * ldo,
                                                     lo + r0 * ldo, ldo);
        count_launches(1);
    }
    return launch_status("to_bf16x2", 0);
}

int mbem_mixed_to_bf16x2(const mbem_mixed_operator* op, uint16_t* hi, uint16_t* lo, int64_t ldo, void* stream) {
    MBEM_REQUIRE(op && op->A32 && hi && ldo >= op->n_cols, MBEM_ERR_ARG, "bad mixed operator or output");
    int e = lo ? mbem_to_bf16x2(op->A32, 0, op->ld32, op->n_rows, op->n_cols, hi, lo, ldo, stream)
               : mbem_to_bf16(op->A32, 0, op->ld32, op->n_rows, op->n_cols, hi, ldo, stream);
    if (e) return e;
    for (int t = 0; t < op->n_near; t++) {
        const mbem_near_blocks& nb = op->near[t];
        if (nb.n_field == 0) continue;
        near_to_bf16x2_kernel<<<(unsigned)ceil_div(nb.n_field, BT), BT, 0, (cudaStream_t)stream>>>(op->A32, op->ld32,
                                                                                                   nb, hi, lo, ldo);
        if ((e = launch_status("near_to_bf16x2_kernel"))) return e;
    }
    return MBEM_OK;
}

int mbem_mixed_to_bf16(const mbem_mixed_operator* op, uint16_t* out, int64_t ldo, void* stream) {
    MBEM_REQUIRE(op && op->A32 && out && ldo >= op->n_cols, MBEM_ERR_ARG, "bad mixed operator or output");
    int e = mbem_to_bf16(op->A32, 0, op->ld32, op->n_rows, op->n_cols, out, ldo, stream);
    if (e) return e;
    for (int t = 0; t < op->n_near; t++) {
        const mbem_near_blocks& nb = op->near[t];
        if (nb.n_field == 0) continue;
        near_to_bf16_kernel<<<(unsigned)ceil_div(nb.n_field, BT), BT, 0, (cudaStream_t)stream>>>(op->A32, op->ld32,
                                                                                                 nb, out, ldo);
        if ((e = launch_status("near_to_bf16_kernel"))) return e;
    }
    return MBEM_OK;
}

int mbem_batch_dots(const float* V, int n_vec, const float* W, int64_t k, int64_t n, double* H, void* stream) {
    MBEM_REQUIRE(n_vec >= 1 && n_vec <= 65535 && k >= 1 && k <= INT32_MAX && n >= 1 && V && W && H, MBEM_ERR_ARG,
                 "bad batched dots");
    batch_dots_kernel<<<dim3((unsigned)k, (unsigned)n_vec), BT, 0, (cudaStream_t)stream>>>(V, k, n, W, H);
    return launch_status("batch_dots_kernel");
}

int mbem_batch_axpy(float* W, const float* V, int n_vec, const double* H, double alpha, int64_t k, int64_t n,
                    void* stream) {
    MBEM_REQUIRE(n_vec >= 1 && k >= 1 && k <= 65535 && n >= 1 && V && W && H, MBEM_ERR_ARG, "bad batched axpy");
    batch_axpy_kernel<<<dim3((unsigned)ceil_div(n, BT), (unsigned)k), BT, 0, (cudaStream_t)stream>>>(W, V, n_vec, H,
                                                                                                   alpha, k, n);
    return launch_status("batch_axpy_kernel");
}

int mbem_batch_normalize(const void* W, int w_is_f64, int64_t k, int64_t n, double* norms, float* V, uint16_t* Vbf,
                         void* stream) {
    MBEM_REQUIRE(k >= 1 && n >= 1 && W && norms && V, MBEM_ERR_ARG, "bad batched normalize");
    if (w_is_f64)
        batch_normalize_kernel<double><<<(unsigned)k, BT, 0, (cudaStream_t)stream>>>((const double*)W, n, norms, V,
                                                                                    Vbf);
    else
        batch_normalize_kernel<float><<<(unsigned)k, BT, 0, (cudaStream_t)stream>>>((const float*)W, n, norms, V,
                                                                                   Vbf);
    return launch_status("batch_normalize_kernel");
}

int mbem_batch_update(double* X, const float* V, int n_vec, const double* Y, int64_t k, int64_t n, void* stream) {
    MBEM_REQUIRE(n_vec >= 1 && k >= 1 && k <= 65535 && n >= 1 && X && V && Y, MBEM_ERR_ARG, "bad batched update");
    batch_update_kernel<<<dim3((unsigned)ceil_div(n, BT), (unsigned)k), BT, 0, (cudaStream_t)stream>>>(X, V, n_vec,
                                                                                                     Y, k, n);
    return launch_status("batch_update_kernel");
}

int mbem_batch_project(void* X, int is_f64, int64_t k, int64_t n, const int64_t* u_ranges, int n_u_ranges,
                       void* stream) {
    URanges ur;
    int e = ranges_of(u_ranges, n_u_ranges, ur);
    if (e) return e;
    MBEM_REQUIRE(k >= 1 && n >= 1 && X, MBEM_ERR_ARG, "bad batched projection");
    if (ur.n == 0) return MBEM_OK;
    if (is_f64)
        batch_project_kernel<double><<<(unsigned)k, BT, 0, (cudaStream_t)stream>>>((double*)X, n, ur);
    else
        batch_project_kernel<float><<<(unsigned)k, BT, 0, (cudaStream_t)stream>>>((float*)X, n, ur);
    return launch_status("batch_project_kernel");
}

size_t mbem_batch_residual_workspace_size(int64_t k, int64_t n) { return (size_t)k * n * sizeof(double); }

int mbem_batch_residual_mixed(const mbem_mixed_operator* op, const double* B, const double* X, int64_t k, double* R,
                              void* work, size_t work_bytes, void* stream) {
    MBEM_REQUIRE(op && op->A32 && op->n_rows == op->n_cols && B && X && R && k >= 1 && k <= 65535, MBEM_ERR_ARG,
                 "bad batched residual");
    const int64_t n = op->n_rows;
    MBEM_REQUIRE(work && work_bytes >= mbem_batch_residual_workspace_size(k, n), MBEM_ERR_SIZE,
                 "batched residual workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    double* Y = static_cast<double*>(work);
    df_gemm_kernel<<<dim3((unsigned)ceil_div(n, DF_ROWS), (unsigned)ceil_div(k, DF_RHS)), BT, 0, st>>>(
        op->A32, op->ld32, n, n, X, k, Y);
    int e = launch_status("df_gemm_kernel");
    if (e) return e;
    const dim3 grid((unsigned)ceil_div(n, BT), (unsigned)k);
    if (op->n_near == 0) {
        mbem_near_blocks none;
        memset(&none, 0, sizeof(none));
        residual_near_kernel<<<grid, BT, 0, st>>>(B, Y, X, k, n, none, 1, R);
        return launch_status("residual_near_kernel");
    }
    for (int t = 0; t < op->n_near; t++) {
        residual_near_kernel<<<grid, BT, 0, st>>>(B, Y, X, k, n, op->near[t], t == 0, R);
        if ((e = launch_status("residual_near_kernel"))) return e;
    }
    return MBEM_OK;
}

}  // extern "C"
