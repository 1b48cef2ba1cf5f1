// Dense-system kernels of the calibrated dense backend and the deflated
// FGMRES that solves it, FP64 (sm_103a).
//
// The matvec streams A once from HBM with 128-bit loads (4 rows per warp so
// each x load from L2 serves four rows); every reduction runs in a fixed
// order (per-block partials, then one ordered pass), so results are
// bit-reproducible run to run. The Arnoldi basis of an 83k-unknown system
// at restart 50 is ~34 MB and stays L2-resident.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <utility>
#include <vector>

#include "common.cuh"

namespace mbem {

// ---------------------------------------------------------------------------
// calibration row sums: out[r, j] (+)= alpha * sum_c A[r, 3c + j]
// ---------------------------------------------------------------------------
__global__ void rowsum3_kernel(const double* __restrict__ A, int64_t ld, int64_t n_rows, int64_t n_cols,
                               double alpha, int accumulate, double* __restrict__ out) {
    const int64_t r = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (r >= n_rows) return;
    const double* row = A + r * ld;
    double acc[3] = {0.0, 0.0, 0.0};
    // lane l visits columns l, l+32, ...; column c belongs to component c % 3
    int j = lane % 3;
    for (int64_t c = lane; c < n_cols; c += 32) {
        acc[j] += row[c];
        j += 2;                 // (c + 32) % 3 == (c % 3 + 2) % 3
        if (j >= 3) j -= 3;
    }
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const double v = alpha * acc[k];
            out[3 * r + k] = accumulate ? out[3 * r + k] + v : v;
        }
    }
}

// ---------------------------------------------------------------------------
// free-term diagonal spread over the element's nodes by the collocation shape
// ---------------------------------------------------------------------------
struct ShapeK {
    double w[36];
};

__global__ void add_block_diag_kernel(double* __restrict__ A, int64_t ld, const double* __restrict__ D,
                                      int64_t n_c, int K, ShapeK shape) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_c) return;
    const int64_t s = c / K;
    const int kc = (int)(c % K);
    for (int k = 0; k < K; k++) {
        const double w = shape.w[kc * K + k];
        if (w == 0.0) continue;
        const int64_t col = 3 * (K * s + k);
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) A[(3 * c + a) * ld + col + b] += w * D[9 * c + 3 * a + b];
    }
}

// ---------------------------------------------------------------------------
// Row triples into per-node frames: rows (3c, 3c+1, 3c+2) of A (and of b)
// become F_c times them (equations.py:467-473, the einsum of apply_fault_rows).
// One thread per (node, column); a warp reads 32 consecutive columns.
// ---------------------------------------------------------------------------
__global__ void rotate_row_triples_kernel(double* __restrict__ A, int64_t ld, int64_t n_cols,
                                          double* __restrict__ b, int64_t n_nodes,
                                          const double* __restrict__ F) {
    const int64_t c = blockIdx.y;
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const double* f = F + 9 * c;
    if (j < n_cols) {
        double* a0 = A + (3 * c) * ld + j;
        const double x0 = a0[0], x1 = a0[ld], x2 = a0[2 * ld];
        a0[0] = (f[0] * x0 + f[1] * x1) + f[2] * x2;
        a0[ld] = (f[3] * x0 + f[4] * x1) + f[5] * x2;
        a0[2 * ld] = (f[6] * x0 + f[7] * x1) + f[8] * x2;
    }
    if (b != nullptr && blockIdx.x == 0 && threadIdx.x == 0) {
        double* bb = b + 3 * c;
        const double x0 = bb[0], x1 = bb[1], x2 = bb[2];
        bb[0] = (f[0] * x0 + f[1] * x1) + f[2] * x2;
        bb[1] = (f[3] * x0 + f[4] * x1) + f[5] * x2;
        bb[2] = (f[6] * x0 + f[7] * x1) + f[8] * x2;
    }
}

// ---------------------------------------------------------------------------
// y = alpha A x + beta y: 4 rows per warp, 128-bit streaming loads of A
// ---------------------------------------------------------------------------
constexpr int GEMV_ROWS = 4;
constexpr int GEMV_THREADS = 256;

__global__ void __launch_bounds__(GEMV_THREADS)
dgemv_vec_kernel(const double* __restrict__ A, int64_t ld, int64_t n_rows, int64_t n_cols,
                 const double* __restrict__ x, double alpha, double beta, double* __restrict__ y) {
    const int64_t warp = (int64_t)blockIdx.x * (GEMV_THREADS / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    const int64_t r0 = warp * GEMV_ROWS;
    if (r0 >= n_rows) return;
    const int nr = (int)lmin(GEMV_ROWS, n_rows - r0);
    double acc[GEMV_ROWS] = {0.0, 0.0, 0.0, 0.0};
    const int64_t n2 = n_cols / 2;
    const double2* x2 = reinterpret_cast<const double2*>(x);
    const double2* rows[GEMV_ROWS];
#pragma unroll
    for (int i = 0; i < GEMV_ROWS; i++)
        rows[i] = reinterpret_cast<const double2*>(A + (r0 + min(i, nr - 1)) * ld);
    for (int64_t c = lane; c < n2; c += 32) {
        const double2 xv = __ldg(x2 + c);
#pragma unroll
        for (int i = 0; i < GEMV_ROWS; i++) {
            const double2 av = __ldcs(rows[i] + c);
            acc[i] = fma(av.x, xv.x, acc[i]);
            acc[i] = fma(av.y, xv.y, acc[i]);
        }
    }
    if ((n_cols & 1) && lane == 0) {
        const double xv = x[n_cols - 1];
#pragma unroll
        for (int i = 0; i < GEMV_ROWS; i++)
            acc[i] = fma(A[(r0 + min(i, nr - 1)) * ld + n_cols - 1], xv, acc[i]);
    }
#pragma unroll
    for (int i = 0; i < GEMV_ROWS; i++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
    if (lane < nr) {
        double v = acc[0];
#pragma unroll
        for (int i = 1; i < GEMV_ROWS; i++)
            if (lane == i) v = acc[i];
        const int64_t r = r0 + lane;
        y[r] = (beta == 0.0) ? alpha * v : alpha * v + beta * y[r];
    }
}

__global__ void __launch_bounds__(GEMV_THREADS)
dgemv_scalar_kernel(const double* __restrict__ A, int64_t ld, int64_t n_rows, int64_t n_cols,
                    const double* __restrict__ x, double alpha, double beta, double* __restrict__ y) {
    const int64_t r = (int64_t)blockIdx.x * (GEMV_THREADS / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (r >= n_rows) return;
    double acc = 0.0;
    for (int64_t c = lane; c < n_cols; c += 32) acc = fma(A[r * ld + c], x[c], acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[r] = (beta == 0.0) ? alpha * acc : alpha * acc + beta * y[r];
}

int dgemv(const double* A, int64_t ld, int64_t n_rows, int64_t n_cols, const double* x, double alpha,
          double beta, double* y, cudaStream_t st) {
    if (n_rows == 0) return MBEM_OK;
    const bool vec = ((uintptr_t)A % 16 == 0) && ((uintptr_t)x % 16 == 0) && (ld % 2 == 0);
    if (vec) {
        const int64_t warps = ceil_div(n_rows, GEMV_ROWS);
        dgemv_vec_kernel<<<(unsigned)ceil_div(warps, GEMV_THREADS / 32), GEMV_THREADS, 0, st>>>(
            A, ld, n_rows, n_cols, x, alpha, beta, y);
    } else {
        dgemv_scalar_kernel<<<(unsigned)ceil_div(n_rows, GEMV_THREADS / 32), GEMV_THREADS, 0, st>>>(
            A, ld, n_rows, n_cols, x, alpha, beta, y);
    }
    return launch_status("dgemv");
}

// ---------------------------------------------------------------------------
// Y = A X, X and Y row-major (n, k): one warp per row, k <= 64 per pass
// ---------------------------------------------------------------------------
__global__ void dgemm_multi_kernel(const double* __restrict__ A, int64_t ld, int64_t n_rows, int64_t n_cols,
                                   const double* __restrict__ X, int64_t k, int64_t k0, int kc,
                                   double* __restrict__ Y) {
    const int64_t r = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (r >= n_rows) return;
    double acc[64];
    for (int q = 0; q < kc; q++) acc[q] = 0.0;
    for (int64_t c = lane; c < n_cols; c += 32) {
        const double a = A[r * ld + c];
        const double* xr = X + c * k + k0;
        for (int q = 0; q < kc; q++) acc[q] = fma(a, xr[q], acc[q]);
    }
    for (int q = 0; q < kc; q++) {
        double v = acc[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) Y[r * k + k0 + q] = v;
    }
}

// ---------------------------------------------------------------------------
// Krylov vector kernels (fixed-order reductions)
// ---------------------------------------------------------------------------
constexpr int KV_THREADS = 256;
constexpr int KV_COLS = 2 * KV_THREADS;      // columns per block
constexpr int KV_MAXV = 64;                  // vectors per pass over shared memory

// w[c] += sign * sum_i V[i, c] h[i]
__global__ void multiaxpy_kernel(double* __restrict__ w, const double* __restrict__ V, int64_t ldv, int k,
                                 int64_t n, const double* __restrict__ h, double sign) {
    __shared__ double hs[KV_MAXV];
    for (int i = threadIdx.x; i < k; i += blockDim.x) hs[i] = sign * h[i];
    __syncthreads();
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    double acc = w[c];
    for (int i = 0; i < k; i++) acc = fma(V[(int64_t)i * ldv + c], hs[i], acc);
    w[c] = acc;
}

// v_out = v_in * (1 / sqrt(*nrm2)), nrm2 on the device; a set *stop returns at once
__global__ void scale_by_rnorm_kernel(const double* __restrict__ v_in, double* __restrict__ v_out, int64_t n,
                                      const double* __restrict__ nrm2, const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double s = *nrm2;
    const double inv = (s > 0.0 ? 1.0 / sqrt(s) : 0.0);
    v_out[c] = v_in[c] * inv;
}

__global__ void axpby_kernel(double* __restrict__ y, const double* __restrict__ x, int64_t n, double a,
                             double b) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) y[c] = a * x[c] + b * y[c];
}

// ---------------------------------------------------------------------------
// deflation projection: subtract, per component, the mean over the u-slots
// ---------------------------------------------------------------------------
// Two passes over the whole grid: per-block partial sums of each component
// over the u-slots (fixed block count, fixed order), then every block forms
// the three means from the partials and subtracts them from its entries.
constexpr int PROJ_THREADS = 256;
constexpr int PROJ_BLOCKS = 128;     // partial sums: 3 * PROJ_BLOCKS doubles

__global__ void __launch_bounds__(PROJ_THREADS)
proj_partial_kernel(const double* __restrict__ vin, URanges ur, double* __restrict__ partial,
                    const int* __restrict__ stop) {
    if (stop && *stop) return;
    __shared__ double red[PROJ_THREADS / 32][3];
    double acc[3] = {0.0, 0.0, 0.0};
    const int64_t stride = (int64_t)gridDim.x * PROJ_THREADS;
    for (int q = 0; q < ur.n; q++) {
        const int64_t off = ur.off[q], len = ur.len[q];
        for (int64_t t = (int64_t)blockIdx.x * PROJ_THREADS + threadIdx.x; t < len; t += stride)
            acc[t % 3] += vin[off + t];
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 3; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
        if (lane == 0) red[wid][k] = acc[k];
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int w = 0; w < PROJ_THREADS / 32; w++) s += red[w][threadIdx.x];
        partial[3 * blockIdx.x + threadIdx.x] = s;
    }
}

// the three component means over the u-slots from the partial sums (threads
// 0..2 form them in block order; every thread returns after the barrier)
__device__ void proj_means(URanges ur, const double* __restrict__ partial, int nparts, double* mean) {
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int b = 0; b < nparts; b++) s += partial[3 * b + threadIdx.x];
        int64_t total = 0;
        for (int q = 0; q < ur.n; q++) total += ur.len[q];
        // Z_k = 1/sqrt(M) on component-k u entries: Z (Z^T v) = sum / M
        mean[threadIdx.x] = (total > 0) ? s / (double)(total / 3) : 0.0;
    }
    __syncthreads();
}

__device__ __forceinline__ double proj_mean_at(URanges ur, const double* mean, int64_t c) {
    double m = 0.0;
    for (int q = 0; q < ur.n; q++)
        if (c >= ur.off[q] && c < ur.off[q] + ur.len[q]) m = mean[(c - ur.off[q]) % 3];
    return m;
}

__global__ void __launch_bounds__(PROJ_THREADS)
proj_apply_kernel(const double* __restrict__ vin, double* __restrict__ vout, int64_t n, URanges ur,
                  const double* __restrict__ partial, int nparts, const int* __restrict__ stop) {
    if (stop && *stop) return;
    __shared__ double mean[3];
    proj_means(ur, partial, nparts, mean);
    for (int64_t c = (int64_t)blockIdx.x * PROJ_THREADS + threadIdx.x; c < n;
         c += (int64_t)gridDim.x * PROJ_THREADS)
        vout[c] = vin[c] - proj_mean_at(ur, mean, c);
}

// vout = P vin (vout may alias vin); partial holds 3 * PROJ_BLOCKS doubles
static int project(const double* vin, double* vout, int64_t n, const URanges& ur, double* partial,
                   cudaStream_t st, const int* stop = nullptr) {
    proj_partial_kernel<<<PROJ_BLOCKS, PROJ_THREADS, 0, st>>>(vin, ur, partial, stop);
    const unsigned g = (unsigned)lmin(ceil_div(n, PROJ_THREADS), 4 * 152);
    proj_apply_kernel<<<g, PROJ_THREADS, 0, st>>>(vin, vout, n, ur, partial, PROJ_BLOCKS, stop);
    return launch_status("project", 2);
}

// ---------------------------------------------------------------------------
// Device-side Arnoldi steps (la/solver.py:115-245, with classical
// Gram-Schmidt applied twice). After its product a GMRES step is four
// kernels: kv_dot (the projection's subtraction fused in, then the first
// pass's dots), kv_axpy_dot (the first pass's subtraction, the second pass's
// dots), kv_axpy_norm (the second subtraction, |w|^2 and the Givens rotation
// of the new Hessenberg column) and the scaling of the next basis vector.
// Each of the first three writes per-block partial sums; the last block to
// arrive adds them in block order, so the result does not depend on the
// order in which blocks finish. The rotations, the rotated right-hand side g
// and the triangular factor R stay on the device, next to a control block
// whose `stop` makes every later step kernel return at once: the host can
// enqueue step j + 1 before it has read whether step j ended the basis.
// ---------------------------------------------------------------------------
struct KrylovCtl {
    unsigned int arrive[4];   // block arrivals of the fused kernels, zero between launches
    int stop;                 // the basis has ended: the step kernels return at once
    int used;                 // columns in the least-squares problem
    int breakdown;            // a zero pivot ended the basis
    int steps;                // rotations formed
    double beta;              // |r| at the cycle start
    double beta2;             // beta^2
    double res;               // |g[used]|: the residual estimate
};

struct KvGivens {
    double* cs;
    double* sn;
    double* g;        // m + 1: the rotated beta e1
    double* R;        // m x m, column j at R + m j
    int m;
    int outer;        // 1: FGMRES's sign convention, breakdown only (the host stops it)
    double rtol;      // the inner solve stops once |g[j+1]| < rtol beta (0: never)
};

// every thread of the block calls this after its partial stores; true in the
// block that arrives last, which may then read every block's partials
__device__ __forceinline__ bool kv_last_block(unsigned int* arrive) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(arrive, 1u) == gridDim.x - 1;
    __syncthreads();
    if (last) __threadfence();
    return last;
}

__device__ __forceinline__ double kv_sum_blocks(const double* partial, int nb, int k, int i) {
    double s = 0.0;
    for (int b = 0; b < nb; b++) s += __ldcg(partial + (int64_t)b * k + i);
    return s;
}

// partial[b k + i] = sum over block b's two columns per thread of V[i, c] w[c]
__device__ void kv_block_dots(const double* __restrict__ V, int64_t ldv, int k, int64_t n, int64_t c0, double w0,
                              double w1, double* __restrict__ partial) {
    __shared__ double red[KV_THREADS / 32][KV_MAXV];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int i0 = 0; i0 < k; i0 += KV_MAXV) {
        const int kc = min(KV_MAXV, k - i0);
        for (int i = 0; i < kc; i++) {
            const double* v = V + (int64_t)(i0 + i) * ldv;
            double p = 0.0;
            if (c0 < n) p = v[c0] * w0;
            if (c0 + 1 < n) p = fma(v[c0 + 1], w1, p);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
            if (lane == 0) red[wid][i] = p;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < kc; i += KV_THREADS) {
            double s = 0.0;
            for (int q = 0; q < KV_THREADS / 32; q++) s += red[q][i];
            partial[(int64_t)blockIdx.x * k + i0 + i] = s;
        }
        __syncthreads();
    }
}

// (w0, w1) += sign * sum_i V[i, (c0, c0 + 1)] h[i], in i order
__device__ void kv_block_axpy(const double* __restrict__ V, int64_t ldv, int k, int64_t n, int64_t c0,
                              const double* __restrict__ h, double sign, double& w0, double& w1) {
    __shared__ double hs[KV_MAXV];
    for (int i0 = 0; i0 < k; i0 += KV_MAXV) {
        const int kc = min(KV_MAXV, k - i0);
        __syncthreads();
        for (int i = threadIdx.x; i < kc; i += KV_THREADS) hs[i] = sign * h[i0 + i];
        __syncthreads();
        for (int i = 0; i < kc; i++) {
            const double* v = V + (int64_t)(i0 + i) * ldv;
            if (c0 < n) w0 = fma(v[c0], hs[i], w0);
            if (c0 + 1 < n) w1 = fma(v[c0 + 1], hs[i], w1);
        }
    }
}

// partial[b] = sum over block b of w^2
__device__ void kv_block_sumsq(int64_t n, int64_t c0, double w0, double w1, double* __restrict__ partial) {
    __shared__ double red[KV_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    double p = 0.0;
    if (c0 < n) p = w0 * w0;
    if (c0 + 1 < n) p = fma(w1, w1, p);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
    if (lane == 0) red[wid] = p;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < KV_THREADS / 32; q++) s += red[q];
        partial[blockIdx.x] = s;
    }
}

// The rotation of Hessenberg column j (la/solver.py:188-210): h[0..j] are
// its Gram-Schmidt coefficients, h[j + 1] = |w|^2. The earlier rotations are
// applied, a new one zeroes the subdiagonal, g is rotated and the column
// stored in R. A zero pivot ends the basis before column j; on the inner
// solve an invariant Krylov space (|w| = 0) or a residual estimate below
// rtol beta ends it after.
__device__ void kv_givens(KrylovCtl* ctl, const double* h, int j, const KvGivens& G) {
    double* Rj = G.R + (int64_t)G.m * j;
    for (int i = 0; i <= j; i++) Rj[i] = h[i];
    const double sub = sqrt(fmax(h[j + 1], 0.0));
    for (int i = 0; i < j; i++) {
        const double a = Rj[i], b = Rj[i + 1];
        Rj[i] = G.cs[i] * a + G.sn[i] * b;
        Rj[i + 1] = -G.sn[i] * a + G.cs[i] * b;
    }
    const double hjj = Rj[j];
    const double den = sqrt(hjj * hjj + sub * sub);
    if (den == 0.0) {
        ctl->breakdown = 1;
        ctl->stop = 1;
        return;
    }
    double c, s;
    if (G.outer) {
        c = fabs(hjj) > 0 ? fabs(hjj) / den : 0.0;
        s = fabs(hjj) > 0 ? (hjj / fabs(hjj)) * sub / den : 1.0;
        Rj[j] = c * hjj + s * sub;
    } else {
        c = hjj / den;
        s = sub / den;
        Rj[j] = den;
    }
    G.cs[j] = c;
    G.sn[j] = s;
    G.g[j + 1] = -s * G.g[j];
    G.g[j] = c * G.g[j];
    ctl->used = j + 1;
    ctl->steps = j + 1;
    ctl->res = fabs(G.g[j + 1]);
    if (!G.outer && (sub == 0.0 || (G.rtol > 0.0 && ctl->res < G.rtol * ctl->beta))) ctl->stop = 1;
}

// beta = |w| for a new cycle: g[0] = beta and the control block's state
// reset (its arrival counters are zero already); a zero beta ends the basis
__global__ void __launch_bounds__(KV_THREADS)
kv_norm_init_kernel(const double* __restrict__ w, int64_t n, double* __restrict__ partial, double* __restrict__ g,
                    KrylovCtl* __restrict__ ctl) {
    const int64_t c0 = (int64_t)blockIdx.x * KV_COLS + 2 * threadIdx.x;
    const double w0 = c0 < n ? w[c0] : 0.0, w1 = c0 + 1 < n ? w[c0 + 1] : 0.0;
    kv_block_sumsq(n, c0, w0, w1, partial);
    if (!kv_last_block(&ctl->arrive[3])) return;
    if (threadIdx.x == 0) {
        const double s = kv_sum_blocks(partial, gridDim.x, 1, 0);
        const double beta = sqrt(s);
        ctl->beta = beta;
        ctl->beta2 = s;
        ctl->res = beta;
        ctl->used = ctl->steps = ctl->breakdown = 0;
        ctl->stop = !(beta > 0.0);
        g[0] = beta;
        ctl->arrive[3] = 0;
    }
}

// h[i] = V[i] . w, i < k; with proj_part, w is first replaced by P w (the
// projection's subtraction; its partial sums from proj_partial_kernel)
__global__ void __launch_bounds__(KV_THREADS)
kv_dot_kernel(const double* __restrict__ V, int64_t ldv, int k, int64_t n, double* __restrict__ w, URanges ur,
              const double* __restrict__ proj_part, double* __restrict__ partial, double* __restrict__ h,
              KrylovCtl* __restrict__ ctl) {
    if (ctl->stop) return;
    const int64_t c0 = (int64_t)blockIdx.x * KV_COLS + 2 * threadIdx.x;
    double w0 = c0 < n ? w[c0] : 0.0, w1 = c0 + 1 < n ? w[c0 + 1] : 0.0;
    if (proj_part) {
        __shared__ double mean[3];
        proj_means(ur, proj_part, PROJ_BLOCKS, mean);
        if (c0 < n) w[c0] = w0 = w0 - proj_mean_at(ur, mean, c0);
        if (c0 + 1 < n) w[c0 + 1] = w1 = w1 - proj_mean_at(ur, mean, c0 + 1);
    }
    kv_block_dots(V, ldv, k, n, c0, w0, w1, partial);
    if (!kv_last_block(&ctl->arrive[0])) return;
    for (int i = threadIdx.x; i < k; i += KV_THREADS) h[i] = kv_sum_blocks(partial, gridDim.x, k, i);
    if (threadIdx.x == 0) ctl->arrive[0] = 0;
}

// w -= V h (the first pass), then h2[i] = V[i] . w and h[i] += h2[i]
__global__ void __launch_bounds__(KV_THREADS)
kv_axpy_dot_kernel(const double* __restrict__ V, int64_t ldv, int k, int64_t n, double* __restrict__ w,
                   double* __restrict__ h, double* __restrict__ partial, double* __restrict__ h2,
                   KrylovCtl* __restrict__ ctl) {
    if (ctl->stop) return;
    const int64_t c0 = (int64_t)blockIdx.x * KV_COLS + 2 * threadIdx.x;
    double w0 = c0 < n ? w[c0] : 0.0, w1 = c0 + 1 < n ? w[c0 + 1] : 0.0;
    kv_block_axpy(V, ldv, k, n, c0, h, -1.0, w0, w1);
    if (c0 < n) w[c0] = w0;
    if (c0 + 1 < n) w[c0 + 1] = w1;
    kv_block_dots(V, ldv, k, n, c0, w0, w1, partial);
    if (!kv_last_block(&ctl->arrive[1])) return;
    for (int i = threadIdx.x; i < k; i += KV_THREADS) {
        const double s = kv_sum_blocks(partial, gridDim.x, k, i);
        h2[i] = s;
        h[i] += s;
    }
    if (threadIdx.x == 0) ctl->arrive[1] = 0;
}

// w -= V h2 (the second pass), h[k] = |w|^2 and the rotation of column k - 1
__global__ void __launch_bounds__(KV_THREADS)
kv_axpy_norm_kernel(const double* __restrict__ V, int64_t ldv, int k, int64_t n, double* __restrict__ w,
                    const double* __restrict__ h2, double* __restrict__ partial, double* __restrict__ h,
                    KvGivens G, KrylovCtl* __restrict__ ctl) {
    if (ctl->stop) return;
    const int64_t c0 = (int64_t)blockIdx.x * KV_COLS + 2 * threadIdx.x;
    double w0 = c0 < n ? w[c0] : 0.0, w1 = c0 + 1 < n ? w[c0 + 1] : 0.0;
    kv_block_axpy(V, ldv, k, n, c0, h2, -1.0, w0, w1);
    if (c0 < n) w[c0] = w0;
    if (c0 + 1 < n) w[c0 + 1] = w1;
    kv_block_sumsq(n, c0, w0, w1, partial);
    if (!kv_last_block(&ctl->arrive[2])) return;
    if (threadIdx.x == 0) {
        h[k] = kv_sum_blocks(partial, gridDim.x, 1, 0);
        kv_givens(ctl, h, k - 1, G);
        ctl->arrive[2] = 0;
    }
}

// y = R^-1 g over the columns in use: one warp, rows from the bottom, each
// row's sum by lanes then a fixed shuffle tree
constexpr int KV_MAX_BACKSOLVE = 1024;

__global__ void kv_backsolve_kernel(const KrylovCtl* __restrict__ ctl, const double* __restrict__ R, int m,
                                    const double* __restrict__ g, double* __restrict__ y) {
    __shared__ double ys[KV_MAX_BACKSOLVE];
    const int lane = threadIdx.x & 31;
    if (threadIdx.x >= 32) return;
    const int used = min(ctl->used, KV_MAX_BACKSOLVE);
    for (int i = used - 1; i >= 0; i--) {
        double s = 0.0;
        for (int q = i + 1 + lane; q < used; q += 32) s = fma(R[i + (int64_t)m * q], ys[q], s);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) ys[i] = (g[i] - s) / R[i + (int64_t)m * i];
        __syncwarp();
    }
    for (int i = lane; i < used; i += 32) y[i] = ys[i];
}

// Pinned host copies of a control block, in two slots per loop, so that the
// host reads step j - 1's while step j's copy is in flight. One small pinned
// buffer per host thread, kept for the thread's life: the inner solve uses
// slots 0-1, the FGMRES that calls it slots 2-3.
static KrylovCtl* kv_pinned_slots() {
    struct Holder {
        KrylovCtl* p = nullptr;
        ~Holder() {
            if (p) cudaFreeHost(p);
        }
    };
    thread_local Holder h;
    if (!h.p && cudaHostAlloc(reinterpret_cast<void**>(&h.p), 4 * sizeof(KrylovCtl), cudaHostAllocDefault) !=
                    cudaSuccess)
        h.p = nullptr;
    return h.p;
}

struct KvStatus {
    KrylovCtl* slot = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaStream_t st = nullptr;

    int init(cudaStream_t s, int first_slot) {
        st = s;
        KrylovCtl* base = kv_pinned_slots();
        if (!base) return set_error(MBEM_ERR_CUDA, "pinned status buffer: %s", cudaGetErrorString(cudaGetLastError()));
        slot = base + first_slot;
        for (int i = 0; i < 2; i++)
            if (cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) != cudaSuccess)
                return launch_status("status event", 0);
        return MBEM_OK;
    }
    // copy the control block after step j's kernels
    int post(const KrylovCtl* dev, int j) {
        cudaMemcpyAsync(&slot[j & 1], dev, sizeof(KrylovCtl), cudaMemcpyDeviceToHost, st);
        cudaEventRecord(ev[j & 1], st);
        return launch_status("status copy", 0);
    }
    // the control block as step j left it (waits for that step only)
    int wait(int j, KrylovCtl* out) {
        if (cudaEventSynchronize(ev[j & 1]) != cudaSuccess) return launch_status("status wait", 0);
        *out = slot[j & 1];
        return MBEM_OK;
    }
    ~KvStatus() {
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
    }
};

// ---------------------------------------------------------------------------
// FGMRES (la/solver.py:115-245) with classical Gram-Schmidt applied twice
// (CGS2) in place of the reference's modified Gram-Schmidt: the same Arnoldi
// relation to rounding, two fused passes instead of j+1 dependent ones.
// ---------------------------------------------------------------------------
struct FgmresWork {
    double* V;        // (m+1, n)
    double* Z;        // (m, n) preconditioned directions (flexible variant)
    double* w;        // n
    double* t;        // n
    double* r;        // n
    double* partial;  // nblocks * (m+2)
    double* h;        // m+2: the new column's coefficients, |w|^2 at j+1
    double* h2;       // m+2
    double* y;        // m+1
    double* cs;       // m
    double* sn;       // m
    double* g;        // m+1
    double* R;        // m x m
    KrylovCtl* ctl;
    float* xh;        // n (mixed operator: split of the matvec input)
    float* xl;        // n
    double* proj;     // 3 * PROJ_BLOCKS projection partial sums
};

static size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

static size_t fgmres_layout(int64_t n, int m, char* base, FgmresWork* w) {
    const int64_t nb = ceil_div(n, KV_COLS);
    size_t off = 0;
    auto take = [&](size_t count) {
        char* p = base ? base + off : nullptr;
        off += align_up(count * sizeof(double));
        return reinterpret_cast<double*>(p);
    };
    FgmresWork tmp;
    tmp.V = take((size_t)(m + 1) * n);
    tmp.Z = take((size_t)m * n);
    tmp.w = take(n);
    tmp.t = take(n);
    tmp.r = take(n);
    tmp.partial = take((size_t)nb * (m + 2));
    tmp.h = take(m + 2);
    tmp.h2 = take(m + 2);
    tmp.y = take(m + 1);
    tmp.cs = take(m);
    tmp.sn = take(m);
    tmp.g = take(m + 1);
    tmp.R = take((size_t)m * m);
    tmp.ctl = reinterpret_cast<KrylovCtl*>(take((sizeof(KrylovCtl) + 7) / 8));
    tmp.xh = reinterpret_cast<float*>(take((n + 1) / 2));
    tmp.xl = reinterpret_cast<float*>(take((n + 1) / 2));
    tmp.proj = take(3 * PROJ_BLOCKS);
    if (w) *w = tmp;
    return off;
}

struct Fgmres {
    const double* A;                      // dense FP64 operator, or
    const mbem_mixed_operator* mop;       // the mixed operator
    int64_t ld, n;
    URanges ur;
    bool deflate;
    cudaStream_t st;
    FgmresWork W;
    int64_t nb;

    int proj(const double* in, double* out, const int* stop = nullptr) {
        if (!deflate) {
            if (in != out) cudaMemcpyAsync(out, in, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
            return launch_status("copy", 0);
        }
        return project(in, out, n, ur, W.proj, st, stop);
    }
    // out = P A P in (uses W.t)
    int op(const double* in, double* out) {
        int e = proj(in, W.t);
        if (e) return e;
        cudaEvent_t ev[2] = {nullptr, nullptr};
        if (time_matvec) {
            cudaEventCreate(&ev[0]);
            cudaEventCreate(&ev[1]);
            cudaEventRecord(ev[0], st);
        }
        e = mop ? mixed_matvec(mop, W.t, out, W.xh, W.xl, st) : dgemv(A, ld, n, n, W.t, 1.0, 0.0, out, st);
        matvecs++;
        if (time_matvec) {
            cudaEventRecord(ev[1], st);
            pending.push_back({ev[0], ev[1]});
        }
        if (e) return e;
        return proj(out, out);
    }
    // accumulates the device time of the matvecs timed so far (after a sync)
    void collect_times() {
        for (auto& p : pending) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, p.first, p.second) == cudaSuccess) matvec_ms += ms;
            cudaEventDestroy(p.first);
            cudaEventDestroy(p.second);
        }
        pending.clear();
    }
    ~Fgmres() {
        for (auto& p : pending) {
            cudaEventDestroy(p.first);
            cudaEventDestroy(p.second);
        }
    }
    bool time_matvec = false;
    int matvecs = 0;
    double matvec_ms = 0.0;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
    int multiaxpy(double* w, const double* V, int k, const double* h, double sign) {
        for (int i0 = 0; i0 < k; i0 += KV_MAXV) {
            const int kc = min(KV_MAXV, k - i0);
            multiaxpy_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(w, V + (int64_t)i0 * n, n, kc, n,
                                                                       h + i0, sign);
            count_launches(1);
        }
        return launch_status("multiaxpy", 0);
    }
    // beta = |v| into the control block, g[0] = beta (a new cycle)
    int norm_init(const double* v, double* partial, double* g, KrylovCtl* ctl) {
        kv_norm_init_kernel<<<(unsigned)nb, KV_THREADS, 0, st>>>(v, n, partial, g, ctl);
        return launch_status("norm init", 1);
    }
    // one Arnoldi step after its product w: the CGS2 coefficients into h,
    // |w|^2 into h[k], the rotation of column k - 1, and V[k] = w / |w|
    int arnoldi(double* V, int k, double* w, double* partial, double* h, double* h2, const KvGivens& G,
                KrylovCtl* ctl, bool project_w, bool scale_next) {
        const int* stop = &ctl->stop;
        if (project_w) {
            proj_partial_kernel<<<PROJ_BLOCKS, PROJ_THREADS, 0, st>>>(w, ur, W.proj, stop);
            count_launches(1);
        }
        kv_dot_kernel<<<(unsigned)nb, KV_THREADS, 0, st>>>(V, n, k, n, w, ur, project_w ? W.proj : nullptr,
                                                           partial, h, ctl);
        kv_axpy_dot_kernel<<<(unsigned)nb, KV_THREADS, 0, st>>>(V, n, k, n, w, h, partial, h2, ctl);
        kv_axpy_norm_kernel<<<(unsigned)nb, KV_THREADS, 0, st>>>(V, n, k, n, w, h2, partial, h, G, ctl);
        if (scale_next)
            scale_by_rnorm_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(w, V + (int64_t)k * n, n, h + k, stop);
        return launch_status("arnoldi step", 3 + (scale_next ? 1 : 0));
    }
};

// ---------------------------------------------------------------------------
// The BF16 inner solve (precond kind 3): up to `k` GMRES steps from zero on
// P (A16 + near) P, every step on the device (the Arnoldi kernels above).
// The host enqueues step j + 1, then reads step j's control block from
// pinned memory; once a step ended the basis (residual estimate below
// rtol |P r|, an invariant Krylov space, or a zero pivot) it stops
// enqueueing, and the one step already queued after it returns at once.
// Then z = V y from the device back substitution. No stream-wide wait.
// ---------------------------------------------------------------------------
// inner steps and applications since the last mbem_inner_bf16_stats call,
// and (when timing is on) the device time of their BF16 products, read from
// their events at that call
static int64_t g_inner_steps = 0, g_inner_applies = 0;
static int g_inner_timing = 0;
static double g_inner_matvec_ms = 0.0;
static std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_inner_events;

struct InnerWork {
    double* V;        // (k+1, n)
    double* w;        // n
    double* partial;  // nblocks * (k+2)
    double* h;        // k+2: the new column's coefficients, |w|^2 at j+1
    double* h2;       // k+1
    double* y;        // k
    double* cs;       // k
    double* sn;       // k
    double* g;        // k+1
    double* R;        // k x k
    KrylovCtl* ctl;
    float* xf;        // n
    double* proj;     // 3 * PROJ_BLOCKS
    double* t;        // n: M v_j (right preconditioner), then V y
};

static size_t inner_layout(int64_t n, int k, char* base, InnerWork* w) {
    const int64_t nb = ceil_div(n, KV_COLS);
    size_t off = 0;
    auto take = [&](size_t count) {
        char* p = base ? base + off : nullptr;
        off += align_up(count * sizeof(double));
        return reinterpret_cast<double*>(p);
    };
    InnerWork t;
    t.V = take((size_t)(k + 1) * n);
    t.w = take(n);
    t.partial = take((size_t)nb * (k + 2));
    t.h = take(k + 2);
    t.h2 = take(k + 1);
    t.y = take(k);
    t.cs = take(k);
    t.sn = take(k);
    t.g = take(k + 1);
    t.R = take((size_t)k * k);
    t.ctl = reinterpret_cast<KrylovCtl*>(take((sizeof(KrylovCtl) + 7) / 8));
    t.xf = reinterpret_cast<float*>(take((n + 1) / 2));
    t.proj = take(3 * PROJ_BLOCKS);
    t.t = take(n);
    if (w) *w = t;
    return off;
}

int inner_bf16_apply(const void* state, const double* r, double* z, cudaStream_t st) {
    const mbem_inner_bf16* p = static_cast<const mbem_inner_bf16*>(state);
    MBEM_REQUIRE(p && p->A16 && p->n > 0 && p->ld16 >= p->n, MBEM_ERR_ARG, "bad BF16 inner solve");
    const int k = p->iterations;
    MBEM_REQUIRE(k >= 1 && k <= MBEM_INNER_MAX_ITERS, MBEM_ERR_ARG, "inner iterations must be in [1, %d]",
                 MBEM_INNER_MAX_ITERS);
    MBEM_REQUIRE(p->rtol >= 0.0 && p->rtol < 1.0, MBEM_ERR_ARG, "inner rtol must be in [0, 1)");
    MBEM_REQUIRE(p->precond == 0 || ((p->precond == 1 || p->precond == 2) && p->precond_state != nullptr),
                 MBEM_ERR_ARG, "inner preconditioner must be 0, or 1 / 2 with a state");
    const int64_t n = p->n;
    const size_t need = inner_layout(n, k, nullptr, nullptr);
    MBEM_REQUIRE(p->work && p->work_bytes >= need, MBEM_ERR_SIZE, "inner workspace %zu < %zu bytes",
                 p->work_bytes, need);
    InnerWork I;
    inner_layout(n, k, (char*)p->work, &I);
    Fgmres F;
    F.A = nullptr; F.mop = nullptr; F.ld = 0; F.n = n; F.st = st;
    F.nb = ceil_div(n, KV_COLS);
    int e = make_ranges(p->u_ranges, p->n_u_ranges, F.ur);
    if (e) return e;
    F.deflate = p->n_u_ranges > 0;
    F.W.partial = I.partial;
    F.W.proj = I.proj;
    KvStatus S;
    if ((e = S.init(st, 0))) return e;
    const KvGivens G{I.cs, I.sn, I.g, I.R, k, 0, p->rtol};
    const int* stop = &I.ctl->stop;

    // beta = |P r|, V[0] = P r / beta
    cudaMemsetAsync(I.ctl, 0, sizeof(KrylovCtl), st);
    cudaMemsetAsync(z, 0, n * sizeof(double), st);
    if ((e = F.proj(r, I.w))) return e;
    if ((e = F.norm_init(I.w, I.partial, I.g, I.ctl))) return e;
    scale_by_rnorm_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(I.w, I.V, n, &I.ctl->beta2, stop);
    count_launches(1);
    KrylovCtl seen;
    memset(&seen, 0, sizeof(seen));
    int posted = -1;
    bool ended = false;
    for (int j = 0; j < k; j++) {
        const double* vj = I.V + (int64_t)j * n;
        if (p->precond) {
            // right preconditioning: the step multiplies A16 by P M v_j
            if ((e = precond_apply(p->precond, p->precond_state, vj, I.t, st))) return e;
            if ((e = F.proj(I.t, I.t, stop))) return e;
            vj = I.t;
        }
        if (g_inner_timing) {
            cudaEvent_t ev[2];
            cudaEventCreate(&ev[0]);
            cudaEventCreate(&ev[1]);
            cudaEventRecord(ev[0], st);
            e = bf16_matvec(p->A16, p->ld16, n, n, p->n_near, p->near, vj, I.w, I.xf, st, stop);
            cudaEventRecord(ev[1], st);
            g_inner_events.push_back({ev[0], ev[1]});
            if (e) return e;
        } else if ((e = bf16_matvec(p->A16, p->ld16, n, n, p->n_near, p->near, vj, I.w, I.xf, st, stop))) {
            return e;
        }
        if ((e = F.arnoldi(I.V, j + 1, I.w, I.partial, I.h, I.h2, G, I.ctl, F.deflate, j + 1 < k))) return e;
        if ((e = S.post(I.ctl, j))) return e;
        posted = j;
        if (j >= 1) {
            if ((e = S.wait(j - 1, &seen))) return e;
            if (seen.stop) {
                ended = true;
                break;
            }
        }
    }
    if (!ended && (e = S.wait(posted, &seen))) return e;
    const int used = seen.used;
    g_inner_steps += used;
    g_inner_applies += 1;
    if (used == 0) return launch_status("inner solve", 0);       // a zero P r: z = 0
    kv_backsolve_kernel<<<1, 32, 0, st>>>(I.ctl, I.R, k, I.g, I.y);
    count_launches(1);
    if (p->precond) {
        // z = P M (V y)
        cudaMemsetAsync(I.w, 0, n * sizeof(double), st);
        if ((e = F.multiaxpy(I.w, I.V, used, I.y, 1.0))) return e;
        if ((e = precond_apply(p->precond, p->precond_state, I.w, z, st))) return e;
        if ((e = F.proj(z, z))) return e;
    } else if ((e = F.multiaxpy(z, I.V, used, I.y, 1.0))) {
        return e;
    }
    return launch_status("inner solve", 0);
}

// the device time of the inner products recorded since the last call
static void collect_inner_events() {
    for (auto& pr : g_inner_events) {
        float ms = 0.f;
        if (cudaEventSynchronize(pr.second) == cudaSuccess &&
            cudaEventElapsedTime(&ms, pr.first, pr.second) == cudaSuccess)
            g_inner_matvec_ms += ms;
        cudaEventDestroy(pr.first);
        cudaEventDestroy(pr.second);
    }
    g_inner_events.clear();
}

}  // namespace mbem

using namespace mbem;

extern "C" {

int mbem_block_rowsum3(const double* A, int64_t ld, int64_t n_rows, int64_t n_col_nodes, double alpha,
                       int accumulate, double* out, void* stream) {
    MBEM_REQUIRE(n_rows >= 0 && n_col_nodes >= 0 && ld >= 3 * n_col_nodes, MBEM_ERR_ARG,
                 "bad rowsum3 shape");
    if (n_rows == 0) return MBEM_OK;
    rowsum3_kernel<<<(unsigned)ceil_div(n_rows, 8), 256, 0, (cudaStream_t)stream>>>(
        A, ld, n_rows, 3 * n_col_nodes, alpha, accumulate, out);
    return launch_status("rowsum3_kernel");
}

int mbem_add_block_diagonal(double* A, int64_t ld, const double* D, int64_t n_c, int K, const double* shape,
                            void* stream) {
    MBEM_REQUIRE(K == 1 || K == 3 || K == 6, MBEM_ERR_ARG, "K must be 1, 3 or 6 (got %d)", K);
    MBEM_REQUIRE(n_c >= 0 && n_c % K == 0, MBEM_ERR_ARG, "n_c must be a multiple of K");
    MBEM_REQUIRE(shape != nullptr, MBEM_ERR_ARG, "shape is NULL");
    if (n_c == 0) return MBEM_OK;
    ShapeK sk;
    memset(&sk, 0, sizeof(sk));
    for (int i = 0; i < K * K; i++) sk.w[i] = shape[i];
    add_block_diag_kernel<<<(unsigned)ceil_div(n_c, 128), 128, 0, (cudaStream_t)stream>>>(A, ld, D, n_c, K, sk);
    return launch_status("add_block_diag_kernel");
}

int mbem_rotate_row_triples(double* A, int64_t ld, int64_t n_cols, double* b, int64_t n_nodes,
                            const double* frames, void* stream) {
    MBEM_REQUIRE(n_nodes >= 0 && n_cols >= 0 && ld >= n_cols, MBEM_ERR_ARG, "bad row-triple shape");
    MBEM_REQUIRE(n_nodes == 0 || (A && frames), MBEM_ERR_ARG, "NULL A or frames");
    int64_t launches = 0;
    for (int64_t c0 = 0; c0 < n_nodes; c0 += 65535) {     // grid rows per launch
        const int64_t nc = lmin(65535, n_nodes - c0);
        const dim3 grid((unsigned)lmax(1, ceil_div(n_cols, 256)), (unsigned)nc);
        rotate_row_triples_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(
            A + 3 * c0 * ld, ld, n_cols, b ? b + 3 * c0 : nullptr, nc, frames + 9 * c0);
        launches++;
    }
    return launch_status("rotate_row_triples_kernel", launches);
}

int mbem_dgemv(const double* A, int64_t ld, int64_t n_rows, int64_t n_cols, const double* x, double alpha,
               double beta, double* y, void* stream) {
    MBEM_REQUIRE(n_rows >= 0 && n_cols >= 0 && ld >= n_cols, MBEM_ERR_ARG, "bad dgemv shape");
    return dgemv(A, ld, n_rows, n_cols, x, alpha, beta, y, (cudaStream_t)stream);
}

int mbem_dgemm_multi(const double* A, int64_t ld, int64_t n_rows, int64_t n_cols, const double* X, int64_t k,
                     double* Y, void* stream) {
    MBEM_REQUIRE(n_rows >= 0 && n_cols >= 0 && ld >= n_cols && k >= 0, MBEM_ERR_ARG, "bad dgemm shape");
    for (int64_t k0 = 0; k0 < k; k0 += 64) {
        const int kc = (int)lmin(64, k - k0);
        dgemm_multi_kernel<<<(unsigned)ceil_div(n_rows, 8), 256, 0, (cudaStream_t)stream>>>(A, ld, n_rows, n_cols,
                                                                                           X, k, k0, kc, Y);
        count_launches(1);
    }
    return launch_status("dgemm_multi_kernel", 0);
}

int mbem_project_translation(const double* v_in, double* v_out, int64_t n, const int64_t* u_ranges,
                             int n_u_ranges, double* work, void* stream) {
    URanges ur;
    int e = make_ranges(u_ranges, n_u_ranges, ur);
    if (e) return e;
    MBEM_REQUIRE(work != nullptr, MBEM_ERR_ARG, "work is NULL (needs %d doubles)", 3 * PROJ_BLOCKS);
    if (n == 0) return MBEM_OK;
    return project(v_in, v_out, n, ur, work, (cudaStream_t)stream);
}

size_t mbem_inner_bf16_workspace_size(int64_t n, int iterations) {
    return inner_layout(n, iterations < 1 ? 1 : iterations, nullptr, nullptr);
}

void mbem_inner_bf16_stats(int timing, int64_t* steps, int64_t* applies, double* matvec_ms) {
    collect_inner_events();
    if (steps) *steps = g_inner_steps;
    if (applies) *applies = g_inner_applies;
    if (matvec_ms) *matvec_ms = g_inner_matvec_ms;
    g_inner_steps = g_inner_applies = 0;
    g_inner_matvec_ms = 0.0;
    g_inner_timing = timing != 0;
}

int mbem_inner_bf16_apply(const mbem_inner_bf16* p, const double* r, double* z, void* stream) {
    MBEM_REQUIRE(r != nullptr && z != nullptr && r != z, MBEM_ERR_ARG, "r and z must be distinct device vectors");
    return inner_bf16_apply(p, r, z, (cudaStream_t)stream);
}

size_t mbem_fgmres_workspace_size(int64_t n, int restart) {
    return fgmres_layout(n, restart, nullptr, nullptr);
}

static int fgmres_run(const double* A, int64_t ld, const mbem_mixed_operator* mop, int64_t n, const double* b,
                      double* x, const mbem_fgmres_params* prm, void* work, size_t work_bytes,
                      mbem_fgmres_report* rep, void* stream);

int mbem_fgmres_dense(const double* A, int64_t ld, int64_t n, const double* b, double* x,
                      const mbem_fgmres_params* prm, void* work, size_t work_bytes, mbem_fgmres_report* rep,
                      void* stream) {
    MBEM_REQUIRE(A != nullptr && ld >= n, MBEM_ERR_ARG, "bad dense operator");
    return fgmres_run(A, ld, nullptr, n, b, x, prm, work, work_bytes, rep, stream);
}

int mbem_fgmres_mixed(const mbem_mixed_operator* op, const double* b, double* x, const mbem_fgmres_params* prm,
                      void* work, size_t work_bytes, mbem_fgmres_report* rep, void* stream) {
    MBEM_REQUIRE(op != nullptr && op->A32 != nullptr && op->n_rows == op->n_cols && op->ld32 >= op->n_cols,
                 MBEM_ERR_ARG, "bad mixed operator (must be square)");
    MBEM_REQUIRE(op->n_near >= 0 && (op->n_near == 0 || op->near), MBEM_ERR_ARG, "bad near blocks");
    return fgmres_run(nullptr, 0, op, op->n_rows, b, x, prm, work, work_bytes, rep, stream);
}

}  // extern "C"

static int fgmres_run(const double* A, int64_t ld, const mbem_mixed_operator* mop, int64_t n, const double* b,
                      double* x, const mbem_fgmres_params* prm, void* work, size_t work_bytes,
                      mbem_fgmres_report* rep, void* stream) {
    MBEM_REQUIRE(prm != nullptr && rep != nullptr, MBEM_ERR_ARG, "params/report is NULL");
    MBEM_REQUIRE(n > 0, MBEM_ERR_ARG, "bad system size");
    const int m = prm->restart;
    MBEM_REQUIRE(m >= 1 && m <= 1000, MBEM_ERR_ARG, "restart must be in [1, 1000]");
    MBEM_REQUIRE(prm->precond >= 0 && prm->precond <= 3, MBEM_ERR_ARG, "unknown preconditioner %d", prm->precond);
    MBEM_REQUIRE(prm->precond == 0 || prm->precond_state != nullptr, MBEM_ERR_ARG, "preconditioner state is NULL");
    const bool flexible = prm->precond != 0;
    const size_t need = fgmres_layout(n, m, nullptr, nullptr);
    MBEM_REQUIRE(work != nullptr && work_bytes >= need, MBEM_ERR_SIZE, "workspace %zu < %zu bytes", work_bytes,
                 need);
    Fgmres F;
    F.A = A; F.mop = mop; F.ld = ld; F.n = n; F.st = (cudaStream_t)stream;
    F.nb = ceil_div(n, KV_COLS);
    fgmres_layout(n, m, (char*)work, &F.W);
    int e = make_ranges(prm->u_ranges, prm->n_u_ranges, F.ur);
    if (e) return e;
    F.deflate = prm->n_u_ranges > 0;
    F.time_matvec = prm->time_matvec != 0;
    FgmresWork& W = F.W;
    cudaStream_t st = F.st;
    KvStatus S;
    if ((e = S.init(st, 2))) return e;
    const KvGivens G{W.cs, W.sn, W.g, W.R, m, 1, 0.0};

    double* history = rep->history;
    memset(rep, 0, sizeof(*rep));
    rep->history = history;
    KrylovCtl seen;

    // |P b|
    cudaMemsetAsync(W.ctl, 0, sizeof(KrylovCtl), st);
    if ((e = F.proj(b, W.r))) return e;
    if ((e = F.norm_init(W.r, W.partial, W.g, W.ctl))) return e;
    if ((e = S.post(W.ctl, 0)) || (e = S.wait(0, &seen))) return e;
    const double bnorm = seen.beta;
    if (bnorm == 0.0) {
        cudaMemsetAsync(x, 0, n * sizeof(double), st);
        rep->converged = 1;
        return launch_status("fgmres zero rhs", 0);
    }
    const int maxiter = prm->maxiter;
    int total = 0, restarts = 0;
    double best = INFINITY;
    int best_at = 0;
    bool stagnated = false, breakdown = false;
    double arnoldi = 1.0;
    // every cycle either adds an iteration or ends the solve; the cap makes
    // termination independent of that argument
    const int max_cycles = maxiter + 2;
    int cycles = 0;
    // prm->x_is_zero: the caller's x is zero on entry, so the first residual
    // is P b with no product; the true residual of the current x, once
    // computed at a cycle start, is reused as the final one when the loop
    // ends there
    bool x_zero = prm->x_is_zero != 0;
    double rnorm2_final = -1.0;
    while (total < maxiter && !stagnated && !breakdown && cycles++ < max_cycles) {
        // r = P b - P A P x (P b itself while x is zero)
        if ((e = F.proj(b, W.r))) return e;
        if (!x_zero) {
            if ((e = F.op(x, W.w))) return e;
            axpby_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(W.r, W.w, n, -1.0, 1.0);
            count_launches(1);
        }
        // beta = |r| and g = beta e1 on the device; the host reads beta to
        // decide whether the cycle runs
        if ((e = F.norm_init(W.r, W.partial, W.g, W.ctl))) return e;
        if ((e = S.post(W.ctl, 0)) || (e = S.wait(0, &seen))) return e;
        const double beta = seen.beta;
        arnoldi = beta / bnorm;
        if (arnoldi < prm->rtol) {
            rnorm2_final = seen.beta2;
            break;
        }
        const int mm = min(m, maxiter - total);
        scale_by_rnorm_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(W.r, W.V, n, &W.ctl->beta2, nullptr);
        count_launches(1);
        int jdone = 0;
        for (int j = 0; j < mm; j++) {
            double* vj = W.V + (int64_t)j * n;
            if (flexible) {
                // z_j = M^-1 v_j, w = P A P z_j (right preconditioning, flexible: la/solver.py:160-170)
                double* zj = W.Z + (int64_t)j * n;
                if ((e = precond_apply(prm->precond, prm->precond_state, vj, zj, st))) return e;
                // keep z_j in the deflated complement: the update x += Z y
                // then never feeds the null space
                if ((e = F.proj(zj, zj))) return e;
                if ((e = F.op(zj, W.w))) return e;
            } else if ((e = F.op(vj, W.w))) {               // w = P A P v_j
                return e;
            }
            // CGS2, |w| and the rotation on the device; the host reads the
            // residual estimate for its stopping and stagnation tests (the
            // next step's preconditioner solve costs far more than this wait)
            if ((e = F.arnoldi(W.V, j + 1, W.w, W.partial, W.h, W.h2, G, W.ctl, false, true))) return e;
            if ((e = S.post(W.ctl, j)) || (e = S.wait(j, &seen))) return e;
            if (seen.breakdown) {
                // exact breakdown with a zero pivot: the Krylov space is
                // invariant and this column adds nothing; finish with the
                // iterate of the columns before it
                jdone = j;
                breakdown = true;
                break;
            }
            total++;
            jdone = j + 1;
            arnoldi = seen.res / bnorm;
            if (rep->history && total <= maxiter) rep->history[total - 1] = arnoldi;
            if (arnoldi < best / prm->stagnation_factor) {
                best = arnoldi;
                best_at = total;
            } else if (total - best_at >= prm->stagnation_window) {
                stagnated = true;
                break;
            }
            if (arnoldi < prm->rtol || total >= maxiter) break;
        }
        if (jdone > 0) {
            // back substitution (solver.py:503-510) on the device, then x += V[:j]^T y
            kv_backsolve_kernel<<<1, 32, 0, st>>>(W.ctl, W.R, m, W.g, W.y);
            count_launches(1);
            if ((e = F.multiaxpy(x, flexible ? W.Z : W.V, jdone, W.y, 1.0))) return e;
            x_zero = false;
        }
        restarts++;
        if (stagnated) break;
    }
    // true residual (solver.py:234) and the zero-mean representative P x
    // (P A P x = P A P (P x): projecting x leaves the residual unchanged)
    double rnorm2 = rnorm2_final;
    if (rnorm2 < 0.0) {
        if ((e = F.proj(b, W.r))) return e;
        if (!x_zero) {
            if ((e = F.op(x, W.w))) return e;
            axpby_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(W.r, W.w, n, -1.0, 1.0);
            count_launches(1);
        }
        if ((e = F.norm_init(W.r, W.partial, W.g, W.ctl))) return e;
        if ((e = S.post(W.ctl, 0)) || (e = S.wait(0, &seen))) return e;
        rnorm2 = seen.beta2;
    }
    if ((e = F.proj(x, x))) return e;
    if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("fgmres sync", 0);
    if (mop && (e = mixed_wait_check(st))) return e;
    rep->true_relres = sqrt(rnorm2) / bnorm;
    rep->arnoldi_relres = arnoldi;
    rep->iterations = total;
    F.collect_times();
    rep->matvecs = F.matvecs;
    rep->matvec_ms = F.matvec_ms;
    rep->restarts = restarts - 1 < 0 ? 0 : restarts - 1;
    rep->converged = rep->true_relres < prm->rtol;
    rep->stagnated = (stagnated || breakdown) && !rep->converged;
    return MBEM_OK;
}
