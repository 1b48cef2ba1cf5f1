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
constexpr int KV_MAXV = 64;                  // vectors per multi-dot pass

// partial[b * k + i] = sum over block b's columns of V[i, c] * w[c]
__global__ void __launch_bounds__(KV_THREADS)
multidot_partial_kernel(const double* __restrict__ V, int64_t ldv, int k, int64_t n,
                        const double* __restrict__ w, double* __restrict__ partial) {
    __shared__ double red[KV_THREADS / 32][KV_MAXV];
    const int64_t c0 = (int64_t)blockIdx.x * KV_COLS + 2 * threadIdx.x;
    double w0 = 0.0, w1 = 0.0;
    if (c0 < n) w0 = w[c0];
    if (c0 + 1 < n) w1 = w[c0 + 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int i = 0; i < k; i++) {
        const double* v = V + (int64_t)i * ldv;
        double p = 0.0;
        if (c0 < n) p = v[c0] * w0;
        if (c0 + 1 < n) p = fma(v[c0 + 1], w1, p);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
        if (lane == 0) red[wid][i] = p;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < k; i += KV_THREADS) {
        double s = 0.0;
        for (int q = 0; q < KV_THREADS / 32; q++) s += red[q][i];
        partial[(int64_t)blockIdx.x * k + i] = s;
    }
}

// h[i] (+)= sum_b partial[b * k + i], in block order
__global__ void multidot_final_kernel(const double* __restrict__ partial, int nblocks, int k, int accumulate,
                                      double* __restrict__ h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; b++) s += partial[(int64_t)b * k + i];
    h[i] = accumulate ? h[i] + s : s;
}

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

// v_out = v_in * (1 / sqrt(*nrm2)), nrm2 on the device
__global__ void scale_by_rnorm_kernel(const double* __restrict__ v_in, double* __restrict__ v_out, int64_t n,
                                      const double* __restrict__ nrm2) {
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
proj_partial_kernel(const double* __restrict__ vin, URanges ur, double* __restrict__ partial) {
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

__global__ void __launch_bounds__(PROJ_THREADS)
proj_apply_kernel(const double* __restrict__ vin, double* __restrict__ vout, int64_t n, URanges ur,
                  const double* __restrict__ partial, int nparts) {
    __shared__ double mean[3];
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int b = 0; b < nparts; b++) s += partial[3 * b + threadIdx.x];
        int64_t total = 0;
        for (int q = 0; q < ur.n; q++) total += ur.len[q];
        // Z_k = 1/sqrt(M) on component-k u entries: Z (Z^T v) = sum / M
        mean[threadIdx.x] = (total > 0) ? s / (double)(total / 3) : 0.0;
    }
    __syncthreads();
    for (int64_t c = (int64_t)blockIdx.x * PROJ_THREADS + threadIdx.x; c < n;
         c += (int64_t)gridDim.x * PROJ_THREADS) {
        double m = 0.0;
        for (int q = 0; q < ur.n; q++)
            if (c >= ur.off[q] && c < ur.off[q] + ur.len[q]) m = mean[(c - ur.off[q]) % 3];
        vout[c] = vin[c] - m;
    }
}

// vout = P vin (vout may alias vin); partial holds 3 * PROJ_BLOCKS doubles
static int project(const double* vin, double* vout, int64_t n, const URanges& ur, double* partial,
                   cudaStream_t st) {
    proj_partial_kernel<<<PROJ_BLOCKS, PROJ_THREADS, 0, st>>>(vin, ur, partial);
    const unsigned g = (unsigned)lmin(ceil_div(n, PROJ_THREADS), 4 * 152);
    proj_apply_kernel<<<g, PROJ_THREADS, 0, st>>>(vin, vout, n, ur, partial, PROJ_BLOCKS);
    return launch_status("project", 2);
}


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
    double* partial;  // nblocks * (m+1)
    double* h;        // m+2
    double* h2;       // m+2
    double* y;        // m
    double* scal;     // 8
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
    tmp.scal = take(8);
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

    int proj(const double* in, double* out) {
        if (!deflate) {
            if (in != out) cudaMemcpyAsync(out, in, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
            return launch_status("copy", 0);
        }
        return project(in, out, n, ur, W.proj, st);
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
    // h[0..k) (+)= V[0..k) . w
    int multidot(const double* V, int k, const double* w, double* h, int accumulate) {
        for (int i0 = 0; i0 < k; i0 += KV_MAXV) {
            const int kc = min(KV_MAXV, k - i0);
            multidot_partial_kernel<<<(unsigned)nb, KV_THREADS, 0, st>>>(V + (int64_t)i0 * n, n, kc, n, w,
                                                                        W.partial);
            multidot_final_kernel<<<1, 64, 0, st>>>(W.partial, (int)nb, kc, accumulate, h + i0);
            count_launches(2);
        }
        return launch_status("multidot", 0);
    }
    int multiaxpy(double* w, const double* V, int k, const double* h, double sign) {
        for (int i0 = 0; i0 < k; i0 += KV_MAXV) {
            const int kc = min(KV_MAXV, k - i0);
            multiaxpy_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(w, V + (int64_t)i0 * n, n, kc, n,
                                                                       h + i0, sign);
            count_launches(1);
        }
        return launch_status("multiaxpy", 0);
    }
    int norm2(const double* v, double* out_dev) { return multidot(v, 1, v, out_dev, 0); }
};

// ---------------------------------------------------------------------------
// The BF16 inner solve (precond kind 3): up to `k` GMRES steps from zero on
// P (A16 + near) P. The Arnoldi steps (CGS2, as in FGMRES) write each
// Hessenberg column straight into device memory. With rtol = 0 the k steps
// run with no host synchronisation and the host reads the (k+1) x k matrix
// once; with rtol > 0 it reads each new column, applies the Givens rotations
// as it goes and stops once the residual estimate is below rtol |P r|. Then
// z = V y from the small least-squares solution. A column whose new norm is
// zero (an invariant Krylov space) ends the basis.
// ---------------------------------------------------------------------------
__global__ void add_vec_kernel(double* __restrict__ h, const double* __restrict__ d, int k) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < k) h[i] += d[i];
}

// inner steps and applications since the last mbem_inner_bf16_stats call,
// and (when timing is on) the device time of their BF16 products
static int64_t g_inner_steps = 0, g_inner_applies = 0;
static int g_inner_timing = 0;
static double g_inner_matvec_ms = 0.0;

struct InnerWork {
    double* V;        // (k+1, n)
    double* w;        // n
    double* partial;  // nblocks * (k+1)
    double* H;        // k columns of (k+2): h[0..j], |w|^2 at j+1; then beta^2
    double* h2;       // k+1
    double* y;        // k
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
    t.H = take((size_t)(k + 1) * (k + 2));
    t.h2 = take(k + 1);
    t.y = take(k);
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
    const int ldh = k + 2;
    double* beta2 = I.H + (size_t)k * ldh;
    const unsigned gn = (unsigned)ceil_div(n, 256);
    const bool adaptive = p->rtol > 0.0;

    if ((e = F.proj(r, I.w))) return e;
    if ((e = F.norm2(I.w, beta2))) return e;
    scale_by_rnorm_kernel<<<gn, 256, 0, st>>>(I.w, I.V, n, beta2);
    count_launches(1);
    cudaMemsetAsync(z, 0, n * sizeof(double), st);
    double beta = -1.0;
    if (adaptive) {
        cudaMemcpyAsync(&beta, beta2, sizeof(double), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("inner solve sync", 0);
        beta = sqrt(beta);
        if (!(beta > 0.0)) return launch_status("inner solve zero rhs", 0);
    }
    // Givens least squares min |beta e1 - Hbar y| (la/solver.py:188-210),
    // one column at a time; returns true when the basis ends at column j
    std::vector<double> R((size_t)k * k, 0.0), g(k + 1, 0.0), cs(k), sn(k), y(k, 0.0);
    int used = 0;
    auto absorb = [&](int j, const double* hc) -> bool {
        std::vector<double> col(j + 2);
        for (int i = 0; i <= j; i++) col[i] = hc[i];
        col[j + 1] = sqrt(fmax(hc[j + 1], 0.0));
        for (int i = 0; i < j; i++) {
            const double a = col[i], b = col[i + 1];
            col[i] = cs[i] * a + sn[i] * b;
            col[i + 1] = -sn[i] * a + cs[i] * b;
        }
        const double den = sqrt(col[j] * col[j] + col[j + 1] * col[j + 1]);
        if (den == 0.0) return true;
        cs[j] = col[j] / den;
        sn[j] = col[j + 1] / den;
        col[j] = den;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        for (int i = 0; i <= j; i++) R[(size_t)i * k + j] = col[i];
        used = j + 1;
        if (col[j + 1] == 0.0) return true;                         // invariant Krylov space: exact
        return adaptive && fabs(g[j + 1]) < p->rtol * beta;
    };
    if (adaptive) g[0] = beta;
    std::vector<double> hcol(k + 2);
    for (int j = 0; j < k; j++) {
        const double* vj = I.V + (int64_t)j * n;
        double* hc = I.H + (size_t)j * ldh;
        if (p->precond) {
            // right preconditioning: the step multiplies A16 by P M v_j
            if ((e = precond_apply(p->precond, p->precond_state, vj, I.t, st))) return e;
            if ((e = F.proj(I.t, I.t))) return e;
            vj = I.t;
        }
        if (g_inner_timing) {
            cudaEvent_t ev[2];
            cudaEventCreate(&ev[0]);
            cudaEventCreate(&ev[1]);
            cudaEventRecord(ev[0], st);
            e = bf16_matvec(p->A16, p->ld16, n, n, p->n_near, p->near, vj, I.w, I.xf, st);
            cudaEventRecord(ev[1], st);
            F.pending.push_back({ev[0], ev[1]});
            if (e) return e;
        } else if ((e = bf16_matvec(p->A16, p->ld16, n, n, p->n_near, p->near, vj, I.w, I.xf, st))) {
            return e;
        }
        if ((e = F.proj(I.w, I.w))) return e;
        if ((e = F.multidot(I.V, j + 1, I.w, hc, 0))) return e;
        if ((e = F.multiaxpy(I.w, I.V, j + 1, hc, -1.0))) return e;
        if ((e = F.multidot(I.V, j + 1, I.w, I.h2, 0))) return e;
        if ((e = F.multiaxpy(I.w, I.V, j + 1, I.h2, -1.0))) return e;
        add_vec_kernel<<<1, 64, 0, st>>>(hc, I.h2, j + 1);
        count_launches(1);
        if ((e = F.norm2(I.w, hc + (j + 1)))) return e;
        if (adaptive) {
            cudaMemcpyAsync(hcol.data(), hc, (j + 2) * sizeof(double), cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("inner solve sync", 0);
            if (absorb(j, hcol.data())) break;
        }
        if (j + 1 < k) {
            scale_by_rnorm_kernel<<<gn, 256, 0, st>>>(I.w, I.V + (int64_t)(j + 1) * n, n, hc + (j + 1));
            count_launches(1);
        }
    }
    if (!adaptive) {
        std::vector<double> H((size_t)(k + 1) * ldh);
        cudaMemcpyAsync(H.data(), I.H, H.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("inner solve sync", 0);
        beta = sqrt(H[(size_t)k * ldh]);
        if (!(beta > 0.0)) return launch_status("inner solve zero rhs", 0);
        g[0] = beta;
        for (int j = 0; j < k; j++)
            if (absorb(j, H.data() + (size_t)j * ldh)) break;
    }
    for (int i = used - 1; i >= 0; i--) {
        double s2 = g[i];
        for (int q = i + 1; q < used; q++) s2 -= R[(size_t)i * k + q] * y[q];
        y[i] = s2 / R[(size_t)i * k + i];
    }
    g_inner_steps += used;
    g_inner_applies += 1;
    if (!adaptive && cudaStreamSynchronize(st) != cudaSuccess) return launch_status("inner solve sync", 0);
    F.collect_times();
    g_inner_matvec_ms += F.matvec_ms;
    if (used == 0) return launch_status("inner solve", 0);
    cudaMemcpyAsync(I.y, y.data(), used * sizeof(double), cudaMemcpyHostToDevice, st);
    if (p->precond) {
        // z = P M (V y)
        cudaMemsetAsync(I.w, 0, n * sizeof(double), st);
        if ((e = F.multiaxpy(I.w, I.V, used, I.y, 1.0))) return e;
        if ((e = precond_apply(p->precond, p->precond_state, I.w, z, st))) return e;
        if ((e = F.proj(z, z))) return e;
    } else if ((e = F.multiaxpy(z, I.V, used, I.y, 1.0))) {
        return e;
    }
    // the host vector y must outlive the copy
    if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("inner solve sync", 0);
    return launch_status("inner solve", 0);
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

    double* history = rep->history;
    memset(rep, 0, sizeof(*rep));
    rep->history = history;
    std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m, 0.0), sn(m, 0.0), g(m + 1, 0.0), hcol(m + 2);
    double bnorm2 = 0.0, tmp;

    // b' = P b (kept in W.r until the first residual overwrites it)
    if ((e = F.proj(b, W.r))) return e;
    if ((e = F.norm2(W.r, W.scal))) return e;
    cudaMemcpyAsync(&bnorm2, W.scal, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("fgmres sync", 0);
    const double bnorm = sqrt(bnorm2);
    double* bproj = W.w;   // hold P b in w across cycles would clash; recompute each cycle instead
    (void)bproj;
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
        if ((e = F.norm2(W.r, W.scal))) return e;
        cudaMemcpyAsync(&tmp, W.scal, sizeof(double), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("fgmres sync", 0);
        const double beta = sqrt(tmp);
        arnoldi = beta / bnorm;
        if (arnoldi < prm->rtol) {
            rnorm2_final = tmp;
            break;
        }
        const int mm = min(m, maxiter - total);
        std::fill(H.begin(), H.end(), 0.0);
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        scale_by_rnorm_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(W.r, W.V, n, W.scal);
        count_launches(1);
        int jdone = 0;
        for (int j = 0; j < mm; j++) {
            double* vj = W.V + (int64_t)j * n;
            double* vn = W.V + (int64_t)(j + 1) * n;
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
            if ((e = F.multidot(W.V, j + 1, W.w, W.h, 0))) return e;
            if ((e = F.multiaxpy(W.w, W.V, j + 1, W.h, -1.0))) return e;
            if ((e = F.multidot(W.V, j + 1, W.w, W.h2, 0))) return e;
            if ((e = F.multiaxpy(W.w, W.V, j + 1, W.h2, -1.0))) return e;
            if ((e = F.norm2(W.w, W.h + (j + 1)))) return e;
            scale_by_rnorm_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(W.w, vn, n, W.h + (j + 1));
            count_launches(1);
            cudaMemcpyAsync(hcol.data(), W.h, (j + 2) * sizeof(double), cudaMemcpyDeviceToHost, st);
            std::vector<double> h2col(j + 1);
            cudaMemcpyAsync(h2col.data(), W.h2, (j + 1) * sizeof(double), cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("fgmres sync", 0);
            for (int i = 0; i <= j; i++) H[(size_t)i * m + j] = hcol[i] + h2col[i];
            H[(size_t)(j + 1) * m + j] = sqrt(hcol[j + 1]);
            // apply accumulated Givens rotations, then form a new one (solver.py:188-205)
            for (int i = 0; i < j; i++) {
                const double hi = H[(size_t)i * m + j], hi1 = H[(size_t)(i + 1) * m + j];
                H[(size_t)i * m + j] = cs[i] * hi + sn[i] * hi1;
                H[(size_t)(i + 1) * m + j] = -sn[i] * hi + cs[i] * hi1;
            }
            const double hjj = H[(size_t)j * m + j], hj1 = H[(size_t)(j + 1) * m + j];
            const double den = sqrt(hjj * hjj + hj1 * hj1);
            if (den == 0.0) {
                // exact breakdown with a zero pivot: the Krylov space is
                // invariant and this column adds nothing; finish with the
                // iterate of the columns before it
                jdone = j;
                breakdown = true;
                break;
            }
            cs[j] = fabs(hjj) > 0 ? fabs(hjj) / den : 0.0;
            sn[j] = fabs(hjj) > 0 ? (hjj / fabs(hjj)) * hj1 / den : 1.0;
            H[(size_t)j * m + j] = cs[j] * hjj + sn[j] * hj1;
            H[(size_t)(j + 1) * m + j] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            total++;
            jdone = j + 1;
            arnoldi = fabs(g[j + 1]) / bnorm;
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
            // back substitution (solver.py:503-510), then x += V[:j]^T y
            std::vector<double> y(jdone, 0.0);
            for (int i = jdone - 1; i >= 0; i--) {
                double s = g[i];
                for (int q = i + 1; q < jdone; q++) s -= H[(size_t)i * m + q] * y[q];
                y[i] = s / H[(size_t)i * m + i];
            }
            cudaMemcpyAsync(W.y, y.data(), jdone * sizeof(double), cudaMemcpyHostToDevice, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("fgmres sync", 0);
            if ((e = F.multiaxpy(x, flexible ? W.Z : W.V, jdone, W.y, 1.0))) return e;
            x_zero = false;
        }
        restarts++;
        if (stagnated) break;
    }
    // true residual (solver.py:234) and the zero-mean representative P x
    // (P A P x = P A P (P x): projecting x leaves the residual unchanged)
    if (rnorm2_final < 0.0) {
        if ((e = F.proj(b, W.r))) return e;
        if (!x_zero) {
            if ((e = F.op(x, W.w))) return e;
            axpby_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(W.r, W.w, n, -1.0, 1.0);
            count_launches(1);
        }
        if ((e = F.norm2(W.r, W.scal))) return e;
        cudaMemcpyAsync(&tmp, W.scal, sizeof(double), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("fgmres sync", 0);
    } else {
        tmp = rnorm2_final;
    }
    if ((e = F.proj(x, x))) return e;
    if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("fgmres sync", 0);
    if (mop && (e = mixed_wait_check(st))) return e;
    rep->true_relres = sqrt(tmp) / bnorm;
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
