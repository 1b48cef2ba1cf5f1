// Learned preconditioner: block-Jacobi with a learned coarse space.
//
// The unknowns are split into the block-Jacobi chunks. Each chunk c gets six
// coarse vectors: the chunk's three translations and three learned vectors
// whose 3x3 block on node i of the chunk is phi_i, the output of a small MLP
// on the node's geometry (its place in the chunk, its normal, its slot kind,
// the shape of its neighbourhood). On node i the coarse basis is the 3x6
// block B_i = [I | phi_i]. With Phi (n x 6C) and A_c = Phi^T A Phi, the
// preconditioner is multiplicative:
//
//   y = A_c^-1 Phi^T r,   z = Phi y + BJ (r - (A Phi) y).
//
// Setup per mesh: phi (MLP forward), the chunk bases orthonormalised (the
// span is what matters; an orthonormal basis keeps A_c as well conditioned
// as A), A Phi (one pass over A), A_c, and A_c^-1 by Gauss-Jordan with
// partial pivoting (FP64). An apply is five small
// kernels plus the block-Jacobi apply; it never touches A.
//
// Training: the coarse space should hold what block-Jacobi misses, the error
// eps = A^-1 r - BJ r of training pairs. The loss is the chunk-wise
// least-squares projection error of eps onto the chunk's six vectors,
//   loss = (1/S) sum_s sum_c |eps_sc - Phi_c y_sc|^2 / |eps_s|^2,
//   y_sc = (G_c + delta I)^-1 Phi_c^T eps_sc,  G_c = Phi_c^T Phi_c,
//   delta = 1e-8 trace(G_c) / 6,
// and, y being the (regularised) minimiser, the gradient needs no
// derivative of y:
//   dloss/dphi_i = -(2/S) sum_s (eps_si - B_i y_sc) y_sc[3:6]^T / |eps_s|^2.
// MLP: MBEM_NN_FEAT -> MBEM_NN_HIDDEN (tanh) -> MBEM_NN_HIDDEN (tanh) -> 9
// (phi_i row-major); flat FP32 parameters W1 (H x F), b1, W2 (H x H), b2,
// W3 (9 x H), b3. Every reduction runs in a fixed order: training and setup
// are deterministic.
#include <math.h>

#include "common.cuh"

namespace mbem {

constexpr int NF = MBEM_NN_FEAT;
constexpr int NH = MBEM_NN_HIDDEN;
constexpr int NP = MBEM_NN_PARAMS;
constexpr int OFF_W1 = 0, OFF_B1 = NH * NF, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + 9 * NH;
static_assert(OFF_B3 + 9 == NP, "parameter layout");
constexpr int ACT = 2 * NH;          // stored activations per item (h1, h2)
constexpr int DEL = 2 * NH + 9;      // stored deltas per item (d1, d2, d3)
constexpr int NN_THREADS = 256;
constexpr int GRAD_CHUNK = 512;      // items per partial parameter-gradient sum
constexpr int NCV = 6;               // coarse vectors per chunk: 3 translations + 3 learned

// ---------------------------------------------------------------------------
// MLP forward: one thread per item (node), parameters in shared memory
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NN_THREADS)
nn_forward_kernel(const float* __restrict__ feat, int64_t E, const float* __restrict__ params,
                  float* __restrict__ act, float* __restrict__ w) {
    __shared__ float P[NP];
    for (int p = threadIdx.x; p < NP; p += NN_THREADS) P[p] = params[p];
    __syncthreads();
    const int64_t e = (int64_t)blockIdx.x * NN_THREADS + threadIdx.x;
    if (e >= E) return;
    float g[NF], h1[NH], h2[NH];
#pragma unroll
    for (int f = 0; f < NF; f++) g[f] = feat[e * NF + f];
#pragma unroll 4
    for (int o = 0; o < NH; o++) {
        float s = P[OFF_B1 + o];
#pragma unroll
        for (int f = 0; f < NF; f++) s = fmaf(P[OFF_W1 + o * NF + f], g[f], s);
        h1[o] = tanhf(s);
    }
#pragma unroll 4
    for (int o = 0; o < NH; o++) {
        float s = P[OFF_B2 + o];
#pragma unroll
        for (int i = 0; i < NH; i++) s = fmaf(P[OFF_W2 + o * NH + i], h1[i], s);
        h2[o] = tanhf(s);
    }
#pragma unroll
    for (int o = 0; o < 9; o++) {
        float s = P[OFF_B3 + o];
#pragma unroll
        for (int i = 0; i < NH; i++) s = fmaf(P[OFF_W3 + o * NH + i], h2[i], s);
        w[e * 9 + o] = s;
    }
    if (act) {
#pragma unroll
        for (int i = 0; i < NH; i++) {
            act[e * ACT + i] = h1[i];
            act[e * ACT + NH + i] = h2[i];
        }
    }
}

// ---------------------------------------------------------------------------
// coarse-space projection loss and its gradient: one CTA per chunk, one
// thread per node of the chunk
// ---------------------------------------------------------------------------
__device__ __forceinline__ double block_sum(double v, double* red) {
    // 128-thread block: warp shuffles, then the four warp sums in order
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    return ((red[0] + red[1]) + red[2]) + red[3];
}

// inverse of a symmetric positive 6x6 (Gauss-Jordan, no pivoting needed)
__device__ void inv6(double M[6][6], double R[6][6]) {
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++) R[i][j] = (i == j) ? 1.0 : 0.0;
    for (int k = 0; k < 6; k++) {
        const double d = (M[k][k] != 0.0) ? 1.0 / M[k][k] : 0.0;
        for (int j = 0; j < 6; j++) {
            M[k][j] *= d;
            R[k][j] *= d;
        }
        for (int i = 0; i < 6; i++) {
            if (i == k) continue;
            const double f = M[i][k];
            for (int j = 0; j < 6; j++) {
                M[i][j] -= f * M[k][j];
                R[i][j] -= f * R[k][j];
            }
        }
    }
}

__global__ void __launch_bounds__(128)
nn_coarse_loss_grad_kernel(const int64_t* __restrict__ chunk_ptr, const int64_t* __restrict__ dofs,
                           const float* __restrict__ phi, const float* __restrict__ eps,
                           const float* __restrict__ inv_e2, int64_t S, int64_t N, float* __restrict__ dphi,
                           double* __restrict__ partial) {
    __shared__ double red[4];
    __shared__ double Ginv[6][6];
    const int c = blockIdx.x;
    const int64_t c0 = chunk_ptr[c];
    const int m = (int)((chunk_ptr[c + 1] - c0) / 3);
    const int t = threadIdx.x;
    const bool live = t < m;
    int64_t node = 0;
    float P[9];
#pragma unroll
    for (int q = 0; q < 9; q++) P[q] = 0.0f;
    if (live) {
        node = dofs[c0 + 3 * t] / 3;
#pragma unroll
        for (int q = 0; q < 9; q++) P[q] = phi[node * 9 + q];
    }
    // G = sum_i B_i^T B_i with B_i = [I | phi_i]:
    // [[m I, sum phi_i], [sum phi_i^T, sum phi_i^T phi_i]]
    double sp[9], gl[9];
    for (int q = 0; q < 9; q++) sp[q] = block_sum(live ? (double)P[q] : 0.0, red);
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            double v = 0.0;
            for (int r = 0; r < 3; r++) v += (double)P[3 * r + a] * (double)P[3 * r + b];
            gl[3 * a + b] = block_sum(v, red);
        }
    if (t == 0) {
        double G[6][6];
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                G[a][b] = (a == b) ? (double)m : 0.0;
                G[a][3 + b] = sp[3 * a + b];
                G[3 + b][a] = sp[3 * a + b];
                G[3 + a][3 + b] = gl[3 * a + b];
            }
        double tr = 0.0;
        for (int a = 0; a < 6; a++) tr += G[a][a];
        for (int a = 0; a < 6; a++) G[a][a] += 1e-8 * tr / 6.0;
        double R[6][6];
        inv6(G, R);
        for (int a = 0; a < 6; a++)
            for (int b = 0; b < 6; b++) Ginv[a][b] = R[a][b];
    }
    __syncthreads();
    double gr[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double lsum = 0.0;
    for (int64_t s = 0; s < S; s++) {
        float ev[3] = {0.0f, 0.0f, 0.0f};
        if (live) {
            const float* es = eps + s * N + 3 * node;
            ev[0] = es[0]; ev[1] = es[1]; ev[2] = es[2];
        }
        double b[6];
        for (int k = 0; k < 3; k++) b[k] = block_sum(live ? (double)ev[k] : 0.0, red);
        for (int k = 0; k < 3; k++) {
            const double v = (double)P[k] * ev[0] + (double)P[3 + k] * ev[1] + (double)P[6 + k] * ev[2];
            b[3 + k] = block_sum(v, red);
        }
        double y[6];
        for (int a = 0; a < 6; a++) {
            double v = 0.0;
            for (int q = 0; q < 6; q++) v += Ginv[a][q] * b[q];
            y[a] = v;
        }
        if (live) {
            const double w = (double)inv_e2[s] / (double)S;
            for (int a = 0; a < 3; a++) {
                const double res = ev[a] - (y[a] + (double)P[3 * a] * y[3] + (double)P[3 * a + 1] * y[4] +
                                            (double)P[3 * a + 2] * y[5]);
                lsum += res * res * w;
                gr[3 * a] -= 2.0 * w * res * y[3];
                gr[3 * a + 1] -= 2.0 * w * res * y[4];
                gr[3 * a + 2] -= 2.0 * w * res * y[5];
            }
        }
    }
    if (live)
        for (int q = 0; q < 9; q++) dphi[node * 9 + q] = (float)gr[q];
    const double tot = block_sum(lsum, red);
    if (t == 0) partial[c] = tot;
}

__global__ void nn_sum_kernel(const double* __restrict__ partial, int64_t n, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int64_t i = 0; i < n; i++) s += partial[i];
    *out = s;
}

// ---------------------------------------------------------------------------
// MLP backward and Adam
// ---------------------------------------------------------------------------
// per-item deltas: d3 = G, d2 = (W3^T d3)(1 - h2^2), d1 = (W2^T d2)(1 - h1^2)
__global__ void __launch_bounds__(NN_THREADS)
nn_backward_items_kernel(int64_t E, const float* __restrict__ params, const float* __restrict__ act,
                         const float* __restrict__ G, float* __restrict__ del) {
    __shared__ float P[NP];
    for (int p = threadIdx.x; p < NP; p += NN_THREADS) P[p] = params[p];
    __syncthreads();
    const int64_t e = (int64_t)blockIdx.x * NN_THREADS + threadIdx.x;
    if (e >= E) return;
    float d3[9], d2[NH];
#pragma unroll
    for (int o = 0; o < 9; o++) d3[o] = G[e * 9 + o];
#pragma unroll 4
    for (int i = 0; i < NH; i++) {
        float s = 0.0f;
#pragma unroll
        for (int o = 0; o < 9; o++) s = fmaf(P[OFF_W3 + o * NH + i], d3[o], s);
        const float h = act[e * ACT + NH + i];
        d2[i] = s * (1.0f - h * h);
    }
#pragma unroll 4
    for (int i = 0; i < NH; i++) {
        float s = 0.0f;
#pragma unroll
        for (int o = 0; o < NH; o++) s = fmaf(P[OFF_W2 + o * NH + i], d2[o], s);
        const float h = act[e * ACT + i];
        del[e * DEL + i] = s * (1.0f - h * h);
    }
#pragma unroll
    for (int i = 0; i < NH; i++) del[e * DEL + NH + i] = d2[i];
#pragma unroll
    for (int o = 0; o < 9; o++) del[e * DEL + 2 * NH + o] = d3[o];
}

// partial[c][p]: the gradient contributions of the items of chunk c to
// parameter p; the threads of a warp take consecutive parameters
__global__ void __launch_bounds__(NN_THREADS)
nn_param_grad_kernel(int64_t E, const float* __restrict__ feat, const float* __restrict__ act,
                     const float* __restrict__ del, float* __restrict__ partial) {
    const int p = blockIdx.x * NN_THREADS + threadIdx.x;
    const int64_t c = blockIdx.y;
    if (p >= NP) return;
    const int64_t e0 = c * GRAD_CHUNK, e1 = lmin(E, e0 + GRAD_CHUNK);
    int di, ii = -1, istride = 0;
    const float* ibase = nullptr;
    if (p < OFF_B1) { di = p / NF; ii = p % NF; ibase = feat; istride = NF; }
    else if (p < OFF_W2) { di = p - OFF_B1; }
    else if (p < OFF_B2) { di = NH + (p - OFF_W2) / NH; ii = (p - OFF_W2) % NH; ibase = act; istride = ACT; }
    else if (p < OFF_W3) { di = NH + (p - OFF_B2); }
    else if (p < OFF_B3) { di = 2 * NH + (p - OFF_W3) / NH; ii = NH + (p - OFF_W3) % NH; ibase = act; istride = ACT; }
    else { di = 2 * NH + (p - OFF_B3); }
    float s = 0.0f;
    if (ii >= 0) {
        for (int64_t e = e0; e < e1; e++) s = fmaf(del[e * DEL + di], ibase[e * istride + ii], s);
    } else {
        for (int64_t e = e0; e < e1; e++) s += del[e * DEL + di];
    }
    partial[c * NP + p] = s;
}

__global__ void nn_param_reduce_kernel(const float* __restrict__ partial, int64_t n_chunks,
                                       float* __restrict__ grad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NP) return;
    float s = 0.0f;
    for (int64_t c = 0; c < n_chunks; c++) s += partial[c * NP + p];
    grad[p] = s;
}

__global__ void nn_adam_kernel(float* __restrict__ params, const float* __restrict__ grad, float* __restrict__ m,
                               float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                               float c1, float c2) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float g = grad[p];
    const float mp = b1 * m[p] + (1.0f - b1) * g;
    const float vp = b2 * v[p] + (1.0f - b2) * g * g;
    m[p] = mp;
    v[p] = vp;
    params[p] -= lr * (mp / c1) / (sqrtf(vp / c2) + eps);
}

// ---------------------------------------------------------------------------
// setup: A Phi, A_c = Phi^T (A Phi), A_c^-1
// ---------------------------------------------------------------------------
constexpr int APHI_ROWS = 64;     // rows of A per CTA

// APhi[r, 6c + k] = sum_{i in c} sum_a A[r, 3i + a] B_i[a][k]; a CTA per
// (chunk, 64-row tile), a warp per row, lanes along the chunk's columns
__global__ void __launch_bounds__(256)
nn_aphi_kernel(const double* __restrict__ A, int64_t ld, int64_t n, const int64_t* __restrict__ chunk_ptr,
               const int64_t* __restrict__ dofs, const float* __restrict__ basis, int64_t n_coarse,
               double* __restrict__ APhi) {
    __shared__ int64_t col[MBEM_BJ_MAX_DOF];
    __shared__ float bs[MBEM_BJ_MAX_DOF][NCV];
    const int c = blockIdx.x;
    const int64_t c0 = chunk_ptr[c];
    const int m = (int)(chunk_ptr[c + 1] - c0);
    for (int t = threadIdx.x; t < m; t += 256) {
        const int64_t d = dofs[c0 + t];
        col[t] = d;
#pragma unroll
        for (int k = 0; k < NCV; k++) bs[t][k] = basis[d * NCV + k];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t r0 = (int64_t)blockIdx.y * APHI_ROWS;
    for (int64_t r = r0 + warp; r < lmin(n, r0 + APHI_ROWS); r += 8) {
        const double* Ar = A + r * ld;
        double s[NCV] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int t = lane; t < m; t += 32) {
            const double v = Ar[col[t]];
#pragma unroll
            for (int k = 0; k < NCV; k++) s[k] += v * (double)bs[t][k];
        }
#pragma unroll
        for (int k = 0; k < NCV; k++)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s[k] += __shfl_xor_sync(0xffffffffu, s[k], o);
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < NCV; k++) APhi[r * n_coarse + NCV * c + k] = s[k];
    }
}

// Ac[6c + k, q] = sum_{d in c} basis[d][k] APhi[d, q]: a CTA per (chunk,
// 256 columns), a thread per column
__global__ void __launch_bounds__(256)
nn_coarse_matrix_kernel(const double* __restrict__ APhi, int64_t n_coarse, const int64_t* __restrict__ chunk_ptr,
                        const int64_t* __restrict__ dofs, const float* __restrict__ basis, double* __restrict__ Ac) {
    const int c = blockIdx.x;
    const int64_t q = (int64_t)blockIdx.y * 256 + threadIdx.x;
    if (q >= n_coarse) return;
    const int64_t c0 = chunk_ptr[c];
    const int m = (int)(chunk_ptr[c + 1] - c0);
    double s[NCV] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int t = 0; t < m; t++) {
        const int64_t d = dofs[c0 + t];
        const double v = APhi[d * n_coarse + q];
#pragma unroll
        for (int k = 0; k < NCV; k++) s[k] += (double)basis[d * NCV + k] * v;
    }
    for (int k = 0; k < NCV; k++) Ac[(NCV * c + k) * n_coarse + q] = s[k];
}

// Ac[p, q] += sum_j U[p, j] U[q, j]: the rank-n_shift shift that makes the
// coarse operator of a calibrated (singular) system invertible
__global__ void nn_coarse_shift_kernel(double* __restrict__ Ac, int64_t nc, const double* __restrict__ U,
                                       int n_shift) {
    const int64_t p = blockIdx.y;
    const int64_t q = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (q >= nc) return;
    double s = 0.0;
    for (int j = 0; j < n_shift; j++) s += U[p * n_shift + j] * U[q * n_shift + j];
    Ac[p * nc + q] += s;
}

// Gauss-Jordan with partial pivoting, out of place per step (Min -> Mout,
// so no thread reads an entry another is writing). gj_pivot_kernel (one
// block) finds p = argmax_{i >= k} |Min[i, k]| and 1 / Min[p, k];
// gj_update_kernel writes Mout, a thread per (row group, column): row k of
// Mout is the scaled pivot row, row p the old row k (the swap).
constexpr int GJ_ROWS = 8;        // rows of Mout per thread

__global__ void __launch_bounds__(256)
gj_pivot_kernel(const double* __restrict__ Min, int64_t m, int64_t k, int* __restrict__ piv,
                double* __restrict__ dinv, int* __restrict__ bad) {
    __shared__ double bv[256];
    __shared__ int64_t bi[256];
    double best = -1.0;
    int64_t besti = k;
    for (int64_t i = k + threadIdx.x; i < m; i += 256) {
        const double v = fabs(Min[i * m + k]);
        if (v > best) { best = v; besti = i; }
    }
    bv[threadIdx.x] = best;
    bi[threadIdx.x] = besti;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            const double ob = bv[threadIdx.x + o];
            const int64_t oi = bi[threadIdx.x + o];
            if (ob > bv[threadIdx.x] || (ob == bv[threadIdx.x] && oi < bi[threadIdx.x])) {
                bv[threadIdx.x] = ob;
                bi[threadIdx.x] = oi;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int64_t p = bi[0];
        piv[k] = (int)p;
        const double pv = Min[p * m + k];
        *dinv = (pv != 0.0) ? 1.0 / pv : 1.0;
        if (!(bv[0] > 0.0)) *bad = 1;
    }
}

__global__ void __launch_bounds__(256)
gj_update_kernel(const double* __restrict__ Min, double* __restrict__ Mout, int64_t m, int64_t k,
                 const int* __restrict__ piv, const double* __restrict__ dinv) {
    const int64_t j = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (j >= m) return;
    const int64_t p = piv[k];
    const double d = *dinv;
    const double rk = (j == k ? 1.0 : Min[p * m + j]) * d;
    const int64_t r0 = (int64_t)blockIdx.y * GJ_ROWS;
    for (int64_t i = r0; i < lmin(m, r0 + GJ_ROWS); i++) {
        const int64_t src = (i == k) ? p : (i == p ? k : i);     // the row swap
        if (i == k) {
            Mout[i * m + j] = rk;
        } else {
            const double fi = Min[src * m + k];
            Mout[i * m + j] = (j == k ? 0.0 : Min[src * m + j]) - fi * rk;
        }
    }
}

__global__ void gj_swap_columns_kernel(double* __restrict__ M, int64_t m, const int* __restrict__ piv) {
    const int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (i >= m) return;
    for (int64_t k = m - 1; k >= 0; k--) {
        const int64_t p = piv[k];
        if (p != k) {
            const double t = M[i * m + k];
            M[i * m + k] = M[i * m + p];
            M[i * m + p] = t;
        }
    }
}

// ---------------------------------------------------------------------------
// k nearest nodes of every node (the learned features' neighbourhoods): one
// thread a query node scanning all nodes through shared-memory tiles, keeping
// its k best in registers (squared FP32 distances of coordinates centred on
// the mesh's mean; ties to the lower index). The node itself comes first.
// ---------------------------------------------------------------------------
constexpr int KNN_MAX = 16, KNN_TILE = 1024, KNN_PARTS = 8, KNN_QPB = 32;   // queries a CTA of 256

__device__ __forceinline__ bool knn_before(float d, int i, float e, int j) { return d < e || (d == e && i < j); }

// KNN_PARTS threads per query node, each scanning the points j = part mod
// KNN_PARTS of every shared-memory tile and keeping its best KNN_MAX in
// registers (order: squared FP32 distance, then index; the node itself first);
// the parts' lists are then merged in shared memory.
__global__ void __launch_bounds__(256)
knn_kernel(const float* __restrict__ p, int64_t n, int k, int64_t* __restrict__ idx_out) {
    __shared__ float tile[KNN_TILE * 3];
    __shared__ float md[KNN_QPB][KNN_PARTS * KNN_MAX];
    __shared__ int mi[KNN_QPB][KNN_PARTS * KNN_MAX];
    const int ql = threadIdx.x / KNN_PARTS, part = threadIdx.x % KNN_PARTS;
    const int64_t q = (int64_t)blockIdx.x * KNN_QPB + ql;
    float qx = 0.f, qy = 0.f, qz = 0.f;
    if (q < n) { qx = p[3 * q]; qy = p[3 * q + 1]; qz = p[3 * q + 2]; }
    float bd[KNN_MAX];
    int bi[KNN_MAX];
#pragma unroll
    for (int t = 0; t < KNN_MAX; t++) { bd[t] = INFINITY; bi[t] = 0x7fffffff; }
    for (int64_t j0 = 0; j0 < n; j0 += KNN_TILE) {
        const int m = (int)lmin(KNN_TILE, n - j0);
        __syncthreads();
        for (int t = threadIdx.x; t < 3 * m; t += 256) tile[t] = p[3 * j0 + t];
        __syncthreads();
        if (q >= n) continue;
        for (int j = part; j < m; j += KNN_PARTS) {
            const float dx = tile[3 * j] - qx, dy = tile[3 * j + 1] - qy, dz = tile[3 * j + 2] - qz;
            const int jj = (int)(j0 + j);
            float d = (jj == q) ? -1.0f : fmaf(dx, dx, fmaf(dy, dy, dz * dz));    // self first
            if (!knn_before(d, jj, bd[KNN_MAX - 1], bi[KNN_MAX - 1])) continue;
            int ci = jj;
#pragma unroll
            for (int t = 0; t < KNN_MAX; t++) {                 // insertion
                if (knn_before(d, ci, bd[t], bi[t])) {
                    const float td = bd[t];
                    const int ti = bi[t];
                    bd[t] = d; bi[t] = ci;
                    d = td; ci = ti;
                }
            }
        }
    }
#pragma unroll
    for (int t = 0; t < KNN_MAX; t++) {
        md[ql][part * KNN_MAX + t] = bd[t];
        mi[ql][part * KNN_MAX + t] = bi[t];
    }
    __syncthreads();
    if (part != 0 || q >= n) return;
    // merge: the other parts' lists into this thread's (already sorted) list
    for (int e = KNN_MAX; e < KNN_PARTS * KNN_MAX; e++) {
        float d = md[ql][e];
        int ci = mi[ql][e];
        if (!knn_before(d, ci, bd[KNN_MAX - 1], bi[KNN_MAX - 1])) continue;
#pragma unroll
        for (int t = 0; t < KNN_MAX; t++) {
            if (knn_before(d, ci, bd[t], bi[t])) {
                const float td = bd[t];
                const int ti = bi[t];
                bd[t] = d; bi[t] = ci;
                d = td; ci = ti;
            }
        }
    }
#pragma unroll
    for (int t = 0; t < KNN_MAX; t++)
        if (t < k) idx_out[q * k + t] = bi[t];
}

// ---------------------------------------------------------------------------
// A Phi for the BF16 inner operator of the mixed solve (A16 far field plus
// its FP64 near blocks), stored FP32 at ldp: a CTA per (group of
// APHI16_GROUP chunks, APHI16_ROWS rows) holds the group's columns and basis
// rows in shared memory. A warp takes APHI16_RW (eight) rows at a time and two
// chunks at once, sixteen lanes a chunk over its columns (each chunk's
// columns ascending, so a lane group's loads run along the mesh's element
// runs); the six basis columns go as three packed pairs (FFMA2), and each
// chunk's 24 sums close with a four-level shuffle tree over its lanes (fixed
// order). Every APhi entry has one writer. The near blocks follow as FP32
// atomic adds (nn_aphi_near_kernel).
// ---------------------------------------------------------------------------
constexpr int APHI16_GROUP = 8, APHI16_ROWS = 128, APHI16_RW = 8, APHI16_LG = 16;

__device__ __forceinline__ float aphi_load(const uint16_t* row, int c) {
    return __uint_as_float((uint32_t)row[c] << 16);
}
__device__ __forceinline__ float aphi_load(const double* row, int c) { return (float)row[c]; }

// T = uint16_t: the BF16 inner operator's far field; T = double: a dense FP64
// operator (FP32 products: the coarse operator is a preconditioner's)
template <typename T>
__global__ void __launch_bounds__(256, 2)
nn_aphi_gather_kernel(const T* __restrict__ A16, int64_t ld16, int64_t n, const int64_t* __restrict__ chunk_ptr,
                      const int64_t* __restrict__ dofs, int64_t n_chunks, const float* __restrict__ basis,
                      float* __restrict__ APhi, int64_t ldp) {
    extern __shared__ __align__(16) float gsm[];
    constexpr int RW = APHI16_RW, LG = APHI16_LG, NG = 32 / APHI16_LG;
    const int64_t cb = (int64_t)blockIdx.x * APHI16_GROUP;
    const int64_t ce = lmin(n_chunks, cb + APHI16_GROUP);
    const int64_t d0 = chunk_ptr[cb];
    const int m = (int)(chunk_ptr[ce] - d0);
    float2* bs = reinterpret_cast<float2*>(gsm);                // [m][3] pairs of basis columns
    int* col = reinterpret_cast<int*>(gsm + (size_t)m * NCV);   // [m]
    __shared__ int cptr[APHI16_GROUP + 1];
    for (int t = threadIdx.x; t < m; t += 256) {
        const int64_t d = dofs[d0 + t];
        col[t] = (int)d;
#pragma unroll
        for (int p = 0; p < NCV / 2; p++) bs[t * 3 + p] = make_float2(basis[d * NCV + 2 * p], basis[d * NCV + 2 * p + 1]);
    }
    if (threadIdx.x <= ce - cb) cptr[threadIdx.x] = (int)(chunk_ptr[cb + threadIdx.x] - d0);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grp = lane / LG, gl = lane % LG;
    const int64_t rb = (int64_t)blockIdx.y * APHI16_ROWS;
    const int64_t r1 = lmin(n, rb + APHI16_ROWS);
    for (int64_t r0 = rb + (int64_t)warp * RW; r0 < r1; r0 += 8 * RW) {
        const T* Ar[RW];
#pragma unroll
        for (int q = 0; q < RW; q++) Ar[q] = A16 + lmin(r0 + q, n - 1) * ld16;
        for (int64_t c0 = cb; c0 < ce; c0 += NG) {
            const int64_t c = c0 + grp;
            const bool cv = c < ce;
            const int lo = cv ? cptr[c - cb] : 0, hi = cv ? cptr[c - cb + 1] : 0;
            float2 acc[RW][NCV / 2];
#pragma unroll
            for (int q = 0; q < RW; q++)
#pragma unroll
                for (int p = 0; p < NCV / 2; p++) acc[q][p] = make_float2(0.f, 0.f);
            // two columns a lane per pass: eight loads in flight before the products
            for (int t = lo + gl; t < hi; t += 2 * LG) {
                const int t2 = t + LG;
                const bool two = t2 < hi;
                const int cc = col[t], cc2 = col[two ? t2 : t];
                float v[RW], v2[RW];
#pragma unroll
                for (int q = 0; q < RW; q++) {
                    v[q] = aphi_load(Ar[q], cc);
                    v2[q] = aphi_load(Ar[q], cc2);
                }
#pragma unroll
                for (int p = 0; p < NCV / 2; p++) {
                    const float2 b = bs[t * 3 + p];
#pragma unroll
                    for (int q = 0; q < RW; q++) acc[q][p] = __ffma2_rn(make_float2(v[q], v[q]), b, acc[q][p]);
                }
                if (two) {
#pragma unroll
                    for (int p = 0; p < NCV / 2; p++) {
                        const float2 b = bs[t2 * 3 + p];
#pragma unroll
                        for (int q = 0; q < RW; q++)
                            acc[q][p] = __ffma2_rn(make_float2(v2[q], v2[q]), b, acc[q][p]);
                    }
                }
            }
            // the group's lanes: a fixed xor tree; every lane ends with the sums
#pragma unroll
            for (int q = 0; q < RW; q++)
#pragma unroll
                for (int p = 0; p < NCV / 2; p++)
#pragma unroll
                    for (int o = LG / 2; o > 0; o >>= 1) {
                        acc[q][p].x += __shfl_xor_sync(0xffffffffu, acc[q][p].x, o);
                        acc[q][p].y += __shfl_xor_sync(0xffffffffu, acc[q][p].y, o);
                    }
            // output e = q * NCV + k (24 of them) is written by the group's lane e % LG
            if (cv) {
#pragma unroll
                for (int q = 0; q < RW; q++)
#pragma unroll
                    for (int k = 0; k < NCV; k++) {
                        const int e = q * NCV + k;
                        if (gl == e % LG && r0 + q < r1)
                            APhi[(r0 + q) * ldp + NCV * c + k] = (k & 1) ? acc[q][k / 2].y : acc[q][k / 2].x;
                    }
            }
        }
    }
}

// APhi[row0 + 3f + i, 6 c(s) + k] += sum_j vals[e][i][j] basis[col0 + 3s + j][k]
// for every near block e = (f, s) of one list; a warp per field point
__global__ void __launch_bounds__(256)
nn_aphi_near_kernel(mbem_near_blocks nb, const int32_t* __restrict__ chunk_of, const float* __restrict__ basis,
                    float* __restrict__ APhi, int64_t ldp) {
    const int64_t f = ((int64_t)blockIdx.x * 256 + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (f >= nb.n_field) return;
    for (int64_t e = nb.rowptr[f] + lane; e < nb.rowptr[f + 1]; e += 32) {
        const int64_t d = nb.col0 + 3 * nb.cols[e];
        const int64_t c = chunk_of[d];
        const double* v = nb.vals + 9 * e;
        for (int i = 0; i < 3; i++) {
            float* out = APhi + (nb.row0 + 3 * f + i) * ldp + NCV * c;
#pragma unroll
            for (int k = 0; k < NCV; k++) {
                const double s = v[3 * i] * basis[d * NCV + k] + v[3 * i + 1] * basis[(d + 1) * NCV + k] +
                                 v[3 * i + 2] * basis[(d + 2) * NCV + k];
                atomicAdd(out + k, (float)s);
            }
        }
    }
}

// Ac[6c + k, q] = sum_{d in c} basis[d][k] APhi[d, q] from the FP32 A Phi;
// a CTA per (chunk, 256 columns), a thread per column, FP32 output at ldc
__global__ void __launch_bounds__(256)
nn_coarse_matrix_f32_kernel(const float* __restrict__ APhi, int64_t ldp, int64_t n_coarse,
                            const int64_t* __restrict__ chunk_ptr, const int64_t* __restrict__ dofs,
                            const float* __restrict__ basis, float* __restrict__ Ac, int64_t ldc) {
    const int c = blockIdx.x;
    const int64_t q = (int64_t)blockIdx.y * 256 + threadIdx.x;
    if (q >= n_coarse) return;
    const int64_t c0 = chunk_ptr[c];
    const int m = (int)(chunk_ptr[c + 1] - c0);
    float s[NCV] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int t = 0; t < m; t++) {
        const int64_t d = dofs[c0 + t];
        const float v = APhi[d * ldp + q];
#pragma unroll
        for (int k = 0; k < NCV; k++) s[k] = fmaf(basis[d * NCV + k], v, s[k]);
    }
    for (int k = 0; k < NCV; k++) Ac[(NCV * c + k) * ldc + q] = s[k];
}

// Ac[p, q] += sum_j U[p, j] U[q, j] (FP32 coarse matrix at ldc)
__global__ void nn_coarse_shift_f32_kernel(float* __restrict__ Ac, int64_t ldc, int64_t nc,
                                           const double* __restrict__ U, int n_shift) {
    const int64_t p = blockIdx.y;
    const int64_t q = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (q >= nc) return;
    double s = 0.0;
    for (int j = 0; j < n_shift; j++) s += U[p * n_shift + j] * U[q * n_shift + j];
    Ac[p * ldc + q] += (float)s;
}

// out[i] = a[i] - b[i]
__global__ void nn_sub_kernel(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out,
                              int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (i < n) out[i] = a[i] - b[i];
}

// ---------------------------------------------------------------------------
// Blocked Gauss-Jordan inverse in FP32 (the coarse matrix of the mixed-operator
// preconditioner), with partial pivoting but no row interchanges: column k
// takes as its pivot the unused row pi(k) of largest magnitude, and the
// in-place result R holds the inverse with its rows and columns renamed,
// A^-1[k, pi(j)] = R[pi(k), j] (gj_unpermute_kernel writes it out).
// Pivot columns go GJB_BLOCK at a time:
//  - the panel kernel (one CTA; the panel's n x b values in shared memory,
//    each thread owning fixed rows, so a pivot step needs two barriers: one
//    after the candidates, one after the pivot row is read) runs the b pivot
//    steps; the panel then holds, in GJ form, [B^-1 ; -A_RB B^-1] on the
//    pivot rows B and the others R;
//  - the gather kernel copies the pivot rows X_B of every other column;
//  - the update kernel: X_B <- B^-1 X_B, X_R <- X_R + (-A_RB B^-1) X_B, i.e.
//    every row gets P[i, :] X_B (pivot rows replaced, others added to).
// A column with no usable pivot (all zero or NaN) sets *bad.
// ---------------------------------------------------------------------------
constexpr int GJB_BLOCK = 16;
constexpr int GJB_LDS = GJB_BLOCK + 1;       // odd row stride: a warp's row accesses fall in distinct banks
constexpr int GJB_PANEL_THREADS = 1024;

__global__ void __launch_bounds__(GJB_PANEL_THREADS)
gjb_panel_kernel(float* __restrict__ M, int64_t n, int64_t ld, int64_t k0, int b, int* __restrict__ piv,
                 int* __restrict__ used, int* __restrict__ bad) {
    extern __shared__ float P[];                  // [n][GJB_LDS], then the used flags (n ints)
    int* us = reinterpret_cast<int*>(P + n * GJB_LDS);
    __shared__ float rv[GJB_PANEL_THREADS / 32];
    __shared__ int ri[GJB_PANEL_THREADS / 32];
    __shared__ int rf[GJB_PANEL_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int64_t e = tid; e < n * GJB_BLOCK; e += GJB_PANEL_THREADS) {
        const int64_t i = e / GJB_BLOCK;
        const int c = (int)(e % GJB_BLOCK);
        P[i * GJB_LDS + c] = c < b ? M[i * ld + k0 + c] : 0.0f;
    }
    for (int64_t i = tid; i < n; i += GJB_PANEL_THREADS) us[i] = used[i];
    __syncthreads();
    for (int t = 0; t < b; t++) {
        const int64_t k = k0 + t;
        // candidates: the largest |P[i][t]| over this thread's unused rows
        // (lowest row on ties; NaN never wins), and the lowest unused row
        float bv = -1.0f;
        int bi = -1, fi = 0x7fffffff;
        for (int64_t i = tid; i < n; i += GJB_PANEL_THREADS) {
            if (us[i]) continue;
            if (fi == 0x7fffffff) fi = (int)i;
            const float v = fabsf(P[i * GJB_LDS + t]);
            if (v > bv) { bv = v; bi = (int)i; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            const int of = __shfl_xor_sync(0xffffffffu, fi, o);
            if (ov > bv || (ov == bv && oi >= 0 && (bi < 0 || oi < bi))) { bv = ov; bi = oi; }
            fi = min(fi, of);
        }
        if (lane == 0) { rv[wid] = bv; ri[wid] = bi; rf[wid] = fi; }
        __syncthreads();
        // every warp reduces the warps' candidates: every thread knows the pivot
        bv = rv[lane];
        bi = ri[lane];
        fi = rf[lane];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            const int of = __shfl_xor_sync(0xffffffffu, fi, o);
            if (ov > bv || (ov == bv && oi >= 0 && (bi < 0 || oi < bi))) { bv = ov; bi = oi; }
            fi = min(fi, of);
        }
        int64_t p = bi;
        if (bi < 0 || !(bv > 0.0f)) {               // no usable pivot: the column is singular
            if (tid == 0) atomicExch(bad, 1);
            p = fi < (int)n ? fi : k;
        }
        float prow[GJB_BLOCK];
#pragma unroll
        for (int c = 0; c < GJB_BLOCK; c++) prow[c] = P[p * GJB_LDS + c];
        const float pv = prow[t];
        const float inv = pv != 0.0f ? 1.0f / pv : 0.0f;
        if (tid == 0) piv[k] = (int)p;
        __syncthreads();                             // row p read by all before it changes
        for (int64_t i = tid; i < n; i += GJB_PANEL_THREADS) {
            float* row = P + i * GJB_LDS;
            if (i == p) {
#pragma unroll
                for (int c = 0; c < GJB_BLOCK; c++) row[c] = (c == t) ? inv : prow[c] * inv;
                us[i] = (int)(k + 1);
            } else {
                const float g = -row[t] * inv;
#pragma unroll
                for (int c = 0; c < GJB_BLOCK; c++) row[c] = (c == t) ? g : fmaf(g, prow[c], row[c]);
            }
        }
    }
    __syncthreads();
    for (int64_t e = tid; e < n * GJB_BLOCK; e += GJB_PANEL_THREADS) {
        const int64_t i = e / GJB_BLOCK;
        const int c = (int)(e % GJB_BLOCK);
        if (c < b) M[i * ld + k0 + c] = P[i * GJB_LDS + c];
    }
    for (int64_t i = tid; i < n; i += GJB_PANEL_THREADS) used[i] = us[i];
}

// X_B: the block's pivot rows on every other column
__global__ void gjb_gather_kernel(const float* __restrict__ M, int64_t n, int64_t ld, int64_t k0, int b,
                                  const int* __restrict__ piv, float* __restrict__ XB) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n || (j >= k0 && j < k0 + b)) return;
    for (int t = 0; t < b; t++) XB[(int64_t)t * n + j] = M[(int64_t)piv[k0 + t] * ld + j];
}

// M[i, j] = (i pivot row of the block ? 0 : M[i, j]) + sum_t P[i, t] XB[t, j]
// for every column j outside the panel; a CTA per 32 rows x 128 columns
constexpr int GJB_TR = 32, GJB_TC = 128;
__global__ void __launch_bounds__(256)
gjb_update_kernel(float* __restrict__ M, int64_t n, int64_t ld, int64_t k0, int b, const float* __restrict__ XB,
                  const int* __restrict__ used) {
    __shared__ float Ps[GJB_TR][GJB_BLOCK];
    __shared__ float Xs[GJB_BLOCK][GJB_TC];
    __shared__ int pivrow[GJB_TR];
    const int64_t i0 = (int64_t)blockIdx.y * GJB_TR, j0 = (int64_t)blockIdx.x * GJB_TC;
    for (int e = threadIdx.x; e < GJB_TR * GJB_BLOCK; e += 256) {
        const int r = e / GJB_BLOCK, t = e % GJB_BLOCK;
        Ps[r][t] = (i0 + r < n && t < b) ? M[(i0 + r) * ld + k0 + t] : 0.0f;
    }
    for (int e = threadIdx.x; e < GJB_BLOCK * GJB_TC; e += 256) {
        const int t = e / GJB_TC, c = e % GJB_TC;
        Xs[t][c] = (t < b && j0 + c < n) ? XB[(int64_t)t * n + j0 + c] : 0.0f;
    }
    if (threadIdx.x < GJB_TR) {
        const int64_t i = i0 + threadIdx.x;
        const int u = i < n ? used[i] - 1 : -1;
        pivrow[threadIdx.x] = (u >= k0 && u < k0 + b) ? 1 : 0;
    }
    __syncthreads();
    const int c = threadIdx.x % GJB_TC;
    const int64_t j = j0 + c;
    if (j >= n || (j >= k0 && j < k0 + b)) return;
    for (int r = threadIdx.x / GJB_TC; r < GJB_TR; r += 256 / GJB_TC) {
        const int64_t i = i0 + r;
        if (i >= n) break;
        float acc = pivrow[r] ? 0.0f : M[i * ld + j];
#pragma unroll
        for (int t = 0; t < GJB_BLOCK; t++) acc = fmaf(Ps[r][t], Xs[t][c], acc);
        M[i * ld + j] = acc;
    }
}

// A^-1[k, pi(j)] = R[pi(k), j], from a copy R of the in-place result
__global__ void gj_unpermute_kernel(const float* __restrict__ R, float* __restrict__ M, int64_t n, int64_t ld,
                                    const int* __restrict__ piv) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * n) return;
    const int64_t k = e / n, j = e % n;
    M[k * ld + piv[j]] = R[(int64_t)piv[k] * n + j];
}

// ---------------------------------------------------------------------------
// Blocked Gauss-Jordan inverse without row interchanges: the first attempt of
// the FP32 inverse at n >= GJNP_MIN_N. Block columns of GJNP_B; for block K
// (its rows and columns K, the rest R), with D = M[K, K]:
//   M[K, K] <- D^-1 (one CTA, D in shared memory),
//   M[K, R] <- D^-1 M[K, R],
//   M[R, R] <- M[R, R] - M[R, K] M[K, R]   (on the tensor cores: both blocks
//                                           in three BF16 pieces, six piece
//                                           products, FP32 accumulation),
//   M[R, K] <- -M[R, K] D^-1,
// and after the last block M holds A^-1. Without a pivot search a block
// column costs a few short kernels instead of a pass over every row for each
// column, but its stability rests on the matrix (the coarse Galerkin matrix
// of a second-kind operator has dominant diagonal blocks). So a zero or
// non-finite pivot flags the attempt, the result must satisfy
// |A X v - v| <= GJNP_CHECK |v| for two fixed vectors v, and otherwise the
// pivoted inverse runs from the saved copy of A.
// ---------------------------------------------------------------------------
constexpr int GJNP_B = 64;
constexpr int GJNP_MIN_N = 1024;
constexpr double GJNP_CHECK = 1e-3;
constexpr int GJNP_K6 = 6 * GJNP_B;         // the update's K: six BF16 pieces of each block

// D^-1 in place in M[K, K] and into Dinv (b x b, row stride GJNP_B). Thread
// (c, g) holds column c's rows 16 g .. 16 g + 15 in registers; a block of
// b < GJNP_B rows is padded with the identity, whose pivot steps change
// nothing. The row and the column of pivot t go through shared memory,
// double-buffered, so a step has one barrier.
__global__ void __launch_bounds__(256)
gjnp_diag_kernel(float* __restrict__ M, int64_t ld, int64_t k0, int b, float* __restrict__ Dinv,
                 int* __restrict__ bad) {
    __shared__ float prow[2][GJNP_B], pcol[2][GJNP_B];
    const int c = threadIdx.x & (GJNP_B - 1), g = threadIdx.x / GJNP_B;
    float v[16];
#pragma unroll
    for (int j = 0; j < 16; j++) {
        const int i = 16 * g + j;
        v[j] = (i < b && c < b) ? M[(k0 + i) * ld + k0 + c] : (i == c ? 1.0f : 0.0f);
    }
    int flag = 0;
#pragma unroll
    for (int t = 0; t < GJNP_B; t++) {
        const int buf = t & 1;
        if (g == t / 16) prow[buf][c] = v[t % 16];
        if (c == t) {
#pragma unroll
            for (int j = 0; j < 16; j++) pcol[buf][16 * g + j] = v[j];
        }
        __syncthreads();
        const float p = prow[buf][t];
        const bool ok = isfinite(p) && p != 0.0f;
        flag |= !ok;
        const float inv = ok ? 1.0f / p : 1.0f;
        const float rc = prow[buf][c];
#pragma unroll
        for (int j = 0; j < 16; j++) {
            const int i = 16 * g + j;
            if (i == t) {
                v[j] = (c == t) ? inv : rc * inv;
            } else {
                const float gg = pcol[buf][i] * inv;
                v[j] = (c == t) ? -gg : fmaf(-gg, rc, v[j]);
            }
        }
    }
    if (flag && threadIdx.x == 0) atomicExch(bad, 1);
#pragma unroll
    for (int j = 0; j < 16; j++) {
        const int i = 16 * g + j;
        if (i < b && c < b) {
            M[(k0 + i) * ld + k0 + c] = v[j];
            Dinv[i * GJNP_B + c] = v[j];
        }
    }
}

// M[K, j] <- D^-1 M[K, j] for the columns j outside K; a CTA per 64 columns
__global__ void __launch_bounds__(256)
gjnp_row_kernel(float* __restrict__ M, int64_t n, int64_t ld, int64_t k0, int b, const float* __restrict__ Dinv) {
    __shared__ float Ds[GJNP_B][GJNP_B + 1];
    __shared__ float X[GJNP_B][GJNP_B + 1];
    const int64_t j0 = (int64_t)blockIdx.x * GJNP_B;
    for (int e = threadIdx.x; e < GJNP_B * GJNP_B; e += 256) {
        const int r = e / GJNP_B, c = e % GJNP_B;
        Ds[r][c] = (r < b && c < b) ? Dinv[r * GJNP_B + c] : 0.0f;
        X[r][c] = (r < b && j0 + c < n) ? M[(k0 + r) * ld + j0 + c] : 0.0f;
    }
    __syncthreads();
    const int c = threadIdx.x & (GJNP_B - 1);
    const int64_t j = j0 + c;
    if (j >= n || (j >= k0 && j < k0 + b)) return;
    for (int r = threadIdx.x / GJNP_B; r < b; r += 256 / GJNP_B) {
        float acc = 0.0f;
        for (int t = 0; t < b; t++) acc = fmaf(Ds[r][t], X[t][c], acc);
        M[(k0 + r) * ld + j] = acc;
    }
}

// M[i, K] <- -M[i, K] D^-1 for the rows i outside K; a CTA per 64 rows
__global__ void __launch_bounds__(256)
gjnp_col_kernel(float* __restrict__ M, int64_t n, int64_t ld, int64_t k0, int b, const float* __restrict__ Dinv) {
    __shared__ float Ds[GJNP_B][GJNP_B + 1];
    __shared__ float Y[GJNP_B][GJNP_B + 1];
    const int64_t i0 = (int64_t)blockIdx.x * GJNP_B;
    for (int e = threadIdx.x; e < GJNP_B * GJNP_B; e += 256) {
        const int r = e / GJNP_B, c = e % GJNP_B;
        Ds[r][c] = (r < b && c < b) ? Dinv[r * GJNP_B + c] : 0.0f;
        Y[r][c] = (c < b && i0 + r < n) ? M[(i0 + r) * ld + k0 + c] : 0.0f;
    }
    __syncthreads();
    const int c = threadIdx.x & (GJNP_B - 1);
    if (c >= b) return;
    for (int r = threadIdx.x / GJNP_B; r < GJNP_B; r += 256 / GJNP_B) {
        const int64_t i = i0 + r;
        if (i >= n || (i >= k0 && i < k0 + b)) continue;
        float acc = 0.0f;
        for (int t = 0; t < b; t++) acc = fmaf(Y[r][t], Ds[t][c], acc);
        M[i * ld + k0 + c] = -acc;
    }
}

// the two fixed check vectors: v0 = 1, v1 alternates in sign by a hash of i
__device__ __forceinline__ double gjnp_v(int64_t i, int q) {
    if (q == 0) return 1.0;
    uint32_t h = (uint32_t)i * 2654435761u;
    h ^= h >> 15;
    return (h & 1u) ? 1.0 : -1.0;
}

// y[:, q] = A x[:, q] (x = the check vectors when x is NULL): a warp per
// row, FP64 sums in a fixed lane order
__global__ void __launch_bounds__(256)
gjnp_gemv2_kernel(const float* __restrict__ A, int64_t n, int64_t lda, const double* __restrict__ x,
                  double* __restrict__ y) {
    const int64_t row = (int64_t)blockIdx.x * 8 + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    double s0 = 0.0, s1 = 0.0;
    for (int64_t c = lane; c < n; c += 32) {
        const double a = A[row * lda + c];
        const double x0 = x ? x[2 * c] : gjnp_v(c, 0), x1 = x ? x[2 * c + 1] : gjnp_v(c, 1);
        s0 = fma(a, x0, s0);
        s1 = fma(a, x1, s1);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    if (lane == 0) {
        y[2 * row] = s0;
        y[2 * row + 1] = s1;
    }
}

// out[q] = |y[:, q] - v_q| / |v_q|, one CTA
__global__ void __launch_bounds__(256)
gjnp_check_kernel(const double* __restrict__ y, int64_t n, double* __restrict__ out) {
    __shared__ double red[4][256 / 32];
    double e0 = 0.0, e1 = 0.0, v0 = 0.0, v1 = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += 256) {
        const double a = gjnp_v(i, 0), c = gjnp_v(i, 1);
        const double d0 = y[2 * i] - a, d1 = y[2 * i + 1] - c;
        e0 += d0 * d0;
        e1 += d1 * d1;
        v0 += a * a;
        v1 += c * c;
    }
    double vals[4] = {e0, e1, v0, v1};
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 4; q++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) vals[q] += __shfl_xor_sync(0xffffffffu, vals[q], o);
        if (lane == 0) red[q][wid] = vals[q];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s[4] = {0.0, 0.0, 0.0, 0.0};
        for (int q = 0; q < 4; q++)
            for (int w = 0; w < 256 / 32; w++) s[q] += red[q][w];
        // a non-finite result fails the check
        out[0] = (s[0] >= 0.0) ? sqrt(s[0] / s[2]) : INFINITY;
        out[1] = (s[1] >= 0.0) ? sqrt(s[1] / s[3]) : INFINITY;
    }
}

// ---------------------------------------------------------------------------
// apply pieces
// ---------------------------------------------------------------------------
// q[6c + k] = sum_{d in c} basis[d][k] r[d]; a CTA per chunk
__global__ void __launch_bounds__(128)
nn_phit_kernel(const int64_t* __restrict__ chunk_ptr, const int64_t* __restrict__ dofs,
               const float* __restrict__ basis, const double* __restrict__ r, double* __restrict__ q) {
    __shared__ double red[4];
    const int c = blockIdx.x;
    const int64_t c0 = chunk_ptr[c];
    const int m = (int)(chunk_ptr[c + 1] - c0);
    double s[NCV] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int t = threadIdx.x; t < m; t += 128) {
        const int64_t d = dofs[c0 + t];
        const double v = r[d];
#pragma unroll
        for (int k = 0; k < NCV; k++) s[k] += (double)basis[d * NCV + k] * v;
    }
    for (int k = 0; k < NCV; k++) {
        const double tot = block_sum(s[k], red);
        if (threadIdx.x == 0) q[NCV * c + k] = tot;
    }
}

// z[d] += sum_k basis[d][k] y[6 c(d) + k]
__global__ void __launch_bounds__(256)
nn_phi_add_kernel(int64_t n, const int32_t* __restrict__ chunk_of, const float* __restrict__ basis,
                  const double* __restrict__ y, double* __restrict__ z) {
    const int64_t d = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (d >= n) return;
    const double* yc = y + NCV * (int64_t)chunk_of[d];
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < NCV; k++) s += (double)basis[d * NCV + k] * yc[k];
    z[d] += s;
}

// The coarse basis of every chunk: the 3m x 6 block [I | phi_i] over the
// chunk's nodes orthonormalised by modified Gram-Schmidt (FP64 sums), and its
// projection on the rigid translations of the u-ranges,
// U[6c + k, j] = sum_{d in c, d in u, d % 3 = j} basis[d, k] / sqrt(u nodes).
// A CTA of 128 threads per chunk, the chunk's rows in shared memory.
__global__ void __launch_bounds__(128)
nn_basis_kernel(const int64_t* __restrict__ chunk_ptr, const int64_t* __restrict__ dofs,
                const float* __restrict__ phi, URanges ur, double inv_sqrt_u, float* __restrict__ basis,
                double* __restrict__ U) {
    __shared__ double Bs[MBEM_BJ_MAX_DOF][NCV];
    __shared__ double red[4];
    const int c = blockIdx.x;
    const int64_t c0 = chunk_ptr[c];
    const int m = (int)(chunk_ptr[c + 1] - c0);
    for (int t = threadIdx.x; t < m; t += 128) {
        const int64_t d = dofs[c0 + t];
        const int64_t node = d / 3;
        const int a = (int)(d % 3);
        for (int k = 0; k < 3; k++) Bs[t][k] = (a == k) ? 1.0 : 0.0;
        for (int k = 0; k < 3; k++) Bs[t][3 + k] = (double)phi[node * 9 + 3 * a + k];
    }
    __syncthreads();
    for (int k = 0; k < NCV; k++) {
        for (int p = 0; p < k; p++) {
            double v = 0.0;
            for (int t = threadIdx.x; t < m; t += 128) v += Bs[t][p] * Bs[t][k];
            const double dot = block_sum(v, red);
            for (int t = threadIdx.x; t < m; t += 128) Bs[t][k] -= dot * Bs[t][p];
            __syncthreads();
        }
        double v = 0.0;
        for (int t = threadIdx.x; t < m; t += 128) v += Bs[t][k] * Bs[t][k];
        const double nrm = sqrt(block_sum(v, red));
        const double inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
        for (int t = threadIdx.x; t < m; t += 128) Bs[t][k] *= inv;
        __syncthreads();
    }
    for (int t = threadIdx.x; t < m; t += 128) {
        const int64_t d = dofs[c0 + t];
        for (int k = 0; k < NCV; k++) basis[d * NCV + k] = (float)Bs[t][k];
    }
    if (U == nullptr) return;
    for (int k = 0; k < NCV; k++)
        for (int j = 0; j < 3; j++) {
            double v = 0.0;
            for (int t = threadIdx.x; t < m; t += 128) {
                const int64_t d = dofs[c0 + t];
                bool in_u = false;
                for (int q = 0; q < ur.n; q++) in_u |= (d >= ur.off[q] && d < ur.off[q] + ur.len[q]);
                if (in_u && d % 3 == j) v += (double)(float)Bs[t][k];
            }
            const double tot = block_sum(v, red);
            if (threadIdx.x == 0) U[(NCV * c + k) * 3 + j] = tot * inv_sqrt_u;
        }
}

static int nn_check(const mbem_nn_precond* nn) {
    MBEM_REQUIRE(nn != nullptr && nn->bj != nullptr, MBEM_ERR_ARG, "learned preconditioner descriptor is NULL");
    MBEM_REQUIRE(nn->n == nn->bj->n && nn->n_coarse == NCV * nn->bj->n_chunks && nn->n % 3 == 0, MBEM_ERR_ARG,
                 "learned preconditioner sizes (n=%lld, coarse=%lld, chunks=%lld)", (long long)nn->n,
                 (long long)nn->n_coarse, (long long)nn->bj->n_chunks);
    const bool f64 = nn->APhi && nn->Ac_inv, f32 = nn->APhi32 && nn->Ac_inv32;
    MBEM_REQUIRE(nn->n == 0 || (nn->basis && (f64 || f32) && nn->work && nn->bj->chunk_of), MBEM_ERR_ARG,
                 "NULL learned preconditioner arrays");
    MBEM_REQUIRE(!f32 || (nn->ld32 >= nn->n_coarse && nn->ld32 % 4 == 0), MBEM_ERR_ARG,
                 "FP32 coarse arrays need ld32 >= n_coarse, a multiple of 4");
    return MBEM_OK;
}

int nn_precond_apply(const void* state, const double* r, double* z, cudaStream_t st) {
    const mbem_nn_precond* nn = static_cast<const mbem_nn_precond*>(state);
    int e = nn_check(nn);
    if (e) return e;
    if (nn->n == 0) return MBEM_OK;
    const int64_t n = nn->n, nc = nn->n_coarse;
    double* t = nn->work;          // n: r - (A Phi) y
    double* q = t + n;             // nc: Phi^T r
    double* y = q + nc;            // nc: A_c^-1 q
    MBEM_REQUIRE(z != t && r != t, MBEM_ERR_ARG, "r/z alias the learned preconditioner's scratch");
    const mbem_block_jacobi* bj = nn->bj;
    nn_phit_kernel<<<(unsigned)bj->n_chunks, 128, 0, st>>>(bj->chunk_ptr, bj->dofs, nn->basis, r, q);
    if ((e = launch_status("nn_phit_kernel"))) return e;
    if (nn->APhi32 != nullptr) {
        // FP32 A Phi and A_c^-1 (the mixed operator's setup): the streaming
        // FP32 products with double-float sums, scratch after y
        float* xh = reinterpret_cast<float*>(y + nc);
        float* xl = xh + ((lmax(n, nc) + 15) / 16) * 16;
        mbem_mixed_operator op;
        op.n_rows = nc; op.n_cols = nc; op.A32 = nn->Ac_inv32; op.ld32 = nn->ld32; op.n_near = 0; op.near = nullptr;
        if ((e = mixed_matvec(&op, q, y, xh, xl, st))) return e;
        op.n_rows = n; op.A32 = nn->APhi32;
        if ((e = mixed_matvec(&op, y, t, xh, xl, st))) return e;
        nn_sub_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(r, t, t, n);
        if ((e = launch_status("nn_sub_kernel"))) return e;
    } else {
        if ((e = dgemv(nn->Ac_inv, nc, nc, nc, q, 1.0, 0.0, y, st))) return e;
        cudaMemcpyAsync(t, r, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
        if ((e = dgemv(nn->APhi, nc, n, nc, y, -1.0, 1.0, t, st))) return e;
    }
    if ((e = bj_apply(bj, t, z, st))) return e;
    nn_phi_add_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(n, bj->chunk_of, nn->basis, y, z);
    return launch_status("nn_phi_add_kernel");
}

}  // namespace mbem

using namespace mbem;

extern "C" {

int mbem_nn_forward(const float* feat, int64_t n_items, const float* params, float* act, float* out,
                    void* stream) {
    MBEM_REQUIRE(n_items >= 0 && (n_items == 0 || (feat && params && out)), MBEM_ERR_ARG, "bad forward args");
    if (n_items == 0) return MBEM_OK;
    nn_forward_kernel<<<(unsigned)ceil_div(n_items, NN_THREADS), NN_THREADS, 0, (cudaStream_t)stream>>>(
        feat, n_items, params, act, out);
    return launch_status("nn_forward_kernel");
}

int mbem_nn_coarse_loss_grad(const mbem_block_jacobi* bj, const float* phi, const float* eps, const float* inv_e2,
                             int64_t n_samples, float* dphi, double* partial, double* loss, void* stream) {
    MBEM_REQUIRE(bj && bj->n_chunks >= 1 && bj->m_max <= MBEM_BJ_MAX_DOF && phi && eps && inv_e2 && dphi &&
                     partial && loss && n_samples >= 1,
                 MBEM_ERR_ARG, "bad coarse-loss args");
    MBEM_REQUIRE(bj->m_max / 3 <= 128, MBEM_ERR_ARG, "chunks of more than 128 nodes");
    cudaStream_t st = (cudaStream_t)stream;
    nn_coarse_loss_grad_kernel<<<(unsigned)bj->n_chunks, 128, 0, st>>>(bj->chunk_ptr, bj->dofs, phi, eps, inv_e2,
                                                                      n_samples, bj->n, dphi, partial);
    nn_sum_kernel<<<1, 32, 0, st>>>(partial, bj->n_chunks, loss);
    return launch_status("nn_coarse_loss_grad_kernel", 2);
}

size_t mbem_nn_backward_workspace_size(int64_t n_items) {
    const int64_t chunks = ceil_div(n_items, GRAD_CHUNK);
    return (size_t)n_items * DEL * sizeof(float) + (size_t)chunks * NP * sizeof(float);
}

int mbem_nn_backward(const float* feat, int64_t n_items, const float* params, const float* act, const float* G,
                     float* grad, void* work, size_t work_bytes, void* stream) {
    MBEM_REQUIRE(n_items >= 1 && feat && params && act && G && grad, MBEM_ERR_ARG, "bad backward args");
    const size_t need = mbem_nn_backward_workspace_size(n_items);
    MBEM_REQUIRE(work != nullptr && work_bytes >= need, MBEM_ERR_SIZE, "backward workspace %zu < %zu", work_bytes,
                 need);
    cudaStream_t st = (cudaStream_t)stream;
    float* del = static_cast<float*>(work);
    float* partial = del + (size_t)n_items * DEL;
    const int64_t chunks = ceil_div(n_items, GRAD_CHUNK);
    MBEM_REQUIRE(chunks <= 65535, MBEM_ERR_UNSUPPORTED, "%lld items exceed the gradient grid",
                 (long long)n_items);
    nn_backward_items_kernel<<<(unsigned)ceil_div(n_items, NN_THREADS), NN_THREADS, 0, st>>>(n_items, params, act,
                                                                                           G, del);
    dim3 grid((unsigned)ceil_div(NP, NN_THREADS), (unsigned)chunks);
    nn_param_grad_kernel<<<grid, NN_THREADS, 0, st>>>(n_items, feat, act, del, partial);
    nn_param_reduce_kernel<<<(unsigned)ceil_div(NP, 256), 256, 0, st>>>(partial, chunks, grad);
    return launch_status("nn_backward", 3);
}

int mbem_nn_adam(float* params, const float* grad, float* m, float* v, int64_t n, float lr, float beta1,
                 float beta2, float eps, int step, void* stream) {
    MBEM_REQUIRE(n >= 1 && params && grad && m && v && step >= 1, MBEM_ERR_ARG, "bad Adam args");
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    nn_adam_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, (cudaStream_t)stream>>>(params, grad, m, v, n, lr, beta1,
                                                                               beta2, eps, c1, c2);
    return launch_status("nn_adam_kernel");
}

int mbem_nn_basis(const mbem_block_jacobi* bj, const float* phi, const int64_t* u_ranges, int n_u_ranges,
                  float* basis, double* U, void* stream) {
    MBEM_REQUIRE(bj && bj->n_chunks >= 0 && bj->m_max <= MBEM_BJ_MAX_DOF && phi && basis, MBEM_ERR_ARG,
                 "bad coarse-basis args");
    URanges ur;
    int e = make_ranges(u_ranges, n_u_ranges, ur);
    if (e) return e;
    int64_t u_nodes = 0;
    for (int q = 0; q < ur.n; q++) u_nodes += ur.len[q] / 3;
    if (bj->n_chunks == 0) return MBEM_OK;
    nn_basis_kernel<<<(unsigned)bj->n_chunks, 128, 0, (cudaStream_t)stream>>>(
        bj->chunk_ptr, bj->dofs, phi, ur, u_nodes > 0 ? 1.0 / sqrt((double)u_nodes) : 0.0, basis,
        u_nodes > 0 ? U : nullptr);
    return launch_status("nn_basis_kernel");
}

size_t mbem_dense_inverse_workspace_size(int64_t n) {
    return (size_t)(n * n + 1) * sizeof(double) + (size_t)(n + 8) * sizeof(int);
}

int mbem_dense_inverse(double* M, int64_t n, void* work, size_t work_bytes, void* stream) {
    MBEM_REQUIRE(n >= 0 && n <= 65535 * GJ_ROWS && (n == 0 || M), MBEM_ERR_ARG, "bad matrix for the inverse");
    if (n == 0) return MBEM_OK;
    MBEM_REQUIRE(work && work_bytes >= mbem_dense_inverse_workspace_size(n), MBEM_ERR_SIZE,
                 "inverse workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    double* buf = static_cast<double*>(work);
    double* dinv = buf + n * n;
    int* piv = reinterpret_cast<int*>(dinv + 1);
    int* bad = piv + n;
    cudaMemsetAsync(bad, 0, sizeof(int), st);
    double* src = M;
    double* dst = buf;
    const dim3 grid((unsigned)ceil_div(n, 256), (unsigned)ceil_div(n, GJ_ROWS));
    for (int64_t k = 0; k < n; k++) {
        gj_pivot_kernel<<<1, 256, 0, st>>>(src, n, k, piv, dinv, bad);
        gj_update_kernel<<<grid, 256, 0, st>>>(src, dst, n, k, piv, dinv);
        double* t = src;
        src = dst;
        dst = t;
    }
    count_launches((int)(2 * n));
    if (src != M) cudaMemcpyAsync(M, src, n * n * sizeof(double), cudaMemcpyDeviceToDevice, st);
    gj_swap_columns_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(M, n, piv);
    int e = launch_status("gauss_jordan");
    if (e) return e;
    int hbad = 0;
    cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("inverse sync", 0);
    MBEM_REQUIRE(hbad == 0, MBEM_ERR_NUMERIC, "singular matrix");
    return MBEM_OK;
}

int mbem_knn(const float* points, int64_t n, int k, int64_t* idx, void* stream) {
    MBEM_REQUIRE(n >= 0 && k >= 1 && k <= KNN_MAX && k <= n && (n == 0 || (points && idx)), MBEM_ERR_ARG,
                 "knn needs 1 <= k <= min(%d, n)", KNN_MAX);
    MBEM_REQUIRE(n < INT32_MAX, MBEM_ERR_SIZE, "too many nodes for knn");
    if (n == 0) return MBEM_OK;
    knn_kernel<<<(unsigned)ceil_div(n, KNN_QPB), 256, 0, (cudaStream_t)stream>>>(points, n, k, idx);
    return launch_status("knn_kernel");
}

}  // extern "C"

namespace mbem {

// inverses that stood without row interchanges, and pivoted ones, since the
// last mbem_dense_inverse_f32_stats call
static int64_t g_inverse_counts[2] = {0, 0};

// The blocked inverse without row interchanges: 1 when it passed its checks
// (M holds A^-1), 0 when the pivoted inverse must run (M holds A again), or
// minus an error code. R (n x n) keeps the copy of A; scratch holds D^-1,
// the check's vectors and its result.
static int gjnp_try(float* M, int64_t n, int64_t ld, float* R, char* scratch, size_t scratch_bytes, uint16_t* Ls,
                    uint16_t* Us, int* bad, cudaStream_t st) {
    const size_t need = (size_t)GJNP_B * GJNP_B * sizeof(float) + 4 * (size_t)n * sizeof(double) + 64;
    if (scratch_bytes < need) return 0;
    float* Dinv = reinterpret_cast<float*>(scratch);
    double* wv = reinterpret_cast<double*>(scratch + (size_t)GJNP_B * GJNP_B * sizeof(float));
    double* yv = wv + 2 * n;
    double* res = yv + 2 * n;
    cudaMemcpy2DAsync(R, n * sizeof(float), M, ld * sizeof(float), n * sizeof(float), n, cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(bad, 0, sizeof(int), st);
    const unsigned g64 = (unsigned)ceil_div(n, GJNP_B);
    int launches = 0;
    for (int64_t k0 = 0; k0 < n; k0 += GJNP_B) {
        const int b = (int)lmin(GJNP_B, n - k0);
        gjnp_diag_kernel<<<1, 256, 0, st>>>(M, ld, k0, b, Dinv, bad);
        gjnp_row_kernel<<<g64, 256, 0, st>>>(M, n, ld, k0, b, Dinv);
        const int e = gj_block_update_tc(M, n, ld, k0, b, Ls, Us, st);
        if (e) return -e;
        gjnp_col_kernel<<<g64, 256, 0, st>>>(M, n, ld, k0, b, Dinv);
        launches += 3;
    }
    // A (X v) against v for the two check vectors
    gjnp_gemv2_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, st>>>(M, n, ld, nullptr, wv);
    gjnp_gemv2_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, st>>>(R, n, n, wv, yv);
    gjnp_check_kernel<<<1, 256, 0, st>>>(yv, n, res);
    count_launches(launches + 3);
    int e = launch_status("gauss_jordan_f32 (no interchanges)", 0);
    if (e) return -e;
    double hres[2] = {INFINITY, INFINITY};
    int hbad = 1;
    cudaMemcpyAsync(hres, res, sizeof(hres), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return -launch_status("inverse sync", 0);
    if (hbad == 0 && hres[0] <= GJNP_CHECK && hres[1] <= GJNP_CHECK) return 1;
    // back to A for the pivoted inverse
    cudaMemcpy2DAsync(M, ld * sizeof(float), R, n * sizeof(float), n * sizeof(float), n, cudaMemcpyDeviceToDevice, st);
    return 0;
}

}  // namespace mbem

extern "C" {

void mbem_dense_inverse_f32_stats(int64_t* no_interchange, int64_t* pivoted) {
    if (no_interchange) *no_interchange = g_inverse_counts[0];
    if (pivoted) *pivoted = g_inverse_counts[1];
    g_inverse_counts[0] = g_inverse_counts[1] = 0;
}

size_t mbem_dense_inverse_f32_workspace_size(int64_t n) {
    const size_t pieces = n >= GJNP_MIN_N ? 2 * (((size_t)n * GJNP_K6 * sizeof(uint16_t) + 255) & ~(size_t)255) : 0;
    return (size_t)GJB_BLOCK * n * sizeof(float) + (size_t)n * n * sizeof(float) + (size_t)(2 * n + 8) * sizeof(int) +
           4 * 256 + pieces;
}

int mbem_dense_inverse_f32(float* M, int64_t n, int64_t ld, void* work, size_t work_bytes, void* stream) {
    MBEM_REQUIRE(n >= 0 && ld >= n && (n == 0 || M), MBEM_ERR_ARG, "bad matrix for the inverse");
    if (n == 0) return MBEM_OK;
    const size_t panel = (size_t)n * (GJB_LDS + 1) * sizeof(float);
    constexpr size_t kSmem = 227 * 1024 - 1024;      // the panel kernel's static arrays take the rest
    MBEM_REQUIRE(panel <= kSmem && ceil_div(n, GJB_TR) <= 65535, MBEM_ERR_UNSUPPORTED,
                 "the FP32 inverse holds its n x %d panel in shared memory: n <= %d", GJB_BLOCK,
                 (int)(kSmem / ((GJB_LDS + 1) * sizeof(float))));
    MBEM_REQUIRE(work && work_bytes >= mbem_dense_inverse_f32_workspace_size(n), MBEM_ERR_SIZE,
                 "inverse workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    char* w = static_cast<char*>(work);
    auto take = [&](size_t bytes) { char* p = w; w += (bytes + 255) & ~(size_t)255; return p; };
    float* XB = reinterpret_cast<float*>(take((size_t)GJB_BLOCK * n * sizeof(float)));
    float* R = reinterpret_cast<float*>(take((size_t)n * n * sizeof(float)));
    int* piv = reinterpret_cast<int*>(take((size_t)n * sizeof(int)));
    int* used = reinterpret_cast<int*>(take((size_t)n * sizeof(int)));
    int* bad = reinterpret_cast<int*>(take(sizeof(int)));
    if (n >= GJNP_MIN_N) {
        // the inverse without row interchanges first (XB's room as its scratch)
        uint16_t* Ls = reinterpret_cast<uint16_t*>(take((size_t)n * GJNP_K6 * sizeof(uint16_t)));
        uint16_t* Us = reinterpret_cast<uint16_t*>(take((size_t)n * GJNP_K6 * sizeof(uint16_t)));
        const int got = gjnp_try(M, n, ld, R, reinterpret_cast<char*>(XB), (size_t)GJB_BLOCK * n * sizeof(float),
                                 Ls, Us, bad, st);
        if (got < 0) return -got;
        if (got == 1) {
            g_inverse_counts[0]++;
            return MBEM_OK;
        }
    }
    g_inverse_counts[1]++;
    cudaMemsetAsync(used, 0, n * sizeof(int), st);
    cudaMemsetAsync(bad, 0, sizeof(int), st);
    cudaError_t ce = cudaFuncSetAttribute(gjb_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
    if (ce != cudaSuccess) return set_error(MBEM_ERR_CUDA, "inverse smem attribute: %s", cudaGetErrorString(ce));
    const dim3 ug((unsigned)ceil_div(n, GJB_TC), (unsigned)ceil_div(n, GJB_TR));
    int launches = 0;
    for (int64_t k0 = 0; k0 < n; k0 += GJB_BLOCK) {
        const int b = (int)lmin(GJB_BLOCK, n - k0);
        gjb_panel_kernel<<<1, GJB_PANEL_THREADS, panel, st>>>(M, n, ld, k0, b, piv, used, bad);
        gjb_gather_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(M, n, ld, k0, b, piv, XB);
        gjb_update_kernel<<<ug, 256, 0, st>>>(M, n, ld, k0, b, XB, used);
        launches += 3;
    }
    cudaMemcpy2DAsync(R, n * sizeof(float), M, ld * sizeof(float), n * sizeof(float), n, cudaMemcpyDeviceToDevice, st);
    gj_unpermute_kernel<<<(unsigned)ceil_div(n * n, 256), 256, 0, st>>>(R, M, n, ld, piv);
    count_launches(launches + 1);
    int e = launch_status("gauss_jordan_f32");
    if (e) return e;
    int hbad = 0;
    cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("inverse sync", 0);
    MBEM_REQUIRE(hbad == 0, MBEM_ERR_NUMERIC, "singular matrix");
    return MBEM_OK;
}

int mbem_nn_coarse_operator_dense(const double* A, int64_t ld, const mbem_nn_precond* nn, const double* shift,
                                  int n_shift, void* stream) {
    int e = nn_check(nn);
    if (e) return e;
    MBEM_REQUIRE(A != nullptr && ld >= nn->n, MBEM_ERR_ARG, "bad dense operator");
    const int64_t n = nn->n, nc = nn->n_coarse;
    if (n == 0) return MBEM_OK;
    MBEM_REQUIRE(ceil_div(n, APHI_ROWS) <= 65535 && ceil_div(nc, 256) <= 65535 && nc <= 65535, MBEM_ERR_UNSUPPORTED,
                 "learned preconditioner sizes beyond one launch");
    MBEM_REQUIRE(n_shift >= 0 && (n_shift == 0 || shift != nullptr), MBEM_ERR_ARG, "bad coarse shift");
    cudaStream_t st = (cudaStream_t)stream;
    const mbem_block_jacobi* bj = nn->bj;
    double* APhi = const_cast<double*>(nn->APhi);
    double* Ac = const_cast<double*>(nn->Ac_inv);
    nn_aphi_kernel<<<dim3((unsigned)bj->n_chunks, (unsigned)ceil_div(n, APHI_ROWS)), 256, 0, st>>>(
        A, ld, n, bj->chunk_ptr, bj->dofs, nn->basis, nc, APhi);
    nn_coarse_matrix_kernel<<<dim3((unsigned)bj->n_chunks, (unsigned)ceil_div(nc, 256)), 256, 0, st>>>(
        APhi, nc, bj->chunk_ptr, bj->dofs, nn->basis, Ac);
    if ((e = launch_status("nn_coarse_setup", 2))) return e;
    if (n_shift > 0) {
        nn_coarse_shift_kernel<<<dim3((unsigned)ceil_div(nc, 256), (unsigned)nc), 256, 0, st>>>(Ac, nc, shift,
                                                                                            n_shift);
        if ((e = launch_status("nn_coarse_shift_kernel"))) return e;
    }
    return MBEM_OK;
}

size_t mbem_nn_setup_workspace_size(int64_t n_coarse) { return mbem_dense_inverse_workspace_size(n_coarse); }

int mbem_nn_setup_dense(const double* A, int64_t ld, const mbem_nn_precond* nn, const double* shift,
                        int n_shift, void* work, size_t work_bytes, void* stream) {
    int e = mbem_nn_coarse_operator_dense(A, ld, nn, shift, n_shift, stream);
    if (e) return e;
    return mbem_dense_inverse(const_cast<double*>(nn->Ac_inv), nn->n_coarse, work, work_bytes, stream);
}

size_t mbem_nn_apply_workspace_size(int64_t n, int64_t n_coarse) {
    // t (n), q, y (n_coarse) doubles, then the hi/lo split of the FP32 path
    return (size_t)(n + 2 * n_coarse) * sizeof(double) + 2 * (size_t)((lmax(n, n_coarse) + 15) / 16 * 16) * 4 + 64;
}

}  // extern "C"

namespace mbem {

// A Phi (FP32) by the gather kernel from A (BF16 or FP64 rows at ld), the
// near blocks added, then A_c (+ U U^T) and its FP32 inverse
template <typename T>
static int nn_setup32(const T* A, int64_t ld, int n_near, const mbem_near_blocks* near, const mbem_nn_precond* nn,
                      const double* shift, int n_shift, void* work, size_t work_bytes, cudaStream_t st) {
    int e = nn_check(nn);
    if (e) return e;
    MBEM_REQUIRE(A && ld >= nn->n, MBEM_ERR_ARG, "bad operator for the coarse setup");
    MBEM_REQUIRE(nn->APhi32 && nn->Ac_inv32, MBEM_ERR_ARG, "the FP32 setup writes APhi32 and Ac_inv32");
    MBEM_REQUIRE(n_shift >= 0 && (n_shift == 0 || shift != nullptr), MBEM_ERR_ARG, "bad coarse shift");
    const int64_t n = nn->n, nc = nn->n_coarse, ldp = nn->ld32;
    if (n == 0) return MBEM_OK;
    const mbem_block_jacobi* bj = nn->bj;
    const int64_t groups = ceil_div(bj->n_chunks, APHI16_GROUP);
    MBEM_REQUIRE(groups <= 65535 * 32 && ceil_div(n, APHI16_ROWS) <= 65535 && nc <= 65535, MBEM_ERR_UNSUPPORTED,
                 "learned preconditioner sizes beyond one launch");
    const size_t smem = (size_t)APHI16_GROUP * MBEM_BJ_MAX_DOF * (NCV * sizeof(float) + sizeof(int));
    cudaError_t ce = cudaFuncSetAttribute(nn_aphi_gather_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem);
    if (ce != cudaSuccess) return set_error(MBEM_ERR_CUDA, "APhi smem attribute: %s", cudaGetErrorString(ce));
    float* APhi = const_cast<float*>(nn->APhi32);
    float* Ac = const_cast<float*>(nn->Ac_inv32);
    nn_aphi_gather_kernel<T><<<dim3((unsigned)groups, (unsigned)ceil_div(n, APHI16_ROWS)), 256, smem, st>>>(
        A, ld, n, bj->chunk_ptr, bj->dofs, bj->n_chunks, nn->basis, APhi, ldp);
    if ((e = launch_status("nn_aphi_gather_kernel"))) return e;
    for (int q = 0; q < n_near; q++) {
        const mbem_near_blocks& nb = near[q];
        if (nb.n_field == 0) continue;
        nn_aphi_near_kernel<<<(unsigned)ceil_div(nb.n_field * 32, 256), 256, 0, st>>>(nb, bj->chunk_of, nn->basis,
                                                                                    APhi, ldp);
        if ((e = launch_status("nn_aphi_near_kernel"))) return e;
    }
    nn_coarse_matrix_f32_kernel<<<dim3((unsigned)bj->n_chunks, (unsigned)ceil_div(nc, 256)), 256, 0, st>>>(
        APhi, ldp, nc, bj->chunk_ptr, bj->dofs, nn->basis, Ac, ldp);
    if ((e = launch_status("nn_coarse_matrix_f32_kernel"))) return e;
    if (n_shift > 0) {
        nn_coarse_shift_f32_kernel<<<dim3((unsigned)ceil_div(nc, 256), (unsigned)nc), 256, 0, st>>>(Ac, ldp, nc, shift,
                                                                                                n_shift);
        if ((e = launch_status("nn_coarse_shift_f32_kernel"))) return e;
    }
    return mbem_dense_inverse_f32(Ac, nc, ldp, work, work_bytes, st);
}

}  // namespace mbem

extern "C" {

int mbem_nn_setup_mixed(const mbem_inner_bf16* inner, const mbem_nn_precond* nn, const double* shift, int n_shift,
                        void* work, size_t work_bytes, void* stream) {
    MBEM_REQUIRE(inner && inner->A16 && nn && inner->n == nn->n && inner->ld16 >= inner->n, MBEM_ERR_ARG,
                 "bad BF16 inner operator");
    return nn_setup32(inner->A16, inner->ld16, inner->n_near, inner->near, nn, shift, n_shift, work, work_bytes,
                      (cudaStream_t)stream);
}

int mbem_nn_setup_dense32(const double* A, int64_t ld, const mbem_nn_precond* nn, const double* shift, int n_shift,
                          void* work, size_t work_bytes, void* stream) {
    return nn_setup32(A, ld, 0, (const mbem_near_blocks*)nullptr, nn, shift, n_shift, work, work_bytes,
                      (cudaStream_t)stream);
}

int mbem_nn_apply(const mbem_nn_precond* nn, const double* r, double* z, void* stream) {
    MBEM_REQUIRE(r && z && r != z, MBEM_ERR_ARG, "r and z must be distinct device vectors");
    return nn_precond_apply(nn, r, z, (cudaStream_t)stream);
}

}  // extern "C"
