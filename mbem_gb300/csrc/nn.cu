// Learned preconditioner: a mesh-local network that corrects the cluster
// block-Jacobi step with the residuals of each node's k nearest nodes.
//
//   rho = BJ r,   z_i = rho_i + sum_{j in nbr(i)} W_ij rho_j,
//   W_ij = MLP(g_ij) (3x3),  g_ij = geometry of the pair (i, j)
//
// The network sees geometry only, so its edge blocks W are computed once per
// mesh; every FGMRES apply is then one block-Jacobi apply and one sparse
// 3x3-block product over the k-nearest-neighbour graph. z is linear in r,
// so the preconditioner is a fixed linear map per mesh.
//
// MLP: MBEM_NN_FEAT -> MBEM_NN_HIDDEN (tanh) -> MBEM_NN_HIDDEN (tanh) -> 9.
// Parameters, flat FP32: W1 (H x F), b1 (H), W2 (H x H), b2 (H), W3 (9 x H),
// b3 (9). Training minimises (1/S) sum_s |z_s - e_s|^2 / |e_s|^2 over pairs
// (r_s, e_s = A^-1 r_s) with the kernels below: forward, batched apply, loss
// gradient, per-edge gradient, backward through the MLP, fixed-order
// parameter-gradient reduction, Adam. Every reduction runs in a fixed order,
// so a training run is deterministic.
#include <math.h>

#include "common.cuh"

namespace mbem {

constexpr int NF = MBEM_NN_FEAT;
constexpr int NH = MBEM_NN_HIDDEN;
constexpr int NP = MBEM_NN_PARAMS;
constexpr int OFF_W1 = 0, OFF_B1 = NH * NF, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + 9 * NH;
static_assert(OFF_B3 + 9 == NP, "parameter layout");
constexpr int ACT = 2 * NH;          // stored activations per edge (h1, h2)
constexpr int DEL = 2 * NH + 9;      // stored deltas per edge (d1, d2, d3)
constexpr int NN_THREADS = 256;
constexpr int GRAD_CHUNK = 512;      // edges per partial parameter-gradient sum

// ---------------------------------------------------------------------------
// forward: one thread per edge, parameters in shared memory
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
// batched apply (training): z[s] = rho[s] + W rho[s], FP32, (S, 3 n_nodes)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NN_THREADS)
nn_apply_batch_kernel(const int32_t* __restrict__ nbr, int64_t n_nodes, int k, const float* __restrict__ w,
                      const float* __restrict__ rho, int64_t S, float* __restrict__ z) {
    const int64_t t = (int64_t)blockIdx.x * NN_THREADS + threadIdx.x;
    if (t >= S * n_nodes) return;
    const int64_t s = t / n_nodes, i = t % n_nodes;
    const int64_t N = 3 * n_nodes;
    const float* rs = rho + s * N;
    float a0 = rs[3 * i], a1 = rs[3 * i + 1], a2 = rs[3 * i + 2];
    for (int q = 0; q < k; q++) {
        const int64_t j = nbr[i * k + q];
        const float* W = w + (i * k + q) * 9;
        const float r0 = rs[3 * j], r1 = rs[3 * j + 1], r2 = rs[3 * j + 2];
        a0 = fmaf(W[0], r0, fmaf(W[1], r1, fmaf(W[2], r2, a0)));
        a1 = fmaf(W[3], r0, fmaf(W[4], r1, fmaf(W[5], r2, a1)));
        a2 = fmaf(W[6], r0, fmaf(W[7], r1, fmaf(W[8], r2, a2)));
    }
    float* zs = z + s * N;
    zs[3 * i] = a0;
    zs[3 * i + 1] = a1;
    zs[3 * i + 2] = a2;
}

// loss = (1/S) sum_s |z_s - e_s|^2 inv_e2[s]; dz = (2/S) (z - e) inv_e2[s].
// Per-block partial sums in FP64, summed in block order by nn_sum_kernel.
__global__ void __launch_bounds__(NN_THREADS)
nn_loss_grad_kernel(const float* __restrict__ z, const float* __restrict__ e, const float* __restrict__ inv_e2,
                    int64_t S, int64_t N, float* __restrict__ dz, double* __restrict__ partial) {
    __shared__ double red[NN_THREADS];
    const int64_t t = (int64_t)blockIdx.x * NN_THREADS + threadIdx.x;
    double l = 0.0;
    if (t < S * N) {
        const int64_t s = t / N;
        const float d = z[t] - e[t];
        dz[t] = (2.0f / (float)S) * d * inv_e2[s];
        l = (double)d * (double)d * (double)inv_e2[s] / (double)S;
    }
    red[threadIdx.x] = l;
    __syncthreads();
    for (int o = NN_THREADS / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void nn_sum_kernel(const double* __restrict__ partial, int64_t n, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int64_t i = 0; i < n; i++) s += partial[i];
    *out = s;
}

// G_e = sum_s dz[s, i] rho[s, j]^T for edge e = (i, j): one thread per edge
__global__ void __launch_bounds__(NN_THREADS)
nn_edge_grad_kernel(const int32_t* __restrict__ nbr, int64_t n_nodes, int k, const float* __restrict__ dz,
                    const float* __restrict__ rho, int64_t S, float* __restrict__ G) {
    const int64_t e = (int64_t)blockIdx.x * NN_THREADS + threadIdx.x;
    if (e >= n_nodes * k) return;
    const int64_t i = e / k, j = nbr[e];
    const int64_t N = 3 * n_nodes;
    float g[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t s = 0; s < S; s++) {
        const float* d = dz + s * N + 3 * i;
        const float* r = rho + s * N + 3 * j;
        const float d0 = d[0], d1 = d[1], d2 = d[2], r0 = r[0], r1 = r[1], r2 = r[2];
        g[0] = fmaf(d0, r0, g[0]); g[1] = fmaf(d0, r1, g[1]); g[2] = fmaf(d0, r2, g[2]);
        g[3] = fmaf(d1, r0, g[3]); g[4] = fmaf(d1, r1, g[4]); g[5] = fmaf(d1, r2, g[5]);
        g[6] = fmaf(d2, r0, g[6]); g[7] = fmaf(d2, r1, g[7]); g[8] = fmaf(d2, r2, g[8]);
    }
#pragma unroll
    for (int o = 0; o < 9; o++) G[e * 9 + o] = g[o];
}

// per-edge deltas of the MLP: d3 = G, d2 = (W3^T d3)(1 - h2^2), d1 = (W2^T d2)(1 - h1^2)
__global__ void __launch_bounds__(NN_THREADS)
nn_backward_edges_kernel(int64_t E, const float* __restrict__ params, const float* __restrict__ act,
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

// partial[c][p] = sum over edges of chunk c of dL/dparam_p contributions;
// threads of a warp take consecutive parameters (coalesced inputs)
__global__ void __launch_bounds__(NN_THREADS)
nn_param_grad_kernel(int64_t E, const float* __restrict__ feat, const float* __restrict__ act,
                     const float* __restrict__ del, float* __restrict__ partial) {
    const int p = blockIdx.x * NN_THREADS + threadIdx.x;
    const int64_t c = blockIdx.y;
    if (p >= NP) return;
    const int64_t e0 = c * GRAD_CHUNK, e1 = lmin(E, e0 + GRAD_CHUNK);
    // parameter p = (delta index, input index or -1 for a bias)
    const float* dbase;
    int dstride = DEL, di, ii = -1, istride = 0;
    const float* ibase = nullptr;
    if (p < OFF_B1) { di = p / NF; ii = p % NF; ibase = feat; istride = NF; }
    else if (p < OFF_W2) { di = p - OFF_B1; }
    else if (p < OFF_B2) { di = NH + (p - OFF_W2) / NH; ii = (p - OFF_W2) % NH; ibase = act; istride = ACT; }
    else if (p < OFF_W3) { di = NH + (p - OFF_B2); }
    else if (p < OFF_B3) { di = 2 * NH + (p - OFF_W3) / NH; ii = NH + (p - OFF_W3) % NH; ibase = act; istride = ACT; }
    else { di = 2 * NH + (p - OFF_B3); }
    dbase = del;
    float s = 0.0f;
    if (ii >= 0) {
        for (int64_t e = e0; e < e1; e++) s = fmaf(dbase[e * dstride + di], ibase[e * istride + ii], s);
    } else {
        for (int64_t e = e0; e < e1; e++) s += dbase[e * dstride + di];
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

// inference: z = rho + W rho in FP64 (FP32 edge blocks)
__global__ void __launch_bounds__(NN_THREADS)
nn_apply_kernel(const int32_t* __restrict__ nbr, int64_t n_nodes, int k, const float* __restrict__ w,
                const double* __restrict__ rho, double* __restrict__ z) {
    const int64_t i = (int64_t)blockIdx.x * NN_THREADS + threadIdx.x;
    if (i >= n_nodes) return;
    double a0 = rho[3 * i], a1 = rho[3 * i + 1], a2 = rho[3 * i + 2];
    for (int q = 0; q < k; q++) {
        const int64_t j = nbr[i * k + q];
        const float* W = w + (i * k + q) * 9;
        const double r0 = rho[3 * j], r1 = rho[3 * j + 1], r2 = rho[3 * j + 2];
        a0 += (double)W[0] * r0 + (double)W[1] * r1 + (double)W[2] * r2;
        a1 += (double)W[3] * r0 + (double)W[4] * r1 + (double)W[5] * r2;
        a2 += (double)W[6] * r0 + (double)W[7] * r1 + (double)W[8] * r2;
    }
    z[3 * i] = a0;
    z[3 * i + 1] = a1;
    z[3 * i + 2] = a2;
}

static int nn_check(const mbem_nn_precond* nn) {
    MBEM_REQUIRE(nn != nullptr && nn->bj != nullptr, MBEM_ERR_ARG, "learned preconditioner descriptor is NULL");
    MBEM_REQUIRE(nn->n_nodes >= 0 && nn->k >= 1 && 3 * nn->n_nodes == nn->bj->n, MBEM_ERR_ARG,
                 "learned preconditioner sizes (n_nodes=%lld, k=%d, n=%lld)", (long long)nn->n_nodes, nn->k,
                 (long long)nn->bj->n);
    MBEM_REQUIRE(nn->n_nodes == 0 || (nn->nbr && nn->w && nn->work), MBEM_ERR_ARG, "NULL learned arrays");
    return MBEM_OK;
}

int nn_precond_apply(const void* state, const double* r, double* z, cudaStream_t st) {
    const mbem_nn_precond* nn = static_cast<const mbem_nn_precond*>(state);
    int e = nn_check(nn);
    if (e) return e;
    MBEM_REQUIRE(z != nn->work && r != nn->work, MBEM_ERR_ARG, "r/z alias the learned preconditioner's scratch");
    if ((e = bj_apply(nn->bj, r, nn->work, st))) return e;
    if (nn->n_nodes == 0) return MBEM_OK;
    nn_apply_kernel<<<(unsigned)ceil_div(nn->n_nodes, NN_THREADS), NN_THREADS, 0, st>>>(nn->nbr, nn->n_nodes, nn->k,
                                                                                       nn->w, nn->work, z);
    return launch_status("nn_apply_kernel");
}

}  // namespace mbem

using namespace mbem;

extern "C" {

int mbem_nn_forward(const float* feat, int64_t n_edges, const float* params, float* act, float* w,
                    void* stream) {
    MBEM_REQUIRE(n_edges >= 0 && (n_edges == 0 || (feat && params && w)), MBEM_ERR_ARG, "bad forward args");
    if (n_edges == 0) return MBEM_OK;
    nn_forward_kernel<<<(unsigned)ceil_div(n_edges, NN_THREADS), NN_THREADS, 0, (cudaStream_t)stream>>>(
        feat, n_edges, params, act, w);
    return launch_status("nn_forward_kernel");
}

int mbem_nn_apply_batch(const int32_t* nbr, int64_t n_nodes, int k, const float* w, const float* rho,
                        int64_t n_samples, float* z, void* stream) {
    MBEM_REQUIRE(n_nodes >= 0 && k >= 1 && n_samples >= 0, MBEM_ERR_ARG, "bad batch apply sizes");
    MBEM_REQUIRE(n_nodes * n_samples == 0 || (nbr && w && rho && z && rho != z), MBEM_ERR_ARG,
                 "bad batch apply pointers");
    if (n_nodes * n_samples == 0) return MBEM_OK;
    nn_apply_batch_kernel<<<(unsigned)ceil_div(n_nodes * n_samples, NN_THREADS), NN_THREADS, 0,
                            (cudaStream_t)stream>>>(nbr, n_nodes, k, w, rho, n_samples, z);
    return launch_status("nn_apply_batch_kernel");
}

int mbem_nn_loss_grad(const float* z, const float* e, const float* inv_e2, int64_t n_samples, int64_t n,
                      float* dz, double* partial, double* loss, void* stream) {
    MBEM_REQUIRE(n_samples >= 1 && n >= 1 && z && e && inv_e2 && dz && partial && loss, MBEM_ERR_ARG,
                 "bad loss args");
    const int64_t blocks = ceil_div(n_samples * n, NN_THREADS);
    nn_loss_grad_kernel<<<(unsigned)blocks, NN_THREADS, 0, (cudaStream_t)stream>>>(z, e, inv_e2, n_samples, n, dz,
                                                                                   partial);
    nn_sum_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(partial, blocks, loss);
    return launch_status("nn_loss_grad_kernel", 2);
}

size_t mbem_nn_loss_partial_count(int64_t n_samples, int64_t n) {
    return (size_t)ceil_div(n_samples * n, NN_THREADS);
}

int mbem_nn_edge_grad(const int32_t* nbr, int64_t n_nodes, int k, const float* dz, const float* rho,
                      int64_t n_samples, float* G, void* stream) {
    MBEM_REQUIRE(n_nodes >= 1 && k >= 1 && n_samples >= 1 && nbr && dz && rho && G, MBEM_ERR_ARG,
                 "bad edge-gradient args");
    nn_edge_grad_kernel<<<(unsigned)ceil_div(n_nodes * k, NN_THREADS), NN_THREADS, 0, (cudaStream_t)stream>>>(
        nbr, n_nodes, k, dz, rho, n_samples, G);
    return launch_status("nn_edge_grad_kernel");
}

size_t mbem_nn_backward_workspace_size(int64_t n_edges) {
    const int64_t chunks = ceil_div(n_edges, GRAD_CHUNK);
    return (size_t)n_edges * DEL * sizeof(float) + (size_t)chunks * NP * sizeof(float);
}

int mbem_nn_backward(const float* feat, int64_t n_edges, const float* params, const float* act, const float* G,
                     float* grad, void* work, size_t work_bytes, void* stream) {
    MBEM_REQUIRE(n_edges >= 1 && feat && params && act && G && grad, MBEM_ERR_ARG, "bad backward args");
    const size_t need = mbem_nn_backward_workspace_size(n_edges);
    MBEM_REQUIRE(work != nullptr && work_bytes >= need, MBEM_ERR_SIZE, "backward workspace %zu < %zu", work_bytes,
                 need);
    cudaStream_t st = (cudaStream_t)stream;
    float* del = static_cast<float*>(work);
    float* partial = del + (size_t)n_edges * DEL;
    const int64_t chunks = ceil_div(n_edges, GRAD_CHUNK);
    MBEM_REQUIRE(chunks <= 65535, MBEM_ERR_UNSUPPORTED, "%lld edges exceed the gradient grid",
                 (long long)n_edges);
    nn_backward_edges_kernel<<<(unsigned)ceil_div(n_edges, NN_THREADS), NN_THREADS, 0, st>>>(n_edges, params, act,
                                                                                           G, del);
    dim3 grid((unsigned)ceil_div(NP, NN_THREADS), (unsigned)chunks);
    nn_param_grad_kernel<<<grid, NN_THREADS, 0, st>>>(n_edges, feat, act, del, partial);
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

int mbem_nn_apply(const mbem_nn_precond* nn, const double* r, double* z, void* stream) {
    MBEM_REQUIRE(r && z && r != z, MBEM_ERR_ARG, "r and z must be distinct device vectors");
    return nn_precond_apply(nn, r, z, (cudaStream_t)stream);
}

}  // extern "C"
