// Cluster block-Jacobi preconditioner (la/preconditioner.py:421-470, the
// "block_jacobi" rung): the unknowns are partitioned into spatial chunks
// (principal-axis bisection of the node centroids, la/cluster.py:56-75, done
// by the host), and M^-1 is the block diagonal of the inverses of A's
// diagonal chunks.
//
// GB300 layout: a chunk holds at most MBEM_BJ_MAX_DOF unknowns so that its
// FP32 copy (<= 203 KB) sits in one CTA's shared memory; the CTA gathers it
// from the FP64 matrix (or from the mixed operator's FP32 far field plus its
// FP64 near blocks), inverts it there by Gauss-Jordan with partial pivoting,
// and writes the FP32 inverse (row-major, m_max stride). The apply is one
// CTA per chunk, a warp per row, coalesced along the row. The reference
// factors 9000-DOF chunks with LAPACK on the host; a preconditioner of a
// flexible Krylov method needs no FP64, and the GPU spends its time better
// on more, smaller chunks.
#include <math.h>

#include "common.cuh"

namespace mbem {

__device__ int g_bj_singular;

constexpr int BJ_THREADS = 256;
constexpr int BJ_MAX_NEAR = 8;

struct NearSet {
    int n;
    mbem_near_blocks b[BJ_MAX_NEAR];
};

__host__ __device__ inline size_t bj_smem_bytes(int m_max) {
    return (size_t)m_max * m_max * sizeof(float) + 2 * (size_t)m_max * sizeof(float) + m_max * sizeof(int) + 64;
}

// Gathers chunk c of A (dense FP64 at ld, or FP32 far field + near blocks),
// inverts it in shared memory and writes inv[c].
template <bool MIXED>
__global__ void __launch_bounds__(BJ_THREADS)
bj_build_kernel(const double* __restrict__ A, const float* __restrict__ A32, int64_t ld, NearSet near,
                const int64_t* __restrict__ chunk_ptr, const int64_t* __restrict__ dofs,
                const int32_t* __restrict__ local, const int32_t* __restrict__ chunk_of, int m_max,
                float* __restrict__ inv) {
    extern __shared__ float smem[];
    const int c = blockIdx.x;
    const int64_t c0 = chunk_ptr[c];
    const int m = (int)(chunk_ptr[c + 1] - c0);
    float* D = smem;                          // m x m, row stride m
    float* fcol = D + (size_t)m_max * m_max;  // column k before the update
    float* rowk = fcol + m_max;               // pivot row after scaling
    int* piv = reinterpret_cast<int*>(rowk + m_max);
    __shared__ int s_pivot;
    __shared__ int s_bad;
    if (threadIdx.x == 0) s_bad = 0;

    const int warp = threadIdx.x / 32, lane = threadIdx.x & 31;
    constexpr int NW = BJ_THREADS / 32;
    // gather: a warp per row, lanes along the row
    for (int i = warp; i < m; i += NW) {
        const int64_t gi = dofs[c0 + i];
        for (int j = lane; j < m; j += 32) {
            const int64_t gj = dofs[c0 + j];
            D[(size_t)i * m + j] = MIXED ? A32[gi * ld + gj] : (float)A[gi * ld + gj];
        }
    }
    __syncthreads();
    if (MIXED) {
        // near 3x3 blocks whose row and column both lie in this chunk; each
        // DOF belongs to one chunk, so one thread owns each row's entries
        for (int i = threadIdx.x; i < m; i += BJ_THREADS) {
            const int64_t gi = dofs[c0 + i];
            for (int t = 0; t < near.n; t++) {
                const mbem_near_blocks& nb = near.b[t];
                const int64_t r = gi - nb.row0;
                if (r < 0 || r >= 3 * nb.n_field) continue;
                const int64_t f = r / 3;
                const int a = (int)(r % 3);
                for (int64_t q = nb.rowptr[f]; q < nb.rowptr[f + 1]; q++) {
                    const int64_t col3 = nb.col0 + 3 * nb.cols[q];
                    for (int b = 0; b < 3; b++) {
                        const int64_t gj = col3 + b;
                        if (chunk_of[gj] != c) continue;
                        D[(size_t)i * m + local[gj]] += (float)nb.vals[9 * q + 3 * a + b];
                    }
                }
            }
        }
        __syncthreads();
    }

    // Gauss-Jordan with partial pivoting, in place
    for (int k = 0; k < m; k++) {
        if (warp == 0) {
            float best = -1.0f;
            int bi = k;
            for (int i = k + lane; i < m; i += 32) {
                const float v = fabsf(D[(size_t)i * m + k]);
                if (v > best) { best = v; bi = i; }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (lane == 0) {
                s_pivot = bi;
                piv[k] = bi;
                if (!(best > 0.0f)) s_bad = 1;
            }
        }
        __syncthreads();
        const int p = s_pivot;
        if (p != k)
            for (int j = threadIdx.x; j < m; j += BJ_THREADS) {
                const float t = D[(size_t)k * m + j];
                D[(size_t)k * m + j] = D[(size_t)p * m + j];
                D[(size_t)p * m + j] = t;
            }
        __syncthreads();
        const float pv = D[(size_t)k * m + k];
        const float d = (pv != 0.0f) ? 1.0f / pv : 1.0f;
        for (int j = threadIdx.x; j < m; j += BJ_THREADS) {
            rowk[j] = (j == k ? 1.0f : D[(size_t)k * m + j]) * d;
            fcol[j] = D[(size_t)j * m + k];
        }
        __syncthreads();
        for (int i = warp; i < m; i += NW) {
            float* Di = D + (size_t)i * m;
            const float fi = fcol[i];
            if (i == k) {
                for (int j = lane; j < m; j += 32) Di[j] = rowk[j];
            } else {
                for (int j = lane; j < m; j += 32) Di[j] = (j == k ? 0.0f : Di[j]) - fi * rowk[j];
            }
        }
        __syncthreads();
    }
    // undo the row interchanges as column interchanges, last first
    for (int k = m - 1; k >= 0; k--) {
        const int p = piv[k];
        if (p != k)
            for (int i = threadIdx.x; i < m; i += BJ_THREADS) {
                const float t = D[(size_t)i * m + k];
                D[(size_t)i * m + k] = D[(size_t)i * m + p];
                D[(size_t)i * m + p] = t;
            }
        __syncthreads();
    }
    float* out = inv + (size_t)c * m_max * m_max;
    const bool bad = s_bad != 0;
    for (int i = warp; i < m; i += NW)
        for (int j = lane; j < m_max; j += 32)
            out[(size_t)i * m_max + j] = bad ? (i == j ? 1.0f : 0.0f) : (j < m ? D[(size_t)i * m + j] : 0.0f);
    if (bad && threadIdx.x == 0) atomicAdd(&g_bj_singular, 1);
}

// z[dofs] = inv_c r[dofs], one CTA per chunk, a warp per row
__global__ void __launch_bounds__(BJ_THREADS)
bj_apply_kernel(const int64_t* __restrict__ chunk_ptr, const int64_t* __restrict__ dofs, int m_max,
                const float* __restrict__ inv, const double* __restrict__ r, double* __restrict__ z) {
    __shared__ float rc[MBEM_BJ_MAX_DOF];
    const int c = blockIdx.x;
    const int64_t c0 = chunk_ptr[c];
    const int m = (int)(chunk_ptr[c + 1] - c0);
    for (int j = threadIdx.x; j < m; j += BJ_THREADS) rc[j] = (float)r[dofs[c0 + j]];
    __syncthreads();
    const float* Mi = inv + (size_t)c * m_max * m_max;
    const int warp = threadIdx.x / 32, lane = threadIdx.x & 31;
    for (int i = warp; i < m; i += BJ_THREADS / 32) {
        const float* row = Mi + (size_t)i * m_max;
        float acc = 0.0f;
        for (int j = lane; j < m; j += 32) acc = fmaf(__ldg(row + j), rc[j], acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) z[dofs[c0 + i]] = (double)acc;
    }
}

static int bj_check(const mbem_block_jacobi* bj) {
    MBEM_REQUIRE(bj != nullptr, MBEM_ERR_ARG, "block-Jacobi descriptor is NULL");
    MBEM_REQUIRE(bj->n >= 0 && bj->n_chunks >= 0 && bj->m_max >= 1 && bj->m_max <= MBEM_BJ_MAX_DOF, MBEM_ERR_ARG,
                 "bad block-Jacobi sizes (n=%lld, chunks=%lld, m_max=%d; m_max <= %d)", (long long)bj->n,
                 (long long)bj->n_chunks, bj->m_max, MBEM_BJ_MAX_DOF);
    MBEM_REQUIRE(bj->n_chunks == 0 || (bj->chunk_ptr && bj->dofs && bj->inv), MBEM_ERR_ARG,
                 "NULL block-Jacobi arrays");
    return MBEM_OK;
}

static int bj_build(const double* A, const float* A32, int64_t ld, const NearSet& near, const mbem_block_jacobi* bj,
                    cudaStream_t st) {
    int e = bj_check(bj);
    if (e) return e;
    if (bj->n_chunks == 0) return MBEM_OK;
    const size_t smem = bj_smem_bytes(bj->m_max);
    const int zero = 0;
    cudaMemcpyToSymbolAsync(g_bj_singular, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st);
    if (A32) {
        cudaFuncSetAttribute(bj_build_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        bj_build_kernel<true><<<(unsigned)bj->n_chunks, BJ_THREADS, smem, st>>>(
            nullptr, A32, ld, near, bj->chunk_ptr, bj->dofs, bj->local, bj->chunk_of, bj->m_max, bj->inv);
    } else {
        cudaFuncSetAttribute(bj_build_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        bj_build_kernel<false><<<(unsigned)bj->n_chunks, BJ_THREADS, smem, st>>>(
            A, nullptr, ld, near, bj->chunk_ptr, bj->dofs, bj->local, bj->chunk_of, bj->m_max, bj->inv);
    }
    e = launch_status("bj_build_kernel");
    if (e) return e;
    int bad = 0;
    cudaMemcpyFromSymbolAsync(&bad, g_bj_singular, sizeof(int), 0, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("bj_build sync", 0);
    MBEM_REQUIRE(bad == 0, MBEM_ERR_NUMERIC, "%d singular diagonal chunk(s) (identity used)", bad);
    return MBEM_OK;
}

int bj_apply(const mbem_block_jacobi* bj, const double* r, double* z, cudaStream_t st) {
    if (bj->n_chunks == 0) return MBEM_OK;
    bj_apply_kernel<<<(unsigned)bj->n_chunks, BJ_THREADS, 0, st>>>(bj->chunk_ptr, bj->dofs, bj->m_max, bj->inv,
                                                                    r, z);
    return launch_status("bj_apply_kernel");
}

int precond_apply(int kind, const void* state, const double* r, double* z, cudaStream_t st) {
    if (kind == 1) return bj_apply(static_cast<const mbem_block_jacobi*>(state), r, z, st);
    if (kind == 2) return nn_precond_apply(state, r, z, st);
    if (kind == 3) return inner_bf16_apply(state, r, z, st);
    return set_error(MBEM_ERR_ARG, "unknown preconditioner %d", kind);
}

}  // namespace mbem

using namespace mbem;

extern "C" {

size_t mbem_bj_inverse_bytes(int64_t n_chunks, int m_max) {
    return (size_t)n_chunks * m_max * m_max * sizeof(float);
}

int mbem_bj_build_dense(const double* A, int64_t ld, const mbem_block_jacobi* bj, void* stream) {
    MBEM_REQUIRE(A != nullptr && bj != nullptr && ld >= bj->n, MBEM_ERR_ARG, "bad dense operator");
    NearSet none;
    none.n = 0;
    return bj_build(A, nullptr, ld, none, bj, (cudaStream_t)stream);
}

int mbem_bj_build_mixed(const mbem_mixed_operator* op, const mbem_block_jacobi* bj, void* stream) {
    MBEM_REQUIRE(op != nullptr && op->A32 != nullptr && bj != nullptr && op->n_rows == bj->n &&
                     op->n_cols == bj->n,
                 MBEM_ERR_ARG, "bad mixed operator for block-Jacobi");
    MBEM_REQUIRE(op->n_near >= 0 && op->n_near <= BJ_MAX_NEAR, MBEM_ERR_UNSUPPORTED,
                 "%d near-block sets (at most %d)", op->n_near, BJ_MAX_NEAR);
    MBEM_REQUIRE(bj->local != nullptr && bj->chunk_of != nullptr, MBEM_ERR_ARG,
                 "the mixed build needs local and chunk_of");
    NearSet ns;
    ns.n = op->n_near;
    for (int t = 0; t < op->n_near; t++) ns.b[t] = op->near[t];
    return bj_build(nullptr, op->A32, op->ld32, ns, bj, (cudaStream_t)stream);
}

int mbem_bj_apply(const mbem_block_jacobi* bj, const double* r, double* z, void* stream) {
    int e = bj_check(bj);
    if (e) return e;
    MBEM_REQUIRE(bj->n == 0 || (r && z && r != z), MBEM_ERR_ARG, "r and z must be distinct device vectors");
    return bj_apply(bj, r, z, (cudaStream_t)stream);
}

}  // extern "C"
