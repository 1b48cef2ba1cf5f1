// Many unevenly sized meshes solved together on one GB300 (sm_103a).
//
// Every mesh keeps its own mixed-precision operator (FP32 far field, FP64
// near blocks by field point). The batch vectors concatenate the meshes'
// unknowns in segments padded to MBEM_MM_SEGMENT entries, so every
// reduction chunk belongs to one mesh and every vector kernel runs once over
// the whole batch.
//
// The operator is applied by ONE persistent launch: one CTA per SM walks a
// static list of (mesh, 16-row) work items, largest meshes first and dealt
// round-robin to the CTAs, streaming each item's rows and the matching x
// chunks (double-float hi/lo) through a warp-specialised bulk-copy ring that
// runs on across items; each consumer warp sums two rows in double-float and
// adds them to the rows' FP64 near part, which a kernel before it wrote
// into y (fetched at the item's start, so its latency hides behind the rows).
//
// The solver is deflated GMRES(m) on all meshes in lockstep: per-mesh dot
// products (fixed-order chunk partials), CGS2, normalisation and the Givens
// rotations of every mesh on the device (one thread per mesh), so a restart
// cycle of m Arnoldi steps needs no host synchronisation. It is captured once
// as a CUDA graph and replayed; a mesh whose residual estimate falls below
// the tolerance drops out of the remaining steps (its work items are
// skipped). Between cycles the host reads one residual norm per mesh.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "common.cuh"
#include "dfloat.cuh"
#include "tma_pipe.cuh"
#include "tune.cuh"

namespace mbem {

constexpr int MM_SEG = MBEM_MM_SEGMENT;  // segment alignment = reduction chunk (columns)
constexpr int MM_ROWS = 16;              // rows per work item
constexpr int MM_WARPS = MM_ROWS / 2;    // consumer warps, two rows each
constexpr int MM_THREADS = 32 * (MM_WARPS + 1);
// ring chunk (columns) and stages: template parameters, chosen from kMmTiles
template <int CH, int S>
constexpr size_t mm_smem() { return (size_t)S * (MM_ROWS + 2) * CH * sizeof(float) + 2 * S * 8; }
constexpr uint32_t MM_WAIT_LIMIT = 1u << 26;
constexpr int MM_RED = MM_SEG / 2;       // reduction threads per chunk (two columns each)
constexpr int MM_MAXV = MBEM_MM_MAX_RESTART;


// set by a ring wait that gave up; read (and cleared) by the host
__device__ int g_mm_wait_error = 0;

struct MMItem {
    int32_t mesh;
    int32_t row0;
};

// ---------------------------------------------------------------------------
// the persistent batched operator: y[seg m] = A_m x[seg m] for active meshes
// ---------------------------------------------------------------------------
template <int MM_CH, int MM_STAGES>
__global__ void __launch_bounds__(MM_THREADS)
mm_matvec_kernel(const mbem_mm_mesh* __restrict__ meshes, const MMItem* __restrict__ items, int64_t n_items,
                 const int* __restrict__ active, const float* __restrict__ xh, const float* __restrict__ xl,
                 double* __restrict__ y) {
    extern __shared__ __align__(128) unsigned char smem[];
    float* sA = reinterpret_cast<float*>(smem);                     // [S][ROWS][CH]
    float* sX = sA + MM_STAGES * MM_ROWS * MM_CH;                   // [S][2][CH]
    uint64_t* full = reinterpret_cast<uint64_t*>(sX + MM_STAGES * 2 * MM_CH);
    uint64_t* empty = full + MM_STAGES;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < MM_STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], MM_WARPS);
        }
        mbar_init_fence();
    }
    __syncthreads();
    int64_t g = 0;   // ring chunks so far; every warp walks the same sequence

    if (warp == MM_WARPS) {
        bool ok = true;
        for (int64_t it = blockIdx.x; it < n_items && ok; it += gridDim.x) {
            const MMItem item = items[it];
            if (!active[item.mesh]) continue;
            const mbem_mm_mesh M = meshes[item.mesh];
            const int nrow = (int)lmin(MM_ROWS, M.n - item.row0);
            const int64_t n_main = M.n & ~(int64_t)3;
            const int64_t nch = ceil_div(n_main, MM_CH);
            for (int64_t k = 0; k < nch; k++, g++) {
                const int s = (int)(g % MM_STAGES);
                int okl = 1;
                if (lane == 0 && g >= MM_STAGES &&
                    !mbar_wait(&empty[s], (uint32_t)(((g / MM_STAGES) - 1) & 1), MM_WAIT_LIMIT)) {
                    atomicExch(&g_mm_wait_error, 1);
                    okl = 0;
                }
                okl = __shfl_sync(0xffffffffu, okl, 0);
                if (!okl) {
                    ok = false;
                    break;
                }
                const int64_t c0 = k * MM_CH;
                const uint32_t bytes = (uint32_t)lmin(MM_CH, n_main - c0) * 4u;
                if (lane == 0) mbar_arrive_expect_tx(&full[s], bytes * (uint32_t)(nrow + 2));
                __syncwarp();
                if (lane < nrow)
                    bulk_g2s(sA + ((int64_t)s * MM_ROWS + lane) * MM_CH, M.A32 + (item.row0 + lane) * M.ld32 + c0,
                             bytes, &full[s]);
                else if (lane == MM_ROWS)
                    bulk_g2s(sX + (int64_t)s * 2 * MM_CH, xh + M.offset + c0, bytes, &full[s]);
                else if (lane == MM_ROWS + 1)
                    bulk_g2s(sX + ((int64_t)s * 2 + 1) * MM_CH, xl + M.offset + c0, bytes, &full[s]);
            }
        }
        // do not leave the block while copies into its shared memory are in flight
        if (lane == 0)
            for (int64_t q = (g > MM_STAGES ? g - MM_STAGES : 0); q < g; q++)
                if (!mbar_wait(&full[q % MM_STAGES], (uint32_t)((q / MM_STAGES) & 1), MM_WAIT_LIMIT))
                    atomicExch(&g_mm_wait_error, 1);
        return;
    }

    const int ra = 2 * warp, rb = 2 * warp + 1;
    for (int64_t it = blockIdx.x; it < n_items; it += gridDim.x) {
        const MMItem item = items[it];
        if (!active[item.mesh]) continue;
        const mbem_mm_mesh M = meshes[item.mesh];
        const int nrow = (int)lmin(MM_ROWS, M.n - item.row0);
        const int64_t n_main = M.n & ~(int64_t)3;
        const int64_t nch = ceil_div(n_main, MM_CH);
        const bool va = ra < nrow, vb = rb < nrow;
        const int rb_eff = vb ? rb : ra;
        // the rows' near part (written by mm_near_kernel), fetched now and
        // added at the end so its latency hides behind the far rows
        const double near_a = (va && lane == 0) ? y[M.offset + item.row0 + ra] : 0.0;
        const double near_b = (vb && lane == 0) ? y[M.offset + item.row0 + rb] : 0.0;
        float ah[4], al[4], bh[4], bl[4];
#pragma unroll
        for (int t = 0; t < 4; t++) ah[t] = al[t] = bh[t] = bl[t] = 0.0f;
        for (int64_t k = 0; k < nch; k++, g++) {
            const int s = (int)(g % MM_STAGES);
            if (!mbar_wait(&full[s], (uint32_t)((g / MM_STAGES) & 1), MM_WAIT_LIMIT)) {
                atomicExch(&g_mm_wait_error, 1);
                return;
            }
            if (va) {
                const int w4 = (int)(lmin(MM_CH, n_main - k * MM_CH) / 4);
                const float4* pa = reinterpret_cast<const float4*>(sA + ((int64_t)s * MM_ROWS + ra) * MM_CH);
                const float4* pb = reinterpret_cast<const float4*>(sA + ((int64_t)s * MM_ROWS + rb_eff) * MM_CH);
                const float4* h4 = reinterpret_cast<const float4*>(sX + (int64_t)s * 2 * MM_CH);
                const float4* l4 = reinterpret_cast<const float4*>(sX + ((int64_t)s * 2 + 1) * MM_CH);
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
        if (!va) continue;
        const int64_t rowa = item.row0 + ra, rowb = item.row0 + rb_eff;
        const float* xhs = xh + M.offset;
        const float* xls = xl + M.offset;
        for (int64_t c = n_main + lane; c < M.n; c += 32) {
            df_acc(ah[0], al[0], M.A32[rowa * M.ld32 + c], xhs[c], xls[c]);
            df_acc(bh[0], bl[0], M.A32[rowb * M.ld32 + c], xhs[c], xls[c]);
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
            y[M.offset + rowa] = sa + near_a;
            if (vb) y[M.offset + rowb] = sb + near_b;
        }
    }
}

// The same walk over the BF16 copies of the far fields (the inner operator
// of the mixed batch solve): 2-byte rows and FP32 x through the ring, FP32
// sums (four chains a row, two rows a warp), the FP64 near part added.
constexpr int M16_CH = 2048, M16_STAGES = 3;
constexpr size_t M16_SMEM = (size_t)M16_STAGES * (MM_ROWS * M16_CH * 2 + M16_CH * 4) + 2 * M16_STAGES * 8;

__global__ void __launch_bounds__(MM_THREADS)
mm_matvec16_kernel(const mbem_mm_mesh* __restrict__ meshes, const MMItem* __restrict__ items, int64_t n_items,
                   const int* __restrict__ active, const float* __restrict__ xf, double* __restrict__ y) {
    extern __shared__ __align__(128) unsigned char smem[];
    uint16_t* sA = reinterpret_cast<uint16_t*>(smem);                                 // [S][ROWS][CH]
    float* sX = reinterpret_cast<float*>(sA + (size_t)M16_STAGES * MM_ROWS * M16_CH);  // [S][CH]
    uint64_t* full = reinterpret_cast<uint64_t*>(sX + M16_STAGES * M16_CH);
    uint64_t* empty = full + M16_STAGES;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < M16_STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], MM_WARPS);
        }
        mbar_init_fence();
    }
    __syncthreads();
    int64_t g = 0;
    if (warp == MM_WARPS) {
        bool ok = true;
        for (int64_t it = blockIdx.x; it < n_items && ok; it += gridDim.x) {
            const MMItem item = items[it];
            if (!active[item.mesh]) continue;
            const mbem_mm_mesh M = meshes[item.mesh];
            const int nrow = (int)lmin(MM_ROWS, M.n - item.row0);
            const int64_t n_main = M.n & ~(int64_t)7;
            const int64_t nch = ceil_div(n_main, M16_CH);
            for (int64_t k = 0; k < nch; k++, g++) {
                const int s = (int)(g % M16_STAGES);
                int okl = 1;
                if (lane == 0 && g >= M16_STAGES &&
                    !mbar_wait(&empty[s], (uint32_t)(((g / M16_STAGES) - 1) & 1), MM_WAIT_LIMIT)) {
                    atomicExch(&g_mm_wait_error, 1);
                    okl = 0;
                }
                okl = __shfl_sync(0xffffffffu, okl, 0);
                if (!okl) {
                    ok = false;
                    break;
                }
                const int64_t c0 = k * M16_CH;
                const uint32_t cols = (uint32_t)lmin(M16_CH, n_main - c0);
                if (lane == 0) mbar_arrive_expect_tx(&full[s], cols * 2u * (uint32_t)nrow + cols * 4u);
                __syncwarp();
                if (lane < nrow)
                    bulk_g2s(sA + ((int64_t)s * MM_ROWS + lane) * M16_CH, M.A16 + (item.row0 + lane) * M.ld16 + c0,
                             cols * 2u, &full[s]);
                else if (lane == MM_ROWS)
                    bulk_g2s(sX + (int64_t)s * M16_CH, xf + M.offset + c0, cols * 4u, &full[s]);
            }
        }
        if (lane == 0)
            for (int64_t q = (g > M16_STAGES ? g - M16_STAGES : 0); q < g; q++)
                if (!mbar_wait(&full[q % M16_STAGES], (uint32_t)((q / M16_STAGES) & 1), MM_WAIT_LIMIT))
                    atomicExch(&g_mm_wait_error, 1);
        return;
    }
    const int ra = 2 * warp, rb = 2 * warp + 1;
    for (int64_t it = blockIdx.x; it < n_items; it += gridDim.x) {
        const MMItem item = items[it];
        if (!active[item.mesh]) continue;
        const mbem_mm_mesh M = meshes[item.mesh];
        const int nrow = (int)lmin(MM_ROWS, M.n - item.row0);
        const int64_t n_main = M.n & ~(int64_t)7;
        const int64_t nch = ceil_div(n_main, M16_CH);
        const bool va = ra < nrow, vb = rb < nrow;
        const int rb_eff = vb ? rb : ra;
        const double near_a = (va && lane == 0) ? y[M.offset + item.row0 + ra] : 0.0;
        const double near_b = (vb && lane == 0) ? y[M.offset + item.row0 + rb] : 0.0;
        float a4[4] = {0.f, 0.f, 0.f, 0.f}, b4[4] = {0.f, 0.f, 0.f, 0.f};
        for (int64_t k = 0; k < nch; k++, g++) {
            const int s = (int)(g % M16_STAGES);
            if (!mbar_wait(&full[s], (uint32_t)((g / M16_STAGES) & 1), MM_WAIT_LIMIT)) {
                atomicExch(&g_mm_wait_error, 1);
                return;
            }
            if (va) {
                const int w4 = (int)(lmin(M16_CH, n_main - k * M16_CH) / 4);
                const uint2* pa = reinterpret_cast<const uint2*>(sA + ((int64_t)s * MM_ROWS + ra) * M16_CH);
                const uint2* pb = reinterpret_cast<const uint2*>(sA + ((int64_t)s * MM_ROWS + rb_eff) * M16_CH);
                const float4* x4 = reinterpret_cast<const float4*>(sX + (int64_t)s * M16_CH);
#pragma unroll 4
                for (int q = lane; q < w4; q += 32) {
                    const float4 u = x4[q];
                    const uint2 p = pa[q], r = pb[q];
                    a4[0] = fmaf(__uint_as_float(p.x << 16), u.x, a4[0]);
                    a4[1] = fmaf(__uint_as_float(p.x & 0xffff0000u), u.y, a4[1]);
                    a4[2] = fmaf(__uint_as_float(p.y << 16), u.z, a4[2]);
                    a4[3] = fmaf(__uint_as_float(p.y & 0xffff0000u), u.w, a4[3]);
                    b4[0] = fmaf(__uint_as_float(r.x << 16), u.x, b4[0]);
                    b4[1] = fmaf(__uint_as_float(r.x & 0xffff0000u), u.y, b4[1]);
                    b4[2] = fmaf(__uint_as_float(r.y << 16), u.z, b4[2]);
                    b4[3] = fmaf(__uint_as_float(r.y & 0xffff0000u), u.w, b4[3]);
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[s]);
        }
        if (!va) continue;
        const int64_t rowa = item.row0 + ra, rowb = item.row0 + rb_eff;
        const float* xs = xf + M.offset;
        for (int64_t c = n_main + lane; c < M.n; c += 32) {
            a4[0] = fmaf(__uint_as_float((uint32_t)M.A16[rowa * M.ld16 + c] << 16), xs[c], a4[0]);
            b4[0] = fmaf(__uint_as_float((uint32_t)M.A16[rowb * M.ld16 + c] << 16), xs[c], b4[0]);
        }
        double sa = ((double)a4[0] + (double)a4[1]) + ((double)a4[2] + (double)a4[3]);
        double sb = ((double)b4[0] + (double)b4[1]) + ((double)b4[2] + (double)b4[3]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sa += __shfl_xor_sync(0xffffffffu, sa, o);
            sb += __shfl_xor_sync(0xffffffffu, sb, o);
        }
        if (lane == 0) {
            y[M.offset + rowa] = sa + near_a;
            if (vb) y[M.offset + rowb] = sb + near_b;
        }
    }
}

// y[row] = the row's FP64 near blocks times x (one warp per batch row; the
// padding and inactive meshes are skipped). mm_matvec_kernel adds the far
// part to it.
__global__ void mm_near_kernel(const mbem_mm_mesh* __restrict__ meshes, const int* __restrict__ chunk_mesh,
                               const int* __restrict__ active, const double* __restrict__ x, double* __restrict__ y,
                               int64_t n_total) {
    const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= n_total) return;
    const int m = chunk_mesh[c / MBEM_MM_SEGMENT];
    if (!active[m]) return;
    const mbem_mm_mesh& M = meshes[m];
    const int64_t row = c - M.offset;
    if (row >= M.n) return;
    const int64_t f = row / 3;
    const int comp = (int)(row % 3);
    const double* xs = x + M.offset;
    double acc = 0.0;
    for (int64_t q = M.rowptr[f] + lane; q < M.rowptr[f + 1]; q += 32) {
        const int64_t col = 3 * M.cols[q];
        const double* v = M.vals + 9 * q + 3 * comp;
        acc += v[0] * xs[col] + v[1] * xs[col + 1] + v[2] * xs[col + 2];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[c] = acc;
}

// ---------------------------------------------------------------------------
// batch vector kernels (a chunk of MM_SEG columns belongs to one mesh)
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool mesh_on(const int* active, int m) { return active == nullptr || active[m] != 0; }

__global__ void mm_split_kernel(const double* __restrict__ x, int64_t n, float* __restrict__ xh,
                                float* __restrict__ xl) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const F2 v = split_d(x[i]);
    xh[i] = v.hi;
    xl[i] = v.lo;
}

// out = in on each mesh's unknowns, 0 on the padding
__global__ void mm_masked_copy_kernel(const double* __restrict__ in, double* __restrict__ out,
                                      const mbem_mm_mesh* __restrict__ meshes, const int* __restrict__ chunk_mesh,
                                      int64_t n_total) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_total) return;
    const mbem_mm_mesh& M = meshes[chunk_mesh[c / MM_SEG]];
    out[c] = (c - M.offset < M.n) ? in[c] : 0.0;
}

// partial[c * k + i] = sum over chunk c of V[i][col] w[col]
__global__ void __launch_bounds__(MM_RED)
mm_dots_partial_kernel(const double* __restrict__ V, int64_t ldv, int k, const double* __restrict__ w,
                       const int* __restrict__ chunk_mesh, const int* __restrict__ active,
                       double* __restrict__ partial) {
    __shared__ double red[MM_RED / 32][MM_MAXV];
    const int64_t chunk = blockIdx.x;
    if (!mesh_on(active, chunk_mesh[chunk])) return;
    const int64_t c0 = chunk * MM_SEG + 2 * threadIdx.x;
    const double w0 = w[c0], w1 = w[c0 + 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int i = 0; i < k; i++) {
        const double* v = V + (int64_t)i * ldv;
        double p = fma(v[c0 + 1], w1, v[c0] * w0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
        if (lane == 0) red[wid][i] = p;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < k; i += MM_RED) {
        double s = 0.0;
        for (int q = 0; q < MM_RED / 32; q++) s += red[q][i];
        partial[chunk * k + i] = s;
    }
}

// h[m * ldh + i] (+)= sum of mesh m's chunk partials, in chunk order
__global__ void mm_dots_final_kernel(const double* __restrict__ partial, int k, const int* __restrict__ cbeg,
                                     const int* __restrict__ active, int n_mesh, int accumulate,
                                     double* __restrict__ h, int ldh) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = idx / k, i = idx % k;
    if (m >= n_mesh || !mesh_on(active, m)) return;
    double s = 0.0;
    for (int c = cbeg[m]; c < cbeg[m + 1]; c++) s += partial[(int64_t)c * k + i];
    h[(int64_t)m * ldh + i] = accumulate ? h[(int64_t)m * ldh + i] + s : s;
}

// w[col] += sign * sum_{i < min(k, cnt[m])} V[i][col] h[m * ldh + i]
__global__ void mm_axpy_kernel(double* __restrict__ w, const double* __restrict__ V, int64_t ldv, int k,
                               const double* __restrict__ h, int ldh, const int* __restrict__ cnt,
                               const int* __restrict__ chunk_mesh, const int* __restrict__ active, double sign,
                               int64_t n_total) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_total) return;
    const int m = chunk_mesh[c / MM_SEG];
    if (!mesh_on(active, m)) return;
    const int kk = cnt ? min(k, cnt[m]) : k;
    if (kk <= 0) return;
    const double* hm = h + (int64_t)m * ldh;
    double acc = w[c];
    for (int i = 0; i < kk; i++) acc = fma(V[(int64_t)i * ldv + c], sign * hm[i], acc);
    w[c] = acc;
}

// out = in / sqrt(s[m * stride]) (zero when that is not positive)
__global__ void mm_scale_kernel(const double* __restrict__ in, double* __restrict__ out,
                                const double* __restrict__ s, int stride, const int* __restrict__ chunk_mesh,
                                const int* __restrict__ active, int64_t n_total) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_total) return;
    const int m = chunk_mesh[c / MM_SEG];
    if (!mesh_on(active, m)) return;
    const double v = s[(int64_t)m * stride];
    out[c] = in[c] * (v > 0.0 ? 1.0 / sqrt(v) : 0.0);
}

// y = a x + b y on the active meshes
__global__ void mm_axpby_kernel(double* __restrict__ y, const double* __restrict__ x, double a, double b,
                                const int* __restrict__ chunk_mesh, const int* __restrict__ active,
                                int64_t n_total) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_total) return;
    if (!mesh_on(active, chunk_mesh[c / MM_SEG])) return;
    y[c] = a * x[c] + b * y[c];
}

// deflation: per-chunk sums of the three components over the mesh's u-range
__global__ void __launch_bounds__(MM_RED)
mm_proj_partial_kernel(const double* __restrict__ v, const mbem_mm_mesh* __restrict__ meshes,
                       const int* __restrict__ chunk_mesh, const int* __restrict__ active,
                       double* __restrict__ partial3) {
    __shared__ double red[MM_RED / 32][3];
    const int64_t chunk = blockIdx.x;
    const int m = chunk_mesh[chunk];
    if (!mesh_on(active, m)) return;
    const mbem_mm_mesh& M = meshes[m];
    double acc[3] = {0.0, 0.0, 0.0};
    for (int t = 0; t < 2; t++) {
        const int64_t c = chunk * MM_SEG + 2 * threadIdx.x + t;
        const int64_t u = c - M.offset - M.u_off;
        if (u >= 0 && u < M.u_len) acc[u % 3] += v[c];
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
        for (int q = 0; q < MM_RED / 32; q++) s += red[q][threadIdx.x];
        partial3[chunk * 3 + threadIdx.x] = s;
    }
}

__global__ void mm_proj_final_kernel(const double* __restrict__ partial3, const int* __restrict__ cbeg,
                                     const mbem_mm_mesh* __restrict__ meshes, const int* __restrict__ active,
                                     int n_mesh, double* __restrict__ mean) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = idx / 3, k = idx % 3;
    if (m >= n_mesh || !mesh_on(active, m)) return;
    double s = 0.0;
    for (int c = cbeg[m]; c < cbeg[m + 1]; c++) s += partial3[(int64_t)c * 3 + k];
    const int64_t nodes = meshes[m].u_len / 3;
    mean[3 * m + k] = nodes > 0 ? s / (double)nodes : 0.0;
}

__global__ void mm_proj_apply_kernel(double* __restrict__ v, const mbem_mm_mesh* __restrict__ meshes,
                                     const int* __restrict__ chunk_mesh, const int* __restrict__ active,
                                     const double* __restrict__ mean, int64_t n_total) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_total) return;
    const int m = chunk_mesh[c / MM_SEG];
    if (!mesh_on(active, m)) return;
    const mbem_mm_mesh& M = meshes[m];
    const int64_t u = c - M.offset - M.u_off;
    if (u >= 0 && u < M.u_len) v[c] -= mean[3 * m + u % 3];
}

// one Givens step per mesh (la/solver.py:188-205): rotates Hessenberg
// column j of mesh m, forms the new rotation, updates g and the residual
// estimate; a mesh below rtol (or at an exact breakdown) leaves the cycle
__global__ void mm_givens_kernel(int n_mesh, int j, int ldm, const double* __restrict__ hcol, int ldh,
                                 double* __restrict__ R, double* __restrict__ cs, double* __restrict__ sn,
                                 double* __restrict__ g, int* __restrict__ active, int* __restrict__ jdone,
                                 int* __restrict__ iters, const double* __restrict__ bnorm, double rtol) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n_mesh || !active[m]) return;
    const double* h = hcol + (int64_t)m * ldh;
    double* Rm = R + (int64_t)m * ldm * ldm;
    double* c = cs + (int64_t)m * ldm;
    double* s = sn + (int64_t)m * ldm;
    double* gm = g + (int64_t)m * (ldm + 1);
    double prev = h[0];
    for (int i = 0; i < j; i++) {
        const double nxt = h[i + 1];
        Rm[(int64_t)i * ldm + j] = c[i] * prev + s[i] * nxt;
        prev = -s[i] * prev + c[i] * nxt;
    }
    const double hjj = prev, hj1 = sqrt(fmax(h[j + 1], 0.0));
    const double den = sqrt(hjj * hjj + hj1 * hj1);
    if (den == 0.0) {
        active[m] = 0;
        return;
    }
    c[j] = fabs(hjj) > 0 ? fabs(hjj) / den : 0.0;
    s[j] = fabs(hjj) > 0 ? (hjj / fabs(hjj)) * hj1 / den : 1.0;
    Rm[(int64_t)j * ldm + j] = c[j] * hjj + s[j] * hj1;
    gm[j + 1] = -s[j] * gm[j];
    gm[j] = c[j] * gm[j];
    jdone[m] = j + 1;
    iters[m] += 1;
    if (fabs(gm[j + 1]) < rtol * bnorm[m] || hj1 == 0.0) active[m] = 0;
}

// y_m = R_m^-1 g_m over the mesh's jdone columns (zeros beyond)
__global__ void mm_backsolve_kernel(int n_mesh, int ldm, const double* __restrict__ R,
                                    const double* __restrict__ g, const int* __restrict__ jdone,
                                    double* __restrict__ y) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n_mesh) return;
    const int jd = jdone[m];
    const double* Rm = R + (int64_t)m * ldm * ldm;
    const double* gm = g + (int64_t)m * (ldm + 1);
    double* ym = y + (int64_t)m * ldm;
    for (int i = ldm - 1; i >= 0; i--) {
        if (i >= jd) {
            ym[i] = 0.0;
            continue;
        }
        double v = gm[i];
        for (int q = i + 1; q < jd; q++) v -= Rm[(int64_t)i * ldm + q] * ym[q];
        ym[i] = v / Rm[(int64_t)i * ldm + i];
    }
}

// hcol[m, i] += h2[m, i] for i <= j on the active meshes
__global__ void mm_hadd_kernel(int n_mesh, int j, double* __restrict__ hcol, const double* __restrict__ h2, int ldh,
                               const int* __restrict__ active) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = idx / (j + 1), i = idx % (j + 1);
    if (m >= n_mesh || !active[m]) return;
    hcol[(int64_t)m * ldh + i] += h2[(int64_t)m * ldh + i];
}

__global__ void mm_cycle_start_kernel(int n_mesh, int ldm, const double* __restrict__ rn2,
                                      double* __restrict__ g, int* __restrict__ jdone, const int* __restrict__ active) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n_mesh) return;
    double* gm = g + (int64_t)m * (ldm + 1);
    for (int i = 0; i <= ldm; i++) gm[i] = 0.0;
    gm[0] = active[m] ? sqrt(fmax(rn2[m], 0.0)) : 0.0;
    jdone[m] = 0;
}

}  // namespace mbem

using namespace mbem;

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct mbem_mm_solver {
    int n_mesh = 0, restart = 0;
    int64_t n_total = 0, n_chunks = 0, n_items = 0;
    int grid = 0;
    std::vector<mbem_mm_mesh> meshes;
    // device buffers (inside the caller's workspace)
    mbem_mm_mesh* d_meshes = nullptr;
    MMItem* d_items = nullptr;
    int* chunk_mesh = nullptr;
    int* cbeg = nullptr;
    int* active = nullptr;    // Arnoldi flags
    int* all_on = nullptr;    // every mesh (whole-batch operations)
    int* jdone = nullptr;
    int* iters = nullptr;
    double* V = nullptr;      // (restart + 1) x n_total
    double* W = nullptr;
    double* R = nullptr;      // residual
    double* Bz = nullptr;     // the right-hand side with zero padding
    float* xh = nullptr;
    float* xl = nullptr;
    double* partial = nullptr;  // n_chunks x MM_MAXV
    double* hcol = nullptr;     // n_mesh x (restart + 2)
    double* h2 = nullptr;
    double* Rh = nullptr;       // n_mesh x restart x restart
    double* cs = nullptr;
    double* sn = nullptr;
    double* g = nullptr;        // n_mesh x (restart + 1)
    double* y = nullptr;        // n_mesh x restart
    double* rn2 = nullptr;      // n_mesh
    double* bnorm = nullptr;    // n_mesh
    double* mean = nullptr;     // n_mesh x 3
    double* Bfull = nullptr;    // the outer right-hand side (mixed solve)
    double* D = nullptr;        // an inner correction (mixed solve)
    bool has16 = false;         // every mesh has its BF16 far field
    int op16 = 0;               // the operator of the next products: 1 = BF16 inner
    // the captured restart cycle of each operator (0 FP32, 1 BF16)
    cudaGraphExec_t cycle[2] = {nullptr, nullptr};
    double cycle_rtol[2] = {-1.0, -1.0};
    int cycle_cfg[2] = {-1, -1};      // tile configuration captured in the cycle
    long long cycle_kernels[2] = {0, 0};
};

namespace {

size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

struct MMCounts {
    int64_t n_total, n_chunks, n_items;
};

int mm_check(const mbem_mm_mesh* meshes, int n_mesh, int restart, MMCounts* out) {
    MBEM_REQUIRE(meshes != nullptr && n_mesh >= 1, MBEM_ERR_ARG, "no meshes");
    MBEM_REQUIRE(restart >= 1 && restart <= MM_MAXV, MBEM_ERR_ARG, "restart must be in [1, %d]", MM_MAXV);
    int64_t end = 0, items = 0;
    for (int m = 0; m < n_mesh; m++) {
        const mbem_mm_mesh& M = meshes[m];
        MBEM_REQUIRE(M.n > 0 && M.n % 3 == 0 && M.n <= 0x7fffffff, MBEM_ERR_ARG, "mesh %d: bad size %lld", m,
                     (long long)M.n);
        MBEM_REQUIRE(M.A32 && (uintptr_t)M.A32 % 16 == 0 && M.ld32 >= M.n && M.ld32 % 4 == 0, MBEM_ERR_ARG,
                     "mesh %d: the FP32 far field must be 16-byte aligned with ld32 >= n, ld32 %% 4 == 0", m);
        MBEM_REQUIRE(M.rowptr && M.cols && M.vals, MBEM_ERR_ARG, "mesh %d: NULL near blocks", m);
        MBEM_REQUIRE(M.A16 == nullptr || ((uintptr_t)M.A16 % 16 == 0 && M.ld16 >= M.n && M.ld16 % 8 == 0),
                     MBEM_ERR_ARG, "mesh %d: the BF16 far field must be 16-byte aligned with ld16 >= n, ld16 %% 8 == 0",
                     m);
        MBEM_REQUIRE(M.offset == end, MBEM_ERR_ARG,
                     "mesh %d: offset %lld must be %lld (segments follow one another, each rounded up to %d)", m,
                     (long long)M.offset, (long long)end, MM_SEG);
        MBEM_REQUIRE(M.u_off >= 0 && M.u_len >= 0 && M.u_len % 3 == 0 && M.u_off + M.u_len <= M.n, MBEM_ERR_ARG,
                     "mesh %d: bad u-range", m);
        end = M.offset + ceil_div(M.n, MM_SEG) * MM_SEG;
        items += ceil_div(M.n, MM_ROWS);
    }
    out->n_total = end;
    out->n_chunks = end / MM_SEG;
    out->n_items = items;
    return MBEM_OK;
}

// carves the workspace (base == nullptr: sizes only)
size_t mm_layout(int n_mesh, int restart, const MMCounts& k, char* base, mbem_mm_solver* s) {
    size_t off = 0;
    auto take = [&](size_t bytes) -> char* {
        char* p = base ? base + off : nullptr;
        off += al256(bytes);
        return p;
    };
    const size_t nm = (size_t)n_mesh, m = (size_t)restart, nt = (size_t)k.n_total;
    char* p_meshes = take(nm * sizeof(mbem_mm_mesh));
    char* p_items = take((size_t)k.n_items * sizeof(MMItem));
    char* p_chunk = take((size_t)k.n_chunks * sizeof(int));
    char* p_cbeg = take((nm + 1) * sizeof(int));
    char* p_active = take(nm * sizeof(int));
    char* p_all = take(nm * sizeof(int));
    char* p_jdone = take(nm * sizeof(int));
    char* p_iters = take(nm * sizeof(int));
    char* p_V = take((m + 1) * nt * sizeof(double));
    char* p_W = take(nt * sizeof(double));
    char* p_R = take(nt * sizeof(double));
    char* p_B = take(nt * sizeof(double));
    char* p_xh = take(nt * sizeof(float));
    char* p_xl = take(nt * sizeof(float));
    char* p_partial = take((size_t)k.n_chunks * MM_MAXV * sizeof(double));
    char* p_hcol = take(nm * (m + 2) * sizeof(double));
    char* p_h2 = take(nm * (m + 2) * sizeof(double));
    char* p_Rh = take(nm * m * m * sizeof(double));
    char* p_cs = take(nm * m * sizeof(double));
    char* p_sn = take(nm * m * sizeof(double));
    char* p_g = take(nm * (m + 1) * sizeof(double));
    char* p_y = take(nm * m * sizeof(double));
    char* p_rn2 = take(nm * sizeof(double));
    char* p_bn = take(nm * sizeof(double));
    char* p_mean = take(nm * 3 * sizeof(double));
    char* p_bfull = take(nt * sizeof(double));
    char* p_d = take(nt * sizeof(double));
    if (s) {
        s->d_meshes = (mbem_mm_mesh*)p_meshes;
        s->d_items = (MMItem*)p_items;
        s->chunk_mesh = (int*)p_chunk;
        s->cbeg = (int*)p_cbeg;
        s->active = (int*)p_active;
        s->all_on = (int*)p_all;
        s->jdone = (int*)p_jdone;
        s->iters = (int*)p_iters;
        s->V = (double*)p_V;
        s->W = (double*)p_W;
        s->R = (double*)p_R;
        s->Bz = (double*)p_B;
        s->xh = (float*)p_xh;
        s->xl = (float*)p_xl;
        s->partial = (double*)p_partial;
        s->hcol = (double*)p_hcol;
        s->h2 = (double*)p_h2;
        s->Rh = (double*)p_Rh;
        s->cs = (double*)p_cs;
        s->sn = (double*)p_sn;
        s->g = (double*)p_g;
        s->y = (double*)p_y;
        s->rn2 = (double*)p_rn2;
        s->bnorm = (double*)p_bn;
        s->mean = (double*)p_mean;
        s->Bfull = (double*)p_bfull;
        s->D = (double*)p_d;
    }
    return off;
}

unsigned blocks(int64_t n, int t = 256) { return (unsigned)ceil_div(n > 0 ? n : 1, t); }

template <int CH, int S>
int mm_far_launch(mbem_mm_solver* s, double* y, const int* on, cudaStream_t st) {
    constexpr size_t smem = mm_smem<CH, S>();
    static_assert(smem <= 232448, "ring exceeds 227 KB of shared memory");
    // one CTA per SM, or two where two rings fit
    const unsigned grid = (unsigned)(s->grid * (2 * smem <= 232448 ? 2 : 1));
    mm_matvec_kernel<CH, S><<<grid, MM_THREADS, smem, st>>>(s->d_meshes, s->d_items, s->n_items, on, s->xh,
                                                           s->xl, y);
    return MBEM_OK;
}

template <int CH, int S>
cudaError_t mm_far_attribute() {
    return cudaFuncSetAttribute(mm_matvec_kernel<CH, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)mm_smem<CH, S>());
}

#define MBEM_MM_CASES(X) X(0) X(1) X(2) X(3)
static_assert(count_of(kMmTiles) == 4, "one case per configuration");

// y = A x on the meshes flagged in `on` (s->op16: the BF16 inner operator)
int mm_apply(mbem_mm_solver* s, const double* x, double* y, const int* on, cudaStream_t st) {
    mm_split_kernel<<<blocks(s->n_total), 256, 0, st>>>(x, s->n_total, s->xh, s->xl);
    mm_near_kernel<<<blocks(s->n_total * 32), 256, 0, st>>>(s->d_meshes, s->chunk_mesh, on, x, y, s->n_total);
    if (s->op16) {
        // xh = x rounded to FP32
        mm_matvec16_kernel<<<(unsigned)s->grid, MM_THREADS, M16_SMEM, st>>>(s->d_meshes, s->d_items, s->n_items, on,
                                                                            s->xh, y);
        return launch_status("mm_matvec16_kernel", 3);
    }
    int e = set_error(MBEM_ERR_ARG, "no multi-mesh tile configuration %d", tune_get(MBEM_TUNE_MM_MATVEC));
    switch (tune_get(MBEM_TUNE_MM_MATVEC)) {
#define MBEM_MM_CASE(i) \
        case i: e = mm_far_launch<kMmTiles[i].ch, kMmTiles[i].stages>(s, y, on, st); break;
        MBEM_MM_CASES(MBEM_MM_CASE)
#undef MBEM_MM_CASE
        default: break;
    }
    if (e) return e;
    return launch_status("mm_matvec_kernel", 3);
}

// h[m * ldh + i] (+)= V[i] . w over mesh m, i < k
int mm_dots(mbem_mm_solver* s, const double* V, int k, const double* w, const int* on, int accumulate, double* h,
            int ldh, cudaStream_t st) {
    mm_dots_partial_kernel<<<(unsigned)s->n_chunks, MM_RED, 0, st>>>(V, s->n_total, k, w, s->chunk_mesh, on,
                                                                      s->partial);
    mm_dots_final_kernel<<<blocks((int64_t)s->n_mesh * k, 128), 128, 0, st>>>(s->partial, k, s->cbeg, on,
                                                                              s->n_mesh, accumulate, h, ldh);
    return launch_status("mm_dots", 2);
}

int mm_project(mbem_mm_solver* s, double* v, const int* on, cudaStream_t st) {
    mm_proj_partial_kernel<<<(unsigned)s->n_chunks, MM_RED, 0, st>>>(v, s->d_meshes, s->chunk_mesh, on,
                                                                      s->partial);
    mm_proj_final_kernel<<<blocks((int64_t)s->n_mesh * 3, 128), 128, 0, st>>>(s->partial, s->cbeg, s->d_meshes, on,
                                                                              s->n_mesh, s->mean);
    mm_proj_apply_kernel<<<blocks(s->n_total), 256, 0, st>>>(v, s->d_meshes, s->chunk_mesh, on, s->mean,
                                                             s->n_total);
    return launch_status("mm_project", 3);
}

// one Arnoldi step j on the active meshes (no host synchronisation)
int mm_step(mbem_mm_solver* s, int j, double rtol, cudaStream_t st) {
    const int m = s->restart, ldh = m + 2;
    const int64_t nt = s->n_total;
    double* vj = s->V + (int64_t)j * nt;
    int e;
    if ((e = mm_apply(s, vj, s->W, s->active, st))) return e;
    if ((e = mm_project(s, s->W, s->active, st))) return e;
    // CGS2: h = V^T w, w -= V h, twice; the column is the sum
    if ((e = mm_dots(s, s->V, j + 1, s->W, s->active, 0, s->hcol, ldh, st))) return e;
    mm_axpy_kernel<<<blocks(nt), 256, 0, st>>>(s->W, s->V, nt, j + 1, s->hcol, ldh, nullptr, s->chunk_mesh,
                                               s->active, -1.0, nt);
    if ((e = mm_dots(s, s->V, j + 1, s->W, s->active, 0, s->h2, ldh, st))) return e;
    mm_axpy_kernel<<<blocks(nt), 256, 0, st>>>(s->W, s->V, nt, j + 1, s->h2, ldh, nullptr, s->chunk_mesh,
                                               s->active, -1.0, nt);
    // hcol += h2 (the norm pass below writes entry j + 1)
    mm_hadd_kernel<<<blocks((int64_t)s->n_mesh * (j + 1), 128), 128, 0, st>>>(s->n_mesh, j, s->hcol, s->h2, ldh,
                                                                              s->active);
    if ((e = mm_dots(s, s->W, 1, s->W, s->active, 0, s->hcol + (j + 1), ldh, st))) return e;
    mm_scale_kernel<<<blocks(nt), 256, 0, st>>>(s->W, s->V + (int64_t)(j + 1) * nt, s->hcol + (j + 1), ldh,
                                                s->chunk_mesh, s->active, nt);
    mm_givens_kernel<<<blocks(s->n_mesh, 64), 64, 0, st>>>(s->n_mesh, j, m, s->hcol, ldh, s->Rh, s->cs, s->sn, s->g,
                                                           s->active, s->jdone, s->iters, s->bnorm, rtol);
    return launch_status("mm_step", 5);
}

}  // namespace


extern "C" {

size_t mbem_mm_workspace_size(const mbem_mm_mesh* meshes, int n_mesh, int restart) {
    MMCounts k;
    if (mm_check(meshes, n_mesh, restart, &k) != MBEM_OK) return 0;
    return mm_layout(n_mesh, restart, k, nullptr, nullptr);
}

int64_t mbem_mm_total(const mbem_mm_mesh* meshes, int n_mesh) {
    MMCounts k;
    if (mm_check(meshes, n_mesh, 1, &k) != MBEM_OK) return -1;
    return k.n_total;
}

int mbem_mm_create(const mbem_mm_mesh* meshes, int n_mesh, int restart, void* work, size_t work_bytes, void* stream,
                   mbem_mm_solver** out) {
    MBEM_REQUIRE(out != nullptr, MBEM_ERR_ARG, "out is NULL");
    *out = nullptr;
    MMCounts k;
    int e = mm_check(meshes, n_mesh, restart, &k);
    if (e) return e;
    const size_t need = mm_layout(n_mesh, restart, k, nullptr, nullptr);
    MBEM_REQUIRE(work && work_bytes >= need, MBEM_ERR_SIZE, "multi-mesh workspace %zu < %zu bytes", work_bytes,
                 need);
    MBEM_REQUIRE((uintptr_t)work % 256 == 0, MBEM_ERR_ARG, "the workspace must be 256-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    mbem_mm_solver* s = new (std::nothrow) mbem_mm_solver();
    MBEM_REQUIRE(s != nullptr, MBEM_ERR_ARG, "out of host memory");
    s->n_mesh = n_mesh;
    s->restart = restart;
    s->n_total = k.n_total;
    s->n_chunks = k.n_chunks;
    s->n_items = k.n_items;
    s->meshes.assign(meshes, meshes + n_mesh);
    s->has16 = true;
    for (int m = 0; m < n_mesh; m++)
        if (meshes[m].A16 == nullptr) s->has16 = false;
    mm_layout(n_mesh, restart, k, (char*)work, s);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    s->grid = sms > 0 ? sms : 1;
    // shared-memory limits of every tile configuration, set before any capture
    cudaError_t ce = cudaSuccess;
#define MBEM_MM_ATTR(i) \
    if (ce == cudaSuccess) ce = mm_far_attribute<kMmTiles[i].ch, kMmTiles[i].stages>();
    MBEM_MM_CASES(MBEM_MM_ATTR)
#undef MBEM_MM_ATTR
    if (ce == cudaSuccess)
        ce = cudaFuncSetAttribute(mm_matvec16_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)M16_SMEM);
    if (ce != cudaSuccess) {
        delete s;
        return set_error(MBEM_ERR_CUDA, "multi-mesh matvec smem attribute: %s", cudaGetErrorString(ce));
    }
    // work items: meshes by decreasing size, 16 rows each, dealt round-robin
    // to the persistent CTAs by their position in this list
    std::vector<int> order(n_mesh);
    for (int m = 0; m < n_mesh; m++) order[m] = m;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return meshes[a].n > meshes[b].n; });
    std::vector<MMItem> items;
    items.reserve((size_t)k.n_items);
    for (int m : order)
        for (int64_t r = 0; r < meshes[m].n; r += MM_ROWS) items.push_back({m, (int32_t)r});
    std::vector<int> chunk_mesh((size_t)k.n_chunks, 0), cbeg(n_mesh + 1, 0), ones(n_mesh, 1);
    // mesh m owns chunks [cbeg[m], cbeg[m + 1]) (segments are contiguous)
    for (int m = 0; m < n_mesh; m++) {
        const int64_t c0 = meshes[m].offset / MM_SEG, c1 = c0 + ceil_div(meshes[m].n, MM_SEG);
        for (int64_t c = c0; c < c1; c++) chunk_mesh[c] = m;
        cbeg[m] = (int)c0;
    }
    cbeg[n_mesh] = (int)k.n_chunks;
    cudaMemcpyAsync(s->d_meshes, meshes, sizeof(mbem_mm_mesh) * n_mesh, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(s->d_items, items.data(), sizeof(MMItem) * items.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(s->chunk_mesh, chunk_mesh.data(), sizeof(int) * chunk_mesh.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(s->cbeg, cbeg.data(), sizeof(int) * cbeg.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(s->all_on, ones.data(), sizeof(int) * n_mesh, cudaMemcpyHostToDevice, st);
    // zero padding stays zero in every batch vector
    cudaMemsetAsync(s->V, 0, sizeof(double) * (size_t)(restart + 1) * k.n_total, st);
    cudaMemsetAsync(s->W, 0, sizeof(double) * (size_t)k.n_total, st);
    cudaMemsetAsync(s->R, 0, sizeof(double) * (size_t)k.n_total, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        delete s;
        return launch_status("multi-mesh setup", 0);
    }
    *out = s;
    return MBEM_OK;
}

void mbem_mm_destroy(mbem_mm_solver* s) {
    if (!s) return;
    for (int op = 0; op < 2; op++)
        if (s->cycle[op]) cudaGraphExecDestroy(s->cycle[op]);
    delete s;
}

int mbem_mm_matvec(mbem_mm_solver* s, const double* x, double* y, void* stream) {
    MBEM_REQUIRE(s && x && y, MBEM_ERR_ARG, "bad multi-mesh matvec args");
    return mm_apply(s, x, y, s->all_on, (cudaStream_t)stream);
}

static int mm_wait_check(cudaStream_t st) {
    int flag = 0;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaMemcpyFromSymbol(&flag, g_mm_wait_error, sizeof(int));
    if (e != cudaSuccess) return set_error(MBEM_ERR_CUDA, "multi-mesh wait check: %s", cudaGetErrorString(e));
    if (flag) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_mm_wait_error, &zero, sizeof(int));
        return set_error(MBEM_ERR_WAIT, "a bulk-copy ring wait expired in the multi-mesh matvec");
    }
    return MBEM_OK;
}

int mbem_mm_check(void* stream) { return mm_wait_check((cudaStream_t)stream); }

// The lockstep deflated GMRES(restart) core: every mesh not flagged in
// `conv` solves (its operator: s->op16) for the right-hand side in s->Bz
// from X = 0 to rtol of its own |P b|, at most max_cycles restart cycles.
// relres: each mesh's true relative residual at its last check; conv: set
// for the meshes that reached rtol (or have b = 0).
static int mm_gmres(mbem_mm_solver* s, double* X, double rtol, int max_cycles, int use_graph, std::vector<int>& conv,
                    std::vector<double>& relres, int& cycles, cudaStream_t st) {
    const int nm = s->n_mesh, m = s->restart;
    const int64_t nt = s->n_total;
    const int op = s->op16 ? 1 : 0;
    int e;
    std::vector<double> bn2(nm), rn2(nm), bnorm(nm);
    std::vector<int> act(nm);
    cudaMemcpyAsync(s->R, s->Bz, sizeof(double) * nt, cudaMemcpyDeviceToDevice, st);
    if ((e = mm_project(s, s->R, s->all_on, st))) return e;
    if ((e = mm_dots(s, s->R, 1, s->R, s->all_on, 0, s->rn2, 1, st))) return e;
    cudaMemcpyAsync(bn2.data(), s->rn2, sizeof(double) * nm, cudaMemcpyDeviceToHost, st);
    cudaMemsetAsync(X, 0, sizeof(double) * nt, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("multi-mesh solve", 0);
    for (int q = 0; q < nm; q++) bnorm[q] = sqrt(bn2[q]);
    cudaMemcpyAsync(s->bnorm, bnorm.data(), sizeof(double) * nm, cudaMemcpyHostToDevice, st);
    bool x_zero = true;
    cycles = 0;
    for (;;) {
        // r = P (b - A x) on the meshes not yet converged (P b while x == 0)
        for (int q = 0; q < nm; q++) act[q] = conv[q] ? 0 : 1;
        cudaMemcpyAsync(s->active, act.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, st);
        if (!x_zero) {
            if ((e = mm_apply(s, X, s->W, s->active, st))) return e;
            cudaMemcpyAsync(s->R, s->Bz, sizeof(double) * nt, cudaMemcpyDeviceToDevice, st);
            mm_axpby_kernel<<<blocks(nt), 256, 0, st>>>(s->R, s->W, -1.0, 1.0, s->chunk_mesh, s->active, nt);
            if ((e = mm_project(s, s->R, s->active, st))) return e;
            if ((e = mm_dots(s, s->R, 1, s->R, s->active, 0, s->rn2, 1, st))) return e;
            cudaMemcpyAsync(rn2.data(), s->rn2, sizeof(double) * nm, cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("multi-mesh solve", 0);
        } else {
            rn2 = bn2;
        }
        bool any = false;
        for (int q = 0; q < nm; q++) {
            if (conv[q]) continue;
            relres[q] = bnorm[q] > 0.0 ? sqrt(rn2[q]) / bnorm[q] : 0.0;
            if (bnorm[q] == 0.0 || relres[q] < rtol) conv[q] = 1;
            else any = true;
        }
        if (!any || cycles >= max_cycles) break;
        // the cycle: V_0 = r / |r|, then m Arnoldi steps on the device
        for (int q = 0; q < nm; q++) act[q] = conv[q] ? 0 : 1;
        cudaMemcpyAsync(s->active, act.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(s->rn2, rn2.data(), sizeof(double) * nm, cudaMemcpyHostToDevice, st);
        mm_cycle_start_kernel<<<blocks(nm, 64), 64, 0, st>>>(nm, m, s->rn2, s->g, s->jdone, s->active);
        mm_scale_kernel<<<blocks(nt), 256, 0, st>>>(s->R, s->V, s->rn2, 1, s->chunk_mesh, s->active, nt);
        if (use_graph) {
            if (s->cycle[op] == nullptr || s->cycle_rtol[op] != rtol ||
                s->cycle_cfg[op] != tune_get(MBEM_TUNE_MM_MATVEC)) {
                if (s->cycle[op]) {
                    cudaGraphExecDestroy(s->cycle[op]);
                    s->cycle[op] = nullptr;
                }
                cudaGraph_t graph = nullptr;
                const unsigned long long before = mbem_launch_count();
                cudaError_t ce = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
                if (ce != cudaSuccess) return set_error(MBEM_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
                int es = MBEM_OK;
                for (int j = 0; j < m && es == MBEM_OK; j++) es = mm_step(s, j, rtol, st);
                ce = cudaStreamEndCapture(st, &graph);
                // captured launches run when the graph does: count them per replay
                s->cycle_kernels[op] = (long long)(mbem_launch_count() - before);
                count_launches((int)-s->cycle_kernels[op]);
                if (es) {
                    if (graph) cudaGraphDestroy(graph);
                    return es;
                }
                if (ce != cudaSuccess) return set_error(MBEM_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
                ce = cudaGraphInstantiate(&s->cycle[op], graph, 0);
                cudaGraphDestroy(graph);
                if (ce != cudaSuccess) {
                    s->cycle[op] = nullptr;
                    return set_error(MBEM_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
                }
                s->cycle_rtol[op] = rtol;
                s->cycle_cfg[op] = tune_get(MBEM_TUNE_MM_MATVEC);
            }
            cudaError_t ce = cudaGraphLaunch(s->cycle[op], st);
            if (ce != cudaSuccess) return set_error(MBEM_ERR_CUDA, "graph launch: %s", cudaGetErrorString(ce));
            count_launches((int)s->cycle_kernels[op]);
        } else {
            for (int j = 0; j < m; j++)
                if ((e = mm_step(s, j, rtol, st))) return e;
        }
        // x += V y on every mesh that took steps
        mm_backsolve_kernel<<<blocks(nm, 64), 64, 0, st>>>(nm, m, s->Rh, s->g, s->jdone, s->y);
        mm_axpy_kernel<<<blocks(nt), 256, 0, st>>>(X, s->V, nt, m, s->y, m, s->jdone, s->chunk_mesh, nullptr, 1.0,
                                                   nt);
        if ((e = launch_status("mm_update", 4))) return e;
        x_zero = false;
        cycles++;
    }
    return MBEM_OK;
}

static int mm_finish(mbem_mm_solver* s, double* X, const std::vector<int>& conv, const std::vector<double>& relres,
                     int cycles, mbem_mm_report* rep, cudaStream_t st) {
    const int nm = s->n_mesh;
    int e;
    // the zero-mean representative P x
    if ((e = mm_project(s, X, s->all_on, st))) return e;
    std::vector<int> its(nm);
    cudaMemcpyAsync(its.data(), s->iters, sizeof(int) * nm, cudaMemcpyDeviceToHost, st);
    if ((e = mm_wait_check(st))) return e;
    for (int q = 0; q < nm; q++) {
        rep->iterations[q] = its[q];
        rep->converged[q] = conv[q];
        rep->relres[q] = relres[q];
    }
    rep->cycles = cycles;
    return MBEM_OK;
}

int mbem_mm_solve(mbem_mm_solver* s, const double* B, double* X, double rtol, int max_cycles, int use_graph,
                  mbem_mm_report* rep, void* stream) {
    MBEM_REQUIRE(s && B && X && rep, MBEM_ERR_ARG, "bad multi-mesh solve args");
    MBEM_REQUIRE(rtol > 0.0 && rtol < 1.0 && max_cycles >= 1, MBEM_ERR_ARG, "bad rtol / max_cycles");
    MBEM_REQUIRE(rep->iterations && rep->relres && rep->converged, MBEM_ERR_ARG,
                 "report arrays (n_mesh each) are NULL");
    cudaStream_t st = (cudaStream_t)stream;
    const int nm = s->n_mesh;
    const int64_t nt = s->n_total;
    std::vector<int> conv(nm, 0);
    std::vector<double> relres(nm, 0.0);
    int cycles = 0;
    s->op16 = 0;
    mm_masked_copy_kernel<<<blocks(nt), 256, 0, st>>>(B, s->Bz, s->d_meshes, s->chunk_mesh, nt);
    cudaMemsetAsync(s->iters, 0, sizeof(int) * nm, st);
    int e = mm_gmres(s, X, rtol, max_cycles, use_graph, conv, relres, cycles, st);
    if (e) return e;
    return mm_finish(s, X, conv, relres, cycles, rep, st);
}

// The mixed-precision batch solve: refinement on the accurate operator (FP32
// far field with double-float sums, FP64 near blocks) whose corrections are
// lockstep GMRES solves on the BF16 far fields to inner_rtol of each
// residual. rep->iterations: the inner steps of each mesh; rep->relres: the
// true residual of the accurate operator; rep->cycles: refinement steps.
int mbem_mm_solve_mixed(mbem_mm_solver* s, const double* B, double* X, double rtol, double inner_rtol, int max_outer,
                        int max_cycles, int use_graph, mbem_mm_report* rep, void* stream) {
    MBEM_REQUIRE(s && B && X && rep, MBEM_ERR_ARG, "bad multi-mesh solve args");
    MBEM_REQUIRE(s->has16, MBEM_ERR_ARG, "the mixed batch solve needs every mesh's BF16 far field (A16)");
    MBEM_REQUIRE(rtol > 0.0 && rtol < 1.0 && inner_rtol > 0.0 && inner_rtol < 1.0 && max_outer >= 1 &&
                     max_cycles >= 1,
                 MBEM_ERR_ARG, "bad tolerances or step limits");
    MBEM_REQUIRE(rep->iterations && rep->relres && rep->converged, MBEM_ERR_ARG,
                 "report arrays (n_mesh each) are NULL");
    cudaStream_t st = (cudaStream_t)stream;
    const int nm = s->n_mesh;
    const int64_t nt = s->n_total;
    int e;
    std::vector<int> conv(nm, 0), act(nm);
    std::vector<double> relres(nm, 0.0), bn2(nm), rn2(nm);
    // B with zero padding, |P B| per mesh
    mm_masked_copy_kernel<<<blocks(nt), 256, 0, st>>>(B, s->Bfull, s->d_meshes, s->chunk_mesh, nt);
    cudaMemcpyAsync(s->Bz, s->Bfull, sizeof(double) * nt, cudaMemcpyDeviceToDevice, st);
    if ((e = mm_project(s, s->Bz, s->all_on, st))) return e;
    if ((e = mm_dots(s, s->Bz, 1, s->Bz, s->all_on, 0, s->rn2, 1, st))) return e;
    cudaMemcpyAsync(bn2.data(), s->rn2, sizeof(double) * nm, cudaMemcpyDeviceToHost, st);
    cudaMemsetAsync(X, 0, sizeof(double) * nt, st);
    cudaMemsetAsync(s->iters, 0, sizeof(int) * nm, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("multi-mesh solve", 0);
    int outer = 0;
    for (;;) {
        // the accurate residual P (B - A X) of the meshes not yet converged
        if (outer > 0) {
            for (int q = 0; q < nm; q++) act[q] = conv[q] ? 0 : 1;
            cudaMemcpyAsync(s->active, act.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, st);
            s->op16 = 0;
            if ((e = mm_apply(s, X, s->W, s->active, st))) return e;
            cudaMemcpyAsync(s->Bz, s->Bfull, sizeof(double) * nt, cudaMemcpyDeviceToDevice, st);
            mm_axpby_kernel<<<blocks(nt), 256, 0, st>>>(s->Bz, s->W, -1.0, 1.0, s->chunk_mesh, s->active, nt);
            if ((e = mm_project(s, s->Bz, s->active, st))) return e;
            if ((e = mm_dots(s, s->Bz, 1, s->Bz, s->active, 0, s->rn2, 1, st))) return e;
            cudaMemcpyAsync(rn2.data(), s->rn2, sizeof(double) * nm, cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("multi-mesh solve", 0);
        } else {
            rn2 = bn2;
        }
        bool any = false;
        for (int q = 0; q < nm; q++) {
            if (conv[q]) continue;
            relres[q] = bn2[q] > 0.0 ? sqrt(rn2[q] / bn2[q]) : 0.0;
            if (bn2[q] == 0.0 || relres[q] < rtol) conv[q] = 1;
            else any = true;
        }
        if (!any || outer >= max_outer) break;
        // the correction: the BF16 operator's GMRES for the residual (in s->Bz)
        std::vector<int> iconv = conv;
        std::vector<double> irel(nm, 0.0);
        int icycles = 0;
        s->op16 = 1;
        e = mm_gmres(s, s->D, inner_rtol, max_cycles, use_graph, iconv, irel, icycles, st);
        s->op16 = 0;
        if (e) return e;
        for (int q = 0; q < nm; q++) act[q] = conv[q] ? 0 : 1;
        cudaMemcpyAsync(s->active, act.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, st);
        mm_axpby_kernel<<<blocks(nt), 256, 0, st>>>(X, s->D, 1.0, 1.0, s->chunk_mesh, s->active, nt);
        if ((e = launch_status("mm_refine", 1))) return e;
        outer++;
    }
    return mm_finish(s, X, conv, relres, outer, rep, st);
}

}  // extern "C"
