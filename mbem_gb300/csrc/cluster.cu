// Principal-axis bisection of a point cloud, one tree level per call pair
// (la/cluster.py:56-75 rule, as the block-Jacobi chunks use it): for every
// segment (a run of `order`) with more than max_nodes points,
//   mbem_cluster_stats:  the segment's mean and the 3 x 3 sums of (p - mean)
//                        (p - mean)^T, for the host's symmetric eigensolver;
//   mbem_cluster_split:  projections on the leading principal axis, the median
//                        (the mean of the two middle order statistics, found
//                        exactly by a radix select on the 64-bit keys), and a
//                        stable partition: proj < median to the left, in the
//                        current order, then the rest.
// One CTA a segment; every sum runs in a fixed order. A segment whose split
// would leave one side empty (coincident projections) is left in place and
// reported, for the host's rank rule.
#include "common.cuh"

namespace mbem {

constexpr int CL_THREADS = 256;

__device__ double cl_block_sum(double v, double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < CL_THREADS / 32; w++) s += red[w];
    return s;
}

// stats[s] = (count, sum (p - mean)(p - mean)^T as xx, xy, xz, yx, yy, yz, zx, zy, zz); mean[s] (3)
__global__ void __launch_bounds__(CL_THREADS)
cluster_stats_kernel(const double* __restrict__ pts, const int64_t* __restrict__ order,
                     const int64_t* __restrict__ seg_start, const int64_t* __restrict__ seg_size, int max_nodes,
                     double* __restrict__ mean, double* __restrict__ stats) {
    __shared__ double red[CL_THREADS / 32];
    const int s = blockIdx.x;
    const int64_t a = seg_start[s], m = seg_size[s];
    if (m <= max_nodes) {
        if (threadIdx.x < 10) stats[10 * s + threadIdx.x] = threadIdx.x == 0 ? (double)m : 0.0;
        return;
    }
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int64_t t = threadIdx.x; t < m; t += CL_THREADS) {
        const double* p = pts + 3 * order[a + t];
        sx += p[0];
        sy += p[1];
        sz += p[2];
    }
    const double mx = cl_block_sum(sx, red) / (double)m;
    const double my = cl_block_sum(sy, red) / (double)m;
    const double mz = cl_block_sum(sz, red) / (double)m;
    double c[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int64_t t = threadIdx.x; t < m; t += CL_THREADS) {
        const double* p = pts + 3 * order[a + t];
        const double x = p[0] - mx, y = p[1] - my, z = p[2] - mz;
        c[0] += x * x;
        c[1] += x * y;
        c[2] += x * z;
        c[3] += y * y;
        c[4] += y * z;
        c[5] += z * z;
    }
    double cs[6];
    for (int q = 0; q < 6; q++) cs[q] = cl_block_sum(c[q], red);
    if (threadIdx.x == 0) {
        mean[3 * s] = mx;
        mean[3 * s + 1] = my;
        mean[3 * s + 2] = mz;
        double* o = stats + 10 * s;
        o[0] = (double)m;
        o[1] = cs[0]; o[2] = cs[1]; o[3] = cs[2];
        o[4] = cs[1]; o[5] = cs[3]; o[6] = cs[4];
        o[7] = cs[2]; o[8] = cs[4]; o[9] = cs[5];
    }
}

// order-preserving 64-bit key of a double
__device__ __forceinline__ uint64_t cl_key(double v) {
    const uint64_t u = (uint64_t)__double_as_longlong(v);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

__device__ __forceinline__ double cl_unkey(uint64_t k) {
    const uint64_t u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)u);
}

// the k-th smallest (0-based) of the m keys at proj[0..m): eight passes of
// eight bits each, a 256-bin histogram of the keys that share the prefix so far
__device__ uint64_t cl_select(const double* __restrict__ proj, int64_t m, int64_t k, unsigned int* hist,
                              uint64_t* sh_prefix, int64_t* sh_k) {
    uint64_t prefix = 0;
    for (int pass = 0; pass < 8; pass++) {
        const int shift = 56 - 8 * pass;
        const uint64_t mask_hi = pass == 0 ? 0ull : (~0ull << (shift + 8));
        for (int b = threadIdx.x; b < 256; b += CL_THREADS) hist[b] = 0u;
        __syncthreads();
        for (int64_t t = threadIdx.x; t < m; t += CL_THREADS) {
            const uint64_t key = cl_key(proj[t]);
            if ((key & mask_hi) == prefix) atomicAdd(&hist[(key >> shift) & 0xffu], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int64_t kk = k;
            int b = 0;
            for (; b < 255; b++) {
                if (kk < (int64_t)hist[b]) break;
                kk -= hist[b];
            }
            *sh_prefix = prefix | ((uint64_t)b << shift);
            *sh_k = kk;
        }
        __syncthreads();
        prefix = *sh_prefix;
        k = *sh_k;
        __syncthreads();
    }
    return prefix;
}

// the split of every big segment; nl[s] = its left count, -1 when one side
// would be empty (the segment is then copied unchanged), the size for a leaf
__global__ void __launch_bounds__(CL_THREADS)
cluster_split_kernel(const double* __restrict__ pts, const int64_t* __restrict__ order, int64_t* __restrict__ order_out,
                     const int64_t* __restrict__ seg_start, const int64_t* __restrict__ seg_size, int max_nodes,
                     const double* __restrict__ mean, const double* __restrict__ axis, double* __restrict__ proj,
                     int64_t* __restrict__ nl_out) {
    __shared__ unsigned int hist[256];
    __shared__ uint64_t sh_prefix;
    __shared__ int64_t sh_k;
    __shared__ int64_t wsum[CL_THREADS / 32];
    __shared__ double red[CL_THREADS / 32];
    __shared__ int64_t base_l, base_r;
    const int s = blockIdx.x;
    const int64_t a = seg_start[s], m = seg_size[s];
    if (m <= max_nodes) {
        for (int64_t t = threadIdx.x; t < m; t += CL_THREADS) order_out[a + t] = order[a + t];
        if (threadIdx.x == 0) nl_out[s] = m;
        return;
    }
    const double mx = mean[3 * s], my = mean[3 * s + 1], mz = mean[3 * s + 2];
    const double ax = axis[3 * s], ay = axis[3 * s + 1], az = axis[3 * s + 2];
    double* pr = proj + a;
    for (int64_t t = threadIdx.x; t < m; t += CL_THREADS) {
        const double* p = pts + 3 * order[a + t];
        pr[t] = __dadd_rn(__dadd_rn(__dmul_rn(p[0] - mx, ax), __dmul_rn(p[1] - my, ay)), __dmul_rn(p[2] - mz, az));
    }
    __syncthreads();
    const double v1 = cl_unkey(cl_select(pr, m, (m - 1) / 2, hist, &sh_prefix, &sh_k));
    const double v2 = cl_unkey(cl_select(pr, m, m / 2, hist, &sh_prefix, &sh_k));
    const double median = 0.5 * (v1 + v2);
    double cnt = 0.0;
    for (int64_t t = threadIdx.x; t < m; t += CL_THREADS) cnt += pr[t] < median ? 1.0 : 0.0;
    const int64_t nl = (int64_t)cl_block_sum(cnt, red);
    if (nl == 0 || nl == m) {
        for (int64_t t = threadIdx.x; t < m; t += CL_THREADS) order_out[a + t] = order[a + t];
        if (threadIdx.x == 0) nl_out[s] = -1;
        return;
    }
    // stable partition, CL_THREADS members at a time
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        base_l = 0;
        base_r = nl;
    }
    __syncthreads();
    for (int64_t t0 = 0; t0 < m; t0 += CL_THREADS) {
        const int64_t t = t0 + threadIdx.x;
        const bool valid = t < m;
        const bool left = valid && pr[t] < median;
        const unsigned bl = __ballot_sync(0xffffffffu, left);
        if (lane == 0) wsum[wid] = __popc(bl);
        __syncthreads();
        int64_t before_l = 0, tot_l = 0;
        for (int w = 0; w < CL_THREADS / 32; w++) {
            if (w < wid) before_l += wsum[w];
            tot_l += wsum[w];
        }
        const unsigned lt = (1u << lane) - 1u;
        const int64_t my_l = before_l + __popc(bl & lt);
        // the members before this one in the group are threadIdx.x; the
        // right ones among them follow
        const int64_t my_r = (int64_t)threadIdx.x - my_l;
        if (valid) {
            const int64_t dst = left ? base_l + my_l : base_r + my_r;
            order_out[a + dst] = order[a + t];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const int64_t in_group = lmin(CL_THREADS, m - t0);
            base_l += tot_l;
            base_r += in_group - tot_l;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) nl_out[s] = nl;
}

}  // namespace mbem

using namespace mbem;

extern "C" {

int mbem_cluster_stats(const double* pts, const int64_t* order, const int64_t* seg_start, const int64_t* seg_size,
                       int64_t n_seg, int max_nodes, double* mean, double* stats, void* stream) {
    MBEM_REQUIRE(n_seg >= 0 && n_seg <= 0x7fffffff && max_nodes >= 1, MBEM_ERR_ARG, "bad cluster level");
    if (n_seg == 0) return MBEM_OK;
    MBEM_REQUIRE(pts && order && seg_start && seg_size && mean && stats, MBEM_ERR_ARG, "bad cluster arrays");
    cluster_stats_kernel<<<(unsigned)n_seg, CL_THREADS, 0, (cudaStream_t)stream>>>(pts, order, seg_start, seg_size,
                                                                                  max_nodes, mean, stats);
    return launch_status("cluster_stats_kernel");
}

int mbem_cluster_split(const double* pts, const int64_t* order, int64_t* order_out, const int64_t* seg_start,
                       const int64_t* seg_size, int64_t n_seg, int max_nodes, const double* mean, const double* axis,
                       double* proj, int64_t* nl, void* stream) {
    MBEM_REQUIRE(n_seg >= 0 && n_seg <= 0x7fffffff && max_nodes >= 1, MBEM_ERR_ARG, "bad cluster level");
    if (n_seg == 0) return MBEM_OK;
    MBEM_REQUIRE(pts && order && order_out && order_out != order && seg_start && seg_size && mean && axis && proj &&
                     nl,
                 MBEM_ERR_ARG, "bad cluster arrays");
    cluster_split_kernel<<<(unsigned)n_seg, CL_THREADS, 0, (cudaStream_t)stream>>>(
        pts, order, order_out, seg_start, seg_size, max_nodes, mean, axis, proj, nl);
    return launch_status("cluster_split_kernel");
}

}  // extern "C"
