// Multi-RHS product Y = A X on the 5th-generation tensor cores (sm_103a):
// BF16 operands staged by TMA into 128-byte-swizzled shared memory,
// tcgen05.mma (kind::f16, FP32 accumulation) into tensor memory, read back
// with tcgen05.ld. It serves the many-right-hand-side solves, where the
// matvec of FGMRES becomes a true GEMM (N x N times N x n_rhs).
//
// Layout: A (M x K) row-major BF16 (K-major), X given transposed as
// Xt (NR x K) row-major BF16 (K-major too), Y (M x NR) row-major FP32.
// One CTA owns a 128-row block of Y and all NR <= 256 columns, so it reads
// its rows of A once; Xt (a few MB) is shared through L2.
//
// Warp roles (6 warps): warps 0-3 read the accumulator (warp w owns TMEM
// lanes 32w..32w+31 = rows 32w..), warp 4 issues the TMA loads, warp 5
// allocates TMEM and issues the MMAs. A 4-stage ring of (A, B) tiles with
// full/empty mbarriers; tcgen05.commit releases a stage when its MMAs have
// read it. Every wait is bounded: on a timeout the kernel records an error
// and carries on without waiting, so it always ends.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "common.cuh"
#include "tune.cuh"
#include "tma_pipe.cuh"

namespace mbem {

constexpr int TC_BM = 128;            // rows per CTA (the MMA's M)
constexpr int TC_BK = 64;             // K per stage: one 128-byte swizzle row of BF16
constexpr int TC_STAGES = 4;
constexpr int TC_THREADS = 192;
constexpr uint32_t TC_WAIT_LIMIT = 1u << 24;

__device__ int g_tc_error;

// tcgen05 shared-memory matrix descriptor, K-major operand with 128-byte
// swizzle: start address, leading-dimension offset (unused for this layout),
// stride between 8-row groups (1024 bytes), descriptor version 1, swizzle
// mode 2 (128B).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(16u >> 4) << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t f16_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cta.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_addr(dst)),
        "l"(map), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// SUB: Y[M x N] -= A B^T over 128 x BN tiles (a grid of row tiles x column
// tiles, visited in row-tile groups; n_cols = N, the whole of K in each CTA); else Y (or its slice of the K
// split blockIdx.y) = A B^T for n_cols <= BN columns.
// ring stages: the update (short K, two CTAs an SM) keeps two
template <bool SUB>
constexpr int tc_stages() { return SUB ? 2 : TC_STAGES; }
// row tiles in one raster group of the update (16 x 128 rows of A with the
// column tiles of 304 resident CTAs: about 20 MB of operands at K = 1,536)
constexpr int TC_GROUP_M = 16;

template <int BN, bool TRANS, bool SUB = false>
__global__ void __launch_bounds__(TC_THREADS, SUB ? 2 : 1)
tc_gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int64_t M,
               int64_t K, float* __restrict__ Y, int64_t ldy, int n_cols, int kb_per, int64_t split_stride) {
    static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256, "MMA N for M = 128");
    constexpr int NS = tc_stages<SUB>();
    constexpr int A_BYTES = TC_BM * TC_BK * 2;
    constexpr int B_BYTES = BN * TC_BK * 2;
    constexpr int STAGE = A_BYTES + B_BYTES;
    constexpr uint32_t TMEM_COLS = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
    extern __shared__ __align__(1024) uint8_t tc_smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)tc_smem_raw + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t full[NS], empty[NS], accum;
    __shared__ uint32_t tmem_base;


    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // SUB: the (row tile, column tile) of this CTA in groups of
    // TC_GROUP_M row tiles, column-major within a group, so the CTAs
    // resident at one time share a few operand row panels in L2 instead of
    // each column tile streaming all of A
    int64_t mt = blockIdx.x, nt = blockIdx.y;
    if (SUB) {
        const int64_t lin = (int64_t)blockIdx.y * gridDim.x + blockIdx.x;
        const int64_t per_group = (int64_t)TC_GROUP_M * gridDim.y;
        const int64_t first = lin / per_group * TC_GROUP_M;
        const int64_t gsize = min((int64_t)TC_GROUP_M, (int64_t)gridDim.x - first);
        const int64_t local = lin % per_group;
        mt = first + local % gsize;
        nt = local / gsize;
    }
    const int64_t m0 = mt * TC_BM;
    // this CTA's share of K (a split of K over blockIdx.y; its partial sum
    // goes to slice blockIdx.y of Y)
    const int kb_all = (int)((K + TC_BK - 1) / TC_BK);
    const int kb_first = SUB ? 0 : (int)blockIdx.y * kb_per;
    const int kb_total = SUB ? kb_all : min(kb_per, kb_all - kb_first);
    const int n0 = SUB ? (int)nt * BN : 0;
    if (SUB) {
        Y += n0;
        n_cols = min(BN, n_cols - n0);
    } else {
        Y += (int64_t)blockIdx.y * split_stride;
    }

    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&accum, 1);
        mbar_init_fence();
    }
    if (warp == 5) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;

    if (warp == 4 && lane == 0) {
        // producer
        for (int kb = 0; kb < kb_total; kb++) {
            const int s = kb % NS;
            const uint32_t ph = (uint32_t)(kb / NS) & 1u;
            if (!mbar_wait(&empty[s], ph ^ 1u, TC_WAIT_LIMIT)) atomicExch(&g_tc_error, 1);
            uint8_t* st = smem + s * STAGE;
            mbar_arrive_expect_tx(&full[s], STAGE);
            tma_load_2d(st, &mapA, (kb_first + kb) * TC_BK, (int)m0, &full[s]);
            tma_load_2d(st + A_BYTES, &mapB, (kb_first + kb) * TC_BK, n0, &full[s]);
        }
        // the last copies have landed before the CTA can end
        for (int kb = (kb_total > NS ? kb_total - NS : 0); kb < kb_total; kb++)
            if (!mbar_wait(&full[kb % NS], (uint32_t)(kb / NS) & 1u, TC_WAIT_LIMIT))
                atomicExch(&g_tc_error, 1);
    } else if (warp == 5 && lane == 0) {
        // MMA issuer
        constexpr uint32_t idesc = f16_idesc(TC_BM, BN);
        for (int kb = 0; kb < kb_total; kb++) {
            const int s = kb % NS;
            const uint32_t ph = (uint32_t)(kb / NS) & 1u;
            if (!mbar_wait(&full[s], ph, TC_WAIT_LIMIT)) atomicExch(&g_tc_error, 1);
            tc_fence_after();
            const uint32_t a0 = smem_addr(smem + s * STAGE), b0 = a0 + A_BYTES;
#pragma unroll
            for (int k = 0; k < TC_BK / 16; k++) {
                const uint64_t ad = sw128_desc(a0 + k * 32), bd = sw128_desc(b0 + k * 32);
                const uint32_t acc = (kb > 0 || k > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_addr(&empty[s]))
                         : "memory");
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_addr(&accum))
                     : "memory");
    } else if (warp < 4) {
        // epilogue: row m0 + 32 warp + lane, BN columns from TMEM
        if (SUB) {
            // while the MMAs run: this warp's 32 rows of the Y tile into L2
            const int64_t prow = m0 + 32 * warp + lane;
            if (prow < M) {
                const char* p0 = reinterpret_cast<const char*>(Y + prow * ldy);
                for (int off = 0; off < n_cols * 4; off += 128)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(p0 + off));
            }
        }
        if (!mbar_wait(&accum, 0u, TC_WAIT_LIMIT)) atomicExch(&g_tc_error, 1);
        tc_fence_after();
        if (SUB) {
            // 32 columns at a time: TMEM -> registers -> this warp's block in
            // shared memory -> Y, one row per pass with the lanes along it.
            // Every MMA has completed (accum), so no copy or MMA still reads
            // the ring.
            const int64_t rbase = m0 + 32 * warp;
            constexpr int CW = BN >= 64 ? 64 : 32;      // columns a pass
            constexpr int LDE = CW + 1;
            float* epi = reinterpret_cast<float*>(smem) + warp * 32 * LDE;
#pragma unroll 1
            for (int c = 0; c < BN; c += CW) {
#pragma unroll
                for (int h = 0; h < CW; h += 16) {
                    uint32_t v[16];
                    const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(c + h);
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                        "%12, %13, %14, %15}, [%16];"
                        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                          "=r"(v[14]), "=r"(v[15])
                        : "r"(ta));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                    for (int q = 0; q < 16; q++) epi[lane * LDE + h + q] = __uint_as_float(v[q]);
                }
                __syncwarp();
                // the warp's 32 rows x CW columns: CW / 32 columns a lane, all
                // loads in flight before the first subtraction
                constexpr int PER = CW / 32;
                float yv[32 * PER];
#pragma unroll
                for (int r = 0; r < 32; r++)
#pragma unroll
                    for (int t = 0; t < PER; t++) {
                        const int col = c + 32 * t + lane;
                        yv[r * PER + t] = (rbase + r < M && col < n_cols) ? Y[(rbase + r) * ldy + col] : 0.0f;
                    }
#pragma unroll
                for (int r = 0; r < 32; r++)
#pragma unroll
                    for (int t = 0; t < PER; t++) {
                        const int col = c + 32 * t + lane;
                        if (rbase + r < M && col < n_cols)
                            Y[(rbase + r) * ldy + col] = yv[r * PER + t] - epi[r * LDE + 32 * t + lane];
                    }
                __syncwarp();
            }
        } else {
        const int64_t row = m0 + 32 * warp + lane;
        float* yr = TRANS ? Y + row : Y + row * ldy;   // Y^T: element (row, c) at c ldy + row
#pragma unroll 1
        for (int c = 0; c < BN; c += 16) {
            uint32_t v[16];
            const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(ta));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < M) {
#pragma unroll
                for (int j = 0; j < 16; j++)
                    if (c + j < n_cols) yr[TRANS ? (int64_t)(c + j) * ldy : (c + j)] = __uint_as_float(v[j]);
            }
        }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 5) {
        // every MMA has completed (the epilogue waited for the final commit)
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// ---------------------------------------------------------------------------
// host: tensor maps through the driver entry point (no libcuda link)
// ---------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::mutex g_encode_mutex;

static int get_encode() {
    std::lock_guard<std::mutex> lock(g_encode_mutex);
    if (g_encode) return MBEM_OK;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &fn, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || fn == nullptr)
        return set_error(MBEM_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    return MBEM_OK;
}

// BF16 row-major (rows x cols) at ld elements, box (64 cols x box_rows), 128B swizzle
static int make_map(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int64_t ld, int box_rows) {
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
    const cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(MBEM_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return MBEM_OK;
}

template <int BN, bool TRANS>
static int launch_tc(const CUtensorMap& ma, const CUtensorMap& mb, int64_t M, int64_t K, float* Y, int64_t ldy,
                     int n_cols, int splits, int kb_per, int64_t split_stride, cudaStream_t st) {
    const size_t smem = (size_t)TC_STAGES * (TC_BM * TC_BK * 2 + BN * TC_BK * 2) + 1024;
    cudaFuncSetAttribute(tc_gemm_kernel<BN, TRANS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const dim3 grid((unsigned)ceil_div(M, TC_BM), (unsigned)splits);
    tc_gemm_kernel<BN, TRANS><<<grid, TC_THREADS, smem, st>>>(ma, mb, M, K, Y, ldy, n_cols, kb_per, split_stride);
    return launch_status("tc_gemm_kernel");
}

template <bool TRANS>
static int launch_bn(int bn, const CUtensorMap& ma, const CUtensorMap& mb, int64_t M, int64_t K, float* Y,
                     int64_t ldy, int n_rhs, int splits, int kb_per, int64_t split_stride, cudaStream_t st) {
    switch (bn) {
        case 16: return launch_tc<16, TRANS>(ma, mb, M, K, Y, ldy, n_rhs, splits, kb_per, split_stride, st);
        case 32: return launch_tc<32, TRANS>(ma, mb, M, K, Y, ldy, n_rhs, splits, kb_per, split_stride, st);
        case 64: return launch_tc<64, TRANS>(ma, mb, M, K, Y, ldy, n_rhs, splits, kb_per, split_stride, st);
        case 128: return launch_tc<128, TRANS>(ma, mb, M, K, Y, ldy, n_rhs, splits, kb_per, split_stride, st);
        case 256: return launch_tc<256, TRANS>(ma, mb, M, K, Y, ldy, n_rhs, splits, kb_per, split_stride, st);
        default: break;
    }
    return set_error(MBEM_ERR_UNSUPPORTED, "no GEMM tile for %d right-hand sides", bn);
}

// Y[i] = sum_s P[s][i] over the K splits, in split order
__global__ void split_sum_kernel(const float* __restrict__ P, int splits, int64_t stride, int64_t rows,
                                 int64_t cols, float* __restrict__ Y, int64_t ldy) {
    const int64_t r = blockIdx.y;
    const int64_t c = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (c >= cols) return;
    float acc = 0.0f;
    for (int s = 0; s < splits; s++) acc += P[s * stride + r * cols + c];
    Y[r * ldy + c] = acc;
}

// K splits that fill the SMs evenly: the smallest count of waves per unit of
// work over 1..8 splits, each split keeping at least 8 K blocks
static int choose_splits(int64_t tiles, int kb_all, int sms) {
    int best = 1;
    double best_cost = 1e30;
    for (int s = 1; s <= 8; s++) {
        if (kb_all / s < 8 && s > 1) break;
        const double waves = (double)ceil_div(tiles * s, sms);
        const double cost = waves / s + 0.02 * (s - 1);     // the partial sums' traffic
        if (cost < best_cost - 1e-12) {
            best_cost = cost;
            best = s;
        }
    }
    return best;
}

int tc_gemm_check(cudaStream_t st) {
    int err = 0;
    cudaMemcpyFromSymbolAsync(&err, g_tc_error, sizeof(int), 0, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return launch_status("tc_gemm sync", 0);
    if (err) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int));
        return set_error(MBEM_ERR_WAIT, "a tensor-core GEMM pipeline wait ran out");
    }
    return MBEM_OK;
}

static int gemm_bf16(const void* A, int64_t lda, const void* Xt, int64_t ldx, int64_t M, int64_t K, int n_rhs,
                     float* Y, int64_t ldy, bool trans, float* work, size_t work_bytes, cudaStream_t st) {
    MBEM_REQUIRE(M >= 0 && K >= 1 && n_rhs >= 1 && n_rhs <= 256, MBEM_ERR_ARG,
                 "bad GEMM sizes (M=%lld, K=%lld, n_rhs=%d; n_rhs <= 256)", (long long)M, (long long)K, n_rhs);
    MBEM_REQUIRE(A && Xt && Y && lda >= K && ldx >= K && ldy >= (trans ? M : n_rhs), MBEM_ERR_ARG,
                 "bad GEMM pointers/strides");
    MBEM_REQUIRE(lda % 8 == 0 && ldx % 8 == 0 && (uintptr_t)A % 16 == 0 && (uintptr_t)Xt % 16 == 0, MBEM_ERR_ARG,
                 "TMA needs 16-byte aligned bases and row strides (lda, ldx multiples of 8)");
    if (M == 0) return MBEM_OK;
    int e = get_encode();
    if (e) return e;
    const int bn = n_rhs <= 16 ? 16 : (n_rhs <= 32 ? 32 : (n_rhs <= 64 ? 64 : (n_rhs <= 128 ? 128 : 256)));
    CUtensorMap ma, mb;
    if ((e = make_map(&ma, A, M, K, lda, TC_BM))) return e;
    if ((e = make_map(&mb, Xt, n_rhs, K, ldx, bn))) return e;
    const int kb_all = (int)ceil_div(K, TC_BK);
    int sms = 152;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int splits = 1;
    const int64_t rows_out = trans ? n_rhs : M, cols_out = trans ? M : n_rhs;
    const int64_t slice = rows_out * cols_out;
    if (work != nullptr) {
        const int forced = kGemmSplits[tune_get(MBEM_TUNE_GEMM_SPLIT)];
        splits = forced > 0 ? (int)lmin(forced, kb_all) : choose_splits(ceil_div(M, TC_BM), kb_all, sms);
        while (splits > 1 && work_bytes < (size_t)splits * slice * sizeof(float)) splits--;
    }
    const int kb_per = (int)ceil_div(kb_all, splits);
    splits = (int)ceil_div(kb_all, kb_per);                // every split non-empty
    if (splits == 1)
        return trans ? launch_bn<true>(bn, ma, mb, M, K, Y, ldy, n_rhs, 1, kb_per, 0, st)
                     : launch_bn<false>(bn, ma, mb, M, K, Y, ldy, n_rhs, 1, kb_per, 0, st);
    // partial sums in the workspace (dense, leading dimension = cols_out), then their sum
    e = trans ? launch_bn<true>(bn, ma, mb, M, K, work, cols_out, n_rhs, splits, kb_per, slice, st)
              : launch_bn<false>(bn, ma, mb, M, K, work, cols_out, n_rhs, splits, kb_per, slice, st);
    if (e) return e;
    split_sum_kernel<<<dim3((unsigned)ceil_div(cols_out, 256), (unsigned)rows_out), 256, 0, st>>>(
        work, splits, slice, rows_out, cols_out, Y, ldy);
    return launch_status("split_sum_kernel");
}

size_t tc_gemm_workspace_size(int64_t M, int n_rhs) { return (size_t)8 * M * n_rhs * sizeof(float); }

// C[M x N] -= A[M x K] B[N x K]^T (BF16 operands, FP32 C at ldc): column
// tiles of 256 (fewer for a narrow N) over grid.y
int gemm_bf16_sub(const void* A, int64_t lda, const void* Bt, int64_t ldb, int64_t M, int64_t N, int64_t K, float* C,
                  int64_t ldc, cudaStream_t st) {
    MBEM_REQUIRE(M >= 0 && N >= 0 && K >= 1 && A && Bt && C && lda >= K && ldb >= K && ldc >= N, MBEM_ERR_ARG,
                 "bad GEMM-update arguments");
    MBEM_REQUIRE(lda % 8 == 0 && ldb % 8 == 0 && (uintptr_t)A % 16 == 0 && (uintptr_t)Bt % 16 == 0, MBEM_ERR_ARG,
                 "TMA needs 16-byte aligned bases and row strides (lda, ldb multiples of 8)");
    MBEM_REQUIRE(N <= (int64_t)65535 * 256 && M <= (int64_t)0x7fffffff, MBEM_ERR_ARG, "GEMM update too large");
    if (M == 0 || N == 0) return MBEM_OK;
    int e = get_encode();
    if (e) return e;
    const int bn = N >= 256 ? 256 : (N > 128 ? 256 : (N > 64 ? 128 : (N > 32 ? 64 : (N > 16 ? 32 : 16))));
    CUtensorMap ma, mb;
    if ((e = make_map(&ma, A, M, K, lda, TC_BM))) return e;
    if ((e = make_map(&mb, Bt, N, K, ldb, bn))) return e;
    const dim3 grid((unsigned)ceil_div(M, TC_BM), (unsigned)ceil_div(N, bn));
#define MBEM_SUB_LAUNCH(B)                                                                                    \
    {                                                                                                         \
        const size_t smem = (size_t)tc_stages<true>() * (TC_BM * TC_BK * 2 + B * TC_BK * 2) + 1024;          \
        cudaFuncSetAttribute(tc_gemm_kernel<B, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        tc_gemm_kernel<B, false, true><<<grid, TC_THREADS, smem, st>>>(ma, mb, M, K, C, ldc, (int)N, 0, 0); \
    }
    switch (bn) {
        case 16: MBEM_SUB_LAUNCH(16) break;
        case 32: MBEM_SUB_LAUNCH(32) break;
        case 64: MBEM_SUB_LAUNCH(64) break;
        case 128: MBEM_SUB_LAUNCH(128) break;
        default: MBEM_SUB_LAUNCH(256) break;
    }
#undef MBEM_SUB_LAUNCH
    return launch_status("tc_gemm_kernel<sub>");
}

}  // namespace mbem

using namespace mbem;

extern "C" int mbem_gemm_bf16(const void* A, int64_t lda, const void* Xt, int64_t ldx, int64_t M, int64_t K,
                              int n_rhs, float* Y, int64_t ldy, void* stream) {
    return gemm_bf16(A, lda, Xt, ldx, M, K, n_rhs, Y, ldy, false, nullptr, 0, (cudaStream_t)stream);
}

extern "C" int mbem_gemm_bf16_t(const void* A, int64_t lda, const void* Xt, int64_t ldx, int64_t M, int64_t K,
                                int n_rhs, float* Yt, int64_t ldy, void* stream) {
    return gemm_bf16(A, lda, Xt, ldx, M, K, n_rhs, Yt, ldy, true, nullptr, 0, (cudaStream_t)stream);
}

extern "C" size_t mbem_gemm_bf16_workspace_size(int64_t M, int n_rhs) { return tc_gemm_workspace_size(M, n_rhs); }

extern "C" int mbem_gemm_bf16_t_split(const void* A, int64_t lda, const void* Xt, int64_t ldx, int64_t M, int64_t K,
                                      int n_rhs, float* Yt, int64_t ldy, void* work, size_t work_bytes,
                                      void* stream) {
    return gemm_bf16(A, lda, Xt, ldx, M, K, n_rhs, Yt, ldy, true, static_cast<float*>(work), work_bytes,
                     (cudaStream_t)stream);
}

extern "C" int mbem_gemm_bf16_check(void* stream) { return tc_gemm_check((cudaStream_t)stream); }

extern "C" int mbem_gemm_bf16_sub(const void* A, int64_t lda, const void* Bt, int64_t ldb, int64_t M, int64_t N,
                                  int64_t K, float* C, int64_t ldc, void* stream) {
    return gemm_bf16_sub(A, lda, Bt, ldb, M, N, K, C, ldc, (cudaStream_t)stream);
}
