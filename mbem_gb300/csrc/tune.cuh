// Tile configurations of the streaming kernels: the candidates the
// autotuner times, and the process-wide choice for each kernel family
// (MBEM_TUNE_* in the public header; configuration 0 is the default).
#pragma once

#include "common.cuh"

namespace mbem {

struct TileCfg {
    int rows, ch, stages;   // rows per CTA, columns per ring chunk, ring stages
};

// FP32 double-float matvec (sgemv_df_tma_kernel): shared memory
// stages x (rows + 2) x ch x 4 bytes <= 227 KB; the last one fits two CTAs per SM
constexpr TileCfg kDfTiles[] = {{16, 1024, 3}, {8, 1024, 5}, {32, 512, 3}, {16, 512, 6}, {8, 2048, 2}, {8, 512, 4}};
// BF16 matvec (sgemv_bf16_tma_kernel): stages x (rows x ch x 2 + ch x 4) bytes
constexpr TileCfg kBf16Tiles[] = {{16, 2048, 3}, {16, 1024, 6}, {32, 1024, 3}, {8, 2048, 4}, {32, 512, 6}, {8, 1024, 4}};
// persistent multi-mesh matvec (work items of 16 rows): chunk and stages
constexpr TileCfg kMmTiles[] = {{16, 1024, 3}, {16, 512, 6}, {16, 512, 4}, {16, 256, 8}};
// tensor-core GEMM K split: 0 = the wave cost model, else a fixed count
constexpr int kGemmSplits[] = {0, 1, 2, 4, 8};

template <typename T, int N>
constexpr int count_of(const T (&)[N]) { return N; }

// the configuration in use for a family (0 until set)
int tune_get(int family);

}  // namespace mbem
