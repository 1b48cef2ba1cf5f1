// Process-wide tile choices of the tunable kernel families.
#include <stdio.h>

#include <atomic>

#include "tune.cuh"

namespace mbem {

static std::atomic<int> g_tune[MBEM_TUNE_FAMILIES] = {};

static int family_count(int family) {
    switch (family) {
        case MBEM_TUNE_MIXED_MATVEC: return count_of(kDfTiles);
        case MBEM_TUNE_BF16_MATVEC: return count_of(kBf16Tiles);
        case MBEM_TUNE_MM_MATVEC: return count_of(kMmTiles);
        case MBEM_TUNE_GEMM_SPLIT: return count_of(kGemmSplits);
        default: return 0;
    }
}

int tune_get(int family) {
    if (family < 0 || family >= MBEM_TUNE_FAMILIES) return 0;
    return g_tune[family].load(std::memory_order_relaxed);
}

}  // namespace mbem

using namespace mbem;

extern "C" {

int mbem_tune_count(int family) { return family_count(family); }

int mbem_tune_get(int family) { return tune_get(family); }

int mbem_tune_set(int family, int config) {
    const int n = family_count(family);
    MBEM_REQUIRE(n > 0, MBEM_ERR_ARG, "unknown tunable kernel family %d", family);
    MBEM_REQUIRE(config >= 0 && config < n, MBEM_ERR_ARG, "family %d has configurations 0..%d (got %d)", family,
                 n - 1, config);
    g_tune[family].store(config, std::memory_order_relaxed);
    return MBEM_OK;
}

int mbem_tune_describe(int family, int config, char* buf, int len) {
    const int n = family_count(family);
    MBEM_REQUIRE(n > 0 && config >= 0 && config < n, MBEM_ERR_ARG, "bad family/configuration %d/%d", family,
                 config);
    MBEM_REQUIRE(buf != nullptr && len > 0, MBEM_ERR_ARG, "no buffer");
    if (family == MBEM_TUNE_GEMM_SPLIT) {
        if (kGemmSplits[config] == 0) snprintf(buf, (size_t)len, "splits=model");
        else snprintf(buf, (size_t)len, "splits=%d", kGemmSplits[config]);
        return MBEM_OK;
    }
    const TileCfg c = family == MBEM_TUNE_MIXED_MATVEC ? kDfTiles[config]
                      : family == MBEM_TUNE_BF16_MATVEC ? kBf16Tiles[config] : kMmTiles[config];
    snprintf(buf, (size_t)len, "rows=%d ch=%d stages=%d", c.rows, c.ch, c.stages);
    return MBEM_OK;
}

}  // extern "C"
