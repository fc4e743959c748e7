// Host-side pieces of the C ABI: error state, version, level-table setup.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "common.cuh"

namespace gbsdf {

static thread_local char g_err[512] = {0};

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

void clear_error() { g_err[0] = 0; }

int launch_status(const char* what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: %s", what, cudaGetErrorString(e));
        return GBSDF_ERR_CUDA;
    }
    return GBSDF_OK;
}

}  // namespace gbsdf

using namespace gbsdf;

extern "C" int gbsdf_version(void) { return 100; }

extern "C" const char* gbsdf_last_error(void) { return g_err; }

extern "C" int gbsdf_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// Level table following tiny-cuda-nn's grid setup (the encoder configured at
// projects/neuralangelo/utils/modules.py:42-50):
//   scale_l = 2^(l * log2(per_level_scale)) * base_resolution - 1   (float32)
//   resolution_l = ceil(scale_l) + 1
//   size_l = min(roundup8(resolution_l^3), 2^log2_hashmap_size); hashed iff resolution_l^3 > size_l
// log2 and exp2 are evaluated in double and rounded to float32 once, so the
// host-side table is reproducible across compilers and libm versions.
extern "C" int gbsdf_grid_init(gbsdf_grid* g, int n_levels, int n_features, int log2_hashmap_size,
                               int base_resolution, float per_level_scale) {
    clear_error();
    GBSDF_CHECK_ARG(g != nullptr, "grid is NULL");
    GBSDF_CHECK_ARG(n_levels >= 1 && n_levels <= GBSDF_MAX_LEVELS, "n_levels %d not in [1, %d]", n_levels,
                    GBSDF_MAX_LEVELS);
    GBSDF_CHECK_ARG(n_features == 1 || n_features == 2 || n_features == 4 || n_features == 8,
                    "n_features %d not in {1, 2, 4, 8}", n_features);
    GBSDF_CHECK_ARG(log2_hashmap_size >= 3 && log2_hashmap_size <= 30, "log2_hashmap_size %d not in [3, 30]",
                    log2_hashmap_size);
    GBSDF_CHECK_ARG(base_resolution >= 1, "base_resolution must be >= 1");
    GBSDF_CHECK_ARG(per_level_scale >= 1.0f && std::isfinite(per_level_scale), "per_level_scale must be >= 1");
    std::memset(g, 0, sizeof(*g));
    g->n_levels = n_levels;
    g->n_features = n_features;
    g->log2_hashmap_size = log2_hashmap_size;
    g->base_resolution = base_resolution;
    g->per_level_scale = per_level_scale;
    const float log2_pls = (float)std::log2((double)per_level_scale);
    const uint64_t hashmap = 1ull << log2_hashmap_size;
    uint64_t off = 0;
    for (int l = 0; l < n_levels; ++l) {
        const float e = (float)l * log2_pls;
        const float s = (float)std::exp2((double)e) * (float)base_resolution - 1.0f;
        const uint64_t res = (uint64_t)std::ceil((double)s) + 1;
        const uint64_t dense = res * res * res;
        uint64_t size = (dense + 7) / 8 * 8;
        if (size > hashmap) size = hashmap;
        g->scale[l] = s;
        g->resolution[l] = (uint32_t)res;
        g->size[l] = (uint32_t)size;
        g->hashed[l] = dense > size ? 1u : 0u;
        g->offset[l] = off;
        off += size;
    }
    g->offset[n_levels] = off;
    return GBSDF_OK;
}
