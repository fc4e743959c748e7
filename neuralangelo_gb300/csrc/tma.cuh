// Host-side TMA tensor maps (cuTensorMapEncodeTiled through the runtime's driver
// entry point, so the library does not link libcuda).
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include "common.cuh"

namespace gbsdf {

inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }
    return fn;
}

// 2D map of a row-major fp16 or fp32 matrix [rows x cols] with a row stride of ld
// elements; boxes of box_cols x box_rows.  The encoder rejects a base that is not
// 16-byte aligned, a stride that is not a multiple of 16 bytes and a box row that
// exceeds the swizzle span.
inline int tensor_map_2d(CUtensorMap* map, bool f32, const void* base, int64_t rows, int64_t cols, int64_t ld,
                         int box_cols, int box_rows, CUtensorMapSwizzle swizzle, CUtensorMapL2promotion l2,
                         const char* what) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return GBSDF_ERR_CUDA;
    }
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * (f32 ? 4 : 2)};
    const cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
    const cuuint32_t es[2] = {1, 1};
    const CUresult r = enc(map, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
                           const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle, l2,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled (%s) failed (%d)", what, (int)r);
        return GBSDF_ERR_CUDA;
    }
    return GBSDF_OK;
}

// 3D map that loads 8-row groups of a row-major fp16 matrix [rows x (8 chunks)] straight into the
// no-swizzle K-major core-matrix layout of the MMA operands: dims (feature within a 16-byte chunk,
// row, chunk) with strides (row pitch, 16 B), so a box {8, 8, box_chunks} lands as box_chunks
// consecutive 128-byte core matrices of 8 rows.  Rows past `rows` and chunks past `chunks` read
// as zeros.  The encoder takes the non-monotonic strides (checked on GB300: bit-exact layout).
inline int tensor_map_kmajor_groups(CUtensorMap* map, const void* base, int64_t rows, int64_t chunks, int64_t ld,
                                    int box_chunks, const char* what) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return GBSDF_ERR_CUDA;
    }
    const cuuint64_t dims[3] = {8, (cuuint64_t)rows, (cuuint64_t)chunks};
    const cuuint64_t strides[2] = {(cuuint64_t)ld * 2, 16};
    const cuuint32_t box[3] = {8, 8, (cuuint32_t)box_chunks};
    const cuuint32_t es[3] = {1, 1, 1};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, const_cast<void*>(base), dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled (%s) failed (%d)", what, (int)r);
        return GBSDF_ERR_CUDA;
    }
    return GBSDF_OK;
}

}  // namespace gbsdf
