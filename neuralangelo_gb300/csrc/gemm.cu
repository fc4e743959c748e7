// Weight-gradient GEMMs (dW = dZ^T X, a reduction over millions of sample rows)
// through cuBLAS: fp16 operands, fp32 accumulation and fp32 output.  These are
// plain library GEMMs with no fusion opportunity beyond the fp16 operands the
// fused kernels already wrote; the handle is created once per device and
// thread and reused.
#include <cublas_v2.h>

#include "common.cuh"

namespace gbsdf {

static cublasHandle_t handle_for_current_device() {
    static thread_local cublasHandle_t handles[64] = {nullptr};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return nullptr;
    if (!handles[dev]) {
        if (cublasCreate(&handles[dev]) != CUBLAS_STATUS_SUCCESS) handles[dev] = nullptr;
    }
    return handles[dev];
}

}  // namespace gbsdf

using namespace gbsdf;

// dW[N, K] (row-major, ldw) = alpha * dZ[M, N]^T X[M, K] + beta * dW
// dZ: fp16 row-major with row stride ldz; X: fp16 row-major with row stride ldx.
extern "C" int gbsdf_gemm_wgrad(int64_t M, int N, int K, const void* dZ, int ldz, const void* X, int ldx, float* dW,
                                int ldw, float alpha, float beta, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(M >= 0 && N > 0 && K > 0, "bad sizes");
    GBSDF_CHECK_ARG(dZ && X && dW, "NULL pointer");
    GBSDF_CHECK_ARG(ldz >= N && ldx >= K && ldw >= K, "leading dimensions");
    GBSDF_CHECK_ARG(M <= INT32_MAX, "M too large for one GEMM");
    cublasHandle_t h = handle_for_current_device();
    if (!h) {
        set_error("cublasCreate failed");
        return GBSDF_ERR_CUDA;
    }
    cublasSetStream(h, as_stream(stream));
    // column-major view: dW^T [K x N] = X^T [K x M] * dZ [M x N]
    //   X row-major [M x K] == column-major [K x M] (lda = ldx), op N
    //   dZ row-major [M x N] == column-major [N x M] (ldb = ldz), op T
    const cublasStatus_t st = cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_T, K, N, (int)M, &alpha, X, CUDA_R_16F, ldx,
                                           dZ, CUDA_R_16F, ldz, &beta, dW, CUDA_R_32F, ldw, CUBLAS_COMPUTE_32F,
                                           CUBLAS_GEMM_DEFAULT);
    if (st != CUBLAS_STATUS_SUCCESS) {
        set_error("cublasGemmEx failed (status %d)", (int)st);
        return GBSDF_ERR_CUDA;
    }
    return launch_status("gemm_wgrad");
}
