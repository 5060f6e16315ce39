// Trailing-update GEMM for the mixed-precision LU (C -= A * B, FP32 storage).
#include "kd_gemm_tc.hpp"

namespace kd {

void gemm_update_f32(Context* ctx, cublasHandle_t blas, int m, int n, int k, const float* A, long long lda,
                     const float* B, long long ldb, float* C, long long ldc, bool tf32) {
  const float one = 1.0f, mone = -1.0f;
  ProfScope ps(ctx, Context::PROF_LU_GEMM, 2.0 * m * n * k);
  cublasComputeType_t ct = tf32 ? CUBLAS_COMPUTE_32F_FAST_TF32 : CUBLAS_COMPUTE_32F;
  cublasStatus_t st = cublasGemmEx(blas, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &mone, A, CUDA_R_32F, static_cast<int>(lda),
                                   B, CUDA_R_32F, static_cast<int>(ldb), &one, C, CUDA_R_32F, static_cast<int>(ldc), ct,
                                   CUBLAS_GEMM_DEFAULT);
  if (st != CUBLAS_STATUS_SUCCESS) throw KdError(KD_ERR_CUDA, "cublasGemmEx (trailing update) failed");
  ctx->launches++;
}

}  // namespace kd
