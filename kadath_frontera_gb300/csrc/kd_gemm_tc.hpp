// Trailing-update GEMM of the mixed-precision LU: C -= A * B with FP32
// storage, column-major.  `tf32` selects TF32 tensor-core products with FP32
// accumulation; otherwise plain FP32.
#pragma once
#include <cublas_v2.h>

#include "kd_context.hpp"

namespace kd {

void gemm_update_f32(Context* ctx, cublasHandle_t blas, int m, int n, int k, const float* A, long long lda,
                     const float* B, long long ldb, float* C, long long ldc, bool tf32);

}  // namespace kd
