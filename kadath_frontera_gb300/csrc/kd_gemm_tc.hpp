// Trailing-update GEMM of the mixed-precision LU: C -= A * B with FP32
// storage, column-major.  `tf32` selects the tcgen05 TF32 tensor-core kernel
// (FP32 accumulation in tensor memory); otherwise a plain FP32 product.
#pragma once
#include <cublas_v2.h>

#include "kd_context.hpp"

namespace kd {

// c_rows_writable: rows [m, c_rows_writable) of every column of C are
// scratch that the update may overwrite (the padding of a matrix whose
// leading dimension is rounded up); pass m when there is none.
// terms: 1 = plain TF32 products; 3 = 3xTF32 (hi*hi + hi*lo + lo*hi, about
// FP32 accuracy), used where possible (k <= 96, TMA-aligned C).
// clusters: 0 runs the persistent tensor-core update on the whole GPU;
// 1 runs it as 16-CTA clusters, one cluster fewer than the GPU can hold, so
// that a 16-CTA cluster kernel launched beside it (the next panel) always
// finds a free GPC; 2 as many 16-CTA clusters as the GPU holds (the SMs
// outside them stay free for a kernel of independent CTAs beside it).
// max_ctas (> 0, clusters = 0 only): at most that many CTAs, for an update
// that runs beside another kernel's clusters (its CTAs loop over the tiles).
void gemm_update_f32(Context* ctx, cublasHandle_t blas, int m, int n, int k, const float* A, long long lda,
                     const float* B, long long ldb, float* C, long long ldc, bool tf32, int c_rows_writable,
                     int terms = 1, int clusters = 0, int max_ctas = 0);
// Clusters of 16 update CTAs the GPU holds at once (0: none).
int tf32_update_max_clusters16();

// The tcgen05 kernels on their own (k <= 128).
bool tf32_gemm_supported(int k);
void tf32_gemm_update(Context* ctx, int m, int n, int k, const float* A, long long lda, const float* B, long long ldb,
                      float* C, long long ldc, int c_rows_writable, int terms = 1, int clusters = 0,
                      int max_ctas = 0);
bool tf32x3_gemm_possible(int k, const float* C, long long ldc, int m, int c_rows_writable);
// Returns (and clears) the flag a CTA sets when its wait for the tensor-core
// results ran out of polls.
int tf32_gemm_error_flag(Context* ctx);

}  // namespace kd
