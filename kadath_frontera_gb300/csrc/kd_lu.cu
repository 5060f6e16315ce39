// Dense LU with partial pivoting (column-major) and triangular solves.
// Panel: one kernel per column (pivot search + row swap + scaling in one
// CTA, then a multi-CTA rank-1 update of the rest of the panel); TRSM of the
// U row block with the unit-lower L11 staged in shared memory; trailing
// update as a GEMM (FP64 library GEMM, or the TF32 tensor-core kernel of
// kd_gemm_tc.cu for the mixed mode).
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "kd_gemm_tc.hpp"
#include "kd_lu.hpp"

namespace kd {

namespace {

constexpr int PIV_THREADS = 1024;

template <class T>
__global__ void pivot_swap_scale(T* __restrict__ A, long long ld, int N, int j, int c0, int c1, int* ipiv,
                                 int* info) {
  // argmax |A[i, j]| over i in [j, N)
  __shared__ double sv[32];
  __shared__ int si[32];
  double best = -1.0;
  int bi = j;
  const T* col = A + static_cast<long long>(j) * ld;
  for (int i = j + threadIdx.x; i < N; i += blockDim.x) {
    double v = fabs(static_cast<double>(col[i]));
    if (v > best) {
      best = v;
      bi = i;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_xor_sync(0xffffffffu, best, o);
    int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ov > best || (ov == best && oi < bi)) {
      best = ov;
      bi = oi;
    }
  }
  if ((threadIdx.x & 31) == 0) {
    sv[threadIdx.x >> 5] = best;
    si[threadIdx.x >> 5] = bi;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    int nw = blockDim.x >> 5;
    best = (threadIdx.x < nw) ? sv[threadIdx.x] : -1.0;
    bi = (threadIdx.x < nw) ? si[threadIdx.x] : j;
    for (int o = 16; o > 0; o >>= 1) {
      double ov = __shfl_xor_sync(0xffffffffu, best, o);
      int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) {
        best = ov;
        bi = oi;
      }
    }
    if (threadIdx.x == 0) {
      si[0] = bi;
      sv[0] = best;
      ipiv[j] = bi;
      if (!(best > 0.0) && *info == 0) *info = j + 1;  // zero (or NaN) pivot
    }
  }
  __syncthreads();
  const int p = si[0];
  // swap rows j and p inside the panel columns [c0, c1)
  if (p != j)
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
      T* cc = A + static_cast<long long>(c) * ld;
      T t = cc[j];
      cc[j] = cc[p];
      cc[p] = t;
    }
  __syncthreads();
  double piv = static_cast<double>(col[j]);
  if (piv != 0.0) {
    double inv = 1.0 / piv;
    T* cj = A + static_cast<long long>(j) * ld;
    for (int i = j + 1 + threadIdx.x; i < N; i += blockDim.x) cj[i] = static_cast<T>(static_cast<double>(cj[i]) * inv);
  }
}

// A[i, k] -= A[i, j] * A[j, k]  for i in (j, N), k in (j, c1)
template <class T>
__global__ void panel_rank1(T* __restrict__ A, long long ld, int N, int j, int c1) {
  int i = j + 1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double lij = static_cast<double>(A[static_cast<long long>(j) * ld + i]);
  for (int k = j + 1; k < c1; k++) {
    T* ck = A + static_cast<long long>(k) * ld;
    ck[i] = static_cast<T>(static_cast<double>(ck[i]) - lij * static_cast<double>(ck[j]));
  }
}

// Applies the pivots ipiv[j0..j1) to columns [c0, c1) (dlaswp).
template <class T>
__global__ void laswp(T* __restrict__ A, long long ld, int j0, int j1, const int* __restrict__ ipiv, int c0, int c1) {
  int c = c0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= c1) return;
  T* cc = A + static_cast<long long>(c) * ld;
  for (int j = j0; j < j1; j++) {
    int p = ipiv[j];
    if (p != j) {
      T t = cc[j];
      cc[j] = cc[p];
      cc[p] = t;
    }
  }
}

// A12 := L11^{-1} A12, L11 unit lower (nb x nb at (j0, j0)), A12 = rows
// [j0, j0+nb) of columns [c0, c1).  One thread per column, TRSM_COLS columns
// per CTA; L11 and the column tile live in shared memory.
constexpr int TRSM_COLS = 64;
template <class T>
__global__ void trsm_unit_lower(T* __restrict__ A, long long ld, int j0, int nbk, int c0, int c1) {
  extern __shared__ unsigned char smraw[];
  double* L = reinterpret_cast<double*>(smraw);     // nbk x nbk, row-major L[i*nbk+k]
  double* X = L + nbk * nbk;                        // nbk x TRSM_COLS, X[i*TRSM_COLS + c]
  int cbase = c0 + blockIdx.x * TRSM_COLS;
  for (int e = threadIdx.x; e < nbk * nbk; e += blockDim.x) {
    int i = e % nbk, k = e / nbk;  // column-major read of L11
    L[i * nbk + k] = static_cast<double>(A[static_cast<long long>(j0 + k) * ld + j0 + i]);
  }
  for (int e = threadIdx.x; e < nbk * TRSM_COLS; e += blockDim.x) {
    int i = e % nbk, c = e / nbk;
    int col = cbase + c;
    X[i * TRSM_COLS + c] = (col < c1) ? static_cast<double>(A[static_cast<long long>(col) * ld + j0 + i]) : 0.0;
  }
  __syncthreads();
  int c = threadIdx.x;
  if (c < TRSM_COLS) {
    for (int i = 1; i < nbk; i++) {
      double s = X[i * TRSM_COLS + c];
      for (int k = 0; k < i; k++) s -= L[i * nbk + k] * X[k * TRSM_COLS + c];
      X[i * TRSM_COLS + c] = s;
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nbk * TRSM_COLS; e += blockDim.x) {
    int i = e % nbk, cc = e / nbk;
    int col = cbase + cc;
    if (col < c1) A[static_cast<long long>(col) * ld + j0 + i] = static_cast<T>(X[i * TRSM_COLS + cc]);
  }
}

__global__ void d2s(const double* __restrict__ A, long long lda, float* __restrict__ B, long long ldb, int N) {
  long long total = static_cast<long long>(N) * N;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    long long c = t / N, r = t % N;
    B[c * ldb + r] = static_cast<float>(A[c * lda + r]);
  }
}

// ---- triangular solves on one right-hand side (blocked by TB rows) --------
constexpr int TB = 64;

__global__ void apply_pivots_vec(double* b, const int* ipiv, int N, int reverse) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (!reverse) {
    for (int j = 0; j < N; j++) {
      int p = ipiv[j];
      if (p != j) {
        double t = b[j];
        b[j] = b[p];
        b[p] = t;
      }
    }
  } else {
    for (int j = N - 1; j >= 0; j--) {
      int p = ipiv[j];
      if (p != j) {
        double t = b[j];
        b[j] = b[p];
        b[p] = t;
      }
    }
  }
}

// Solves the diagonal block [r0, r1) of M x = b with M = A or A^T (trans):
// forward or backward substitution, unit or stored diagonal.
template <class T>
__global__ void trsv_block(const T* __restrict__ A, long long ld, double* b, int r0, int r1, int unit, int forward,
                           int trans) {
  __shared__ double x[TB];
  int n = r1 - r0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = b[r0 + i];
  __syncthreads();
  if (threadIdx.x == 0) {
    auto M = [&](int i, int k) -> double {
      return trans ? static_cast<double>(A[static_cast<long long>(r0 + i) * ld + r0 + k])
                   : static_cast<double>(A[static_cast<long long>(r0 + k) * ld + r0 + i]);
    };
    if (forward) {
      for (int i = 0; i < n; i++) {
        double s = x[i];
        for (int k = 0; k < i; k++) s -= M(i, k) * x[k];
        x[i] = unit ? s : s / M(i, i);
      }
    } else {
      for (int i = n - 1; i >= 0; i--) {
        double s = x[i];
        for (int k = i + 1; k < n; k++) s -= M(i, k) * x[k];
        x[i] = unit ? s : s / M(i, i);
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) b[r0 + i] = x[i];
}

// b[rows] -= M[rows, r0:r1] * b[r0:r1]  (M = A or A^T), rows = [q0, q1)
template <class T>
__global__ void gemv_update(const T* __restrict__ A, long long ld, double* b, int r0, int r1, int q0, int q1,
                            int trans) {
  __shared__ double x[TB];
  int n = r1 - r0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = b[r0 + i];
  __syncthreads();
  if (!trans) {
    int row = q0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= q1) return;
    double s = 0.0;
    for (int k = 0; k < n; k++) s += static_cast<double>(A[static_cast<long long>(r0 + k) * ld + row]) * x[k];
    b[row] -= s;
  } else {
    // one warp per output row: M^T[row, k] = A[k, row] is contiguous in k
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    int row = q0 + warp;
    if (row >= q1) return;
    double s = 0.0;
    const T* colp = A + static_cast<long long>(row) * ld + r0;
    for (int k = lane; k < n; k += 32) s += static_cast<double>(colp[k]) * x[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) b[row] -= s;
  }
}

// y = A x (FP64, column-major), one warp per 32-row stripe, FP64 accumulate.
__global__ void gemv_fp64(const double* __restrict__ A, long long ld, int N, const double* __restrict__ x,
                          double* __restrict__ y, double alpha, double beta, const double* __restrict__ b) {
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= N) return;
  double s = 0.0;
  for (int k = 0; k < N; k++) s = fma(A[static_cast<long long>(k) * ld + row], x[k], s);
  y[row] = alpha * s + (b ? beta * b[row] : 0.0);
}

int blocks(long long n, int t) { return static_cast<int>((n + t - 1) / t); }

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

DenseLU::DenseLU(Context* ctx) : ctx_(ctx) {
  if (cublasCreate(&blas_) != CUBLAS_STATUS_SUCCESS) throw KdError(KD_ERR_CUDA, "cublasCreate failed");
  cublasSetStream(blas_, ctx_->stream());
  cuda_check(cudaMalloc(&d_info_, sizeof(int)), "cudaMalloc(info)");
}

DenseLU::~DenseLU() {
  cudaStreamSynchronize(ctx_->stream());
  if (blas_) cublasDestroy(blas_);
  cudaFree(A32_);
  cudaFree(ipiv_);
  cudaFree(d_info_);
  cudaFree(work_);
  cudaFree(work32_);
}

void DenseLU::ensure_work(size_t n) {
  if (n > work_cap_) {
    cudaFree(work_);
    cuda_check(cudaMalloc(&work_, n * sizeof(double)), "cudaMalloc(lu work)");
    work_cap_ = n;
  }
}

template <class T>
static void panel_factor(Context* ctx, T* A, long long ld, int N, int j0, int jb, int* ipiv, int* info) {
  cudaStream_t s = ctx->stream();
  double fl = 0;
  for (int j = j0; j < j0 + jb; j++) fl += 2.0 * (N - j - 1) * (j0 + jb - j - 1) + (N - j);
  ProfScope ps(ctx, Context::PROF_LU_PANEL, fl);
  for (int j = j0; j < j0 + jb; j++) {
    pivot_swap_scale<T><<<1, PIV_THREADS, 0, s>>>(A, ld, N, j, j0, j0 + jb, ipiv, info);
    if (j + 1 < j0 + jb && j + 1 < N) panel_rank1<T><<<blocks(N - j - 1, 256), 256, 0, s>>>(A, ld, N, j, j0 + jb);
    ctx->launches += 2;
  }
  cuda_check(cudaGetLastError(), "panel kernels");
}

template <class T>
static void trsm_and_swaps(Context* ctx, T* A, long long ld, int N, int j0, int jb, const int* ipiv) {
  cudaStream_t s = ctx->stream();
  ProfScope ps(ctx, Context::PROF_LU_SWAP_TRSM, double(jb) * jb * (N - j0 - jb));
  if (j0 > 0) laswp<T><<<blocks(j0, 128), 128, 0, s>>>(A, ld, j0, j0 + jb, ipiv, 0, j0);
  if (j0 + jb < N) {
    laswp<T><<<blocks(N - j0 - jb, 128), 128, 0, s>>>(A, ld, j0, j0 + jb, ipiv, j0 + jb, N);
    size_t smem = sizeof(double) * (static_cast<size_t>(jb) * jb + static_cast<size_t>(jb) * TRSM_COLS);
    static bool attr_set = false;
    if (!attr_set) {
      cudaFuncSetAttribute(trsm_unit_lower<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      attr_set = true;
    }
    trsm_unit_lower<T><<<blocks(N - j0 - jb, TRSM_COLS), TRSM_COLS, smem, s>>>(A, ld, j0, jb, j0 + jb, N);
    ctx->launches += 1;
  }
  ctx->launches += 2;
  cuda_check(cudaGetLastError(), "laswp/trsm kernels");
}

void DenseLU::factor_fp64(double* A, long long ld, int N) {
  const int NB = nb > 96 ? 96 : nb;  // L11 + one column tile fit in shared memory
  cudaStream_t s = ctx_->stream();
  cuda_check(cudaMemsetAsync(d_info_, 0, sizeof(int), s), "memset info");
  for (int j0 = 0; j0 < N; j0 += NB) {
    int jb = (N - j0 < NB) ? N - j0 : NB;
    panel_factor<double>(ctx_, A, ld, N, j0, jb, ipiv_, d_info_);
    trsm_and_swaps<double>(ctx_, A, ld, N, j0, jb, ipiv_);
    int m = N - j0 - jb;
    if (m > 0) {
      // A22 -= A21 * A12 (FP64 library GEMM)
      const double one = 1.0, mone = -1.0;
      ProfScope ps(ctx_, Context::PROF_LU_GEMM, 2.0 * m * m * jb);
      double* A21 = A + static_cast<long long>(j0) * ld + j0 + jb;
      double* A12 = A + static_cast<long long>(j0 + jb) * ld + j0;
      double* A22 = A + static_cast<long long>(j0 + jb) * ld + j0 + jb;
      if (cublasDgemm(blas_, CUBLAS_OP_N, CUBLAS_OP_N, m, m, jb, &mone, A21, static_cast<int>(ld), A12,
                      static_cast<int>(ld), &one, A22, static_cast<int>(ld)) != CUBLAS_STATUS_SUCCESS)
        throw KdError(KD_ERR_CUDA, "cublasDgemm failed");
      ctx_->launches++;
    }
  }
}

void DenseLU::factor_f32(float* A, long long ld, int N, bool tf32) {
  const int NB = nb > 96 ? 96 : nb;
  cudaStream_t s = ctx_->stream();
  cuda_check(cudaMemsetAsync(d_info_, 0, sizeof(int), s), "memset info");
  for (int j0 = 0; j0 < N; j0 += NB) {
    int jb = (N - j0 < NB) ? N - j0 : NB;
    panel_factor<float>(ctx_, A, ld, N, j0, jb, ipiv_, d_info_);
    trsm_and_swaps<float>(ctx_, A, ld, N, j0, jb, ipiv_);
    int m = N - j0 - jb;
    if (m > 0) {
      float* A21 = A + static_cast<long long>(j0) * ld + j0 + jb;
      float* A12 = A + static_cast<long long>(j0 + jb) * ld + j0;
      float* A22 = A + static_cast<long long>(j0 + jb) * ld + j0 + jb;
      gemm_update_f32(ctx_, blas_, m, m, jb, A21, ld, A12, ld, A22, ld, tf32);
    }
  }
}

void DenseLU::factor(double* A, long long ld, int N, int mode) {
  if (N <= 0) throw KdError(KD_ERR_ARG, "empty matrix");
  double t0 = now_ms();
  mode_ = mode;
  N_ = N;
  ld_ = ld;
  A_ = A;
  if (static_cast<size_t>(N) > ipiv_cap_) {
    cudaFree(ipiv_);
    cuda_check(cudaMalloc(&ipiv_, sizeof(int) * N), "cudaMalloc(ipiv)");
    ipiv_cap_ = N;
  }
  stats = LuStats();
  stats.flops = static_cast<long long>(2.0 / 3.0 * double(N) * N * N);
  if (mode == LU_FP64) {
    factor_fp64(A, ld, N);
  } else {
    size_t need = static_cast<size_t>(N) * N;
    if (need > a32_cap_) {
      cudaFree(A32_);
      cuda_check(cudaMalloc(&A32_, need * sizeof(float)), "cudaMalloc(A32)");
      a32_cap_ = need;
    }
    d2s<<<152 * 8, 256, 0, ctx_->stream()>>>(A, ld, A32_, N, N);
    ctx_->launches++;
    factor_f32(A32_, N, N, mode == LU_TF32_IR);
  }
  int info = 0;
  cuda_check(cudaMemcpyAsync(&info, d_info_, sizeof(int), cudaMemcpyDeviceToHost, ctx_->stream()), "D2H info");
  cuda_check(cudaStreamSynchronize(ctx_->stream()), "sync after LU");
  stats.t_factor_ms = now_ms() - t0;
  if (info != 0) throw KdError(KD_ERR_SINGULAR, "Jacobian is singular (zero pivot at column " + std::to_string(info) + ")");
}

void DenseLU::solve_fp64(const double* LU, long long ld, int N, double* b, int trans) {
  cudaStream_t s = ctx_->stream();
  ProfScope ps(ctx_, Context::PROF_LU_SOLVE, 2.0 * N * N);
  if (!trans) {
    apply_pivots_vec<<<1, 1, 0, s>>>(b, ipiv_, N, 0);
    for (int r0 = 0; r0 < N; r0 += TB) {
      int r1 = r0 + TB < N ? r0 + TB : N;
      trsv_block<double><<<1, 64, 0, s>>>(LU, ld, b, r0, r1, 1, 1, 0);
      if (r1 < N) gemv_update<double><<<blocks(N - r1, 256), 256, 0, s>>>(LU, ld, b, r0, r1, r1, N, 0);
    }
    for (int r1 = N; r1 > 0; r1 -= TB) {
      int r0 = r1 - TB > 0 ? r1 - TB : 0;
      trsv_block<double><<<1, 64, 0, s>>>(LU, ld, b, r0, r1, 0, 0, 0);
      if (r0 > 0) gemv_update<double><<<blocks(r0, 256), 256, 0, s>>>(LU, ld, b, r0, r1, 0, r0, 0);
    }
  } else {
    // A^T = U^T L^T P: solve U^T y = b (forward), L^T z = y (backward), x = P^T z
    for (int r0 = 0; r0 < N; r0 += TB) {
      int r1 = r0 + TB < N ? r0 + TB : N;
      trsv_block<double><<<1, 64, 0, s>>>(LU, ld, b, r0, r1, 0, 1, 1);
      if (r1 < N) gemv_update<double><<<blocks(static_cast<long long>(N - r1) * 32, 256), 256, 0, s>>>(LU, ld, b, r0, r1, r1, N, 1);
    }
    for (int r1 = N; r1 > 0; r1 -= TB) {
      int r0 = r1 - TB > 0 ? r1 - TB : 0;
      trsv_block<double><<<1, 64, 0, s>>>(LU, ld, b, r0, r1, 1, 0, 1);
      if (r0 > 0) gemv_update<double><<<blocks(static_cast<long long>(r0) * 32, 256), 256, 0, s>>>(LU, ld, b, r0, r1, 0, r0, 1);
    }
    apply_pivots_vec<<<1, 1, 0, s>>>(b, ipiv_, N, 1);
  }
  ctx_->launches += 4 * ((N + TB - 1) / TB) + 1;
  cuda_check(cudaGetLastError(), "triangular solve");
}

void DenseLU::solve_f32(double* b) {
  cudaStream_t s = ctx_->stream();
  ProfScope ps(ctx_, Context::PROF_LU_SOLVE, 2.0 * N_ * N_);
  int N = N_;
  apply_pivots_vec<<<1, 1, 0, s>>>(b, ipiv_, N, 0);
  for (int r0 = 0; r0 < N; r0 += TB) {
    int r1 = r0 + TB < N ? r0 + TB : N;
    trsv_block<float><<<1, 64, 0, s>>>(A32_, N, b, r0, r1, 1, 1, 0);
    if (r1 < N) gemv_update<float><<<blocks(N - r1, 256), 256, 0, s>>>(A32_, N, b, r0, r1, r1, N, 0);
  }
  for (int r1 = N; r1 > 0; r1 -= TB) {
    int r0 = r1 - TB > 0 ? r1 - TB : 0;
    trsv_block<float><<<1, 64, 0, s>>>(A32_, N, b, r0, r1, 0, 0, 0);
    if (r0 > 0) gemv_update<float><<<blocks(r0, 256), 256, 0, s>>>(A32_, N, b, r0, r1, 0, r0, 0);
  }
  ctx_->launches += 4 * ((N + TB - 1) / TB) + 1;
  cuda_check(cudaGetLastError(), "fp32 triangular solve");
}

// Right-preconditioned GMRES(m) in FP64 with the FP32 LU as preconditioner:
// solves A x = b to a relative residual below gmres_tol.  Small dense
// Hessenberg algebra runs on the host (m <= 50), vectors stay on the device.
void DenseLU::gmres_ir(double* b) {
  const int N = N_;
  const int m = gmres_max_iter;
  cudaStream_t s = ctx_->stream();
  ensure_work(static_cast<size_t>(N) * (m + 4));
  double* V = work_;                                  // m+1 basis vectors
  double* w = work_ + static_cast<size_t>(N) * (m + 1);
  double* x = w + N;
  double* r = x + N;
  auto dot = [&](const double* a, const double* c) {
    double res;
    cublasDdot(blas_, N, a, 1, c, 1, &res);
    return res;
  };
  auto nrm = [&](const double* a) {
    double res;
    cublasDnrm2(blas_, N, a, 1, &res);
    return res;
  };
  cudaMemsetAsync(x, 0, sizeof(double) * N, s);
  double bnorm = nrm(b);
  if (bnorm == 0) return;
  int total_it = 0;
  for (int restart = 0; restart < 4; restart++) {
    // r = b - A x
    {
      ProfScope ps(ctx_, Context::PROF_GMRES, 8.0 * double(N) * N);
      gemv_fp64<<<blocks(N, 128), 128, 0, s>>>(A_, ld_, N, x, r, -1.0, 1.0, b);
    }
    ctx_->launches++;
    double beta = nrm(r);
    stats.final_rel_residual = beta / bnorm;
    if (beta / bnorm < gmres_tol) break;
    std::vector<double> H(static_cast<size_t>(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1, 0.0);
    g[0] = beta;
    double inv = 1.0 / beta;
    cublasDcopy(blas_, N, r, 1, V, 1);
    cublasDscal(blas_, N, &inv, V, 1);
    int k = 0;
    for (; k < m; k++) {
      // w = A M^{-1} v_k
      cublasDcopy(blas_, N, V + static_cast<size_t>(k) * N, 1, r, 1);
      solve_f32(r);
      {
        ProfScope ps(ctx_, Context::PROF_GMRES, 8.0 * double(N) * N);
        gemv_fp64<<<blocks(N, 128), 128, 0, s>>>(A_, ld_, N, r, w, 1.0, 0.0, nullptr);
      }
      ctx_->launches++;
      for (int i = 0; i <= k; i++) {  // modified Gram-Schmidt
        double h = dot(w, V + static_cast<size_t>(i) * N);
        H[i * m + k] = h;
        double mh = -h;
        cublasDaxpy(blas_, N, &mh, V + static_cast<size_t>(i) * N, 1, w, 1);
      }
      double hn = nrm(w);
      H[(k + 1) * m + k] = hn;
      if (hn > 0) {
        double ih = 1.0 / hn;
        cublasDcopy(blas_, N, w, 1, V + static_cast<size_t>(k + 1) * N, 1);
        cublasDscal(blas_, N, &ih, V + static_cast<size_t>(k + 1) * N, 1);
      }
      for (int i = 0; i < k; i++) {
        double t = cs[i] * H[i * m + k] + sn[i] * H[(i + 1) * m + k];
        H[(i + 1) * m + k] = -sn[i] * H[i * m + k] + cs[i] * H[(i + 1) * m + k];
        H[i * m + k] = t;
      }
      double a = H[k * m + k], c = H[(k + 1) * m + k];
      double d = std::sqrt(a * a + c * c);
      cs[k] = d > 0 ? a / d : 1.0;
      sn[k] = d > 0 ? c / d : 0.0;
      H[k * m + k] = d;
      H[(k + 1) * m + k] = 0;
      g[k + 1] = -sn[k] * g[k];
      g[k] = cs[k] * g[k];
      total_it++;
      if (std::fabs(g[k + 1]) / bnorm < gmres_tol || hn == 0) {
        k++;
        break;
      }
    }
    // y = H^{-1} g, x += M^{-1} V y
    std::vector<double> y(k, 0.0);
    for (int i = k - 1; i >= 0; i--) {
      double sum = g[i];
      for (int j = i + 1; j < k; j++) sum -= H[i * m + j] * y[j];
      y[i] = sum / H[i * m + i];
    }
    cudaMemsetAsync(r, 0, sizeof(double) * N, s);
    for (int i = 0; i < k; i++) cublasDaxpy(blas_, N, &y[i], V + static_cast<size_t>(i) * N, 1, r, 1);
    solve_f32(r);
    const double one = 1.0;
    cublasDaxpy(blas_, N, &one, r, 1, x, 1);
  }
  {
    ProfScope ps(ctx_, Context::PROF_GMRES, 8.0 * double(N) * N);
    gemv_fp64<<<blocks(N, 128), 128, 0, s>>>(A_, ld_, N, x, r, -1.0, 1.0, b);
  }
  ctx_->launches++;
  stats.final_rel_residual = nrm(r) / bnorm;
  stats.refine_iters = total_it;
  cublasDcopy(blas_, N, x, 1, b, 1);
}

void DenseLU::solve(double* b, int trans) {
  double t0 = now_ms();
  if (mode_ == LU_FP64) {
    solve_fp64(A_, ld_, N_, b, trans);
  } else {
    if (trans) throw KdError(KD_ERR_UNSUPPORTED, "transposed solve needs the FP64 factors");
    gmres_ir(b);
    if (!(stats.final_rel_residual < 1e-10))
      throw KdError(KD_ERR_NOCONV, "GMRES-IR did not converge (relative residual " +
                                       std::to_string(stats.final_rel_residual) + ")");
  }
  cuda_check(cudaStreamSynchronize(ctx_->stream()), "sync after solve");
  stats.t_solve_ms = now_ms() - t0;
}

}  // namespace kd
