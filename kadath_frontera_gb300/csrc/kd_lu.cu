// Dense LU with partial pivoting (column-major) and triangular solves.
// Blocked right-looking factorisation, per panel of jb <= 96 columns:
//   panel    one cooperative kernel over the whole GPU, rows of the panel
//            held in shared memory, one grid barrier per column;
//   swaps    the panel's row exchanges as one list of row moves, applied
//            to the other columns by one warp per column;
//   TRSM     U12 = L11^{-1} A12 with L11 staged in shared memory;
//   update   A22 -= L21 U12 as a GEMM (FP64 library GEMM, or the TF32
//            tensor-core kernel of kd_gemm_tc.cu for the mixed modes).
// Solves use inverses of the 64 x 64 diagonal blocks (one launch per block).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "kd_gemm_tc.hpp"
#include "kd_lu.hpp"

namespace kd {

namespace {

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

// U12 = L11^-1 A12 (L11 unit lower, jb <= 96) for FP32 factors, 128 columns
// per CTA of 512 threads.  L11, transposed (LT[k][i] = l_ik), and the CTA's
// 96 x 128 column tile X go through shared memory.  The solve runs by 32-row
// chunks: a chunk's own triangle by columns (one thread per column, threads
// 0..127), and its products with the finished chunks as a register-tiled
// product (8 rows x 4 columns per thread, 128 threads).  Those products are
// split by k: right after chunk 0's triangle, chunks 1 and 2 take off their
// products with chunk 0 at the same time (threads 0..127 and 128..255).
// Every element still receives its multiply-adds in increasing k: the
// operations of a column-by-column forward substitution, in its order.  All
// 512 threads stage the tile (every load of a thread in flight before its
// stores) and write it back.
constexpr int TS_THREADS = 512;
constexpr int TS_COLS = 128;
constexpr int TS_LDL = 100;  // row stride of LT: 16-byte aligned rows
constexpr int TS_LDX = 132;  // row stride of X: 16-byte aligned rows
constexpr size_t TS_SMEM = sizeof(float) * (96 * TS_LDL + 96 * TS_LDX);

// X[r][c] -= sum_{k0 <= k < k1} l_rk X[k][c] (k in order) for the rows
// r = R0 + 8 tr + a and columns c = 4 tc + b of thread t = 32 tr + tc < 128.
__device__ __forceinline__ void ts_cross(const float* __restrict__ LT, float* __restrict__ X, int R0, int k0, int k1,
                                         int t) {
  const int tr = t >> 5, tc = t & 31;
  const int r0 = R0 + 8 * tr;
  float acc[8][4];
#pragma unroll
  for (int a = 0; a < 8; a++) {
    const float4 q = *reinterpret_cast<const float4*>(X + (r0 + a) * TS_LDX + 4 * tc);
    acc[a][0] = q.x;
    acc[a][1] = q.y;
    acc[a][2] = q.z;
    acc[a][3] = q.w;
  }
#pragma unroll 4
  for (int k = k0; k < k1; k++) {
    const float4 la = *reinterpret_cast<const float4*>(LT + k * TS_LDL + r0);  // the same for the whole warp
    const float4 lb = *reinterpret_cast<const float4*>(LT + k * TS_LDL + r0 + 4);
    const float4 y = *reinterpret_cast<const float4*>(X + k * TS_LDX + 4 * tc);
    const float l[8] = {la.x, la.y, la.z, la.w, lb.x, lb.y, lb.z, lb.w};
    const float yy[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
    for (int a = 0; a < 8; a++)
#pragma unroll
      for (int b = 0; b < 4; b++) acc[a][b] = fmaf(-l[a], yy[b], acc[a][b]);
  }
#pragma unroll
  for (int a = 0; a < 8; a++)
    *reinterpret_cast<float4*>(X + (r0 + a) * TS_LDX + 4 * tc) = make_float4(acc[a][0], acc[a][1], acc[a][2], acc[a][3]);
}

// The 32 x 32 unit lower triangle of chunk R0 for column t (< 128).
__device__ __forceinline__ void ts_diag(const float* __restrict__ LT, float* __restrict__ X, int R0, int t) {
  float x[32];
#pragma unroll
  for (int j = 0; j < 32; j++) x[j] = X[(R0 + j) * TS_LDX + t];
#pragma unroll
  for (int kk = 0; kk < 32; kk++) {
    const float y = x[kk];
    const float* lrow = LT + (R0 + kk) * TS_LDL + R0;
#pragma unroll
    for (int j = 0; j < 32; j++)
      if (j > kk) x[j] = fmaf(-lrow[j], y, x[j]);
  }
#pragma unroll
  for (int j = 0; j < 32; j++) X[(R0 + j) * TS_LDX + t] = x[j];
}

__global__ void __launch_bounds__(TS_THREADS) trsm_chunk_f32(float* __restrict__ A, long long ld, int j0, int jb,
                                                             int c0, int c1) {
  extern __shared__ __align__(16) float ts_sm[];
  float* LT = ts_sm;                // LT[k * TS_LDL + i] = l_ik (i > k, i < jb), zero elsewhere
  float* X = ts_sm + 96 * TS_LDL;  // X[i * TS_LDX + c]
  const int tid = threadIdx.x;
  const int cb = c0 + blockIdx.x * TS_COLS;
  {
    constexpr int NL = (96 * 96 + TS_THREADS - 1) / TS_THREADS, NX = 96 * TS_COLS / TS_THREADS;
    float v[NL], w[NX];
#pragma unroll
    for (int u = 0; u < NL; u++) {
      const int e = u * TS_THREADS + tid;
      const int i = e % 96, k = e / 96;  // down the columns: coalesced reads
      v[u] = (e < 96 * 96 && i < jb && k < i) ? A[static_cast<long long>(j0 + k) * ld + j0 + i] : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < NX; u++) {
      const int e = u * TS_THREADS + tid;
      const int i = e % 96, col = cb + e / 96;
      w[u] = (i < jb && col < c1) ? A[static_cast<long long>(col) * ld + j0 + i] : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < NL; u++) {
      const int e = u * TS_THREADS + tid;
      if (e < 96 * 96) LT[(e / 96) * TS_LDL + e % 96] = v[u];
    }
#pragma unroll
    for (int u = 0; u < NX; u++) {
      const int e = u * TS_THREADS + tid;
      X[(e % 96) * TS_LDX + e / 96] = w[u];
    }
  }
  __syncthreads();
  const int nch = (jb + 31) / 32;
  if (tid < 128) ts_diag(LT, X, 0, tid);
  __syncthreads();
  if (nch > 1) {
    if (tid < 128)
      ts_cross(LT, X, 32, 0, 32, tid);
    else if (tid < 256 && nch > 2)
      ts_cross(LT, X, 64, 0, 32, tid - 128);
    __syncthreads();
    if (tid < 128) ts_diag(LT, X, 32, tid);
    __syncthreads();
  }
  if (nch > 2) {
    if (tid < 128) ts_cross(LT, X, 64, 32, 64, tid);
    __syncthreads();
    if (tid < 128) ts_diag(LT, X, 64, tid);
    __syncthreads();
  }
  // write-back: four consecutive rows of one column per thread and step, as
  // one 16-byte store where the rows start 16-byte aligned
  const bool vec = (reinterpret_cast<unsigned long long>(A) & 15) == 0 && (ld & 3) == 0 && (j0 & 3) == 0;
#pragma unroll
  for (int q = 0; q < 96 * TS_COLS / 4 / TS_THREADS; q++) {
    const int e = tid + q * TS_THREADS;
    const int i = 4 * (e % 24), c = e / 24;
    const int col = cb + c;
    if (col < c1 && i < jb) {
      float* dst = A + static_cast<long long>(col) * ld + j0 + i;
      const float4 r = make_float4(X[i * TS_LDX + c], X[(i + 1) * TS_LDX + c], X[(i + 2) * TS_LDX + c],
                                   X[(i + 3) * TS_LDX + c]);
      if (vec && i + 3 < jb) {
        *reinterpret_cast<float4*>(dst) = r;
      } else {
        dst[0] = r.x;
        if (i + 1 < jb) dst[1] = r.y;
        if (i + 2 < jb) dst[2] = r.z;
        if (i + 3 < jb) dst[3] = r.w;
      }
    }
  }
}

// ---- equilibration of the FP32 working copy (mixed modes) --------------
// Row scales r_i = 2^-round(log2 max_j |A_ij|), then column scales
// c_j = 2^-round(log2 max_i |r_i A_ij|): powers of two, so scaling is exact
// and only the FP32 rounding remains.  The factors are those of
// D_r A D_c; the preconditioner is M^-1 b = D_c (LU)^-1 (D_r b).
__device__ __forceinline__ double pow2_inverse(double m) {
  if (!(m > 0.0) || !isfinite(m)) return 1.0;
  int e;
  frexp(m, &e);  // m = f 2^e, f in [0.5, 1)
  return ldexp(1.0, 1 - e);  // 2^-(e-1): scaled max in [1, 2)
}

// Maxima of |A_ij| over column chunks, merged with atomicMax on the bit
// patterns of non-negative doubles (order-independent, deterministic).
__global__ void row_absmax_kernel(const double* __restrict__ A, long long ld, int N, int chunk,
                                  unsigned long long* __restrict__ rmax) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int c0 = blockIdx.y * chunk;
  const int c1 = (c0 + chunk < N) ? c0 + chunk : N;
  double m = 0.0;
  for (int j = c0; j < c1; j++) m = fmax(m, fabs(A[static_cast<long long>(j) * ld + i]));
  atomicMax(rmax + i, static_cast<unsigned long long>(__double_as_longlong(m)));
}

__global__ void row_scale_kernel(const unsigned long long* __restrict__ rmax, int N, double* __restrict__ rs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) rs[i] = pow2_inverse(__longlong_as_double(static_cast<long long>(rmax[i])));
}

// One CTA per column: c_j from max_i |r_i A_ij|, then the scaled FP32 column.
__global__ void col_scale_convert_kernel(const double* __restrict__ A, long long lda, const double* __restrict__ rs,
                                         int N, double* __restrict__ cs, float* __restrict__ B, long long ldb) {
  __shared__ double red[32];
  const int j = blockIdx.x;
  const double* col = A + static_cast<long long>(j) * lda;
  double m = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) m = fmax(m, fabs(rs[i] * col[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) red[0] = m;
  }
  __syncthreads();
  const double c = pow2_inverse(red[0]);
  if (threadIdx.x == 0) cs[j] = c;
  float* out = B + static_cast<long long>(j) * ldb;
  for (int i = threadIdx.x; i < N; i += blockDim.x) out[i] = static_cast<float>(rs[i] * col[i] * c);
}

// ---- panel of a static-pivot factorisation (FP32, rows in pivot order) ----
// The rows of the working copy were gathered in the pivot order of an
// earlier partial-pivoting factorisation, so this panel does no row search:
// A11 = L11 U11 without exchanges, then L21 = A21 U11^-1.  Every CTA factors
// the (at most 96 x 96) diagonal block itself in shared memory -- redundant,
// but it removes every grid-wide synchronisation -- and then solves
// x U11 = a for NP_THREADS rows of A21, one row per thread with the row in
// registers.  The last CTA to finish writes L11 \ U11 back.  A zero or non-finite pivot sets
// *info (the caller then factors with partial pivoting instead).
constexpr int NP_NB = 96;
constexpr int NP_LD = NP_NB + 4;  // row stride: 16-byte aligned rows, read four elements at a time by L21
constexpr int NP_THREADS = 256;
constexpr int NP_XS_BYTES = (NP_NB - 32) * NP_THREADS * 4;  // the solved chunks 0 and 1 of every thread's row
constexpr int NP_MAX_CTAS = 38;  // SMs outside the seven 16-CTA clusters of a GB300's trailing update: 152 - 112 = 40
static_assert(NP_THREADS == 256 && NP_NB == 96, "three 32-column blocks; 16 x 16 threads tile the trailing blocks");

// Rank-32 update of the trailing block of the diagonal block after its
// 32-column block o: a_ij -= l_ik u_kj for k = o .. o+31 in order, rows and
// columns o+32 .. 95; thread (ty, tx) holds rows ty + 16 a and columns
// tx + 16 c (a, c < R) in registers.
template <int R>
__device__ __forceinline__ void np_trailing(float* __restrict__ U, int o, int tid) {
  const int ty = tid >> 4, tx = tid & 15, b = o + 32;
  float acc[R][R];
#pragma unroll
  for (int a = 0; a < R; a++)
#pragma unroll
    for (int c = 0; c < R; c++) acc[a][c] = U[(b + ty + 16 * a) * NP_LD + b + tx + 16 * c];
#pragma unroll 4
  for (int k = 0; k < 32; k++) {
    float l[R], u[R];
#pragma unroll
    for (int a = 0; a < R; a++) l[a] = U[(b + ty + 16 * a) * NP_LD + o + k];
#pragma unroll
    for (int c = 0; c < R; c++) u[c] = U[(o + k) * NP_LD + b + tx + 16 * c];
#pragma unroll
    for (int a = 0; a < R; a++)
#pragma unroll
      for (int c = 0; c < R; c++) acc[a][c] = fmaf(-l[a], u[c], acc[a][c]);
  }
#pragma unroll
  for (int a = 0; a < R; a++)
#pragma unroll
    for (int c = 0; c < R; c++) U[(b + ty + 16 * a) * NP_LD + b + tx + 16 * c] = acc[a][c];
}

// Eight elimination steps k0 .. k0+7 of a 32 x 32 diagonal block held by
// one warp, lane l holding row l with its values shifted so that d[0] is
// column k (see panel_nopiv_kernel).  From step k0 on at most W = 32 - k0
// columns are live, so only W - 1 values of the pivot row are broadcast.
// rp enters as __frcp_rn of step k0's pivot and leaves as the next one's;
// each step stores the element of column k that became final.
template <int W>
__device__ __forceinline__ void np_diag_steps(float (&d)[32], float& rp, float* __restrict__ urow,
                                              float* __restrict__ rpv, int lane, int k0) {
#pragma unroll 1
  for (int k = k0; k < k0 + 8; k++) {
    float pr[W];  // the pivot row (lane k's values)
#pragma unroll
    for (int j = 1; j < W; j++) pr[j] = __shfl_sync(0xffffffffu, d[j], k);
    // rows up to k (the finished ones and the pivot row) take a zero
    // multiplier: their multiply-adds leave them as they are
    const float lm = (lane > k) ? d[0] * rp : 0.0f;
    if (lane == 0) rpv[k] = rp;
    urow[k] = (lane > k) ? lm : d[0];
    // the next pivot first, so that its reciprocal overlaps this step
    d[0] = fmaf(-lm, pr[1], d[1]);
    const float rpn = __frcp_rn(__shfl_sync(0xffffffffu, d[0], (k + 1) & 31));
#pragma unroll
    for (int j = 2; j < W; j++) d[j - 1] = fmaf(-lm, pr[j], d[j]);
    d[W - 1] = 0.0f;
    rp = rpn;
  }
}

__global__ void __launch_bounds__(NP_THREADS) panel_nopiv_kernel(float* __restrict__ A, long long ld, int N, int j0,
                                                                 int jb, int rpt, int* __restrict__ info,
                                                                 unsigned* __restrict__ done) {
  __shared__ __align__(16) float U[NP_NB * NP_LD];
  __shared__ float rdiag[NP_NB];
  __shared__ float rpv[NP_NB];  // __frcp_rn of the pivots
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  {
    // all 36 loads of the thread in flight before the shared stores
    constexpr int NV = NP_NB * NP_NB / NP_THREADS;
    static_assert(NV * NP_THREADS == NP_NB * NP_NB, "the diagonal block splits evenly over the threads");
    float v[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) {
      const int e = tid + q * NP_THREADS;
      const int i = e % NP_NB, k = e / NP_NB;  // down the columns: coalesced reads
      v[q] = (i < jb && k < jb) ? A[static_cast<long long>(j0 + k) * ld + j0 + i]
                                : ((i == k) ? 1.0f : 0.0f);  // identity padding past jb
    }
#pragma unroll
    for (int q = 0; q < NV; q++) {
      const int e = tid + q * NP_THREADS;
      U[(e % NP_NB) * NP_LD + e / NP_NB] = v[q];
    }
  }
  __syncthreads();
  // Blocked right-looking elimination in shared memory, by 32-column
  // blocks o = 0, 32, 64 (identity padding past jb stays identity):
  //  (a) warp 0 factors the diagonal block in registers, lane l holding row
  //      o + l; step k broadcasts the pivot row by shuffles, no barrier;
  //  (b) threads 0..rest-1 solve the block row U12 by columns and threads
  //      128..128+rest-1 the block column L21 by rows;
  //  (c) all threads apply the rank-32 update to the trailing block, a
  //      register tile each.
  // Every element receives its multiply-adds in increasing k and every
  // multiplier is (value) * __frcp_rn(pivot), the unblocked right-looking
  // elimination's own operations in its own order: the factors are the same.
  // The loop over k of (a) stays rolled: one warp running unrolled
  // straight-line code once per launch waits on instruction fetch most of
  // the time.  So that registers are never indexed by k, each step shifts
  // the lane's values down by one (column o + k is always d[0]) and stores
  // the element that became final.
#pragma unroll
  for (int o = 0; o < NP_NB; o += 32) {
    if (warp == 0) {
      float d[32];  // row o + lane, columns o + k + j
#pragma unroll
      for (int j = 0; j < 32; j++) d[j] = U[(o + lane) * NP_LD + o + j];
      float* urow = U + (o + lane) * NP_LD + o;
      float rp = __frcp_rn(__shfl_sync(0xffffffffu, d[0], 0));  // the correctly rounded 1 / pivot
      np_diag_steps<32>(d, rp, urow, rpv + o, lane, 0);
      np_diag_steps<24>(d, rp, urow, rpv + o, lane, 8);
      np_diag_steps<16>(d, rp, urow, rpv + o, lane, 16);
      np_diag_steps<8>(d, rp, urow, rpv + o, lane, 24);
    }
    __syncthreads();
    const int rest = NP_NB - o - 32;
    if (rest == 0) break;
    if (tid < rest) {  // column j of U12: u_tj -= l_tk u_kj, k < t
      const int j = o + 32 + tid;
      float c[32];
#pragma unroll
      for (int t = 0; t < 32; t++) c[t] = U[(o + t) * NP_LD + j];
#pragma unroll
      for (int k = 0; k < 31; k++)
#pragma unroll
        for (int t = k + 1; t < 32; t++) c[t] = fmaf(-U[(o + t) * NP_LD + o + k], c[k], c[t]);
#pragma unroll
      for (int t = 1; t < 32; t++) U[(o + t) * NP_LD + j] = c[t];
    } else if (tid >= 128 && tid < 128 + rest) {  // row i of L21: l_ik = (a_ik - l_it u_tk, t < k) / u_kk
      const int i = o + 32 + tid - 128;
      float r[32];
#pragma unroll
      for (int k = 0; k < 32; k++) r[k] = U[i * NP_LD + o + k];
#pragma unroll
      for (int k = 0; k < 32; k++) {
        r[k] *= rpv[o + k];
#pragma unroll
        for (int t = k + 1; t < 32; t++) r[t] = fmaf(-r[k], U[(o + k) * NP_LD + o + t], r[t]);
      }
#pragma unroll
      for (int k = 0; k < 32; k++) U[i * NP_LD + o + k] = r[k];
    }
    __syncthreads();
    if (rest == 64)
      np_trailing<4>(U, o, tid);
    else
      np_trailing<2>(U, o, tid);
    __syncthreads();
  }
  if (tid < NP_NB) {
    const float d = U[tid * NP_LD + tid];
    if (tid < jb && !(fabsf(d) > 0.0f && isfinite(d)) && blockIdx.x == 0) atomicExch(info, j0 + tid + 1);
    rdiag[tid] = 1.0f / d;
  }
  __syncthreads();
  // L21: x U11 = a for each of this thread's rpt rows (CTA b owns rows
  // j0 + jb + [b rpt NP_THREADS, (b + 1) rpt NP_THREADS)), by 32-column
  // chunks with the chunk in registers: a chunk first takes off the products
  // with the finished chunks (kept in the thread's column of np_xs, dynamic
  // shared memory, rather than re-read from global memory), then is solved
  // against its 32 x 32 diagonal block of U11, then written back.
  extern __shared__ float np_xs[];  // [64][NP_THREADS]
  for (int rr = 0; rr < rpt; rr++) {
  const int row = j0 + jb + (blockIdx.x * rpt + rr) * NP_THREADS + tid;
  if (row >= N) break;
  float* arow = A + static_cast<long long>(j0) * ld + row;  // element k at arow[k * ld]
#pragma unroll
  for (int c = 0; c < NP_NB / 32; c++) {
    if (c * 32 >= jb) break;
    float x[32];
#pragma unroll
    for (int j = 0; j < 32; j++) x[j] = (c * 32 + j < jb) ? arow[static_cast<long long>(c * 32 + j) * ld] : 0.0f;
#pragma unroll
    for (int cp = 0; cp < c; cp++) {
#pragma unroll 8
      for (int kk = 0; kk < 32; kk++) {
        const float yk = np_xs[(cp * 32 + kk) * NP_THREADS + tid];
        const float4* urow = reinterpret_cast<const float4*>(U + (cp * 32 + kk) * NP_LD + c * 32);
#pragma unroll
        for (int j4 = 0; j4 < 8; j4++) {
          const float4 u = urow[j4];
          x[4 * j4] = fmaf(-yk, u.x, x[4 * j4]);
          x[4 * j4 + 1] = fmaf(-yk, u.y, x[4 * j4 + 1]);
          x[4 * j4 + 2] = fmaf(-yk, u.z, x[4 * j4 + 2]);
          x[4 * j4 + 3] = fmaf(-yk, u.w, x[4 * j4 + 3]);
        }
      }
    }
#pragma unroll
    for (int kk = 0; kk < 32; kk++) {
      x[kk] *= rdiag[c * 32 + kk];
      const float xk = x[kk];
      const float4* urow = reinterpret_cast<const float4*>(U + (c * 32 + kk) * NP_LD + c * 32);
#pragma unroll
      for (int j4 = (kk + 1) / 4; j4 < 8; j4++) {
        const float4 u = urow[j4];
        if (4 * j4 > kk) x[4 * j4] = fmaf(-xk, u.x, x[4 * j4]);
        if (4 * j4 + 1 > kk) x[4 * j4 + 1] = fmaf(-xk, u.y, x[4 * j4 + 1]);
        if (4 * j4 + 2 > kk) x[4 * j4 + 2] = fmaf(-xk, u.z, x[4 * j4 + 2]);
        if (4 * j4 + 3 > kk) x[4 * j4 + 3] = fmaf(-xk, u.w, x[4 * j4 + 3]);
      }
    }
#pragma unroll
    for (int j = 0; j < 32; j++)
      if (c * 32 + j < jb) arow[static_cast<long long>(c * 32 + j) * ld] = x[j];
    if (c < NP_NB / 32 - 1) {
#pragma unroll
      for (int j = 0; j < 32; j++) np_xs[(c * 32 + j) * NP_THREADS + tid] = x[j];
    }
  }
  }
  // L11 \ U11 goes back to A only when every CTA has read the diagonal
  // block: the last CTA to finish writes it (each holds the same factors)
  // and resets the counter for the next panel.  CTAs need not be resident
  // together, as they are beside the trailing update on a side stream.
  __shared__ int np_last;
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    np_last = (atomicAdd(done, 1u) == gridDim.x - 1) ? 1 : 0;
    __threadfence();
  }
  __syncthreads();
  if (np_last) {
    for (int e = tid; e < jb * jb; e += NP_THREADS) {
      const int i = e % jb, k = e / jb;
      A[static_cast<long long>(j0 + k) * ld + j0 + i] = U[i * NP_LD + k];
    }
    if (tid == 0) *done = 0u;
  }
}

// The FP32 working copy with its rows in a given order:
// B[i][j] = r_{p(i)} A[p(i)][j] c_j, c_j = 2^-round(log2 max_i |r_i A_ij|)
// (the same column scales as col_scale_convert_kernel, whose maximum does
// not depend on the row order).  rs == nullptr: no scaling.
__global__ void convert_rows_kernel(const double* __restrict__ A, long long lda, const double* __restrict__ rs,
                                    int N, double* __restrict__ cs, float* __restrict__ B, long long ldb,
                                    const int* __restrict__ perm) {
  __shared__ double red[32];
  const int j = blockIdx.x;
  const double* col = A + static_cast<long long>(j) * lda;
  double c = 1.0;
  if (rs) {
    double m = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) m = fmax(m, fabs(rs[i] * col[i]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
      m = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
      if (threadIdx.x == 0) red[0] = m;
    }
    __syncthreads();
    c = pow2_inverse(red[0]);
    if (threadIdx.x == 0) cs[j] = c;
  }
  float* out = B + static_cast<long long>(j) * ldb;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const int p = perm[i];
    out[i] = static_cast<float>((rs ? rs[p] : 1.0) * col[p] * c);
  }
}

__global__ void scale_vec_kernel(double* __restrict__ x, const double* __restrict__ s, int N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) x[i] *= s[i];
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

// ipiv[j] = j: every pivot entry holds a valid row before the panels write
// theirs, so that a panel which gave up (a grid barrier wait ran out) leaves
// only in-range rows behind for the row exchanges that follow it.
__global__ void iota_kernel(int* __restrict__ v, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

// perm such that (P b)[i] = b[perm[i]] for the sequential row swaps ipiv.
__global__ void build_perm(const int* __restrict__ ipiv, int N, int* __restrict__ perm) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int i = 0; i < N; i++) perm[i] = i;
  for (int j = 0; j < N; j++) {
    int p = ipiv[j];
    int t = perm[j];
    perm[j] = perm[p];
    perm[p] = t;
  }
}

__global__ void gather_perm(const double* __restrict__ b, const int* __restrict__ perm, int N, double* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) out[i] = b[perm[i]];
}

__global__ void scatter_perm(const double* __restrict__ z, const int* __restrict__ perm, int N, double* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) out[perm[i]] = z[i];
}

// One CTA per TB x TB diagonal block: inverse of its unit-lower part (L) and
// of its upper part (U), row-major, zero padded to TB x TB.  Thread c builds
// column c of each inverse by substitution in FP64.
template <class T>
__global__ void invert_diag_blocks(const T* __restrict__ A, long long ld, int N, double* __restrict__ Linv,
                                   double* __restrict__ Uinv) {
  extern __shared__ double sm[];
  double* D = sm;                 // D[i*TB + k]
  double* XL = sm + TB * TB;      // XL[i*TB + c]
  double* XU = sm + 2 * TB * TB;  // XU[i*TB + c]
  const int blk = blockIdx.x;
  const int r0 = blk * TB;
  const int n = (N - r0 < TB) ? N - r0 : TB;
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    int i = e / TB, k = e % TB;
    D[e] = (i < n && k < n) ? static_cast<double>(A[static_cast<long long>(r0 + k) * ld + r0 + i]) : 0.0;
    XL[e] = 0.0;
    XU[e] = 0.0;
  }
  __syncthreads();
  const int c = threadIdx.x;
  if (c < n) {
    XL[c * TB + c] = 1.0;
    for (int i = c + 1; i < n; i++) {
      double s = 0.0;
      for (int k = c; k < i; k++) s += D[i * TB + k] * XL[k * TB + c];
      XL[i * TB + c] = -s;
    }
    XU[c * TB + c] = 1.0 / D[c * TB + c];
    for (int i = c - 1; i >= 0; i--) {
      double s = 0.0;
      for (int k = i + 1; k <= c; k++) s += D[i * TB + k] * XU[k * TB + c];
      XU[i * TB + c] = -s / D[i * TB + i];
    }
  }
  __syncthreads();
  double* lo = Linv + static_cast<size_t>(blk) * TB * TB;
  double* uo = Uinv + static_cast<size_t>(blk) * TB * TB;
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    lo[e] = XL[e];
    uo[e] = XU[e];
  }
}

// One block step of a triangular solve with M = A (trans = 0) or A^T:
//   x = Dinv * b[r0 : r0+n]  (Dinv^T when dinv_t),  y[r0 : r0+n] = x,
//   b[row] -= sum_k M(row, r0+k) x_k  for row in [q0, q1).
// Rows of the block itself are only read, so every CTA sees the same x.
template <class T>
__global__ void trsv_step(const T* __restrict__ A, long long ld, double* __restrict__ b, double* __restrict__ y, int r0,
                          int n, const double* __restrict__ Dinv, int dinv_t, int q0, int q1, int trans) {
  __shared__ double bb[TB];
  __shared__ double xx[TB];
  for (int i = threadIdx.x; i < TB; i += blockDim.x) bb[i] = (i < n) ? b[r0 + i] : 0.0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < n; k++) s += (dinv_t ? Dinv[k * TB + i] : Dinv[i * TB + k]) * bb[k];
    xx[i] = s;
  }
  __syncthreads();
  if (blockIdx.x == 0)
    for (int i = threadIdx.x; i < n; i += blockDim.x) y[r0 + i] = xx[i];
  if (q1 <= q0) return;
  if (!trans) {
    int row = q0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= q1) return;
    double s = 0.0;
    for (int k = 0; k < n; k++) s += static_cast<double>(A[static_cast<long long>(r0 + k) * ld + row]) * xx[k];
    b[row] -= s;
  } else {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    int row = q0 + warp;
    if (row >= q1) return;
    const T* colp = A + static_cast<long long>(row) * ld + r0;
    double s = 0.0;
    for (int k = lane; k < n; k += 32) s += static_cast<double>(colp[k]) * xx[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) b[row] -= s;
  }
}

// y = alpha A x + beta b (FP64, column-major).  The columns are split into
// chunks so that the grid covers the GPU: gemv_partial writes one partial
// sum per (chunk, row), gemv_finish adds them in chunk order (deterministic).
constexpr int GEMV_ROWS = 256;
__global__ void __launch_bounds__(GEMV_ROWS) gemv_partial(const double* __restrict__ A, long long ld, int N,
                                                          const double* __restrict__ x, int chunk,
                                                          double* __restrict__ part) {
  const int row = blockIdx.x * GEMV_ROWS + threadIdx.x;
  if (row >= N) return;
  const int c0 = blockIdx.y * chunk;
  const int c1 = (c0 + chunk < N) ? c0 + chunk : N;
  const double* a = A + static_cast<long long>(c0) * ld + row;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  int k = c0;
  // eight column loads in flight per thread, then the multiply-adds
  for (; k + 7 < c1; k += 8) {
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; u++) v[u] = __ldcs(a + u * ld);
    s0 = fma(v[0], x[k], s0);
    s1 = fma(v[1], x[k + 1], s1);
    s2 = fma(v[2], x[k + 2], s2);
    s3 = fma(v[3], x[k + 3], s3);
    s0 = fma(v[4], x[k + 4], s0);
    s1 = fma(v[5], x[k + 5], s1);
    s2 = fma(v[6], x[k + 6], s2);
    s3 = fma(v[7], x[k + 7], s3);
    a += 8 * ld;
  }
  for (; k + 3 < c1; k += 4) {
    s0 = fma(a[0], x[k], s0);
    s1 = fma(a[ld], x[k + 1], s1);
    s2 = fma(a[2 * ld], x[k + 2], s2);
    s3 = fma(a[3 * ld], x[k + 3], s3);
    a += 4 * ld;
  }
  for (; k < c1; k++) {
    s0 = fma(a[0], x[k], s0);
    a += ld;
  }
  part[static_cast<size_t>(blockIdx.y) * N + row] = (s0 + s1) + (s2 + s3);
}

__global__ void gemv_finish(const double* __restrict__ part, int nchunk, int N, double alpha, double beta,
                            const double* __restrict__ b, double* __restrict__ y) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= N) return;
  double s = 0.0;
  for (int c = 0; c < nchunk; c++) s += part[static_cast<size_t>(c) * N + row];
  y[row] = alpha * s + (b ? beta * b[row] : 0.0);
}

// y = alpha A^T x + beta b: one warp per column of A (a row of A^T), the
// column read coalesced, lane partial sums reduced by xor shuffles (fixed
// order).
constexpr int GEMVT_WARPS = 8;
__global__ void __launch_bounds__(GEMVT_WARPS * 32) gemv_t_kernel(const double* __restrict__ A, long long ld, int N,
                                                                 const double* __restrict__ x, double alpha,
                                                                 double beta, const double* __restrict__ b,
                                                                 double* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int col = blockIdx.x * GEMVT_WARPS + (threadIdx.x >> 5);
  if (col >= N) return;
  const double* a = A + static_cast<long long>(col) * ld;
  double s0 = 0.0, s1 = 0.0;
  int k = lane;
  for (; k + 32 < N; k += 64) {
    s0 = fma(a[k], x[k], s0);
    s1 = fma(a[k + 32], x[k + 32], s1);
  }
  if (k < N) s0 = fma(a[k], x[k], s0);
  double sum = s0 + s1;
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) y[col] = alpha * sum + (b ? beta * b[col] : 0.0);
}

// ---- vector algebra of GMRES (fixed reduction order: bitwise reproducible) --
constexpr int VA_THREADS = 256;

// h[i] = V_i . w for the k basis vectors V_i = V + i N: one CTA per i.
__global__ void basis_dots(const double* __restrict__ V, int N, int k, const double* __restrict__ w,
                           double* __restrict__ h) {
  __shared__ double part[VA_THREADS];
  const int i = blockIdx.x;
  const double* v = V + static_cast<size_t>(i) * N;
  double acc = 0.0;
  for (int t = threadIdx.x; t < N; t += VA_THREADS) acc = fma(v[t], w[t], acc);
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int st = VA_THREADS / 2; st > 0; st >>= 1) {
    if (static_cast<int>(threadIdx.x) < st) part[threadIdx.x] += part[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0 && i < k) h[i] = part[0];
}

// w -= sum_i h[i] V_i over the k basis vectors.
__global__ void basis_subtract(const double* __restrict__ V, int N, int k, const double* __restrict__ h,
                               double* __restrict__ w) {
  const int t = blockIdx.x * VA_THREADS + threadIdx.x;
  if (t >= N) return;
  double acc = 0.0;
  for (int i = 0; i < k; i++) acc = fma(h[i], V[static_cast<size_t>(i) * N + t], acc);
  w[t] -= acc;
}

// out = sum_t x[t]^2 (a single CTA, fixed order).
__global__ void sum_squares(const double* __restrict__ x, int N, double* __restrict__ out) {
  __shared__ double part[VA_THREADS];
  double acc = 0.0;
  for (int t = threadIdx.x; t < N; t += VA_THREADS) acc = fma(x[t], x[t], acc);
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int st = VA_THREADS / 2; st > 0; st >>= 1) {
    if (static_cast<int>(threadIdx.x) < st) part[threadIdx.x] += part[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = part[0];
}

// y = alpha x, or y += alpha x when accumulate is set.
__global__ void scaled_copy(int N, double alpha, const double* __restrict__ x, double* __restrict__ y,
                            int accumulate) {
  const int t = blockIdx.x * VA_THREADS + threadIdx.x;
  if (t >= N) return;
  y[t] = accumulate ? fma(alpha, x[t], y[t]) : alpha * x[t];
}

int blocks(long long n, int t) { return static_cast<int>((n + t - 1) / t); }

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

DenseLU::DenseLU(Context* ctx) : ctx_(ctx) {
  if (const char* e = std::getenv("KD_SWEEP")) {
    const std::string v(e);
    sweep_kind = v == "barrier" ? 0 : v == "pull" ? 1 : 2;
  }
  if (cublasCreate(&blas_) != CUBLAS_STATUS_SUCCESS) throw KdError(KD_ERR_CUDA, "cublasCreate failed");
  cublasSetStream(blas_, ctx_->stream());
  cuda_check(cudaMalloc(&d_info_, sizeof(int)), "cudaMalloc(info)");
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  cuda_check(cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, dev), "SM count");
  // panel exchange slots (sized for FP64 rows), barrier counter, error flag,
  // then the row-move list of one panel
  const size_t slot_bytes = sizeof(double) * (2 * 128 * static_cast<size_t>(nsm_) + 2 * nsm_ + 2 * 128) +
                            sizeof(int) * 2 * static_cast<size_t>(nsm_) + 32;
  const size_t map_bytes = sizeof(int) * (1 + 4 * 128) + 60;  // + padding to 16 bytes
  cuda_check(cudaMalloc(&slot_mem_, slot_bytes + map_bytes + 32), "cudaMalloc(panel slots)");
  cuda_check(cudaMemsetAsync(slot_mem_, 0, slot_bytes + map_bytes + 32, ctx_->stream()), "memset panel slots");
  swap_map_ = reinterpret_cast<int*>(static_cast<char*>(slot_mem_) + slot_bytes);
  tri_bar_ = reinterpret_cast<unsigned*>(static_cast<char*>(slot_mem_) + slot_bytes + map_bytes);
  panel_err_ = reinterpret_cast<int*>(static_cast<char*>(slot_mem_) + slot_bytes - 16);
  np_done_ = tri_bar_ + 4;
}

DenseLU::~DenseLU() {
  cudaStreamSynchronize(ctx_->stream());
  if (blas_) cublasDestroy(blas_);
  cudaFree(A32_);
  cudaFree(ipiv_);
  cudaFree(d_info_);
  cudaFree(slot_mem_);
  cudaFree(eq_buf_);
  cudaFree(part_);
  cudaFree(work_);
  if (hproj_) cudaFreeHost(hproj_);
  cudaFree(work32_);
  cudaFree(dinv_l_);
  cudaFree(dinv_u_);
  cudaFree(dinv2_l_);
  cudaFree(dinv2_u_);
  cudaFree(perm_);
  cudaFree(tri_work_);
  cudaFree(bsave_);
}

void DenseLU::ensure_work(size_t n) {
  if (n > work_cap_) {
    cudaFree(work_);
    cuda_check(cudaMalloc(&work_, n * sizeof(double)), "cudaMalloc(lu work)");
    work_cap_ = n;
  }
}

// Panel of jb columns factored by one thread-block cluster: CTA r owns a
// contiguous slice of the rows [j0, N).  Per column: local arg-max, cluster
// barrier, every CTA reads the CL candidates from distributed shared memory
// and agrees on the pivot, CTA 0 swaps the two rows of the panel, cluster
// barrier, then each CTA scales and rank-1-updates its own rows.  Panel data
// stays in global memory (it fits in L2).
constexpr int PANEL_CL = 8;
constexpr int PANEL_THREADS = 1024;

template <class T>
__global__ void panel_cluster_kernel(T* __restrict__ A, long long ld, int N, int j0, int jb, int* __restrict__ ipiv,
                                     int* __restrict__ info) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  __shared__ double cand_v[1];
  __shared__ int cand_i[1];
  __shared__ double red_v[32];
  __shared__ int red_i[32];
  __shared__ double prow[128];  // pivot row segment (jb <= 128)
  __shared__ int s_piv;
  const int rank = static_cast<int>(cluster.block_rank());
  const int nrows = N - j0;
  const int per = (nrows + PANEL_CL - 1) / PANEL_CL;
  const int my0 = j0 + rank * per;
  const int my1 = (my0 + per < N) ? my0 + per : N;
  const int c1 = j0 + jb;
  for (int j = j0; j < c1; j++) {
    // 1. local arg-max of |A[i, j]| over my rows i >= j
    const T* col = A + static_cast<long long>(j) * ld;
    double best = -1.0;
    int bi = N;  // "no row" sentinel, larger than any row index
    int start = my0 > j ? my0 : j;
    for (int i = start + threadIdx.x; i < my1; i += blockDim.x) {
      double v = fabs(static_cast<double>(col[i]));
      if (v > best || (v == best && i < bi)) {
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
      red_v[threadIdx.x >> 5] = best;
      red_i[threadIdx.x >> 5] = bi;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      int nw = blockDim.x >> 5;
      best = (threadIdx.x < nw) ? red_v[threadIdx.x] : -1.0;
      bi = (threadIdx.x < nw) ? red_i[threadIdx.x] : N;
      for (int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_xor_sync(0xffffffffu, best, o);
        int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      if (threadIdx.x == 0) {
        cand_v[0] = best;
        cand_i[0] = bi;
      }
    }
    __threadfence();
    cluster.sync();
    // 2. every CTA combines the CL candidates (same order, same result)
    if (threadIdx.x == 0) {
      double gb = -1.0;
      int gi = N;
      for (int r = 0; r < PANEL_CL; r++) {
        double v = *cluster.map_shared_rank(&cand_v[0], r);
        int ii = *cluster.map_shared_rank(&cand_i[0], r);
        if (v > gb || (v == gb && ii < gi)) {
          gb = v;
          gi = ii;
        }
      }
      if (gi >= N) gi = j;  // empty column below the diagonal
      s_piv = gi;
      if (rank == 0) {
        ipiv[j] = gi;
        if (!(gb > 0.0) && *info == 0) *info = j + 1;  // zero or NaN pivot
      }
    }
    __syncthreads();
    const int p = s_piv;
    // 3. CTA 0 swaps rows j and p inside the panel
    if (rank == 0 && p != j)
      for (int c = j0 + threadIdx.x; c < c1; c += blockDim.x) {
        T* cc = A + static_cast<long long>(c) * ld;
        T t = cc[j];
        cc[j] = cc[p];
        cc[p] = t;
      }
    __threadfence();
    cluster.sync();
    // 4. scale and rank-1 update of my rows below j
    for (int k = threadIdx.x; k < c1 - j; k += blockDim.x)
      prow[k] = static_cast<double>(A[static_cast<long long>(j + k) * ld + j]);
    __syncthreads();
    const double piv = prow[0];
    if (piv != 0.0) {
      // the update runs in the storage precision (FP32 for the mixed modes)
      const T inv = static_cast<T>(1.0 / piv);
      int rs = my0 > j + 1 ? my0 : j + 1;
      for (int i = rs + threadIdx.x; i < my1; i += blockDim.x) {
        T* ci = A + static_cast<long long>(j) * ld + i;
        T l = *ci * inv;
        *ci = l;
        for (int k = 1; k < c1 - j; k++) {
          T* ck = A + static_cast<long long>(j + k) * ld + i;
          *ck = fma(-l, static_cast<T>(prow[k]), *ck);
        }
      }
    }
    __syncthreads();
  }
}

// ---- panel over the whole GPU (cooperative launch) ------------------------
// CTA b owns rows [j0 + b*per, j0 + (b+1)*per) of the panel and keeps them in
// shared memory, column-major (tile[k*per + r]), for the whole panel.  Per
// column j, ONE grid barrier:
//   before it, every CTA publishes its local arg-max |a(i, j)| with the full
//   panel row of that candidate, and the CTA owning row j publishes row j
//   (double-buffered slots, indexed by the column's parity);
//   after it, every CTA reduces the candidates in the same order (largest
//   modulus, ties to the lowest row, as idamax), reads the winning row as the
//   pivot row, the owner of the pivot row takes row j in its place, the owner
//   of row j takes the pivot row, and each CTA scales and rank-1-updates its
//   own rows.
// Slot reuse is safe: a CTA writes slot (jj & 1) at column jj only after
// barrier jj-1, by which every CTA has finished reading that slot (column
// jj-2).  Cross-CTA data is read with L1-bypassing loads.
constexpr int GP_THREADS = 256;
constexpr int GP_MIN_ROWS = 32;
constexpr size_t GP_MAX_SMEM = 200 * 1024;

template <class T>
struct PanelSlots {
  T* cand_rows;     // [2][nblk][jb]
  double* cand_v;   // [2][nblk]
  int* cand_i;      // [2][nblk]
  T* jrow;          // [2][jb]
  unsigned* bar;    // arrival counter, zeroed before the launch
  int* err;         // set when a barrier wait runs out
  unsigned long long wait_ns;  // limit of one barrier wait (Context::grid_wait_ns)
  unsigned stall;   // added to every barrier target (Context::stall_waits)
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier of a cooperative launch (all CTAs resident): the CTA's
// writes are published by thread 0's release increment (after the block
// barrier), the other CTAs' writes acquired by its polling loads.  Returns
// false, with *err set, when the counter did not reach `target` within
// limit_ns; the caller then leaves its loops.
__device__ bool grid_barrier(unsigned* bar, unsigned target, int* err, int* s_ok, unsigned long long limit_ns) {
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(bar), "r"(1u) : "memory");
    const unsigned long long t0 = globaltimer_ns();
    int ok = 1;
    for (unsigned it = 0;; it++) {
      unsigned v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
      if (v >= target) break;
      if ((it & 31) == 31 && globaltimer_ns() - t0 > limit_ns) {
        ok = 0;
        atomicExch(err, 1);
        break;
      }
      __nanosleep(20);
    }
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

template <class V>
__device__ __forceinline__ bool better(V v, int i, V bv, int bi) {
  return v > bv || (v == bv && i < bi);
}

// Block-wide arg-max of (v, i) carrying a tag; every thread gets the result.
template <class V>
__device__ void block_argmax(V& v, int& i, int& tag, V* rv, int* ri, int* rt) {
  for (int o = 16; o > 0; o >>= 1) {
    V ov = __shfl_xor_sync(0xffffffffu, v, o);
    int oi = __shfl_xor_sync(0xffffffffu, i, o);
    int ot = __shfl_xor_sync(0xffffffffu, tag, o);
    if (better(ov, oi, v, i)) {
      v = ov;
      i = oi;
      tag = ot;
    }
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    rv[w] = v;
    ri[w] = i;
    rt[w] = tag;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < static_cast<int>(blockDim.x >> 5); q++)
      if (better(rv[q], ri[q], rv[0], ri[0])) {
        rv[0] = rv[q];
        ri[0] = ri[q];
        rt[0] = rt[q];
      }
  }
  __syncthreads();
  v = rv[0];
  i = ri[0];
  tag = rt[0];
  __syncthreads();
}

// A whole triangular sweep with the factors in one cooperative launch: per
// 64-row block k (in order for L, reversed for U), every CTA forms
// x_k = Dinv_k b[block] (Dinv_k row-major; warp w owns rows 8w..8w+7, lanes
// along the row, all loads issued before the reductions), CTA 0 stores x_k
// in y, and the rows below (L) or above (U) get b[row] -= A(row, block) x_k;
// then one grid barrier.  Rows go by 64-row tiles, tile t to CTA t % grid:
// within a CTA, warp w takes rows 32 (w >> 2) .. + 31 of the tile and the
// 16 block columns 16 (w & 3) .. + 15 (16 independent loads per thread), and
// the four column quarters are added in shared memory.  A row of b is only
// ever written by its tile's CTA; block rows written by other CTAs are read
// past L1.
constexpr int SW_TILE = 64;
constexpr int SW_MAXT = 24;  // tiles a CTA keeps in shared memory during a sweep

// Geometry of one block step of a sweep.
struct SweepStep {
  int k, r0, n, q0, q1, first, t1;
};

__device__ __forceinline__ SweepStep sweep_step(int step, int nblk, int N, int lower, int ntiles) {
  SweepStep s;
  s.k = lower ? step : nblk - 1 - step;
  s.r0 = s.k * TB;
  s.n = (N - s.r0 < TB) ? N - s.r0 : TB;
  s.q0 = lower ? s.r0 + s.n : 0;
  s.q1 = lower ? N : s.r0;
  const int t0 = s.q0 / SW_TILE;
  s.t1 = (s.q1 + SW_TILE - 1) / SW_TILE;
  if (s.t1 > ntiles) s.t1 = ntiles;
  s.first = t0 - (t0 % static_cast<int>(gridDim.x)) + static_cast<int>(blockIdx.x);
  if (s.first < t0) s.first += gridDim.x;
  return s;
}

// The values this thread needs from Dinv_k and from the factor's block
// columns for its first two tiles: loaded one step ahead, before the grid
// barrier, since they do not depend on b.
template <class T>
struct SweepPrefetch {
  double lo[8], hi[8];  // Dinv_k entries (FP64 factors)
  float2 dlo[8], dhi[8];  // Dinv_k entries as (hi, lo) FP32 pairs (FP32 factors)
  T va[16], vb[16];
};

// Double-float arithmetic (a value is an unevaluated sum hi + lo of two
// floats): Dekker's product with a fused multiply-add and Knuth's two-sum,
// about 48 significant bits on the FP32 pipe.
struct DF {
  float h, l;
};
__device__ __forceinline__ DF df_mul(float ah, float al, float bh, float bl) {
  const float p = ah * bh;
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, fmaf(al, bh, e));
  const float s = p + e;
  return {s, e - (s - p)};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  const float s = a.h + b.h;
  const float v = s - a.h;
  float e = (a.h - (s - v)) + (b.h - v);
  e += a.l + b.l;
  const float r = s + e;
  return {r, e - (r - s)};
}

// FP64 inverse blocks as (hi, lo) FP32 pairs: hi = fl32(d), lo = fl32(d - hi).
__global__ void split_df_kernel(const double* __restrict__ d, float2* __restrict__ out, long long n) {
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < n;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double v = d[t];
    const float h = static_cast<float>(v);
    out[t] = make_float2(h, static_cast<float>(v - static_cast<double>(h)));
  }
}

template <class T>
__device__ __forceinline__ void sweep_prefetch(const T* __restrict__ A, long long ld, const double* __restrict__ Dinv,
                                               const float2* __restrict__ Dinv2, const SweepStep& s,
                                               SweepPrefetch<T>& pf) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int quarter = warp & 3, half = warp >> 2;
  const size_t dofs = static_cast<size_t>(s.k) * TB * TB + static_cast<size_t>(warp) * 8 * TB;
  if constexpr (std::is_same<T, float>::value) {
    const float2* D = Dinv2 + dofs;
#pragma unroll
    for (int q = 0; q < 8; q++) {
      pf.dlo[q] = D[q * TB + lane];
      pf.dhi[q] = D[q * TB + lane + 32];
    }
  } else {
    const double* D = Dinv + dofs;
#pragma unroll
    for (int q = 0; q < 8; q++) {
      pf.lo[q] = D[q * TB + lane];
      pf.hi[q] = D[q * TB + lane + 32];
    }
  }
  const int c0 = quarter * 16;
  {
    const int t = s.first;
    const int row = t * SW_TILE + half * 32 + lane;
    const bool act = t < s.t1 && row >= s.q0 && row < s.q1;
    const T* a = A + static_cast<long long>(s.r0 + c0) * ld + row;
#pragma unroll
    for (int j = 0; j < 16; j++) pf.va[j] = (act && c0 + j < s.n) ? a[static_cast<long long>(j) * ld] : T(0);
  }
  {
    const int t = s.first + gridDim.x;
    const int row = t * SW_TILE + half * 32 + lane;
    const bool act = t < s.t1 && row >= s.q0 && row < s.q1;
    const T* a = A + static_cast<long long>(s.r0 + c0) * ld + row;
#pragma unroll
    for (int j = 0; j < 16; j++) pf.vb[j] = (act && c0 + j < s.n) ? a[static_cast<long long>(j) * ld] : T(0);
  }
}

// A whole triangular sweep with the factors in one cooperative launch: per
// 64-row block k (in order for L, reversed for U), every CTA forms
// x_k = Dinv_k b[block] in FP64 (Dinv_k row-major; warp w owns rows
// 8w..8w+7, lanes along the row), CTA 0 stores x_k in y, and the rows below
// (L) or above (U) get b[row] -= A(row, block) x_k; then one grid barrier.
// Rows go by 64-row tiles, tile t to CTA t % grid: within a CTA, warp w
// takes rows 32 (w >> 2) .. + 31 of the tile and the 16 block columns
// 16 (w & 3) .. + 15, and the four column quarters are added in shared
// memory.  Dinv_k and the block columns of the first two tiles are loaded
// a step ahead (before the barrier).  A row of b is only ever written by
// its tile's CTA; block rows written by other CTAs are read past L1.
template <class T>
__global__ void __launch_bounds__(256) trsv_sweep(const T* __restrict__ A, long long ld, int N, double* b,
                                                  double* __restrict__ y, const double* __restrict__ Dinv,
                                                  const float2* __restrict__ Dinv2, int lower, unsigned* bar,
                                                  int* err, unsigned long long wait_ns, unsigned stall) {
  // x_k = Dinv_k b in FP64, or in double-float with FP32 factors (an
  // explicit inverse amplifies rounding by its condition number, so a plain
  // FP32 product would cost refinement iterations); the row updates in the
  // factors' precision T
  __shared__ double bb[TB];
  __shared__ float bh[TB], bl[TB];
  __shared__ double xx[TB];
  __shared__ T xt[TB];
  __shared__ T part[4][SW_TILE];
  // The right-hand side of the rows this CTA updates (its tiles t with
  // t = blockIdx.x mod gridDim.x), kept in shared memory for the whole
  // sweep; a tile goes back to global memory when it is the next block.
  __shared__ double bown[SW_MAXT][SW_TILE];
  __shared__ int s_ok;
  const int nblk = (N + TB - 1) / TB;
  const int ntiles = (N + SW_TILE - 1) / SW_TILE;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int quarter = warp & 3, half = warp >> 2;
  const bool own = ntiles <= SW_MAXT * static_cast<int>(gridDim.x);
  if (own && tid < SW_TILE)
    for (int j = 0, t = blockIdx.x; t < ntiles; j++, t += gridDim.x) {
      const int r = t * SW_TILE + tid;
      bown[j][tid] = (r < N) ? b[r] : 0.0;
    }
  SweepPrefetch<T> pf;
  sweep_prefetch(A, ld, Dinv, Dinv2, sweep_step(0, nblk, N, lower, ntiles), pf);
  for (int step = 0; step < nblk; step++) {
    const SweepStep s = sweep_step(step, nblk, N, lower, ntiles);
    if (tid < TB) {
      const double v = (tid < s.n) ? __ldcg(b + s.r0 + tid) : 0.0;
      bb[tid] = v;
      const float h = static_cast<float>(v);
      bh[tid] = h;
      bl[tid] = static_cast<float>(v - static_cast<double>(h));
    }
    __syncthreads();
    if constexpr (std::is_same<T, float>::value) {
      const float b0h = bh[lane], b0l = bl[lane], b1h = bh[lane + 32], b1l = bl[lane + 32];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        DF p = df_add(df_mul(pf.dlo[q].x, pf.dlo[q].y, b0h, b0l), df_mul(pf.dhi[q].x, pf.dhi[q].y, b1h, b1l));
        for (int o = 16; o > 0; o >>= 1) {
          DF r;
          r.h = __shfl_xor_sync(0xffffffffu, p.h, o);
          r.l = __shfl_xor_sync(0xffffffffu, p.l, o);
          p = df_add(p, r);
        }
        if (lane == 0) {
          const double x = static_cast<double>(p.h) + static_cast<double>(p.l);
          xx[warp * 8 + q] = x;
          xt[warp * 8 + q] = static_cast<T>(x);
        }
      }
    } else {
      const double b0 = bb[lane], b1 = bb[lane + 32];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        double p = pf.lo[q] * b0 + pf.hi[q] * b1;
        for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
        if (lane == 0) {
          xx[warp * 8 + q] = p;
          xt[warp * 8 + q] = static_cast<T>(p);
        }
      }
    }
    __syncthreads();
    if (blockIdx.x == 0 && tid < s.n) y[s.r0 + tid] = xx[tid];
    const int c0 = quarter * 16;
    int tix = 0;
    for (int t = s.first; t < s.t1; t += gridDim.x, tix++) {
      const int row = t * SW_TILE + half * 32 + lane;
      T acc = T(0);
      if (tix == 0) {
#pragma unroll
        for (int j = 0; j < 16; j++) acc = fma(pf.va[j], xt[c0 + j], acc);
      } else if (tix == 1) {
#pragma unroll
        for (int j = 0; j < 16; j++) acc = fma(pf.vb[j], xt[c0 + j], acc);
      } else if (row >= s.q0 && row < s.q1) {
        const T* a = A + static_cast<long long>(s.r0 + c0) * ld + row;
        T v[16];
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = (c0 + j < s.n) ? a[static_cast<long long>(j) * ld] : T(0);
#pragma unroll
        for (int j = 0; j < 16; j++) acc = fma(v[j], xt[c0 + j], acc);
      }
      part[quarter][half * 32 + lane] = acc;
      __syncthreads();
      if (tid < SW_TILE) {
        const int r = t * SW_TILE + tid;
        if (r >= s.q0 && r < s.q1) {
          const double sub = static_cast<double>((part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]));
          if (own) {
            const int j = (t - static_cast<int>(blockIdx.x)) / static_cast<int>(gridDim.x);
            const double v = bown[j][tid] - sub;
            bown[j][tid] = v;
            // the next block in sweep order reads its rows from global memory
            if (t == (lower ? s.k + 1 : s.k - 1)) b[r] = v;
          } else {
            b[r] = __ldcg(b + r) - sub;
          }
        }
      }
      __syncthreads();
    }
    if (step + 1 < nblk) sweep_prefetch(A, ld, Dinv, Dinv2, sweep_step(step + 1, nblk, N, lower, ntiles), pf);
    if (!grid_barrier(bar, gridDim.x * static_cast<unsigned>(step + 1) + stall, err, &s_ok, wait_ns)) return;
  }
}

// ---- triangular sweeps that pull finished blocks (no grid barrier) --------
// Block k of the solution, x_k = Dinv_k (b_k - sum_i T_ki x_i) over the
// blocks i before k in sweep order (T = L forward, U backward).  CTA c owns
// the blocks at sweep positions c, c + G, ... (G = gridDim.x, every CTA
// resident: cooperative launch).  A CTA accumulates the products of its
// block's rows with every finished x_i as soon as that block is done, so
// only the last product and the Dinv_k product remain on the critical path
// once x_{k-1} appears.  Finished blocks are announced through one progress
// counter (release max by the producer, acquire loads by the consumers),
// the number of sweep positions whose x is in y.  Thread (warp w, lane):
// row h*32 + lane of the block (h = w >> 2), columns 16 q .. 16 q + 15
// (q = w & 3) of each contributing block; products in the factors'
// precision T, 16 at a time, summed in FP64.  Every wait is bounded by
// wait_ns: on timeout the CTA sets *err and leaves.
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Waits until *progress >= target; returns the value seen, or 0 on timeout.
__device__ __forceinline__ unsigned wait_progress(const unsigned* progress, unsigned target,
                                                  unsigned long long wait_ns) {
  unsigned v = ld_acquire_u32(progress);
  if (v >= target) return v;
  const unsigned long long t0 = globaltimer_ns();
  for (unsigned it = 0;; it++) {
    __nanosleep(32);
    v = ld_acquire_u32(progress);
    if (v >= target) return v;
    if ((it & 15) == 15 && globaltimer_ns() - t0 > wait_ns) return 0;
  }
}

template <class T>
__global__ void __launch_bounds__(256) trsv_pull(const T* __restrict__ A, long long ld, int N,
                                                 const double* __restrict__ b, double* __restrict__ y,
                                                 const double* __restrict__ Dinv, const float2* __restrict__ Dinv2,
                                                 int lower, unsigned* progress, int* err,
                                                 unsigned long long wait_ns, unsigned stall) {
  __shared__ double part[4][TB];
  __shared__ float vh[TB], vl[TB];
  __shared__ double vd[TB];
  __shared__ int s_abort;
  const int nblk = (N + TB - 1) / TB;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int q = warp & 3, h = warp >> 2;
  const int rr = h * 32 + lane;  // row within the block
  const int c0 = q * 16;
  if (tid == 0) s_abort = 0;
  __syncthreads();
  unsigned avail = 0;  // sweep positions known finished
  for (int p = blockIdx.x; p < nblk; p += gridDim.x) {
    const int k = lower ? p : nblk - 1 - p;
    const int r0 = k * TB;
    const int n = (N - r0 < TB) ? N - r0 : TB;
    const int row = r0 + rr;
    // this warp's 8 rows of Dinv_k, loaded before any wait
    float2 dlo[8], dhi[8];
    double lo[8], hi[8];
    const size_t dofs = static_cast<size_t>(k) * TB * TB + static_cast<size_t>(warp) * 8 * TB;
    if constexpr (std::is_same<T, float>::value) {
#pragma unroll
      for (int j = 0; j < 8; j++) {
        dlo[j] = Dinv2[dofs + j * TB + lane];
        dhi[j] = Dinv2[dofs + j * TB + lane + 32];
      }
    } else {
#pragma unroll
      for (int j = 0; j < 8; j++) {
        lo[j] = Dinv[dofs + j * TB + lane];
        hi[j] = Dinv[dofs + j * TB + lane + 32];
      }
    }
    double acc = 0.0;
    bool ok = true;
    for (int pi = 0; pi < p; pi++) {
      const int i = lower ? pi : nblk - 1 - pi;
      const int cb = i * TB + c0;  // first column of this thread's quarter
      T a[16];
#pragma unroll
      for (int j = 0; j < 16; j++)
        a[j] = (row < N && cb + j < N) ? A[static_cast<long long>(cb + j) * ld + row] : T(0);
      if (static_cast<unsigned>(pi) >= avail) {
        const unsigned v = wait_progress(progress, static_cast<unsigned>(pi) + 1 + stall, wait_ns);
        if (v == 0) {
          ok = false;
          break;
        }
        avail = v - stall;  // positions known finished
      }
      T sum = T(0);
#pragma unroll
      for (int j = 0; j < 16; j++) {
        const double xj = (cb + j < N) ? __ldcg(y + cb + j) : 0.0;
        sum = fma(a[j], static_cast<T>(xj), sum);
      }
      acc += static_cast<double>(sum);
    }
    if (!ok) s_abort = 1;
    part[q][rr] = acc;
    __syncthreads();
    if (s_abort) {
      if (tid == 0) atomicExch(err, 1);
      return;
    }
    if (tid < TB) {
      const double v = (tid < n) ? b[r0 + tid] - ((part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]))
                                 : 0.0;
      vd[tid] = v;
      const float hv = static_cast<float>(v);
      vh[tid] = hv;
      vl[tid] = static_cast<float>(v - static_cast<double>(hv));
    }
    __syncthreads();
    // x_k = Dinv_k v: warp w computes rows 8 w .. 8 w + 7
    if constexpr (std::is_same<T, float>::value) {
      const float b0h = vh[lane], b0l = vl[lane], b1h = vh[lane + 32], b1l = vl[lane + 32];
#pragma unroll
      for (int j = 0; j < 8; j++) {
        DF pr = df_add(df_mul(dlo[j].x, dlo[j].y, b0h, b0l), df_mul(dhi[j].x, dhi[j].y, b1h, b1l));
        for (int o = 16; o > 0; o >>= 1) {
          DF r;
          r.h = __shfl_xor_sync(0xffffffffu, pr.h, o);
          r.l = __shfl_xor_sync(0xffffffffu, pr.l, o);
          pr = df_add(pr, r);
        }
        const int xr = warp * 8 + j;
        if (lane == 0 && xr < n) y[r0 + xr] = static_cast<double>(pr.h) + static_cast<double>(pr.l);
      }
    } else {
      const double b0 = vd[lane], b1 = vd[lane + 32];
#pragma unroll
      for (int j = 0; j < 8; j++) {
        double pr = lo[j] * b0 + hi[j] * b1;
        for (int o = 16; o > 0; o >>= 1) pr += __shfl_xor_sync(0xffffffffu, pr, o);
        const int xr = warp * 8 + j;
        if (lane == 0 && xr < n) y[r0 + xr] = pr;
      }
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      asm volatile("red.release.gpu.global.max.u32 [%0], %1;" ::"l"(progress), "r"(static_cast<unsigned>(p) + 1)
                   : "memory");
    }
  }
}

// The same sweep with CH_R consecutive blocks per CTA: CTA c owns sweep
// positions c R .. c R + R - 1.  While earlier CTAs work it accumulates, for
// all its blocks at once, the products with every finished x (phase A, one
// progress wait per finished block).  Its own blocks then chain inside the
// CTA (phase B): x_p from the accumulated rows and Dinv, published, and its
// products with the CTA's later blocks from the internal L blocks, which
// were staged in shared memory before phase A.  Only ceil(nblk / R)
// hand-offs between CTAs remain on the critical path.
constexpr int CH_R = 3;
constexpr int CH_DST = TB + 1;  // row stride of the staged Dinv blocks (8-byte entries: conflict-free row reads)
// dynamic shared memory: the internal L blocks, then Dinv of the own blocks
// (8 bytes an entry: a (hi, lo) float pair or a double)
template <class T>
constexpr size_t chain_smem() {
  return static_cast<size_t>(CH_R * (CH_R - 1) / 2) * TB * TB * sizeof(T) +
         static_cast<size_t>(CH_R) * TB * CH_DST * 8;
}

// With FP32 factors every value a thread multiplies is a float: the
// producer stores x twice (y in FP64, yf in FP32), phase A and the internal
// products read the FP32 copy, and the sums go in double-float.  (On this
// GPU FP64 adds and FP64 <-> FP32 conversions run at the FP64 rate, a few
// per clock per SM: one conversion per product would cost more than the
// products.)
template <class T>
__global__ void __launch_bounds__(256) trsv_chain(const T* __restrict__ A, long long ld, int N,
                                                  const double* __restrict__ b, double* __restrict__ y,
                                                  float* __restrict__ yf, const double* __restrict__ Dinv,
                                                  const float2* __restrict__ Dinv2, int lower, unsigned* progress,
                                                  int* err, unsigned long long wait_ns, unsigned stall) {
  constexpr bool kF = std::is_same<T, float>::value;
  extern __shared__ __align__(16) unsigned char ch_raw[];
  T* Lin = reinterpret_cast<T*>(ch_raw);  // internal blocks (r2, r1), r1 < r2: column-major 64 x 64
  // Dinv of the own blocks, row-major 64 x 64 each with row stride CH_DST
  unsigned char* dsm = ch_raw + static_cast<size_t>(CH_R * (CH_R - 1) / 2) * TB * TB * sizeof(T);
  float2* D2s = reinterpret_cast<float2*>(dsm);
  double* Dds = reinterpret_cast<double*>(dsm);
  __shared__ double bsm[CH_R][TB];
  __shared__ double part[4][TB];
  __shared__ float parth[4][TB], partl[4][TB];
  __shared__ float vh[TB], vl[TB];
  __shared__ double vd[TB];
  __shared__ double xs[TB];
  __shared__ float xsf[TB];
  __shared__ int s_abort;
  const int nblk = (N + TB - 1) / TB;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int q = warp & 3, h = warp >> 2;
  const int rr = h * 32 + lane;
  const int c0 = q * 16;
  const int p0 = blockIdx.x * CH_R;
  const int np = (nblk - p0 < CH_R) ? nblk - p0 : CH_R;
  auto blk = [&](int pos) { return lower ? pos : nblk - 1 - pos; };
  auto tri = [](int r2, int r1) { return r2 * (r2 - 1) / 2 + r1; };  // index of block (r2, r1), r1 < r2
  if (tid == 0) s_abort = 0;
  // Stage what the own blocks need besides the x of earlier blocks: the
  // internal L blocks (rows of position p0 + r2, columns of p0 + r1), the
  // Dinv blocks and the right-hand side, 16 independent loads in flight
  // per thread.
  for (int r2 = 1; r2 < np; r2++)
    for (int r1 = 0; r1 < r2; r1++) {
      const int kr = blk(p0 + r2), kc = blk(p0 + r1);
      T* dst = Lin + static_cast<size_t>(tri(r2, r1)) * TB * TB;
      for (int e0 = 0; e0 < TB * TB; e0 += 16 * 256) {
        T v[16];
#pragma unroll
        for (int u = 0; u < 16; u++) {
          const int e = e0 + u * 256 + tid;
          const int row = kr * TB + e % TB, col = kc * TB + e / TB;
          v[u] = (row < N && col < N) ? A[static_cast<long long>(col) * ld + row] : T(0);
        }
#pragma unroll
        for (int u = 0; u < 16; u++) dst[e0 + u * 256 + tid] = v[u];  // dst[j * TB + i], e = j * TB + i
      }
    }
  for (int r = 0; r < np; r++) {
    const size_t src = static_cast<size_t>(blk(p0 + r)) * TB * TB;
    for (int e0 = 0; e0 < TB * TB; e0 += 16 * 256) {
      // entry e = row * TB + col of the block goes to row * CH_DST + col
      if constexpr (std::is_same<T, float>::value) {
        float2 v[16];
#pragma unroll
        for (int u = 0; u < 16; u++) v[u] = Dinv2[src + e0 + u * 256 + tid];
#pragma unroll
        for (int u = 0; u < 16; u++) {
          const int e = e0 + u * 256 + tid;
          D2s[static_cast<size_t>(r) * TB * CH_DST + (e / TB) * CH_DST + e % TB] = v[u];
        }
      } else {
        double v[16];
#pragma unroll
        for (int u = 0; u < 16; u++) v[u] = Dinv[src + e0 + u * 256 + tid];
#pragma unroll
        for (int u = 0; u < 16; u++) {
          const int e = e0 + u * 256 + tid;
          Dds[static_cast<size_t>(r) * TB * CH_DST + (e / TB) * CH_DST + e % TB] = v[u];
        }
      }
    }
    if (tid < TB) {
      const int row = blk(p0 + r) * TB + tid;
      bsm[r][tid] = (row < N) ? b[row] : 0.0;
    }
  }
  __syncthreads();
  double acc[CH_R];  // FP64 factors
  DF accf[CH_R];     // FP32 factors
#pragma unroll
  for (int r = 0; r < CH_R; r++) {
    acc[r] = 0.0;
    accf[r] = {0.f, 0.f};
  }
  // phase A: the finished blocks of earlier CTAs.  With FP32 factors the L
  // tile of the next block is loaded while the current one is used (it
  // does not depend on x), so the factor's HBM latency overlaps the
  // progress waits and the x loads.
  unsigned avail = 0;
  bool ok = true;
  constexpr bool kAhead = sizeof(T) == 4;  // FP64 tiles would not fit twice in registers
  T a[CH_R][16], an[kAhead ? CH_R : 1][16];
  // 16-byte vector loads of x only from an aligned y (callers pass offset
  // vectors, e.g. a work vector at an odd offset N)
  const bool y_aligned = (reinterpret_cast<unsigned long long>(y) & 15ull) == 0;
  const bool yf_aligned = kF && (reinterpret_cast<unsigned long long>(yf) & 15ull) == 0;
  // rows of this thread in its CTA's blocks (N when past the matrix)
  int rowof[CH_R];
#pragma unroll
  for (int r = 0; r < CH_R; r++) {
    const int row = blk(p0 + r) * TB + rr;
    rowof[r] = (r < np && row < N) ? row : N;
  }
  auto load_tile = [&](int pi, T(&dst)[CH_R][16]) {
    const int cb = blk(pi) * TB + c0;
    const T* colp = A + static_cast<long long>(cb) * ld;
    if (cb + 16 <= N) {  // whole column quarter inside the matrix: no column predicates
#pragma unroll
      for (int r = 0; r < CH_R; r++) {
        if (rowof[r] < N) {
          const T* q = colp + rowof[r];
#pragma unroll
          for (int j = 0; j < 16; j++) {
            dst[r][j] = *q;
            q += ld;
          }
        } else {
#pragma unroll
          for (int j = 0; j < 16; j++) dst[r][j] = T(0);
        }
      }
    } else {
#pragma unroll
      for (int r = 0; r < CH_R; r++)
#pragma unroll
        for (int j = 0; j < 16; j++)
          dst[r][j] = (rowof[r] < N && cb + j < N) ? colp[static_cast<long long>(j) * ld + rowof[r]] : T(0);
    }
  };
  if constexpr (kAhead) {
    if (p0 > 0) load_tile(0, an);
  }
  for (int pi = 0; pi < p0; pi++) {
    const int cb = blk(pi) * TB + c0;
    if constexpr (kAhead) {
#pragma unroll
      for (int r = 0; r < CH_R; r++)
#pragma unroll
        for (int j = 0; j < 16; j++) a[r][j] = an[r][j];
      if (pi + 1 < p0) load_tile(pi + 1, an);
    } else {
      load_tile(pi, a);
    }
    if (static_cast<unsigned>(pi) >= avail) {
      const unsigned v = wait_progress(progress, static_cast<unsigned>(pi) + 1 + stall, wait_ns);
      if (v == 0) {
        ok = false;
        break;
      }
      avail = v - stall;  // positions known finished
    }
    T xq[16];
    if constexpr (kF) {
      if (yf_aligned && cb + 16 <= N) {  // yf + cb is then 16-byte aligned (cb is a multiple of 16)
        const float4* y4 = reinterpret_cast<const float4*>(yf + cb);
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const float4 v = __ldcg(y4 + j);
          xq[4 * j] = v.x;
          xq[4 * j + 1] = v.y;
          xq[4 * j + 2] = v.z;
          xq[4 * j + 3] = v.w;
        }
      } else {
#pragma unroll
        for (int j = 0; j < 16; j++) xq[j] = (cb + j < N) ? __ldcg(yf + cb + j) : 0.f;
      }
    } else if (y_aligned && cb + 16 <= N) {  // y + cb is then 16-byte aligned (cb is a multiple of 16)
      const double2* y2 = reinterpret_cast<const double2*>(y + cb);
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const double2 v = __ldcg(y2 + j);
        xq[2 * j] = static_cast<T>(v.x);
        xq[2 * j + 1] = static_cast<T>(v.y);
      }
    } else {
#pragma unroll
      for (int j = 0; j < 16; j++) xq[j] = static_cast<T>((cb + j < N) ? __ldcg(y + cb + j) : 0.0);
    }
#pragma unroll
    for (int r = 0; r < CH_R; r++) {
      T sum = T(0);
#pragma unroll
      for (int j = 0; j < 16; j++) sum = fma(a[r][j], xq[j], sum);
      if constexpr (kF) {
        accf[r] = df_add(accf[r], {static_cast<float>(sum), 0.f});
      } else {
        acc[r] += static_cast<double>(sum);
      }
    }
  }
  if (!ok) s_abort = 1;
  // phase B: this CTA's own blocks, chained in shared memory
#pragma unroll
  for (int r = 0; r < CH_R; r++) {
    if (r >= np) break;
    const int k = blk(p0 + r);
    const int r0 = k * TB;
    const int n = (N - r0 < TB) ? N - r0 : TB;
    if constexpr (kF) {
      parth[q][rr] = accf[r].h;
      partl[q][rr] = accf[r].l;
    } else {
      part[q][rr] = acc[r];
    }
    __syncthreads();
    if (s_abort) {
      if (tid == 0) atomicExch(err, 1);
      return;
    }
    if (tid < TB) {
      double sacc;
      if constexpr (kF) {
        const DF a = df_add({parth[0][tid], partl[0][tid]}, {parth[1][tid], partl[1][tid]});
        const DF c = df_add({parth[2][tid], partl[2][tid]}, {parth[3][tid], partl[3][tid]});
        const DF t = df_add(a, c);
        sacc = static_cast<double>(t.h) + static_cast<double>(t.l);
      } else {
        sacc = (part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]);
      }
      const double v = (tid < n) ? bsm[r][tid] - sacc : 0.0;
      vd[tid] = v;
      const float hv = static_cast<float>(v);
      vh[tid] = hv;
      vl[tid] = static_cast<float>(v - static_cast<double>(hv));
    }
    __syncthreads();
    // x = Dinv v: thread (h, q, lane) forms row rr over columns c0 .. c0 + 15
    // (two accumulators), the four column quarters are added in shared
    // memory in a fixed order
    const size_t drow = static_cast<size_t>(r) * TB * CH_DST + static_cast<size_t>(rr) * CH_DST + c0;
    if constexpr (std::is_same<T, float>::value) {
      DF s0 = {0.f, 0.f}, s1 = {0.f, 0.f};
#pragma unroll
      for (int j = 0; j < 16; j += 2) {
        const float2 d0 = D2s[drow + j], d1 = D2s[drow + j + 1];
        s0 = df_add(s0, df_mul(d0.x, d0.y, vh[c0 + j], vl[c0 + j]));
        s1 = df_add(s1, df_mul(d1.x, d1.y, vh[c0 + j + 1], vl[c0 + j + 1]));
      }
      const DF sq = df_add(s0, s1);
      parth[q][rr] = sq.h;
      partl[q][rr] = sq.l;
    } else {
      double s0 = 0.0, s1 = 0.0;
#pragma unroll
      for (int j = 0; j < 16; j += 2) {
        s0 = fma(Dds[drow + j], vd[c0 + j], s0);
        s1 = fma(Dds[drow + j + 1], vd[c0 + j + 1], s1);
      }
      part[q][rr] = s0 + s1;
    }
    __syncthreads();
    if (tid < TB) {
      double x;
      if constexpr (std::is_same<T, float>::value) {
        const DF a = df_add({parth[0][tid], partl[0][tid]}, {parth[1][tid], partl[1][tid]});
        const DF c = df_add({parth[2][tid], partl[2][tid]}, {parth[3][tid], partl[3][tid]});
        const DF t = df_add(a, c);
        x = static_cast<double>(t.h) + static_cast<double>(t.l);
      } else {
        x = (part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]);
      }
      if (tid >= n) x = 0.0;
      xs[tid] = x;
      if (tid < n) y[r0 + tid] = x;
      if constexpr (kF) {
        const float xf = static_cast<float>(x);
        xsf[tid] = xf;
        if (tid < n) yf[r0 + tid] = xf;
      }
    }
    __syncthreads();
    // release after the block barrier: the barrier orders every thread's
    // store of x before thread 0's release (no separate fence)
    if (tid == 0)
      asm volatile("red.release.gpu.global.max.u32 [%0], %1;" ::"l"(progress), "r"(static_cast<unsigned>(p0 + r) + 1)
                   : "memory");
    // products of the later own blocks with x_p
#pragma unroll
    for (int r2 = r + 1; r2 < CH_R; r2++) {
      if (r2 >= np) break;
      const T* L = Lin + static_cast<size_t>(tri(r2, r)) * TB * TB;
      T sum = T(0);
      if constexpr (kF) {
#pragma unroll
        for (int j = 0; j < 16; j++) sum = fmaf(L[(c0 + j) * TB + rr], xsf[c0 + j], sum);
        accf[r2] = df_add(accf[r2], {sum, 0.f});
      } else {
#pragma unroll
        for (int j = 0; j < 16; j++) sum = fma(L[(c0 + j) * TB + rr], static_cast<T>(xs[c0 + j]), sum);
        acc[r2] += static_cast<double>(sum);
      }
    }
  }
}

template <class T>
__global__ void __launch_bounds__(GP_THREADS) panel_grid_kernel(T* __restrict__ A, long long ld, int N, int j0, int jb,
                                                                int per, int* __restrict__ ipiv,
                                                                int* __restrict__ info, PanelSlots<T> ps) {
  extern __shared__ __align__(16) unsigned char gp_raw[];
  T* tile = reinterpret_cast<T*>(gp_raw);
  __shared__ T prow[128];
  __shared__ T rv[GP_THREADS / 32];
  __shared__ int ri[GP_THREADS / 32], rt[GP_THREADS / 32];
  __shared__ int s_ok;
  const int nblk = gridDim.x, b = blockIdx.x, tid = threadIdx.x, bd = blockDim.x;
  const int r0 = j0 + b * per;
  const int r1 = (r0 + per < N) ? r0 + per : N;
  const int nr = r1 - r0;
  for (int e = tid; e < jb * nr; e += bd) {
    int k = e / nr, r = e % nr;
    tile[k * per + r] = A[static_cast<long long>(j0 + k) * ld + r0 + r];
  }
  __syncthreads();
  for (int jj = 0; jj < jb; jj++) {
    const int j = j0 + jj;
    const int slot = jj & 1;
    // 1. local candidate
    T best = T(-1);
    int bi = N, tag = 0;
    for (int i = (r0 > j ? r0 : j) + tid; i < r1; i += bd) {
      T v = fabs(tile[jj * per + i - r0]);
      if (better(v, i, best, bi)) {
        best = v;
        bi = i;
      }
    }
    block_argmax(best, bi, tag, rv, ri, rt);
    // 2. publish it (and row j when this CTA owns it)
    T* mine = ps.cand_rows + (static_cast<size_t>(slot) * nblk + b) * jb;
    if (bi < N)
      for (int k = tid; k < jb; k += bd) mine[k] = tile[k * per + bi - r0];
    if (tid == 0) {
      ps.cand_v[slot * nblk + b] = static_cast<double>(best);
      ps.cand_i[slot * nblk + b] = bi;
    }
    if (j >= r0 && j < r1)
      for (int k = tid; k < jb; k += bd) ps.jrow[slot * jb + k] = tile[k * per + j - r0];
    // 3. one barrier per column
    if (!grid_barrier(ps.bar, static_cast<unsigned>(nblk) * (jj + 1) + ps.stall, ps.err, &s_ok, ps.wait_ns)) return;
    // 4. every CTA reduces the candidates identically
    best = T(-1);
    bi = N;
    tag = -1;
    for (int t = tid; t < nblk; t += bd) {
      T v = static_cast<T>(__ldcg(ps.cand_v + slot * nblk + t));
      int ii = __ldcg(ps.cand_i + slot * nblk + t);
      if (better(v, ii, best, bi)) {
        best = v;
        bi = ii;
        tag = t;
      }
    }
    block_argmax(best, bi, tag, rv, ri, rt);
    int gi = bi;
    if (gi >= N) {  // nothing usable below the diagonal: no swap
      gi = j;
      tag = -1;
    }
    if (b == 0 && tid == 0) {
      ipiv[j] = gi;
      if (!(best > T(0)) && *info == 0) *info = j + 1;  // zero (or NaN) pivot
    }
    // 5. pivot row, row exchange
    const T* src = (tag >= 0) ? ps.cand_rows + (static_cast<size_t>(slot) * nblk + tag) * jb : ps.jrow + slot * jb;
    for (int k = tid; k < jb; k += bd) prow[k] = __ldcg(src + k);
    if (gi != j && gi >= r0 && gi < r1)
      for (int k = tid; k < jb; k += bd) tile[k * per + gi - r0] = __ldcg(ps.jrow + slot * jb + k);
    __syncthreads();
    if (j >= r0 && j < r1)
      for (int k = tid; k < jb; k += bd) tile[k * per + j - r0] = prow[k];
    // 6. scale the column below the pivot, rank-1 update of the rest
    const T piv = prow[jj];
    const int rs = (r0 > j + 1) ? r0 : j + 1;
    __syncthreads();
    if (piv != T(0) && rs < r1) {
      const T inv = T(1) / piv;
      for (int i = rs + tid; i < r1; i += bd) tile[jj * per + i - r0] *= inv;
      __syncthreads();
      // thread -> (row, column phase): rows along the low 7 bits (conflict-free
      // shared memory), columns strided by the number of phases
      const int nrr = r1 - rs;
      const int nph = bd >> 7, ph = tid >> 7;
      for (int i0 = 0; i0 < nrr; i0 += 128) {
        const int ii = i0 + (tid & 127);
        if (ii < nrr) {
          const int li = rs - r0 + ii;
          const T l = tile[jj * per + li];
          for (int k = jj + 1 + ph; k < jb; k += nph)
            tile[k * per + li] = fma(-l, prow[k], tile[k * per + li]);
        }
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < jb * nr; e += bd) {
    int k = e / nr, r = e % nr;
    A[static_cast<long long>(j0 + k) * ld + r0 + r] = tile[k * per + r];
  }
}

// The row exchanges of one panel (pivots piv[0 .. jb), rows j0 .. ) as a
// list of moves row dst[t] <- row src[t] over the rows they touch (at most
// 2 jb): rows j0 .. j0+jb-1 first, then the pivot rows below the panel in
// order of first appearance.  One warp: lane 0 replays the exchanges with
// the rows below the panel found through a small hash table.  piv, rows
// (2 jb), content (2 jb), hkey and hidx (256 each) and cnt in shared memory.
// map[0] = count, map[1 .. 1+2jb) = dst, map[1+2jb .. 1+4jb) = src.
constexpr int SWAP_HASH = 256;
__device__ void swap_map_warp(const int* piv, int j0, int jb, int* __restrict__ map, int* rows, int* content,
                              int* hkey, int* hidx, int* cnt_s) {
  const int lane = threadIdx.x & 31;
  for (int t = lane; t < jb; t += 32) {
    rows[t] = j0 + t;
    content[t] = j0 + t;
  }
  for (int t = lane; t < SWAP_HASH; t += 32) hkey[t] = -1;
  __syncwarp();
  if (lane == 0) {
    int cnt = jb;
    for (int jj = 0; jj < jb; jj++) {
      const int p = piv[jj];
      int idx;
      if (p < j0 + jb) {
        idx = p - j0;
      } else {
        unsigned h = (static_cast<unsigned>(p) * 2654435761u) >> 24;  // 8 bits
        while (hkey[h] != -1 && hkey[h] != p) h = (h + 1) & (SWAP_HASH - 1);
        if (hkey[h] == p) {
          idx = hidx[h];
        } else {
          idx = cnt++;
          hkey[h] = p;
          hidx[h] = idx;
          rows[idx] = p;
          content[idx] = p;
        }
      }
      const int t = content[jj];
      content[jj] = content[idx];
      content[idx] = t;
    }
    *cnt_s = cnt;
  }
  __syncwarp();
  const int n = *cnt_s;
  for (int t = lane; t < n; t += 32) {
    map[1 + t] = rows[t];
    map[1 + 2 * jb + t] = content[t];
  }
  if (lane == 0) map[0] = n;
}

__global__ void build_swap_map(const int* __restrict__ ipiv, int j0, int jb, int* __restrict__ map) {
  __shared__ int rows[256], content[256], piv[128], hkey[SWAP_HASH], hidx[SWAP_HASH];
  __shared__ int cnt;
  for (int t = threadIdx.x; t < jb; t += 32) piv[t] = ipiv[j0 + t];
  __syncwarp();
  swap_map_warp(piv, j0, jb, map, rows, content, hkey, hidx, &cnt);
}

// ---- panel on one 16-CTA cluster (FP32 factors) --------------------------
// The same algorithm as panel_grid_kernel with the exchange in distributed
// shared memory: CTA r of the cluster keeps rows [j0 + r*per, ...) of the
// panel in its shared memory, row by row (stride cp_row_stride(jb) floats,
// so that a row's 16-column inner block is four aligned 128-bit words and
// eight consecutive rows hit distinct banks).  Per column, one block
// barrier and one cluster barrier:
//  - every thread already holds its best candidate for the column (found
//    while updating it in the previous column step); a warp reduction and
//    one block barrier give the CTA's candidate;
//  - warp 0 pushes (value, row, the row's inner block) into every CTA's
//    receive slot, and warp 1 of the owner of row j pushes row j's inner
//    block; the CTA keeps its candidate's full row and row j locally;
//  - after the cluster barrier every warp picks the winner from its own
//    receive slot (same order everywhere); each thread then swaps, scales
//    and updates the inner block of its rows in registers and tracks its
//    candidate for column j + 1, all in one pass;
//  - the other columns of the two swapped rows are fetched from the owners'
//    shared memory off the critical path (they are read again only after
//    the next cluster barrier).
// Receive slots, candidate rows and row j are double-buffered by column
// parity: a CTA can only overwrite a slot after every CTA has passed the
// next cluster barrier, i.e. has finished reading it.
constexpr int CP_CL = 16;
constexpr int CP_THREADS = 384;  // 251 rows per CTA and warp-level reductions over 12 warps (512 and 768 were slower)
constexpr int CP_WARPS = CP_THREADS / 32;
constexpr size_t CP_MAX_SMEM = 212 * 1024;
constexpr int CP_IB = 16;  // inner block: columns updated per column step

// Row stride (floats) of the panel in shared memory: whole 16-column inner
// blocks plus 4, i.e. an odd number of 16-byte words.
__host__ __device__ constexpr int cp_row_stride(int jb) { return ((jb + 15) / 16) * 16 + 4; }

struct CpSlot {
  float4 seg[CP_CL][CP_IB / 4];  // candidate rows' inner blocks, by source CTA
  float4 jseg[CP_IB / 4];        // row j's inner block
  float v[CP_CL];                // candidate |values|, by source CTA
  int i[CP_CL];                  // candidate rows (N: none), by source CTA
};

// One column step on this thread's rows of the inner block, for column Q0
// of the block: swap (row j <- pivot row, row gi <- row j), scale column
// Q0, update columns Q0+1..15, and the thread's candidate for column Q0+1.
// Q0 is a template parameter so that the column selections cost nothing.
template <int Q0>
__device__ __forceinline__ void cp_column_step(float* __restrict__ tile, int S, int b0, int r0, int nr, int j, int gi,
                                               int nb, const float (&ps)[CP_IB], const float4* jseg4, float inv,
                                               bool nonzero, int N, float& best, int& bi) {
  best = -1.0f;
  bi = N;
  for (int li = threadIdx.x; li < nr; li += blockDim.x) {
    const int i = r0 + li;
    if (i < j) continue;
    float4* row = reinterpret_cast<float4*>(tile + static_cast<size_t>(li) * S + b0);
    if (i == j) {  // row j becomes the pivot row (inner block)
#pragma unroll
      for (int c = 0; c < CP_IB / 4; c++) row[c] = make_float4(ps[4 * c], ps[4 * c + 1], ps[4 * c + 2], ps[4 * c + 3]);
      continue;
    }
    // the row's inner block in registers (row gi takes row j's)
    const float4* in = (i == gi) ? jseg4 : row;
    float t[CP_IB];
#pragma unroll
    for (int c = 0; c < CP_IB / 4; c++) {
      const float4 x = in[c];
      t[4 * c] = x.x;
      t[4 * c + 1] = x.y;
      t[4 * c + 2] = x.z;
      t[4 * c + 3] = x.w;
    }
    if (nonzero) {
      const float l = t[Q0] * inv;
      t[Q0] = l;
#pragma unroll
      for (int q = Q0 + 1; q < CP_IB; q++) t[q] = fmaf(-l, ps[q], t[q]);
    }
    if (Q0 + 1 < CP_IB && Q0 + 1 < nb) {
      const float v = fabsf(t[(Q0 + 1) % CP_IB]);
      if (better(v, i, best, bi)) {
        best = v;
        bi = i;
      }
    }
    // columns before Q0 only change in the swapped rows
    constexpr int cfirst = Q0 / 4;
    const int cstart = (i == gi) ? 0 : cfirst;
#pragma unroll
    for (int c = 0; c < CP_IB / 4; c++)
      if (c >= cstart) row[c] = make_float4(t[4 * c], t[4 * c + 1], t[4 * c + 2], t[4 * c + 3]);
  }
}

// The per-column exchange of the cluster panel: each CTA's candidate (and the
// owner's row j) go to every CTA's receive slot by st.async, which completes
// on that CTA's mbarrier for the slot (its complete-tx has release semantics
// at cluster scope); a CTA waits on its own mbarrier (acquire at cluster
// scope), bounded by wait_ns.  False (and *err set) when the wait ran out.
__device__ __forceinline__ unsigned cp_smem(const void* p) { return static_cast<unsigned>(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ unsigned cp_mapa(unsigned a, unsigned rank) {
  unsigned d;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(rank));
  return d;
}
__device__ __forceinline__ void cp_push4(unsigned dst, float4 v, unsigned bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(dst),
               "r"(__float_as_uint(v.x)), "r"(__float_as_uint(v.y)), "r"(__float_as_uint(v.z)),
               "r"(__float_as_uint(v.w)), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void cp_push1(unsigned dst, unsigned v, unsigned bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];" ::"r"(dst), "r"(v), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void cp_arm(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(cp_smem(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool cp_wait(unsigned long long* bar, unsigned parity, unsigned long long wait_ns,
                                        int* err) {
  const unsigned a = cp_smem(bar);
  unsigned long long t0 = 0;
  for (int spin = 0;; spin++) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\tselp.u32 "
        "%0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
    if (spin == 0) {
      t0 = globaltimer_ns();
    } else if ((spin & 15) == 0 && globaltimer_ns() - t0 > wait_ns) {
      atomicExch(err, 1);
      return false;
    }
  }
}

__global__ void __launch_bounds__(CP_THREADS) panel_cluster16_kernel(float* __restrict__ A, long long ld, int N,
                                                                     int j0, int jb, int per,
                                                                     int* __restrict__ ipiv,
                                                                     int* __restrict__ info,
                                                                     int* __restrict__ swap_map,
                                                                     int* __restrict__ err,
                                                                     unsigned long long wait_ns, unsigned stall) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char cp_raw[];
  float* tile = reinterpret_cast<float*>(cp_raw);  // tile[r * S + k]
  __shared__ int pivs[128];  // the panel's pivots (CTA 0)
  __shared__ __align__(16) float cand_row[2][128];
  __shared__ __align__(16) float jrow[2][128];
  __shared__ __align__(16) CpSlot recv[2];
  __shared__ __align__(16) float ublk[CP_IB][128];  // rows of the current inner block (L11 | A12 -> U12)
  __shared__ float wv[CP_WARPS];
  __shared__ int wi[CP_WARPS];
  __shared__ __align__(8) unsigned long long xmb[2];  // the exchange's mbarriers, one per receive slot
  const int S = cp_row_stride(jb);
  const int rank = static_cast<int>(cluster.block_rank());
  const int ncl = static_cast<int>(cluster.num_blocks());  // 2, 4, 8 or 16 CTAs
  const int tid = threadIdx.x, bd = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int r0 = j0 + rank * per;
  const int r1 = (r0 + per < N) ? r0 + per : N;
  const int nr = r1 > r0 ? r1 - r0 : 0;
  for (int e = tid; e < jb * nr; e += bd) {
    int k = e / nr, r = e % nr;
    tile[r * S + k] = A[static_cast<long long>(j0 + k) * ld + r0 + r];
  }
  // bytes one column's exchange brings to each CTA: every CTA's candidate
  // (its 16-column segment, value and row) and the owner's segment of row j;
  // stall_waits asks for bytes that never come
  const unsigned xbytes = static_cast<unsigned>(ncl) * (4 * 16 + 8) + 4 * 16 + (stall ? 16u : 0u);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(cp_smem(&xmb[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(cp_smem(&xmb[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    cp_arm(&xmb[0], xbytes);
    cp_arm(&xmb[1], xbytes);
  }
  bool dead = false;  // this thread's exchange wait ran out: no more waits
  cluster.sync();     // every CTA's mbarriers exist before the first push
  for (int b0 = 0; b0 < jb; b0 += CP_IB) {
    const int be = (b0 + CP_IB < jb) ? b0 + CP_IB : jb;
    const int nb = be - b0;
    // this thread's candidate for the block's first column
    float best = -1.0f;
    int bi = N;
    for (int li = tid; li < nr; li += bd) {
      const int i = r0 + li;
      if (i < j0 + b0) continue;
      const float v = fabsf(tile[li * S + b0]);
      if (better(v, i, best, bi)) {
        best = v;
        bi = i;
      }
    }
    for (int jj = b0; jj < be; jj++) {
      const int j = j0 + jj;
      const int slot = jj & 1;
      const int q0 = jj - b0;  // column jj within the inner block
      for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (better(ov, oi, best, bi)) {
          best = ov;
          bi = oi;
        }
      }
      if (lane == 0) {
        wv[warp] = best;
        wi[warp] = bi;
      }
      __syncthreads();  // also orders the previous column step's tile writes
      if (warp == 0) {
        float cv = (lane < CP_WARPS) ? wv[lane] : -1.0f;
        int ci = (lane < CP_WARPS) ? wi[lane] : N;
        for (int o = 16; o > 0; o >>= 1) {
          const float ov = __shfl_xor_sync(0xffffffffu, cv, o);
          const int oi = __shfl_xor_sync(0xffffffffu, ci, o);
          if (better(ov, oi, cv, ci)) {
            cv = ov;
            ci = oi;
          }
        }
        const int crow = (ci < N) ? ci - r0 : 0;  // row 0's words stand in when there is no candidate
        if (ci < N)
          for (int k = lane; k < jb; k += 32) cand_row[slot][k] = tile[crow * S + k];
        __syncwarp();  // the whole row copy before any lane's (releasing) push
        const float4* src = reinterpret_cast<const float4*>(tile + static_cast<size_t>(crow) * S + b0);
        for (int e = lane; e < 2 * ncl; e += 32) {  // (destination CTA, half of the inner block)
          const unsigned d = static_cast<unsigned>(e >> 1);
          const int c0 = (e & 1) * 2;
          const unsigned bar = cp_mapa(cp_smem(&xmb[slot]), d);
          cp_push4(cp_mapa(cp_smem(&recv[slot].seg[rank][c0]), d), src[c0], bar);
          cp_push4(cp_mapa(cp_smem(&recv[slot].seg[rank][c0 + 1]), d), src[c0 + 1], bar);
          if ((e & 1) == 0) {
            cp_push1(cp_mapa(cp_smem(&recv[slot].v[rank]), d), __float_as_uint(cv), bar);
            cp_push1(cp_mapa(cp_smem(&recv[slot].i[rank]), d), static_cast<unsigned>(ci), bar);
          }
        }
      } else if (warp == 1 && j >= r0 && j < r1) {
        for (int k = lane; k < jb; k += 32) jrow[slot][k] = tile[(j - r0) * S + k];
        __syncwarp();
        const float4* src = reinterpret_cast<const float4*>(tile + static_cast<size_t>(j - r0) * S + b0);
        for (int e = lane; e < 2 * ncl; e += 32) {
          const unsigned d = static_cast<unsigned>(e >> 1);
          const int c0 = (e & 1) * 2;
          const unsigned bar = cp_mapa(cp_smem(&xmb[slot]), d);
          cp_push4(cp_mapa(cp_smem(&recv[slot].jseg[c0]), d), src[c0], bar);
          cp_push4(cp_mapa(cp_smem(&recv[slot].jseg[c0 + 1]), d), src[c0 + 1], bar);
        }
      }
      // every CTA's push of this column; the slot's next phase is column jj + 2
      // (its pushes come only after this CTA's own push of column jj + 1)
      if (!dead) dead = !cp_wait(&xmb[slot], static_cast<unsigned>(jj >> 1) & 1u, wait_ns, err);
      if (tid == 0 && !dead) cp_arm(&xmb[slot], xbytes);
      // the winner, from this CTA's own receive slot: every warp reduces the
      // candidates across its lanes (same result everywhere)
      float gv = -1.0f;
      int gi = N, tag = -1;
      if (lane < ncl) {
        gv = recv[slot].v[lane];
        gi = recv[slot].i[lane];
        tag = lane;
      }
      for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, gv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, gi, o);
        const int ot = __shfl_xor_sync(0xffffffffu, tag, o);
        if (better(ov, oi, gv, gi)) {
          gv = ov;
          gi = oi;
          tag = ot;
        }
      }
      // nothing usable below the diagonal: no swap.  (A winner is always a
      // row at or below j; a thread whose exchange wait ran out may read a
      // stale slot, and the row-move list must still hold rows of the panel.)
      if (gi < j || gi >= N) {
        gi = j;
        tag = -1;
      }
      if (rank == 0 && tid == 0) {
        ipiv[j] = gi;
        pivs[jj] = gi;
        if (!(gv > 0.0f) && *info == 0) *info = j + 1;  // zero (or NaN) pivot
      }
      // the pivot row's inner block
      const float4* p4 = (tag >= 0) ? recv[slot].seg[tag] : recv[slot].jseg;
      float ps[CP_IB];
#pragma unroll
      for (int c = 0; c < CP_IB / 4; c++) {
        const float4 x = p4[c];
        ps[4 * c] = x.x;
        ps[4 * c + 1] = x.y;
        ps[4 * c + 2] = x.z;
        ps[4 * c + 3] = x.w;
      }
      float piv = ps[0];
#pragma unroll
      for (int q = 1; q < CP_IB; q++)
        if (q == q0) piv = ps[q];
      const float inv = (piv != 0.0f) ? 1.0f / piv : 0.0f;
      const float4* jseg4 = recv[slot].jseg;
      switch (q0) {
#define KD_CP_CASE(Q) \
  case Q: cp_column_step<Q>(tile, S, b0, r0, nr, j, gi, nb, ps, jseg4, inv, piv != 0.0f, N, best, bi); break;
        KD_CP_CASE(0) KD_CP_CASE(1) KD_CP_CASE(2) KD_CP_CASE(3) KD_CP_CASE(4) KD_CP_CASE(5) KD_CP_CASE(6)
        KD_CP_CASE(7) KD_CP_CASE(8) KD_CP_CASE(9) KD_CP_CASE(10) KD_CP_CASE(11) KD_CP_CASE(12) KD_CP_CASE(13)
        KD_CP_CASE(14) KD_CP_CASE(15)
#undef KD_CP_CASE
        default: break;
      }
      // the swapped rows' other columns, from the owners' shared memory
      if (gi != j) {
        if (gi >= r0 && gi < r1) {
          const float* src = cluster.map_shared_rank(&jrow[slot][0], (j - j0) / per);
          for (int k = tid; k < jb; k += bd)
            if (k < b0 || k >= be) tile[(gi - r0) * S + k] = src[k];
        }
        if (j >= r0 && j < r1) {
          const float* src = cluster.map_shared_rank(&cand_row[slot][0], tag);
          for (int k = tid; k < jb; k += bd)
            if (k < b0 || k >= be) tile[(j - r0) * S + k] = src[k];
        }
      }
    }
    if (be < jb) {
      // Rows j0+b0 .. j0+be-1 are final in columns b0..be-1 (L11 below the
      // diagonal); every CTA fetches them whole and forms
      // U12 = L11^{-1} A12 for columns be..jb-1.
      cluster.sync();
      for (int e = tid; e < nb * jb; e += bd) {
        const int t = e / jb, k = e % jb;
        const int row = j0 + b0 + t;
        const int owner = (row - j0) / per;
        const float* ot = cluster.map_shared_rank(tile, owner);
        ublk[t][k] = ot[static_cast<long long>(row - (j0 + owner * per)) * S + k];
      }
      __syncthreads();
      for (int k = be + tid; k < jb; k += bd)  // one column of U12 per thread
        for (int t = 1; t < nb; t++) {
          float acc = ublk[t][k];
          for (int q = 0; q < t; q++) acc = fmaf(-ublk[t][b0 + q], ublk[q][k], acc);
          ublk[t][k] = acc;
        }
      cluster.sync();  // remote reads of the block rows are done
      // owners store U12; rows below the block get the rank-16 update, one
      // row per thread with its 16 multipliers in registers and four
      // columns per step
      for (int e = tid; e < nb * (jb - be); e += bd) {
        const int t = e / (jb - be), k = be + e % (jb - be);
        const int row = j0 + b0 + t;
        if (row >= r0 && row < r1) tile[(row - r0) * S + k] = ublk[t][k];
      }
      const int rs = (r0 > j0 + be) ? r0 : j0 + be;
      for (int i = rs + tid; i < r1; i += bd) {
        const int li = i - r0;
        const float4* lrow = reinterpret_cast<const float4*>(tile + static_cast<size_t>(li) * S + b0);
        float l[CP_IB];
#pragma unroll
        for (int c = 0; c < CP_IB / 4; c++) {
          const float4 x = lrow[c];
          l[4 * c] = x.x;
          l[4 * c + 1] = x.y;
          l[4 * c + 2] = x.z;
          l[4 * c + 3] = x.w;
        }
        float4* arow = reinterpret_cast<float4*>(tile + static_cast<size_t>(li) * S);
        // (inside this branch the block is full: nb == CP_IB; columns past
        // jb up to the stride are padding, updated but never read)
        for (int k4 = be / 4; k4 < (jb + 3) / 4; k4++) {
          float4 acc = arow[k4];
#pragma unroll
          for (int q = 0; q < CP_IB; q++) {
            const float4 u = *reinterpret_cast<const float4*>(&ublk[q][4 * k4]);
            acc.x = fmaf(-l[q], u.x, acc.x);
            acc.y = fmaf(-l[q], u.y, acc.y);
            acc.z = fmaf(-l[q], u.z, acc.z);
            acc.w = fmaf(-l[q], u.w, acc.w);
          }
          arow[k4] = acc;
        }
      }
      __syncthreads();
    }
  }
  __syncthreads();
  for (int e = tid; e < jb * nr; e += bd) {
    int k = e / nr, r = e % nr;
    A[static_cast<long long>(j0 + k) * ld + r0 + r] = tile[r * S + k];
  }
  cluster.sync();  // remote readers of this CTA's shared memory are done
  // the panel's row moves for the swaps outside it (ublk is free now)
  if (swap_map && rank == 0 && warp == 0) {
    int* rows = reinterpret_cast<int*>(&ublk[0][0]);
    swap_map_warp(pivs, j0, jb, swap_map, rows, rows + 256, rows + 512, rows + 512 + SWAP_HASH,
                  rows + 512 + 2 * SWAP_HASH);
  }
}

// Widest panel (96, 64 or 32 columns) whose rows fit in the shared memory of
// one 16-CTA cluster; 0 when none does.
// Widest panel (96, 64 or 32 columns, no narrower than min_w) whose rows fit
// the shared memory of one 16-CTA cluster; 0 when none does.
static int cluster_panel_width(int rows, int min_w = 32) {
  const int per = (rows + CP_CL - 1) / CP_CL;
  for (int w : {96, 64, 32})
    if (w >= min_w && static_cast<size_t>(per) * cp_row_stride(w) * sizeof(float) <= CP_MAX_SMEM) return w;
  return 0;
}

// True when the cooperative grid kernel on `nsm` SMs holds a panel of this
// height and width in shared memory (panel_grid's own test).
static bool grid_panel_fits(int rows, int jb, int nsm, size_t elem) {
  int nblk = (rows + GP_MIN_ROWS - 1) / GP_MIN_ROWS;
  if (nblk > nsm) nblk = nsm;
  const int per = (rows + nblk - 1) / nblk;
  return static_cast<size_t>(per) * jb * elem <= GP_MAX_SMEM;
}

// Launches the cluster panel on the smallest cluster (2, 4, 8 or 16 CTAs)
// whose shared memory holds the panel; false when none does or the GPU
// cannot host a 16-CTA cluster (the caller then uses the cooperative grid
// kernel).
static bool panel_cluster16(Context* ctx, float* A, long long ld, int N, int j0, int jb, int* ipiv, int* info,
                            int* swap_map, int* err, unsigned long long wait_ns, unsigned stall) {
  const int rows = N - j0;
  int ncl = 2;
  while (ncl < CP_CL &&
         static_cast<size_t>((rows + ncl - 1) / ncl) * cp_row_stride(jb) * sizeof(float) > CP_MAX_SMEM)
    ncl *= 2;
  const int per = (rows + ncl - 1) / ncl;
  const size_t smem = static_cast<size_t>(per) * cp_row_stride(jb) * sizeof(float);
  if (smem > CP_MAX_SMEM) return false;
  static int usable = 0;
  static std::once_flag probe;
  std::call_once(probe, [] {
    if (cudaFuncSetAttribute(panel_cluster16_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
            cudaSuccess &&
        cudaFuncSetAttribute(panel_cluster16_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(CP_MAX_SMEM)) == cudaSuccess) {
      cudaLaunchConfig_t q = {};
      q.gridDim = dim3(CP_CL, 1, 1);
      q.blockDim = dim3(CP_THREADS, 1, 1);
      q.dynamicSmemBytes = CP_MAX_SMEM;
      cudaLaunchAttribute qa[1];
      qa[0].id = cudaLaunchAttributeClusterDimension;
      qa[0].val.clusterDim.x = CP_CL;
      qa[0].val.clusterDim.y = 1;
      qa[0].val.clusterDim.z = 1;
      q.attrs = qa;
      q.numAttrs = 1;
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, panel_cluster16_kernel, &q) == cudaSuccess && nclusters > 0)
        usable = 1;
    }
    cudaGetLastError();  // clear a refused attribute or query
  });
  if (!usable) return false;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ncl, 1, 1);
  cfg.blockDim = dim3(CP_THREADS, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = ctx->stream();
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = ncl;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cuda_check(cudaLaunchKernelEx(&cfg, panel_cluster16_kernel, A, ld, N, j0, jb, per, ipiv, info, swap_map, err, wait_ns,
                                stall),
             "panel cluster kernel");
  ctx->launches += 1;
  return true;
}

// Applies a panel's row moves to every column outside the panel, one warp
// per column: all sources are read into registers before any write.
constexpr int SWAP_PER_LANE = 8;  // 2 jb <= 256 = 32 x 8 moves
template <class T>
__global__ void laswp_map(T* __restrict__ A, long long ld, int N, int j0, int jb, const int* __restrict__ map) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int ncol = N - jb;
  if (warp >= ncol) return;
  const int c = (warp < j0) ? warp : warp + jb;
  T* col = A + static_cast<long long>(c) * ld;
  const int n = map[0];
  const int* dst = map + 1;
  const int* src = map + 1 + 2 * jb;
  T v[SWAP_PER_LANE];
#pragma unroll
  for (int q = 0; q < SWAP_PER_LANE; q++) {
    int t = lane + 32 * q;
    if (t < n) v[q] = col[src[t]];
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < SWAP_PER_LANE; q++) {
    int t = lane + 32 * q;
    if (t < n && dst[t] != src[t]) col[dst[t]] = v[q];
  }
}

template <class T>
static bool panel_grid(Context* ctx, T* A, long long ld, int N, int j0, int jb, int* ipiv, int* info, int nsm,
                       const PanelSlots<T>& slots) {
  const int rows = N - j0;
  int nblk = (rows + GP_MIN_ROWS - 1) / GP_MIN_ROWS;
  if (nblk > nsm) nblk = nsm;
  const int per = (rows + nblk - 1) / nblk;
  nblk = (rows + per - 1) / per;
  const size_t smem = static_cast<size_t>(per) * jb * sizeof(T);
  if (smem > GP_MAX_SMEM) return false;
  static std::once_flag attr;
  std::call_once(attr, [] {
    cuda_check(cudaFuncSetAttribute(panel_grid_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(GP_MAX_SMEM)),
               "cudaFuncSetAttribute(panel)");
  });
  cudaStream_t s = ctx->stream();
  cuda_check(cudaMemsetAsync(slots.bar, 0, sizeof(unsigned), s), "memset barrier");
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nblk, 1, 1);
  cfg.blockDim = dim3(GP_THREADS, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cuda_check(cudaLaunchKernelEx(&cfg, panel_grid_kernel<T>, A, ld, N, j0, jb, per, ipiv, info, slots),
             "panel grid kernel");
  ctx->launches += 1;
  return true;
}

template <class T>
// Factors one panel; returns true when the panel kernel also wrote the
// panel's row-move list into swap_map (the FP32 cluster path).
static bool panel_factor(Context* ctx, T* A, long long ld, int N, int j0, int jb, int* ipiv, int* info, int nsm,
                         void* slot_mem, int* swap_map) {
  cudaStream_t s = ctx->stream();
  ProfScope ps(ctx, Context::PROF_LU_PANEL, 2.0 * sizeof(T) * jb * (N - j0));
  if (jb > 128) throw KdError(KD_ERR_ARG, "panel width above 128");
  PanelSlots<T> slots;
  {
    char* p = static_cast<char*>(slot_mem);
    slots.cand_rows = reinterpret_cast<T*>(p);
    p += sizeof(double) * 2 * 128 * static_cast<size_t>(nsm);
    slots.cand_v = reinterpret_cast<double*>(p);
    p += sizeof(double) * 2 * static_cast<size_t>(nsm);
    slots.jrow = reinterpret_cast<T*>(p);
    p += sizeof(double) * 2 * 128;
    slots.cand_i = reinterpret_cast<int*>(p);
    p += sizeof(int) * 2 * static_cast<size_t>(nsm);
    slots.bar = reinterpret_cast<unsigned*>(p);
    slots.err = reinterpret_cast<int*>(p + 16);
    slots.wait_ns = ctx->grid_wait_ns;
    slots.stall = ctx->stall_waits ? 1u : 0u;
  }
  if constexpr (std::is_same<T, float>::value) {
    if (panel_cluster16(ctx, A, ld, N, j0, jb, ipiv, info, swap_map, slots.err, slots.wait_ns, slots.stall)) return true;
  }
  if (panel_grid<T>(ctx, A, ld, N, j0, jb, ipiv, info, nsm < ctx->sms() ? nsm : ctx->sms(), slots)) return false;
  // Panels too tall for the shared memory of the GPU: one 8-CTA cluster
  // working on the panel in global memory.
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(PANEL_CL, 1, 1);
  cfg.blockDim = dim3(PANEL_THREADS, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = PANEL_CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cuda_check(cudaLaunchKernelEx(&cfg, panel_cluster_kernel<T>, A, ld, N, j0, jb, ipiv, info), "panel cluster kernel");
  ctx->launches += 1;
  return false;
}

static void launch_trsm_chunk(Context* ctx, float* A, long long ld, int j0, int jb, int c0, int c1) {
  static std::once_flag attr;
  std::call_once(attr, [] {
    cuda_check(cudaFuncSetAttribute(trsm_chunk_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(TS_SMEM)),
               "cudaFuncSetAttribute(trsm)");
  });
  trsm_chunk_f32<<<blocks(c1 - c0, TS_COLS), TS_THREADS, TS_SMEM, ctx->stream()>>>(A, ld, j0, jb, c0, c1);
  ctx->launches += 1;
  cuda_check(cudaGetLastError(), "trsm kernel");
}

template <class T>
static void trsm_and_swaps(Context* ctx, T* A, long long ld, int N, int j0, int jb, const int* ipiv, int* map,
                           bool map_ready) {
  cudaStream_t s = ctx->stream();
  ProfScope ps(ctx, Context::PROF_LU_SWAP_TRSM, 2.0 * sizeof(T) * jb * (N - j0 - jb));
  if (N > jb) {
    if (!map_ready) {
      build_swap_map<<<1, 32, 0, s>>>(ipiv, j0, jb, map);
      ctx->launches += 1;
    }
    laswp_map<T><<<blocks(static_cast<long long>(N - jb) * 32, 256), 256, 0, s>>>(A, ld, N, j0, jb, map);
    ctx->launches += 1;
  }
  if (j0 + jb < N) {
    size_t smem = sizeof(double) * (static_cast<size_t>(jb) * jb + static_cast<size_t>(jb) * TRSM_COLS);
    static std::once_flag attr_set;
    std::call_once(attr_set,
                   [] { cudaFuncSetAttribute(trsm_unit_lower<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024); });
    if constexpr (std::is_same<T, float>::value) {
      if (jb <= 96) {
        launch_trsm_chunk(ctx, A, ld, j0, jb, j0 + jb, N);
        return;
      }
    }
    trsm_unit_lower<T><<<blocks(N - j0 - jb, TRSM_COLS), TRSM_COLS, smem, s>>>(A, ld, j0, jb, j0 + jb, N);
    ctx->launches += 1;
  }
  cuda_check(cudaGetLastError(), "laswp/trsm kernels");
}

void DenseLU::factor_fp64(double* A, long long ld, int N) {
  const int NB = nb > 96 ? 96 : nb;  // L11 + one column tile fit in shared memory
  cudaStream_t s = ctx_->stream();
  cuda_check(cudaMemsetAsync(d_info_, 0, sizeof(int), s), "memset info");
  for (int j0 = 0; j0 < N; j0 += NB) {
    int jb = (N - j0 < NB) ? N - j0 : NB;
    const bool map_ready = panel_factor<double>(ctx_, A, ld, N, j0, jb, ipiv_, d_info_, nsm_, slot_mem_, swap_map_);
    trsm_and_swaps<double>(ctx_, A, ld, N, j0, jb, ipiv_, swap_map_, map_ready);
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
  // Panel width (blocked LU allows any widths).  A cluster panel of 96 or
  // 64 columns when its rows fit one 16-CTA cluster.  Taller panels: 96
  // columns on the cooperative grid when it holds them, since each panel
  // costs one pass of the trailing matrix through HBM in the update and a
  // 32-column panel triples that traffic; a 32-column cluster panel when the
  // grid cannot (a context limited to a share of the SMs).
  const int nsm_eff = nsm_ < ctx_->sms() ? nsm_ : ctx_->sms();
  auto on_cluster = [&](int rows) {
    if (NB != 96) return false;
    if (cluster_panel_width(rows, 64) > 0) return true;
    return !grid_panel_fits(rows, 96, nsm_eff, sizeof(float)) && cluster_panel_width(rows) > 0;
  };
  auto width = [&](int j0) {
    const int rows = N - j0;
    int w = NB;
    if (on_cluster(rows)) w = cluster_panel_width(rows);
    return (rows < w) ? rows : w;
  };
  // Look-ahead (tensor-core update only): the columns of the next panel are
  // updated first, then the rest of the trailing update runs on a side
  // stream as 16-CTA clusters that leave one GPC free, while the next panel
  // is factored on the main stream; the next row exchanges wait for both.
  // A panel on the cooperative grid needs every SM, so it cannot run beside
  // the update: look-ahead only when the next panel fits a cluster.
  const bool lookahead = tf32 && tf32_update_max_clusters16() >= 2;
  int j0 = 0, jb = width(0);
  bool map_ready = panel_factor<float>(ctx_, A, ld, N, j0, jb, ipiv_, d_info_, nsm_, slot_mem_, swap_map_);
  bool side_pending = false;
  for (;;) {
    if (side_pending) {
      ctx_->join();
      side_pending = false;
    }
    trsm_and_swaps<float>(ctx_, A, ld, N, j0, jb, ipiv_, swap_map_, map_ready);
    const int m = N - j0 - jb;
    if (m <= 0) break;
    const int j0n = j0 + jb, jbn = width(j0n);
    float* A21 = A + static_cast<long long>(j0) * ld + j0 + jb;
    float* A12 = A + static_cast<long long>(j0 + jb) * ld + j0;
    float* A22 = A + static_cast<long long>(j0 + jb) * ld + j0 + jb;
    // rows N .. ld of the working matrix are padding
    const int writable = static_cast<int>(ld - j0 - jb);
    if (lookahead && m > jbn && on_cluster(N - j0n)) {
      gemm_update_f32(ctx_, blas_, m, jbn, jb, A21, ld, A12, ld, A22, ld, tf32, writable, tf32_terms);
      ctx_->fork(1);
      ctx_->use(0);
      gemm_update_f32(ctx_, blas_, m, m - jbn, jb, A21, ld, A12 + static_cast<long long>(jbn) * ld, ld,
                      A22 + static_cast<long long>(jbn) * ld, ld, tf32, writable, tf32_terms, true);
      ctx_->use(-1);
      side_pending = true;
    } else {
      gemm_update_f32(ctx_, blas_, m, m, jb, A21, ld, A12, ld, A22, ld, tf32, writable, tf32_terms);
    }
    map_ready = panel_factor<float>(ctx_, A, ld, N, j0n, jbn, ipiv_, d_info_, nsm_, slot_mem_, swap_map_);
    j0 = j0n;
    jb = jbn;
  }
  if (side_pending) ctx_->join();
}

// Static-pivot factorisation of the FP32 working copy, whose rows are
// already in the pivot order of an earlier factorisation.  Panels are 192
// columns wide, each made of two 96-column halves: the left half is factored
// (panel_nopiv_kernel: the diagonal block and L21 in one launch), its U12
// over the right half solved, the right half updated below it, then
// factored.  The U12 solve of a wide panel goes the same way by halves, and
// the trailing update runs with k = 192 on the tensor cores, which streams
// the trailing matrix through HBM half as often as 96-column panels would.
// Columns that do not fill a wide panel take 96-column panels.  No row
// exchanges, no grid-wide synchronisation.
void DenseLU::factor_f32_nopiv(float* A, long long ld, int N, bool tf32) {
  cudaStream_t s = ctx_->stream();
  cuda_check(cudaMemsetAsync(d_info_, 0, sizeof(int), s), "memset info");
  const int NB = NP_NB, NW = 2 * NP_NB;
  auto at = [&](int row, int col) { return A + static_cast<long long>(col) * ld + row; };
  auto panel = [&](int j0, int jb) {
    const int m = N - j0 - jb;
    ProfScope ps(ctx_, Context::PROF_LU_PANEL_STATIC, 2.0 * sizeof(float) * jb * (N - j0));
    // at most NP_MAX_CTAS CTAs (several 256-row groups each): the SMs left
    // beside the trailing update's 16-CTA clusters
    const int groups = m > 0 ? blocks(m, NP_THREADS) : 1;
    const int rpt = (groups + NP_MAX_CTAS - 1) / NP_MAX_CTAS;
    const int grid = (groups + rpt - 1) / rpt;
    static std::once_flag attr;
    std::call_once(attr, [] {
      cuda_check(cudaFuncSetAttribute(panel_nopiv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, NP_XS_BYTES),
                 "panel_nopiv smem");
    });
    panel_nopiv_kernel<<<grid, NP_THREADS, NP_XS_BYTES, ctx_->stream()>>>(A, ld, N, j0, jb, rpt, d_info_, np_done_);
    ctx_->launches++;
  };
  auto trsm = [&](int j0, int jb, int c0, int c1) {
    ProfScope ps(ctx_, Context::PROF_LU_SWAP_TRSM, 2.0 * sizeof(float) * jb * (c1 - c0));
    launch_trsm_chunk(ctx_, A, ld, j0, jb, c0, c1);
  };
  // a panel of jb <= 96 columns, or a wide one of 192 as two halves
  auto wide_panel = [&](int j0, int jb) {
    if (jb <= NB) {
      panel(j0, jb);
      return;
    }
    panel(j0, NB);
    trsm(j0, NB, j0 + NB, j0 + jb);
    const int mr = N - j0 - NB;
    gemm_update_f32(ctx_, blas_, mr, jb - NB, NB, at(j0 + NB, j0), ld, at(j0, j0 + NB), ld, at(j0 + NB, j0 + NB), ld,
                    tf32, static_cast<int>(ld - j0 - NB), tf32_terms, 0, NP_MAX_CTAS);
    panel(j0 + NB, jb - NB);
  };
  // U12 = L11^-1 A12 for the panel's rows over columns [c0, c1)
  auto wide_trsm = [&](int j0, int jb, int c0, int c1) {
    if (jb <= NB) {
      trsm(j0, jb, c0, c1);
      return;
    }
    trsm(j0, NB, c0, c1);
    gemm_update_f32(ctx_, blas_, jb - NB, c1 - c0, NB, at(j0 + NB, j0), ld, at(j0, c0), ld, at(j0 + NB, c0), ld, tf32,
                    jb - NB, tf32_terms);
    trsm(j0 + NB, jb - NB, c0, c1);
  };
  auto width = [&](int j0) { return N - j0 >= NW ? NW : (N - j0 < NB ? N - j0 : NB); };
  // Look-ahead (tensor-core update): the next panel's columns are updated
  // first, then the rest of the trailing update runs on a side stream as
  // every 16-CTA cluster the GPU holds, while the next panel is factored on
  // the main stream on the SMs left; the next U12 solve waits for both.
  const bool lookahead = tf32 && tf32_update_max_clusters16() >= 2;
  int j0 = 0, jb = width(0);
  wide_panel(j0, jb);
  bool side_pending = false;
  for (;;) {
    if (side_pending) {
      ctx_->join();
      side_pending = false;
    }
    const int m = N - j0 - jb;
    if (m <= 0) break;
    wide_trsm(j0, jb, j0 + jb, N);
    const int j0n = j0 + jb, jbn = width(j0n);
    float* A21 = at(j0 + jb, j0);
    float* A12 = at(j0, j0 + jb);
    float* A22 = at(j0 + jb, j0 + jb);
    const int writable = static_cast<int>(ld - j0 - jb);
    if (lookahead && m > jbn) {
      gemm_update_f32(ctx_, blas_, m, jbn, jb, A21, ld, A12, ld, A22, ld, tf32, writable, tf32_terms);
      ctx_->fork(1);
      ctx_->use(0);
      gemm_update_f32(ctx_, blas_, m, m - jbn, jb, A21, ld, A12 + static_cast<long long>(jbn) * ld, ld,
                      A22 + static_cast<long long>(jbn) * ld, ld, tf32, writable, tf32_terms, 2);
      ctx_->use(-1);
      side_pending = true;
    } else {
      gemm_update_f32(ctx_, blas_, m, m, jb, A21, ld, A12, ld, A22, ld, tf32, writable, tf32_terms);
    }
    wide_panel(j0n, jbn);
    j0 = j0n;
    jb = jbn;
  }
  if (side_pending) ctx_->join();
  cuda_check(cudaGetLastError(), "static-pivot factorisation");
}

// FP32 working copy of the FP64 matrix (equilibrated, rows in the order
// `perm` when it is given) and its factorisation: with perm, the
// static-pivot path; without, partial pivoting.
void DenseLU::factor_mixed(double* A, long long ld, int N, int mode, const int* perm) {
  double* rs = eq_buf_;
  double* cs = eq_buf_ + N;
  unsigned long long* rmax = reinterpret_cast<unsigned long long*>(eq_buf_ + 2 * static_cast<size_t>(N));
  cudaStream_t st = ctx_->stream();
  if (equilibrate) {
    cuda_check(cudaMemsetAsync(rmax, 0, sizeof(unsigned long long) * N, st), "memset row max");
    const int rb = blocks(N, 256);
    int nch = (4 * nsm_ + rb - 1) / rb;
    if (nch < 1) nch = 1;
    const int chunk = (N + nch - 1) / nch;
    nch = (N + chunk - 1) / chunk;
    row_absmax_kernel<<<dim3(rb, nch), 256, 0, st>>>(A, ld, N, chunk, rmax);
    row_scale_kernel<<<rb, 256, 0, st>>>(rmax, N, rs);
    if (perm)
      convert_rows_kernel<<<N, 256, 0, st>>>(A, ld, rs, N, cs, A32_, ld32_, perm);
    else
      col_scale_convert_kernel<<<N, 256, 0, st>>>(A, ld, rs, N, cs, A32_, ld32_);
    ctx_->launches += 3;
  } else if (perm) {
    convert_rows_kernel<<<N, 256, 0, st>>>(A, ld, nullptr, N, nullptr, A32_, ld32_, perm);
    ctx_->launches++;
  } else {
    d2s<<<152 * 8, 256, 0, st>>>(A, ld, A32_, ld32_, N);
    ctx_->launches++;
  }
  scaled_ = equilibrate;
  iota_kernel<<<blocks(N, 256), 256, 0, st>>>(ipiv_, N);
  ctx_->launches++;
  if (perm) {
    factor_f32_nopiv(A32_, ld32_, N, mode == LU_TF32_IR);
    prepare_solves<float>(A32_, ld32_, N, true);
  } else {
    factor_f32(A32_, ld32_, N, mode == LU_TF32_IR);
    prepare_solves<float>(A32_, ld32_, N, false);
  }
  nopiv_ = perm != nullptr;
}

int DenseLU::read_info() {
  int info = 0;
  cuda_check(cudaMemcpyAsync(&info, d_info_, sizeof(int), cudaMemcpyDeviceToHost, ctx_->stream()), "D2H info");
  cuda_check(cudaStreamSynchronize(ctx_->stream()), "sync after LU");
  return info;
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
  iota_kernel<<<blocks(N, 256), 256, 0, ctx_->stream()>>>(ipiv_, N);
  ctx_->launches++;
  if (mode == LU_FP64) {
    factor_fp64(A, ld, N);
    prepare_solves<double>(A, ld, N, false);
    nopiv_ = false;
  } else {
    ld32_ = ((static_cast<long long>(N) + 31) / 32) * 32;  // 128-byte aligned columns
    const size_t need = static_cast<size_t>(ld32_) * N;
    if (need > a32_cap_) {
      cudaFree(A32_);
      cuda_check(cudaMalloc(&A32_, need * sizeof(float)), "cudaMalloc(A32)");
      a32_cap_ = need;
    }
    if (static_cast<size_t>(N) > eq_cap_) {
      cudaFree(eq_buf_);
      cuda_check(cudaMalloc(&eq_buf_, sizeof(double) * 3 * static_cast<size_t>(N)), "cudaMalloc(equilibration)");
      eq_cap_ = N;
    }
    // later factorisations of a matrix of the same size reuse the pivot
    // order of the last partial-pivoting factorisation (static pivoting)
    const bool reuse = reuse_pivots && perm_n_ == N;
    factor_mixed(A, ld, N, mode, reuse ? perm_ : nullptr);
    if (reuse && read_info() != 0) {
      // a zero or non-finite pivot in that order: factor with partial pivoting
      stats.static_pivot_fallback = 1;
      perm_n_ = 0;
      factor_mixed(A, ld, N, mode, nullptr);
    }
  }
  int info = read_info();
  stats.t_factor_ms = now_ms() - t0;
  int perr = 0;
  cuda_check(cudaMemcpyAsync(&perr, panel_err_, sizeof(int), cudaMemcpyDeviceToHost, ctx_->stream()),
             "D2H panel flag");
  cuda_check(cudaStreamSynchronize(ctx_->stream()), "sync panel flag");
  if (perr) {
    cuda_check(cudaMemsetAsync(panel_err_, 0, sizeof(int), ctx_->stream()), "reset panel flag");
    throw KdError(KD_ERR_TIMEOUT, "panel factorisation: a grid barrier wait ran out (or a cluster panel's exchange wait)");
  }
  if (mode == LU_TF32_IR && tf32_gemm_error_flag(ctx_))
    throw KdError(KD_ERR_TIMEOUT, "tensor-core trailing update timed out waiting for its MMAs");
  if (info != 0) throw KdError(KD_ERR_SINGULAR, "Jacobian is singular (zero pivot at column " + std::to_string(info) + ")");
  if (!nopiv_) perm_n_ = N;  // perm_ holds this factorisation's pivot order
  stats.static_pivots = nopiv_ ? 1 : 0;
}

// Triangular solves by 64-row blocks with precomputed inverses of the
// diagonal blocks: one launch per block computes the block's unknowns as a
// small GEMV and subtracts their contribution from the remaining rows.
template <class T>
void DenseLU::tri_solve(const T* LU, long long ld, int N, double* b, int trans) {
  cudaStream_t s = ctx_->stream();
  // work of one sweep: the triangle of the factors it reads
  const double sweep_bytes = 0.5 * sizeof(T) * N * static_cast<double>(N);
  const int nblk = (N + TB - 1) / TB;
  const size_t rnd = ((static_cast<size_t>(N) + 31) / 32) * 32;
  double* w1 = tri_work_;
  double* w2 = tri_work_ + rnd;  // 256-byte aligned second vector
  const size_t bs = static_cast<size_t>(TB) * TB;
  if (!trans) {
    gather_perm<<<blocks(N, 256), 256, 0, s>>>(b, perm_, N, w1);
    // L y = P b, then U x = y: one cooperative launch per sweep
    int g = blocks(N, SW_TILE);
    if (g > ctx_->sms()) g = ctx_->sms();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(g, 1, 1);
    cfg.blockDim = dim3(256, 1, 1);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cuda_check(cudaMemsetAsync(tri_bar_, 0, 2 * sizeof(unsigned), s), "memset sweep barriers");
    const double* dl = dinv_l_;
    const double* du = dinv_u_;
    const float2* dl2 = std::is_same<T, float>::value ? dinv2_l_ : nullptr;
    const float2* du2 = std::is_same<T, float>::value ? dinv2_u_ : nullptr;
    const unsigned long long wait = ctx_->grid_wait_ns;
    const unsigned stall = ctx_->stall_waits ? 1u : 0u;
    const int gch = (nblk + CH_R - 1) / CH_R;
    // the choice depends on the device only (not on a context's SM budget),
    // so that concurrent and serial solves sum in the same order
    if (sweep_kind == 2 && gch <= nsm_) {
      static std::once_flag ch_attr;
      std::call_once(ch_attr, [] {
        cuda_check(cudaFuncSetAttribute(trsv_chain<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(chain_smem<float>())),
                   "cudaFuncSetAttribute(chain sweep)");
        cuda_check(cudaFuncSetAttribute(trsv_chain<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(chain_smem<double>())),
                   "cudaFuncSetAttribute(chain sweep)");
      });
      cfg.gridDim = dim3(gch, 1, 1);
      cfg.dynamicSmemBytes = chain_smem<T>();
      const double* w1c = w1;
      const double* w2c = w2;
      // FP32 copies of the two sweeps' outputs (FP32 factors only)
      float* yf1 = std::is_same<T, float>::value ? reinterpret_cast<float*>(tri_work_ + 2 * rnd) : nullptr;
      float* yf2 = std::is_same<T, float>::value ? yf1 + rnd : nullptr;
      {
        ProfScope ps(ctx_, Context::PROF_LU_SOLVE, sweep_bytes);
        cuda_check(cudaLaunchKernelEx(&cfg, trsv_chain<T>, LU, ld, N, w1c, w2, yf1, dl, dl2, 1, tri_bar_, panel_err_,
                                      wait, stall),
                   "forward sweep");
      }
      {
        ProfScope ps(ctx_, Context::PROF_LU_SOLVE, sweep_bytes);
        cuda_check(cudaLaunchKernelEx(&cfg, trsv_chain<T>, LU, ld, N, w2c, b, yf2, du, du2, 0, tri_bar_ + 1,
                                      panel_err_, wait, stall),
                   "backward sweep");
      }
    } else if (sweep_kind == 1) {
      int gp = nblk < ctx_->sms() ? nblk : ctx_->sms();
      cfg.gridDim = dim3(gp, 1, 1);
      const double* w1c = w1;
      const double* w2c = w2;
      ProfScope ps(ctx_, Context::PROF_LU_SOLVE, 2 * sweep_bytes);
      cuda_check(cudaLaunchKernelEx(&cfg, trsv_pull<T>, LU, ld, N, w1c, w2, dl, dl2, 1, tri_bar_, panel_err_, wait,
                                    stall),
                 "forward sweep");
      cuda_check(cudaLaunchKernelEx(&cfg, trsv_pull<T>, LU, ld, N, w2c, b, du, du2, 0, tri_bar_ + 1, panel_err_,
                                    wait, stall),
                 "backward sweep");
    } else {
      ProfScope ps(ctx_, Context::PROF_LU_SOLVE, 2 * sweep_bytes);
      cuda_check(cudaLaunchKernelEx(&cfg, trsv_sweep<T>, LU, ld, N, w1, w2, dl, dl2, 1, tri_bar_, panel_err_, wait,
                                    stall),
                 "forward sweep");
      cuda_check(cudaLaunchKernelEx(&cfg, trsv_sweep<T>, LU, ld, N, w2, b, du, du2, 0, tri_bar_ + 1, panel_err_,
                                    wait, stall),
                 "backward sweep");
    }
    ctx_->launches += 3;
    cuda_check(cudaGetLastError(), "triangular solve");
    return;
  } else {
    // A^T = U^T L^T P: U^T y = b (forward, lower), L^T z = y (backward), x = P^T z
    ProfScope ps(ctx_, Context::PROF_LU_SOLVE, 2 * sweep_bytes);
    for (int k = 0; k < nblk; k++) {
      int r0 = k * TB, n = (N - r0 < TB) ? N - r0 : TB;
      int q0 = r0 + n, q1 = N;
      int g = q1 > q0 ? blocks(static_cast<long long>(q1 - q0) * 32, 256) : 1;
      trsv_step<T><<<g, 256, 0, s>>>(LU, ld, b, w2, r0, n, dinv_u_ + k * bs, 1, q0, q1, 1);
    }
    for (int k = nblk - 1; k >= 0; k--) {
      int r0 = k * TB, n = (N - r0 < TB) ? N - r0 : TB;
      int q0 = 0, q1 = r0;
      int g = q1 > q0 ? blocks(static_cast<long long>(q1 - q0) * 32, 256) : 1;
      trsv_step<T><<<g, 256, 0, s>>>(LU, ld, w2, w1, r0, n, dinv_l_ + k * bs, 1, q0, q1, 1);
    }
    scatter_perm<<<blocks(N, 256), 256, 0, s>>>(w1, perm_, N, b);
  }
  ctx_->launches += 2 * nblk + 1;
  cuda_check(cudaGetLastError(), "triangular solve");
}

void DenseLU::solve_fp64(const double* LU, long long ld, int N, double* b, int trans) {
  tri_solve<double>(LU, ld, N, b, trans);
}

void DenseLU::solve_f32(double* b, int trans) {
  // M^-1 b = D_c (LU)^-1 (D_r b) with the equilibrated factors LU of
  // P D_r A D_c; transposed, M^-T b = D_r (LU)^-T (D_c b)
  cudaStream_t st = ctx_->stream();
  const double* first = trans ? eq_buf_ + N_ : eq_buf_;
  const double* last = trans ? eq_buf_ : eq_buf_ + N_;
  if (scaled_) {
    scale_vec_kernel<<<blocks(N_, 256), 256, 0, st>>>(b, first, N_);
    ctx_->launches++;
  }
  tri_solve<float>(A32_, ld32_, N_, b, trans);
  if (scaled_) {
    scale_vec_kernel<<<blocks(N_, 256), 256, 0, st>>>(b, last, N_);
    ctx_->launches++;
  }
}

// A sweep that gave up is reported first (its garbage also stops the
// refinement), and its flag is cleared so the context stays usable.
void DenseLU::check_sweeps() {
  cuda_check(cudaStreamSynchronize(ctx_->stream()), "sync after solve");
  int perr = 0;
  cuda_check(cudaMemcpyAsync(&perr, panel_err_, sizeof(int), cudaMemcpyDeviceToHost, ctx_->stream()),
             "D2H sweep flag");
  cuda_check(cudaStreamSynchronize(ctx_->stream()), "sync sweep flag");
  if (perr) {
    cuda_check(cudaMemsetAsync(panel_err_, 0, sizeof(int), ctx_->stream()), "reset sweep flag");
    cuda_check(cudaStreamSynchronize(ctx_->stream()), "sync sweep flag reset");
    throw KdError(KD_ERR_TIMEOUT, "triangular solve: a grid barrier wait ran out");
  }
}

void DenseLU::ensure_bsave() {
  if (static_cast<size_t>(N_) > bsave_cap_) {
    cudaFree(bsave_);
    bsave_ = nullptr;
    cuda_check(cudaMalloc(&bsave_, sizeof(double) * N_), "cudaMalloc(rhs copy)");
    bsave_cap_ = N_;
  }
}

// After factorisation: pivots as one permutation, inverses of the 64 x 64
// diagonal blocks of L (unit lower) and U.
template <class T>
void DenseLU::prepare_solves(const T* LU, long long ld, int N, bool keep_perm) {
  cudaStream_t s = ctx_->stream();
  const int nblk = (N + TB - 1) / TB;
  size_t need = static_cast<size_t>(nblk) * TB * TB;
  if (need > dinv_cap_) {
    cudaFree(dinv_l_);
    cudaFree(dinv_u_);
    cuda_check(cudaMalloc(&dinv_l_, need * sizeof(double)), "cudaMalloc(Linv)");
    cuda_check(cudaMalloc(&dinv_u_, need * sizeof(double)), "cudaMalloc(Uinv)");
    cudaFree(dinv2_l_);
    cudaFree(dinv2_u_);
    dinv2_l_ = dinv2_u_ = nullptr;
    cuda_check(cudaMalloc(&dinv2_l_, need * sizeof(float2)), "cudaMalloc(Linv pairs)");
    cuda_check(cudaMalloc(&dinv2_u_, need * sizeof(float2)), "cudaMalloc(Uinv pairs)");
    dinv_cap_ = need;
  }
  if (static_cast<size_t>(N) > perm_cap_) {
    cudaFree(perm_);
    cudaFree(tri_work_);
    cuda_check(cudaMalloc(&perm_, sizeof(int) * N), "cudaMalloc(perm)");
    // two FP64 vectors, then two FP32 vectors (the chained sweeps' copies)
    cuda_check(cudaMalloc(&tri_work_, sizeof(double) * 3 * (((static_cast<size_t>(N) + 31) / 32) * 32)),
               "cudaMalloc(tri work)");
    perm_cap_ = N;
  }
  if (!keep_perm) build_perm<<<1, 1, 0, s>>>(ipiv_, N, perm_);
  size_t smem = sizeof(double) * 3 * TB * TB;
  static std::once_flag attr_set;
  std::call_once(attr_set, [smem] {
    cudaFuncSetAttribute(invert_diag_blocks<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    cudaFuncSetAttribute(invert_diag_blocks<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  });
  invert_diag_blocks<T><<<nblk, TB, smem, s>>>(LU, ld, N, dinv_l_, dinv_u_);
  if constexpr (std::is_same<T, float>::value) {
    const long long n2 = static_cast<long long>(nblk) * TB * TB;
    split_df_kernel<<<blocks(n2, 256) < 152 * 8 ? blocks(n2, 256) : 152 * 8, 256, 0, s>>>(dinv_l_, dinv2_l_, n2);
    split_df_kernel<<<blocks(n2, 256) < 152 * 8 ? blocks(n2, 256) : 152 * 8, 256, 0, s>>>(dinv_u_, dinv2_u_, n2);
    ctx_->launches += 2;
  }
  ctx_->launches += 2;
  cuda_check(cudaGetLastError(), "solve preparation");
}

// Right-preconditioned GMRES(m) in FP64 with the FP32 LU as preconditioner:
// solves A x = b to a relative residual below gmres_tol.  Small dense
// Hessenberg algebra runs on the host (m <= 50), vectors stay on the device.
void DenseLU::gemv(const double* x, double* y, double alpha, double beta, const double* b, int trans) {
  const int N = N_;
  cudaStream_t s = ctx_->stream();
  if (trans) {
    gemv_t_kernel<<<blocks(N, GEMVT_WARPS), GEMVT_WARPS * 32, 0, s>>>(A_, ld_, N, x, alpha, beta, b, y);
    ctx_->launches++;
    return;
  }
  const int rb = blocks(N, GEMV_ROWS);
  int nchunk = (4 * nsm_ + rb - 1) / rb;  // the device's SMs: the split of the sums stays fixed
  if (nchunk > 32) nchunk = 32;
  if (nchunk < 1) nchunk = 1;
  const int chunk = (N + nchunk - 1) / nchunk;
  nchunk = (N + chunk - 1) / chunk;
  const size_t need = static_cast<size_t>(32) * N;
  if (need > part_cap_) {
    cudaFree(part_);
    cuda_check(cudaMalloc(&part_, need * sizeof(double)), "cudaMalloc(gemv partials)");
    part_cap_ = need;
  }
  gemv_partial<<<dim3(rb, nchunk), GEMV_ROWS, 0, s>>>(A_, ld_, N, x, chunk, part_);
  gemv_finish<<<blocks(N, 256), 256, 0, s>>>(part_, nchunk, N, alpha, beta, b, y);
  ctx_->launches += 2;
}

void DenseLU::gmres_ir(double* b, int trans) {
  // Right-preconditioned GMRES(m), M^-1 = the FP32 factors.  The basis is
  // orthogonalised by classical Gram-Schmidt run twice (CGS2): per
  // iteration two passes of dot products and one norm on the device, one
  // copy of the results to the host; the small Hessenberg least-squares
  // problem is solved on the host.  At most gmres_restarts cycles.  With
  // trans the operator is A^T and the preconditioner M^-T.
  const int N = N_;
  const int m = gmres_max_iter;
  cudaStream_t s = ctx_->stream();
  const size_t hn_at = 2 * static_cast<size_t>(m + 1);  // projections of both passes, then |w|^2
  ensure_work(static_cast<size_t>(N) * (m + 4) + hn_at + 1);
  if (hproj_cap_ < hn_at + 1) {
    if (hproj_) cudaFreeHost(hproj_);
    hproj_ = nullptr;
    hproj_cap_ = 0;
    cuda_check(cudaMallocHost(&hproj_, (hn_at + 1) * sizeof(double)), "cudaMallocHost(projections)");
    hproj_cap_ = hn_at + 1;
  }
  double* V = work_;  // m + 1 basis vectors
  double* w = work_ + static_cast<size_t>(N) * (m + 1);
  double* x = w + N;
  double* r = x + N;
  double* dproj = r + N;  // [0, m+1): first pass, [m+1, 2m+2): second pass, [2m+2]: |w|^2
  const int nb = blocks(N, VA_THREADS);
  auto copy_scaled = [&](const double* src, double alpha, double* dst) {
    scaled_copy<<<nb, VA_THREADS, 0, s>>>(N, alpha, src, dst, 0);
    ctx_->launches++;
  };
  auto add_scaled = [&](const double* src, double alpha, double* dst) {
    scaled_copy<<<nb, VA_THREADS, 0, s>>>(N, alpha, src, dst, 1);
    ctx_->launches++;
  };
  auto norm = [&](const double* v) {
    sum_squares<<<1, VA_THREADS, 0, s>>>(v, N, dproj + hn_at);
    ctx_->launches++;
    cuda_check(cudaMemcpyAsync(hproj_ + hn_at, dproj + hn_at, sizeof(double), cudaMemcpyDeviceToHost, s),
               "D2H norm");
    cuda_check(cudaStreamSynchronize(s), "sync norm");
    return std::sqrt(hproj_[hn_at]);
  };
  cuda_check(cudaMemsetAsync(x, 0, sizeof(double) * N, s), "memset x");
  const double bnorm = norm(b);
  if (bnorm == 0) return;
  int total_it = 0;
  for (int restart = 0; restart < gmres_restarts; restart++) {
    // r = b - A x (x = 0 on the first cycle: r = b, no matvec)
    if (restart == 0) {
      cuda_check(cudaMemcpyAsync(r, b, sizeof(double) * N, cudaMemcpyDeviceToDevice, s), "copy b");
    } else {
      ProfScope ps(ctx_, Context::PROF_GMRES, 8.0 * double(N) * N);
      gemv(x, r, -1.0, 1.0, b, trans);
    }
    const double beta = norm(r);
    stats.final_rel_residual = beta / bnorm;
    if (beta / bnorm < gmres_tol) break;
    std::vector<double> H(static_cast<size_t>(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1, 0.0);
    g[0] = beta;
    copy_scaled(r, 1.0 / beta, V);
    int k = 0;
    for (; k < m; k++) {
      // w = A M^-1 v_k
      copy_scaled(V + static_cast<size_t>(k) * N, 1.0, r);
      solve_f32(r, trans);
      {
        ProfScope ps(ctx_, Context::PROF_GMRES, 8.0 * double(N) * N);
        gemv(r, w, 1.0, 0.0, nullptr, trans);
      }
      // two passes of w -= V (V^T w) over v_0 .. v_k, then |w|^2
      const int kk = k + 1;
      for (int pass = 0; pass < 2; pass++) {
        double* h = dproj + static_cast<size_t>(pass) * (m + 1);
        basis_dots<<<kk, VA_THREADS, 0, s>>>(V, N, kk, w, h);
        basis_subtract<<<nb, VA_THREADS, 0, s>>>(V, N, kk, h, w);
        ctx_->launches += 2;
      }
      sum_squares<<<1, VA_THREADS, 0, s>>>(w, N, dproj + hn_at);
      ctx_->launches++;
      cuda_check(cudaMemcpyAsync(hproj_, dproj, (hn_at + 1) * sizeof(double), cudaMemcpyDeviceToHost, s),
                 "D2H projections");
      cuda_check(cudaStreamSynchronize(s), "sync projections");
      const double hn = std::sqrt(hproj_[hn_at]);
      for (int i = 0; i <= k; i++) H[static_cast<size_t>(i) * m + k] = hproj_[i] + hproj_[m + 1 + i];
      H[static_cast<size_t>(k + 1) * m + k] = hn;
      if (hn > 0) copy_scaled(w, 1.0 / hn, V + static_cast<size_t>(k + 1) * N);
      for (int i = 0; i < k; i++) {
        const double t = cs[i] * H[i * m + k] + sn[i] * H[(i + 1) * m + k];
        H[(i + 1) * m + k] = -sn[i] * H[i * m + k] + cs[i] * H[(i + 1) * m + k];
        H[i * m + k] = t;
      }
      const double a = H[k * m + k], c = H[(k + 1) * m + k];
      const double d = std::sqrt(a * a + c * c);
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
    // y = H^-1 g, x += M^-1 V y
    std::vector<double> y(k, 0.0);
    for (int i = k - 1; i >= 0; i--) {
      double sum = g[i];
      for (int j = i + 1; j < k; j++) sum -= H[i * m + j] * y[j];
      y[i] = sum / H[i * m + i];
    }
    cuda_check(cudaMemsetAsync(r, 0, sizeof(double) * N, s), "memset r");
    for (int i = 0; i < k; i++) add_scaled(V + static_cast<size_t>(i) * N, y[i], r);
    solve_f32(r, trans);
    add_scaled(r, 1.0, x);
  }
  {
    ProfScope ps(ctx_, Context::PROF_GMRES, 8.0 * double(N) * N);
    gemv(x, r, -1.0, 1.0, b, trans);
  }
  stats.final_rel_residual = norm(r) / bnorm;
  stats.refine_iters = total_it;
  cuda_check(cudaMemcpyAsync(b, x, sizeof(double) * N, cudaMemcpyDeviceToDevice, s), "copy x");
}

void DenseLU::solve(double* b, int trans) {
  double t0 = now_ms();
  if (mode_ == LU_FP64) {
    solve_fp64(A_, ld_, N_, b, trans);
  } else if (trans) {
    // A^T x = b: GMRES on A^T preconditioned by the transposed factors
    // (no fallback to new factors: the caller decides)
    gmres_ir(b, 1);
    check_sweeps();
  } else {
    if (nopiv_) {
      ensure_bsave();
      cuda_check(cudaMemcpyAsync(bsave_, b, sizeof(double) * N_, cudaMemcpyDeviceToDevice, ctx_->stream()),
                 "keep right-hand side");
    }
    gmres_ir(b);
    check_sweeps();
    if (nopiv_) {
      if (!(stats.final_rel_residual < 1e-10)) {
        // the reused pivot order does not precondition this matrix: factor
        // it with partial pivoting and solve again
        stats.static_pivot_fallback = 1;
        perm_n_ = 0;
        factor_mixed(A_, ld_, N_, mode_, nullptr);
        const int info = read_info();
        if (info != 0)
          throw KdError(KD_ERR_SINGULAR, "Jacobian is singular (zero pivot at column " + std::to_string(info) + ")");
        perm_n_ = N_;
        cuda_check(cudaMemcpyAsync(b, bsave_, sizeof(double) * N_, cudaMemcpyDeviceToDevice, ctx_->stream()),
                   "restore right-hand side");
        gmres_ir(b);
        check_sweeps();
      } else if (stats.refine_iters > pivoted_iters_ + 4) {
        perm_n_ = 0;  // the order has drifted: the next factorisation pivots again
      }
    }
    if (!nopiv_) pivoted_iters_ = stats.refine_iters;
  }
  check_sweeps();
  if (mode_ != LU_FP64 && !(stats.final_rel_residual < 1e-10))
    throw KdError(KD_ERR_NOCONV, "GMRES-IR did not converge (relative residual " +
                                     std::to_string(stats.final_rel_residual) + ")");
  stats.t_solve_ms = now_ms() - t0;
}

}  // namespace kd
