// FP64 kernels for the spectral layer: fused separable transforms (one CTA
// per field, the field staged whole in shared memory), elementwise algebra
// on collocation values, and the sparse gathers used by the tau/Galerkin
// export.  All arithmetic is FP64, as in the reference.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "kd_device.hpp"

namespace kd {

namespace {

__device__ __forceinline__ int line_matrix(const KdPass& p, int c1, int c2) {
  if (p.dim == 0) return p.mat[c1 * p.mat_ld + c2];
  if (p.dim == 1) return p.mat[c2];
  return p.mat[0];
}

// One pass: X has dims (d0,d1,d2); Y has the pass dim replaced by n_out.
// Outputs e = e0 + threadIdx.x + k * estride; store(e, value) writes them.
template <class Store>
__device__ void run_pass_part(const KdPass& p, const double* __restrict__ X, int d0, int d1, int d2,
                              const double* __restrict__ pool, double scale, int e0, int estride, Store store) {
  int o0 = d0, o1 = d1, o2 = d2;
  if (p.dim == 0) o0 = p.n_out;
  if (p.dim == 1) o1 = p.n_out;
  if (p.dim == 2) o2 = p.n_out;
  const int total = o0 * o1 * o2;
  const int nin = p.n_in;
  for (int e = e0 + threadIdx.x; e < total; e += estride) {
    int c2 = e % o2;
    int t = e / o2;
    int c1 = t % o1;
    int c0 = t / o1;
    int row, off, base, stride;
    if (p.dim == 0) {
      row = c0;
      off = line_matrix(p, c1, c2);
      base = c1 * d2 + c2;
      stride = d1 * d2;
    } else if (p.dim == 1) {
      row = c1;
      off = line_matrix(p, c0, c2);
      base = c0 * d1 * d2 + c2;
      stride = d2;
    } else {
      row = c2;
      off = line_matrix(p, c0, c1);
      base = (c0 * d1 + c1) * d2;
      stride = 1;
    }
    double acc = 0.0;
    if (off >= 0) {
      const double* M = pool + off + static_cast<long long>(row) * nin;
#pragma unroll 4
      for (int q = 0; q < nin; q++) acc = fma(__ldg(M + q), X[base + q * stride], acc);
    }
    store(e, acc * scale);
  }
}

__device__ void run_pass(const KdPass& p, const double* __restrict__ X, double* __restrict__ Y, int d0, int d1,
                         int d2, const double* __restrict__ pool, double scale) {
  run_pass_part(p, X, d0, d1, d2, pool, scale, 0, blockDim.x, [Y](int e, double v) { Y[e] = v; });
}

__global__ void line_passes_kernel(const __grid_constant__ KdItemList list, const double* __restrict__ pool) {
  extern __shared__ double smem[];
  const int total_fields = list.prefix[list.nitems];
  // Grid-stride over fields so that any grid size covers the work.
  for (int f = blockIdx.x; f < total_fields; f += gridDim.x) {
    int item = 0;
    while (item + 1 < list.nitems && list.prefix[item + 1] <= f) item++;
    const KdItem& it = list.items[item];
    const int field_in_item = f - list.prefix[item];
    const int n_in_elems = it.n0 * it.n1 * it.n2;
    // Buffer sizes: every stage fits in half of the dynamic shared memory.
    int d0 = it.n0, d1 = it.n1, d2 = it.n2;
    int maxe = n_in_elems;
    {
      int e0 = d0, e1 = d1, e2 = d2;
      for (int q = 0; q < it.npass; q++) {
        if (it.pass[q].dim == 0) e0 = it.pass[q].n_out;
        if (it.pass[q].dim == 1) e1 = it.pass[q].n_out;
        if (it.pass[q].dim == 2) e2 = it.pass[q].n_out;
        int e = e0 * e1 * e2;
        if (e > maxe) maxe = e;
      }
    }
    double* bufA = smem;
    double* bufB = smem + maxe;
    const double* src = it.in + static_cast<long long>(field_in_item) * it.in_stride;
    double* dst = it.out + static_cast<long long>(field_in_item) * it.out_stride;
    for (int e = threadIdx.x; e < n_in_elems; e += blockDim.x) bufA[e] = src[e];
    __syncthreads();
    double* X = bufA;
    double* Y = bufB;
    for (int q = 0; q < it.npass; q++) {
      const KdPass& p = it.pass[q];
      bool last = (q == it.npass - 1);
      int o0 = d0, o1 = d1, o2 = d2;
      if (p.dim == 0) o0 = p.n_out;
      if (p.dim == 1) o1 = p.n_out;
      if (p.dim == 2) o2 = p.n_out;
      // The last pass writes straight to global memory.
      run_pass(p, X, last ? dst : Y, d0, d1, d2, pool, last ? it.scale : 1.0);
      __syncthreads();
      d0 = o0;
      d1 = o1;
      d2 = o2;
      double* tmp = X;
      X = Y;
      Y = tmp;
    }
    if (it.npass == 0) {
      for (int e = threadIdx.x; e < n_in_elems; e += blockDim.x) dst[e] = bufA[e] * it.scale;
    }
    __syncthreads();
  }
}

// Small batches: one LP_CL-CTA cluster per field.  Each CTA computes every
// LP_CL-th block of a pass's outputs and stores them into all the cluster's
// shared buffers (distributed shared memory), then one cluster barrier; the
// last pass writes straight to global memory.  A field's FP64 work is spread
// over LP_CL SMs instead of one.
constexpr int LP_CLUSTER_MAX_FIELDS = 32;
template <int LP_CL>
__global__ void line_passes_cluster_kernel(const __grid_constant__ KdItemList list, const double* __restrict__ pool) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ double smem[];
  const int rank = static_cast<int>(cluster.block_rank());
  const int f = blockIdx.x / LP_CL;
  int item = 0;
  while (item + 1 < list.nitems && list.prefix[item + 1] <= f) item++;
  const KdItem& it = list.items[item];
  const int field_in_item = f - list.prefix[item];
  const int n_in_elems = it.n0 * it.n1 * it.n2;
  int d0 = it.n0, d1 = it.n1, d2 = it.n2;
  int maxe = n_in_elems;
  {
    int e0 = d0, e1 = d1, e2 = d2;
    for (int q = 0; q < it.npass; q++) {
      if (it.pass[q].dim == 0) e0 = it.pass[q].n_out;
      if (it.pass[q].dim == 1) e1 = it.pass[q].n_out;
      if (it.pass[q].dim == 2) e2 = it.pass[q].n_out;
      int e = e0 * e1 * e2;
      if (e > maxe) maxe = e;
    }
  }
  double* bufA = smem;
  double* bufB = smem + maxe;
  const double* src = it.in + static_cast<long long>(field_in_item) * it.in_stride;
  double* dst = it.out + static_cast<long long>(field_in_item) * it.out_stride;
  for (int e = threadIdx.x; e < n_in_elems; e += blockDim.x) bufA[e] = src[e];
  __syncthreads();
  double* X = bufA;
  double* Y = bufB;
  const int e0 = rank * blockDim.x, estride = LP_CL * blockDim.x;
  for (int q = 0; q < it.npass; q++) {
    const KdPass& p = it.pass[q];
    const bool last = (q == it.npass - 1);
    int o0 = d0, o1 = d1, o2 = d2;
    if (p.dim == 0) o0 = p.n_out;
    if (p.dim == 1) o1 = p.n_out;
    if (p.dim == 2) o2 = p.n_out;
    if (last) {
      const double sc = it.scale;
      run_pass_part(p, X, d0, d1, d2, pool, sc, e0, estride, [dst](int e, double v) { dst[e] = v; });
    } else {
      double* Yr[LP_CL];
      for (int r = 0; r < LP_CL; r++) Yr[r] = cluster.map_shared_rank(Y, r);
      run_pass_part(p, X, d0, d1, d2, pool, 1.0, e0, estride, [&Yr](int e, double v) {
#pragma unroll
        for (int r = 0; r < LP_CL; r++) Yr[r][e] = v;
      });
      cluster.sync();  // every CTA's Y is complete and nobody reads X any more
    }
    d0 = o0;
    d1 = o1;
    d2 = o2;
    double* tmp = X;
    X = Y;
    Y = tmp;
  }
  if (it.npass == 0) {
    if (rank == 0)
      for (int e = threadIdx.x; e < n_in_elems; e += blockDim.x) dst[e] = bufA[e] * it.scale;
  }
}

__global__ void ew_kernel(int op, long long npts, long long total, int ba, const double* __restrict__ a,
                          int bb, const double* __restrict__ b, double* __restrict__ out, double alpha,
                          double beta) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    long long p = i % npts;
    double x = (a != nullptr) ? a[ba == 1 ? p : i] : 0.0;
    double y = (b != nullptr) ? b[bb == 1 ? p : i] : 0.0;
    double r;
    switch (op) {
      case EW_ADD: r = x + y; break;
      case EW_SUB: r = x - y; break;
      case EW_MUL: r = x * y; break;
      case EW_DIV: r = x / y; break;
      case EW_AXPBY: r = alpha * x + beta * y; break;
      case EW_SCALE: r = alpha * x; break;
      case EW_ADDC: r = x + alpha; break;
      case EW_CSUB: r = alpha - x; break;
      case EW_CDIV: r = alpha / x; break;
      case EW_POWD: r = pow(x, alpha); break;
      case EW_EXP: r = exp(x); break;
      case EW_LOG: r = log(x); break;
      case EW_SQRT: r = sqrt(x); break;
      case EW_SIN: r = sin(x); break;
      case EW_COS: r = cos(x); break;
      case EW_NEG: r = -x; break;
      case EW_FILL: r = alpha; break;
      case EW_COPY: r = x; break;
      case EW_POWI: r = pow(x, alpha); break;
      case EW_ATAN: r = atan(x); break;
      case EW_MULC_ADD: r = x * y * alpha; break;
      case EW_DIVC: r = x / alpha; break;
      case EW_COSH: r = cosh(x); break;
      case EW_SINH: r = sinh(x); break;
      case EW_ATANH: r = atanh(x); break;
      default: r = 0.0; break;
    }
    out[i] = r;
  }
}

__global__ void gather_csr_kernel(const double* __restrict__ in, long long in_stride, int batch, int nrows,
                                  const int* __restrict__ rowptr, const int* __restrict__ idx,
                                  const double* __restrict__ w, double* __restrict__ out, long long osf,
                                  long long osr, double alpha, int accumulate) {
  long long total = static_cast<long long>(batch) * nrows;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    int r = static_cast<int>(t % nrows);
    long long f = t / nrows;
    const double* src = in + f * in_stride;
    double acc = 0.0;
    for (int e = rowptr[r]; e < rowptr[r + 1]; e++) acc = fma(w[e], src[idx[e]], acc);
    double* dst = out + f * osf + r * osr;
    if (accumulate) *dst += alpha * acc; else *dst = alpha * acc;
  }
}

__global__ void scatter_seeds_kernel(double* out, long long stride, int nent, const int* seed, const int* pos,
                                     const double* w) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nent; e += gridDim.x * blockDim.x)
    out[seed[e] * stride + pos[e]] = w[e];
}

__global__ void absmax_kernel(const double* __restrict__ x, long long n, double* out) {
  __shared__ double red[32];
  double m = 0.0;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double a = fabs(x[i]);
    m = (a == a) ? fmax(m, a) : INFINITY;  // NaN counts as infinite (fmax would drop it)
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) {
      // Non-negative doubles order like their bit patterns.
      atomicMax(reinterpret_cast<unsigned long long*>(out), __double_as_longlong(m));
    }
  }
}

template <int CL>
cudaError_t launch_lp_cluster(const KdItemList& list, int total_fields, size_t smem, const double* d_pool,
                              cudaStream_t s) {
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(line_passes_cluster_kernel<CL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(total_fields * CL, 1, 1);
  cfg.blockDim = dim3(128, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaError_t e = cudaLaunchKernelEx(&cfg, line_passes_cluster_kernel<CL>, list, d_pool);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

int grid_for(long long n, int threads) {
  long long g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > 152 * 16) g = 152 * 16;
  return static_cast<int>(g);
}

}  // namespace

LpShape lp_default_shape(int total_fields) {
  LpShape sh;
  if (total_fields <= LP_CLUSTER_MAX_FIELDS) sh.cluster = 8;
  return sh;
}

cudaError_t launch_line_passes(const KdItemList& list, int smem_doubles, const double* d_pool, cudaStream_t s,
                               LpShape shape) {
  const int total_fields = list.prefix[list.nitems];
  if (total_fields <= 0) return cudaSuccess;
  size_t smem = static_cast<size_t>(smem_doubles) * 2 * sizeof(double);
  switch (shape.cluster) {
    case 2: return launch_lp_cluster<2>(list, total_fields, smem, d_pool, s);
    case 4: return launch_lp_cluster<4>(list, total_fields, smem, d_pool, s);
    case 8: return launch_lp_cluster<8>(list, total_fields, smem, d_pool, s);
    default: break;
  }
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(line_passes_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
  }
  const int threads = (shape.threads == 64 || shape.threads == 256) ? shape.threads : 128;
  int grid = total_fields < 152 * 8 ? total_fields : 152 * 8;
  line_passes_kernel<<<grid, threads, smem, s>>>(list, d_pool);
  return cudaGetLastError();
}

cudaError_t launch_line_passes(const KdItemList& list, int smem_doubles, const double* d_pool,
                               cudaStream_t s) {
  return launch_line_passes(list, smem_doubles, d_pool, s, lp_default_shape(list.prefix[list.nitems]));
}

cudaError_t launch_ew(int op, long long npts, int ba, const double* a, int bb, const double* b, double* out,
                      double alpha, double beta, cudaStream_t s) {
  int nf = ba > bb ? ba : bb;
  if (nf < 1) nf = 1;
  long long total = npts * nf;
  if (total <= 0) return cudaSuccess;
  ew_kernel<<<grid_for(total, 256), 256, 0, s>>>(op, npts, total, ba, a, bb, b, out, alpha, beta);
  return cudaGetLastError();
}

cudaError_t launch_gather_csr(const double* in, long long in_stride, int batch, int nrows, const int* rowptr,
                              const int* idx, const double* w, double* out, long long osf, long long osr,
                              double alpha, int accumulate, cudaStream_t s) {
  long long total = static_cast<long long>(batch) * nrows;
  if (total <= 0) return cudaSuccess;
  gather_csr_kernel<<<grid_for(total, 256), 256, 0, s>>>(in, in_stride, batch, nrows, rowptr, idx, w, out, osf, osr,
                                                        alpha, accumulate);
  return cudaGetLastError();
}

cudaError_t launch_scatter_seeds(double* out, long long stride, int nent, const int* seed, const int* pos,
                                 const double* w, cudaStream_t s) {
  if (nent <= 0) return cudaSuccess;
  scatter_seeds_kernel<<<grid_for(nent, 256), 256, 0, s>>>(out, stride, nent, seed, pos, w);
  return cudaGetLastError();
}

// One CTA, fixed summation order (deterministic): op 0 = sum of squares,
// op 1 = maximum (signed).
__global__ void reduce1_kernel(const double* __restrict__ x, long long n, int op, double* out) {
  __shared__ double part[1024];
  double acc = op == 0 ? 0.0 : -INFINITY;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) acc = op == 0 ? fma(x[i], x[i], acc) : fmax(acc, x[i]);
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (static_cast<int>(threadIdx.x) < w)
      part[threadIdx.x] = op == 0 ? part[threadIdx.x] + part[threadIdx.x + w] : fmax(part[threadIdx.x], part[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = part[0];
}

cudaError_t launch_reduce1(const double* x, long long n, int op, double* out_scalar, cudaStream_t s) {
  reduce1_kernel<<<1, 1024, 0, s>>>(x, n, op, out_scalar);
  return cudaGetLastError();
}

__global__ void lincomb2_kernel(int n, double ca, const double* __restrict__ a, double as, double cb,
                                const double* __restrict__ b, double bs, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = ca * (a ? a[i] : as) + cb * (b ? b[i] : bs);
}

cudaError_t launch_lincomb2(int n, double ca, const double* a, double as, double cb, const double* b, double bs,
                            double* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  lincomb2_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, ca, a, as, cb, b, bs, out);
  return cudaGetLastError();
}

__global__ void first_integral_kernel(int B, int npts, int n0, const double* __restrict__ v, long long vs,
                                      const double* __restrict__ ori, long long os, int inject,
                                      const double* __restrict__ cst, long long cs, double cst_scalar,
                                      double* __restrict__ out) {
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= static_cast<long long>(B) * npts) return;
  const int b = static_cast<int>(i / npts), p = static_cast<int>(i % npts);
  double r;
  if (inject && p < n0) r = cst ? cst[b * cs] : cst_scalar;
  else r = (v ? v[b * vs + p] : 0.0) - (ori ? ori[b * os] : 0.0);
  out[i] = r;
}

cudaError_t launch_first_integral(int B, int npts, int n0, const double* v, long long vs, const double* ori,
                                  long long os, int inject, const double* cst, long long cs, double cst_scalar,
                                  double* out, cudaStream_t s) {
  const long long n = static_cast<long long>(B) * npts;
  if (n <= 0) return cudaSuccess;
  first_integral_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(B, npts, n0, v, vs, ori, os, inject,
                                                                              cst, cs, cst_scalar, out);
  return cudaGetLastError();
}

__device__ __forceinline__ double eos_clamp_rho(const KdEos& e, double rho) {
  return rho < e.rhomin ? e.rhomin : (rho > e.rhomax ? e.rhomax : rho);  // check_range
}

__device__ __forceinline__ int eos_piece_rho(const KdEos& e, double rho) {
  for (int nn = 1; nn < e.npieces; nn++)
    if (rho <= e.rho[nn] && rho > e.rho[nn - 1]) return nn - 1;
  return e.npieces - 1;
}

__device__ __forceinline__ double eos_rho_of_h(const KdEos& e, double h) {
  if (h <= 1.0) return e.rho[0];  // rho__h_cold range check
  int idx = e.npieces - 1;
  for (int nn = 1; nn < e.npieces; nn++)
    if (h <= e.h[nn] && h > e.h[nn - 1]) {
      idx = nn - 1;
      break;
    }
  const double gm1 = e.gamma[idx] - 1.0;
  double rho = pow(gm1 * (h - 1.0 - e.eps[idx]) / (e.gamma[idx] * e.k[idx]), 1.0 / gm1);
  return eos_clamp_rho(e, rho);
}

// press_cold_eps_cold__rho and dpress_cold_drho__rho (both clamp rho first)
__device__ __forceinline__ double eos_press(const KdEos& e, double rho, double* eps_out) {
  rho = eos_clamp_rho(e, rho);
  const int i = eos_piece_rho(e, rho);
  const double p = e.k[i] * pow(rho, e.gamma[i]);
  if (eps_out) *eps_out = e.eps[i] + p / (rho * (e.gamma[i] - 1.0));
  return p;
}

__device__ __forceinline__ double eos_dpdrho(const KdEos& e, double rho) {
  rho = eos_clamp_rho(e, rho);
  const int i = eos_piece_rho(e, rho);
  return e.gamma[i] * e.k[i] * pow(rho, e.gamma[i]) / rho;
}

__global__ void eos_kernel(const __grid_constant__ KdEos e, int var, long long npts, const double* __restrict__ h,
                           int B, const double* __restrict__ dh, double* __restrict__ out) {
  const long long total = npts * (dh ? B : 1);
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long pt = t % npts;
    // rho__h_cold clamps h to 1 and the later calls clamp rho to
    // [rhomin, rhomax] in the caller's variables (all by reference)
    const double hv = h[pt] <= 1.0 ? 1.0 : h[pt];
    const double rho = eos_clamp_rho(e, eos_rho_of_h(e, h[pt]));
    double epsc = 0.0;
    const double p = eos_press(e, rho, &epsc);
    if (!dh) {
      double v;
      if (var == EOS_EPSILON) v = epsc;
      else if (var == EOS_DENSITY) v = rho;
      else if (var == EOS_PRESSURE) v = p;
      else v = 1.0 / hv * eos_dpdrho(e, rho);
      out[t] = v;
    } else {
      const double dpdrho = eos_dpdrho(e, rho);
      const double drho = rho * 1.0 / dpdrho * dh[t];
      double v;
      if (var == EOS_EPSILON) v = p / (rho * rho) * drho;
      else if (var == EOS_PRESSURE) v = dpdrho * drho;
      else if (var == EOS_DENSITY) v = drho;
      else v = 0.0;  // the reference sets the variation of dH/dln(rho) to zero
      out[t] = v;
    }
  }
}

cudaError_t launch_eos(const KdEos& eos, int var, long long npts, const double* h, int B, const double* dh,
                       double* out, cudaStream_t s) {
  const long long total = npts * (dh ? B : 1);
  if (total <= 0) return cudaSuccess;
  eos_kernel<<<grid_for(total, 256), 256, 0, s>>>(eos, var, npts, h, B, dh, out);
  return cudaGetLastError();
}

// One thread that idles for ns nanoseconds (at most 4096 sleeps of ~1 us).
__global__ void hold_kernel(unsigned long long ns) {
  unsigned long long t0, t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (int it = 0; it < 4096; it++) {
    __nanosleep(1000);
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 >= ns) break;
  }
}

cudaError_t launch_hold(unsigned long long ns, cudaStream_t s) {
  hold_kernel<<<1, 1, 0, s>>>(ns);
  return cudaGetLastError();
}

cudaError_t launch_absmax(const double* x, long long n, double* out_scalar, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out_scalar, 0, sizeof(double), s);
  if (e != cudaSuccess) return e;
  if (n <= 0) return cudaSuccess;
  absmax_kernel<<<grid_for(n, 256), 256, 0, s>>>(x, n, out_scalar);
  return cudaGetLastError();
}

}  // namespace kd
