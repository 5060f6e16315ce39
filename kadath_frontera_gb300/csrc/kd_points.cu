// Spectral summation at arbitrary points (Scalar::val_point,
// include/scalar.hpp:221; Base_spectral::summation, src/Ope_1d/summation_1d.cpp)
// for many points and several fields at once: the step the reference's
// exporters (src/Utilities/Exporters) run point by point on the host.
//
// One thread per point.  The point is located (the first domain whose radial
// range holds it, as Space::locate), turned into numerical coordinates
// (xi, theta, phi), and every field is summed there:
//   sum_k Phi_k(phi) sum_j Theta_jk(theta) sum_i c_ijk R_ijk(xi)
// with the radial sums by Clenshaw's recurrence (T_2i(x) = T_i(2x^2 - 1) for
// the even basis), and the trigonometric factors by rotation of (cos, sin)
// pairs, so that no basis table is stored per thread.  Coefficients are read
// through the read-only cache: every thread of a domain reads the same lines.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <vector>

#include "kd_points.hpp"

namespace kd {

namespace {

struct PtDom {
  int type;
  double alpha, beta, rin, rout;
  int nc0, nc1, nc2;
};

struct PtArgs {
  int ndom, nfields;
  double cx, cy, cz;
  PtDom d[PT_MAX_DOM];
  // per (field, domain): offsets of the coefficients in `cf` and of the
  // basis tables (r: nc1*nc2 codes, then t: nc2 codes, then p) in `tab`
  int cf_off[PT_MAX_FIELDS][PT_MAX_DOM];
  int tab_off[PT_MAX_FIELDS][PT_MAX_DOM];
};

constexpr int B_CHEB = 1, B_CHEB_EVEN = 2, B_CHEB_ODD = 3;
constexpr int B_COS_EVEN = 6, B_COS_ODD = 7, B_SIN_EVEN = 9, B_SIN_ODD = 10;

// sum_{i < n} c[i * stride] T_i(y)
__device__ __forceinline__ double clenshaw(const double* __restrict__ c, int stride, int n, double y) {
  double b1 = 0.0, b2 = 0.0;
  for (int i = n - 1; i >= 1; i--) {
    const double b0 = fma(2.0 * y, b1, __ldg(c + static_cast<long long>(i) * stride) - b2);
    b2 = b1;
    b1 = b0;
  }
  return fma(y, b1, __ldg(c) - b2);
}

// sum_{i < n} c[i * stride] T_{2i+1}(x), as the full series with zero even terms
__device__ __forceinline__ double clenshaw_odd(const double* __restrict__ c, int stride, int n, double x) {
  double b1 = 0.0, b2 = 0.0;
  for (int m = 2 * n - 1; m >= 1; m--) {
    const double a = (m & 1) ? __ldg(c + static_cast<long long>(m >> 1) * stride) : 0.0;
    const double b0 = fma(2.0 * x, b1, a - b2);
    b2 = b1;
    b1 = b0;
  }
  return x * b1 - b2;  // a_0 = 0
}

__global__ void __launch_bounds__(256) val_points_kernel(PtArgs a, const double* __restrict__ cf,
                                                         const int* __restrict__ tab, long long npts,
                                                         const double* __restrict__ xyz, double* __restrict__ out) {
  for (long long p = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; p < npts;
       p += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double x = xyz[3 * p] - a.cx, y = xyz[3 * p + 1] - a.cy, z = xyz[3 * p + 2] - a.cz;
    const double r = sqrt(x * x + y * y + z * z);
    int dd = -1;
    for (int d = 0; d < a.ndom; d++)
      if (a.d[d].rin - 1e-12 <= r && r <= a.d[d].rout + 1e-12) {
        dd = d;
        break;
      }
    if (dd < 0) {
      for (int f = 0; f < a.nfields; f++) out[f * npts + p] = nan("");
      continue;
    }
    const PtDom& D = a.d[dd];
    double xi;
    if (D.type == 1) xi = r / D.alpha;
    else if (D.type == 2) xi = (r - D.beta) / D.alpha;
    else xi = 1.0 + 1.0 / r / D.alpha;
    const double rho = sqrt(x * x + y * y);
    double th, ph;
    if (rho == 0.0) {
      th = (z >= 0) ? 0.0 : M_PI;
      ph = 0.0;
    } else {
      th = (z != 0.0) ? atan(rho / z) : M_PI / 2;
      ph = atan2(y, x);
    }
    if (th < 0) th += M_PI;
    double st1, ct1, st2, ct2, sp1, cp1;
    sincos(th, &st1, &ct1);
    sincos(2.0 * th, &st2, &ct2);
    sincos(ph, &sp1, &cp1);
    const double y2 = fma(2.0 * xi, xi, -1.0);
    const int lstride = D.nc1 * D.nc2;
    for (int f = 0; f < a.nfields; f++) {
      const double* c = cf + a.cf_off[f][dd];
      const int* rb = tab + a.tab_off[f][dd];
      const int* tb = rb + lstride;
      double val = 0.0;
      double cm = 1.0, sm = 0.0;  // cos(m phi), sin(m phi), m = k / 2 (COSSIN)
      for (int k = 0; k < D.nc2; k++) {
        const double phik = (k & 1) ? sm : cm;
        if (k & 1) {  // advance m
          const double cn = cm * cp1 - sm * sp1;
          sm = sm * cp1 + cm * sp1;
          cm = cn;
        }
        if (phik == 0.0) continue;
        const int bt = __ldg(tb + k);
        // first angle of the theta series and its step (2 theta)
        double ct, st;
        if (bt == B_COS_EVEN || bt == B_SIN_EVEN) {
          ct = 1.0;
          st = 0.0;
        } else {
          ct = ct1;
          st = st1;
        }
        const bool use_cos = (bt == B_COS_EVEN || bt == B_COS_ODD);
        double acc = 0.0;
        for (int j = 0; j < D.nc1; j++) {
          const double thj = use_cos ? ct : st;
          const int br = __ldg(rb + j * D.nc2 + k);
          const double* line = c + j * D.nc2 + k;
          double rad;
          if (br == B_CHEB) rad = clenshaw(line, lstride, D.nc0, xi);
          else if (br == B_CHEB_EVEN) rad = clenshaw(line, lstride, D.nc0, y2);
          else rad = clenshaw_odd(line, lstride, D.nc0, xi);
          acc = fma(thj, rad, acc);
          const double cn = ct * ct2 - st * st2;
          st = st * ct2 + ct * st2;
          ct = cn;
        }
        val = fma(phik, acc, val);
      }
      out[f * npts + p] = val;
    }
  }
}

// ---- sorted evaluation with a per-point Chebyshev table -------------------
// Points are first classified (domain, numerical coordinates) and grouped
// by domain, so that the threads of a warp run the same loops over the same
// coefficients.  Each thread then tabulates T_n(xi), n < 2 nc0, once (three
// term recurrence) in shared memory, and every radial line is a plain dot
// product with its coefficients: one FP64 multiply-add per coefficient
// instead of Clenshaw's two operations.
constexpr int PT_TAB = 64;      // T_0 .. T_63: radial resolutions up to 32
constexpr int PT_THREADS = 128;

__global__ void pt_classify(PtArgs a, long long npts, const double* __restrict__ xyz, double* __restrict__ num,
                            int* __restrict__ dom, int* __restrict__ count) {
  for (long long p = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; p < npts;
       p += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double x = xyz[3 * p] - a.cx, y = xyz[3 * p + 1] - a.cy, z = xyz[3 * p + 2] - a.cz;
    const double r = sqrt(x * x + y * y + z * z);
    int dd = -1;
    for (int d = 0; d < a.ndom; d++)
      if (a.d[d].rin - 1e-12 <= r && r <= a.d[d].rout + 1e-12) {
        dd = d;
        break;
      }
    const int bucket = (dd < 0) ? a.ndom : dd;  // points in no domain last
    dom[p] = dd;
    atomicAdd(count + bucket, 1);
    if (dd < 0) continue;
    const PtDom& D = a.d[dd];
    double xi;
    if (D.type == 1) xi = r / D.alpha;
    else if (D.type == 2) xi = (r - D.beta) / D.alpha;
    else xi = 1.0 + 1.0 / r / D.alpha;
    const double rho = sqrt(x * x + y * y);
    double th, ph;
    if (rho == 0.0) {
      th = (z >= 0) ? 0.0 : M_PI;
      ph = 0.0;
    } else {
      th = (z != 0.0) ? atan(rho / z) : M_PI / 2;
      ph = atan2(y, x);
    }
    if (th < 0) th += M_PI;
    num[3 * p] = xi;
    num[3 * p + 1] = th;
    num[3 * p + 2] = ph;
  }
}

// Exclusive scan of the (ndom + 1) bucket counts into two copies of the
// offsets (one is advanced by the scatter).
__global__ void pt_offsets(const int* __restrict__ count, int nb, int* __restrict__ off, int* __restrict__ cursor) {
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int b = 0; b < nb; b++) {
      off[b] = acc;
      cursor[b] = acc;
      acc += count[b];
    }
  }
}

__global__ void pt_scatter(long long npts, const int* __restrict__ dom, int ndom, int* __restrict__ cursor,
                           int* __restrict__ perm) {
  for (long long p = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; p < npts;
       p += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int d = dom[p];
    perm[atomicAdd(cursor + ((d < 0) ? ndom : d), 1)] = static_cast<int>(p);
  }
}

__global__ void __launch_bounds__(PT_THREADS) val_points_sorted_kernel(PtArgs a, const double* __restrict__ cf,
                                                                       const int* __restrict__ tab, long long npts,
                                                                       const int* __restrict__ perm,
                                                                       const int* __restrict__ dom,
                                                                       const double* __restrict__ num,
                                                                       double* __restrict__ out) {
  extern __shared__ double pt_T[];  // T_n(xi) of thread t at pt_T[n * PT_THREADS + t]
  const int tid = threadIdx.x;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + tid; t < npts;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int p = perm[t];
    const int dd = dom[p];
    if (dd < 0) {
      for (int f = 0; f < a.nfields; f++) out[f * npts + p] = nan("");
      continue;
    }
    const PtDom& D = a.d[dd];
    const double xi = num[3 * p], th = num[3 * p + 1], ph = num[3 * p + 2];
    {
      double tm2 = 1.0, tm1 = xi;
      pt_T[tid] = 1.0;
      pt_T[PT_THREADS + tid] = xi;
      for (int n = 2; n < 2 * D.nc0; n++) {
        const double tn = fma(2.0 * xi, tm1, -tm2);
        pt_T[n * PT_THREADS + tid] = tn;
        tm2 = tm1;
        tm1 = tn;
      }
    }
    double st1, ct1, st2, ct2, sp1, cp1;
    sincos(th, &st1, &ct1);
    sincos(2.0 * th, &st2, &ct2);
    sincos(ph, &sp1, &cp1);
    const int lstride = D.nc1 * D.nc2;
    for (int f = 0; f < a.nfields; f++) {
      const double* c = cf + a.cf_off[f][dd];
      const int* rb = tab + a.tab_off[f][dd];
      const int* tb = rb + lstride;
      double val = 0.0;
      double cm = 1.0, sm = 0.0;  // cos(m phi), sin(m phi), m = k / 2 (COSSIN)
      for (int k = 0; k < D.nc2; k++) {
        const double phik = (k & 1) ? sm : cm;
        if (k & 1) {
          const double cn = cm * cp1 - sm * sp1;
          sm = sm * cp1 + cm * sp1;
          cm = cn;
        }
        if (phik == 0.0) continue;
        const int bt = __ldg(tb + k);
        double ct, st;
        if (bt == B_COS_EVEN || bt == B_SIN_EVEN) {
          ct = 1.0;
          st = 0.0;
        } else {
          ct = ct1;
          st = st1;
        }
        const bool use_cos = (bt == B_COS_EVEN || bt == B_COS_ODD);
        double acc = 0.0;
        for (int j = 0; j < D.nc1; j++) {
          const double thj = use_cos ? ct : st;
          const int br = __ldg(rb + j * D.nc2 + k);
          const int ts = (br == B_CHEB) ? 1 : 2, t0 = (br == B_CHEB_ODD) ? 1 : 0;
          const double* line = c + j * D.nc2 + k;
          double rad = 0.0;
          for (int i = 0; i < D.nc0; i++) rad = fma(__ldg(line + static_cast<long long>(i) * lstride), pt_T[(ts * i + t0) * PT_THREADS + tid], rad);
          acc = fma(thj, rad, acc);
          const double cn = ct * ct2 - st * st2;
          st = st * ct2 + ct * st2;
          ct = cn;
        }
        val = fma(phik, acc, val);
      }
      out[f * npts + p] = val;
    }
  }
}

}  // namespace

void fields_val_points(Context* ctx, const std::vector<const Field*>& fields, long long npts, const double* d_xyz,
                       double* d_out) {
  if (fields.empty() || npts <= 0) return;
  if (static_cast<int>(fields.size()) > PT_MAX_FIELDS)
    throw KdError(KD_ERR_ARG, "val_points: too many fields in one call");
  const Space* sp = fields[0]->sp;
  if (sp->ndom() > PT_MAX_DOM) throw KdError(KD_ERR_UNSUPPORTED, "val_points: too many domains");
  PtArgs a{};
  a.ndom = sp->ndom();
  a.nfields = static_cast<int>(fields.size());
  a.cx = sp->dom(0).center[0];
  a.cy = sp->dom(0).center[1];
  a.cz = sp->dom(0).center[2];
  for (int d = 0; d < a.ndom; d++) {
    const Domain& dm = sp->dom(d);
    a.d[d].type = dm.type;
    a.d[d].alpha = dm.alpha;
    a.d[d].beta = dm.beta;
    a.d[d].rin = dm.inner_radius();
    a.d[d].rout = dm.outer_radius();
    a.d[d].nc0 = dm.nc[0];
    a.d[d].nc1 = dm.nc[1];
    a.d[d].nc2 = dm.nc[2];
  }
  // gather every (field, domain) coefficient array and basis table
  std::vector<int> tab;
  long long ncf = 0;
  for (int f = 0; f < a.nfields; f++) {
    if (fields[f]->sp != sp) throw KdError(KD_ERR_ARG, "val_points: fields on different spaces");
    for (int d = 0; d < a.ndom; d++) {
      const Domain& dm = sp->dom(d);
      const Field::PerDom& pd = fields[f]->d[d];
      a.cf_off[f][d] = static_cast<int>(ncf);
      ncf += dm.ncoefs();
      a.tab_off[f][d] = static_cast<int>(tab.size());
      const Base b = (pd.zero || !pd.base.def) ? dm.std_base() : pd.base;
      if (b.p != KD_COSSIN) throw KdError(KD_ERR_UNSUPPORTED, "val_points: phi basis other than COSSIN");
      for (int code : b.r)
        if (code != KD_CHEB && code != KD_CHEB_EVEN && code != KD_CHEB_ODD)
          throw KdError(KD_ERR_UNSUPPORTED, "val_points: radial basis not handled");
      for (int code : b.t)
        if (code != KD_COS_EVEN && code != KD_COS_ODD && code != KD_SIN_EVEN && code != KD_SIN_ODD)
          throw KdError(KD_ERR_UNSUPPORTED, "val_points: theta basis not handled");
      tab.insert(tab.end(), b.r.begin(), b.r.end());
      tab.insert(tab.end(), b.t.begin(), b.t.end());
    }
  }
  if (ncf > (1LL << 31)) throw KdError(KD_ERR_ARG, "val_points: fields too large");
  cudaStream_t s = ctx->stream();
  DeviceArena& ar = ctx->scratch();
  const size_t mark = ar.mark();
  double* cf = ar.alloc_doubles(static_cast<size_t>(ncf));
  for (int f = 0; f < a.nfields; f++)
    for (int d = 0; d < a.ndom; d++) {
      const Domain& dm = sp->dom(d);
      double* dst = cf + a.cf_off[f][d];
      const Field::PerDom& pd = fields[f]->d[d];
      if (pd.zero) {
        cuda_check(cudaMemsetAsync(dst, 0, sizeof(double) * dm.ncoefs(), s), "memset coefficients");
        continue;
      }
      DVal v = fields[f]->val(d);
      v.coef();
      cuda_check(cudaMemcpyAsync(dst, v.cf, sizeof(double) * dm.ncoefs(), cudaMemcpyDeviceToDevice, s),
                 "copy coefficients");
    }
  const int* d_tab = ctx->table(tab);
  int nc0max = 0;
  for (int d = 0; d < a.ndom; d++) nc0max = (a.d[d].nc0 > nc0max) ? a.d[d].nc0 : nc0max;
  if (2 * nc0max <= PT_TAB && npts <= (1LL << 31) - 1) {
    // classify, group by domain, then evaluate with the Chebyshev table
    double* num = ar.alloc_doubles(static_cast<size_t>(3 * npts));
    int* dom = static_cast<int*>(ar.alloc_bytes(sizeof(int) * static_cast<size_t>(npts)));
    int* perm = static_cast<int*>(ar.alloc_bytes(sizeof(int) * static_cast<size_t>(npts)));
    int* cnt = static_cast<int*>(ar.alloc_bytes(sizeof(int) * 3 * (PT_MAX_DOM + 1)));
    int* off = cnt + (PT_MAX_DOM + 1);
    int* cursor = off + (PT_MAX_DOM + 1);
    cuda_check(cudaMemsetAsync(cnt, 0, sizeof(int) * (PT_MAX_DOM + 1), s), "memset counts");
    long long nb = (npts + 255) / 256;
    if (nb > 152LL * 16) nb = 152LL * 16;
    ProfScope ps(ctx, Context::PROF_LINE_PASS, 0.0);
    pt_classify<<<static_cast<int>(nb), 256, 0, s>>>(a, npts, d_xyz, num, dom, cnt);
    pt_offsets<<<1, 32, 0, s>>>(cnt, a.ndom + 1, off, cursor);
    pt_scatter<<<static_cast<int>(nb), 256, 0, s>>>(npts, dom, a.ndom, cursor, perm);
    long long ne = (npts + PT_THREADS - 1) / PT_THREADS;
    if (ne > 152LL * 12) ne = 152LL * 12;
    constexpr size_t tsmem = sizeof(double) * PT_TAB * PT_THREADS;
    static std::once_flag attr;
    std::call_once(attr, [] {
      cuda_check(cudaFuncSetAttribute(val_points_sorted_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(tsmem)),
                 "cudaFuncSetAttribute(val_points)");
    });
    val_points_sorted_kernel<<<static_cast<int>(ne), PT_THREADS, tsmem, s>>>(a, cf, d_tab, npts, perm, dom, num,
                                                                             d_out);
    ctx->launches += 4;
  } else {
    long long nb = (npts + 255) / 256;
    if (nb > 152LL * 16) nb = 152LL * 16;
    ProfScope ps(ctx, Context::PROF_LINE_PASS, 0.0);
    val_points_kernel<<<static_cast<int>(nb), 256, 0, s>>>(a, cf, d_tab, npts, d_xyz, d_out);
    ctx->launches++;
  }
  cuda_check(cudaGetLastError(), "val_points kernels");
  // the coefficient copies are read by the kernel: keep them until it ran
  cuda_check(cudaStreamSynchronize(s), "sync val_points");
  ar.release_to(mark);
}

}  // namespace kd
