// Device-side descriptors and kernel launchers (implemented in kd_device.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace kd {

// One 1-D pass of a separable operator over a 3-D block (r, theta, phi),
// phi fastest.  The matrix applied to a line is looked up per line:
//   dim 0 (r):     mat[j * mat_ld + k]   (basis depends on theta/phi indices)
//   dim 1 (theta): mat[k]                (basis depends on the phi index)
//   dim 2 (phi):   mat[0]
// An entry < 0 means "this line's output is zero".  Offsets are in doubles
// into the shared matrix pool; the matrix is row-major n_out x n_in.
struct KdPass {
  int dim;
  int n_in;
  int n_out;
  int mat_ld;
  const int* mat;
};

// A run of `batch` fields of identical shape processed by the same pass list.
struct KdItem {
  const double* in;
  double* out;
  long long in_stride;   // elements between consecutive fields of the batch
  long long out_stride;
  int n0, n1, n2;        // input dims
  int npass;
  double scale;          // applied to the final result
  KdPass pass[3];
};

// Up to KD_MAX_ITEMS runs packed in one launch (uneven domains together).
// Passed by value as a kernel parameter so that launches can be captured in
// a CUDA graph without staging descriptors through host memory.
constexpr int KD_MAX_ITEMS = 12;
struct KdItemList {
  int nitems;
  int prefix[KD_MAX_ITEMS + 1];  // prefix sums of batch sizes
  KdItem items[KD_MAX_ITEMS];
};

// Launch shape of a line-pass launch: one CTA of `threads` threads per field
// (cluster = 1), or a cluster of `cluster` CTAs (2, 4 or 8) of 128 threads
// per field, each CTA computing every cluster-th block of a pass's outputs.
// Every output value is summed in the same order whatever the shape, so the
// shape changes no result bit.
struct LpShape {
  int cluster = 1;
  int threads = 128;
};
// The rule without a tuning table: 8-CTA clusters up to 32 fields, else one
// 128-thread CTA per field.
LpShape lp_default_shape(int total_fields);

// Runs the pass lists of all items with the given shape (default rule: the
// overload without one).
cudaError_t launch_line_passes(const KdItemList& list, int smem_doubles, const double* d_pool,
                               cudaStream_t s, LpShape shape);
cudaError_t launch_line_passes(const KdItemList& list, int smem_doubles, const double* d_pool,
                               cudaStream_t s);

// Elementwise ops on fields of npts values. a has ba fields, b has bb fields
// (ba, bb in {1, B}); out has max(ba, bb) fields.
enum EwOp : int {
  EW_ADD = 0,    // a + b
  EW_SUB = 1,    // a - b
  EW_MUL = 2,    // a * b
  EW_DIV = 3,    // a / b
  EW_AXPBY = 4,  // alpha*a + beta*b
  EW_SCALE = 5,  // alpha*a
  EW_ADDC = 6,   // a + alpha
  EW_CSUB = 7,   // alpha - a
  EW_CDIV = 8,   // alpha / a
  EW_POWD = 9,   // pow(a, alpha)
  EW_EXP = 10,
  EW_LOG = 11,
  EW_SQRT = 12,
  EW_SIN = 13,
  EW_COS = 14,
  EW_NEG = 15,
  EW_FILL = 16,  // alpha
  EW_COPY = 17,  // a
  EW_POWI = 18,  // pow(a, (int)alpha) for alpha <= 0 (reference uses std::pow)
  EW_ATAN = 19,
  EW_MULC_ADD = 20,  // out = a*b*alpha (product with constant)
  EW_DIVC = 21,      // a / alpha (Val_domain / double divides, it does not scale by 1/alpha)
  EW_COSH = 22,
  EW_SINH = 23,
  EW_ATANH = 24,
};

cudaError_t launch_ew(int op, long long npts, int ba, const double* a, int bb, const double* b,
                      double* out, double alpha, double beta, cudaStream_t s);

// Sparse row gather (CSR): for each field f of the batch and row r,
//   out[f*osf + r*osr] (+)= alpha * sum_{e in [rowptr[r], rowptr[r+1])} w[e] * in[f*in_stride + idx[e]]
// in_stride = 0 broadcasts one input field to every output field.
cudaError_t launch_gather_csr(const double* in, long long in_stride, int batch, int nrows, const int* rowptr,
                              const int* idx, const double* w, double* out, long long osf, long long osr,
                              double alpha, int accumulate, cudaStream_t s);

// Sum over the last axis reduction helpers used by residual norms.
cudaError_t launch_absmax(const double* x, long long n, double* out_scalar, cudaStream_t s);
// Occupies the stream for about ns nanoseconds (profile mode queues the
// launches it times behind it, so that their event pairs see no host gaps).
cudaError_t launch_hold(unsigned long long ns, cudaStream_t s);
// Cold piecewise polytrope (Margherita Cold_PWPoly, include/EOS/standalone/
// cold_pwpoly_implementation.hh), geometrised units, tables derived as in
// Margherita_setup_polytrope (setup_polytrope.cc).
constexpr int KD_EOS_MAX_PIECES = 8;
struct KdEos {
  int npieces;
  double rhomin, rhomax;
  double k[KD_EOS_MAX_PIECES], gamma[KD_EOS_MAX_PIECES], rho[KD_EOS_MAX_PIECES], eps[KD_EOS_MAX_PIECES],
      h[KD_EOS_MAX_PIECES];
};
enum EosVar : int { EOS_EPSILON = 0, EOS_PRESSURE = 1, EOS_DENSITY = 2, EOS_DHDRHO = 3 };
// Value (dh == nullptr): out = var(h) pointwise (EOS::term_by_term).
// Variation: out[b] = d var for the tangent batch dh (B fields) at h
// (EOS::term_by_term_variation, include/EOS/EOS.hh:67-160).
cudaError_t launch_eos(const KdEos& eos, int var, long long npts, const double* h, int B, const double* dh,
                       double* out, cudaStream_t s);

// Deterministic single-CTA reduction: op 0 = sum of squares, 1 = max.
cudaError_t launch_reduce1(const double* x, long long n, int op, double* out_scalar, cudaStream_t s);
// out[i] = ca * (a ? a[i] : as) + cb * (b ? b[i] : bs), i < n: the tangent of
// a linear combination of doubles whose tangents differ from seed to seed.
cudaError_t launch_lincomb2(int n, double ca, const double* a, double as, double cb, const double* b, double bs,
                            double* out, cudaStream_t s);

// The first integral's residual in one domain (Eq_first_integral::export_val /
// export_der, src/Equation/eq_first_integral.cpp:44-120), for B seeds:
//   out[b][p] = (v ? v[b*vs + p] : 0) - (ori ? ori[b*os] : 0),
// and, when inject != 0, the first n0 points (radial index 0) replaced by
// (cst ? cst[b*cs] : cst_scalar).  All arrays at the collocation points.
cudaError_t launch_first_integral(int B, int npts, int n0, const double* v, long long vs, const double* ori,
                                  long long os, int inject, const double* cst, long long cs, double cst_scalar,
                                  double* out, cudaStream_t s);

}  // namespace kd
