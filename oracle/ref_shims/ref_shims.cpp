// Implementations behind the stand-in headers of this folder: the third-party
// entry points that the reference's own sources call on the serial Newton
// path (FFTW r2r, LAPACK dgetrf/dgetrs, GSL permutations and spherical Bessel
// functions, single-rank MPI).  Test infrastructure only: the oracle compiles
// the reference's sources against these to produce golden vectors; nothing in
// the product links them.
//
// Everything here is this project's own code written from the published
// definitions of each routine (FFTW's halfcomplex layout, LAPACK's getrf/getrs
// contract with idamax's first-maximum pivot rule, GSL's lexicographic
// permutation order).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fftw3.h"
#include "gsl/gsl_permutation.h"
#include "gsl/gsl_sf_bessel.h"
#include "mpi.h"

namespace {

[[noreturn]] void unsupported(const char* what) {
  std::fprintf(stderr, "ref_shims: %s is not provided by the oracle's shims\n", what);
  std::abort();
}

// cos/sin of 2 pi m / n with the argument reduced exactly (m taken mod n).
inline void twiddle(long long m, int n, long double& c, long double& s) {
  const long double two_pi = 6.283185307179586476925286766559005768L;
  long long r = m % n;
  long double a = two_pi * static_cast<long double>(r) / static_cast<long double>(n);
  c = cosl(a);
  s = sinl(a);
}

}  // namespace

// ---------------------------------------------------------------- FFTW r2r --

struct kd_shim_fftw_plan_s {
  int n;
  double* in;
  double* out;
  fftw_r2r_kind kind;
  std::vector<long double> cs, sn;  // cos/sin(2 pi m / n), m = 0..n-1
};

extern "C" double* fftw_alloc_real(unsigned long n) {
  void* p = nullptr;
  if (posix_memalign(&p, 64, (n ? n : 1) * sizeof(double)) != 0) return nullptr;
  return static_cast<double*>(p);
}

extern "C" void fftw_free(void* p) { std::free(p); }

extern "C" fftw_plan fftw_plan_r2r_1d(int n, double* in, double* out, fftw_r2r_kind kind, unsigned) {
  auto* p = new kd_shim_fftw_plan_s;
  p->n = n;
  p->in = in;
  p->out = out;
  p->kind = kind;
  p->cs.resize(n);
  p->sn.resize(n);
  for (int m = 0; m < n; m++) twiddle(m, n, p->cs[m], p->sn[m]);
  return p;
}

extern "C" void fftw_execute(const fftw_plan p) {
  const int n = p->n;
  std::vector<long double> x(p->in, p->in + n), y(n, 0.0L);
  if (p->kind == FFTW_R2HC) {
    for (int k = 0; k <= n / 2; k++) {
      long double re = 0.0L, im = 0.0L;
      for (int j = 0; j < n; j++) {
        int m = static_cast<int>((static_cast<long long>(j) * k) % n);
        re += x[j] * p->cs[m];
        im -= x[j] * p->sn[m];
      }
      y[k] = re;
      if (k > 0 && k < (n + 1) / 2 && n - k != k) y[n - k] = im;
    }
  } else {
    // x_j = hc_0 + 2 sum_{0<k<(n+1)/2} (hc_k cos - hc_{n-k} sin) + [n even] hc_{n/2} (-1)^j
    for (int j = 0; j < n; j++) {
      long double acc = x[0];
      for (int k = 1; k < (n + 1) / 2; k++) {
        int m = static_cast<int>((static_cast<long long>(j) * k) % n);
        acc += 2.0L * (x[k] * p->cs[m] - x[n - k] * p->sn[m]);
      }
      if (n % 2 == 0) acc += (j % 2 == 0 ? 1.0L : -1.0L) * x[n / 2];
      y[j] = acc;
    }
  }
  for (int j = 0; j < n; j++) p->out[j] = static_cast<double>(y[j]);
}

extern "C" void fftw_destroy_plan(fftw_plan p) { delete p; }

// ------------------------------------------------------------------ LAPACK --

// Right-looking blocked LU with partial pivoting (LAPACK dgetrf's contract:
// A = P L U, column-major, 1-based ipiv, pivot = first entry of largest
// modulus).  The panel is factored column by column; its row exchanges are
// then applied to the other columns, U12 = L11^-1 A12, and A22 -= L21 U12 in
// parallel over column blocks (OpenMP when compiled with it).
extern "C" void dgetrf_(int* m_, int* n_, double* a, int* lda_, int* ipiv, int* info) {
  const int m = *m_, n = *n_, lda = *lda_;
  *info = 0;
  const int kmax = m < n ? m : n;
  const int nb = 64;
  auto col = [&](int j) { return a + static_cast<size_t>(j) * lda; };
  for (int k0 = 0; k0 < kmax; k0 += nb) {
    const int kb = (kmax - k0) < nb ? (kmax - k0) : nb;
    for (int k = k0; k < k0 + kb; k++) {  // panel
      double* colk = col(k);
      int p = k;
      double best = std::fabs(colk[k]);
      for (int i = k + 1; i < m; i++) {
        double v = std::fabs(colk[i]);
        if (v > best) {
          best = v;
          p = i;
        }
      }
      ipiv[k] = p + 1;
      if (p != k)
        for (int j = k0; j < k0 + kb; j++) std::swap(col(j)[k], col(j)[p]);
      if (colk[k] == 0.0) {
        if (*info == 0) *info = k + 1;
        continue;
      }
      const double inv = 1.0 / colk[k];
      for (int i = k + 1; i < m; i++) colk[i] *= inv;
      for (int j = k + 1; j < k0 + kb; j++) {
        double* cj = col(j);
        const double u = cj[k];
        if (u == 0.0) continue;
        for (int i = k + 1; i < m; i++) cj[i] -= colk[i] * u;
      }
    }
    // the panel's exchanges on the columns left and right of it
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; j++) {
      if (j >= k0 && j < k0 + kb) continue;
      double* cj = col(j);
      for (int k = k0; k < k0 + kb; k++)
        if (ipiv[k] - 1 != k) std::swap(cj[k], cj[ipiv[k] - 1]);
    }
    const int j0 = k0 + kb;
    if (j0 >= n) continue;
    const int jblk = 16, iblk = 512;
#pragma omp parallel for schedule(dynamic)
    for (int jb = j0; jb < n; jb += jblk) {
      const int je = (jb + jblk < n) ? jb + jblk : n;
      for (int j = jb; j < je; j++) {  // U12 = L11^-1 A12 (unit lower)
        double* cj = col(j);
        for (int k = k0; k < k0 + kb; k++) {
          const double u = cj[k];
          if (u == 0.0) continue;
          const double* ck = col(k);
          for (int i = k + 1; i < k0 + kb; i++) cj[i] -= ck[i] * u;
        }
      }
      for (int i0 = j0; i0 < m; i0 += iblk) {  // A22 -= L21 U12
        const int ie = (i0 + iblk < m) ? i0 + iblk : m;
        for (int j = jb; j < je; j++) {
          double* cj = col(j);
          for (int k = k0; k < k0 + kb; k++) {
            const double u = cj[k];
            if (u == 0.0) continue;
            const double* ck = col(k);
            for (int i = i0; i < ie; i++) cj[i] -= ck[i] * u;
          }
        }
      }
    }
  }
}

extern "C" void dgetrs_(char* trans, int* n_, int* nrhs_, double* a, int* lda_, int* ipiv, double* b, int* ldb_,
                        int* info) {
  const int n = *n_, nrhs = *nrhs_, lda = *lda_, ldb = *ldb_;
  *info = 0;
  const bool t = (*trans == 'T' || *trans == 't' || *trans == 'C' || *trans == 'c');
  auto A = [&](int i, int j) { return a[i + static_cast<size_t>(j) * lda]; };
  for (int r = 0; r < nrhs; r++) {
    double* x = b + static_cast<size_t>(r) * ldb;
    if (!t) {
      for (int i = 0; i < n; i++)
        if (ipiv[i] - 1 != i) std::swap(x[i], x[ipiv[i] - 1]);
      for (int j = 0; j < n; j++)  // L (unit lower), column oriented
        for (int i = j + 1; i < n; i++) x[i] -= A(i, j) * x[j];
      for (int j = n - 1; j >= 0; j--) {  // U
        x[j] /= A(j, j);
        for (int i = 0; i < j; i++) x[i] -= A(i, j) * x[j];
      }
    } else {
      for (int i = 0; i < n; i++) {  // U^T y = b
        double s = x[i];
        for (int k = 0; k < i; k++) s -= A(k, i) * x[k];
        x[i] = s / A(i, i);
      }
      for (int i = n - 1; i >= 0; i--) {  // L^T z = y
        double s = x[i];
        for (int k = i + 1; k < n; k++) s -= A(k, i) * x[k];
        x[i] = s;
      }
      for (int i = n - 1; i >= 0; i--)
        if (ipiv[i] - 1 != i) std::swap(x[i], x[ipiv[i] - 1]);
    }
  }
}

extern "C" void dgbtrf_(int*, int*, int*, int*, double*, int*, int*, int*) { unsupported("dgbtrf_"); }
extern "C" void dgbtrs_(char*, int*, int*, int*, int*, double*, int*, int*, double*, int*, int*) {
  unsupported("dgbtrs_");
}
extern "C" void dgeev_(char*, char*, int*, double*, int*, double*, double*, double*, int*, double*, int*, double*,
                       int*, int*) {
  unsupported("dgeev_");
}

// ------------------------------------------------- ScaLAPACK / BLACS (unused) --

extern "C" {
void sl_init_(int*, int*, int*) { unsupported("sl_init_"); }
void blacs_gridexit_(int*) { unsupported("blacs_gridexit_"); }
void blacs_gridinfo_(int*, int*, int*, int*, int*) { unsupported("blacs_gridinfo_"); }
void blacs_gridinit_(int*, char*, int*, int*) { unsupported("blacs_gridinit_"); }
int numroc_(int*, int*, int*, int*, int*) { unsupported("numroc_"); }
int indxl2g_(int*, int*, int*, int*, int*) { unsupported("indxl2g_"); }
void descinit_(int*, int*, int*, int*, int*, int*, int*, int*, int*, int*) { unsupported("descinit_"); }
void pdgesv_(int*, int*, double*, int*, int*, int*, int*, double*, int*, int*, int*, int*) { unsupported("pdgesv_"); }
void pdtran_(int*, int*, double*, double*, int*, int*, int*, double*, double*, int*, int*, int*) {
  unsupported("pdtran_");
}
void pdgemv_(char*, int*, int*, double*, double*, int*, int*, int*, double*, int*, int*, int*, int*, double*, double*,
             int*, int*, int*, int*) {
  unsupported("pdgemv_");
}
void pdgemm_(char*, char*, int*, int*, int*, double*, double*, int*, int*, int*, double*, int*, int*, int*, double*,
             double*, int*, int*, int*) {
  unsupported("pdgemm_");
}
int blacs_pnum_(int*, int*, int*) { unsupported("blacs_pnum_"); }
void pdgemr2d_(int*, int*, double*, int*, int*, int*, double*, int*, int*, int*, int*) { unsupported("pdgemr2d_"); }
void Cpdgemr2d(int, int, double*, int, int, int*, double*, int, int, int*, int) { unsupported("Cpdgemr2d"); }
}

// --------------------------------------------------------------------- GSL --

extern "C" gsl_permutation* gsl_permutation_calloc(size_t n) {
  auto* p = static_cast<gsl_permutation*>(std::malloc(sizeof(gsl_permutation)));
  p->size = n;
  p->data = static_cast<size_t*>(std::malloc((n ? n : 1) * sizeof(size_t)));
  for (size_t i = 0; i < n; i++) p->data[i] = i;
  return p;
}

extern "C" void gsl_permutation_free(gsl_permutation* p) {
  if (!p) return;
  std::free(p->data);
  std::free(p);
}

extern "C" size_t gsl_permutation_get(const gsl_permutation* p, size_t i) { return p->data[i]; }
extern "C" size_t gsl_permutation_size(const gsl_permutation* p) { return p->size; }

// Next permutation in lexicographic order; GSL_FAILURE (and no change) after the last.
extern "C" int gsl_permutation_next(gsl_permutation* p) {
  const size_t n = p->size;
  if (n < 2) return GSL_FAILURE;
  size_t i = n - 2;
  while (p->data[i] > p->data[i + 1]) {
    if (i == 0) return GSL_FAILURE;
    i--;
  }
  size_t j = n - 1;
  while (p->data[j] < p->data[i]) j--;
  std::swap(p->data[i], p->data[j]);
  for (size_t lo = i + 1, hi = n - 1; lo < hi; lo++, hi--) std::swap(p->data[lo], p->data[hi]);
  return GSL_SUCCESS;
}

extern "C" double gsl_sf_bessel_jl(int l, double x) {
  if (x == 0.0) return l == 0 ? 1.0 : 0.0;
  double j0 = std::sin(x) / x;
  if (l == 0) return j0;
  double j1 = std::sin(x) / (x * x) - std::cos(x) / x;
  for (int k = 1; k < l; k++) {
    double j2 = (2 * k + 1) / x * j1 - j0;
    j0 = j1;
    j1 = j2;
  }
  return j1;
}

extern "C" double gsl_sf_bessel_yl(int l, double x) {
  double y0 = -std::cos(x) / x;
  if (l == 0) return y0;
  double y1 = -std::cos(x) / (x * x) - std::sin(x) / x;
  for (int k = 1; k < l; k++) {
    double y2 = (2 * k + 1) / x * y1 - y0;
    y0 = y1;
    y1 = y2;
  }
  return y1;
}

// --------------------------------------------------------------- MPI (1 rank) --

namespace {
size_t type_size(MPI_Datatype t) { return t == MPI_INT ? sizeof(int) : sizeof(double); }
}  // namespace

extern "C" {
int MPI_Init(int*, char***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int* rank) {
  *rank = 0;
  return MPI_SUCCESS;
}
int MPI_Comm_size(MPI_Comm, int* size) {
  *size = 1;
  return MPI_SUCCESS;
}
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
int MPI_Allreduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (in != out) std::memmove(out, in, n * type_size(t));
  return MPI_SUCCESS;
}
int MPI_Reduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  if (in != out) std::memmove(out, in, n * type_size(t));
  return MPI_SUCCESS;
}
int MPI_Allgatherv(const void* in, int n, MPI_Datatype t, void* out, const int*, const int* displs, MPI_Datatype,
                   MPI_Comm) {
  std::memmove(static_cast<char*>(out) + displs[0] * type_size(t), in, n * type_size(t));
  return MPI_SUCCESS;
}
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
}
