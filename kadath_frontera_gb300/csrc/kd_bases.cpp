// 1-D spectral operators of Kadath, restated so that they can be turned into
// matrices.  Each function below names the reference routine it follows; the
// steps (symmetric fold, real DFT in FFTW's halfcomplex order, recurrence for
// the odd Chebyshev coefficients, ...) are kept in the same order so that the
// matrices reproduce the reference's results for every input line, including
// lines that do not have the symmetry the basis assumes.
#include "kd_bases.hpp"

#include <cmath>
#include <stdexcept>

namespace kd {

namespace {

const double PI = 3.14159265358979323846;

// Real DFT of length n in FFTW's R2HC layout: h[k] = Re Y_k (0<=k<=n/2),
// h[n-k] = Im Y_k (0<k<(n+1)/2), Y_k = sum_j x_j exp(-2 pi i j k / n).
// This is the transform FFTW_R2HC documents; the reference calls it through
// fftw_plan_r2r_1d (include/base_fftw.hpp:33).
void r2hc(const double* x, double* h, int n) {
  std::vector<double> re(n / 2 + 1, 0.0), im(n / 2 + 1, 0.0);
  for (int k = 0; k <= n / 2; k++) {
    double sr = 0, si = 0;
    for (int j = 0; j < n; j++) {
      long long p = (static_cast<long long>(j) * k) % n;
      double ang = 2.0 * PI * static_cast<double>(p) / n;
      sr += x[j] * std::cos(ang);
      si -= x[j] * std::sin(ang);
    }
    re[k] = sr;
    im[k] = si;
  }
  for (int k = 0; k <= n / 2; k++) h[k] = re[k];
  for (int k = 1; k < (n + 1) / 2; k++) h[n - k] = im[k];
}

// Inverse of r2hc without normalisation (FFTW_HC2R): x_j = sum_k Y_k e^{+...}.
void hc2r(const double* h, double* x, int n) {
  for (int j = 0; j < n; j++) {
    double s = h[0];
    for (int k = 1; k < (n + 1) / 2; k++) {
      long long p = (static_cast<long long>(j) * k) % n;
      double ang = 2.0 * PI * static_cast<double>(p) / n;
      s += 2.0 * (h[k] * std::cos(ang) - h[n - k] * std::sin(ang));
    }
    if (n % 2 == 0) s += h[n / 2] * ((j % 2 == 0) ? 1.0 : -1.0);
    x[j] = s;
  }
}

using Vec = std::vector<double>;

// ---------------------------------------------------------------- forward --
// Shared fold of a Gauss-Lobatto line before the R2HC of length n-1, used by
// coef_1d_cheb/cheb_even/cos/cos_even/... (src/Coef/coef_1d.cpp:57-100 and
// siblings).  `odd_sign` is +1 when the antisymmetric part enters as
// (t_i - t_{n-1-i}) and -1 when it enters as (t_{n-1-i} - t_i).
void fold_even(const double* t, int n, double odd_sign, Vec& a) {
  a.assign(n - 1, 0.0);
  for (int i = 1; i < (n - 1) / 2; i++) {
    double fp = 0.5 * (t[i] + t[n - 1 - i]);
    double fms = odd_sign * 0.5 * (t[i] - t[n - 1 - i]) * std::sin(PI * i / (n - 1));
    a[i] = fp + fms;
    a[n - 1 - i] = fp - fms;
  }
  a[0] = 0.5 * (t[0] + t[n - 1]);
  a[(n - 1) / 2] = t[(n - 1) / 2];
}

// Unscramble of the Chebyshev-type transforms: even coefficients straight from
// the cosine part, odd ones by the running recurrence and the c_1 closure.
// `rec_sign` is the sign in front of 4*A[...]; c1 = (fm - som)/((n-1)/2) with
// fm_sign applied as in the reference (cheb: c1 = -(f0 + som)/h).
void unscramble_cheb(const Vec& A, int n, double rec_sign, double fmoins0, bool cheb_style,
                     double* out) {
  out[0] = A[0] / (n - 1);
  for (int i = 2; i < n - 1; i += 2) out[i] = 2 * A[i / 2] / (n - 1);
  out[n - 1] = A[(n - 1) / 2] / (n - 1);
  out[1] = 0;
  double som = 0;
  for (int i = 3; i < n; i += 2) {
    out[i] = out[i - 2] + rec_sign * 4 * A[n - 1 - i / 2] / (n - 1);
    som += out[i];
  }
  int half = (n - 1) / 2;
  double c1 = cheb_style ? -(fmoins0 + som) / half : (fmoins0 - som) / half;
  out[1] = c1;
  for (int i = 3; i < n; i += 2) out[i] += c1;
}

// coef_1d_cheb, src/Coef/coef_1d.cpp:57
int coef_cheb(Vec& t, int n) {
  double f0 = 0.5 * (t[0] - t[n - 1]);
  Vec a, A(n - 1);
  fold_even(t.data(), n, +1.0, a);
  r2hc(a.data(), A.data(), n - 1);
  unscramble_cheb(A, n, -1.0, f0, true, t.data());
  return CHEB;
}

// coef_1d_cheb_even, src/Coef/coef_1d.cpp:102
int coef_cheb_even(Vec& t, int n) {
  double f0 = -0.5 * (t[0] - t[n - 1]);
  Vec a, A(n - 1);
  fold_even(t.data(), n, -1.0, a);
  r2hc(a.data(), A.data(), n - 1);
  unscramble_cheb(A, n, +1.0, f0, false, t.data());
  return CHEB_EVEN;
}

// Final step of the odd-parity transforms: coefficients of x*f (or cos(t)*f)
// turned into those of f by the two-term recurrence (coef_1d.cpp:190-196).
void divide_back(Vec& cf, int n, double sign) {
  cf[0] = 2 * cf[0];
  for (int i = 1; i < n - 1; i++) cf[i] = 2 * cf[i] + sign * cf[i - 1];
  cf[n - 1] = 0;
}

// coef_1d_cheb_odd, src/Coef/coef_1d.cpp:146
int coef_cheb_odd(Vec& t, int n) {
  Vec cf(n);
  for (int i = 0; i < n; i++) cf[i] = t[i] * std::sin(PI / 2. * i / (n - 1));
  double f0 = -0.5 * (cf[0] - cf[n - 1]);
  Vec a, A(n - 1);
  fold_even(cf.data(), n, -1.0, a);
  r2hc(a.data(), A.data(), n - 1);
  unscramble_cheb(A, n, +1.0, f0, false, cf.data());
  divide_back(cf, n, -1.0);
  for (int i = 0; i < n; i++) t[i] = cf[i];
  return CHEB_ODD;
}

// coef_1d_cossin, src/Coef/coef_1d.cpp:254.  t has nbr = n_phi + 2 entries.
int coef_cossin(Vec& t, int nbr) {
  if (nbr > 3) {
    int np = nbr - 2;
    Vec cf(np);
    for (int i = 0; i < np; i++) cf[i] = t[i];
    Vec h(np);
    r2hc(cf.data(), h.data(), np);
    int index = 0;
    int pc = 0;         // cosine cursor
    int ps = nbr - 3;   // sine cursor (walks down)
    t[index++] = h[pc++] / double(np);
    t[index++] = 0;
    for (int i = 1; i < nbr / 2 - 1; i++) {
      t[index++] = 2. * h[pc++] / double(np);
      t[index++] = -2. * h[ps--] / double(np);
    }
    t[index++] = h[pc] / double(np);
    t[index] = 0;
  } else {
    t[1] = 0;
    t[2] = 0;
  }
  return COSSIN;
}

// coef_1d_cos, src/Coef/coef_1d.cpp:294 (same algebra as cheb_even with the
// symmetric-part sign of cheb).
int coef_cos(Vec& t, int n) {
  double f0 = 0.5 * (t[0] - t[n - 1]);
  Vec a, A(n - 1);
  fold_even(t.data(), n, +1.0, a);
  r2hc(a.data(), A.data(), n - 1);
  unscramble_cheb(A, n, +1.0, f0, false, t.data());
  return COS;
}

// Fold used by the sine transforms: the symmetric part carries the sine
// weight (coef_1d.cpp:345-350, 479-484).  `a0_minus` selects t0 - t_{n-1}.
void fold_sin(const double* t, int n, bool a0_minus, Vec& a) {
  a.assign(n - 1, 0.0);
  for (int i = 1; i < (n - 1) / 2; i++) {
    double fp = 0.5 * (t[i] + t[n - 1 - i]) * std::sin(PI * i / (n - 1));
    double fms = 0.5 * (t[i] - t[n - 1 - i]);
    a[i] = fp + fms;
    a[n - 1 - i] = fp - fms;
  }
  a[0] = a0_minus ? 0.5 * (t[0] - t[n - 1]) : 0.5 * (t[0] + t[n - 1]);
  a[(n - 1) / 2] = t[(n - 1) / 2];
}

void unscramble_sin(const Vec& A, int n, double* out) {
  out[0] = 0;
  for (int i = 2; i < n - 1; i += 2) out[i] = -2 * A[n - 1 - i / 2] / (n - 1);
  out[n - 1] = 0;
  out[1] = 2 * A[0] / (n - 1);
  for (int i = 3; i < n; i += 2) out[i] = out[i - 2] + 4 * A[i / 2] / (n - 1);
}

// coef_1d_sin, src/Coef/coef_1d.cpp:338
int coef_sin(Vec& t, int n) {
  Vec a, A(n - 1);
  fold_sin(t.data(), n, false, a);
  r2hc(a.data(), A.data(), n - 1);
  unscramble_sin(A, n, t.data());
  return SIN;
}

// coef_1d_cos_even, src/Coef/coef_1d.cpp:369
int coef_cos_even(Vec& t, int n) {
  if (n > 3) coef_cos(t, n);
  return COS_EVEN;
}

// coef_1d_cos_odd, src/Coef/coef_1d.cpp:414
int coef_cos_odd(Vec& t, int n) {
  if (n > 3) {
    Vec cf(n);
    for (int i = 0; i < n - 1; i++) cf[i] = t[i] * std::sin(PI * (n - 1 - i) / 2. / (n - 1));
    cf[n - 1] = 0;
    double f0 = 0.5 * (cf[0] - cf[n - 1]);
    Vec a, A(n - 1);
    fold_even(cf.data(), n, +1.0, a);
    r2hc(a.data(), A.data(), n - 1);
    // The reference stores A[(n-1)/2] undivided in the last slot; that slot
    // is overwritten with 0 by the recurrence below, so the scaling is moot.
    unscramble_cheb(A, n, +1.0, f0, false, cf.data());
    divide_back(cf, n, -1.0);
    for (int i = 0; i < n; i++) t[i] = cf[i];
  }
  return COS_ODD;
}

// coef_1d_sin_even, src/Coef/coef_1d.cpp:473
int coef_sin_even(Vec& t, int n) {
  if (n > 3) {
    Vec a, A(n - 1);
    fold_sin(t.data(), n, true, a);
    r2hc(a.data(), A.data(), n - 1);
    unscramble_sin(A, n, t.data());
  }
  return SIN_EVEN;
}

// coef_1d_sin_odd, src/Coef/coef_1d.cpp:505
int coef_sin_odd(Vec& t, int n) {
  if (n > 3) {
    Vec cf(n);
    cf[0] = 0;
    for (int i = 1; i < n; i++) cf[i] = t[i] * std::sin(PI * i / 2. / (n - 1));
    double f0 = 0.5 * (cf[0] - cf[n - 1]);
    Vec a, A(n - 1);
    fold_even(cf.data(), n, +1.0, a);
    r2hc(a.data(), A.data(), n - 1);
    unscramble_cheb(A, n, +1.0, f0, false, cf.data());
    divide_back(cf, n, +1.0);
    for (int i = 0; i < n; i++) t[i] = cf[i];
  }
  return SIN_ODD;
}

// coef_1d_cossin_even / _odd, src/Coef/coef_1d.cpp:563-605: the line is
// extended to a double period and sent through the COSSIN transform.
int coef_cossin_parity(Vec& t, int nbr, bool odd) {
  Vec t2(2 * nbr - 2, 0.0);
  for (int i = 0; i < nbr - 2; i++) {
    t2[i] = t[i];
    t2[i + nbr - 2] = odd ? -t[i] : t[i];
  }
  coef_cossin(t2, 2 * nbr - 2);
  if (!odd) {
    int c = 0;
    for (int k = 0; k < nbr - 1; k += 2) {
      t[k] = t2[c];
      t[k + 1] = t2[c + 1];
      c += 4;
    }
    return COSSIN_EVEN;
  }
  int c = 2;
  for (int k = 0; k < nbr - 3; k += 2) {
    t[k] = t2[c];
    t[k + 1] = t2[c + 1];
    c += 4;
  }
  t[nbr - 2] = 0.;
  t[nbr - 1] = 0.;
  return COSSIN_ODD;
}

// ---------------------------------------------------------------- inverse --
// Shared core of coef_i_1d_cheb/cos/... (src/Coef/coef_i_1d.cpp:49-92): build
// the halfcomplex input from the coefficients, run HC2R of length n-1, then
// unfold into the Gauss-Lobatto values.  Variants differ in the sign of the
// odd part (`sgn`) and in which end receives +fmoins0.
void build_hc_cheb(const double* c, int n, double sgn, Vec& h, double& fmoins0) {
  h.assign(n - 1, 0.0);
  Vec cf(n, 0.0);
  double c1 = c[1];
  double somme = 0;
  cf[1] = 0;
  for (int i = 3; i < n; i += 2) {
    cf[i] = c[i] - c1;
    somme += cf[i];
  }
  // The reference evaluates (nbr-1)/2 in integer arithmetic.
  int half = (n - 1) / 2;
  fmoins0 = sgn * (half * c1 + somme);
  for (int i = 3; i < n; i += 2) h[n - 1 - i / 2] = sgn * 0.25 * (cf[i] - cf[i - 2]);
  h[0] = c[0];
  for (int i = 1; i < (n - 1) / 2; i++) h[i] = 0.5 * c[2 * i];
  h[(n - 1) / 2] = c[n - 1];
}

void unfold_cheb(const Vec& x, int n, double fmoins0, bool reversed, double* out) {
  for (int i = 1; i < (n - 1) / 2; i++) {
    double fp = 0.5 * (x[i] + x[n - 1 - i]);
    double fm = 0.5 * (x[i] - x[n - 1 - i]) / std::sin(PI * i / (n - 1));
    if (!reversed) {
      out[i] = fp + fm;
      out[n - i - 1] = fp - fm;
    } else {
      out[n - 1 - i] = fp + fm;
      out[i] = fp - fm;
    }
  }
  if (!reversed) {
    out[0] = x[0] + fmoins0;
    out[n - 1] = x[0] - fmoins0;
  } else {
    out[0] = x[0] - fmoins0;
    out[n - 1] = x[0] + fmoins0;
  }
  out[(n - 1) / 2] = x[(n - 1) / 2];
}

// coef_i_1d_cheb, src/Coef/coef_i_1d.cpp:49
int coefi_cheb(Vec& t, int n) {
  if (n > 3) {
    Vec h, x(n - 1);
    double f0;
    build_hc_cheb(t.data(), n, -1.0, h, f0);
    hc2r(h.data(), x.data(), n - 1);
    unfold_cheb(x, n, f0, false, t.data());
  }
  return CHEB;
}

// coef_i_1d_cheb_even, src/Coef/coef_i_1d.cpp:94
int coefi_cheb_even(Vec& t, int n) {
  Vec h, x(n - 1);
  double f0;
  build_hc_cheb(t.data(), n, +1.0, h, f0);
  hc2r(h.data(), x.data(), n - 1);
  unfold_cheb(x, n, f0, true, t.data());
  return CHEB_EVEN;
}

// Pre-step of the odd-parity inverses: coefficients of f turned into those of
// x*f (cheb_odd, cos_odd: ti_i = (c_i + c_{i-1})/2) or sin*f (sin_odd: minus).
Vec times_x_coefs(const double* c, int n, double sign) {
  Vec ti(n);
  ti[0] = 0.5 * c[0];
  for (int i = 1; i < n - 1; i++) ti[i] = 0.5 * (c[i] + sign * c[i - 1]);
  ti[n - 1] = sign * 0.5 * c[n - 2];
  return ti;
}

// coef_i_1d_cheb_odd, src/Coef/coef_i_1d.cpp:139
int coefi_cheb_odd(Vec& t, int n) {
  Vec ti = times_x_coefs(t.data(), n, +1.0);
  Vec h, x(n - 1);
  double f0;
  build_hc_cheb(ti.data(), n, +1.0, h, f0);
  hc2r(h.data(), x.data(), n - 1);
  for (int i = 1; i < (n - 1) / 2; i++) {
    double fp = 0.5 * (x[i] + x[n - 1 - i]);
    double fm = 0.5 * (x[i] - x[n - 1 - i]) / std::sin(PI * i / (n - 1));
    t[n - 1 - i] = (fp + fm) / std::sin(PI * (n - 1 - i) / 2 / (n - 1));
    t[i] = (fp - fm) / std::sin(PI * i / 2 / (n - 1));
  }
  t[0] = 0;
  t[n - 1] = x[0] + f0;
  t[(n - 1) / 2] = x[(n - 1) / 2] / std::sin(PI * (n - 1) / 4 / (n - 1));
  return CHEB_ODD;
}

// coef_i_1d_cossin, src/Coef/coef_i_1d.cpp:226
int coefi_cossin(Vec& t, int nbr) {
  int np = nbr - 2;
  if (np > 1) {
    Vec cf(np, 0.0), x(np);
    cf[0] = t[0];
    for (int i = 1; i < np / 2; i++) {
      cf[i] = 0.5 * t[2 * i];
      cf[np - i] = -0.5 * t[2 * i + 1];
    }
    cf[np / 2] = t[np];
    hc2r(cf.data(), x.data(), np);
    for (int i = 0; i < np; i++) t[i] = x[i];
  }
  return COSSIN;
}

// coef_i_1d_cos, src/Coef/coef_i_1d.cpp:248
int coefi_cos(Vec& t, int n) {
  Vec h, x(n - 1);
  double f0;
  build_hc_cheb(t.data(), n, +1.0, h, f0);
  hc2r(h.data(), x.data(), n - 1);
  unfold_cheb(x, n, f0, false, t.data());
  return COS;
}

// coef_i_1d_sin, src/Coef/coef_i_1d.cpp:286
int coefi_sin(Vec& t, int n) {
  Vec h(n - 1, 0.0), x(n - 1);
  for (int i = 2; i < n - 1; i += 2) h[n - 1 - i / 2] = -0.5 * t[i];
  h[0] = 0.5 * t[1];
  for (int i = 3; i < n; i += 2) h[i / 2] = 0.25 * (t[i] - t[i - 2]);
  h[(n - 1) / 2] = -0.5 * t[n - 2];
  hc2r(h.data(), x.data(), n - 1);
  for (int i = 1; i < (n - 1) / 2; i++) {
    double fp = 0.5 * (x[i] + x[n - 1 - i]) / std::sin(PI * i / (n - 1));
    double fm = 0.5 * (x[i] - x[n - 1 - i]);
    t[i] = fp + fm;
    t[n - i - 1] = fp - fm;
  }
  t[0] = 0;
  t[n - 1] = -2 * x[0];
  t[(n - 1) / 2] = x[(n - 1) / 2];
  return SIN;
}

// coef_i_1d_cos_even, src/Coef/coef_i_1d.cpp:318
int coefi_cos_even(Vec& t, int n) {
  if (n > 3) coefi_cos(t, n);
  return COS_EVEN;
}

// coef_i_1d_cos_odd, src/Coef/coef_i_1d.cpp:360
int coefi_cos_odd(Vec& t, int n) {
  if (n > 3) {
    Vec ti = times_x_coefs(t.data(), n, +1.0);
    Vec h, x(n - 1);
    double f0;
    build_hc_cheb(ti.data(), n, +1.0, h, f0);
    hc2r(h.data(), x.data(), n - 1);
    for (int i = 1; i < (n - 1) / 2; i++) {
      double fp = 0.5 * (x[i] + x[n - 1 - i]);
      double fm = 0.5 * (x[i] - x[n - 1 - i]) / std::sin(PI * i / (n - 1));
      t[i] = (fp + fm) / std::sin(PI * (n - 1 - i) / 2 / (n - 1));
      t[n - i - 1] = (fp - fm) / std::sin(PI * i / 2 / (n - 1));
    }
    t[0] = x[0] + f0;
    t[n - 1] = 0;
    t[(n - 1) / 2] = x[(n - 1) / 2] / std::sin(PI * (n - 1) / 4 / (n - 1));
  }
  return COS_ODD;
}

// coef_i_1d_sin_even, src/Coef/coef_i_1d.cpp:408
int coefi_sin_even(Vec& t, int n) {
  if (n > 3) {
    Vec h(n - 1, 0.0), x(n - 1);
    for (int i = 2; i < n - 1; i += 2) h[n - 1 - i / 2] = -0.5 * t[i];
    h[0] = 0.5 * t[1];
    for (int i = 1; i < (n - 1) / 2; i++) h[i] = 0.25 * (t[2 * i + 1] - t[2 * i - 1]);
    h[(n - 1) / 2] = -0.5 * t[n - 2];
    hc2r(h.data(), x.data(), n - 1);
    for (int i = 1; i < (n - 1) / 2; i++) {
      double fp = 0.5 * (x[i] + x[n - 1 - i]) / std::sin(PI * i / (n - 1));
      double fm = 0.5 * (x[i] - x[n - 1 - i]);
      t[i] = fp + fm;
      t[n - i - 1] = fp - fm;
    }
    t[0] = 0;
    t[n - 1] = -2 * x[0];
    t[(n - 1) / 2] = x[(n - 1) / 2];
  }
  return SIN_EVEN;
}

// coef_i_1d_sin_odd, src/Coef/coef_i_1d.cpp:440
int coefi_sin_odd(Vec& t, int n) {
  if (n > 3) {
    Vec ti = times_x_coefs(t.data(), n, -1.0);
    Vec h, x(n - 1);
    double f0;
    build_hc_cheb(ti.data(), n, +1.0, h, f0);
    hc2r(h.data(), x.data(), n - 1);
    for (int i = 1; i < (n - 1) / 2; i++) {
      double fp = 0.5 * (x[i] + x[n - 1 - i]);
      double fm = 0.5 * (x[i] - x[n - 1 - i]) / std::sin(PI * i / (n - 1));
      t[i] = (fp + fm) / std::sin(PI * i / 2 / (n - 1));
      t[n - i - 1] = (fp - fm) / std::sin(PI * (n - 1 - i) / 2 / (n - 1));
    }
    t[0] = 0;
    t[n - 1] = x[0] - f0;
    t[(n - 1) / 2] = x[(n - 1) / 2] / std::sin(PI * (n - 1) / 4 / (n - 1));
  }
  return SIN_ODD;
}

// coef_i_1d_cossin_even / _odd, src/Coef/coef_i_1d.cpp:481-525
int coefi_cossin_parity(Vec& t, int nbr, bool odd) {
  Vec t2(2 * nbr - 2, 0.0);
  int c = 0;
  for (int i = 0; i < nbr - 2; i += 2) {
    if (!odd) {
      t2[c] = t[i];
      t2[c + 1] = t[i + 1];
      t2[c + 2] = 0.;
      t2[c + 3] = 0.;
    } else {
      t2[c] = 0.;
      t2[c + 1] = 0.;
      t2[c + 2] = t[i];
      t2[c + 3] = t[i + 1];
    }
    c += 4;
  }
  t2[c] = t[nbr - 2];
  t2[c + 1] = t[nbr - 1];
  coefi_cossin(t2, 2 * nbr - 2);
  for (int i = 0; i < nbr - 2; i++) t[i] = t2[i];
  t[nbr - 2] = 0;
  t[nbr - 1] = 0;
  return odd ? COSSIN_ODD : COSSIN_EVEN;
}

// ------------------------------------------------------------- derivative --
// der_1d_*, src/Ope_1d/der_1d.cpp:31-289
int der_line(int basis, Vec& t, int n) {
  Vec r(n, 0.0);
  switch (basis) {
    case CHEB:
      for (int i = 0; i < n; i++)
        for (int p = i + 1; p < n; p += 2) r[i] += p * t[p];
      for (auto& v : r) v *= 2;
      r[0] /= 2;
      t = r;
      return CHEB;
    case CHEB_EVEN:
      for (int i = 0; i < n; i++)
        for (int p = i + 1; p < n; p++) r[i] += 2 * p * t[p];
      r[n - 1] = 0;
      for (auto& v : r) v *= 2;
      t = r;
      return CHEB_ODD;
    case CHEB_ODD:
      for (int i = 0; i < n; i++)
        for (int p = i; p < n; p++) r[i] += (2 * p + 1) * t[p];
      for (auto& v : r) v *= 2;
      r[0] /= 2;
      t = r;
      return CHEB_EVEN;
    case COSSIN:
      for (int i = 0; i < n - 1; i += 2) r[i + 1] = -(i / 2) * t[i];
      for (int i = 1; i < n; i += 2) r[i - 1] = ((i - 1) / 2) * t[i];
      r[n - 1] = 0;
      t = r;
      return COSSIN;
    case COSSIN_EVEN:
      for (int i = 0; i < n - 1; i += 2) r[i + 1] = -i * t[i];
      for (int i = 1; i < n; i += 2) r[i - 1] = (i - 1) * t[i];
      t = r;
      return COSSIN_EVEN;
    case COSSIN_ODD:
      for (int i = 0; i < n - 1; i += 2) r[i + 1] = -(i + 1) * t[i];
      for (int i = 1; i < n; i += 2) r[i - 1] = i * t[i];
      t = r;
      return COSSIN_ODD;
    case COS:
      for (int i = 0; i < n; i++) r[i] = -i * t[i];
      t = r;
      return SIN;
    case SIN:
      for (int i = 0; i < n; i++) r[i] = i * t[i];
      t = r;
      return COS;
    case COS_EVEN:
      for (int i = 0; i < n; i++) r[i] = -2 * i * t[i];
      r[n - 1] = 0;
      t = r;
      return SIN_EVEN;
    case COS_ODD:
      for (int i = 0; i < n; i++) r[i] = -(2 * i + 1) * t[i];
      t = r;
      return SIN_ODD;
    case SIN_EVEN:
      for (int i = 0; i < n; i++) r[i] = 2 * i * t[i];
      t = r;
      return COS_EVEN;
    case SIN_ODD:
      for (int i = 0; i < n; i++) r[i] = (2 * i + 1) * t[i];
      r[n - 1] = 0;
      t = r;
      return COS_ODD;
    default:
      return -1;
  }
}

// ------------------------------------------------- multiplication by sin --
// mult_sin_1d_*, src/Ope_1d/mult_sin_1d.cpp
int mult_sin_line(int basis, Vec& t, int n) {
  Vec r(n, 0.0);
  switch (basis) {
    case COSSIN:
      r[0] = 0.5 * t[3];
      r[1] = 0;
      r[2] = 0.5 * t[5];
      r[3] = t[0] - 0.5 * t[4];
      for (int k = 4; k < n - 2; k += 2) {
        r[k] = 0.5 * (t[3 + k] - t[k - 1]);
        r[k + 1] = 0.5 * (t[k - 2] - t[k + 2]);
      }
      r[n - 2] = -0.5 * t[n - 3];
      r[n - 1] = 0.;
      t = r;
      return COSSIN;
    case COS:
      r[0] = 0.;
      r[1] = t[0] - 0.5 * t[2];
      for (int k = 2; k < n - 1; k++) r[k] = 0.5 * (t[k - 1] - t[k + 1]);
      r[n - 1] = 0;
      t = r;
      return SIN;
    case SIN:
      r[0] = 0.5 * t[1];
      r[1] = 0.5 * t[2];
      for (int k = 2; k < n - 1; k++) r[k] = 0.5 * (-t[k - 1] + t[k + 1]);
      r[n - 1] = 0;
      t = r;
      return COS;
    case COS_EVEN:
      r[0] = t[0] - 0.5 * t[1];
      for (int k = 1; k < n - 1; k++) r[k] = 0.5 * (t[k] - t[k + 1]);
      r[n - 1] = 0;
      t = r;
      return SIN_ODD;
    case COS_ODD:
      r[0] = 0.;
      for (int k = 1; k < n; k++) r[k] = 0.5 * (t[k - 1] - t[k]);
      t = r;
      return SIN_EVEN;
    case SIN_EVEN:
      r[0] = 0.5 * t[1];
      for (int k = 1; k < n - 1; k++) r[k] = 0.5 * (-t[k] + t[k + 1]);
      r[n - 1] = 0;
      t = r;
      return COS_ODD;
    case SIN_ODD:
      r[0] = 0.5 * t[0];
      for (int k = 1; k < n; k++) r[k] = 0.5 * (-t[k - 1] + t[k]);
      t = r;
      return COS_EVEN;
    default:
      return -1;
  }
}

// div_sin_1d_*, src/Ope_1d/div_sin_1d.cpp
int div_sin_line(int basis, Vec& t, int n) {
  Vec r(n, 0.0);
  double s = 0;
  switch (basis) {
    case COS:
      r[n - 1] = 0.;
      for (int k = n - 2; k >= 0; k -= 2) {
        s -= 2 * t[k];
        if (k - 1 >= 0) r[k - 1] = s;
      }
      s = 0;
      for (int k = n - 3; k >= 0; k -= 2) {
        s -= 2 * t[k + 2];
        r[k + 1] = s;
      }
      r[0] = 0;
      t = r;
      return SIN;
    case SIN:
      r[n - 1] = 0.;
      for (int k = n - 2; k >= 0; k -= 2) {
        s += 2 * t[k];
        if (k - 1 >= 0) r[k - 1] = s;
      }
      s = 0;
      for (int k = n - 3; k >= 0; k -= 2) {
        s += 2 * t[k + 2];
        r[k + 1] = s;
      }
      r[0] *= 0.5;
      t = r;
      return COS;
    case COS_EVEN:
      r[n - 1] = 0.;
      for (int k = n - 2; k >= 0; k--) {
        s -= 2 * t[k + 1];
        r[k] = s;
      }
      t = r;
      return SIN_ODD;
    case COS_ODD:
      r[n - 1] = 0.;
      for (int k = n - 2; k >= 0; k--) {
        s -= 2 * t[k];
        r[k] = s;
      }
      t = r;
      return SIN_EVEN;
    case SIN_EVEN:
      r[n - 1] = 0.;
      for (int k = n - 2; k >= 0; k--) {
        s += 2 * t[k + 1];
        r[k] = s;
      }
      t = r;
      return COS_ODD;
    case SIN_ODD:
      r[n - 1] = 0.;
      for (int k = n - 2; k >= 0; k--) {
        s += 2 * t[k];
        r[k] = s;
      }
      r[0] *= 0.5;
      t = r;
      return COS_EVEN;
    default:
      return -1;
  }
}

// mult_cos_1d_*, src/Ope_1d/mult_cos_1d.cpp
int mult_cos_line(int basis, Vec& t, int n) {
  Vec r(n, 0.0);
  switch (basis) {
    case COSSIN:
      r[0] = 0.5 * t[2];
      r[1] = 0;
      r[2] = t[0] + 0.5 * t[4];
      r[3] = 0.5 * t[5];
      for (int k = 4; k < n - 2; k++) r[k] = 0.5 * (t[2 + k] + t[k - 2]);
      r[n - 2] = 0.5 * t[n - 4];
      r[n - 1] = 0.;
      t = r;
      return COSSIN;
    case COS:
      r[0] = 0.5 * t[1];
      r[1] = t[0] + 0.5 * t[2];
      for (int k = 2; k < n - 1; k++) r[k] = 0.5 * (t[k - 1] + t[k + 1]);
      r[n - 1] = 0;
      t = r;
      return COS;
    case SIN:
      r[0] = 0.;
      r[1] = 0.5 * t[2];
      for (int k = 2; k < n - 1; k++) r[k] = 0.5 * (t[k - 1] + t[k + 1]);
      r[n - 1] = 0;
      t = r;
      return SIN;
    case COS_EVEN:
      r[0] = t[0] + 0.5 * t[1];
      for (int k = 1; k < n - 1; k++) r[k] = 0.5 * (t[k] + t[k + 1]);
      r[n - 1] = 0.;
      t = r;
      return COS_ODD;
    case COS_ODD:
      r[0] = 0.5 * t[0];
      for (int k = 1; k < n; k++) r[k] = 0.5 * (t[k - 1] + t[k]);
      t = r;
      return COS_EVEN;
    case SIN_EVEN:
      r[0] = 0.5 * t[1];
      for (int k = 1; k < n - 1; k++) r[k] = 0.5 * (t[k] + t[k + 1]);
      r[n - 1] = 0.;
      t = r;
      return SIN_ODD;
    case SIN_ODD:
      r[0] = 0.;
      for (int k = 1; k < n; k++) r[k] = 0.5 * (t[k - 1] + t[k]);
      t = r;
      return SIN_EVEN;
    default:
      return -1;
  }
}

// div_cos_1d_*, src/Ope_1d/div_cos_1d.cpp
int div_cos_line(int basis, Vec& t, int n) {
  Vec r(n, 0.0);
  double s = 0;
  int sg;
  switch (basis) {
    case COS_EVEN:
      r[n - 1] = 0.;
      sg = 1;
      for (int k = n - 2; k >= 0; k--) {
        s -= 2 * sg * t[k + 1];
        sg *= -1;
        r[k] = (k % 2 == 0) ? s : -s;
      }
      t = r;
      return COS_ODD;
    case SIN_ODD:
      r[n - 1] = 0.;
      sg = -1;
      for (int k = n - 2; k > 0; k--) {
        s -= 2 * sg * t[k];
        sg *= -1;
        r[k] = (k % 2 == 0) ? -s : +s;
      }
      t = r;
      return SIN_EVEN;
    case COS_ODD:
      r[n - 1] = 0.;
      sg = -1;
      for (int k = n - 2; k >= 0; k--) {
        s += 2 * t[k] * sg;
        r[k] = (k % 2 == 0) ? s : -s;
        sg *= -1;
      }
      r[0] *= 0.5;
      t = r;
      return COS_EVEN;
    case SIN_EVEN:
      sg = -1;
      r[n - 1] = 0.;
      for (int k = n - 2; k >= 0; k--) {
        s -= 2 * t[k + 1] * sg;
        sg *= -1;
        r[k] = (k % 2 == 0) ? -s : s;
      }
      t = r;
      return SIN_ODD;
    default:
      return -1;
  }
}

// mult_x_1d_*, src/Ope_1d/mult_x_1d.cpp
int mult_x_line(int basis, Vec& t, int n) {
  Vec r(n, 0.0);
  switch (basis) {
    case CHEB:
      r[0] = 0.5 * t[1];
      r[1] = t[0] + 0.5 * t[2];
      for (int i = 2; i < n - 1; i++) r[i] = 0.5 * (t[i + 1] + t[i - 1]);
      r[n - 1] = 0.5 * t[n - 2];
      t = r;
      return CHEB;
    case CHEB_EVEN:
      r[0] = t[0] + 0.5 * t[1];
      for (int i = 1; i < n - 1; i++) r[i] = 0.5 * (t[i] + t[i + 1]);
      r[n - 1] = 0.;
      t = r;
      return CHEB_ODD;
    case CHEB_ODD:
      r[0] = 0.5 * t[0];
      for (int i = 1; i < n - 1; i++) r[i] = 0.5 * (t[i] + t[i - 1]);
      r[n - 1] = 0.5 * t[n - 2];
      t = r;
      return CHEB_EVEN;
    default:
      return -1;
  }
}

// div_x_1d_*, src/Ope_1d/div_x_1d.cpp
int div_x_line(int basis, Vec& t, int n) {
  Vec r(n, 0.0);
  int sgn = 1;
  double s;
  switch (basis) {
    case CHEB_EVEN:
      r[n - 1] = 0;
      s = 2 * sgn * t[n - 1];
      r[n - 2] = s;
      for (int i = n - 3; i >= 0; i--) {
        sgn *= -1;
        s += 2 * sgn * t[i + 1];
        r[i] = s;
      }
      for (int i = 0; i < n; i += 2) r[i] *= -1;
      t = r;
      return CHEB_ODD;
    case CHEB_ODD:
      r[n - 1] = 0;
      s = 2 * sgn * t[n - 2];
      r[n - 2] = s;
      for (int i = n - 3; i >= 0; i--) {
        sgn *= -1;
        s += 2 * sgn * t[i];
        r[i] = s;
      }
      for (int i = 0; i < n; i += 2) r[i] *= -1;
      r[0] *= 0.5;
      t = r;
      return CHEB_EVEN;
    default:
      return -1;
  }
}

// mult_xm1_1d_cheb, src/Ope_1d/mult_xm1_1d.cpp:26
int mult_xm1_line(int basis, Vec& t, int n) {
  if (basis != CHEB) return -1;
  Vec r(n, 0.0);
  r[0] = -t[0] + 0.5 * t[1];
  r[1] = t[0] - t[1] + 0.5 * t[2];
  for (int i = 2; i < n - 1; i++) r[i] = 0.5 * t[i - 1] - t[i] + 0.5 * t[i + 1];
  r[n - 1] = 0.5 * t[n - 2] - t[n - 1];
  t = r;
  return CHEB;
}

// div_xm1_1d_cheb, src/Ope_1d/div_xm1_1d.cpp:27
int div_xm1_line(int basis, Vec& t, int n) {
  if (basis != CHEB) return -1;
  Vec r(n, 0.0);
  for (int i = 0; i < n - 1; i++)
    for (int j = i + 1; j < n; j++) r[i] += 2 * (j - i) * t[j];
  r[0] *= 0.5;
  t = r;
  return CHEB;
}

// div_xp1_1d_cheb, src/Ope_1d/div_xp1_1d.cpp:25
int div_xp1_line(int basis, Vec& t, int n) {
  if (basis != CHEB) return -1;
  Vec r(n, 0.0);
  r[n - 1] = 0;
  r[n - 2] = 2 * t[n - 1];
  for (int i = n - 3; i > 0; i--) r[i] = 2 * t[i + 1] - 2 * r[i + 1] - r[i + 2];
  double s = 0;
  for (int i = 0; i < n; i++) s += (i % 2 == 0) ? t[i] : -t[i];
  r[0] = t[0] - r[1] / 2. - s;
  t = r;
  return CHEB;
}

// div_1mx2_1d_*, src/Ope_1d/div_1mx2.cpp
int div_1mx2_line(int basis, Vec& t, int n) {
  Vec r(n, 0.0);
  switch (basis) {
    case CHEB:
      for (int a = 0; a < n; a++)
        for (int p = a + 2; p < n; p += 2) r[a] += -2 * (p - a) * t[p];
      r[0] *= 0.5;
      t = r;
      return CHEB;
    case CHEB_EVEN:
      for (int a = 0; a < n; a++)
        for (int p = a + 1; p < n; p++) r[a] += -4 * (p - a) * t[p];
      r[0] *= 0.5;
      t = r;
      return CHEB_EVEN;
    case CHEB_ODD:
      for (int a = 0; a < n; a++)
        for (int p = a + 1; p < n; p++) r[a] += -4 * (p - a) * t[p];
      t = r;
      return CHEB_ODD;
    default:
      return -1;
  }
}

int coef_line(int basis, Vec& t, int n_in, int n_out) {
  int nbr = n_in > n_out ? n_in : n_out;
  switch (basis) {
    case CHEB: return coef_cheb(t, nbr);
    case CHEB_EVEN: return coef_cheb_even(t, nbr);
    case CHEB_ODD: return coef_cheb_odd(t, nbr);
    case COSSIN: return coef_cossin(t, nbr);
    case COS: return coef_cos(t, nbr);
    case SIN: return coef_sin(t, nbr);
    case COS_EVEN: return coef_cos_even(t, nbr);
    case COS_ODD: return coef_cos_odd(t, nbr);
    case SIN_EVEN: return coef_sin_even(t, nbr);
    case SIN_ODD: return coef_sin_odd(t, nbr);
    case COSSIN_EVEN: return coef_cossin_parity(t, nbr, false);
    case COSSIN_ODD: return coef_cossin_parity(t, nbr, true);
    default: return -1;  // Legendre collocation is not supported
  }
}

int coefi_line(int basis, Vec& t, int n_in, int n_out) {
  int nbr = n_in > n_out ? n_in : n_out;
  switch (basis) {
    case CHEB: return coefi_cheb(t, nbr);
    case CHEB_EVEN: return coefi_cheb_even(t, nbr);
    case CHEB_ODD: return coefi_cheb_odd(t, nbr);
    case COSSIN: return coefi_cossin(t, nbr);
    case COS: return coefi_cos(t, nbr);
    case SIN: return coefi_sin(t, nbr);
    case COS_EVEN: return coefi_cos_even(t, nbr);
    case COS_ODD: return coefi_cos_odd(t, nbr);
    case SIN_EVEN: return coefi_sin_even(t, nbr);
    case SIN_ODD: return coefi_sin_odd(t, nbr);
    case COSSIN_EVEN: return coefi_cossin_parity(t, nbr, false);
    case COSSIN_ODD: return coefi_cossin_parity(t, nbr, true);
    default: return -1;
  }
}

}  // namespace

const char* basis_name(int b) {
  switch (b) {
    case CHEB: return "CHEB";
    case CHEB_EVEN: return "CHEB_EVEN";
    case CHEB_ODD: return "CHEB_ODD";
    case COSSIN: return "COSSIN";
    case COS: return "COS";
    case COS_EVEN: return "COS_EVEN";
    case COS_ODD: return "COS_ODD";
    case SIN: return "SIN";
    case SIN_EVEN: return "SIN_EVEN";
    case SIN_ODD: return "SIN_ODD";
    case LEG: return "LEG";
    case LEG_EVEN: return "LEG_EVEN";
    case LEG_ODD: return "LEG_ODD";
    case COSSIN_EVEN: return "COSSIN_EVEN";
    case COSSIN_ODD: return "COSSIN_ODD";
    default: return "UNDEF";
  }
}

const char* op_name(int op) {
  static const char* names[] = {"coef",   "coef_i", "der",      "mult_sin", "div_sin",
                                "mult_cos", "div_cos", "mult_x", "div_x",    "mult_xm1",
                                "div_xm1", "div_xp1", "div_1mx2", "identity", "resample"};
  return (op >= 0 && op < OP_COUNT) ? names[op] : "?";
}

// The n collocation points of a line of the given basis in the spherical
// domains (Domain_*::do_coloc): Chebyshev x = -cos(pi i/(n-1)), the
// nucleus's half grid x = sin(pi/2 i/(n-1)), theta on the half sphere
// pi/2 j/(n-1) (on the full range pi j/(n-1) for COS/SIN) and phi 2 pi k/n.
static double grid_point(int basis, int i, int n) {
  const double pi = 3.14159265358979323846;
  switch (basis) {
    case CHEB: return n > 1 ? -std::cos(pi * i / (n - 1)) : 0.0;
    case CHEB_EVEN:
    case CHEB_ODD: return n > 1 ? std::sin(pi / 2. * i / (n - 1)) : 0.0;
    case COS_EVEN:
    case COS_ODD:
    case SIN_EVEN:
    case SIN_ODD: return n > 1 ? pi / 2. * i / (n - 1) : 0.0;
    case COS:
    case SIN: return n > 1 ? pi * i / (n - 1) : 0.0;
    default: return 2. * pi * i / n;  // COSSIN, COSSIN_EVEN, COSSIN_ODD
  }
}

static int resample_line(int basis, std::vector<double>& tab, int n_in, int n_out) {
  std::vector<double> w(n_in), out(n_out, 0.0);
  for (int r = 0; r < n_out; r++) {
    if (!summation_weights_1d(basis, n_in, grid_point(basis, r, n_out), w.data())) return -1;
    double v = 0.0;
    for (int c = 0; c < n_in; c++) v += w[c] * tab[c];
    out[r] = v;
  }
  for (int r = 0; r < n_out; r++) tab[r] = out[r];
  for (size_t r = n_out; r < tab.size(); r++) tab[r] = 0.0;
  return basis;
}

int apply_1d(int op, int basis, std::vector<double>& tab, int n_in, int n_out) {
  int n = n_in > n_out ? n_in : n_out;
  if (static_cast<int>(tab.size()) < n) tab.resize(n, 0.0);
  switch (op) {
    case OP_COEF: return coef_line(basis, tab, n_in, n_out);
    case OP_COEF_I: return coefi_line(basis, tab, n_in, n_out);
    case OP_DER: return der_line(basis, tab, n);
    case OP_MULT_SIN: return mult_sin_line(basis, tab, n);
    case OP_DIV_SIN: return div_sin_line(basis, tab, n);
    case OP_MULT_COS: return mult_cos_line(basis, tab, n);
    case OP_DIV_COS: return div_cos_line(basis, tab, n);
    case OP_MULT_X: return mult_x_line(basis, tab, n);
    case OP_DIV_X: return div_x_line(basis, tab, n);
    case OP_MULT_XM1: return mult_xm1_line(basis, tab, n);
    case OP_DIV_XM1: return div_xm1_line(basis, tab, n);
    case OP_DIV_XP1: return div_xp1_line(basis, tab, n);
    case OP_DIV_1MX2: return div_1mx2_line(basis, tab, n);
    case OP_IDENTITY: return basis;
    case OP_RESAMPLE: return resample_line(basis, tab, n_in, n_out);
    default: return -1;
  }
}

bool build_matrix(int op, int basis, int n_in, int n_out, Mat1d& out) {
  out.op = op;
  out.basis = basis;
  out.n_in = n_in;
  out.n_out = n_out;
  out.m.assign(static_cast<size_t>(n_in) * n_out, 0.0);
  int n = n_in > n_out ? n_in : n_out;
  int ob = -1;
  for (int c = 0; c < n_in; c++) {
    std::vector<double> t(n, 0.0);
    t[c] = 1.0;
    ob = apply_1d(op, basis, t, n_in, n_out);
    if (ob < 0) return false;
    for (int r = 0; r < n_out; r++) out.m[static_cast<size_t>(r) * n_in + c] = t[r];
  }
  out.out_basis = ob;
  return true;
}

int MatrixBank::get(int op, int basis, int n_in, int n_out) {
  auto key = std::make_tuple(op, basis, n_in, n_out);
  auto it = index_.find(key);
  if (it != index_.end()) return it->second;
  Mat1d m;
  if (!build_matrix(op, basis, n_in, n_out, m)) return -1;
  // Keep each matrix 32-byte aligned inside the pool.
  while (pool_.size() % 4) pool_.push_back(0.0);
  m.pool_offset = pool_.size();
  pool_.insert(pool_.end(), m.m.begin(), m.m.end());
  int idx = static_cast<int>(mats_.size());
  mats_.push_back(std::move(m));
  index_[key] = idx;
  version_++;
  return idx;
}

// Chebyshev values by the three-term recurrence, in the order the
// reference's summation_1d_cheb* walks them (the even and odd variants step
// the recurrence twice per coefficient).
bool summation_weights_1d(int basis, int n, double x, double* w) {
  if (n <= 0) return true;
  switch (basis) {
    case CHEB: {
      double tm2 = 1.0, tm1 = x;
      w[0] = tm2;
      if (n > 1) w[1] = tm1;
      for (int i = 2; i < n; i++) {
        const double tm = 2 * x * tm1 - tm2;
        w[i] = tm;
        tm2 = tm1;
        tm1 = tm;
      }
      return true;
    }
    case CHEB_EVEN: {
      double tm2 = 1.0, tm1 = x;
      w[0] = tm2;
      for (int i = 1; i < n; i++) {
        double tm = 2 * x * tm1 - tm2;
        w[i] = tm;
        tm2 = tm1;
        tm1 = tm;
        tm = 2 * x * tm1 - tm2;
        tm2 = tm1;
        tm1 = tm;
      }
      return true;
    }
    case CHEB_ODD: {
      double tm2 = 1.0, tm1 = x;
      w[0] = tm1;
      for (int i = 1; i < n; i++) {
        double tm = 2 * x * tm1 - tm2;
        tm2 = tm1;
        tm1 = tm;
        tm = 2 * x * tm1 - tm2;
        w[i] = tm;
        tm2 = tm1;
        tm1 = tm;
      }
      return true;
    }
    case COSSIN:
      for (int i = 0; i < n; i++) w[i] = (i % 2 == 0) ? std::cos((i / 2) * x) : std::sin((i - 1) / 2 * x);
      return true;
    case COSSIN_EVEN:
      for (int i = 0; i < n; i++) w[i] = (i % 2 == 0) ? std::cos(i * x) : std::sin((i - 1) * x);
      return true;
    case COSSIN_ODD:
      for (int i = 0; i < n; i++) w[i] = (i % 2 == 0) ? std::cos((i + 1) * x) : std::sin(i * x);
      return true;
    case COS:
      for (int i = 0; i < n; i++) w[i] = std::cos(i * x);
      return true;
    case SIN:
      for (int i = 0; i < n; i++) w[i] = std::sin(i * x);
      return true;
    case COS_EVEN:
      for (int i = 0; i < n; i++) w[i] = std::cos(2 * i * x);
      return true;
    case COS_ODD:
      for (int i = 0; i < n; i++) w[i] = std::cos((2 * i + 1) * x);
      return true;
    case SIN_EVEN:
      for (int i = 0; i < n; i++) w[i] = std::sin(2 * i * x);
      return true;
    case SIN_ODD:
      for (int i = 0; i < n; i++) w[i] = std::sin((2 * i + 1) * x);
      return true;
    default:
      return false;
  }
}

}  // namespace kd
