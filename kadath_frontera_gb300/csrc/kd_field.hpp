// DVal: Kadath's Val_domain on the GPU (src/Val_domain/val_domain.cpp).
//
// A DVal is the value of one scalar in one domain, held as a batch of B
// fields (B = 1 for values, B = number of Jacobian columns for tangents).
// It keeps the reference's lazy two-representation state machine: the field
// may be known at the collocation points (c), as coefficients (cf), or both;
// coef()/coef_i() fill the missing side on demand.  Every operation launches
// device kernels and never writes into an input's buffers, so DVal copies can
// share storage.  Storage comes from the context's scratch arena.
#pragma once
#include <array>
#include <memory>

#include "kd_domain.hpp"

namespace kd {

class DVal {
 public:
  Context* ctx = nullptr;
  const Domain* dom = nullptr;
  int batch = 1;
  bool zero = true;
  Base base;
  mutable bool in_conf = false, in_coef = false;
  mutable const double* c = nullptr;
  mutable const double* cf = nullptr;

  DVal() = default;
  DVal(Context* ctx_, const Domain* d, int b = 1) : ctx(ctx_), dom(d), batch(b) {}

  static DVal zeros(Context* ctx, const Domain* d, int batch = 1);
  static DVal constant(Context* ctx, const Domain* d, double v);  // conf filled, base undefined
  static DVal from_conf(Context* ctx, const Domain* d, int batch, const double* c, const Base& b);
  static DVal from_coef(Context* ctx, const Domain* d, int batch, const double* cf, const Base& b);

  bool is_zero() const { return zero; }
  int npts() const { return dom->npts(); }
  int ncoefs() const { return dom->ncoefs(); }

  void coef() const;    // Val_domain::coef (val_domain.cpp:551)
  void coef_i() const;  // Val_domain::coef_i (val_domain.cpp:570)

  // Val_domain::der_var / der_abs (val_domain.cpp:603-700); var in 1..3.
  DVal der_var(int var) const;
  DVal der_abs(int var) const;
  // The same value without its lazily computed derivatives.
  DVal plain() const {
    DVal d = *this;
    d.dvar_.reset();
    d.dabs_.reset();
    return d;
  }

 private:
  mutable std::shared_ptr<std::array<std::shared_ptr<DVal>, 3>> dvar_, dabs_;
  void compute_der_var() const;
  void compute_der_abs() const;
};

// Arithmetic (src/Val_domain/val_domain_math.cpp).  Batches broadcast 1 <-> B.
DVal operator+(const DVal& a, const DVal& b);
DVal operator-(const DVal& a, const DVal& b);
DVal operator*(const DVal& a, const DVal& b);
DVal operator/(const DVal& a, const DVal& b);
DVal operator-(const DVal& a);
DVal operator+(const DVal& a, double x);
DVal operator-(const DVal& a, double x);
DVal operator-(double x, const DVal& a);
DVal operator*(const DVal& a, double x);
DVal operator/(const DVal& a, double x);
DVal operator/(double x, const DVal& a);
DVal pow_int(const DVal& a, int n);
DVal pow_double(const DVal& a, double x);
DVal vd_sqrt(const DVal& a);
DVal vd_exp(const DVal& a);
DVal vd_log(const DVal& a);
DVal vd_sin(const DVal& a);
DVal vd_cos(const DVal& a);
DVal vd_atan(const DVal& a);
// cosh / sinh / atanh of Val_domain (src/Val_domain/val_domain_math.cpp):
// at the collocation points.  cosh and sinh of a zero field give 1 with the
// operand's basis (sinh too, as the reference does); otherwise no basis, as
// for sin and cos.  atanh keeps the operand's basis.
DVal vd_cosh(const DVal& a);
DVal vd_sinh(const DVal& a);
DVal vd_atanh(const DVal& a);

// Domain operators (src/Domain/Spheric/domain_*_ope.cpp and do_der_abs_from_der_var).
DVal ope_coef(const DVal& so, int op, int dim);  // generic ope_1d on the coefficients
DVal mult_cos_phi(const DVal& so);
DVal mult_sin_phi(const DVal& so);
DVal mult_cos_theta(const DVal& so);
DVal mult_sin_theta(const DVal& so);
DVal div_sin_theta(const DVal& so);
DVal div_cos_theta(const DVal& so);
DVal div_x(const DVal& so);
DVal mult_xm1(const DVal& so);
DVal div_xm1(const DVal& so);
DVal mult_r(const DVal& so);
DVal div_r(const DVal& so);
DVal der_r(const DVal& so);
// Domain_*::laplacian2 with m = 0 (Ope_lap2): d2/dr2 + (d/dr + d2/dtheta2 / r) / r.
DVal laplacian2(const DVal& so);
DVal der_normal(const DVal& so, int bound);
DVal laplacian(const DVal& so);  // Domain::laplacian (domain.cpp:155)
DVal radius_field(Context* ctx, const Domain* d);

// EOS<eos, var>::action pieces (include/EOS/EOS.hh:67-160): the value of
// var at the enthalpy h (term_by_term) and its variation for a tangent
// batch dh at h (term_by_term_variation), pointwise at collocation points.
DVal eos_value(const DVal& h, const KdEos& e, int var);
DVal eos_variation(const DVal& dh, const DVal& h, const KdEos& e, int var);

}  // namespace kd
