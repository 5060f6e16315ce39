#include "kd_field.hpp"

#include <cmath>

namespace kd {

namespace {

double* alloc(Context* ctx, long long n) { return ctx->scratch().alloc_doubles(static_cast<size_t>(n)); }

void ew(Context* ctx, int op, long long npts, int ba, const double* a, int bb, const double* b, double* out,
        double alpha = 0.0, double beta = 0.0) {
  int nf = ba > bb ? ba : bb;
  ProfScope ps(ctx, Context::PROF_EW,
               8.0 * npts * ((a ? ba : 0) + (b ? bb : 0) + nf));
  cuda_check(launch_ew(op, npts, ba, a, bb, b, out, alpha, beta, ctx->stream()), "elementwise kernel");
  ctx->launches++;
}

void run_specs(Context* ctx, const std::vector<LinePassSpec>& specs, const double* in, double* out,
               const int dims_in[3], long long in_stride, long long out_stride, int batch, double scale = 1.0) {
  KdItem it = make_item(*ctx, specs, in, out, dims_in, in_stride, out_stride, scale);
  ctx->run_items({it}, {batch});
}

int max_batch(const DVal& a, const DVal& b) { return a.batch > b.batch ? a.batch : b.batch; }

void check_same_domain(const DVal& a, const DVal& b) {
  if (a.dom != b.dom) throw KdError(KD_ERR_ARG, "operation between fields of different domains");
}

// Elementwise binary op in configuration space.
DVal conf_binary(int op, const DVal& a, const DVal& b) {
  a.coef_i();
  b.coef_i();
  DVal res(a.ctx, a.dom, max_batch(a, b));
  res.zero = false;
  double* out = alloc(a.ctx, static_cast<long long>(res.batch) * a.npts());
  ew(a.ctx, op, a.npts(), a.batch, a.c, b.batch, b.c, out);
  res.c = out;
  res.in_conf = true;
  return res;
}

// Scales every representation the field holds (Val_domain * double, or
// Val_domain / double when `op` is EW_DIVC).
DVal scaled(const DVal& a, double x, int op = EW_SCALE) {
  DVal res = a;
  res.in_conf = a.in_conf;
  res.in_coef = a.in_coef;
  if (a.in_conf) {
    double* o = alloc(a.ctx, static_cast<long long>(a.batch) * a.npts());
    ew(a.ctx, op, static_cast<long long>(a.batch) * a.npts(), 1, a.c, 1, nullptr, o, x);
    res.c = o;
  }
  if (a.in_coef) {
    double* o = alloc(a.ctx, static_cast<long long>(a.batch) * a.ncoefs());
    ew(a.ctx, op, static_cast<long long>(a.batch) * a.ncoefs(), 1, a.cf, 1, nullptr, o, x);
    res.cf = o;
  }
  return res;
}

DVal conf_unary(int op, const DVal& a, double alpha = 0.0) {
  a.coef_i();
  DVal res(a.ctx, a.dom, a.batch);
  res.zero = false;
  double* o = alloc(a.ctx, static_cast<long long>(a.batch) * a.npts());
  ew(a.ctx, op, static_cast<long long>(a.batch) * a.npts(), 1, a.c, 1, nullptr, o, alpha);
  res.c = o;
  res.in_conf = true;
  return res;
}

DVal filled(Context* ctx, const Domain* d, int batch, double v) {
  DVal res(ctx, d, batch);
  res.zero = false;
  double* o = alloc(ctx, static_cast<long long>(batch) * d->npts());
  ew(ctx, EW_FILL, static_cast<long long>(batch) * d->npts(), 1, nullptr, 1, nullptr, o, v);
  res.c = o;
  res.in_conf = true;
  return res;
}

// Theta basis swap applied by multiplication with cos(phi) or sin(phi).
int swap_theta(int b) {
  switch (b) {
    case COS_EVEN: return SIN_ODD;
    case COS_ODD: return SIN_EVEN;
    case SIN_EVEN: return COS_ODD;
    case SIN_ODD: return COS_EVEN;
    default: throw KdError(KD_ERR_UNSUPPORTED, "Unknown case in Domain::mult_cos_phi");
  }
}

}  // namespace

DVal DVal::zeros(Context* ctx, const Domain* d, int batch) {
  DVal v(ctx, d, batch);
  v.zero = true;
  return v;
}

DVal DVal::constant(Context* ctx, const Domain* d, double x) {
  if (x == 0) return zeros(ctx, d, 1);
  return filled(ctx, d, 1, x);
}

DVal DVal::from_conf(Context* ctx, const Domain* d, int batch, const double* c, const Base& b) {
  DVal v(ctx, d, batch);
  v.zero = false;
  v.c = c;
  v.in_conf = true;
  v.base = b;
  return v;
}

DVal DVal::from_coef(Context* ctx, const Domain* d, int batch, const double* cf, const Base& b) {
  DVal v(ctx, d, batch);
  v.zero = false;
  v.cf = cf;
  v.in_coef = true;
  v.base = b;
  return v;
}

void DVal::coef() const {
  if (in_coef || zero) return;
  if (!base.def) throw KdError(KD_ERR_STATE, "Base not defined in Val_domain::coef");
  double* out = alloc(ctx, static_cast<long long>(batch) * ncoefs());
  auto specs = coef_specs(*ctx, base, dom->np, dom->nc);
  run_specs(ctx, specs, c, out, dom->np, npts(), ncoefs(), batch);
  cf = out;
  in_coef = true;
}

void DVal::coef_i() const {
  if (in_conf || zero) return;
  if (!base.def) throw KdError(KD_ERR_STATE, "Base not defined in Val_domain::coef_i");
  double* out = alloc(ctx, static_cast<long long>(batch) * npts());
  auto specs = coef_i_specs(*ctx, base, dom->np, dom->nc);
  run_specs(ctx, specs, cf, out, dom->nc, ncoefs(), npts(), batch);
  c = out;
  in_conf = true;
}

void DVal::compute_der_var() const {
  coef();
  auto arr = std::make_shared<std::array<std::shared_ptr<DVal>, 3>>();
  std::vector<KdItem> items;
  std::vector<int> batches;
  for (int var = 0; var < 3; var++) {
    auto res = std::make_shared<DVal>(ctx, dom, batch);
    res->zero = false;
    res->base = base;
    auto spec = ope_1d_spec(*ctx, OP_DER, var, base, dom->nc, res->base);
    double* out = alloc(ctx, static_cast<long long>(batch) * ncoefs());
    items.push_back(make_item(*ctx, {spec}, cf, out, dom->nc, ncoefs(), ncoefs(), 1.0));
    batches.push_back(batch);
    res->cf = out;
    res->in_coef = true;
    (*arr)[var] = res;
  }
  // The three derivatives run in one launch.
  ctx->run_items(items, batches);
  dvar_ = arr;
}

DVal DVal::der_var(int var) const {
  if (var < 1 || var > 3) throw KdError(KD_ERR_ARG, "der_var index must be 1..3");
  if (zero) return *this;
  if (!dvar_) compute_der_var();
  return *(*dvar_)[var - 1];
}

void DVal::compute_der_abs() const {
  if (!dvar_) compute_der_var();
  const DVal dv[3] = {*(*dvar_)[0], *(*dvar_)[1], *(*dvar_)[2]};
  auto arr = std::make_shared<std::array<std::shared_ptr<DVal>, 3>>();
  const double alpha = dom->alpha;
  if (dom->type == DOM_SHELL) {
    // Domain_shell::do_der_abs_from_der_var (domain_shell.cpp:665)
    DVal sintdr = mult_sin_theta(dv[0]) / alpha;
    DVal rad = radius_field(ctx, dom);
    DVal dtsr = dv[1] / rad;
    dtsr.base = dv[1].base;
    DVal dpsr = dv[2] / rad;
    dpsr.base = dv[2].base;
    DVal costdtsr = mult_cos_theta(dtsr);
    DVal dpsrssint = div_sin_theta(dpsr);
    DVal s = sintdr + costdtsr;
    (*arr)[0] = std::make_shared<DVal>(mult_cos_phi(s) - mult_sin_phi(dpsrssint));
    (*arr)[1] = std::make_shared<DVal>(mult_sin_phi(s) + mult_cos_phi(dpsrssint));
    (*arr)[2] = std::make_shared<DVal>(mult_cos_theta(dv[0]) / alpha - mult_sin_theta(dtsr));
  } else if (dom->type == DOM_NUCLEUS) {
    // Domain_nucleus::do_der_abs_from_der_var (domain_nucleus.cpp:534)
    DVal sintdr = mult_sin_theta(dv[0]) / alpha;
    DVal dtsr = div_x(dv[1]) / alpha;
    DVal dpsr = div_x(dv[2]) / alpha;
    DVal costdtsr = mult_cos_theta(dtsr);
    DVal dpsrssint = div_sin_theta(dpsr);
    DVal s = sintdr + costdtsr;
    (*arr)[0] = std::make_shared<DVal>(mult_cos_phi(s) - mult_sin_phi(dpsrssint));
    (*arr)[1] = std::make_shared<DVal>(mult_sin_phi(s) + mult_cos_phi(dpsrssint));
    (*arr)[2] = std::make_shared<DVal>(mult_cos_theta(dv[0]) / alpha - mult_sin_theta(dtsr));
  } else {
    // Domain_compact::do_der_abs_from_der_var (domain_compact.cpp:674)
    DVal dr = -mult_xm1(dv[0]);
    DVal sintdr = mult_sin_theta(dr);
    DVal costdt = mult_cos_theta(dv[1]);
    DVal dpssint = div_sin_theta(dv[2]);
    DVal s = sintdr + costdt;
    DVal ax = mult_cos_phi(s) - mult_sin_phi(dpssint);
    (*arr)[0] = std::make_shared<DVal>(mult_xm1(ax) * alpha);
    DVal ay = mult_sin_phi(s) + mult_cos_phi(dpssint);
    (*arr)[1] = std::make_shared<DVal>(mult_xm1(ay) * alpha);
    DVal az = mult_cos_theta(dr) - mult_sin_theta(dv[1]);
    (*arr)[2] = std::make_shared<DVal>(mult_xm1(az) * alpha);
  }
  dabs_ = arr;
}

DVal DVal::der_abs(int var) const {
  if (var < 1 || var > 3) throw KdError(KD_ERR_ARG, "der_abs index must be 1..3");
  if (zero) return *this;
  if (!dabs_) compute_der_abs();
  return *(*dabs_)[var - 1];
}

// ------------------------------------------------------------- algebra --
DVal operator+(const DVal& a, const DVal& b) {
  check_same_domain(a, b);
  if (a.zero) return b;
  if (b.zero) return a;
  DVal res(a.ctx, a.dom, max_batch(a, b));
  res.zero = false;
  if (a.in_conf || b.in_conf) {
    a.coef_i();
    b.coef_i();
    double* o = alloc(a.ctx, static_cast<long long>(res.batch) * a.npts());
    ew(a.ctx, EW_ADD, a.npts(), a.batch, a.c, b.batch, b.c, o);
    res.c = o;
    res.in_conf = true;
  } else {
    a.coef();
    b.coef();
    double* o = alloc(a.ctx, static_cast<long long>(res.batch) * a.ncoefs());
    ew(a.ctx, EW_ADD, a.ncoefs(), a.batch, a.cf, b.batch, b.cf, o);
    res.cf = o;
    res.in_coef = true;
  }
  if (a.base.def && b.base.def) res.base = a.base;
  return res;
}

DVal operator-(const DVal& a) {
  if (a.zero) return a;
  return scaled(a, -1.0);
}

DVal operator-(const DVal& a, const DVal& b) {
  check_same_domain(a, b);
  if (a.zero) return -b;
  if (b.zero) return a;
  DVal res(a.ctx, a.dom, max_batch(a, b));
  res.zero = false;
  if (a.in_conf || b.in_conf) {
    a.coef_i();
    b.coef_i();
    double* o = alloc(a.ctx, static_cast<long long>(res.batch) * a.npts());
    ew(a.ctx, EW_SUB, a.npts(), a.batch, a.c, b.batch, b.c, o);
    res.c = o;
    res.in_conf = true;
  } else {
    a.coef();
    b.coef();
    double* o = alloc(a.ctx, static_cast<long long>(res.batch) * a.ncoefs());
    ew(a.ctx, EW_SUB, a.ncoefs(), a.batch, a.cf, b.batch, b.cf, o);
    res.cf = o;
    res.in_coef = true;
  }
  if (a.base.def && b.base.def) res.base = a.base;
  return res;
}

DVal operator*(const DVal& a, const DVal& b) {
  check_same_domain(a, b);
  if (a.zero) return a.batch >= b.batch ? a : DVal::zeros(a.ctx, a.dom, b.batch);
  if (b.zero) return b.batch >= a.batch ? b : DVal::zeros(a.ctx, a.dom, a.batch);
  DVal res = conf_binary(EW_MUL, a, b);
  res.base = a.dom->mult(a.base, b.base);
  return res;
}

DVal operator/(const DVal& a, const DVal& b) {
  check_same_domain(a, b);
  if (a.zero) return a;
  if (b.zero) throw KdError(KD_ERR_ARG, "Division by zero");
  DVal res = conf_binary(EW_DIV, a, b);
  res.base = a.dom->mult(a.base, b.base);
  return res;
}

DVal operator+(const DVal& a, double x) {
  if (a.zero) {
    DVal res = filled(a.ctx, a.dom, 1, x);
    res.base = a.dom->std_base();
    return res;
  }
  DVal res = conf_unary(EW_ADDC, a, x);
  res.base = a.base;
  return res;
}

DVal operator-(const DVal& a, double x) { return a + (-x); }

DVal operator-(double x, const DVal& a) {
  if (a.zero) {
    DVal res = filled(a.ctx, a.dom, 1, x);
    res.base = a.dom->std_base();
    return res;
  }
  DVal res = conf_unary(EW_CSUB, a, x);
  res.base = a.base;
  return res;
}

DVal operator*(const DVal& a, double x) {
  if (a.zero) return a;
  return scaled(a, x);
}

DVal operator/(const DVal& a, double x) {
  if (a.zero) return a;
  return scaled(a, x, EW_DIVC);
}

DVal operator/(double x, const DVal& a) {
  if (a.zero) throw KdError(KD_ERR_ARG, "Division by zero");
  DVal res = conf_unary(EW_CDIV, a, x);
  res.base = a.dom->std_base();
  return res;
}

DVal pow_int(const DVal& a, int n) {
  if (a.zero) return a;
  if (n <= 0) return conf_unary(EW_POWI, a, static_cast<double>(n));  // base left undefined
  DVal res = a;
  for (int i = 1; i < n; i++) res = res * a;
  return res;
}

DVal pow_double(const DVal& a, double x) {
  if (a.zero) return a;
  return conf_unary(EW_POWD, a, x);  // base left undefined, as in the reference
}

DVal vd_sqrt(const DVal& a) {
  if (a.zero) return a;
  DVal r = conf_unary(EW_SQRT, a);
  r.base = a.base;
  return r;
}

DVal vd_exp(const DVal& a) {
  if (a.zero) return filled(a.ctx, a.dom, a.batch, 1.0);
  DVal r = conf_unary(EW_EXP, a);
  r.base = a.base;
  return r;
}

DVal eos_value(const DVal& h, const KdEos& e, int var) {
  if (h.zero) return h;
  h.coef_i();
  DVal res(h.ctx, h.dom, h.batch);
  res.zero = false;
  const long long n = static_cast<long long>(h.batch) * h.npts();
  double* o = alloc(h.ctx, n);
  ProfScope ps(h.ctx, Context::PROF_EW, 16.0 * n);
  cuda_check(launch_eos(e, var, n, h.c, 1, nullptr, o, h.ctx->stream()), "eos kernel");
  h.ctx->launches++;
  res.c = o;
  res.in_conf = true;
  res.base = h.base;
  return res;
}

DVal eos_variation(const DVal& dh, const DVal& h, const KdEos& e, int var) {
  if (dh.zero) return dh;
  if (h.zero) return DVal::zeros(dh.ctx, dh.dom, dh.batch);
  if (h.batch != 1) throw KdError(KD_ERR_STATE, "eos variation needs a single value field");
  dh.coef_i();
  h.coef_i();
  DVal res(dh.ctx, dh.dom, dh.batch);
  res.zero = false;
  const long long npts = h.npts();
  double* o = alloc(dh.ctx, npts * dh.batch);
  ProfScope ps(dh.ctx, Context::PROF_EW, 16.0 * npts * dh.batch);
  cuda_check(launch_eos(e, var, npts, h.c, dh.batch, dh.c, o, dh.ctx->stream()), "eos variation kernel");
  dh.ctx->launches++;
  res.c = o;
  res.in_conf = true;
  res.base = dh.base;
  return res;
}

DVal vd_log(const DVal& a) {
  DVal r = conf_unary(EW_LOG, a);
  r.base = a.base;
  return r;
}

DVal vd_sin(const DVal& a) {
  if (a.zero) return a;
  return conf_unary(EW_SIN, a);
}

DVal vd_cos(const DVal& a) {
  if (a.zero) return filled(a.ctx, a.dom, a.batch, 1.0);
  return conf_unary(EW_COS, a);
}

DVal vd_atan(const DVal& a) {
  DVal r = conf_unary(EW_ATAN, a);
  r.base = a.base;
  return r;
}

DVal vd_cosh(const DVal& a) {
  if (a.zero) {
    DVal r = filled(a.ctx, a.dom, a.batch, 1.0);
    r.base = a.base;
    return r;
  }
  return conf_unary(EW_COSH, a);
}

DVal vd_sinh(const DVal& a) {
  if (a.zero) {
    DVal r = filled(a.ctx, a.dom, a.batch, 1.0);
    r.base = a.base;
    return r;
  }
  return conf_unary(EW_SINH, a);
}

DVal vd_atanh(const DVal& a) {
  if (a.zero) return a;
  DVal r = conf_unary(EW_ATANH, a);
  r.base = a.base;
  return r;
}

// ------------------------------------------------------- domain operators --
DVal ope_coef(const DVal& so, int op, int dim) {
  so.coef();
  DVal res(so.ctx, so.dom, so.batch);
  res.zero = false;
  res.base = so.base;
  auto spec = ope_1d_spec(*so.ctx, op, dim, so.base, so.dom->nc, res.base);
  double* out = alloc(so.ctx, static_cast<long long>(so.batch) * so.ncoefs());
  run_specs(so.ctx, {spec}, so.cf, out, so.dom->nc, so.ncoefs(), so.ncoefs(), so.batch);
  res.cf = out;
  res.in_coef = true;
  return res;
}

static DVal mult_trig_phi(const DVal& so, int op) {
  if (so.zero) return so;
  so.coef();
  DVal res(so.ctx, so.dom, so.batch);
  res.zero = false;
  res.base = so.base;
  for (int k = 0; k < so.base.n2c; k++) res.base.t[k] = swap_theta(so.base.t[k]);
  if (so.dom->type == DOM_NUCLEUS)
    for (auto& r : res.base.r) {
      if (r == CHEB_EVEN) r = CHEB_ODD;
      else if (r == CHEB_ODD) r = CHEB_EVEN;
      else throw KdError(KD_ERR_UNSUPPORTED, "Unknown case in Domain_nucleus::mult_cos_phi");
    }
  Base tmp = res.base;
  auto spec = ope_1d_spec(*so.ctx, op, 2, so.base, so.dom->nc, tmp);
  res.base.p = tmp.p;
  double* out = alloc(so.ctx, static_cast<long long>(so.batch) * so.ncoefs());
  run_specs(so.ctx, {spec}, so.cf, out, so.dom->nc, so.ncoefs(), so.ncoefs(), so.batch);
  res.cf = out;
  res.in_coef = true;
  return res;
}

DVal mult_cos_phi(const DVal& so) { return mult_trig_phi(so, OP_MULT_COS); }
DVal mult_sin_phi(const DVal& so) { return mult_trig_phi(so, OP_MULT_SIN); }
DVal mult_cos_theta(const DVal& so) { return so.zero ? so : ope_coef(so, OP_MULT_COS, 1); }
DVal mult_sin_theta(const DVal& so) { return so.zero ? so : ope_coef(so, OP_MULT_SIN, 1); }
DVal div_sin_theta(const DVal& so) { return so.zero ? so : ope_coef(so, OP_DIV_SIN, 1); }
DVal div_cos_theta(const DVal& so) { return so.zero ? so : ope_coef(so, OP_DIV_COS, 1); }
DVal div_x(const DVal& so) { return so.zero ? so : ope_coef(so, OP_DIV_X, 0); }
DVal mult_xm1(const DVal& so) { return so.zero ? so : ope_coef(so, OP_MULT_XM1, 0); }
DVal div_xm1(const DVal& so) { return so.zero ? so : ope_coef(so, OP_DIV_XM1, 0); }

DVal radius_field(Context* ctx, const Domain* d) {
  const double* r = ctx->dtable(d->radius_values());
  DVal v = DVal::from_conf(ctx, d, 1, r, Base());
  return v;
}

DVal mult_r(const DVal& so) {
  if (so.zero) return so;
  const Domain* d = so.dom;
  if (d->type == DOM_NUCLEUS) {
    // Domain_nucleus::mult_r: mult_x then *alpha on the coefficients
    return ope_coef(so, OP_MULT_X, 0) * d->alpha;
  }
  if (d->type == DOM_SHELL) {
    // Domain_shell::mult_r: alpha * mult_x(cf) + beta * cf
    so.coef();
    DVal mx = ope_coef(so, OP_MULT_X, 0);
    DVal res(so.ctx, d, so.batch);
    res.zero = false;
    res.base = so.base;
    double* o = alloc(so.ctx, static_cast<long long>(so.batch) * so.ncoefs());
    ew(so.ctx, EW_AXPBY, static_cast<long long>(so.batch) * so.ncoefs(), 1, mx.cf, 1, so.cf, o, d->alpha, d->beta);
    res.cf = o;
    res.in_coef = true;
    return res;
  }
  // Domain_compact::mult_r: div_xm1 then / alpha
  return div_xm1(so) / d->alpha;
}

DVal div_r(const DVal& so) {
  if (so.zero) return so;
  const Domain* d = so.dom;
  if (d->type == DOM_NUCLEUS) return ope_coef(so, OP_DIV_X, 0) / d->alpha;
  if (d->type == DOM_SHELL) {
    DVal res = so / radius_field(so.ctx, d);
    res.base = so.base;
    return res;
  }
  return mult_xm1(so) * d->alpha;
}

DVal der_r(const DVal& so) {
  const Domain* d = so.dom;
  if (d->type == DOM_COMPACT) return mult_xm1(mult_xm1(so.der_var(1))) * (-d->alpha);
  return so.der_var(1) / d->alpha;
}

DVal der_normal(const DVal& so, int bound) {
  const Domain* d = so.dom;
  if (!d->has_boundary(bound)) throw KdError(KD_ERR_ARG, "Unknown boundary case in der_normal");
  if (d->type == DOM_COMPACT) {
    DVal res = mult_xm1(mult_xm1(so.der_var(1)));
    return res * (-d->alpha);
  }
  return so.der_var(1) / d->alpha;
}

// Domain_nucleus::laplacian2 (domain_nucleus_ope.cpp:250), Domain_shell
// (domain_shell_ope.cpp:271), Domain_compact (domain_compact_ope.cpp:217),
// for m = 0 (no m quantum number is set by the equations here).
DVal laplacian2(const DVal& so) {
  const Domain* d = so.dom;
  const DVal dert = so.der_var(2);
  if (d->type == DOM_COMPACT) {
    const DVal derr = mult_xm1(mult_xm1(so.der_var(1))) * (-d->alpha);
    const DVal dderr = mult_xm1(mult_xm1(derr.der_var(1))) * (-d->alpha);
    return dderr + div_r(derr + div_r(dert.der_var(2)));
  }
  const DVal derr = so.der_var(1) / d->alpha;
  return derr.der_var(1) / d->alpha + div_r(derr + div_r(dert.der_var(2)));
}

DVal laplacian(const DVal& so) {
  DVal res = so.der_abs(1).der_abs(1);
  for (int j = 2; j <= 3; j++) res = res + so.der_abs(j).der_abs(j);
  return res;
}

}  // namespace kd
