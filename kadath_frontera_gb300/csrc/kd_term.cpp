#include "kd_term.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "kd_system.hpp"

namespace kd {

// ----------------------------------------------------------- Term algebra --
// src/Term_eq/term_eq_math.cpp.  A tangent that is exactly zero (a double
// constant's der_d = 0, or an untouched field) is skipped: adding or
// multiplying it only produces exact zeros.

namespace {

bool dd_zero(const Term& t) { return !t.has_dd || (t.ddv == nullptr && t.dd == 0.0); }

// A double whose tangent differs from seed to seed only combines with
// other doubles here (the integral and point-value equations).
void no_seed_tangent(const Term& d) {
  if (d.ddv)
    throw KdError(KD_ERR_UNSUPPORTED,
                  "a double depending on the seeded fields (integral or point value) combined with a field");
}

void check_dom(const Term& a, const Term& b) {
  if (a.dom != b.dom) throw KdError(KD_ERR_ARG, "Term_eq operation across domains");
}

Term tensor_like(const Term& t) {
  Term r;
  r.dom = t.dom;
  r.valence = t.valence;
  r.idx = t.idx;
  return r;
}

int ncomp(const Term& t) { return static_cast<int>(t.vt.size()); }

void check_valence(const Term& a, const Term& b) {
  if (a.vt.size() != b.vt.size())
    throw KdError(KD_ERR_UNSUPPORTED, "tensor operation between different valences");
}

int pow3(int n) {
  int r = 1;
  for (int i = 0; i < n; i++) r *= 3;
  return r;
}

// Component position of multi-index m (row-major, 3 values per index).
int flat_index(const int* m, int n) {
  int f = 0;
  for (int i = 0; i < n; i++) f = 3 * f + m[i];
  return f;
}

void unflatten(int f, int n, int* m) {
  for (int i = n - 1; i >= 0; i--) {
    m[i] = f % 3;
    f /= 3;
  }
}

}  // namespace

// b's components in the index order of a (sums of named tensors with the
// same indices in another order, as Ope_add/Ope_sub match name_ind).
Term align_to(const Term& b, const Term& a) {
  if (a.idx.empty() || b.idx.empty() || a.idx == b.idx) return b;
  const int n = static_cast<int>(a.idx.size());
  std::string sa = a.idx, sb = b.idx;
  std::sort(sa.begin(), sa.end());
  std::sort(sb.begin(), sb.end());
  if (sa != sb || static_cast<int>(b.idx.size()) != n)
    throw KdError(KD_ERR_ARG, "sum of tensors with different indices: " + a.idx + " and " + b.idx);
  int where[8];
  for (int i = 0; i < n; i++) where[i] = static_cast<int>(b.idx.find(a.idx[i]));
  Term r = b;
  r.idx = a.idx;
  int ma[8], mb[8];
  for (int f = 0; f < pow3(n); f++) {
    unflatten(f, n, ma);
    for (int i = 0; i < n; i++) mb[where[i]] = ma[i];
    const int g = flat_index(mb, n);
    r.vt[f] = b.vt[g];
    if (b.has_dt) r.dt[f] = b.dt[g];
  }
  return r;
}

// Sum over every index name that appears twice in t (Einstein convention,
// flat metric): the terms in the order 1, 2, 3 of the repeated index.
Term contract_self(const Term& t) {
  const int n = static_cast<int>(t.idx.size());
  int p = -1, q = -1;
  for (int i = 0; i < n && p < 0; i++)
    for (int j = i + 1; j < n; j++)
      if (t.idx[i] == t.idx[j]) {
        p = i;
        q = j;
        break;
      }
  if (p < 0) return t;
  Term r;
  r.dom = t.dom;
  for (int i = 0; i < n; i++)
    if (i != p && i != q) r.idx.push_back(t.idx[i]);
  r.valence = n - 2;
  r.has_dt = t.has_dt;
  int mr[8], mt[8];
  for (int f = 0; f < pow3(n - 2); f++) {
    unflatten(f, n - 2, mr);
    for (int i = 0, k = 0; i < n; i++)
      if (i != p && i != q) mt[i] = mr[k++];
    DVal v, d;
    for (int c = 0; c < 3; c++) {
      mt[p] = mt[q] = c;
      const int g = flat_index(mt, n);
      v = (c == 0) ? t.vt[g] : v + t.vt[g];
      if (t.has_dt) d = (c == 0) ? t.dt[g] : d + t.dt[g];
    }
    r.vt.push_back(v);
    if (t.has_dt) r.dt.push_back(d);
  }
  return contract_self(r);
}

namespace {

// Product of two named tensors: outer product, then the sum over the index
// names the two share; value sum_c a_c b_c and tangent sum_c (a'_c b_c +
// a_c b'_c), the terms in the order of the contracted components.
Term tensor_product(const Term& a, const Term& b, const Term* cv, bool do_der) {
  if (a.idx.empty() || b.idx.empty())
    throw KdError(KD_ERR_UNSUPPORTED, "product of two non-scalar tensors without index names: use scal()");
  const int na = static_cast<int>(a.idx.size()), nb = static_cast<int>(b.idx.size());
  std::string free_a, free_b, shared;
  for (char c : a.idx)
    if (b.idx.find(c) == std::string::npos) free_a.push_back(c);
    else shared.push_back(c);
  for (char c : b.idx)
    if (a.idx.find(c) == std::string::npos) free_b.push_back(c);
  Term r;
  r.dom = a.dom;
  r.idx = free_a + free_b;
  r.valence = static_cast<int>(r.idx.size());
  r.has_dt = do_der;
  const int nr = r.valence, ns = static_cast<int>(shared.size());
  int mr[8], ms[8], ma[8], mb[8];
  for (int f = 0; f < pow3(nr); f++) {
    unflatten(f, nr, mr);
    DVal v, d;
    for (int g = 0; g < pow3(ns); g++) {
      unflatten(g, ns, ms);
      auto value_of = [&](char c) {
        size_t k = r.idx.find(c);
        if (k != std::string::npos) return mr[k];
        return ms[shared.find(c)];
      };
      for (int i = 0; i < na; i++) ma[i] = value_of(a.idx[i]);
      for (int i = 0; i < nb; i++) mb[i] = value_of(b.idx[i]);
      const int ia = flat_index(ma, na), ib = flat_index(mb, nb);
      if (!cv) {
        DVal pv = a.vt[ia] * b.vt[ib];
        v = (g == 0) ? pv : v + pv;
      }
      if (do_der) {
        DVal pd = a.dt[ia] * b.vt[ib] + a.vt[ia] * b.dt[ib];
        d = (g == 0) ? pd : d + pd;
      }
    }
    if (!cv) r.vt.push_back(v);
    if (do_der) r.dt.push_back(d);
  }
  if (cv) r.vt = cv->vt;
  return r;
}

}  // namespace

void dbl_tangent_lincomb(Term& r, double ca, const Term& a, double cb, const Term* b) {
  r.has_dd = true;
  if (!a.ddv && !(b && b->ddv)) {
    r.dd = ca * a.dd + (b ? cb * b->dd : 0.0);
    r.ddv = nullptr;
    return;
  }
  const Term& src = a.ddv ? a : *b;
  if (a.ddv && b && b->ddv && a.ddb != b->ddb) throw KdError(KD_ERR_STATE, "double tangents of different batches");
  Context* ctx = src.ddctx;
  double* out = ctx->scratch().alloc_doubles(src.ddb);
  cuda_check(launch_lincomb2(src.ddb, ca, a.ddv, a.dd, b ? cb : 0.0, b ? b->ddv : nullptr, b ? b->dd : 0.0, out,
                             ctx->stream()),
             "double tangent");
  ctx->launches++;
  r.dd = 0.0;
  r.ddv = out;
  r.ddb = src.ddb;
  r.ddctx = ctx;
}

// Each operation takes an optional `cv`: the value of its result, already
// known (a node value cached from the value pass of the same iterate).  The
// value is then adopted instead of recomputed and only the tangent is
// evaluated; tangents only ever use the operands' values, never the result's.
Term t_add(const Term& a, const Term& b, const Term* cv) {
  check_dom(a, b);
  bool do_der = a.has_der() && b.has_der();
  if (a.is_double && b.is_double) {
    Term r = Term::dbl(a.dom, a.vd + b.vd);
    if (do_der) dbl_tangent_lincomb(r, 1.0, a, 1.0, &b);
    return r;
  }
  if (a.is_double || b.is_double) {
    const Term& t = a.is_double ? b : a;
    const Term& d = a.is_double ? a : b;
    Term r = tensor_like(t);
    if (cv) r.vt = cv->vt;
    else
      for (auto& v : t.vt) r.vt.push_back(v + d.vd);
    if (do_der) {
      no_seed_tangent(d);
      r.has_dt = true;
      for (int i = 0; i < ncomp(t); i++) r.dt.push_back(d.dd == 0.0 ? t.dt[i] : t.dt[i] + d.dd);
    }
    return r;
  }
  check_valence(a, b);
  const Term bb = align_to(b, a);
  Term r = tensor_like(a);
  if (cv) r.vt = cv->vt;
  else
    for (int i = 0; i < ncomp(a); i++) r.vt.push_back(a.vt[i] + bb.vt[i]);
  if (do_der) {
    r.has_dt = true;
    for (int i = 0; i < ncomp(a); i++) r.dt.push_back(a.dt[i] + bb.dt[i]);
  }
  return r;
}

Term t_sub(const Term& a, const Term& b, const Term* cv) {
  check_dom(a, b);
  bool do_der = a.has_der() && b.has_der();
  if (a.is_double && b.is_double) {
    Term r = Term::dbl(a.dom, a.vd - b.vd);
    if (do_der) dbl_tangent_lincomb(r, 1.0, a, -1.0, &b);
    return r;
  }
  if (b.is_double) {
    Term r = tensor_like(a);
    if (cv) r.vt = cv->vt;
    else
      for (auto& v : a.vt) r.vt.push_back(v - b.vd);
    if (do_der) {
      no_seed_tangent(b);
      r.has_dt = true;
      for (int i = 0; i < ncomp(a); i++) r.dt.push_back(b.dd == 0.0 ? a.dt[i] : a.dt[i] - b.dd);
    }
    return r;
  }
  if (a.is_double) {
    Term r = tensor_like(b);
    if (cv) r.vt = cv->vt;
    else
      for (auto& v : b.vt) r.vt.push_back(a.vd - v);
    if (do_der) {
      no_seed_tangent(a);
      r.has_dt = true;
      for (int i = 0; i < ncomp(b); i++) r.dt.push_back(a.dd == 0.0 ? -b.dt[i] : a.dd - b.dt[i]);
    }
    return r;
  }
  check_valence(a, b);
  const Term bb = align_to(b, a);
  Term r = tensor_like(a);
  if (cv) r.vt = cv->vt;
  else
    for (int i = 0; i < ncomp(a); i++) r.vt.push_back(a.vt[i] - bb.vt[i]);
  if (do_der) {
    r.has_dt = true;
    for (int i = 0; i < ncomp(a); i++) r.dt.push_back(a.dt[i] - bb.dt[i]);
  }
  return r;
}

Term t_neg(const Term& a, const Term* cv) {
  // Term_eq operator-(aa) = -1. * aa
  if (a.is_double) {
    Term r = Term::dbl(a.dom, -a.vd);
    if (a.has_dd) dbl_tangent_lincomb(r, -1.0, a, 0.0, nullptr);
    return r;
  }
  Term r = tensor_like(a);
  if (cv) r.vt = cv->vt;
  else
    for (auto& v : a.vt) r.vt.push_back(v * -1.0);
  if (a.has_dt) {
    r.has_dt = true;
    for (auto& v : a.dt) r.dt.push_back(v * -1.0);
  }
  return r;
}

Term t_mul(const Term& a, const Term& b, const Term* cv) {
  check_dom(a, b);
  bool do_der = a.has_der() && b.has_der();
  if (a.is_double && b.is_double) {
    Term r = Term::dbl(a.dom, a.vd * b.vd);
    if (do_der) dbl_tangent_lincomb(r, b.vd, a, a.vd, &b);
    return r;
  }
  if (a.is_double || b.is_double) {
    const Term& t = a.is_double ? b : a;
    const Term& d = a.is_double ? a : b;
    Term r = tensor_like(t);
    if (cv) r.vt = cv->vt;
    else
      for (auto& v : t.vt) r.vt.push_back(v * d.vd);
    if (do_der) {
      no_seed_tangent(d);
      r.has_dt = true;
      for (int i = 0; i < ncomp(t); i++) {
        DVal part = t.dt[i] * d.vd;
        if (!dd_zero(d)) part = part + t.vt[i] * d.dd;
        r.dt.push_back(part);
      }
    }
    return r;
  }
  if (a.vt.size() != 1 && b.vt.size() != 1) return tensor_product(a, b, cv, do_der);
  const Term& s = (a.vt.size() == 1) ? a : b;
  const Term& t = (a.vt.size() == 1) ? b : a;
  bool s_first = (&s == &a);
  Term r = tensor_like(t);
  if (cv) r.vt = cv->vt;
  else
    for (int i = 0; i < ncomp(t); i++) r.vt.push_back(s_first ? s.vt[0] * t.vt[i] : t.vt[i] * s.vt[0]);
  if (do_der) {
    r.has_dt = true;
    for (int i = 0; i < ncomp(t); i++) {
      // der = a' b + a b'
      const DVal& av = s_first ? s.vt[0] : t.vt[i];
      const DVal& bv = s_first ? t.vt[i] : s.vt[0];
      const DVal& ad = s_first ? s.dt[0] : t.dt[i];
      const DVal& bd = s_first ? t.dt[i] : s.dt[0];
      r.dt.push_back(ad * bv + av * bd);
    }
  }
  return r;
}

Term t_div(const Term& a, const Term& b, const Term* cv) {
  check_dom(a, b);
  bool do_der = a.has_der() && b.has_der();
  if (a.is_double && b.is_double) {
    Term r = Term::dbl(a.dom, a.vd / b.vd);
    if (do_der) {
      if (a.ddv || b.ddv) {
        dbl_tangent_lincomb(r, 1.0 / b.vd, a, -a.vd / (b.vd * b.vd), &b);
      } else {
        r.has_dd = true;
        r.dd = (a.dd * b.vd - a.vd * b.dd) / (b.vd * b.vd);
      }
    }
    return r;
  }
  if (b.is_double) {
    Term r = tensor_like(a);
    if (cv) r.vt = cv->vt;
    else
      for (auto& v : a.vt) r.vt.push_back(v / b.vd);
    if (do_der) {
      no_seed_tangent(b);
      r.has_dt = true;
      for (int i = 0; i < ncomp(a); i++) {
        DVal num = a.dt[i] * b.vd;
        if (!dd_zero(b)) num = num - a.vt[i] * b.dd;
        r.dt.push_back(num / (b.vd * b.vd));
      }
    }
    return r;
  }
  if (b.vt.size() != 1) throw KdError(KD_ERR_UNSUPPORTED, "division by a non-scalar tensor");
  if (a.is_double) {
    Term r = tensor_like(b);
    if (cv) r.vt = cv->vt;
    else
      r.vt.push_back(a.vd / b.vt[0]);
    if (do_der) {
      no_seed_tangent(a);
      r.has_dt = true;
      DVal num = (dd_zero(a) ? DVal::zeros(b.vt[0].ctx, b.vt[0].dom, 1) : b.vt[0] * a.dd) - b.dt[0] * a.vd;
      r.dt.push_back(num / (b.vt[0] * b.vt[0]));
    }
    return r;
  }
  Term r = tensor_like(a);
  if (cv) r.vt = cv->vt;
  else
    for (int i = 0; i < ncomp(a); i++) r.vt.push_back(a.vt[i] / b.vt[0]);
  if (do_der) {
    r.has_dt = true;
    DVal bb = b.vt[0] * b.vt[0];
    for (int i = 0; i < ncomp(a); i++) r.dt.push_back((a.dt[i] * b.vt[0] - a.vt[i] * b.dt[0]) / bb);
  }
  return r;
}

Term operator+(const Term& a, const Term& b) { return t_add(a, b, nullptr); }
Term operator-(const Term& a, const Term& b) { return t_sub(a, b, nullptr); }
Term operator*(const Term& a, const Term& b) { return t_mul(a, b, nullptr); }
Term operator/(const Term& a, const Term& b) { return t_div(a, b, nullptr); }
Term operator-(const Term& a) { return t_neg(a, nullptr); }

Term term_pow(const Term& a, int n, const Term* cv) {
  // pow(Term_eq, int), term_eq_math.cpp:547.  Intermediate powers keep
  // their values (the next product's tangent needs them); only the last
  // product may adopt a cached value.
  if (n > 0) {
    Term r = a;
    for (int i = 1; i < n; i++) r = t_mul(r, a, (i == n - 1) ? cv : nullptr);
    return r;
  }
  if (a.is_double) {
    Term one = Term::dbl_der(a.dom, 1.0, 0.0);
    Term r = one;
    for (int i = 0; i < -n; i++) r = t_div(r, a, (i == -n - 1) ? cv : nullptr);
    return r;
  }
  Term one = tensor_like(a);
  DVal o = DVal::constant(a.vt[0].ctx, a.vt[0].dom, 1.0);
  o.base = a.vt[0].dom->std_base();
  one.vt.push_back(o);
  one.has_dt = true;
  one.dt.push_back(DVal::zeros(a.vt[0].ctx, a.vt[0].dom, 1));
  Term r = one;
  for (int i = 0; i < -n; i++) r = t_div(r, a, (i == -n - 1) ? cv : nullptr);
  return r;
}

// --------------------------------------------------------------- Ope tree --
namespace {

Term comp_by_comp(const Term& t, const std::function<DVal(const DVal&)>& f, const Term* cv) {
  if (t.is_double) throw KdError(KD_ERR_UNSUPPORTED, "operator only defined for tensor terms");
  Term r = tensor_like(t);
  if (cv) r.vt = cv->vt;
  else
    for (auto& v : t.vt) r.vt.push_back(v.zero ? v : f(v));
  if (t.has_dt) {
    r.has_dt = true;
    for (auto& v : t.dt) r.dt.push_back(v.zero ? v : f(v));
  }
  return r;
}

class OpeBin : public Ope {
 public:
  OpeBin(int dom, char op, OpePtr a_, OpePtr b_) : Ope(dom), op(op), a(std::move(a_)), b(std::move(b_)) {
    vc = a->vc && b->vc;
    dz = a->dz && b->dz;
    if (op == '+' || op == '-') dc = a->dc && b->dc;
    else if (op == '*') dc = (a->dz || (a->dc && b->vc)) && (b->dz || (b->dc && a->vc));  // a'b + ab'
    else dc = (a->dz || a->dc) && b->dz && b->vc;  // (a'b - ab')/b^2 with b constant
  }
  std::vector<const Ope*> kids() const override { return {a.get(), b.get()}; }
  Term action(EvalState& st, const Term* cv) const override {
    Term x = a->eval(st);
    Term y = b->eval(st);
    switch (op) {
      case '+': return t_add(x, y, cv);
      case '-': return t_sub(x, y, cv);
      case '*': return t_mul(x, y, cv);
      default: return t_div(x, y, cv);
    }
  }
  char op;
  OpePtr a, b;
};

class OpeMinus : public Ope {
 public:
  OpeMinus(int dom, OpePtr a_) : Ope(dom), a(std::move(a_)) {
    vc = a->vc;
    dc = a->dc;
    dz = a->dz;
  }
  std::vector<const Ope*> kids() const override { return {a.get()}; }
  Term action(EvalState& st, const Term* cv) const override { return t_neg(a->eval(st), cv); }
  OpePtr a;
};

class OpePow : public Ope {
 public:
  OpePow(int dom, int n, OpePtr a_) : Ope(dom), n(n), a(std::move(a_)) {
    vc = a->vc;
    dz = a->dz;
    dc = a->dz || (a->vc && a->dc);
  }
  std::vector<const Ope*> kids() const override { return {a.get()}; }
  Term action(EvalState& st, const Term* cv) const override { return term_pow(a->eval(st), n, cv); }
  int n;
  OpePtr a;
};

// Linear functionals turning a scalar field into a number, with their
// tangents (one number per seed): Ope_int_volume (ope_int_volume.cpp),
// Ope_int (ope_int.cpp, Domain_compact::integ), Ope_val (ope_val.cpp, the
// value at one collocation point) and Ope_point (ope_point.cpp, the value at
// a point through the spectral summation).
class OpeFunctional : public Ope {
 public:
  enum Kind { INTEG_VOLUME, INTEG, VAL, POINT };
  OpeFunctional(int dom, Kind k, OpePtr a_, int bound, const int pos[3], const double num[3])
      : Ope(dom), kind(k), a(std::move(a_)), bound(bound) {
    for (int i = 0; i < 3; i++) {
      p[i] = pos ? pos[i] : 0;
      x[i] = num ? num[i] : 0.0;
    }
    vc = a->vc;
    dc = a->dc;
    dz = a->dz;
  }
  std::vector<const Ope*> kids() const override { return {a.get()}; }
  Term action(EvalState& st, const Term* cv) const override {
    Term t = a->eval(st);
    if (t.is_double || t.vt.size() != 1)
      throw KdError(KD_ERR_UNSUPPORTED, "integrals and point values are only defined for a scalar field");
    Term r = Term::dbl(dom, 0.0);
    if (cv) {
      r.vd = cv->vd;
    } else if (!t.vt[0].zero) {
      Context* ctx = t.vt[0].ctx;
      double* out = apply(t.vt[0]);
      cuda_check(cudaMemcpyAsync(&r.vd, out, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream()), "D2H integral");
      cuda_check(cudaStreamSynchronize(ctx->stream()), "sync integral");
    }
    if (t.has_dt) {
      r.has_dd = true;
      const DVal& d = t.dt[0];
      if (!d.zero) {
        r.ddv = apply(d);
        r.ddb = d.batch;
        r.ddctx = d.ctx;
      }
    }
    return r;
  }
  // The functional of every batch member of v, into `batch` doubles of the
  // pass's arena.
  double* apply(const DVal& v) const {
    Context* ctx = v.ctx;
    const Domain& d = *v.dom;
    SparseRow row;
    const double* src = nullptr;
    long long stride = 0;
    DVal w;
    switch (kind) {
      case INTEG_VOLUME: {
        // nucleus, shell: mult_r(mult_r(mult_sin_theta(so))) * alpha;
        // compact: -mult_r^4(mult_sin_theta(so)) * alpha
        w = mult_r(mult_r(mult_sin_theta(v)));
        if (d.type == DOM_COMPACT) w = mult_r(mult_r(w)) * (-d.alpha);
        else w = w * d.alpha;
        w.coef();
        d.integ_volume_row(w.base, row);
        src = w.cf;
        stride = d.ncoefs();
        break;
      }
      case INTEG: {
        w = mult_r(mult_r(mult_sin_theta(v)));
        w.coef();
        d.integ_surface_row(w.base, bound, row);
        src = w.cf;
        stride = d.ncoefs();
        break;
      }
      case VAL: {
        w = v;
        w.coef_i();
        row.add(d.pidx(p[0], p[1], p[2]), 1.0);
        src = w.c;
        stride = d.npts();
        break;
      }
      default: {
        w = v;
        w.coef();
        std::vector<double> pw;
        d.point_weights(w.base, x, pw);
        for (size_t c = 0; c < pw.size(); c++)
          if (pw[c] != 0.0) row.add(static_cast<int>(c), pw[c]);
        src = w.cf;
        stride = d.ncoefs();
      }
    }
    std::vector<int> rp = {0, static_cast<int>(row.e.size())}, idx;
    std::vector<double> wt;
    for (auto& e : row.e) {
      idx.push_back(e.first);
      wt.push_back(e.second);
    }
    double* out = ctx->scratch().alloc_doubles(v.batch);
    if (row.e.empty()) {
      cuda_check(cudaMemsetAsync(out, 0, sizeof(double) * v.batch, ctx->stream()), "memset functional");
      return out;
    }
    cuda_check(launch_gather_csr(src, stride, v.batch, 1, ctx->table(rp), ctx->table(idx), ctx->dtable(wt), out, 1, 0,
                                 1.0, 0, ctx->stream()),
               "functional gather");
    ctx->launches++;
    return out;
  }
  Kind kind;
  OpePtr a;
  int bound;
  int p[3];
  double x[3];
};

// Unary operators acting component by component on value and tangent.
class OpeUnary : public Ope {
 public:
  enum Kind { LAP, DN, DR, MULTR, DIVR, DIVSINT, MULTSINT, DIVCOST, DDR, LAP2 };
  OpeUnary(int dom, Kind k, int bound, OpePtr a_) : Ope(dom), kind(k), bound(bound), a(std::move(a_)) {
    vc = a->vc;  // linear operators: the tangent is the operator of the tangent
    dc = a->dc;
    dz = a->dz;
  }
  std::vector<const Ope*> kids() const override { return {a.get()}; }
  Term action(EvalState& st, const Term* cv) const override {
    Term t = a->eval(st);
    switch (kind) {
      case LAP: return comp_by_comp(t, [](const DVal& v) { return laplacian(v); }, cv);
      case DN: {
        int b = bound;
        return comp_by_comp(t, [b](const DVal& v) { return der_normal(v, b); }, cv);
      }
      case DR: return comp_by_comp(t, [](const DVal& v) { return der_r(v); }, cv);
      // Domain::ddr (src/Domain/domain.cpp:1522): der_r twice (Ope_ddr keeps zero as zero)
      case DDR: return comp_by_comp(t, [](const DVal& v) { return v.zero ? v : der_r(der_r(v)); }, cv);
      case LAP2: return comp_by_comp(t, [](const DVal& v) { return v.zero ? v : laplacian2(v); }, cv);
      case MULTR: return comp_by_comp(t, [](const DVal& v) { return mult_r(v); }, cv);
      case DIVR: return comp_by_comp(t, [](const DVal& v) { return div_r(v); }, cv);
      case DIVSINT: return comp_by_comp(t, [](const DVal& v) { return div_sin_theta(v); }, cv);
      case MULTSINT: return comp_by_comp(t, [](const DVal& v) { return mult_sin_theta(v); }, cv);
      default: return comp_by_comp(t, [](const DVal& v) { return div_cos_theta(v); }, cv);
    }
  }
  Kind kind;
  int bound;
  OpePtr a;
};

// exp / sqrt / log / cos / sin / cosh / sinh / atanh of a scalar
// (src/Ope_eq/ope_exp.cpp, ope_sqrt.cpp, ope_log.cpp, ope_cos.cpp,
// ope_sin.cpp, ope_cosh.cpp, ope_sinh.cpp, ope_atanh.cpp), with their
// tangents in the reference's operand order: -u' sin(u), u' cos(u),
// u' sinh(u), u' cosh(u), u' / (1 - u u).
class OpeFunc : public Ope {
 public:
  enum Kind { EXP, SQRT, LOG, COS, SIN, COSH, SINH, ATANH };
  OpeFunc(int dom, Kind k, OpePtr a_) : Ope(dom), kind(k), a(std::move(a_)) {
    vc = a->vc;
    dz = a->dz;
    dc = a->dz || (a->vc && a->dc);
  }
  std::vector<const Ope*> kids() const override { return {a.get()}; }
  Term action(EvalState& st, const Term* cv) const override {
    Term t = a->eval(st);
    if (t.is_double) {
      const double u = t.vd;
      double v = 0.0;
      switch (kind) {
        case EXP: v = std::exp(u); break;
        case SQRT: v = std::sqrt(u); break;
        case LOG: v = std::log(u); break;
        case COS: v = std::cos(u); break;
        case SIN: v = std::sin(u); break;
        case COSH: v = std::cosh(u); break;
        case SINH: v = std::sinh(u); break;
        case ATANH: v = std::atanh(u); break;
      }
      Term r = Term::dbl(t.dom, v);
      if (t.has_dd && t.ddv) {
        double f1 = 0.0;
        switch (kind) {
          case EXP: f1 = std::exp(u); break;
          case SQRT: f1 = 0.5 / std::sqrt(u); break;
          case LOG: f1 = 1.0 / u; break;
          case COS: f1 = -std::sin(u); break;
          case SIN: f1 = std::cos(u); break;
          case COSH: f1 = std::sinh(u); break;
          case SINH: f1 = std::cosh(u); break;
          case ATANH: f1 = 1.0 / (1 - u * u); break;
        }
        dbl_tangent_lincomb(r, f1, t, 0.0, nullptr);
      } else if (t.has_dd) {
        r.has_dd = true;
        const double d = t.dd;
        switch (kind) {
          case EXP: r.dd = d * std::exp(u); break;
          case SQRT: r.dd = d / 2. / std::sqrt(u); break;
          case LOG: r.dd = d / u; break;
          case COS: r.dd = -d * std::sin(u); break;
          case SIN: r.dd = d * std::cos(u); break;
          case COSH: r.dd = d * std::sinh(u); break;
          case SINH: r.dd = d * std::cosh(u); break;
          case ATANH: r.dd = d / (1 - u * u); break;
        }
      }
      return r;
    }
    if (t.vt.size() != 1) throw KdError(KD_ERR_UNSUPPORTED, "exp/sqrt/log/cos/sin/cosh/sinh/atanh only defined for a scalar");
    Term r = tensor_like(t);
    const DVal& v = t.vt[0];
    if (cv) {
      r.vt = cv->vt;
    } else {
      switch (kind) {
        case EXP: r.vt.push_back(vd_exp(v)); break;
        case SQRT: r.vt.push_back(v.zero ? v : vd_sqrt(v)); break;
        case LOG: r.vt.push_back(vd_log(v)); break;
        case COS: r.vt.push_back(vd_cos(v)); break;
        case SIN: r.vt.push_back(vd_sin(v)); break;
        case COSH: r.vt.push_back(vd_cosh(v)); break;
        case SINH: r.vt.push_back(vd_sinh(v)); break;
        case ATANH: r.vt.push_back(vd_atanh(v)); break;
      }
    }
    if (t.has_dt) {
      // der exp(u) = u' exp(u), der sqrt(u) = u' / 2 / sqrt(u): the result's
      // value is exp(u) / sqrt(u) itself
      r.has_dt = true;
      const DVal& d = t.dt[0];
      switch (kind) {
        case EXP: r.dt.push_back(d * r.vt[0]); break;
        case SQRT: r.dt.push_back(d.zero ? d : d / 2. / r.vt[0]); break;
        case LOG: r.dt.push_back(d / v); break;
        case COS: r.dt.push_back(d.zero ? d : -d * vd_sin(v)); break;
        case SIN: r.dt.push_back(d.zero ? d : d * vd_cos(v)); break;
        case COSH: r.dt.push_back(d.zero ? d : d * vd_sinh(v)); break;
        case SINH: r.dt.push_back(d.zero ? d : d * vd_cosh(v)); break;
        case ATANH: r.dt.push_back(d.zero ? d : d / (1.0 - v * v)); break;
      }
    }
    return r;
  }
  Kind kind;
  OpePtr a;
};

// grad(scalar): Cartesian components der_abs(1..3) (Domain::grad_term_eq)
class OpeGrad : public Ope {
 public:
  OpeGrad(int dom, OpePtr a_) : Ope(dom), a(std::move(a_)) {
    vc = a->vc;
    dc = a->dc;
    dz = a->dz;
  }
  std::vector<const Ope*> kids() const override { return {a.get()}; }
  Term action(EvalState& st, const Term* cv) const override {
    Term t = a->eval(st);
    if (t.is_double || t.vt.size() != 1) throw KdError(KD_ERR_UNSUPPORTED, "grad only defined for scalars");
    Term r;
    r.dom = t.dom;
    r.valence = 1;
    if (cv) r.vt = cv->vt;
    else
      for (int i = 1; i <= 3; i++) r.vt.push_back(t.vt[0].der_abs(i));
    if (t.has_dt) {
      r.has_dt = true;
      for (int i = 1; i <= 3; i++) r.dt.push_back(t.dt[0].der_abs(i));
    }
    return r;
  }
  OpePtr a;
};

// scal(a, b): flat scalar product of two Cartesian vectors (Ope_scal)
class OpeScal : public Ope {
 public:
  OpeScal(int dom, OpePtr a_, OpePtr b_) : Ope(dom), a(std::move(a_)), b(std::move(b_)) {
    vc = a->vc && b->vc;
    dz = a->dz && b->dz;
    dc = (a->dz || (a->dc && b->vc)) && (b->dz || (b->dc && a->vc));
  }
  std::vector<const Ope*> kids() const override { return {a.get(), b.get()}; }
  Term action(EvalState& st, const Term* cv) const override {
    Term x = a->eval(st);
    Term y = b->eval(st);
    if (x.vt.size() != 3 || y.vt.size() != 3) throw KdError(KD_ERR_UNSUPPORTED, "scal needs two vectors");
    Term r;
    r.dom = x.dom;
    r.valence = 0;
    if (cv) {
      r.vt = cv->vt;
    } else {
      DVal v = x.vt[0] * y.vt[0];
      for (int i = 1; i < 3; i++) v = v + x.vt[i] * y.vt[i];
      r.vt.push_back(v);
    }
    if (x.has_dt && y.has_dt) {
      r.has_dt = true;
      DVal d = x.dt[0] * y.vt[0] + x.vt[0] * y.dt[0];
      for (int i = 1; i < 3; i++) d = d + (x.dt[i] * y.vt[i] + x.vt[i] * y.dt[i]);
      r.dt.push_back(d);
    }
    return r;
  }
  OpePtr a, b;
};

// partial_i (Cartesian derivative of each component), i = x, y, z
class OpePartial : public Ope {
 public:
  OpePartial(int dom, int i, OpePtr a_) : Ope(dom), i(i), a(std::move(a_)) {
    vc = a->vc;
    dc = a->dc;
    dz = a->dz;
  }
  std::vector<const Ope*> kids() const override { return {a.get()}; }
  Term action(EvalState& st, const Term* cv) const override {
    int ii = i;
    return comp_by_comp(a->eval(st), [ii](const DVal& v) { return v.der_abs(ii); }, cv);
  }
  int i;
  OpePtr a;
};

// D_i / D^i of the flat metric (Metric_flat::derive_partial_cart,
// src/Metric/metric_flat.cpp:150) and partial_i (Ope_partial): the Cartesian
// derivative of every component, the derivative index first.  When the
// derivative index repeats one of the operand's, that pair is summed over
// (the divergence), term by term in the order 1, 2, 3 of the index; only
// the summed components are differentiated.  Upper and lower indices share
// their components in a flat Cartesian frame.
class OpeDer : public Ope {
 public:
  OpeDer(int dom, char ind, OpePtr a_) : Ope(dom), ind(ind), a(std::move(a_)) {
    vc = a->vc;
    dc = a->dc;
    dz = a->dz;
  }
  std::vector<const Ope*> kids() const override { return {a.get()}; }
  Term action(EvalState& st, const Term* cv) const override {
    Term t = a->eval(st);
    if (t.is_double) throw KdError(KD_ERR_UNSUPPORTED, "derivative of a number");
    // names only when the operand has them (or is a scalar), as donames
    const bool names = !t.idx.empty() || t.valence == 0;
    const size_t p = names ? t.idx.find(ind) : std::string::npos;
    const int n = ncomp(t);
    Term r;
    r.dom = t.dom;
    r.has_dt = t.has_dt;
    if (p == std::string::npos) {
      r.valence = t.valence + 1;
      if (names) r.idx = std::string(1, ind) + t.idx;
      for (int k = 1; k <= 3; k++)
        for (int c = 0; c < n; c++) {
          if (!cv) r.vt.push_back(t.vt[c].der_abs(k));
          if (t.has_dt) r.dt.push_back(t.dt[c].der_abs(k));
        }
    } else {
      const int pp = static_cast<int>(p), nt = t.valence;
      r.valence = nt - 1;
      r.idx = t.idx;
      r.idx.erase(p, 1);
      int mr[8], mt[8];
      for (int f = 0; f < pow3(nt - 1); f++) {
        unflatten(f, nt - 1, mr);
        for (int i = 0, k = 0; i < nt; i++)
          if (i != pp) mt[i] = mr[k++];
        DVal v, d;
        for (int c = 0; c < 3; c++) {
          mt[pp] = c;
          const int g = flat_index(mt, nt);
          if (!cv) v = (c == 0) ? t.vt[g].der_abs(c + 1) : v + t.vt[g].der_abs(c + 1);
          if (t.has_dt) d = (c == 0) ? t.dt[g].der_abs(c + 1) : d + t.dt[g].der_abs(c + 1);
        }
        if (!cv) r.vt.push_back(v);
        if (t.has_dt) r.dt.push_back(d);
      }
    }
    if (cv) r.vt = cv->vt;
    return r;
  }
  char ind;
  OpePtr a;
};

// User-defined EOS operator: Ope_user with EOS<eos, var>::action
// (include/EOS/EOS.hh:235-270).  The tangent depends on the value.
class OpeEos : public Ope {
 public:
  OpeEos(int dom, const KdEos& e, int var, OpePtr a_) : Ope(dom), eos(e), var(var), a(std::move(a_)) {
    vc = a->vc;
    dz = a->dz;
    dc = a->dz;
  }
  std::vector<const Ope*> kids() const override { return {a.get()}; }
  Term action(EvalState& st, const Term* cv) const override {
    Term t = a->eval(st);
    if (t.is_double || t.vt.size() != 1) throw KdError(KD_ERR_UNSUPPORTED, "EOS only defined with respect for a scalar");
    Term r = tensor_like(t);
    const DVal& h = t.vt[0];
    if (cv) r.vt = cv->vt;
    else r.vt.push_back(eos_value(h, eos, var));
    if (t.has_dt) {
      r.has_dt = true;
      r.dt.push_back(h.zero ? DVal::zeros(h.ctx, h.dom, t.dt[0].batch) : eos_variation(t.dt[0], h, eos, var));
    }
    return r;
  }
  KdEos eos;
  int var;
  OpePtr a;
};

class OpeLeaf : public Ope {
 public:
  enum Kind { VAR, VAR_DOUBLE, CST, HARD, DEF, VAR_VECTOR, CST_VECTOR, METRIC };
  OpeLeaf(int dom, Kind k, int which, double v = 0.0, std::string idx = std::string())
      : Ope(dom), kind(k), which(which), val(v), idx(std::move(idx)) {
    // unknowns: tangent = the seed (or 0); constants: zero tangent; numbers
    // and the metric: constant value; definitions: not classified
    vc = (k == HARD || k == METRIC);
    dc = (k != DEF);
    dz = (k == CST || k == HARD || k == CST_VECTOR || k == METRIC);
  }
  Term action(EvalState& st, const Term* cv) const override;
  bool cacheable() const override { return false; }
  Kind kind;
  int which;
  double val;
  // index names written after the symbol ("bet^i", "A_ij"): given to the
  // tensor in order, then repeated names summed (Ope_id with name_ind)
  std::string idx;
};

Term name_indices(Term t, const std::string& idx) {
  if (idx.empty()) return t;
  if (t.is_double || t.valence != static_cast<int>(idx.size()))
    throw KdError(KD_ERR_ARG, "wrong number of indices: " + idx);
  t.idx = idx;
  return contract_self(t);
}

Term OpeLeaf::action(EvalState& st, const Term*) const {
  switch (kind) {
    case VAR: return st.var_term(which, dom);
    case VAR_DOUBLE: return st.var_double_term(which, dom);
    case CST: return st.cst_term(which, dom);
    case DEF: return name_indices(st.def_term(which, dom), idx);
    case VAR_VECTOR: return name_indices(st.var_vector_term(which, dom), idx);
    case CST_VECTOR: return name_indices(st.cst_vector_term(which, dom), idx);
    case METRIC: return name_indices(st.metric_term(dom), idx);
    default: {
      Term t = Term::dbl(dom, val);
      if (st.with_der) {
        t.has_dd = true;
        t.dd = 0.0;
      }
      return t;
    }
  }
}

void mark_tangent_frontier_rec(const Ope* n, bool parent_dc) {
  n->cache_der = n->dc && !n->dz && !parent_dc && n->cacheable();
  for (const Ope* k : n->kids()) mark_tangent_frontier_rec(k, n->dc);
}

}  // namespace

void mark_tangent_frontier(const Ope* root) { mark_tangent_frontier_rec(root, false); }

namespace {

// ----------------------------------------------------------------- parser --
int count_char(const std::string& s, char c) {
  int n = 0;
  for (char x : s)
    if (x == c) n++;
  return n;
}

bool balanced(const std::string& s) { return count_char(s, '(') == count_char(s, ')'); }

// get_parts (src/Utilities/name_tools.cpp:150): split at the place-th
// occurrence of sep counted from the END of the string.
bool get_parts(const std::string& in, std::string& first, std::string& second, char sep, int place) {
  int nfound = -1;
  int pos = static_cast<int>(in.size()) - 1;
  bool fin = false;
  while (!fin) {
    if (pos < 0) break;
    if (in[pos] == sep) nfound++;
    pos--;
    if (nfound == place) fin = true;
    if (pos == -1) fin = true;
  }
  if (pos == -1 && nfound != place) {
    first.clear();
    second = "0";
    return false;
  }
  if (pos == -1 && nfound == place && in[0] == sep) {
    first.clear();
    second = "0";
    return false;
  }
  pos++;
  first = trim_expr(in.substr(0, pos));
  second = trim_expr(in.substr(pos + 1));
  if (first == " ") first.clear();
  if (second == " ") second.clear();
  return true;
}

// is_ope_bin (give_ope.cpp:276)
bool is_ope_bin(const std::string& name, std::string& p1, std::string& p2, char cible) {
  int n = count_char(name, cible);
  for (int conte = 0; conte < n; conte++) {
    if (!get_parts(name, p1, p2, cible, conte)) continue;
    if (!p1.empty() && !p2.empty() && balanced(p1) && balanced(p2)) return true;
  }
  return false;
}

// is_ope_uni (give_ope.cpp:314): "name(" ... ") "
bool is_ope_uni(const std::string& name, std::string& inner, const std::string& ope) {
  std::string head = ope + "(";
  if (name.compare(0, head.size(), head) != 0) return false;
  if (name.size() < head.size() + 2) return false;
  if (name[name.size() - 2] != ')') return false;
  inner = trim_expr(name.substr(head.size(), name.size() - head.size() - 2));
  return balanced(inner);
}

bool is_ope_uni2(const std::string& name, std::string& p1, std::string& p2, const std::string& ope) {
  std::string inner;
  if (!is_ope_uni(name, inner, ope)) return false;
  // split at the only top-level comma
  int depth = 0, at = -1, ncomma = 0;
  for (size_t i = 0; i < inner.size(); i++) {
    if (inner[i] == '(') depth++;
    if (inner[i] == ')') depth--;
    if (inner[i] == ',' && depth == 0) {
      at = static_cast<int>(i);
      ncomma++;
    }
  }
  if (ncomma != 1) return false;
  p1 = trim_expr(inner.substr(0, at));
  p2 = trim_expr(inner.substr(at + 1));
  return true;
}

bool is_double_str(const std::string& name, double& v) {
  std::string s = name;
  while (!s.empty() && s.back() == ' ') s.pop_back();
  if (s.empty()) return false;
  char* end = nullptr;
  v = std::strtod(s.c_str(), &end);
  return end && *end == '\0';
}

}  // namespace

std::string trim_expr(const std::string& s) {
  // trim_spaces (src/Utilities/name_tools.cpp:26): collapse runs of spaces,
  // drop leading spaces, keep one trailing space, strip redundant outer ().
  std::string a;
  bool inspace = !s.empty() && s[0] == ' ';
  for (char c : s) {
    bool sp = (c == ' ');
    if (!sp || !inspace) a.push_back(c);
    inspace = sp;
  }
  if (a.empty() || a.back() != ' ') a.push_back(' ');
  int first = 0, last = static_cast<int>(a.size()) - 2;
  while (true) {
    if (last <= first) break;
    bool need = (a[first] == '(') && (a[last] == ')');
    if (need) {
      int nin = 0;
      for (int i = first; i < last; i++) {
        if (a[i] == '(') nin++;
        if (a[i] == ')') nin--;
        if (a[i] == ')' && nin == 0) need = false;
      }
    }
    if (!need) break;
    first++;
    last--;
  }
  std::string out = a.substr(first, static_cast<size_t>(last - first + 1));
  // trailing single space convention
  while (!out.empty() && out.back() == ' ') out.pop_back();
  while (!out.empty() && out.front() == ' ') out.erase(out.begin());
  return out + " ";
}

OpePtr parse_ope(const System& sys, int dd, const std::string& expr, int bound) {
  std::string name = trim_expr(expr);
  std::string p1, p2;
  if (is_ope_bin(name, p1, p2, '+'))
    return std::make_shared<OpeBin>(dd, '+', parse_ope(sys, dd, p1, bound), parse_ope(sys, dd, p2, bound));
  if (is_ope_bin(name, p1, p2, '-'))
    return std::make_shared<OpeBin>(dd, '-', parse_ope(sys, dd, p1, bound), parse_ope(sys, dd, p2, bound));
  if (name[0] == '-') return std::make_shared<OpeMinus>(dd, parse_ope(sys, dd, name.substr(1), bound));
  if (is_ope_bin(name, p1, p2, '*'))
    return std::make_shared<OpeBin>(dd, '*', parse_ope(sys, dd, p1, bound), parse_ope(sys, dd, p2, bound));
  if (is_ope_bin(name, p1, p2, '/'))
    return std::make_shared<OpeBin>(dd, '/', parse_ope(sys, dd, p1, bound), parse_ope(sys, dd, p2, bound));
  struct U {
    const char* n;
    OpeUnary::Kind k;
  };
  static const U unis[] = {{"Lap", OpeUnary::LAP},       {"lap", OpeUnary::LAP},        {"dn", OpeUnary::DN},
                           {"multr", OpeUnary::MULTR},   {"dr", OpeUnary::DR},          {"divr", OpeUnary::DIVR},
                           {"divsint", OpeUnary::DIVSINT}, {"multsint", OpeUnary::MULTSINT},
                           {"divcost", OpeUnary::DIVCOST}, {"ddr", OpeUnary::DDR},
                           {"Lap2", OpeUnary::LAP2},     {"lap2", OpeUnary::LAP2}};
  for (const auto& u : unis)
    if (is_ope_uni(name, p1, u.n)) {
      if (u.k == OpeUnary::DN && bound < 0) throw KdError(KD_ERR_ARG, "dn() needs a boundary");
      return std::make_shared<OpeUnary>(dd, u.k, bound, parse_ope(sys, dd, p1, bound));
    }
  // multrsint / divrsint (Ope_mult_rsint, Ope_div_rsint): mult_r then
  // mult_sin_theta, div_r then div_sin_theta, component by component
  if (is_ope_uni(name, p1, "multrsint"))
    return std::make_shared<OpeUnary>(dd, OpeUnary::MULTSINT, bound,
                                      std::make_shared<OpeUnary>(dd, OpeUnary::MULTR, bound, parse_ope(sys, dd, p1, bound)));
  if (is_ope_uni(name, p1, "divrsint"))
    return std::make_shared<OpeUnary>(dd, OpeUnary::DIVSINT, bound,
                                      std::make_shared<OpeUnary>(dd, OpeUnary::DIVR, bound, parse_ope(sys, dd, p1, bound)));
  if (is_ope_uni(name, p1, "grad")) return std::make_shared<OpeGrad>(dd, parse_ope(sys, dd, p1, bound));
  if (is_ope_uni(name, p1, "integ"))
    return std::make_shared<OpeFunctional>(dd, OpeFunctional::INTEG, parse_ope(sys, dd, p1, bound), bound, nullptr,
                                           nullptr);
  if (is_ope_uni(name, p1, "integvolume"))
    return std::make_shared<OpeFunctional>(dd, OpeFunctional::INTEG_VOLUME, parse_ope(sys, dd, p1, bound), bound,
                                           nullptr, nullptr);
  if (is_ope_uni(name, p1, "sqrt"))
    return std::make_shared<OpeFunc>(dd, OpeFunc::SQRT, parse_ope(sys, dd, p1, bound));
  if (is_ope_uni(name, p1, "exp")) return std::make_shared<OpeFunc>(dd, OpeFunc::EXP, parse_ope(sys, dd, p1, bound));
  if (is_ope_uni(name, p1, "log")) return std::make_shared<OpeFunc>(dd, OpeFunc::LOG, parse_ope(sys, dd, p1, bound));
  // the order of give_ope.cpp:834-867
  static const std::pair<const char*, OpeFunc::Kind> funcs[] = {
      {"atanh", OpeFunc::ATANH}, {"cos", OpeFunc::COS}, {"sin", OpeFunc::SIN}, {"cosh", OpeFunc::COSH},
      {"sinh", OpeFunc::SINH}};
  for (const auto& f : funcs)
    if (is_ope_uni(name, p1, f.first)) return std::make_shared<OpeFunc>(dd, f.second, parse_ope(sys, dd, p1, bound));
  if (is_ope_uni2(name, p1, p2, "scal"))
    return std::make_shared<OpeScal>(dd, parse_ope(sys, dd, p1, bound), parse_ope(sys, dd, p2, bound));
  // partial_x(f) etc.
  for (int i = 0; i < 3; i++) {
    std::string pn = std::string("partial_") + "xyz"[i];
    if (is_ope_uni(name, p1, pn)) return std::make_shared<OpePartial>(dd, i + 1, parse_ope(sys, dd, p1, bound));
  }
  // D_i X, D^i X (is_ope_deriv, give_ope.cpp:385) and partial_i X
  // (is_ope_partial, give_ope.cpp:491): one index letter, then the operand
  if (name.size() > 3 && name[0] == 'D' && (name[1] == '_' || name[1] == '^') && name[2] != ' ') {
    if (!sys.has_metric()) throw KdError(KD_ERR_ARG, "D_i needs a metric (Metric_flat::set_system): " + name);
    return std::make_shared<OpeDer>(dd, name[2], parse_ope(sys, dd, name.substr(3), bound));
  }
  if (name.size() > 9 && name.compare(0, 8, "partial_") == 0 && name[8] != ' ')
    return std::make_shared<OpeDer>(dd, name[8], parse_ope(sys, dd, name.substr(9), bound));
  // integer power: split at the last '^' (is_ope_pow, give_ope.cpp:519)
  if (count_char(name, '^') >= 1) {
    if (get_parts(name, p1, p2, '^', 0)) {
      std::string e = p2;
      while (!e.empty() && e.back() == ' ') e.pop_back();
      char* end = nullptr;
      long n = std::strtol(e.c_str(), &end, 0);
      if (!e.empty() && end && *end == '\0')
        return std::make_shared<OpePow>(dd, static_cast<int>(n), parse_ope(sys, dd, p1, bound));
    }
  }
  std::string bare = name;
  while (!bare.empty() && bare.back() == ' ') bare.pop_back();
  int which = sys.find_var_double(bare);
  if (which >= 0) return std::make_shared<OpeLeaf>(dd, OpeLeaf::VAR_DOUBLE, which);
  which = sys.find_var(bare);
  if (which >= 0) return std::make_shared<OpeLeaf>(dd, OpeLeaf::VAR, which);
  which = sys.find_cst(bare);
  if (which >= 0) return std::make_shared<OpeLeaf>(dd, OpeLeaf::CST, which);
  double v;
  if (is_double_str(name, v)) return std::make_shared<OpeLeaf>(dd, OpeLeaf::HARD, -1, v);
  which = sys.find_def(bare, dd);
  if (which >= 0) return std::make_shared<OpeLeaf>(dd, OpeLeaf::DEF, which);
  // tensors, with or without index names (is_tensor, name_tools.cpp:187):
  // one word, the name up to the first '_' or '^', then the index letters
  if (bare.find(' ') == std::string::npos) {
    std::string base = bare, idx;
    const size_t p = bare.find_first_of("_^");
    if (p != std::string::npos) {
      base = bare.substr(0, p);
      for (size_t i = p; i < bare.size(); i++)
        if (bare[i] != '_' && bare[i] != '^') idx.push_back(bare[i]);
    }
    if (!base.empty()) {
      which = sys.find_var_vector(base);
      if (which >= 0) return std::make_shared<OpeLeaf>(dd, OpeLeaf::VAR_VECTOR, which, 0.0, idx);
      if (sys.has_metric() && base == sys.metric_name() && idx.size() == 2)
        return std::make_shared<OpeLeaf>(dd, OpeLeaf::METRIC, -1, 0.0, idx);
      which = sys.find_cst_vector(base);
      if (which >= 0) return std::make_shared<OpeLeaf>(dd, OpeLeaf::CST_VECTOR, which, 0.0, idx);
      if (!idx.empty()) {
        which = sys.find_def(base, dd);
        if (which >= 0) return std::make_shared<OpeLeaf>(dd, OpeLeaf::DEF, which, 0.0, idx);
      }
    }
  }
  // user-defined operators come last, as in give_ope.cpp:1107
  for (const auto& u : sys.user_opes())
    if (is_ope_uni(name, p1, u.name.c_str()))
      return std::make_shared<OpeEos>(dd, u.eos, u.var, parse_ope(sys, dd, p1, bound));
  throw KdError(KD_ERR_ARG, "Unknown operator " + bare);
}

OpePtr make_value_at(int dom, OpePtr target, const int pos[3]) {
  return std::make_shared<OpeFunctional>(dom, OpeFunctional::VAL, std::move(target), -1, pos, nullptr);
}

OpePtr make_value_at_point(int dom, OpePtr target, const double num[3]) {
  return std::make_shared<OpeFunctional>(dom, OpeFunctional::POINT, std::move(target), -1, nullptr, num);
}

}  // namespace kd
