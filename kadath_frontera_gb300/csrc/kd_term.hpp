// Term_eq (include/term_eq.hpp:63) and Ope_eq trees (include/ope_eq.hpp:34)
// for one domain, evaluated on the GPU.  A Term carries a value and,
// during Jacobian assembly, a batched tangent ("der"): B forward-mode seeds
// pushed through the same tree in one pass, instead of the reference's one
// column per pass.
#pragma once
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "kd_field.hpp"

namespace kd {

struct Term {
  int dom = -1;
  bool is_double = false;
  // double data
  double vd = 0.0;
  bool has_dd = false;
  double dd = 0.0;  // tangent of a double (same for every seed)
  // Tangent of a double that differs from seed to seed (an integral or a
  // point value of a seeded field): ddb doubles on the device, from the
  // pass's arena; null when every seed has the tangent dd.
  const double* ddv = nullptr;
  int ddb = 0;
  Context* ddctx = nullptr;
  // tensor data: 3^valence Cartesian components, row-major over the indices
  int valence = 0;
  // index names, one letter per index (Kadath's name_ind), when the tensor
  // came from index notation ("bet^i", "D_j ..."); empty otherwise.  With
  // the flat Cartesian metric, upper and lower indices share components.
  std::string idx;
  std::vector<DVal> vt;
  bool has_dt = false;
  std::vector<DVal> dt;

  static Term dbl(int dom, double v) {
    Term t;
    t.dom = dom;
    t.is_double = true;
    t.vd = v;
    return t;
  }
  static Term dbl_der(int dom, double v, double d) {
    Term t = dbl(dom, v);
    t.has_dd = true;
    t.dd = d;
    return t;
  }
  bool has_der() const { return is_double ? has_dd : has_dt; }
};

Term operator+(const Term& a, const Term& b);
Term operator-(const Term& a, const Term& b);
Term operator*(const Term& a, const Term& b);
Term operator/(const Term& a, const Term& b);
Term operator-(const Term& a);
// The same operations with the result's value supplied (cv != nullptr): the
// value is adopted and only the tangent is computed.
Term t_add(const Term& a, const Term& b, const Term* cv);
Term t_sub(const Term& a, const Term& b, const Term* cv);
Term t_mul(const Term& a, const Term& b, const Term* cv);
Term t_div(const Term& a, const Term& b, const Term* cv);
Term t_neg(const Term& a, const Term* cv);
Term term_pow(const Term& a, int n, const Term* cv = nullptr);
// r's tangent = ca a' + cb b' for doubles a and b (b may be null); per seed
// when either operand's tangent is.
void dbl_tangent_lincomb(Term& r, double ca, const Term& a, double cb, const Term* b);

// b's components reordered to a's index names (both named, same letters);
// b itself when either has no names.
Term align_to(const Term& b, const Term& a);
// Sums over every index name that appears twice (flat metric), the terms in
// the order 1, 2, 3 of the summed index (Tensor::do_summation_one_dom).
Term contract_self(const Term& t);

class System;
struct EvalState;

// Expression-tree node.
class Ope {
 public:
  explicit Ope(int dom) : dom(dom) {}
  virtual ~Ope() = default;
  // Evaluates the node.  When the pass carries a value cache, a value pass
  // records the node's value and a tangent pass reuses it: the value part of
  // a Term does not depend on the Jacobian seeds, so it is computed once per
  // iterate instead of once per seed block.
  Term eval(EvalState& st) const;
  // cv: this node's value, already known (tangent-only evaluation), or null.
  virtual Term action(EvalState& st, const Term* cv) const = 0;
  // Leaves are cheap (views of fields or doubles) and are not cached.
  virtual bool cacheable() const { return true; }
  virtual std::vector<const Ope*> kids() const { return {}; }
  int dom;
  // Dependence classes, set at construction from the children:
  //   vc  the value does not depend on the iterate nor on constant fields;
  //   dc  the tangent does not depend on the iterate (only on the seeds):
  //       linear operators of unknowns, products with constant values, ...
  //   dz  the tangent is identically zero.
  bool vc = false, dc = false, dz = false;
  // Outermost dc node of its tree: its batched tangents are kept from one
  // Jacobian assembly to the next (set by mark_tangent_frontier).
  mutable bool cache_der = false;
};

void mark_tangent_frontier(const Ope* root);
using OpePtr = std::shared_ptr<Ope>;

// Parses an expression for domain `dom` (System_of_eqs::give_ope,
// src/System_of_eqs/give_ope.cpp:1127).  `bound` is the boundary used by
// dn(); -1 inside the domain.
OpePtr parse_ope(const System& sys, int dom, const std::string& expr, int bound);

// Ope_val (src/Ope_eq/ope_val.cpp): the value of a scalar expression at the
// collocation point pos (r, theta, phi indices) of domain dom.
OpePtr make_value_at(int dom, OpePtr target, const int pos[3]);
// Ope_point (src/Ope_eq/ope_point.cpp): the value at numerical coordinates
// num = (xi, theta, phi) of domain dom, by the spectral summation.
OpePtr make_value_at_point(int dom, OpePtr target, const double num[3]);

// Trims spaces the way Kadath's trim_spaces does (single spaces, one trailing).
std::string trim_expr(const std::string& s);

}  // namespace kd
