// System_of_eqs (include/system_of_eqs.hpp:54) on the GPU: registry of
// unknowns, constants, definitions and equations; residual F(u)
// (sec_member, src/System_of_eqs/solver.cpp:49); Jacobian assembly that
// replaces the do_col_J column loop (solver.cpp:120) by one batched tangent
// pass per (unknown field, domain); and the update x -> fields
// (xx_to_vars, src/System_of_eqs/system_of_eqs.cpp:597).
#pragma once
#include <map>
#include <tuple>
#include <unordered_map>
#include <memory>
#include <string>
#include <vector>

#include "kd_term.hpp"

namespace kd {

// A user field (Kadath Scalar): one Val_domain per domain, kept in device
// memory owned by the field.
class Field {
 public:
  Field(Context* ctx, const Space* sp);
  ~Field();
  Field(const Field&) = delete;
  Field& operator=(const Field&) = delete;

  struct PerDom {
    bool zero = true;
    bool in_conf = false, in_coef = false;
    double* c = nullptr;
    double* cf = nullptr;
    Base base;
  };
  Context* ctx;
  const Space* sp;
  std::vector<PerDom> d;

  DVal val(int dom) const;
  void assign(int dom, const DVal& v);       // copies v's representations
  void set_conf_host(int dom, const double* values);
  void set_value(double v);                   // Scalar = v (conf)
  void std_base();
  // Scalar::val_point (include/scalar.hpp:221): value at a Cartesian point.
  double val_point(const double point[3]);
  // Host read-back in the requested representation (computes it if needed).
  void get_conf_host(int dom, double* out);
  void get_coef_host(int dom, double* out);
};

struct CsrTable {
  const int* rowptr = nullptr;
  const int* idx = nullptr;
  const double* w = nullptr;
  int nrows = 0;
  long long nnz = 0;
};

class System;

// State of one evaluation pass (residual or one batched Jacobian block).
// Node values of one iterate, recorded by a value pass (the residual) and
// reused by every tangent pass of the Jacobian at the same iterate.  The
// values live in their own arena, so the per-seed-block scratch resets do
// not touch them.
struct ValueCache {
  std::unordered_map<const Ope*, Term> vals;
  DeviceArena arena{size_t(64) << 20};
  bool valid = false;
  void clear() {
    vals.clear();
    arena.reset();
    valid = false;
  }
  // Keeps the value part of t; fields known only by coefficients also get
  // their collocation values now, since tangent products need them.
  void store(const Ope* node, const Term& t);
};

// Tangents of the outermost iterate-independent nodes (Ope::cache_der),
// per seed block: kept from one Jacobian assembly to the next, so that the
// linear parts of the equations (Laplacians of the unknowns, matching and
// boundary conditions, ...) are computed once per system.
struct TangentCache {
  struct Entry {
    bool is_double = false;
    double dd = 0.0;
    const double* ddv = nullptr;  // per-seed tangent of a double (arena copy)
    int ddb = 0;
    std::vector<DVal> dt;
  };
  std::map<std::tuple<const Ope*, int, int>, Entry> ders;
  DeviceArena arena{size_t(256) << 20};
  void clear() {
    ders.clear();
    arena.reset();
  }
  // Deep copy of t's tangent into the arena.
  void store(Context* ctx, const Ope* node, int var, int dom, const Term& t);
};

// Deep copy of a DVal's representations into an arena (metadata kept).
DVal copy_to_arena(Context* ctx, const DVal& d, DeviceArena& arena);

struct EvalState {
  System* sys = nullptr;
  bool with_der = false;
  int B = 1;               // number of tangent seeds
  int seed_var = -1;       // field unknown being seeded (-1: a double unknown)
  int seed_dom = -1;
  int seed_var_double = -1;
  int seed_cst = -1;       // double constant seeded (dF/dp passes)
  DVal seed;               // batch-B coefficient patterns
  // definition values by (definition, domain, stream): equations of
  // different domains run on different streams, and a value is only reused
  // on the stream that computed it (no cross-stream hazard on its buffers or
  // its lazily computed representations)
  std::map<std::tuple<int, int, cudaStream_t>, Term> def_cache;
  // do_JX: every unknown field seeded at once (tangent = x mapped to
  // coefficients per (variable, domain)); var doubles get jx_doubles.
  const std::map<std::pair<int, int>, DVal>* jx_seeds = nullptr;
  const std::vector<double>* jx_doubles = nullptr;
  ValueCache* vcache = nullptr;  // node values: recorded (record) or reused (with_der)
  bool record = false;
  TangentCache* tcache = nullptr;  // tangents of iterate-independent nodes (with_der)

  Term var_term(int which, int dom);
  Term var_double_term(int which, int dom);
  Term cst_term(int which, int dom);
  Term def_term(int which, int dom);
  // Cartesian vectors: the three component entries from `first` on.
  Term var_vector_term(int first, int dom);
  Term cst_vector_term(int first, int dom);
  // The flat metric g_ij = delta_ij (Metric_flat with a Cartesian basis).
  Term metric_term(int dom);
};

struct Equation {
  // INSIDE with order 2 is Eq_inside, any other order Eq_order (order 0:
  // Eq_full, every coefficient); FIRST_INTEGRAL is Eq_first_integral over
  // domains dom..other_dom.
  enum Kind { INSIDE, BC, MATCHING, FIRST_INTEGRAL };
  Kind kind;
  int dom, bound = -1, other_dom = -1, other_bound = -1;
  int order = 2;
  std::string text;
  OpePtr lhs, rhs;
  // FIRST_INTEGRAL: parts[0] the constant part (in dom), parts[1 + k] the
  // first integral in domain dom + k; n_cond_dom the rows of each domain
  std::vector<OpePtr> parts;
  std::vector<int> n_cond_dom;
  int n_cond = -1;
  int row0 = 0;
  bool take_into_account(int d) const {
    if (kind == FIRST_INTEGRAL) return d >= dom && d <= other_dom;
    return d == dom || (kind == MATCHING && d == other_dom);
  }
};

// Integral-type equation (Eq_int, include/system_of_eqs.hpp:1352): one
// condition, the sum of the numbers its parts give (one part per domain of a
// volume integral plus the constant side, or a single point value).  These
// rows come before every other equation (sec_member, solver.cpp:49).
struct IntEquation {
  std::string text;
  std::vector<OpePtr> parts;
  int row = 0;
};

class System {
 public:
  System(Context* ctx, const Space* sp, int dom_min, int dom_max);
  ~System();
  System(const System&) = delete;
  System& operator=(const System&) = delete;

  Context* ctx;
  const Space* sp;
  int dom_min, dom_max;
  int ndom() const { return dom_max - dom_min + 1; }

  // registry (system_of_eqs.cpp:284-440, add_eq.cpp)
  int add_var(const std::string& name, Field* f);
  int add_var_double(const std::string& name, double value);
  int add_cst(const std::string& name, double value);
  int add_cst_field(const std::string& name, Field* f);
  // A Cartesian vector unknown or constant (add_var / add_cst with a Vector
  // of Cartesian basis): three fields, components x, y, z, each with the
  // basis of its component.  Equations name it with one index ("bet^i").
  // Its unknowns come domain by domain, the three components inside each
  // domain (xx_to_vars and affecte_tau of a Tensor).
  int add_var_vector(const std::string& name, Field* const comps[3]);
  int add_cst_vector(const std::string& name, Field* const comps[3]);
  // Metric_flat::set_system: D_i / D^i become the flat covariant
  // derivatives and `name` (with two indices) the metric tensor.
  void set_metric_flat(const std::string& name);
  bool has_metric() const { return !metric_.empty(); }
  const std::string& metric_name() const { return metric_; }
  // "A_ij = ..." defines a tensor whose index order is the left side's.
  void add_def(int dom, const std::string& text);
  void add_eq_inside(int dom, const std::string& eq);
  void add_eq_bc(int dom, int bound, const std::string& eq);
  void add_eq_matching(int dom, int bound, const std::string& eq);
  // add_eq_order (add_eq.cpp:80): the tau export drops `order` radial
  // coefficients; add_eq_full (add_eq.cpp:291, Eq_full) is order 0.
  void add_eq_order(int dom, int order, const std::string& eq);
  void add_eq_full(int dom, const std::string& eq) { add_eq_order(dom, 0, eq); }
  // add_eq_first_integral (add_eq.cpp:414, Eq_first_integral): integ_part
  // minus its value at the first collocation point of dom_min, on every
  // coefficient of dom_min..dom_max; in dom_min the points of radial index
  // 0 carry cst_part's value at that point instead.
  void add_eq_first_integral(int dom_min, int dom_max, const std::string& integ_part, const std::string& cst_part);
  // "integvolume(f) = c": the volume integral of f over domains dmin..dmax
  // equals c (Space_spheric::add_eq_int_volume, spheric_add_eq.cpp:81).
  void add_eq_int_volume(int dmin, int dmax, const std::string& eq);
  // "integ(f) = c" with integ() at the outer boundary of the last
  // (compactified) domain: the surface integral at infinity.
  void add_eq_int_inf(const std::string& eq);
  // The scalar expression vanishes at collocation point pos of domain dom
  // (add_eq_val, add_eq.cpp:343).
  void add_eq_val(int dom, const std::string& eq, const int pos[3]);
  // The scalar expression vanishes at a Cartesian point, evaluated in domain
  // dom by the spectral summation (add_eq_point, add_eq.cpp:355).
  void add_eq_point(int dom, const std::string& eq, const double point[3]);
  int n_int_equations() const { return static_cast<int>(ieqs_.size()); }

  int find_var(const std::string& n) const;
  int find_var_double(const std::string& n) const;
  int find_cst(const std::string& n) const;
  int find_def(const std::string& n, int dom) const;
  int find_var_vector(const std::string& n) const;
  int find_cst_vector(const std::string& n) const;

  // User-defined operators of the EOS kind (System_of_eqs::add_ope with
  // EOS<eos, var>::action, include/system_of_eqs.hpp:277): name(h) gives var
  // of a cold piecewise polytrope at the enthalpy h.
  struct UserOpe {
    std::string name;
    KdEos eos;
    int var;
  };
  void add_ope_eos(const std::string& name, int var, const KdEos& eos);
  const std::vector<UserOpe>& user_opes() const { return user_opes_; }

  double var_double(int i) const { return vdoubles_[i].value; }
  void set_var_double(int i, double v) { vdoubles_[i].value = v; }

  // Sizes (valid after the first residual evaluation).
  int nbr_unknowns();
  int nbr_conditions() const { return nbr_conditions_; }
  int n_equations() const { return static_cast<int>(eqs_.size()); }
  const Equation& equation(int i) const { return eqs_[i]; }

  // F(u) into a device vector of nbr_conditions doubles.
  // record: keep every node value for a following jacobian(..., true).
  void residual(double* d_F, bool record = false);
  // Column-major dense Jacobian (ld >= nbr_conditions) on the device.
  // reuse: take node values from the preceding residual(..., true) at the
  // same iterate; otherwise a value pass is run first.
  // rectangular: allow more conditions than unknowns (Gauss-Newton), J is
  // nbr_conditions x nbr_unknowns with ld >= nbr_conditions.
  void jacobian(double* d_J, long long ld, bool reuse = false, bool rectangular = false);
  // do_JX (src/System_of_eqs/solver.cpp:87): y = J x without forming J, one
  // tangent pass with every unknown seeded by x through affecte_tau.
  void jx(const double* d_x, double* d_y);
  // Keep the tangents of iterate-independent subtrees between assemblies
  // (default on; off frees them).
  void set_tangent_cache(bool on) {
    cache_tangents_ = on;
    if (!on) tcache_.clear();
  }
  // var = old - (fields built from x)  (do_newton's update, src_par/do_newton.cpp:397-414)
  void update_from_x(const double* d_x);
  // The field xx_to_vars would give variable `var` in domain dd from x
  // (affecte_tau), allocated from the current scratch arena.
  DVal x_to_field(int var, int dd, const double* d_x);
  int n_var_doubles() const { return static_cast<int>(vdoubles_.size()); }
  // A double constant's value (add_cst(name, double)); changing it drops
  // the recorded node values.
  void set_cst(int i, double v);
  double cst_value(int i) const { return csts_.at(i).value; }
  // dF/dp for the double constant p, in one tangent pass seeding only p
  // (device vector of nbr_conditions doubles).
  void dres_dcst(int cst, double* d_y);
  // Gradient of var's value at a Cartesian point with respect to the
  // unknown vector (host, nbr_unknowns doubles): the point's summation
  // weights mapped through the unknown coefficient patterns.
  void val_point_gradient(int var, const double point[3], double* g);
  // Q and dQ/dy (device vector of nbr_unknowns) for an integral observable:
  // kind 0, `expr` (the left side of an add_eq_int_volume equation, e.g.
  // "integvolume(psi^5)") summed over domains dmin..dmax; kind 1, the left
  // side of add_eq_int_inf (e.g. "integ(dn(P))") in the last domain.  The gradient is the
  // Jacobian row that equation would have (Eq_int::get_der, eq_int.cpp:45).
  double integral_gradient(int kind, int dmin, int dmax, const std::string& expr, double* d_g);
  // Fields changed outside update_from_x: drop the recorded node values.
  void invalidate_values() { vcache_.clear(); }
  // Replays the value pass of residual(d_F, true) from a CUDA graph when the
  // state it depends on (field representations and bases, the numbers, the
  // equations) is the one it was captured in; captures it otherwise.
  // Systems with integral-type equations are never captured (their values
  // come back to the host in the pass).
  void set_residual_graph(bool on);
  long long residual_graph_replays = 0, residual_graph_captures = 0;
  long long jacobian_graph_replays = 0, jacobian_graph_captures = 0;

  struct VarInfo {
    std::string name;
    Field* f;
    int ncmp = 1;  // 3 for the components of a vector
    int cmp = 0;   // component 0, 1, 2 of a vector
  };
  struct VarDouble {
    std::string name;
    double value;
  };
  struct CstInfo {
    std::string name;
    bool is_field;
    double value;
    Field* f;
    int ncmp = 1;
    int cmp = 0;
  };
  struct DefInfo {
    std::string name;
    int dom;
    OpePtr ope;
    std::string idx;  // index names of the left side, in order
  };
  const std::vector<VarInfo>& vars() const { return vars_; }

  // Column offset of the unknowns of (var, dom); valid after nbr_unknowns().
  int col_offset(int var, int dom) const { return col0_.at({var, dom}); }
  int n_unknowns_of(int var, int dom) const { return nunk_.at({var, dom}); }

  // Export table of a residual value (cached by domain, basis, kind).
  const CsrTable& export_table(const Domain& d, const Base& b, int kind, int order_or_bound);

  long long assembly_launches = 0;

 private:
  friend struct EvalState;
  std::vector<VarInfo> vars_;
  std::vector<VarDouble> vdoubles_;
  std::vector<CstInfo> csts_;
  std::vector<DefInfo> defs_;
  std::vector<UserOpe> user_opes_;
  std::vector<Equation> eqs_;
  std::vector<IntEquation> ieqs_;
  std::string metric_;
  int nbr_conditions_ = -1;
  int nbr_unknowns_ = -1;
  std::map<std::pair<int, int>, int> col0_, nunk_;
  std::map<std::pair<int, int>, const double*> seeds_;  // device seed blocks
  std::map<std::pair<int, int>, CsrTable> xmaps_;      // affecte_tau maps
  std::map<std::vector<int>, CsrTable> tables_;
  ValueCache vcache_;
  TangentCache tcache_;
  bool cache_tangents_ = true;
  // residual graphs, one per state seen at least twice (at most 4)
  struct ValueGraph {
    std::vector<long long> sig;
    cudaGraphExec_t exec = nullptr;
    double* F = nullptr;
    long long launches = 0;
    std::unordered_map<const Ope*, Term> vals;
    size_t mark = 0;
    long long last_use = 0;
  };
  bool graph_on_ = false, graph_failed_ = false;
  std::vector<ValueGraph> graphs_;
  std::vector<std::vector<long long>> seen_sigs_;
  long long graph_clock_ = 0;
  std::vector<long long> state_signature() const;
  void residual_pass(double* d_F, bool record);
  // The Jacobian's seed passes as a CUDA graph: captured the second time a
  // signature is met, with the tangent cache as the pass left it (its host
  // side; the replay refills the device side at the same addresses).
  struct JacGraph {
    std::vector<long long> sig;
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;
    std::map<std::tuple<const Ope*, int, int>, TangentCache::Entry> tders;
    size_t tmark = 0;
    long long last_use = 0;
  };
  bool jgraph_failed_ = false;
  std::vector<JacGraph> jgraphs_;
  std::vector<std::vector<long long>> jseen_;
  std::vector<long long> jacobian_signature(const double* d_J, long long ld, bool rectangular) const;
  void jacobian_pass(double* d_J, long long ld);
  void drop_graph();

  void compute_unknowns();
  void apply(Equation& eq, EvalState& st, Term& lhs, Term& rhs, bool do_lhs, bool do_rhs);
  int count_rows(const Equation& eq, const Term& t);
  void export_term(const Equation& eq, const Term& t, bool der, int side_dom, int side_bound, double* out,
                   long long osf, long long osr, int batch, double alpha, bool accumulate);
  std::vector<Term> eval_parts(const Equation& eq, EvalState& st);
  int count_rows_fi(Equation& eq, const std::vector<Term>& parts);
  void export_first_integral(const Equation& eq, const std::vector<Term>& parts, bool der, double* out, long long osf,
                             long long osr, int batch, bool accumulate);
  // One equation's tangent rows (every side), added into out.
  void export_tangent(Equation& eq, EvalState& st, double* out, long long osf, int batch);
  CsrTable upload_rows(const std::vector<SparseRow>& rows);
  void add_int_equation(IntEquation ie);
  // Adds the tangents of the integral equations to out[row + b * osf],
  // b < B: only the parts in domain dom, or every part when dom < 0.
  void export_int_ders(EvalState& st, int dom, double* out, long long osf, int B);
  const double* seed_block(int var, int dom, int& B, Base& base);
  const CsrTable& xmap(int var, int dom);
};

}  // namespace kd
