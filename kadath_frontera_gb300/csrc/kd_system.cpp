#include "kd_system.hpp"

#include <algorithm>

#include <cstring>
#include <sstream>

namespace kd {

// ------------------------------------------------------------------ Field --
Field::Field(Context* c, const Space* s) : ctx(c), sp(s), d(s->ndom()) {
  for (int i = 0; i < s->ndom(); i++) {
    cuda_check(cudaMalloc(&d[i].c, sizeof(double) * s->dom(i).npts()), "cudaMalloc(field conf)");
    cuda_check(cudaMalloc(&d[i].cf, sizeof(double) * s->dom(i).ncoefs()), "cudaMalloc(field coef)");
  }
}

Field::~Field() {
  for (auto& p : d) {
    cudaFree(p.c);
    cudaFree(p.cf);
  }  cudaGetLastError();  // teardown status is not the next launch's error
}

DVal Field::val(int dom) const {
  const PerDom& p = d.at(dom);
  const Domain* dm = &sp->dom(dom);
  if (p.zero) {
    DVal z = DVal::zeros(ctx, dm, 1);
    z.base = p.base;
    return z;
  }
  DVal v(ctx, dm, 1);
  v.zero = false;
  v.base = p.base;
  if (p.in_conf) {
    v.c = p.c;
    v.in_conf = true;
  }
  if (p.in_coef) {
    v.cf = p.cf;
    v.in_coef = true;
  }
  return v;
}

void Field::assign(int dom, const DVal& v) {
  PerDom& p = d.at(dom);
  if (v.batch != 1) throw KdError(KD_ERR_ARG, "a field holds one value per domain");
  p.base = v.base;
  if (v.zero) {
    p.zero = true;
    p.in_conf = p.in_coef = false;
    return;
  }
  p.zero = false;
  p.in_conf = v.in_conf;
  p.in_coef = v.in_coef;
  const Domain& dm = sp->dom(dom);
  if (v.in_conf && v.c != p.c)
    cuda_check(cudaMemcpyAsync(p.c, v.c, sizeof(double) * dm.npts(), cudaMemcpyDeviceToDevice, ctx->stream()),
               "field copy");
  if (v.in_coef && v.cf != p.cf)
    cuda_check(cudaMemcpyAsync(p.cf, v.cf, sizeof(double) * dm.ncoefs(), cudaMemcpyDeviceToDevice, ctx->stream()),
               "field copy");
}

void Field::set_conf_host(int dom, const double* values) {
  PerDom& p = d.at(dom);
  const Domain& dm = sp->dom(dom);
  cuda_check(cudaMemcpyAsync(p.c, values, sizeof(double) * dm.npts(), cudaMemcpyHostToDevice, ctx->stream()),
             "field upload");
  cuda_check(cudaStreamSynchronize(ctx->stream()), "sync");
  p.zero = false;
  p.in_conf = true;
  p.in_coef = false;
}

void Field::set_value(double v) {
  for (int i = 0; i < sp->ndom(); i++) {
    PerDom& p = d[i];
    if (v == 0.0) {
      p.zero = true;
      p.in_conf = p.in_coef = false;
      continue;
    }
    cuda_check(launch_ew(EW_FILL, sp->dom(i).npts(), 1, nullptr, 1, nullptr, p.c, v, 0.0, ctx->stream()), "fill");
    p.zero = false;
    p.in_conf = true;
    p.in_coef = false;
  }
}

void Field::std_base() {
  for (int i = 0; i < sp->ndom(); i++) d[i].base = sp->dom(i).std_base();
}

void Field::get_conf_host(int dom, double* out) {
  const Domain& dm = sp->dom(dom);
  if (d.at(dom).zero) {
    std::memset(out, 0, sizeof(double) * dm.npts());
    return;
  }
  size_t mark = ctx->scratch().mark();
  DVal v = val(dom);
  v.coef_i();
  cuda_check(cudaMemcpyAsync(out, v.c, sizeof(double) * dm.npts(), cudaMemcpyDeviceToHost, ctx->stream()), "D2H");
  cuda_check(cudaStreamSynchronize(ctx->stream()), "sync");
  ctx->scratch().release_to(mark);
}

double Field::val_point(const double point[3]) {
  double num[3];
  const int dd = sp->locate(point, num);
  if (dd < 0) throw KdError(KD_ERR_ARG, "val_point: the point is in no domain");
  const Domain& dm = sp->dom(dd);
  if (d.at(dd).zero) return 0.0;
  std::vector<double> cf(dm.ncoefs()), w;
  get_coef_host(dd, cf.data());
  dm.point_weights(d[dd].base, num, w);
  double s = 0.0;
  for (size_t c = 0; c < cf.size(); c++) s += w[c] * cf[c];
  return s;
}

void Field::get_coef_host(int dom, double* out) {
  const Domain& dm = sp->dom(dom);
  if (d.at(dom).zero) {
    std::memset(out, 0, sizeof(double) * dm.ncoefs());
    return;
  }
  size_t mark = ctx->scratch().mark();
  DVal v = val(dom);
  v.coef();
  cuda_check(cudaMemcpyAsync(out, v.cf, sizeof(double) * dm.ncoefs(), cudaMemcpyDeviceToHost, ctx->stream()), "D2H");
  cuda_check(cudaStreamSynchronize(ctx->stream()), "sync");
  ctx->scratch().release_to(mark);
}

// -------------------------------------------------------------- EvalState --
Term EvalState::var_term(int which, int dom) {
  Term t;
  t.dom = dom;
  t.valence = 0;
  const auto& vi = sys->vars_.at(which);
  t.vt.push_back(vi.f->val(dom));
  if (with_der) {
    t.has_dt = true;
    if (jx_seeds) {
      auto it = jx_seeds->find(std::make_pair(which, dom));
      t.dt.push_back(it != jx_seeds->end() ? it->second : DVal::zeros(sys->ctx, &sys->sp->dom(dom), B));
    } else if (which == seed_var && dom == seed_dom) {
      t.dt.push_back(seed);
    } else {
      t.dt.push_back(DVal::zeros(sys->ctx, &sys->sp->dom(dom), B));
    }
  }
  return t;
}

Term EvalState::var_double_term(int which, int dom) {
  Term t = Term::dbl(dom, sys->vdoubles_.at(which).value);
  if (with_der) {
    t.has_dd = true;
    if (jx_doubles) t.dd = jx_doubles->at(which);
    else t.dd = (which == seed_var_double) ? 1.0 : 0.0;
  }
  return t;
}

Term EvalState::cst_term(int which, int dom) {
  const auto& c = sys->csts_.at(which);
  if (!c.is_field) {
    Term t = Term::dbl(dom, c.value);
    if (with_der) {
      t.has_dd = true;
      t.dd = (which == seed_cst) ? 1.0 : 0.0;
    }
    return t;
  }
  Term t;
  t.dom = dom;
  t.vt.push_back(c.f->val(dom));
  if (with_der) {
    t.has_dt = true;
    t.dt.push_back(DVal::zeros(sys->ctx, &sys->sp->dom(dom), B));
  }
  return t;
}

Term EvalState::def_term(int which, int dom) {
  auto key = std::make_tuple(which, dom, sys->ctx->stream());
  auto it = def_cache.find(key);
  if (it != def_cache.end()) return it->second;
  const auto& df = sys->defs_.at(which);
  Term t = df.ope->eval(*this);
  if (!df.idx.empty()) {
    if (t.is_double || static_cast<int>(df.idx.size()) != t.valence)
      throw KdError(KD_ERR_ARG, "the definition of " + df.name + " has " + std::to_string(df.idx.size()) +
                                    " indices, its value another valence");
    if (!t.idx.empty()) {
      Term names;
      names.idx = df.idx;
      t = align_to(t, names);
    }
    t.idx = df.idx;
  }
  def_cache[key] = t;
  return t;
}

Term EvalState::var_vector_term(int first, int dom) {
  Term t;
  t.dom = dom;
  t.valence = 1;
  for (int c = 0; c < 3; c++) {
    Term k = var_term(first + c, dom);
    t.vt.push_back(k.vt[0]);
    if (k.has_dt) {
      t.has_dt = true;
      t.dt.push_back(k.dt[0]);
    }
  }
  return t;
}

Term EvalState::cst_vector_term(int first, int dom) {
  Term t;
  t.dom = dom;
  t.valence = 1;
  for (int c = 0; c < 3; c++) {
    Term k = cst_term(first + c, dom);
    t.vt.push_back(k.vt[0]);
    if (k.has_dt) {
      t.has_dt = true;
      t.dt.push_back(k.dt[0]);
    }
  }
  return t;
}

Term EvalState::metric_term(int dom) {
  const Domain* dm = &sys->sp->dom(dom);
  Term t;
  t.dom = dom;
  t.valence = 2;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      if (i == j) {
        DVal one = DVal::constant(sys->ctx, dm, 1.0);
        one.base = dm->std_base();
        t.vt.push_back(one);
      } else {
        t.vt.push_back(DVal::zeros(sys->ctx, dm, 1));
      }
    }
  if (with_der) {
    t.has_dt = true;
    for (int c = 0; c < 9; c++) t.dt.push_back(DVal::zeros(sys->ctx, dm, B));
  }
  return t;
}

// ------------------------------------------------------------ node values --
void ValueCache::store(const Ope* node, const Term& t) {
  Term v;
  v.dom = t.dom;
  v.is_double = t.is_double;
  v.vd = t.vd;
  v.valence = t.valence;
  v.idx = t.idx;
  v.vt = t.vt;
  for (auto& x : v.vt)
    if (!x.zero && !x.in_conf && x.base.def) x.coef_i();
  vals[node] = std::move(v);
}

DVal copy_to_arena(Context* ctx, const DVal& d, DeviceArena& arena) {
  DVal c(d.ctx ? d.ctx : ctx, d.dom, d.batch);
  c.zero = d.zero;
  c.base = d.base;
  if (!d.zero) {
    if (d.in_conf) {
      const size_t n = static_cast<size_t>(d.npts()) * d.batch;
      double* p = arena.alloc_doubles(n);
      cuda_check(cudaMemcpyAsync(p, d.c, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream()), "arena copy");
      c.c = p;
      c.in_conf = true;
    }
    if (d.in_coef) {
      const size_t n = static_cast<size_t>(d.ncoefs()) * d.batch;
      double* p = arena.alloc_doubles(n);
      cuda_check(cudaMemcpyAsync(p, d.cf, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream()), "arena copy");
      c.cf = p;
      c.in_coef = true;
    }
  }
  return c;
}

void TangentCache::store(Context* ctx, const Ope* node, int var, int dom, const Term& t) {
  Entry e;
  e.is_double = t.is_double;
  e.dd = t.dd;
  if (t.ddv) {
    double* p = arena.alloc_doubles(t.ddb);
    cuda_check(cudaMemcpyAsync(p, t.ddv, sizeof(double) * t.ddb, cudaMemcpyDeviceToDevice, ctx->stream()), "arena copy");
    e.ddv = p;
    e.ddb = t.ddb;
  }
  for (const DVal& d : t.dt) e.dt.push_back(copy_to_arena(ctx, d, arena));
  ders[std::make_tuple(node, var, dom)] = std::move(e);
}

Term Ope::eval(EvalState& st) const {
  ValueCache* vc = st.vcache;
  if (!vc || !cacheable()) return action(st, nullptr);
  if (st.with_der) {
    auto it = vc->vals.find(this);
    const Term* cv = it != vc->vals.end() ? &it->second : nullptr;
    if (cache_der && st.tcache && cv) {
      const auto key = std::make_tuple(static_cast<const Ope*>(this), st.seed_var, st.seed_dom);
      auto tt = st.tcache->ders.find(key);
      if (tt != st.tcache->ders.end()) {
        // value of this iterate, tangent from an earlier assembly: the
        // subtree is not evaluated at all
        Term r = *cv;
        if (tt->second.is_double) {
          r.has_dd = true;
          r.dd = tt->second.dd;
          r.ddv = tt->second.ddv;
          r.ddb = tt->second.ddb;
          r.ddctx = st.sys->ctx;
        } else {
          r.has_dt = true;
          r.dt = tt->second.dt;
        }
        return r;
      }
      Term r = action(st, cv);
      st.tcache->store(st.sys->ctx, this, st.seed_var, st.seed_dom, r);
      return r;
    }
    return action(st, cv);
  }
  Term t = action(st, nullptr);
  if (st.record) vc->store(this, t);
  return t;
}

namespace {
// Sends every DVal allocation to another arena for the guard's lifetime.
struct ScratchRedirect {
  Context* ctx;
  DeviceArena* prev;
  ScratchRedirect(Context* c, DeviceArena* a) : ctx(c), prev(c->redirect_scratch(a)) {}
  ~ScratchRedirect() { ctx->redirect_scratch(prev); }
};
}  // namespace

// ----------------------------------------------------------------- System --
System::System(Context* c, const Space* s, int dmin, int dmax) : ctx(c), sp(s), dom_min(dmin), dom_max(dmax) {
  if (dmin < 0 || dmax >= s->ndom() || dmin > dmax) throw KdError(KD_ERR_ARG, "bad domain range for the system");
}

System::~System() { drop_graph(); }

void System::drop_graph() {
  for (auto& g : graphs_)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  graphs_.clear();
  seen_sigs_.clear();
  for (auto& g : jgraphs_)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  jgraphs_.clear();
  jseen_.clear();
}

void System::set_residual_graph(bool on) {
  graph_on_ = on;
  if (!on) drop_graph();
}

// Everything the launches of a value pass depend on besides the fields'
// data: which representations each field holds and its bases, the numbers
// that enter kernels as arguments, the registered symbols and equations.
std::vector<long long> System::state_signature() const {
  std::vector<long long> g;
  auto dbl = [&](double v) {
    long long b;
    std::memcpy(&b, &v, sizeof b);
    g.push_back(b);
  };
  auto field = [&](const Field* f) {
    g.push_back(reinterpret_cast<long long>(f));
    for (const auto& p : f->d) {
      g.push_back((p.zero ? 1 : 0) | (p.in_conf ? 2 : 0) | (p.in_coef ? 4 : 0) | (p.base.def ? 8 : 0));
      g.push_back(p.base.p);
      for (int v : p.base.r) g.push_back(v);
      for (int v : p.base.t) g.push_back(v);
    }
  };
  g.push_back(static_cast<long long>(eqs_.size()));
  g.push_back(static_cast<long long>(ieqs_.size()));
  g.push_back(static_cast<long long>(defs_.size()));
  g.push_back(static_cast<long long>(user_opes_.size()));
  for (const auto& v : vars_) field(v.f);
  for (const auto& v : vdoubles_) dbl(v.value);
  for (const auto& c : csts_) {
    if (c.is_field) field(c.f);
    else dbl(c.value);
  }
  return g;
}

namespace {
std::string bare(const std::string& s) {
  std::string t = trim_expr(s);
  while (!t.empty() && t.back() == ' ') t.pop_back();
  return t;
}

// Splits "lhs = rhs" at the last '=' with balanced parentheses on both sides.
bool split_eq(const std::string& s, std::string& l, std::string& r) {
  for (int p = static_cast<int>(s.size()) - 1; p >= 0; p--)
    if (s[p] == '=') {
      l = s.substr(0, p);
      r = s.substr(p + 1);
      auto cnt = [](const std::string& x, char c) {
        int n = 0;
        for (char y : x) n += (y == c);
        return n;
      };
      if (bare(l).empty() || bare(r).empty()) continue;
      if (cnt(l, '(') == cnt(l, ')') && cnt(r, '(') == cnt(r, ')')) return true;
    }
  return false;
}

// Ope_minus of the constant side of an integral equation.
class OpeMinusPart : public Ope {
 public:
  OpeMinusPart(int dom, OpePtr a_) : Ope(dom), a(std::move(a_)) {
    vc = a->vc;
    dc = a->dc;
    dz = a->dz;
  }
  std::vector<const Ope*> kids() const override { return {a.get()}; }
  Term action(EvalState& st, const Term* cv) const override { return t_neg(a->eval(st), cv); }
  OpePtr a;
};

class OpeSubEq : public Ope {
 public:
  OpeSubEq(int dom, OpePtr a_, OpePtr b_) : Ope(dom), a(std::move(a_)), b(std::move(b_)) {
    vc = a->vc && b->vc;
    dc = a->dc && b->dc;
    dz = a->dz && b->dz;
  }
  std::vector<const Ope*> kids() const override { return {a.get(), b.get()}; }
  Term action(EvalState& st, const Term* cv) const override { return t_sub(a->eval(st), b->eval(st), cv); }
  OpePtr a, b;
};
}  // namespace

int System::find_var(const std::string& n) const {
  for (size_t i = 0; i < vars_.size(); i++)
    if (vars_[i].ncmp == 1 && vars_[i].name == n) return static_cast<int>(i);
  return -1;
}
int System::find_var_vector(const std::string& n) const {
  for (size_t i = 0; i < vars_.size(); i++)
    if (vars_[i].ncmp == 3 && vars_[i].cmp == 0 && vars_[i].name == n) return static_cast<int>(i);
  return -1;
}
int System::find_cst_vector(const std::string& n) const {
  for (size_t i = 0; i < csts_.size(); i++)
    if (csts_[i].ncmp == 3 && csts_[i].cmp == 0 && csts_[i].name == n) return static_cast<int>(i);
  return -1;
}
int System::find_var_double(const std::string& n) const {
  for (size_t i = 0; i < vdoubles_.size(); i++)
    if (vdoubles_[i].name == n) return static_cast<int>(i);
  return -1;
}
int System::find_cst(const std::string& n) const {
  for (size_t i = 0; i < csts_.size(); i++)
    if (csts_[i].ncmp == 1 && csts_[i].name == n) return static_cast<int>(i);
  return -1;
}
int System::find_def(const std::string& n, int dom) const {
  for (size_t i = 0; i < defs_.size(); i++)
    if (defs_[i].name == n && defs_[i].dom == dom) return static_cast<int>(i);
  return -1;
}

int System::add_var(const std::string& name, Field* f) {
  if (name.find('_') != std::string::npos || name.find('^') != std::string::npos)
    throw KdError(KD_ERR_ARG, "No indices allowed in names of variables");
  for (int dd = dom_min; dd <= dom_max; dd++)
    if (!f->d[dd].base.def) throw KdError(KD_ERR_STATE, "unknown field without a basis (call std_base)");
  tcache_.clear();  // a new symbol changes the trees that can follow
  vars_.push_back({bare(name), f});
  nbr_unknowns_ = -1;
  return static_cast<int>(vars_.size()) - 1;
}

int System::add_var_vector(const std::string& name, Field* const comps[3]) {
  if (name.find('_') != std::string::npos || name.find('^') != std::string::npos)
    throw KdError(KD_ERR_ARG, "No indices allowed in names of variables");
  for (int c = 0; c < 3; c++)
    for (int dd = dom_min; dd <= dom_max; dd++)
      if (!comps[c]->d[dd].base.def) throw KdError(KD_ERR_STATE, "vector component without a basis (call std_base)");
  tcache_.clear();
  const int first = static_cast<int>(vars_.size());
  for (int c = 0; c < 3; c++) vars_.push_back({bare(name), comps[c], 3, c});
  nbr_unknowns_ = -1;
  return first;
}

int System::add_cst_vector(const std::string& name, Field* const comps[3]) {
  if (name.find('_') != std::string::npos || name.find('^') != std::string::npos)
    throw KdError(KD_ERR_ARG, "No indices allowed in names of constants");
  tcache_.clear();
  const int first = static_cast<int>(csts_.size());
  for (int c = 0; c < 3; c++) csts_.push_back({bare(name), true, 0.0, comps[c], 3, c});
  return first;
}

void System::set_metric_flat(const std::string& name) {
  const std::string n = bare(name);
  if (n.empty() || n.find('_') != std::string::npos || n.find('^') != std::string::npos)
    throw KdError(KD_ERR_ARG, "bad name for the metric");
  if (!metric_.empty()) throw KdError(KD_ERR_STATE, "Metric already set for the system");
  tcache_.clear();
  metric_ = n;
}

int System::add_var_double(const std::string& name, double value) {
  tcache_.clear();  // a new symbol changes the trees that can follow
  vdoubles_.push_back({bare(name), value});
  nbr_unknowns_ = -1;
  return static_cast<int>(vdoubles_.size()) - 1;
}

int System::add_cst(const std::string& name, double value) {
  tcache_.clear();  // a new symbol changes the trees that can follow
  csts_.push_back({bare(name), false, value, nullptr});
  return static_cast<int>(csts_.size()) - 1;
}

int System::add_cst_field(const std::string& name, Field* f) {
  tcache_.clear();  // a new symbol changes the trees that can follow
  csts_.push_back({bare(name), true, 0.0, f});
  return static_cast<int>(csts_.size()) - 1;
}

void System::add_def(int dom, const std::string& text) {
  std::string l, r;
  if (!split_eq(text, l, r)) throw KdError(KD_ERR_ARG, "= needed for definitions");
  if (dom < 0) {
    for (int dd = dom_min; dd <= dom_max; dd++) add_def(dd, text);
    return;
  }
  // "A_ij": the name, then the index letters after '_' / '^' (is_tensor,
  // src/Utilities/name_tools.cpp:187)
  std::string nm = bare(l), idx;
  const size_t p = nm.find_first_of("_^");
  if (p != std::string::npos) {
    for (size_t i = p; i < nm.size(); i++)
      if (nm[i] != '_' && nm[i] != '^') idx.push_back(nm[i]);
    nm = nm.substr(0, p);
    for (size_t i = 0; i < idx.size(); i++)
      if (idx.find(idx[i], i + 1) != std::string::npos)
        throw KdError(KD_ERR_ARG, "repeated index on the left of a definition");
  }
  DefInfo df{nm, dom, parse_ope(*this, dom, r, -1), idx};
  tcache_.clear();  // a new symbol changes the trees that can follow
  defs_.push_back(df);
}

void System::add_eq_inside(int dom, const std::string& text) {
  std::string l, r;
  if (!split_eq(text, l, r)) throw KdError(KD_ERR_ARG, "= needed for equations");
  Equation eq;
  eq.kind = Equation::INSIDE;
  eq.dom = dom;
  eq.order = 2;
  eq.text = text;
  eq.lhs = (bare(r) == "0") ? parse_ope(*this, dom, l, -1)
                            : std::make_shared<OpeSubEq>(dom, parse_ope(*this, dom, l, -1), parse_ope(*this, dom, r, -1));
  mark_tangent_frontier(eq.lhs.get());
  if (eq.rhs) mark_tangent_frontier(eq.rhs.get());
  tcache_.clear();
  eqs_.push_back(eq);
  nbr_conditions_ = -1;
}

void System::add_eq_bc(int dom, int bound, const std::string& text) {
  std::string l, r;
  if (!split_eq(text, l, r)) throw KdError(KD_ERR_ARG, "= needed for equations");
  if (!sp->dom(dom).has_boundary(bound)) throw KdError(KD_ERR_ARG, "domain has no such boundary");
  Equation eq;
  eq.kind = Equation::BC;
  eq.dom = dom;
  eq.bound = bound;
  eq.text = text;
  eq.lhs = (bare(r) == "0") ? parse_ope(*this, dom, l, bound)
                            : std::make_shared<OpeSubEq>(dom, parse_ope(*this, dom, l, bound),
                                                         parse_ope(*this, dom, r, bound));
  mark_tangent_frontier(eq.lhs.get());
  if (eq.rhs) mark_tangent_frontier(eq.rhs.get());
  tcache_.clear();
  eqs_.push_back(eq);
  nbr_conditions_ = -1;
}

void System::add_eq_matching(int dom, int bound, const std::string& text) {
  Equation eq;
  eq.kind = Equation::MATCHING;
  eq.dom = dom;
  eq.bound = bound;
  eq.text = text;
  sp->dom(dom).find_other_dom(dom, bound, eq.other_dom, eq.other_bound);
  if (eq.other_dom < dom_min || eq.other_dom > dom_max) throw KdError(KD_ERR_ARG, "matching outside the system");
  std::string l, r;
  if (split_eq(text, l, r)) {
    eq.lhs = parse_ope(*this, dom, l, bound);
    eq.rhs = parse_ope(*this, eq.other_dom, r, eq.other_bound);
  } else {
    eq.lhs = parse_ope(*this, dom, text, bound);
    eq.rhs = parse_ope(*this, eq.other_dom, text, eq.other_bound);
  }
  mark_tangent_frontier(eq.lhs.get());
  if (eq.rhs) mark_tangent_frontier(eq.rhs.get());
  tcache_.clear();
  eqs_.push_back(eq);
  nbr_conditions_ = -1;
}

void System::add_eq_order(int dom, int order, const std::string& text) {
  if (order < 0 || order > 2) throw KdError(KD_ERR_ARG, "order of an equation must be 0, 1 or 2");
  std::string l, r;
  if (!split_eq(text, l, r)) throw KdError(KD_ERR_ARG, "= needed for equations");
  Equation eq;
  eq.kind = Equation::INSIDE;
  eq.dom = dom;
  eq.order = order;
  eq.text = text;
  eq.lhs = (bare(r) == "0") ? parse_ope(*this, dom, l, -1)
                            : std::make_shared<OpeSubEq>(dom, parse_ope(*this, dom, l, -1), parse_ope(*this, dom, r, -1));
  mark_tangent_frontier(eq.lhs.get());
  tcache_.clear();
  eqs_.push_back(eq);
  nbr_conditions_ = -1;
}

void System::add_eq_first_integral(int dmin, int dmax, const std::string& integ_part, const std::string& cst_part) {
  if (dmin < dom_min || dmax > dom_max || dmin > dmax) throw KdError(KD_ERR_ARG, "bad domains for a first integral");
  Equation eq;
  eq.kind = Equation::FIRST_INTEGRAL;
  eq.dom = dmin;
  eq.other_dom = dmax;
  eq.text = integ_part;
  eq.parts.push_back(parse_ope(*this, dmin, cst_part, -1));
  for (int d = dmin; d <= dmax; d++) eq.parts.push_back(parse_ope(*this, d, integ_part, -1));
  for (auto& p : eq.parts) mark_tangent_frontier(p.get());
  tcache_.clear();
  eqs_.push_back(eq);
  nbr_conditions_ = -1;
}

void System::add_int_equation(IntEquation ie) {
  for (auto& p : ie.parts) mark_tangent_frontier(p.get());
  tcache_.clear();
  ieqs_.push_back(std::move(ie));
  nbr_conditions_ = -1;
}

void System::add_eq_int_volume(int dmin, int dmax, const std::string& text) {
  std::string l, r;
  if (!split_eq(text, l, r)) throw KdError(KD_ERR_ARG, "= needed for equations");
  if (dmin < 0 || dmax >= sp->ndom() || dmin > dmax) throw KdError(KD_ERR_ARG, "bad domain range for the integral");
  IntEquation ie;
  ie.text = text;
  for (int d = dmin; d <= dmax; d++) ie.parts.push_back(parse_ope(*this, d, l, -1));
  // the constant side, as Ope_minus(give_ope(...)) in the first domain
  ie.parts.push_back(std::make_shared<OpeMinusPart>(dmin, parse_ope(*this, dmin, r, -1)));
  add_int_equation(std::move(ie));
}

void System::add_eq_int_inf(const std::string& text) {
  std::string l, r;
  if (!split_eq(text, l, r)) throw KdError(KD_ERR_ARG, "= needed for equations");
  const int last = sp->ndom() - 1;
  if (sp->dom(last).type != DOM_COMPACT) throw KdError(KD_ERR_ARG, "integral at infinity needs a compactified domain");
  IntEquation ie;
  ie.text = text;
  ie.parts.push_back(parse_ope(*this, last, l, OUTER_BC));
  ie.parts.push_back(std::make_shared<OpeMinusPart>(last, parse_ope(*this, last, r, OUTER_BC)));
  add_int_equation(std::move(ie));
}

void System::add_eq_val(int dom, const std::string& text, const int pos[3]) {
  if (dom < 0 || dom >= sp->ndom()) throw KdError(KD_ERR_ARG, "bad domain");
  const Domain& d = sp->dom(dom);
  for (int i = 0; i < 3; i++)
    if (pos[i] < 0 || pos[i] >= d.np[i]) throw KdError(KD_ERR_ARG, "add_eq_val: collocation index out of range");
  IntEquation ie;
  ie.text = text;
  ie.parts.push_back(make_value_at(dom, parse_ope(*this, dom, text, -1), pos));
  add_int_equation(std::move(ie));
}

void System::add_eq_point(int dom, const std::string& text, const double point[3]) {
  if (dom < 0 || dom >= sp->ndom()) throw KdError(KD_ERR_ARG, "bad domain");
  double num[3];
  sp->absol_to_num(dom, point, num);
  IntEquation ie;
  ie.text = text;
  ie.parts.push_back(make_value_at_point(dom, parse_ope(*this, dom, text, -1), num));
  add_int_equation(std::move(ie));
}

void System::export_int_ders(EvalState& st, int dom, double* out, long long osf, int B) {
  static const std::vector<int> rp = {0, 1}, one_idx = {0};
  static const std::vector<double> one_w = {1.0};
  for (auto& ie : ieqs_)
    for (auto& p : ie.parts) {
      if (dom >= 0 && p->dom != dom) continue;
      Term t = p->eval(st);
      if (!t.is_double) throw KdError(KD_ERR_STATE, "an integral equation's part is not a number: " + ie.text);
      if (!t.has_dd) continue;
      const double* v = t.ddv;
      if (!v) {
        if (t.dd == 0.0) continue;
        double* tmp = ctx->scratch().alloc_doubles(B);
        cuda_check(launch_lincomb2(B, 1.0, nullptr, t.dd, 0.0, nullptr, 0.0, tmp, ctx->stream()), "constant tangent");
        ctx->launches++;
        v = tmp;
      } else if (t.ddb != B) {
        throw KdError(KD_ERR_STATE, "integral tangent of another batch size");
      }
      // out[row + b * osf] += v[b]
      cuda_check(launch_gather_csr(v, 1, B, 1, ctx->table(rp), ctx->table(one_idx), ctx->dtable(one_w), out + ie.row,
                                   osf, 0, 1.0, 1, ctx->stream()),
                 "integral row");
      ctx->launches++;
    }
}

CsrTable System::upload_rows(const std::vector<SparseRow>& rows) {
  std::vector<int> rp(rows.size() + 1, 0), idx;
  std::vector<double> w;
  for (size_t r = 0; r < rows.size(); r++) {
    for (auto& e : rows[r].e) {
      idx.push_back(e.first);
      w.push_back(e.second);
    }
    rp[r + 1] = static_cast<int>(idx.size());
  }
  CsrTable t;
  t.rowptr = ctx->table(rp);
  t.idx = ctx->table(idx);
  t.w = ctx->dtable(w);
  t.nrows = static_cast<int>(rows.size());
  t.nnz = static_cast<long long>(idx.size());
  return t;
}

const CsrTable& System::export_table(const Domain& d, const Base& b, int kind, int arg) {
  std::vector<int> key = {d.num, kind, arg, b.p};
  key.insert(key.end(), b.t.begin(), b.t.end());
  key.insert(key.end(), b.r.begin(), b.r.end());
  auto it = tables_.find(key);
  if (it != tables_.end()) return it->second;
  std::vector<SparseRow> rows;
  if (kind == 0) d.export_tau_rows(b, 0, arg, rows);
  else d.export_tau_boundary_rows(b, 0, arg, rows);
  tables_[key] = upload_rows(rows);
  return tables_[key];
}

int System::count_rows(const Equation& eq, const Term& t) {
  if (t.is_double) throw KdError(KD_ERR_UNSUPPORTED, "equation residual must be a field");
  int n = 0;
  const Domain& d = sp->dom(eq.dom);
  for (auto& v : t.vt) {
    if (!v.base.def) throw KdError(KD_ERR_STATE, "residual without a defined basis: " + eq.text);
    const CsrTable& tab = (eq.kind == Equation::INSIDE) ? export_table(d, v.base, 0, eq.order)
                                                        : export_table(d, v.base, 1, eq.bound);
    n += tab.nrows;
  }
  return n;
}

// Writes the export rows of every component of t (value or tangent).
void System::export_term(const Equation& eq, const Term& t, bool der, int side_dom, int side_bound, double* out,
                         long long osf, long long osr, int batch, double alpha, bool accumulate) {
  const Domain& d = sp->dom(side_dom);
  const auto& comps = der ? t.dt : t.vt;
  if (t.is_double) throw KdError(KD_ERR_UNSUPPORTED, "equation residual must be a field: " + eq.text);
  // The rows written must be exactly the rows the equation owns: a residual
  // whose basis changed since the first evaluation would overflow its block.
  if (eq.n_cond >= 0) {
    long long total = 0;
    for (size_t c = 0; c < t.vt.size(); c++) {
      const Base& bv = t.vt[c].base;
      if (!bv.def) throw KdError(KD_ERR_STATE, "residual without a defined basis: " + eq.text);
      total += (eq.kind == Equation::INSIDE) ? export_table(d, bv, 0, eq.order).nrows
                                             : export_table(d, bv, 1, side_bound).nrows;
    }
    if (total != eq.n_cond)
      throw KdError(KD_ERR_STATE, "the basis of the residual changed the number of conditions of: " + eq.text);
  }
  long long row = 0;
  for (size_t c = 0; c < comps.size(); c++) {
    const DVal& v = comps[c];
    // rows of this component are fixed by the value's basis (n_cond)
    const Base& bval = t.vt[c].base;
    const CsrTable& tv = (eq.kind == Equation::INSIDE) ? export_table(d, bval, 0, eq.order)
                                                       : export_table(d, bval, 1, side_bound);
    if (!v.zero) {
      if (!v.base.def) throw KdError(KD_ERR_STATE, "exported field without basis: " + eq.text);
      v.coef();
      const CsrTable& tab = (eq.kind == Equation::INSIDE) ? export_table(d, v.base, 0, eq.order)
                                                          : export_table(d, v.base, 1, side_bound);
      if (tab.nrows != tv.nrows) throw KdError(KD_ERR_STATE, "tangent basis changes the number of conditions");
      long long in_stride = (v.batch == 1 && batch > 1) ? 0 : v.ncoefs();
      ProfScope ps(ctx, Context::PROF_GATHER, 8.0 * batch * (tab.nnz + 2.0 * tab.nrows));
      cuda_check(launch_gather_csr(v.cf, in_stride, batch, tab.nrows, tab.rowptr, tab.idx, tab.w, out + row * osr,
                                   osf, osr, alpha, accumulate ? 1 : 0, ctx->stream()),
                 "export gather");
      ctx->launches++;
    }
    row += tv.nrows;
  }
}

std::vector<Term> System::eval_parts(const Equation& eq, EvalState& st) {
  std::vector<Term> t;
  for (auto& p : eq.parts) t.push_back(p->eval(st));
  return t;
}

int System::count_rows_fi(Equation& eq, const std::vector<Term>& parts) {
  eq.n_cond_dom.clear();
  int n = 0;
  for (int d = eq.dom; d <= eq.other_dom; d++) {
    const Term& t = parts[1 + d - eq.dom];
    if (t.is_double || t.vt.size() != 1) throw KdError(KD_ERR_UNSUPPORTED, "a first integral must be a scalar field");
    if (!t.vt[0].base.def) throw KdError(KD_ERR_STATE, "first integral without a defined basis: " + eq.text);
    const int r = export_table(sp->dom(d), t.vt[0].base, 0, 0).nrows;
    eq.n_cond_dom.push_back(r);
    n += r;
  }
  return n;
}

// Eq_first_integral::export_val / export_der (eq_first_integral.cpp:44-120):
// in every domain the first integral minus its value at the first
// collocation point of dom_min; in dom_min the radial-index-0 points carry
// the constant part's value at that point; all coefficients exported.
void System::export_first_integral(const Equation& eq, const std::vector<Term>& parts, bool der, double* out,
                                   long long osf, long long osr, int batch, bool accumulate) {
  const Term& cst = parts[0];
  const int dmin = eq.dom;
  auto comp = [&](const Term& t) -> const DVal& { return der ? t.dt[0] : t.vt[0]; };
  const DVal& vmin = comp(parts[1]);
  const Domain& dm0 = sp->dom(dmin);
  const double* ori = nullptr;
  long long os = 0;
  if (!vmin.zero) {
    vmin.coef_i();
    ori = vmin.c;
    os = (vmin.batch == 1) ? 0 : dm0.npts();
  }
  const double* cstp = nullptr;
  long long cs = 0;
  double cst_scalar = 0.0;
  if (cst.is_double) {
    if (der) {
      if (cst.ddv) throw KdError(KD_ERR_UNSUPPORTED, "first integral: a seeded number as constant part");
      cst_scalar = cst.has_dd ? cst.dd : 0.0;
    } else {
      cst_scalar = cst.vd;
    }
  } else {
    if (cst.vt.size() != 1 || cst.vt[0].dom != &dm0)
      throw KdError(KD_ERR_UNSUPPORTED, "first integral: the constant part must be a scalar of the first domain");
    const DVal& c = comp(cst);
    if (!c.zero) {
      c.coef_i();
      cstp = c.c;
      cs = (c.batch == 1) ? 0 : dm0.npts();
    }
  }
  long long row = 0;
  for (int d = dmin; d <= eq.other_dom; d++) {
    const Term& t = parts[1 + d - dmin];
    const Domain& dm = sp->dom(d);
    const DVal& v = comp(t);
    const bool inject = (d == dmin);
    const long long nrows = eq.n_cond_dom.at(d - dmin);
    if (v.zero && !ori && !(inject && (cstp || cst_scalar != 0.0))) {
      row += nrows;
      continue;
    }
    const double* vp = nullptr;
    long long vs = 0;
    if (!v.zero) {
      v.coef_i();
      vp = v.c;
      vs = (v.batch == 1) ? 0 : dm.npts();
    }
    double* w = ctx->scratch().alloc_doubles(static_cast<long long>(batch) * dm.npts());
    cuda_check(launch_first_integral(batch, dm.npts(), dm.np[1] * dm.np[2], vp, vs, ori, os, inject ? 1 : 0, cstp, cs,
                                     cst_scalar, w, ctx->stream()),
               "first integral");
    ctx->launches++;
    const Base& base = (!v.zero && v.base.def) ? v.base : t.vt[0].base;
    DVal wd(ctx, &dm, batch);
    wd.zero = false;
    wd.c = w;
    wd.in_conf = true;
    wd.base = base;
    wd.coef();
    const CsrTable& tab = export_table(dm, base, 0, 0);
    if (tab.nrows != nrows) throw KdError(KD_ERR_STATE, "the basis of the first integral changed its conditions");
    ProfScope ps(ctx, Context::PROF_GATHER, 8.0 * batch * (tab.nnz + 2.0 * tab.nrows));
    cuda_check(launch_gather_csr(wd.cf, dm.ncoefs(), batch, tab.nrows, tab.rowptr, tab.idx, tab.w, out + row * osr, osf,
                                 osr, 1.0, accumulate ? 1 : 0, ctx->stream()),
               "first integral gather");
    ctx->launches++;
    row += nrows;
  }
}

void System::export_tangent(Equation& eq, EvalState& st, double* out, long long osf, int batch) {
  if (eq.kind == Equation::FIRST_INTEGRAL) {
    std::vector<Term> parts = eval_parts(eq, st);
    export_first_integral(eq, parts, true, out + eq.row0, osf, 1, batch, true);
    return;
  }
  Term t = eq.lhs->eval(st);
  export_term(eq, t, true, eq.dom, eq.bound, out + eq.row0, osf, 1, batch, 1.0, true);
  if (eq.kind == Equation::MATCHING) {
    Term r = eq.rhs->eval(st);
    export_term(eq, r, true, eq.other_dom, eq.other_bound, out + eq.row0, osf, 1, batch, -1.0, true);
  }
}

void System::compute_unknowns() {
  col0_.clear();
  nunk_.clear();
  int n = static_cast<int>(vdoubles_.size());
  // xx_to_vars (system_of_eqs.cpp:597): variable by variable, domain by
  // domain; a vector's components are consecutive inside each domain
  for (size_t v = 0; v < vars_.size(); v += vars_[v].ncmp)
    for (int dd = dom_min; dd <= dom_max; dd++)
      for (int c = 0; c < vars_[v].ncmp; c++) {
        const int w = static_cast<int>(v) + c;
        std::vector<SparseRow> pats;
        sp->dom(dd).unknown_patterns(vars_[w].f->d[dd].base, 0, pats);
        col0_[{w, dd}] = n;
        nunk_[{w, dd}] = static_cast<int>(pats.size());
        n += static_cast<int>(pats.size());
      }
  nbr_unknowns_ = n;
}

int System::nbr_unknowns() {
  if (nbr_unknowns_ < 0) compute_unknowns();
  return nbr_unknowns_;
}

void System::residual(double* d_F, bool record) {
  const bool graphable = graph_on_ && !graph_failed_ && record && d_F && nbr_conditions_ >= 0 && ieqs_.empty() &&
                         !ctx->prof_on() && !ctx->capturing;
  if (!graphable) {
    residual_pass(d_F, record);
    return;
  }
  std::vector<long long> sig = state_signature();
  cudaStream_t main = ctx->main_stream();
  graph_clock_++;
  for (auto& g : graphs_)
    if (g.F == d_F && g.sig == sig) {
      // the node values the Jacobian reads: the captured pass's (host
      // side), refilled on the device by the replay
      vcache_.vals = g.vals;
      vcache_.arena.release_to(g.mark);
      vcache_.valid = true;
      ctx->scratch().reset();
      cuda_check(cudaGraphLaunch(g.exec, main), "replay value pass");
      ctx->launches += g.launches;
      g.last_use = graph_clock_;
      residual_graph_replays++;
      return;
    }
  // a state met for the first time runs as it is (it also sizes the arenas
  // and uploads the tables); the second time it is captured
  if (std::find(seen_sigs_.begin(), seen_sigs_.end(), sig) == seen_sigs_.end()) {
    if (seen_sigs_.size() >= 16) seen_sigs_.erase(seen_sigs_.begin());
    seen_sigs_.push_back(sig);
    residual_pass(d_F, record);
    return;
  }
  cudaGraph_t graph = nullptr;
  cuda_check(cudaStreamBeginCapture(main, cudaStreamCaptureModeThreadLocal), "begin capture");
  ctx->capturing = true;
  const long long l0 = ctx->launches;
  try {
    residual_pass(d_F, true);
  } catch (...) {
    ctx->capturing = false;
    cudaStreamEndCapture(main, &graph);
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    graph_failed_ = true;  // something in the pass cannot be captured
    residual_pass(d_F, record);
    return;
  }
  ctx->capturing = false;
  cuda_check(cudaStreamEndCapture(main, &graph), "end capture");
  cudaGraphExec_t exec = nullptr;
  const cudaError_t st = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (st != cudaSuccess) {
    cudaGetLastError();
    graph_failed_ = true;
    residual_pass(d_F, record);
    return;
  }
  if (graphs_.size() >= 4) {
    auto lru = std::min_element(graphs_.begin(), graphs_.end(),
                                [](const ValueGraph& a, const ValueGraph& b) { return a.last_use < b.last_use; });
    cudaGraphExecDestroy(lru->exec);
    graphs_.erase(lru);
  }
  ValueGraph g;
  g.sig = std::move(sig);
  g.exec = exec;
  g.F = d_F;
  g.launches = ctx->launches - l0;
  for (const auto& kv : vcache_.vals) {
    Term t = kv.second;
    for (auto& v : t.vt) v = v.plain();
    g.vals.emplace(kv.first, std::move(t));
  }
  g.mark = vcache_.arena.mark();
  g.last_use = graph_clock_;
  residual_graph_captures++;
  // the capture ran nothing: the pass itself is the first replay
  ctx->launches = l0 + g.launches;
  vcache_.vals = g.vals;
  cuda_check(cudaGraphLaunch(g.exec, main), "replay value pass");
  graphs_.push_back(std::move(g));
}

void System::residual_pass(double* d_F, bool record) {
  ctx->scratch().reset();
  vcache_.clear();
  std::unique_ptr<ScratchRedirect> redirect;
  if (record) redirect = std::make_unique<ScratchRedirect>(ctx, &vcache_.arena);
  EvalState st;
  st.sys = this;
  st.with_der = false;
  st.vcache = record ? &vcache_ : nullptr;
  st.record = record;
  std::vector<Term> lhs(eqs_.size()), rhs(eqs_.size());
  std::vector<std::vector<Term>> fparts(eqs_.size());
  if (d_F && nbr_conditions_ >= 0)
    cuda_check(cudaMemsetAsync(d_F, 0, sizeof(double) * nbr_conditions_, ctx->main_stream()), "memset F");
  // The equations of different domains are independent (fields are only
  // read, temporaries come from the pass's arena): one side stream per
  // domain, so that their small kernels overlap on the GPU.
  struct Fork {
    Context* c;
    Fork(Context* c_, int n) : c(c_) { c->fork(n); }
    ~Fork() { c->join(); }
  } fork(ctx, ndom() < 8 ? ndom() : 8);
  auto stream_of = [&](const Equation& eq) { return eq.dom - dom_min; };
  // integral equations: sums of numbers, on the main stream
  std::vector<double> ivals(ieqs_.size(), 0.0);
  ctx->use(-1);
  for (size_t i = 0; i < ieqs_.size(); i++) {
    double v = 0.0;
    for (auto& p : ieqs_[i].parts) {
      Term t = p->eval(st);
      if (!t.is_double) throw KdError(KD_ERR_STATE, "an integral equation's part is not a number: " + ieqs_[i].text);
      v += t.vd;
    }
    ivals[i] = v;
  }
  for (size_t i = 0; i < eqs_.size(); i++) {
    ctx->use(stream_of(eqs_[i]));
    if (eqs_[i].kind == Equation::FIRST_INTEGRAL) {
      fparts[i] = eval_parts(eqs_[i], st);
      continue;
    }
    lhs[i] = eqs_[i].lhs->eval(st);
    if (eqs_[i].kind == Equation::MATCHING) rhs[i] = eqs_[i].rhs->eval(st);
  }
  vcache_.valid = record;
  if (nbr_conditions_ < 0) {
    int row = 0;
    for (auto& ie : ieqs_) ie.row = row++;
    for (size_t i = 0; i < eqs_.size(); i++) {
      eqs_[i].n_cond = (eqs_[i].kind == Equation::FIRST_INTEGRAL) ? count_rows_fi(eqs_[i], fparts[i])
                                                                  : count_rows(eqs_[i], lhs[i]);
      eqs_[i].row0 = row;
      row += eqs_[i].n_cond;
    }
    nbr_conditions_ = row;
    if (d_F) {
      ctx->use(-1);
      cuda_check(cudaMemsetAsync(d_F, 0, sizeof(double) * nbr_conditions_, ctx->main_stream()), "memset F");
      ctx->join();
      ctx->fork(ndom() < 8 ? ndom() : 8);
    }
  }
  if (!d_F) return;
  if (!ivals.empty()) {
    ctx->use(-1);
    cuda_check(cudaMemcpyAsync(d_F, ivals.data(), sizeof(double) * ivals.size(), cudaMemcpyHostToDevice,
                               ctx->main_stream()),
               "integral rows");
  }
  for (size_t i = 0; i < eqs_.size(); i++) {
    Equation& eq = eqs_[i];
    ctx->use(stream_of(eq));
    double* out = d_F + eq.row0;
    if (eq.kind == Equation::FIRST_INTEGRAL) {
      export_first_integral(eq, fparts[i], false, out, 0, 1, 1, false);
    } else if (eq.kind == Equation::MATCHING) {
      export_term(eq, lhs[i], false, eq.dom, eq.bound, out, 0, 1, 1, 1.0, false);
      export_term(eq, rhs[i], false, eq.other_dom, eq.other_bound, out, 0, 1, 1, -1.0, true);
    } else {
      export_term(eq, lhs[i], false, eq.dom, eq.bound, out, 0, 1, 1, 1.0, false);
    }
  }
}

const double* System::seed_block(int var, int dom, int& B, Base& base) {
  base = vars_[var].f->d[dom].base;
  std::vector<SparseRow> pats;
  const Domain& d = sp->dom(dom);
  d.unknown_patterns(base, 0, pats);
  B = static_cast<int>(pats.size());
  auto key = std::make_pair(var, dom);
  auto it = seeds_.find(key);
  if (it != seeds_.end()) return it->second;
  std::vector<double> block(static_cast<size_t>(B) * d.ncoefs(), 0.0);
  for (int s = 0; s < B; s++)
    for (auto& e : pats[s].e) block[static_cast<size_t>(s) * d.ncoefs() + e.first] = e.second;
  const double* p = ctx->dtable(block);
  seeds_[key] = p;
  return p;
}

// What a Jacobian pass's launches depend on besides the fields' data: the
// state of the value pass (which representations, bases and numbers; the
// node values' device addresses), the output, and the tangent cache's
// contents (which subtrees are skipped) and arena position.
std::vector<long long> System::jacobian_signature(const double* d_J, long long ld, bool rectangular) const {
  std::vector<long long> g = state_signature();
  g.push_back(reinterpret_cast<long long>(d_J));
  g.push_back(ld);
  g.push_back(rectangular ? 1 : 0);
  g.push_back(cache_tangents_ ? 1 : 0);
  g.push_back(static_cast<long long>(tcache_.ders.size()));
  g.push_back(static_cast<long long>(tcache_.arena.mark()));
  g.push_back(static_cast<long long>(vcache_.arena.mark()));
  g.push_back(static_cast<long long>(vcache_.vals.size()));
  // node values: an order-independent sum of per-node hashes
  auto mix = [](unsigned long long x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
  };
  unsigned long long h = 0;
  for (const auto& kv : vcache_.vals) {
    unsigned long long e = mix(reinterpret_cast<unsigned long long>(kv.first));
    unsigned long long vb;
    std::memcpy(&vb, &kv.second.vd, sizeof vb);
    e = mix(e ^ vb);
    for (const auto& d : kv.second.vt) {
      e = mix(e ^ reinterpret_cast<unsigned long long>(d.c));
      e = mix(e ^ reinterpret_cast<unsigned long long>(d.cf));
    }
    h += e;
  }
  g.push_back(static_cast<long long>(h));
  return g;
}

void System::jacobian(double* d_J, long long ld, bool reuse, bool rectangular) {
  int N = nbr_unknowns();
  if (!reuse || !vcache_.valid) residual(nullptr, true);
  if (rectangular ? (nbr_conditions_ < N || ld < nbr_conditions_) : (nbr_conditions_ != N)) {
    std::ostringstream os;
    os << "Number of unknowns (" << N << ") is different from the number of equations (" << nbr_conditions_ << ")";
    throw KdError(KD_ERR_STATE, os.str());
  }
  const bool graphable = graph_on_ && !jgraph_failed_ && ieqs_.empty() && vdoubles_.empty() && !ctx->prof_on() &&
                         !ctx->capturing;
  if (!graphable) {
    jacobian_pass(d_J, ld);
    return;
  }
  std::vector<long long> sig = jacobian_signature(d_J, ld, rectangular);
  cudaStream_t main = ctx->main_stream();
  graph_clock_++;
  for (auto& g : jgraphs_)
    if (g.sig == sig) {
      tcache_.ders = g.tders;
      tcache_.arena.release_to(g.tmark);
      ctx->scratch().reset();
      cuda_check(cudaGraphLaunch(g.exec, main), "replay Jacobian pass");
      ctx->launches += g.launches;
      g.last_use = graph_clock_;
      jacobian_graph_replays++;
      return;
    }
  // first time: as it is (it also sizes the arenas and uploads the seeds
  // and tables); second time: captured
  if (std::find(jseen_.begin(), jseen_.end(), sig) == jseen_.end()) {
    if (jseen_.size() >= 16) jseen_.erase(jseen_.begin());
    jseen_.push_back(sig);
    jacobian_pass(d_J, ld);
    return;
  }
  const auto tders0 = tcache_.ders;
  const size_t tmark0 = tcache_.arena.mark();
  auto fall_back = [&] {
    cudaGetLastError();
    jgraph_failed_ = true;  // something in the pass cannot be captured
    tcache_.ders = tders0;
    tcache_.arena.release_to(tmark0);
    jacobian_pass(d_J, ld);
  };
  cudaGraph_t graph = nullptr;
  cuda_check(cudaStreamBeginCapture(main, cudaStreamCaptureModeThreadLocal), "begin capture");
  ctx->capturing = true;
  const long long l0 = ctx->launches;
  try {
    jacobian_pass(d_J, ld);
  } catch (...) {
    ctx->capturing = false;
    cudaStreamEndCapture(main, &graph);
    if (graph) cudaGraphDestroy(graph);
    fall_back();
    return;
  }
  ctx->capturing = false;
  if (cudaStreamEndCapture(main, &graph) != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    fall_back();
    return;
  }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t st = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (st != cudaSuccess) {
    fall_back();
    return;
  }
  if (jgraphs_.size() >= 4) {
    auto lru = std::min_element(jgraphs_.begin(), jgraphs_.end(),
                                [](const JacGraph& a, const JacGraph& b) { return a.last_use < b.last_use; });
    cudaGraphExecDestroy(lru->exec);
    jgraphs_.erase(lru);
  }
  JacGraph g;
  g.sig = std::move(sig);
  g.exec = exec;
  g.launches = ctx->launches - l0;
  g.tders = tcache_.ders;
  g.tmark = tcache_.arena.mark();
  g.last_use = graph_clock_;
  jacobian_graph_captures++;
  // the capture ran nothing: the pass itself is the first replay
  cuda_check(cudaGraphLaunch(g.exec, main), "replay Jacobian pass");
  jgraphs_.push_back(std::move(g));
}

void System::jacobian_pass(double* d_J, long long ld) {
  const int N = nbr_unknowns();
  cuda_check(cudaMemsetAsync(d_J, 0, sizeof(double) * ld * N, ctx->stream()), "memset J");
  // Columns of the double unknowns (do_col_J with is_var_double): one pass
  // each with that unknown's tangent 1, every field's 0, all equations.
  if (!vdoubles_.empty()) {
    const std::map<std::pair<int, int>, DVal> none;
    for (size_t i = 0; i < vdoubles_.size(); i++) {
      ctx->scratch().reset();
      std::vector<double> e(vdoubles_.size(), 0.0);
      e[i] = 1.0;
      EvalState st;
      st.sys = this;
      st.with_der = true;
      st.B = 1;
      st.jx_seeds = &none;
      st.jx_doubles = &e;
      st.seed_var_double = static_cast<int>(i);
      st.vcache = &vcache_;
      double* Jcol = d_J + static_cast<long long>(i) * ld;
      for (auto& eq : eqs_) export_tangent(eq, st, Jcol, ld, 1);
      export_int_ders(st, -1, Jcol, ld, 1);
    }
  }
  // Seed blocks write disjoint column blocks: a wave of them runs on side
  // streams; the scratch arena is reset only between waves.
  std::vector<std::pair<int, int>> blocks;
  for (size_t v = 0; v < vars_.size(); v++)
    for (int dd = dom_min; dd <= dom_max; dd++) blocks.emplace_back(static_cast<int>(v), dd);
  const int wave = 6;
  for (size_t w0 = 0; w0 < blocks.size(); w0 += wave) {
    ctx->scratch().reset();
    struct Fork {
      Context* c;
      Fork(Context* c_, int n) : c(c_) { c->fork(n); }
      ~Fork() { c->join(); }
    } fork(ctx, wave);
    for (size_t bix = w0; bix < blocks.size() && bix < w0 + wave; bix++) {
      const int v = blocks[bix].first, dd = blocks[bix].second;
      ctx->use(static_cast<int>(bix - w0));
      int B;
      Base base;
      const double* seeds = seed_block(static_cast<int>(v), dd, B, base);
      if (B == 0) continue;
      EvalState st;
      st.sys = this;
      st.with_der = true;
      st.B = B;
      st.seed_var = static_cast<int>(v);
      st.seed_dom = dd;
      st.seed = DVal::from_coef(ctx, &sp->dom(dd), B, seeds, base);
      st.vcache = &vcache_;
      st.tcache = cache_tangents_ ? &tcache_ : nullptr;
      int col0 = col0_[{static_cast<int>(v), dd}];
      double* Jblock = d_J + static_cast<long long>(col0) * ld;
      for (auto& eq : eqs_) {
        if (!eq.take_into_account(dd)) continue;
        if (eq.kind == Equation::FIRST_INTEGRAL) {
          std::vector<Term> parts = eval_parts(eq, st);
          export_first_integral(eq, parts, true, Jblock + eq.row0, ld, 1, B, true);
          continue;
        }
        if (eq.kind != Equation::MATCHING || dd == eq.dom) {
          Term t = eq.lhs->eval(st);
          export_term(eq, t, true, eq.dom, eq.bound, Jblock + eq.row0, ld, 1, B, 1.0, true);
        }
        if (eq.kind == Equation::MATCHING && dd == eq.other_dom) {
          Term t = eq.rhs->eval(st);
          export_term(eq, t, true, eq.other_dom, eq.other_bound, Jblock + eq.row0, ld, 1, B, -1.0, true);
        }
      }
      export_int_ders(st, dd, Jblock, ld, B);
    }
  }
}

// x -> coefficient map of one (variable, domain): affecte_tau
// (domain_*_affecte_tau.cpp), as a CSR table.
const CsrTable& System::xmap(int var, int dd) {
  auto key = std::make_pair(var, dd);
  auto it = xmaps_.find(key);
  if (it != xmaps_.end()) return it->second;
  std::vector<SparseRow> rows;
  const Domain& d = sp->dom(dd);
  int used = d.affecte_tau_map(vars_[var].f->d[dd].base, 0, rows);
  if (used != nunk_[key]) throw KdError(KD_ERR_STATE, "affecte_tau consumes a different number of unknowns");
  xmaps_[key] = upload_rows(rows);
  return xmaps_[key];
}

void System::add_ope_eos(const std::string& name, int var, const KdEos& eos) {
  if (var < EOS_EPSILON || var > EOS_DHDRHO) throw KdError(KD_ERR_ARG, "unknown EOS variable");
  tcache_.clear();
  user_opes_.push_back({name, eos, var});
}

void System::set_cst(int i, double v) {
  if (csts_.at(i).is_field) throw KdError(KD_ERR_ARG, "set_cst: the constant is a field");
  csts_[i].value = v;
  vcache_.clear();
}

void System::dres_dcst(int cst, double* d_y) {
  if (csts_.at(cst).is_field) throw KdError(KD_ERR_UNSUPPORTED, "dF/dp needs a double constant");
  int N = nbr_unknowns();
  residual(nullptr, true);
  if (nbr_conditions_ != N) throw KdError(KD_ERR_STATE, "Number of unknowns is different from the number of equations");
  ctx->scratch().reset();
  const std::map<std::pair<int, int>, DVal> none;
  const std::vector<double> zeros(vdoubles_.size(), 0.0);
  EvalState st;
  st.sys = this;
  st.with_der = true;
  st.B = 1;
  st.jx_seeds = &none;  // no unknown is seeded
  st.jx_doubles = &zeros;
  st.seed_cst = cst;
  st.vcache = &vcache_;
  cuda_check(cudaMemsetAsync(d_y, 0, sizeof(double) * N, ctx->stream()), "memset y");
  for (auto& eq : eqs_) export_tangent(eq, st, d_y, 0, 1);
  export_int_ders(st, -1, d_y, 1, 1);
}

void System::val_point_gradient(int var, const double point[3], double* g) {
  const int N = nbr_unknowns();
  std::fill(g, g + N, 0.0);
  double num[3];
  const int dd = sp->locate(point, num);
  if (dd < 0) throw KdError(KD_ERR_ARG, "val_point: the point is in no domain");
  if (dd < dom_min || dd > dom_max) return;  // the field there does not depend on the unknowns
  const Domain& d = sp->dom(dd);
  std::vector<double> w;
  d.point_weights(vars_.at(var).f->d[dd].base, num, w);
  std::vector<SparseRow> pats;
  d.unknown_patterns(vars_[var].f->d[dd].base, 0, pats);
  const int c0 = col0_.at(std::make_pair(var, dd));
  for (size_t j = 0; j < pats.size(); j++) {
    double s = 0.0;
    for (auto& e : pats[j].e) s += e.second * w[e.first];
    g[c0 + j] = s;
  }
}

double System::integral_gradient(int kind, int dmin, int dmax, const std::string& expr, double* d_g) {
  const int N = nbr_unknowns();
  residual(nullptr, true);  // the unknown layout at the current fields
  std::vector<OpePtr> parts;
  if (kind == 0) {
    if (dmin < 0 || dmax >= sp->ndom() || dmin > dmax) throw KdError(KD_ERR_ARG, "bad domain range for the integral");
    for (int d = dmin; d <= dmax; d++) parts.push_back(parse_ope(*this, d, expr, -1));
  } else if (kind == 1) {
    const int last = sp->ndom() - 1;
    if (sp->dom(last).type != DOM_COMPACT) throw KdError(KD_ERR_ARG, "integral at infinity needs a compactified domain");
    parts.push_back(parse_ope(*this, last, expr, OUTER_BC));
  } else {
    throw KdError(KD_ERR_ARG, "integral kind must be 0 (volume) or 1 (at infinity)");
  }
  static const std::vector<int> rp = {0, 1}, one_idx = {0};
  static const std::vector<double> one_w = {1.0};
  // out[b] += tangent of part b (B numbers, or one constant)
  auto add_tangent = [&](const Term& t, double* out, int B) {
    if (!t.is_double) throw KdError(KD_ERR_STATE, "the integrand does not integrate to a number: " + expr);
    if (!t.has_dd) return;
    const double* v = t.ddv;
    if (!v) {
      if (t.dd == 0.0) return;
      double* tmp = ctx->scratch().alloc_doubles(B);
      cuda_check(launch_lincomb2(B, 1.0, nullptr, t.dd, 0.0, nullptr, 0.0, tmp, ctx->stream()), "constant tangent");
      ctx->launches++;
      v = tmp;
    } else if (t.ddb != B) {
      throw KdError(KD_ERR_STATE, "integral tangent of another batch size");
    }
    cuda_check(launch_gather_csr(v, 1, B, 1, ctx->table(rp), ctx->table(one_idx), ctx->dtable(one_w), out, 1, 0, 1.0,
                                 1, ctx->stream()),
               "integral gradient");
    ctx->launches++;
  };
  ctx->scratch().reset();
  double q = 0.0;
  {
    EvalState st;
    st.sys = this;
    st.with_der = false;
    for (auto& p : parts) {
      Term t = p->eval(st);
      if (!t.is_double) throw KdError(KD_ERR_STATE, "the integrand does not integrate to a number: " + expr);
      q += t.vd;
    }
  }
  cuda_check(cudaMemsetAsync(d_g, 0, sizeof(double) * N, ctx->stream()), "memset gradient");
  // double unknowns: one pass each (their columns come first)
  const std::map<std::pair<int, int>, DVal> none;
  for (size_t i = 0; i < vdoubles_.size(); i++) {
    ctx->scratch().reset();
    std::vector<double> e(vdoubles_.size(), 0.0);
    e[i] = 1.0;
    EvalState st;
    st.sys = this;
    st.with_der = true;
    st.B = 1;
    st.jx_seeds = &none;
    st.jx_doubles = &e;
    st.seed_var_double = static_cast<int>(i);
    for (auto& p : parts) add_tangent(p->eval(st), d_g + i, 1);
  }
  // field unknowns: the seed blocks of the integrand's domains
  for (size_t v = 0; v < vars_.size(); v++)
    for (auto& p : parts) {
      const int dd = p->dom;
      if (dd < dom_min || dd > dom_max) continue;
      ctx->scratch().reset();
      int B;
      Base base;
      const double* seeds = seed_block(static_cast<int>(v), dd, B, base);
      if (B == 0) continue;
      EvalState st;
      st.sys = this;
      st.with_der = true;
      st.B = B;
      st.seed_var = static_cast<int>(v);
      st.seed_dom = dd;
      st.seed = DVal::from_coef(ctx, &sp->dom(dd), B, seeds, base);
      add_tangent(p->eval(st), d_g + col0_[{static_cast<int>(v), dd}], B);
    }
  cuda_check(cudaStreamSynchronize(ctx->stream()), "sync integral gradient");
  return q;
}

DVal System::x_to_field(int var, int dd, const double* d_x) {
  nbr_unknowns();
  const Domain& d = sp->dom(dd);
  const CsrTable& t = xmap(var, dd);
  double* cf = ctx->scratch().alloc_doubles(d.ncoefs());
  cuda_check(launch_gather_csr(d_x + col0_[std::make_pair(var, dd)], 0, 1, t.nrows, t.rowptr, t.idx, t.w, cf, 0, 1, 1.0,
                               0, ctx->stream()),
             "affecte_tau gather");
  ctx->launches++;
  return DVal::from_coef(ctx, &d, 1, cf, vars_[var].f->d[dd].base);
}

void System::jx(const double* d_x, double* d_y) {
  int N = nbr_unknowns();
  residual(nullptr, true);  // values at the current fields (they may have changed since the last residual)
  if (nbr_conditions_ != N) throw KdError(KD_ERR_STATE, "Number of unknowns is different from the number of equations");
  ctx->scratch().reset();
  std::vector<double> xd(vdoubles_.size());
  if (!vdoubles_.empty()) {
    cuda_check(cudaMemcpyAsync(xd.data(), d_x, sizeof(double) * xd.size(), cudaMemcpyDeviceToHost, ctx->stream()),
               "D2H x");
    cuda_check(cudaStreamSynchronize(ctx->stream()), "sync");
  }
  // xx_to_ders: the tangent of every unknown is affecte_tau(x)
  std::map<std::pair<int, int>, DVal> seeds;
  for (size_t v = 0; v < vars_.size(); v++)
    for (int dd = dom_min; dd <= dom_max; dd++) {
      auto key = std::make_pair(static_cast<int>(v), dd);
      const Domain& d = sp->dom(dd);
      const CsrTable& t = xmap(static_cast<int>(v), dd);
      double* cf = ctx->scratch().alloc_doubles(d.ncoefs());
      cuda_check(launch_gather_csr(d_x + col0_[key], 0, 1, t.nrows, t.rowptr, t.idx, t.w, cf, 0, 1, 1.0, 0,
                                   ctx->stream()),
                 "affecte_tau gather");
      ctx->launches++;
      seeds[key] = DVal::from_coef(ctx, &d, 1, cf, vars_[v].f->d[dd].base);
    }
  EvalState st;
  st.sys = this;
  st.with_der = true;
  st.B = 1;
  st.jx_seeds = &seeds;
  st.jx_doubles = &xd;
  st.vcache = &vcache_;
  cuda_check(cudaMemsetAsync(d_y, 0, sizeof(double) * N, ctx->stream()), "memset y");
  for (auto& eq : eqs_) export_tangent(eq, st, d_y, 0, 1);
  export_int_ders(st, -1, d_y, 1, 1);
}

void System::update_from_x(const double* d_x) {
  int N = nbr_unknowns();
  (void)N;
  vcache_.clear();
  ctx->scratch().reset();
  // doubles first
  if (!vdoubles_.empty()) {
    std::vector<double> hx(vdoubles_.size());
    cuda_check(cudaMemcpyAsync(hx.data(), d_x, sizeof(double) * hx.size(), cudaMemcpyDeviceToHost, ctx->stream()),
               "D2H x");
    cuda_check(cudaStreamSynchronize(ctx->stream()), "sync");
    for (size_t i = 0; i < vdoubles_.size(); i++) vdoubles_[i].value -= hx[i];
  }
  for (size_t v = 0; v < vars_.size(); v++) {
    Field* f = vars_[v].f;
    for (int dd = 0; dd < sp->ndom(); dd++) {
      const Domain& d = sp->dom(dd);
      DVal old = f->val(dd);
      if (dd < dom_min || dd > dom_max) {
        // old - old: the reference's update leaves exact zeros outside the system
        if (!old.zero) {
          DVal z = old - old;
          f->assign(dd, z);
        }
        continue;
      }
      auto key = std::make_pair(static_cast<int>(v), dd);
      double* cf = ctx->scratch().alloc_doubles(d.ncoefs());
      const CsrTable& t = xmap(static_cast<int>(v), dd);
      cuda_check(launch_gather_csr(d_x + col0_[key], 0, 1, t.nrows, t.rowptr, t.idx, t.w, cf, 0, 1, 1.0, 0,
                                   ctx->stream()),
                 "affecte_tau gather");
      ctx->launches++;
      DVal nv = DVal::from_coef(ctx, &d, 1, cf, f->d[dd].base);
      DVal res = old - nv;
      f->assign(dd, res);
    }
  }
  cuda_check(cudaStreamSynchronize(ctx->stream()), "sync after update");
}

}  // namespace kd
