// C ABI entry points (declared in include/kadath_gb300.h).  Each call turns
// C++ exceptions into status codes and records the message on the context.
#include <cmath>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <memory>
#include <string>

#include "kadath_gb300.h"
#include "kd_points.hpp"
#include "kd_context.hpp"
#include "kd_noalloc.hpp"
#include "kd_spectral.hpp"
#include "kd_stages.hpp"

// Handles are reference counted: a space keeps its context alive, and a
// field or system keeps its space alive, so a caller (or a garbage
// collector) may destroy them in any order.
struct kd_ctx {
  std::unique_ptr<kd::Context> c;
  std::string err;
  std::atomic<int> refs{1};
};

namespace {

void ctx_retain(kd_ctx* c) { c->refs.fetch_add(1); }
void ctx_release(kd_ctx* c) {
  if (c->refs.fetch_sub(1) == 1) delete c;
}

template <class F>
int guarded(kd_ctx* ctx, F&& f) {
  try {
    f();
    return KD_OK;
  } catch (const kd::KdError& e) {
    if (ctx) ctx->err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    if (ctx) ctx->err = e.what();
    return KD_ERR_ARG;
  }
}

kd::Base base_from_desc(const kd_transform_desc& d) {
  kd::Base b;
  b.def = true;
  b.allocate(d.nbr_coefs[1], d.nbr_coefs[2]);
  std::memcpy(b.r.data(), d.base_r, b.r.size() * sizeof(int));
  std::memcpy(b.t.data(), d.base_t, b.t.size() * sizeof(int));
  b.p = d.base_p;
  return b;
}

void check_desc(const kd_transform_desc& d) {
  for (int i = 0; i < 3; i++)
    if (d.nbr_points[i] <= 0 || d.nbr_coefs[i] <= 0) throw kd::KdError(KD_ERR_ARG, "non-positive dimension");
  if (d.batch < 0) throw kd::KdError(KD_ERR_ARG, "negative batch");
  if (!d.base_r || !d.base_t) throw kd::KdError(KD_ERR_ARG, "null basis table");
  if (d.batch > 0 && (!d.in || !d.out)) throw kd::KdError(KD_ERR_ARG, "null data pointer");
}

long long prod3(const int* d) { return static_cast<long long>(d[0]) * d[1] * d[2]; }

void transform_many(kd_ctx* ctx, int n, const kd_transform_desc* descs, bool inverse) {
  if (n < 0 || (n > 0 && !descs)) throw kd::KdError(KD_ERR_ARG, "bad descriptor list");
  kd::Context& c = *ctx->c;
  std::vector<kd::KdItem> items;
  std::vector<int> batches;
  for (int i = 0; i < n; i++) {
    const kd_transform_desc& d = descs[i];
    check_desc(d);
    if (d.batch == 0) continue;
    kd::Base b = base_from_desc(d);
    auto specs = inverse ? kd::coef_i_specs(c, b, d.nbr_points, d.nbr_coefs)
                         : kd::coef_specs(c, b, d.nbr_points, d.nbr_coefs);
    const int* din = inverse ? d.nbr_coefs : d.nbr_points;
    const int* dout = inverse ? d.nbr_points : d.nbr_coefs;
    items.push_back(kd::make_item(c, specs, d.in, d.out, din, prod3(din), prod3(dout), 1.0));
    batches.push_back(d.batch);
  }
  c.run_items(items, batches);
}

void transform_host(kd_ctx* ctx, const kd_transform_desc* desc, bool inverse) {
  if (!desc) throw kd::KdError(KD_ERR_ARG, "null descriptor");
  check_desc(*desc);
  kd::Context& c = *ctx->c;
  const int* din = inverse ? desc->nbr_coefs : desc->nbr_points;
  const int* dout = inverse ? desc->nbr_points : desc->nbr_coefs;
  size_t nin = static_cast<size_t>(prod3(din)) * desc->batch;
  size_t nout = static_cast<size_t>(prod3(dout)) * desc->batch;
  size_t mark = c.scratch().mark();
  double* din_d = c.scratch().alloc_doubles(nin);
  double* dout_d = c.scratch().alloc_doubles(nout);
  kd::cuda_check(cudaMemcpyAsync(din_d, desc->in, nin * sizeof(double), cudaMemcpyHostToDevice, c.stream()),
                 "H2D");
  kd_transform_desc d = *desc;
  d.in = din_d;
  d.out = dout_d;
  transform_many(ctx, 1, &d, inverse);
  kd::cuda_check(cudaMemcpyAsync(desc->out, dout_d, nout * sizeof(double), cudaMemcpyDeviceToHost, c.stream()),
                 "D2H");
  kd::cuda_check(cudaStreamSynchronize(c.stream()), "sync");
  c.scratch().release_to(mark);
}

}  // namespace

extern "C" {

int kd_ctx_create(kd_ctx** out, int device) {
  if (!out) return KD_ERR_ARG;
  *out = nullptr;
  auto* ctx = new kd_ctx();
  int st = guarded(ctx, [&] { ctx->c = std::make_unique<kd::Context>(device); });
  if (st != KD_OK) {
    // Keep the context object so that the caller can read the message.
    *out = ctx;
    return st;
  }
  *out = ctx;
  return KD_OK;
}

int kd_ctx_set_sm_budget(kd_ctx* ctx, int sms) {
  if (!ctx || !ctx->c) return KD_ERR_ARG;
  if (sms < 0) return KD_ERR_ARG;
  ctx->c->set_sm_budget(sms);
  return KD_OK;
}

int kd_ctx_set_wait_limit(kd_ctx* ctx, double seconds) {
  if (!ctx || !ctx->c) return KD_ERR_ARG;
  if (!(seconds > 0) || seconds > 3600) return KD_ERR_ARG;
  ctx->c->grid_wait_ns = static_cast<unsigned long long>(seconds * 1e9);
  return KD_OK;
}

int kd_ctx_autotune(kd_ctx* ctx, const char* path, int mode) {
  if (!ctx || !ctx->c) return KD_ERR_ARG;
  return guarded(ctx, [&] { ctx->c->set_autotune(path ? std::string(path) : std::string(), mode); });
}

int kd_ctx_autotune_stats(const kd_ctx* ctx, long long* entries, long long* tuned, long long* hits) {
  if (!ctx || !ctx->c || !entries || !tuned || !hits) return KD_ERR_ARG;
  *entries = static_cast<long long>(ctx->c->tuner.table.size());
  *tuned = ctx->c->tuner.tuned;
  *hits = ctx->c->tuner.hits;
  return KD_OK;
}

int kd_ctx_stall_waits(kd_ctx* ctx, int on) {
  if (!ctx || !ctx->c) return KD_ERR_ARG;
  ctx->c->stall_waits = on ? 1 : 0;
  return KD_OK;
}

int kd_ctx_destroy(kd_ctx* ctx) {
  if (!ctx) return KD_ERR_ARG;
  ctx_release(ctx);
  return KD_OK;
}

const char* kd_last_error(const kd_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int kd_ctx_synchronize(kd_ctx* ctx) {
  if (!ctx || !ctx->c) return KD_ERR_ARG;
  return guarded(ctx, [&] { kd::cuda_check(cudaStreamSynchronize(ctx->c->stream()), "sync"); });
}

long long kd_ctx_launch_count(const kd_ctx* ctx) { return (ctx && ctx->c) ? ctx->c->launches : -1; }

int kd_coef_many(kd_ctx* ctx, int n, const kd_transform_desc* descs) {
  if (!ctx || !ctx->c) return KD_ERR_ARG;
  return guarded(ctx, [&] { transform_many(ctx, n, descs, false); });
}

int kd_coef_i_many(kd_ctx* ctx, int n, const kd_transform_desc* descs) {
  if (!ctx || !ctx->c) return KD_ERR_ARG;
  return guarded(ctx, [&] { transform_many(ctx, n, descs, true); });
}

int kd_coef_host(kd_ctx* ctx, const kd_transform_desc* desc) {
  if (!ctx || !ctx->c) return KD_ERR_ARG;
  return guarded(ctx, [&] { transform_host(ctx, desc, false); });
}

int kd_coef_i_host(kd_ctx* ctx, const kd_transform_desc* desc) {
  if (!ctx || !ctx->c) return KD_ERR_ARG;
  return guarded(ctx, [&] { transform_host(ctx, desc, true); });
}

int kd_coef_host_noalloc(kd_ctx* ctx, const kd_transform_desc* desc) {
  if (!ctx || !ctx->c) return KD_ERR_ARG;
  return guarded(ctx, [&] {
    if (!desc) throw kd::KdError(KD_ERR_ARG, "null descriptor");
    check_desc(*desc);
    kd::Base b = base_from_desc(*desc);
    kd::coef_host_noalloc(*ctx->c, b, desc->nbr_points, desc->nbr_coefs, desc->batch, desc->in, desc->out);
  });
}

int kd_ope_1d(kd_ctx* ctx, int op, int dim, const kd_transform_desc* desc, int* base_out_r, int* base_out_t,
              int* base_out_p) {
  if (!ctx || !ctx->c) return KD_ERR_ARG;
  return guarded(ctx, [&] {
    if (!desc) throw kd::KdError(KD_ERR_ARG, "null descriptor");
    check_desc(*desc);
    if (dim < 0 || dim > 2) throw kd::KdError(KD_ERR_ARG, "dim must be 0, 1 or 2");
    if (op < KD_OP_DER || op > KD_OP_DIV_1MX2) throw kd::KdError(KD_ERR_ARG, "unknown 1-D operator");
    kd::Context& c = *ctx->c;
    kd::Base b = base_from_desc(*desc);
    kd::Base bo = b;
    auto spec = kd::ope_1d_spec(c, op, dim, b, desc->nbr_coefs, bo);
    if (desc->batch > 0) {
      auto it = kd::make_item(c, {spec}, desc->in, desc->out, desc->nbr_coefs, prod3(desc->nbr_coefs),
                              prod3(desc->nbr_coefs), 1.0);
      c.run_items({it}, {desc->batch});
    }
    if (base_out_r) std::memcpy(base_out_r, bo.r.data(), bo.r.size() * sizeof(int));
    if (base_out_t) std::memcpy(base_out_t, bo.t.data(), bo.t.size() * sizeof(int));
    if (base_out_p) *base_out_p = bo.p;
  });
}

int kd_matrix_1d(kd_ctx* ctx, int op, int basis, int n_in, int n_out, double* mat, int* out_basis) {
  // Host-only: ctx may be NULL (no GPU needed to inspect an operator).
  return guarded(ctx, [&] {
    if (n_in <= 0 || n_out <= 0 || !mat) throw kd::KdError(KD_ERR_ARG, "bad matrix request");
    kd::Mat1d m;
    if (!kd::build_matrix(op, basis, n_in, n_out, m))
      throw kd::KdError(KD_ERR_UNSUPPORTED, "operator not defined for this basis");
    std::memcpy(mat, m.m.data(), m.m.size() * sizeof(double));
    if (out_basis) *out_basis = m.out_basis;
  });
}

}  // extern "C"

// ------------------------------------------------------------------------
// Spaces, fields, systems, Newton, LU.
#include "kd_gemm_tc.hpp"
#include "kd_io.hpp"
#include "kd_newton.hpp"

struct kd_space {
  kd_ctx* ctx;
  std::unique_ptr<kd::Space> sp;
  std::atomic<int> refs{1};
};

namespace {
void space_retain(kd_space* s) { s->refs.fetch_add(1); }
void space_release(kd_space* s) {
  if (s->refs.fetch_sub(1) == 1) {
    kd_ctx* c = s->ctx;
    delete s;
    ctx_release(c);
  }
}
}  // namespace
struct kd_field {
  kd_space* sp;
  std::unique_ptr<kd::Field> f;
};
struct kd_file {
  std::FILE* f = nullptr;
  bool writing = false;
};
struct kd_system {
  kd_space* sp;
  std::unique_ptr<kd::System> sys;
  std::unique_ptr<kd::Newton> newton;
};
struct kd_lu {
  kd_ctx* ctx;
  std::unique_ptr<kd::DenseLU> lu;
};

namespace {
template <class F>
int guarded_ctx(kd_ctx* ctx, F&& f) {
  if (!ctx) return KD_ERR_ARG;
  return guarded(ctx, std::forward<F>(f));
}
void check_dom(const kd::Space& sp, int dom) {
  if (dom < 0 || dom >= sp.ndom()) throw kd::KdError(KD_ERR_ARG, "domain index out of range");
}
}  // namespace

extern "C" {

int kd_space_spheric_create(kd_ctx* ctx, const double center[3], const int res[3], const double* bounds, int nbounds,
                            int withzec, kd_space** out) {
  if (!ctx || !out) return KD_ERR_ARG;
  return guarded(ctx, [&] {
    if (!center || !res || !bounds || nbounds < 1) throw kd::KdError(KD_ERR_ARG, "bad space arguments");
    for (int i = 0; i < 3; i++)
      if (res[i] < 1) throw kd::KdError(KD_ERR_ARG, "resolution must be positive");
    if (res[0] < 3 || res[1] < 2) throw kd::KdError(KD_ERR_ARG, "need nr >= 3 and ntheta >= 2");
    std::vector<double> b(bounds, bounds + nbounds);
    auto* s = new kd_space{ctx, std::make_unique<kd::Space>(center, res, b, withzec != 0)};
    ctx_retain(ctx);
    *out = s;
  });
}

int kd_file_open(const char* path, const char* mode, kd_file** out) {
  if (!path || !mode || !out) return KD_ERR_ARG;
  const std::string m(mode);
  if (m != "wb" && m != "rb") return KD_ERR_ARG;
  std::FILE* f = std::fopen(path, mode);
  if (!f) return KD_ERR_ARG;
  *out = new kd_file{f, m == "wb"};
  return KD_OK;
}

int kd_file_close(kd_file* f) {
  if (!f) return KD_ERR_ARG;
  const int st = std::fclose(f->f) == 0 ? KD_OK : KD_ERR_ARG;
  delete f;
  return st;
}

int kd_space_save(const kd_space* sp, kd_file* f) {
  if (!sp || !f || !f->writing) return KD_ERR_ARG;
  return guarded(sp->ctx, [&] { kd::save_space(*sp->sp, f->f); });
}

int kd_space_load(kd_ctx* ctx, kd_file* f, int withzec, kd_space** out) {
  if (!ctx || !f || f->writing || !out) return KD_ERR_ARG;
  return guarded(ctx, [&] {
    *out = new kd_space{ctx, kd::load_space(f->f, withzec != 0)};
    ctx_retain(ctx);
  });
}

int kd_field_save(kd_field* fld, kd_file* f) {
  if (!fld || !f || !f->writing) return KD_ERR_ARG;
  return guarded(fld->sp->ctx, [&] { kd::save_field(*fld->f, f->f); });
}

int kd_field_load(kd_field* fld, kd_file* f) {
  if (!fld || !f || f->writing) return KD_ERR_ARG;
  return guarded(fld->sp->ctx, [&] { kd::load_field(*fld->f, f->f); });
}

int kd_vector_save(kd_field* fx, kd_field* fy, kd_field* fz, int type_index, kd_file* f) {
  if (!fx || !fy || !fz || !f || !f->writing || fx->sp != fy->sp || fx->sp != fz->sp) return KD_ERR_ARG;
  return guarded(fx->sp->ctx, [&] {
    kd::Field* const c[3] = {fx->f.get(), fy->f.get(), fz->f.get()};
    kd::save_vector(c, type_index, f->f);
  });
}

int kd_vector_load(kd_field* fx, kd_field* fy, kd_field* fz, int* type_index, kd_file* f) {
  if (!fx || !fy || !fz || !f || f->writing || fx->sp != fy->sp || fx->sp != fz->sp) return KD_ERR_ARG;
  return guarded(fx->sp->ctx, [&] {
    kd::Field* const c[3] = {fx->f.get(), fy->f.get(), fz->f.get()};
    kd::load_vector(c, type_index, f->f);
  });
}

int kd_space_destroy(kd_space* sp) {
  if (!sp) return KD_ERR_ARG;
  space_release(sp);
  return KD_OK;
}

int kd_space_nbr_domains(const kd_space* sp, int* n) {
  if (!sp || !n) return KD_ERR_ARG;
  *n = sp->sp->ndom();
  return KD_OK;
}

int kd_space_domain_info(const kd_space* sp, int dom, int* type, int npts[3], int ncoefs[3], double* alpha,
                         double* beta) {
  if (!sp) return KD_ERR_ARG;
  return guarded(sp->ctx, [&] {
    check_dom(*sp->sp, dom);
    const kd::Domain& d = sp->sp->dom(dom);
    if (type) *type = d.type;
    for (int i = 0; i < 3; i++) {
      if (npts) npts[i] = d.np[i];
      if (ncoefs) ncoefs[i] = d.nc[i];
    }
    if (alpha) *alpha = d.alpha;
    if (beta) *beta = d.beta;
  });
}

int kd_space_radius(const kd_space* sp, int dom, double* out) {
  if (!sp || !out) return KD_ERR_ARG;
  return guarded(sp->ctx, [&] {
    check_dom(*sp->sp, dom);
    auto r = sp->sp->dom(dom).radius_values();
    std::memcpy(out, r.data(), r.size() * sizeof(double));
  });
}

int kd_space_cart(const kd_space* sp, int dom, int c, double* out) {
  if (!sp || !out || c < 0 || c > 2) return KD_ERR_ARG;
  return guarded(sp->ctx, [&] {
    check_dom(*sp->sp, dom);
    auto r = sp->sp->dom(dom).cart_values(c);
    std::memcpy(out, r.data(), r.size() * sizeof(double));
  });
}

int kd_space_std_base(const kd_space* sp, int dom, int* base_r, int* base_t, int* base_p) {
  if (!sp) return KD_ERR_ARG;
  return guarded(sp->ctx, [&] {
    check_dom(*sp->sp, dom);
    kd::Base b = sp->sp->dom(dom).std_base();
    if (base_r) std::memcpy(base_r, b.r.data(), b.r.size() * sizeof(int));
    if (base_t) std::memcpy(base_t, b.t.data(), b.t.size() * sizeof(int));
    if (base_p) *base_p = b.p;
  });
}

int kd_field_create(kd_space* sp, kd_field** out) {
  if (!sp || !out) return KD_ERR_ARG;
  return guarded(sp->ctx, [&] {
    *out = new kd_field{sp, std::make_unique<kd::Field>(sp->ctx->c.get(), sp->sp.get())};
    space_retain(sp);
  });
}

int kd_field_destroy(kd_field* f) {
  if (!f) return KD_ERR_ARG;
  kd_space* sp = f->sp;
  delete f;
  space_release(sp);
  return KD_OK;
}

int kd_field_set_value(kd_field* f, double v) {
  if (!f) return KD_ERR_ARG;
  return guarded(f->sp->ctx, [&] { f->f->set_value(v); });
}

int kd_field_std_base(kd_field* f) {
  if (!f) return KD_ERR_ARG;
  return guarded(f->sp->ctx, [&] { f->f->std_base(); });
}

int kd_field_cart_base(kd_field* f, int c) {
  if (!f || c < 0 || c > 2) return KD_ERR_ARG;
  return guarded(f->sp->ctx, [&] {
    for (int i = 0; i < f->sp->sp->ndom(); i++) f->f->d[i].base = f->sp->sp->dom(i).cart_base(c);
  });
}

int kd_field_set_conf(kd_field* f, int dom, const double* v) {
  if (!f || !v) return KD_ERR_ARG;
  return guarded(f->sp->ctx, [&] {
    check_dom(*f->sp->sp, dom);
    f->f->set_conf_host(dom, v);
  });
}

int kd_field_get_conf(kd_field* f, int dom, double* out) {
  if (!f || !out) return KD_ERR_ARG;
  return guarded(f->sp->ctx, [&] {
    check_dom(*f->sp->sp, dom);
    f->f->get_conf_host(dom, out);
  });
}

int kd_field_get_coef(kd_field* f, int dom, double* out) {
  if (!f || !out) return KD_ERR_ARG;
  return guarded(f->sp->ctx, [&] {
    check_dom(*f->sp->sp, dom);
    f->f->get_coef_host(dom, out);
  });
}

int kd_field_get_base(const kd_field* f, int dom, int* base_r, int* base_t, int* base_p) {
  if (!f) return KD_ERR_ARG;
  return guarded(f->sp->ctx, [&] {
    check_dom(*f->sp->sp, dom);
    const kd::Base& b = f->f->d[dom].base;
    if (!b.def) throw kd::KdError(KD_ERR_STATE, "basis not defined");
    if (base_r) std::memcpy(base_r, b.r.data(), b.r.size() * sizeof(int));
    if (base_t) std::memcpy(base_t, b.t.data(), b.t.size() * sizeof(int));
    if (base_p) *base_p = b.p;
  });
}

int kd_system_create(kd_space* sp, int dom_min, int dom_max, kd_system** out) {
  if (!sp || !out) return KD_ERR_ARG;
  return guarded(sp->ctx, [&] {
    auto* s = new kd_system{sp, std::make_unique<kd::System>(sp->ctx->c.get(), sp->sp.get(), dom_min, dom_max), nullptr};
    s->newton = std::make_unique<kd::Newton>(s->sys.get());
    space_retain(sp);
    *out = s;
  });
}

int kd_system_destroy(kd_system* s) {
  if (!s) return KD_ERR_ARG;
  kd_space* sp = s->sp;
  delete s;
  space_release(sp);
  return KD_OK;
}

#define SYS_GUARD(s) \
  if (!(s)) return KD_ERR_ARG; \
  return guarded((s)->sp->ctx, [&]

int kd_system_add_var(kd_system* s, const char* name, kd_field* f) {
  SYS_GUARD(s) {
    if (!name || !f) throw kd::KdError(KD_ERR_ARG, "null argument");
    s->sys->add_var(name, f->f.get());
  });
}

int kd_system_add_var_double(kd_system* s, const char* name, double v) {
  SYS_GUARD(s) {
    if (!name) throw kd::KdError(KD_ERR_ARG, "null name");
    s->sys->add_var_double(name, v);
  });
}

int kd_system_get_var_double(const kd_system* s, const char* name, double* v) {
  if (!s || !name || !v) return KD_ERR_ARG;
  return guarded(s->sp->ctx, [&] {
    int w = s->sys->find_var_double(kd::trim_expr(name).substr(0, kd::trim_expr(name).size() - 1));
    if (w < 0) throw kd::KdError(KD_ERR_ARG, "unknown double variable");
    *v = s->sys->var_double(w);
  });
}

int kd_system_add_cst(kd_system* s, const char* name, double v) {
  SYS_GUARD(s) {
    if (!name) throw kd::KdError(KD_ERR_ARG, "null name");
    s->sys->add_cst(name, v);
  });
}

int kd_system_add_cst_field(kd_system* s, const char* name, kd_field* f) {
  SYS_GUARD(s) {
    if (!name || !f) throw kd::KdError(KD_ERR_ARG, "null argument");
    s->sys->add_cst_field(name, f->f.get());
  });
}

int kd_system_add_eq_order(kd_system* s, int dom, int order, const char* eq) {
  SYS_GUARD(s) {
    if (!eq) throw kd::KdError(KD_ERR_ARG, "null equation");
    s->sys->add_eq_order(dom, order, eq);
  });
}

int kd_system_add_eq_full(kd_system* s, int dom, const char* eq) {
  SYS_GUARD(s) {
    if (!eq) throw kd::KdError(KD_ERR_ARG, "null equation");
    s->sys->add_eq_full(dom, eq);
  });
}

int kd_system_add_eq_first_integral(kd_system* s, int dom_min, int dom_max, const char* integ_part,
                                    const char* cst_part) {
  SYS_GUARD(s) {
    if (!integ_part || !cst_part) throw kd::KdError(KD_ERR_ARG, "null expression");
    s->sys->add_eq_first_integral(dom_min, dom_max, integ_part, cst_part);
  });
}

int kd_system_add_var_vector(kd_system* s, const char* name, kd_field* fx, kd_field* fy, kd_field* fz) {
  SYS_GUARD(s) {
    if (!name || !fx || !fy || !fz) throw kd::KdError(KD_ERR_ARG, "null argument");
    kd::Field* const comps[3] = {fx->f.get(), fy->f.get(), fz->f.get()};
    s->sys->add_var_vector(name, comps);
  });
}

int kd_system_add_cst_vector(kd_system* s, const char* name, kd_field* fx, kd_field* fy, kd_field* fz) {
  SYS_GUARD(s) {
    if (!name || !fx || !fy || !fz) throw kd::KdError(KD_ERR_ARG, "null argument");
    kd::Field* const comps[3] = {fx->f.get(), fy->f.get(), fz->f.get()};
    s->sys->add_cst_vector(name, comps);
  });
}

int kd_system_set_metric_flat(kd_system* s, const char* name) {
  SYS_GUARD(s) {
    if (!name) throw kd::KdError(KD_ERR_ARG, "null name");
    s->sys->set_metric_flat(name);
  });
}

int kd_system_add_def(kd_system* s, int dom, const char* text) {
  SYS_GUARD(s) {
    if (!text) throw kd::KdError(KD_ERR_ARG, "null text");
    s->sys->add_def(dom, text);
  });
}

int kd_system_add_eq_inside(kd_system* s, int dom, const char* eq) {
  SYS_GUARD(s) {
    if (!eq) throw kd::KdError(KD_ERR_ARG, "null equation");
    s->sys->add_eq_inside(dom, eq);
  });
}

int kd_system_add_eq_bc(kd_system* s, int dom, int bound, const char* eq) {
  SYS_GUARD(s) {
    if (!eq) throw kd::KdError(KD_ERR_ARG, "null equation");
    s->sys->add_eq_bc(dom, bound, eq);
  });
}

int kd_system_add_eq_matching(kd_system* s, int dom, int bound, const char* eq) {
  SYS_GUARD(s) {
    if (!eq) throw kd::KdError(KD_ERR_ARG, "null equation");
    s->sys->add_eq_matching(dom, bound, eq);
  });
}

int kd_system_add_eq_int_volume(kd_system* s, int dom_min, int dom_max, const char* eq) {
  SYS_GUARD(s) {
    if (!eq) throw kd::KdError(KD_ERR_ARG, "null equation");
    s->sys->add_eq_int_volume(dom_min, dom_max, eq);
  });
}

int kd_system_add_eq_int_inf(kd_system* s, const char* eq) {
  SYS_GUARD(s) {
    if (!eq) throw kd::KdError(KD_ERR_ARG, "null equation");
    s->sys->add_eq_int_inf(eq);
  });
}

int kd_system_add_eq_val(kd_system* s, int dom, const char* eq, const int pos[3]) {
  SYS_GUARD(s) {
    if (!eq || !pos) throw kd::KdError(KD_ERR_ARG, "null argument");
    s->sys->add_eq_val(dom, eq, pos);
  });
}

int kd_system_add_eq_point(kd_system* s, int dom, const char* eq, const double point[3]) {
  SYS_GUARD(s) {
    if (!eq || !point) throw kd::KdError(KD_ERR_ARG, "null argument");
    s->sys->add_eq_point(dom, eq, point);
  });
}

int kd_system_sizes(kd_system* s, int* n_unknowns, int* n_conditions) {
  SYS_GUARD(s) {
    if (s->sys->nbr_conditions() < 0) s->sys->residual(nullptr);
    if (n_unknowns) *n_unknowns = s->sys->nbr_unknowns();
    if (n_conditions) *n_conditions = s->sys->nbr_conditions();
  });
}

int kd_system_n_equations(kd_system* s, int* neq) {
  SYS_GUARD(s) {
    if (!neq) throw kd::KdError(KD_ERR_ARG, "null output");
    *neq = s->sys->n_equations();
  });
}

int kd_system_residual(kd_system* s, double* F) {
  SYS_GUARD(s) {
    if (!F) throw kd::KdError(KD_ERR_ARG, "null output");
    kd::Context* c = s->sp->ctx->c.get();
    if (s->sys->nbr_conditions() < 0) s->sys->residual(nullptr);
    int n = s->sys->nbr_conditions();
    s->newton->ensure(n > 0 ? n : 1);
    s->sys->residual(s->newton->d_F);
    kd::cuda_check(cudaMemcpyAsync(F, s->newton->d_F, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream()), "D2H");
    kd::cuda_check(cudaStreamSynchronize(c->stream()), "sync");
  });
}

int kd_system_check_equations(kd_system* s, double* errors) {
  SYS_GUARD(s) {
    if (!errors) throw kd::KdError(KD_ERR_ARG, "null output");
    kd::Context* c = s->sp->ctx->c.get();
    if (s->sys->nbr_conditions() < 0) s->sys->residual(nullptr);
    int n = s->sys->nbr_conditions();
    s->newton->ensure(n > 0 ? n : 1);
    s->sys->residual(s->newton->d_F);
    std::vector<double> F(n);
    kd::cuda_check(cudaMemcpyAsync(F.data(), s->newton->d_F, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream()),
                   "D2H");
    kd::cuda_check(cudaStreamSynchronize(c->stream()), "sync");
    for (int i = 0; i < s->sys->n_equations(); i++) {
      const kd::Equation& e = s->sys->equation(i);
      double m = 0;
      for (int r = 0; r < e.n_cond; r++) m = std::max(m, std::fabs(F[e.row0 + r]));
      errors[i] = m;
    }
  });
}

int kd_system_jacobian_graph_stats(kd_system* s, long long* captures, long long* replays) {
  if (!s || !s->sys || !captures || !replays) return KD_ERR_ARG;
  *captures = s->sys->jacobian_graph_captures;
  *replays = s->sys->jacobian_graph_replays;
  return KD_OK;
}

int kd_system_graph_stats(kd_system* s, long long* captures, long long* replays) {
  if (!s || !s->sys || !captures || !replays) return KD_ERR_ARG;
  *captures = s->sys->residual_graph_captures;
  *replays = s->sys->residual_graph_replays;
  return KD_OK;
}

int kd_system_cache_tangents(kd_system* s, int enable) {
  if (!s || !s->sys) return KD_ERR_ARG;
  return guarded(s->sp->ctx, [&] { s->sys->set_tangent_cache(enable != 0); });
}

int kd_system_jacobian_device(kd_system* s, double* dJ, long long ld) {
  SYS_GUARD(s) {
    if (!dJ) throw kd::KdError(KD_ERR_ARG, "null output");
    s->sys->jacobian(dJ, ld);
    kd::cuda_check(cudaStreamSynchronize(s->sp->ctx->c->stream()), "sync");
  });
}

int kd_system_jx_device(kd_system* s, const double* dx, double* dy) {
  SYS_GUARD(s) {
    if (!dx || !dy) throw kd::KdError(KD_ERR_ARG, "null vector");
    s->sys->jx(dx, dy);
    kd::cuda_check(cudaStreamSynchronize(s->sp->ctx->c->stream()), "sync");
  });
}

int kd_system_jx(kd_system* s, const double* x, double* y) {
  SYS_GUARD(s) {
    if (!x || !y) throw kd::KdError(KD_ERR_ARG, "null vector");
    kd::Context* c = s->sp->ctx->c.get();
    if (s->sys->nbr_conditions() < 0) s->sys->residual(nullptr);
    const int n = s->sys->nbr_unknowns();
    double* d = nullptr;
    kd::cuda_check(cudaMalloc(&d, sizeof(double) * 2 * n), "cudaMalloc(jx)");
    struct Free {
      double* p;
      ~Free() { cudaFree(p); }
    } guard{d};
    kd::cuda_check(cudaMemcpyAsync(d, x, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream()), "H2D x");
    s->sys->jx(d, d + n);
    kd::cuda_check(cudaMemcpyAsync(y, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream()), "D2H y");
    kd::cuda_check(cudaStreamSynchronize(c->stream()), "sync");
  });
}

int kd_system_jacobian(kd_system* s, double* J) {
  SYS_GUARD(s) {
    if (!J) throw kd::KdError(KD_ERR_ARG, "null output");
    kd::Context* c = s->sp->ctx->c.get();
    if (s->sys->nbr_conditions() < 0) s->sys->residual(nullptr);
    int n = s->sys->nbr_unknowns();
    s->newton->ensure(n);
    s->sys->jacobian(s->newton->d_J, n);
    kd::cuda_check(cudaMemcpyAsync(J, s->newton->d_J, sizeof(double) * n * n, cudaMemcpyDeviceToHost, c->stream()),
                   "D2H");
    kd::cuda_check(cudaStreamSynchronize(c->stream()), "sync");
  });
}

int kd_system_update(kd_system* s, const double* x) {
  SYS_GUARD(s) {
    if (!x) throw kd::KdError(KD_ERR_ARG, "null input");
    kd::Context* c = s->sp->ctx->c.get();
    int n = s->sys->nbr_unknowns();
    s->newton->ensure(n);
    kd::cuda_check(cudaMemcpyAsync(s->newton->d_F, x, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream()), "H2D");
    s->sys->update_from_x(s->newton->d_F);
  });
}

namespace {
kd::NewtonOpts to_opts(const kd_newton_opts* opts) {
  kd::NewtonOpts o;
  o.precision = opts->precision;
  o.lu_mode = opts->lu_mode;
  o.gmres_tol = opts->gmres_tol > 0 ? opts->gmres_tol : 1e-14;
  o.max_refine = opts->max_refine > 0 ? opts->max_refine : 50;
  o.gmres_restarts = opts->gmres_restarts > 0 ? opts->gmres_restarts : 4;
  o.pivot_every_step = opts->pivot_every_step;
  o.graph_capture = opts->graph_capture;
  return o;
}

void to_report(const kd::NewtonReport& r, kd_newton_report* rep) {
  rep->error = r.error;
  rep->converged = r.converged;
  rep->n = r.n;
  rep->t_residual_ms = r.t_residual_ms;
  rep->t_assembly_ms = r.t_assembly_ms;
  rep->t_factor_ms = r.t_factor_ms;
  rep->t_solve_ms = r.t_solve_ms;
  rep->t_update_ms = r.t_update_ms;
  rep->refine_iters = r.refine_iters;
  rep->refine_rel_residual = r.refine_rel_residual;
  rep->kernel_launches = r.kernel_launches;
  rep->fp64_fallback = r.fp64_fallback;
  rep->static_pivots = r.static_pivots;
}
}  // namespace

int kd_newton_step(kd_system* s, const kd_newton_opts* opts, kd_newton_report* rep) {
  SYS_GUARD(s) {
    if (!opts || !rep) throw kd::KdError(KD_ERR_ARG, "null argument");
    kd::NewtonReport r;
    s->newton->step(to_opts(opts), r);
    to_report(r, rep);
  });
}

int kd_stage_solve(kd_system* s, const kd_newton_opts* opts, int max_iter, const char* checkpoint, int nfields,
                   kd_field* const* fields, int* iterations, double* error) {
  SYS_GUARD(s) {
    if (!opts || max_iter < 1 || nfields < 0 || (nfields > 0 && !fields))
      throw kd::KdError(KD_ERR_ARG, "bad stage arguments");
    std::vector<kd::Field*> fl;
    for (int i = 0; i < nfields; i++) {
      if (!fields[i] || fields[i]->sp != s->sp)
        throw kd::KdError(KD_ERR_ARG, "checkpoint fields must be on the system's space");
      fl.push_back(fields[i]->f.get());
    }
    int it = 0;
    double err = 0.0;
    kd::stage_solve(*s->sys, *s->newton, to_opts(opts), max_iter, checkpoint, fl, it, err);
    if (iterations) *iterations = it;
    if (error) *error = err;
  });
}

int kd_field_regrid(kd_field* dst, kd_field* src) {
  if (!dst || !src) return KD_ERR_ARG;
  return guarded(dst->sp->ctx, [&] { kd::regrid(*dst->f, *src->f); });
}

int kd_system_reset_pivot_order(kd_system* s) {
  SYS_GUARD(s) { s->newton->lu().forget_pivots(); });
}

int kd_newton_step_gauss_newton(kd_system* s, const kd_newton_opts* opts, kd_newton_report* rep) {
  SYS_GUARD(s) {
    if (!opts || !rep) throw kd::KdError(KD_ERR_ARG, "null argument");
    kd::NewtonReport r;
    s->newton->step_gauss_newton(to_opts(opts), r);
    to_report(r, rep);
  });
}

int kd_system_add_ope_eos(kd_system* s, const char* name, int var, int npieces, double rhomin, double rhomax,
                          double k0, const double* gamma_tab, const double* rho_tab) {
  SYS_GUARD(s) {
    if (!name || !gamma_tab || !rho_tab) throw kd::KdError(KD_ERR_ARG, "null argument");
    if (npieces < 1 || npieces > kd::KD_EOS_MAX_PIECES) throw kd::KdError(KD_ERR_ARG, "1..8 polytrope pieces");
    kd::KdEos e = {};
    e.npieces = npieces;
    e.rhomin = rhomin;
    e.rhomax = rhomax;
    for (int i = 0; i < npieces; i++) {
      e.gamma[i] = gamma_tab[i];
      e.rho[i] = rho_tab[i];
      if (!(gamma_tab[i] > 1.0)) throw kd::KdError(KD_ERR_ARG, "polytropic exponents must exceed 1");
    }
    // Margherita_setup_polytrope (include/EOS/standalone/setup_polytrope.cc),
    // geometrised units: continuity of the pressure and of eps across pieces
    e.k[0] = k0;
    e.eps[0] = 0.0;
    e.h[0] = 0.0;
    for (int i = 1; i < npieces; i++) {
      if (e.rho[i] <= e.rho[i - 1]) throw kd::KdError(KD_ERR_ARG, "rho_tab must increase monotonically");
      const double gim1 = e.gamma[i] - 1.0;
      e.k[i] = e.k[i - 1] * std::pow(e.rho[i], e.gamma[i - 1] - e.gamma[i]);
      e.eps[i] = e.eps[i - 1] + e.k[i - 1] * std::pow(e.rho[i], e.gamma[i - 1] - 1.0) / (e.gamma[i - 1] - 1.0) -
                 e.k[i] * std::pow(e.rho[i], gim1) / gim1;
      const double P = e.k[i] * std::pow(e.rho[i], e.gamma[i]);
      const double eps = e.eps[i] + P / e.rho[i] / gim1;
      e.h[i] = 1. + eps + P / e.rho[i];
    }
    s->sys->add_ope_eos(name, var, e);
  });
}

int kd_system_set_cst(kd_system* s, const char* name, double v) {
  SYS_GUARD(s) {
    if (!name) throw kd::KdError(KD_ERR_ARG, "null name");
    const int i = s->sys->find_cst(name);
    if (i < 0) throw kd::KdError(KD_ERR_ARG, std::string("unknown constant ") + name);
    s->sys->set_cst(i, v);
  });
}

int kd_field_val_point(kd_field* f, const double point[3], double* value) {
  if (!f || !f->f) return KD_ERR_ARG;
  return guarded(f->sp->ctx, [&] {
    if (!point || !value) throw kd::KdError(KD_ERR_ARG, "null argument");
    *value = f->f->val_point(point);
  });
}

static std::vector<const kd::Field*> field_list(int nfields, kd_field* const* fields) {
  if (nfields <= 0 || !fields) throw kd::KdError(KD_ERR_ARG, "no fields");
  std::vector<const kd::Field*> out;
  for (int f = 0; f < nfields; f++) {
    if (!fields[f] || !fields[f]->f) throw kd::KdError(KD_ERR_ARG, "null field");
    if (fields[f]->sp != fields[0]->sp) throw kd::KdError(KD_ERR_ARG, "fields on different spaces");
    out.push_back(fields[f]->f.get());
  }
  return out;
}

int kd_fields_val_points(int nfields, kd_field* const* fields, long long npts, const double* xyz, double* out) {
  if (nfields <= 0 || !fields || !fields[0] || !fields[0]->f) return KD_ERR_ARG;
  return guarded(fields[0]->sp->ctx, [&] {
    auto list = field_list(nfields, fields);
    if (npts < 0 || (npts > 0 && (!xyz || !out))) throw kd::KdError(KD_ERR_ARG, "null argument");
    if (npts == 0) return;
    kd::Context& c = *fields[0]->sp->ctx->c;
    cudaStream_t s = c.stream();
    double *d_xyz = nullptr, *d_out = nullptr;
    kd::cuda_check(cudaMalloc(&d_xyz, sizeof(double) * 3 * npts), "cudaMalloc(points)");
    if (cudaMalloc(&d_out, sizeof(double) * nfields * npts) != cudaSuccess) {
      cudaFree(d_xyz);
      throw kd::KdError(KD_ERR_CUDA, "cudaMalloc(values)");
    }
    try {
      kd::cuda_check(cudaMemcpyAsync(d_xyz, xyz, sizeof(double) * 3 * npts, cudaMemcpyHostToDevice, s), "H2D points");
      kd::fields_val_points(&c, list, npts, d_xyz, d_out);
      kd::cuda_check(cudaMemcpyAsync(out, d_out, sizeof(double) * nfields * npts, cudaMemcpyDeviceToHost, s),
                     "D2H values");
      kd::cuda_check(cudaStreamSynchronize(s), "sync");
    } catch (...) {
      cudaFree(d_xyz);
      cudaFree(d_out);
      throw;
    }
    cudaFree(d_xyz);
    cudaFree(d_out);
  });
}

int kd_fields_val_points_device(int nfields, kd_field* const* fields, long long npts, const double* d_xyz,
                                double* d_out) {
  if (nfields <= 0 || !fields || !fields[0] || !fields[0]->f) return KD_ERR_ARG;
  return guarded(fields[0]->sp->ctx, [&] {
    auto list = field_list(nfields, fields);
    if (npts < 0 || (npts > 0 && (!d_xyz || !d_out))) throw kd::KdError(KD_ERR_ARG, "null argument");
    kd::fields_val_points(fields[0]->sp->ctx->c.get(), list, npts, d_xyz, d_out);
  });
}

int kd_system_val_point_gradient(kd_system* s, const char* var, const double point[3], double* g) {
  SYS_GUARD(s) {
    if (!var || !point || !g) throw kd::KdError(KD_ERR_ARG, "null argument");
    const int v = s->sys->find_var(var);
    if (v < 0) throw kd::KdError(KD_ERR_ARG, std::string("unknown variable ") + var);
    s->sys->val_point_gradient(v, point, g);
  });
}

int kd_system_dres_dcst(kd_system* s, const char* cst, double* fp) {
  SYS_GUARD(s) {
    if (!cst || !fp) throw kd::KdError(KD_ERR_ARG, "null argument");
    const int i = s->sys->find_cst(cst);
    if (i < 0) throw kd::KdError(KD_ERR_ARG, std::string("unknown constant ") + cst);
    kd::Context* c = s->sp->ctx->c.get();
    const int n = s->sys->nbr_unknowns();
    double* d = nullptr;
    kd::cuda_check(cudaMalloc(&d, sizeof(double) * n), "cudaMalloc(dF/dp)");
    struct Free {
      double* p;
      ~Free() { cudaFree(p); }
    } guard{d};
    s->sys->dres_dcst(i, d);
    kd::cuda_check(cudaMemcpyAsync(fp, d, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream()), "D2H");
    kd::cuda_check(cudaStreamSynchronize(c->stream()), "sync");
  });
}

int kd_adjoint(kd_system* s, const double* g, const char* cst, double dq_explicit, double* dqdp, double* lambda) {
  SYS_GUARD(s) {
    if (!g || !cst || !dqdp) throw kd::KdError(KD_ERR_ARG, "null argument");
    const int i = s->sys->find_cst(cst);
    if (i < 0) throw kd::KdError(KD_ERR_ARG, std::string("unknown constant ") + cst);
    *dqdp = s->newton->adjoint(g, i, dq_explicit, lambda);
  });
}

int kd_adjoint_ex(kd_system* s, const double* g, const char* cst, double dq_explicit, int reuse_factors,
                  double* dqdp, double* lambda, kd_adjoint_report* rep) {
  SYS_GUARD(s) {
    if (!g || !cst || !dqdp) throw kd::KdError(KD_ERR_ARG, "null argument");
    const int i = s->sys->find_cst(cst);
    if (i < 0) throw kd::KdError(KD_ERR_ARG, std::string("unknown constant ") + cst);
    kd::Newton::AdjointReport r;
    *dqdp = s->newton->adjoint(g, i, dq_explicit, lambda, reuse_factors != 0, &r);
    if (rep) {
      rep->reused_factors = r.reused_factors;
      rep->refine_iters = r.refine_iters;
      rep->rel_residual = r.rel_residual;
      rep->t_assembly_ms = r.t_assembly_ms;
      rep->t_solve_ms = r.t_solve_ms;
    }
  });
}

int kd_system_integral_gradient(kd_system* s, int kind, int dmin, int dmax, const char* expr, double* q,
                                double* g) {
  SYS_GUARD(s) {
    if (!expr || !q || !g) throw kd::KdError(KD_ERR_ARG, "null argument");
    kd::Context* c = s->sp->ctx->c.get();
    const int n = s->sys->nbr_unknowns();
    double* d = nullptr;
    kd::cuda_check(cudaMalloc(&d, sizeof(double) * (n > 0 ? n : 1)), "cudaMalloc(gradient)");
    struct Free {
      double* p;
      ~Free() { cudaFree(p); }
    } guard{d};
    *q = s->sys->integral_gradient(kind, dmin, dmax, expr, d);
    kd::cuda_check(cudaMemcpyAsync(g, d, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream()), "D2H");
    kd::cuda_check(cudaStreamSynchronize(c->stream()), "sync");
  });
}

int kd_newton_step_linesearch(kd_system* s, const kd_newton_opts* opts, int ntrymax, double stepmax,
                              kd_newton_report* rep, double* lambda) {
  SYS_GUARD(s) {
    if (!opts || !rep) throw kd::KdError(KD_ERR_ARG, "null argument");
    if (ntrymax < 1 || !(stepmax > 0)) throw kd::KdError(KD_ERR_ARG, "need ntrymax >= 1 and stepmax > 0");
    kd::NewtonReport r;
    s->newton->step_linesearch(to_opts(opts), ntrymax, stepmax, r, lambda);
    to_report(r, rep);
  });
}

int kd_lu_create(kd_ctx* ctx, kd_lu** out) {
  if (!ctx || !ctx->c || !out) return KD_ERR_ARG;
  return guarded(ctx, [&] {
    *out = new kd_lu{ctx, std::make_unique<kd::DenseLU>(ctx->c.get())};
    ctx_retain(ctx);
  });
}

int kd_lu_destroy(kd_lu* lu) {
  if (!lu) return KD_ERR_ARG;
  kd_ctx* c = lu->ctx;
  delete lu;
  ctx_release(c);
  return KD_OK;
}

int kd_lu_factor(kd_lu* lu, double* dA, long long ld, int n, int mode) {
  if (!lu) return KD_ERR_ARG;
  return guarded(lu->ctx, [&] {
    if (!dA || n <= 0 || ld < n) throw kd::KdError(KD_ERR_ARG, "bad matrix");
    if (mode < KD_LU_FP64 || mode > KD_LU_FP32_IR) throw kd::KdError(KD_ERR_ARG, "unknown LU mode");
    lu->lu->factor(dA, ld, n, mode);
  });
}

int kd_lu_solve(kd_lu* lu, double* db, int trans) {
  if (!lu) return KD_ERR_ARG;
  return guarded(lu->ctx, [&] {
    if (!db) throw kd::KdError(KD_ERR_ARG, "null vector");
    if (lu->lu->n() <= 0) throw kd::KdError(KD_ERR_STATE, "factor first");
    lu->lu->solve(db, trans);
  });
}

int kd_lu_set_refinement(kd_lu* lu, double tol, int iters, int restarts) {
  if (!lu) return KD_ERR_ARG;
  if (!(tol > 0) || iters < 1 || restarts < 1) return KD_ERR_ARG;
  lu->lu->gmres_tol = tol;
  lu->lu->gmres_max_iter = iters;
  lu->lu->gmres_restarts = restarts;
  return KD_OK;
}

int kd_lu_set_pivot_reuse(kd_lu* lu, int on) {
  if (!lu) return KD_ERR_ARG;
  lu->lu->reuse_pivots = on != 0;
  return KD_OK;
}

int kd_lu_pivot_info(const kd_lu* lu, int* static_pivots, int* fallback) {
  if (!lu) return KD_ERR_ARG;
  if (static_pivots) *static_pivots = lu->lu->stats.static_pivots;
  if (fallback) *fallback = lu->lu->stats.static_pivot_fallback;
  return KD_OK;
}

int kd_lu_stats(const kd_lu* lu, double* t_factor_ms, double* t_solve_ms, int* refine_iters, double* rel_residual) {
  if (!lu) return KD_ERR_ARG;
  if (t_factor_ms) *t_factor_ms = lu->lu->stats.t_factor_ms;
  if (t_solve_ms) *t_solve_ms = lu->lu->stats.t_solve_ms;
  if (refine_iters) *refine_iters = lu->lu->stats.refine_iters;
  if (rel_residual) *rel_residual = lu->lu->stats.final_rel_residual;
  return KD_OK;
}

}  // extern "C"

extern "C" {

int kd_tf32_gemm_update(kd_ctx* ctx, int m, int n, int k, const float* A, long long lda, const float* B,
                        long long ldb, float* C, long long ldc) {
  if (!ctx || !ctx->c) return KD_ERR_ARG;
  return guarded(ctx, [&] {
    if (m < 0 || n < 0 || k < 1 || k > 128) throw kd::KdError(KD_ERR_ARG, "need m, n >= 0 and 1 <= k <= 128");
    if ((m > 0 && lda < m) || ldb < k || (m > 0 && ldc < m)) throw kd::KdError(KD_ERR_ARG, "leading dimension too small");
    if (!A || !B || !C) throw kd::KdError(KD_ERR_ARG, "null matrix");
    kd::tf32_gemm_update(ctx->c.get(), m, n, k, A, lda, B, ldb, C, ldc, m);
    if (kd::tf32_gemm_error_flag(ctx->c.get()))
      throw kd::KdError(KD_ERR_TIMEOUT, "tensor-core update timed out waiting for its MMAs");
  });
}

int kd_tf32x3_gemm_update(kd_ctx* ctx, int m, int n, int k, const float* A, long long lda, const float* B,
                          long long ldb, float* C, long long ldc) {
  if (!ctx || !ctx->c) return KD_ERR_ARG;
  return guarded(ctx, [&] {
    if (m < 0 || n < 0 || k < 1 || k > 192) throw kd::KdError(KD_ERR_ARG, "need m, n >= 0 and 1 <= k <= 192");
    if ((m > 0 && lda < m) || ldb < k || (m > 0 && ldc < m)) throw kd::KdError(KD_ERR_ARG, "leading dimension too small");
    if (!A || !B || !C) throw kd::KdError(KD_ERR_ARG, "null matrix");
    kd::tf32_gemm_update(ctx->c.get(), m, n, k, A, lda, B, ldb, C, ldc, m, 3);
    if (kd::tf32_gemm_error_flag(ctx->c.get()))
      throw kd::KdError(KD_ERR_TIMEOUT, "tensor-core update timed out waiting for its MMAs");
  });
}

void* kd_ctx_stream(const kd_ctx* ctx) {
  return (ctx && ctx->c) ? static_cast<void*>(ctx->c->stream()) : nullptr;
}

int kd_ctx_profile_enable(kd_ctx* ctx, int on) {
  if (!ctx || !ctx->c) return KD_ERR_ARG;
  return guarded(ctx, [&] { ctx->c->prof_enable(on != 0); });
}

static_assert(KD_PROF_NCAT == kd::Context::PROF_NCAT, "profile categories of the C ABI and the context differ");

int kd_ctx_profile_read(kd_ctx* ctx, double* ms, long long* launches, double* work) {
  if (!ctx || !ctx->c || !ms || !launches || !work) return KD_ERR_ARG;
  return guarded(ctx, [&] { ctx->c->prof_read(ms, launches, work); });
}

int kd_field_copy(kd_field* dst, const kd_field* src) {
  if (!dst || !src || dst->sp != src->sp) return KD_ERR_ARG;
  return guarded(dst->sp->ctx, [&] {
    for (int i = 0; i < dst->sp->sp->ndom(); i++) {
      kd::DVal v = src->f->val(i);
      dst->f->assign(i, v);
    }
    kd::cuda_check(cudaStreamSynchronize(dst->sp->ctx->c->stream()), "sync");
  });
}

}  // extern "C"
