// C ABI entry points (declared in include/kadath_gb300.h).  Each call turns
// C++ exceptions into status codes and records the message on the context.
#include <cstring>
#include <memory>
#include <string>

#include "kadath_gb300.h"
#include "kd_context.hpp"
#include "kd_spectral.hpp"

struct kd_ctx {
  std::unique_ptr<kd::Context> c;
  std::string err;
};

namespace {

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

int kd_ctx_destroy(kd_ctx* ctx) {
  if (!ctx) return KD_ERR_ARG;
  delete ctx;
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
