#include "kd_io.hpp"

#include <cstdint>
#include <cstring>

namespace kd {

namespace {

constexpr int KD_CHEB_TYPE = 1;  // Space::type_base of Chebyshev spaces
constexpr int KD_CARTESIAN_BASIS = 0;

// fwrite_be / fread_be: every 4- or 8-byte item stored most significant
// byte first, whatever the host order.
void put_bytes(std::FILE* f, const unsigned char* b, size_t n) {
  if (std::fwrite(b, 1, n, f) != n) throw KdError(KD_ERR_ARG, "write error");
}
void get_bytes(std::FILE* f, unsigned char* b, size_t n) {
  if (std::fread(b, 1, n, f) != n) throw KdError(KD_ERR_ARG, "unexpected end of file");
}
void put_int(std::FILE* f, int v) {
  const uint32_t u = static_cast<uint32_t>(v);
  unsigned char b[4] = {static_cast<unsigned char>(u >> 24), static_cast<unsigned char>(u >> 16),
                        static_cast<unsigned char>(u >> 8), static_cast<unsigned char>(u)};
  put_bytes(f, b, 4);
}
int get_int(std::FILE* f) {
  unsigned char b[4];
  get_bytes(f, b, 4);
  const uint32_t u = (uint32_t(b[0]) << 24) | (uint32_t(b[1]) << 16) | (uint32_t(b[2]) << 8) | uint32_t(b[3]);
  return static_cast<int>(u);
}
void put_double(std::FILE* f, double v) {
  uint64_t u;
  std::memcpy(&u, &v, 8);
  unsigned char b[8];
  for (int i = 0; i < 8; i++) b[i] = static_cast<unsigned char>(u >> (56 - 8 * i));
  put_bytes(f, b, 8);
}
double get_double(std::FILE* f) {
  unsigned char b[8];
  get_bytes(f, b, 8);
  uint64_t u = 0;
  for (int i = 0; i < 8; i++) u = (u << 8) | b[i];
  double v;
  std::memcpy(&v, &u, 8);
  return v;
}

// Dim_array::save: ndim, then the sizes
void put_dims(std::FILE* f, const std::vector<int>& d) {
  put_int(f, static_cast<int>(d.size()));
  for (int v : d) put_int(f, v);
}
std::vector<int> get_dims(std::FILE* f) {
  const int n = get_int(f);
  if (n < 1 || n > 8) throw KdError(KD_ERR_ARG, "bad Dim_array in file");
  std::vector<int> d(n);
  for (auto& v : d) v = get_int(f);
  return d;
}

// Array<int>::save / Array<double>::save: dimensions, count, data
void put_int_array(std::FILE* f, const std::vector<int>& dims, const std::vector<int>& data) {
  put_dims(f, dims);
  put_int(f, static_cast<int>(data.size()));
  for (int v : data) put_int(f, v);
}
std::vector<int> get_int_array(std::FILE* f, std::vector<int>* dims_out) {
  std::vector<int> dims = get_dims(f);
  const int n = get_int(f);
  long long expect = 1;
  for (int v : dims) expect *= v;
  if (n != expect) throw KdError(KD_ERR_ARG, "Array size does not match its dimensions");
  std::vector<int> data(n);
  for (auto& v : data) v = get_int(f);
  if (dims_out) *dims_out = dims;
  return data;
}
void put_double_array(std::FILE* f, const std::vector<int>& dims, const std::vector<double>& data) {
  put_dims(f, dims);
  put_int(f, static_cast<int>(data.size()));
  for (double v : data) put_double(f, v);
}
std::vector<double> get_double_array(std::FILE* f, const std::vector<int>& expect_dims) {
  std::vector<int> dims = get_dims(f);
  if (dims != expect_dims) throw KdError(KD_ERR_ARG, "Array dimensions do not match the domain");
  const int n = get_int(f);
  long long expect = 1;
  for (int v : dims) expect *= v;
  if (n != expect) throw KdError(KD_ERR_ARG, "Array size does not match its dimensions");
  std::vector<double> data(n);
  for (auto& v : data) v = get_double(f);
  return data;
}

// Base_spectral::save: 0 when defined (then ndim and the three tables:
// r (ntheta_c x nphi_c), theta (nphi_c), phi (1)), 1 otherwise
void put_base(std::FILE* f, const Base& b, const Domain& d) {
  put_int(f, b.def ? 0 : 1);
  put_int(f, 3);
  if (!b.def) return;
  put_int_array(f, {d.nc[1], d.nc[2]}, b.r);
  put_int_array(f, {d.nc[2]}, b.t);
  put_int_array(f, {1}, {b.p});
}
Base get_base(std::FILE* f, const Domain& d) {
  const int undefined = get_int(f);
  const int ndim = get_int(f);
  if (ndim != 3) throw KdError(KD_ERR_UNSUPPORTED, "only three-dimensional bases");
  Base b;
  if (undefined) return b;
  b.allocate(d.nc[1], d.nc[2]);
  std::vector<int> dims;
  std::vector<int> r = get_int_array(f, &dims);
  if (dims != std::vector<int>{d.nc[1], d.nc[2]}) throw KdError(KD_ERR_ARG, "radial basis table of another size");
  std::vector<int> t = get_int_array(f, &dims);
  if (dims != std::vector<int>{d.nc[2]}) throw KdError(KD_ERR_ARG, "theta basis table of another size");
  std::vector<int> p = get_int_array(f, &dims);
  if (p.size() != 1) throw KdError(KD_ERR_ARG, "phi basis table of another size");
  b.r = r;
  b.t = t;
  b.p = p[0];
  b.def = true;
  return b;
}

void put_domain(std::FILE* f, const Domain& d) {
  put_dims(f, {d.np[0], d.np[1], d.np[2]});
  put_dims(f, {d.nc[0], d.nc[1], d.nc[2]});
  put_int(f, 3);
  put_int(f, KD_CHEB_TYPE);
  put_int(f, 3);  // Point::save
  for (int i = 0; i < 3; i++) put_double(f, d.center[i]);
  put_double(f, d.alpha);
  if (d.type == DOM_SHELL) put_double(f, d.beta);
}

}  // namespace

void save_space(const Space& sp, std::FILE* f) {
  put_int(f, sp.ndom());
  put_int(f, 3);
  put_int(f, KD_CHEB_TYPE);
  for (const auto& d : sp.domains) put_domain(f, d);
}

std::unique_ptr<Space> load_space(std::FILE* f, bool withzec) {
  const int nd = get_int(f);
  const int ndim = get_int(f);
  const int tb = get_int(f);
  if (nd < 1 || nd > 4096 || ndim != 3) throw KdError(KD_ERR_ARG, "not a three-dimensional Space_spheric file");
  if (tb != KD_CHEB_TYPE) throw KdError(KD_ERR_UNSUPPORTED, "only Chebyshev spaces (CHEB_TYPE)");
  std::vector<Domain> doms;
  for (int i = 0; i < nd; i++) {
    const int type = (i == 0) ? DOM_NUCLEUS : ((withzec && i == nd - 1) ? DOM_COMPACT : DOM_SHELL);
    std::vector<int> np = get_dims(f), nc = get_dims(f);
    if (np.size() != 3 || nc.size() != 3) throw KdError(KD_ERR_ARG, "bad domain dimensions");
    if (get_int(f) != 3 || get_int(f) != KD_CHEB_TYPE) throw KdError(KD_ERR_UNSUPPORTED, "domain of another kind");
    if (get_int(f) != 3) throw KdError(KD_ERR_ARG, "bad domain centre");
    double center[3];
    for (auto& c : center) c = get_double(f);
    const double alpha = get_double(f);
    const double beta = (type == DOM_SHELL) ? get_double(f) : 0.0;
    const int npts[3] = {np[0], np[1], np[2]};
    doms.emplace_back(i, type, npts, alpha, beta, center);
    const Domain& d = doms.back();
    if (d.nc[0] != nc[0] || d.nc[1] != nc[1] || d.nc[2] != nc[2])
      throw KdError(KD_ERR_ARG, "coefficient counts do not match the collocation points");
  }
  return std::make_unique<Space>(std::move(doms));
}

void save_field(Field& fld, std::FILE* f) {
  Context* ctx = fld.ctx;
  for (int dd = 0; dd < fld.sp->ndom(); dd++) {
    const Domain& d = fld.sp->dom(dd);
    const Field::PerDom& p = fld.d[dd];
    put_base(f, p.base, d);
    put_int(f, p.zero ? 1 : 0);
    const bool conf = !p.zero && p.in_conf, coef = !p.zero && p.in_coef;
    put_int(f, conf ? 0 : 1);
    if (conf) {
      std::vector<double> h(d.npts());
      cuda_check(cudaMemcpyAsync(h.data(), p.c, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->stream()),
                 "D2H");
      cuda_check(cudaStreamSynchronize(ctx->stream()), "sync");
      put_double_array(f, {d.np[0], d.np[1], d.np[2]}, h);
    }
    put_int(f, coef ? 0 : 1);
    if (coef) {
      std::vector<double> h(d.ncoefs());
      cuda_check(cudaMemcpyAsync(h.data(), p.cf, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->stream()),
                 "D2H");
      cuda_check(cudaStreamSynchronize(ctx->stream()), "sync");
      put_double_array(f, {d.nc[0], d.nc[1], d.nc[2]}, h);
    }
  }
}

void load_field(Field& fld, std::FILE* f) {
  Context* ctx = fld.ctx;
  for (int dd = 0; dd < fld.sp->ndom(); dd++) {
    const Domain& d = fld.sp->dom(dd);
    Field::PerDom& p = fld.d[dd];
    Base b = get_base(f, d);
    const bool zero = get_int(f) != 0;
    const bool conf = get_int(f) == 0;
    std::vector<double> c, cf;
    if (conf) c = get_double_array(f, {d.np[0], d.np[1], d.np[2]});
    const bool coef = get_int(f) == 0;
    if (coef) cf = get_double_array(f, {d.nc[0], d.nc[1], d.nc[2]});
    if (!zero && !conf && !coef) throw KdError(KD_ERR_ARG, "a nonzero Val_domain without values");
    if (conf)
      cuda_check(cudaMemcpyAsync(p.c, c.data(), sizeof(double) * c.size(), cudaMemcpyHostToDevice, ctx->stream()),
                 "H2D");
    if (coef)
      cuda_check(cudaMemcpyAsync(p.cf, cf.data(), sizeof(double) * cf.size(), cudaMemcpyHostToDevice, ctx->stream()),
                 "H2D");
    cuda_check(cudaStreamSynchronize(ctx->stream()), "sync");
    p.base = b;
    p.zero = zero;
    p.in_conf = !zero && conf;
    p.in_coef = !zero && coef;
  }
}

void save_vector(Field* const comps[3], int type_index, std::FILE* f) {
  if (type_index != 1 && type_index != -1) throw KdError(KD_ERR_ARG, "index type must be CON (+1) or COV (-1)");
  const int nd = comps[0]->sp->ndom();
  put_int_array(f, {nd}, std::vector<int>(nd, KD_CARTESIAN_BASIS));  // Base_tensor::save
  put_int_array(f, {1}, {type_index});                                // type_indice
  put_int(f, 1);                                                      // valence
  put_int(f, 3);                                                      // n_comp
  for (int c = 0; c < 3; c++) save_field(*comps[c], f);
}

void load_vector(Field* const comps[3], int* type_index, std::FILE* f) {
  const int nd = comps[0]->sp->ndom();
  std::vector<int> dims;
  std::vector<int> basis = get_int_array(f, &dims);
  if (static_cast<int>(basis.size()) != nd) throw KdError(KD_ERR_ARG, "tensorial basis of another space");
  for (int b : basis)
    if (b != KD_CARTESIAN_BASIS) throw KdError(KD_ERR_UNSUPPORTED, "only vectors in the Cartesian basis");
  std::vector<int> ti = get_int_array(f, &dims);
  const int valence = get_int(f);
  const int ncomp = get_int(f);
  if (valence != 1 || ti.size() != 1 || ncomp != 3) throw KdError(KD_ERR_UNSUPPORTED, "not a three-component vector");
  if (type_index) *type_index = ti[0];
  for (int c = 0; c < 3; c++) load_field(*comps[c], f);
}

}  // namespace kd
