#include "kd_spectral.hpp"

#include <sstream>

namespace kd {

namespace {

int mat_offset(Context& ctx, int op, int basis, int n_in, int n_out, int* out_basis) {
  int idx = ctx.bank().get(op, basis, n_in, n_out);
  if (idx < 0) {
    std::ostringstream os;
    os << "1-D operator " << op_name(op) << " not defined for basis " << basis_name(basis) << " (n=" << n_in
       << ")";
    throw KdError(KD_ERR_UNSUPPORTED, os.str());
  }
  const Mat1d& m = ctx.bank().at(idx);
  if (out_basis) *out_basis = m.out_basis;
  return static_cast<int>(m.pool_offset);
}

}  // namespace

LinePassSpec ope_1d_spec(Context& ctx, int op, int dim, const Base& base, const int d[3], Base& base_out) {
  if (!base.def) throw KdError(KD_ERR_STATE, "basis not defined in ope_1d");
  LinePassSpec s;
  s.dim = dim;
  s.n_in = d[dim];
  s.n_out = d[dim];
  s.mat_ld = base.n2c;
  if (dim == 0) {
    s.offsets.resize(base.r.size());
    for (int j = 0; j < base.n1c; j++)
      for (int k = 0; k < base.n2c; k++) {
        int ob;
        s.offsets[j * base.n2c + k] = mat_offset(ctx, op, base.rb(j, k), d[0], d[0], &ob);
        base_out.rb(j, k) = ob;
      }
  } else if (dim == 1) {
    s.offsets.resize(base.t.size());
    for (int k = 0; k < base.n2c; k++) {
      int ob;
      s.offsets[k] = mat_offset(ctx, op, base.t[k], d[1], d[1], &ob);
      base_out.t[k] = ob;
    }
  } else {
    int ob;
    s.offsets.assign(1, mat_offset(ctx, op, base.p, d[2], d[2], &ob));
    base_out.p = ob;
  }
  return s;
}

std::vector<LinePassSpec> coef_specs(Context& ctx, const Base& base, const int np[3], const int nc[3]) {
  if (!base.def) throw KdError(KD_ERR_STATE, "Base not defined in Val_domain::coef");
  std::vector<LinePassSpec> v(3);
  // phi first (coef.cpp:98-99 loops d = ndim-1 .. 0)
  v[0].dim = 2;
  v[0].n_in = np[2];
  v[0].n_out = nc[2];
  v[0].mat_ld = 0;
  v[0].offsets = {mat_offset(ctx, OP_COEF, base.p, np[2], nc[2], nullptr)};
  v[1].dim = 1;
  v[1].n_in = np[1];
  v[1].n_out = nc[1];
  v[1].mat_ld = 0;
  v[1].offsets.resize(nc[2]);
  for (int k = 0; k < nc[2]; k++) v[1].offsets[k] = mat_offset(ctx, OP_COEF, base.t[k], np[1], nc[1], nullptr);
  v[2].dim = 0;
  v[2].n_in = np[0];
  v[2].n_out = nc[0];
  v[2].mat_ld = nc[2];
  v[2].offsets.resize(static_cast<size_t>(nc[1]) * nc[2]);
  for (int j = 0; j < nc[1]; j++)
    for (int k = 0; k < nc[2]; k++)
      v[2].offsets[j * nc[2] + k] = mat_offset(ctx, OP_COEF, base.rb(j, k), np[0], nc[0], nullptr);
  return v;
}

std::vector<LinePassSpec> coef_i_specs(Context& ctx, const Base& base, const int np[3], const int nc[3]) {
  if (!base.def) throw KdError(KD_ERR_STATE, "Base not defined in Val_domain::coef_i");
  std::vector<LinePassSpec> v(3);
  v[0].dim = 0;
  v[0].n_in = nc[0];
  v[0].n_out = np[0];
  v[0].mat_ld = nc[2];
  v[0].offsets.resize(static_cast<size_t>(nc[1]) * nc[2]);
  for (int j = 0; j < nc[1]; j++)
    for (int k = 0; k < nc[2]; k++)
      v[0].offsets[j * nc[2] + k] = mat_offset(ctx, OP_COEF_I, base.rb(j, k), nc[0], np[0], nullptr);
  v[1].dim = 1;
  v[1].n_in = nc[1];
  v[1].n_out = np[1];
  v[1].mat_ld = 0;
  v[1].offsets.resize(nc[2]);
  for (int k = 0; k < nc[2]; k++) v[1].offsets[k] = mat_offset(ctx, OP_COEF_I, base.t[k], nc[1], np[1], nullptr);
  v[2].dim = 2;
  v[2].n_in = nc[2];
  v[2].n_out = np[2];
  v[2].mat_ld = 0;
  v[2].offsets = {mat_offset(ctx, OP_COEF_I, base.p, nc[2], np[2], nullptr)};
  return v;
}

std::vector<LinePassSpec> resample_specs(Context& ctx, const Base& base, const int nc_old[3], const int np_new[3]) {
  if (!base.def) throw KdError(KD_ERR_STATE, "Base not defined in the resampling");
  std::vector<LinePassSpec> v(3);
  v[0].dim = 0;
  v[0].n_in = nc_old[0];
  v[0].n_out = np_new[0];
  v[0].mat_ld = nc_old[2];
  v[0].offsets.resize(static_cast<size_t>(nc_old[1]) * nc_old[2]);
  for (int j = 0; j < nc_old[1]; j++)
    for (int k = 0; k < nc_old[2]; k++)
      v[0].offsets[j * nc_old[2] + k] = mat_offset(ctx, OP_RESAMPLE, base.rb(j, k), nc_old[0], np_new[0], nullptr);
  v[1].dim = 1;
  v[1].n_in = nc_old[1];
  v[1].n_out = np_new[1];
  v[1].mat_ld = 0;
  v[1].offsets.resize(nc_old[2]);
  for (int k = 0; k < nc_old[2]; k++)
    v[1].offsets[k] = mat_offset(ctx, OP_RESAMPLE, base.t[k], nc_old[1], np_new[1], nullptr);
  v[2].dim = 2;
  v[2].n_in = nc_old[2];
  v[2].n_out = np_new[2];
  v[2].mat_ld = 0;
  v[2].offsets = {mat_offset(ctx, OP_RESAMPLE, base.p, nc_old[2], np_new[2], nullptr)};
  return v;
}

KdItem make_item(Context& ctx, const std::vector<LinePassSpec>& specs, const double* in, double* out,
                 const int dims_in[3], long long in_stride, long long out_stride, double scale) {
  KdItem it{};
  it.in = in;
  it.out = out;
  it.in_stride = in_stride;
  it.out_stride = out_stride;
  it.n0 = dims_in[0];
  it.n1 = dims_in[1];
  it.n2 = dims_in[2];
  it.npass = static_cast<int>(specs.size());
  it.scale = scale;
  if (it.npass > 3) throw KdError(KD_ERR_ARG, "at most three passes per item");
  for (int q = 0; q < it.npass; q++) {
    it.pass[q].dim = specs[q].dim;
    it.pass[q].n_in = specs[q].n_in;
    it.pass[q].n_out = specs[q].n_out;
    it.pass[q].mat_ld = specs[q].mat_ld;
    it.pass[q].mat = ctx.table(specs[q].offsets);
  }
  return it;
}

}  // namespace kd
