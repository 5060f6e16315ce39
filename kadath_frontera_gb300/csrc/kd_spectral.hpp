// Base_spectral for 3-D spherical-type domains and the separable transforms
// built on it (reference: include/base_spectral.hpp:69, src/Coef/coef.cpp,
// src/Coef/coef_i.cpp, src/Ope_1d/ope_1d.cpp).
#pragma once
#include <vector>

#include "kd_context.hpp"

namespace kd {

// bases_1d[0] is a (nc1 x nc2) table (row-major, index j*nc2+k), bases_1d[1]
// has nc2 entries, bases_1d[2] one entry -- as in Base_spectral::allocate for
// 3-D domains (src/Base_spectral/base_spectral.cpp:92-104).
struct Base {
  bool def = false;
  int n1c = 0, n2c = 0;
  std::vector<int> r;
  std::vector<int> t;
  int p = 0;

  void allocate(int nc1, int nc2) {
    n1c = nc1;
    n2c = nc2;
    r.assign(static_cast<size_t>(nc1) * nc2, 0);
    t.assign(nc2, 0);
    p = 0;
  }
  int& rb(int j, int k) { return r[static_cast<size_t>(j) * n2c + k]; }
  int rb(int j, int k) const { return r[static_cast<size_t>(j) * n2c + k]; }
  bool operator==(const Base& o) const {
    if (def != o.def) return false;
    if (!def) return true;
    return r == o.r && t == o.t && p == o.p;
  }
  bool operator!=(const Base& o) const { return !(*this == o); }
};

// One 1-D operator applied along `dim` to a coefficient (or value) block of
// dims `d` with per-line bases from `base`.  The output basis table of that
// dim is written to `base_out` (Base_spectral::ope_1d, src/Ope_1d/ope_1d.cpp:25).
LinePassSpec ope_1d_spec(Context& ctx, int op, int dim, const Base& base, const int d[3], Base& base_out);

// Pass lists of the full forward (phi, theta, r) and inverse (r, theta, phi)
// transforms (Base_spectral::coef / coef_i).
std::vector<LinePassSpec> coef_specs(Context& ctx, const Base& base, const int np[3], const int nc[3]);
std::vector<LinePassSpec> coef_i_specs(Context& ctx, const Base& base, const int np[3], const int nc[3]);

// Pass list of the evaluation of a field given by coefficients (dims
// nc_old) at the collocation points of another resolution (np_new) of the
// same domain: r, theta, then phi, each line through OP_RESAMPLE.
std::vector<LinePassSpec> resample_specs(Context& ctx, const Base& base, const int nc_old[3], const int np_new[3]);

// Turns pass specs into a kernel item (device tables resolved through ctx).
KdItem make_item(Context& ctx, const std::vector<LinePassSpec>& specs, const double* in, double* out,
                 const int dims_in[3], long long in_stride, long long out_stride, double scale);

}  // namespace kd
