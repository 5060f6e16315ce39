// Spectral basis codes and 1-D coefficient-space operators, turned into small
// dense matrices that the device kernels apply line by line.
//
// Basis codes and their meaning follow Kadath's include/base_spectral.hpp:27-42
// (CHEB=1 ... COSSIN_ODD=15).  Every 1-D operator of the reference
// (src/Coef/coef_1d.cpp, src/Coef/coef_i_1d.cpp, src/Ope_1d/*.cpp) is linear in
// its input line, so it is restated here once, applied to unit vectors, and the
// resulting columns are cached as an n_out x n_in FP64 matrix together with
// the basis the operator returns.
#pragma once
#include <cstddef>
#include <map>
#include <string>
#include <tuple>
#include <vector>

namespace kd {

enum Basis : int {
  BASE_UNDEF = 0,
  CHEB = 1,
  CHEB_EVEN = 2,
  CHEB_ODD = 3,
  COSSIN = 4,
  COS = 5,
  COS_EVEN = 6,
  COS_ODD = 7,
  SIN = 8,
  SIN_EVEN = 9,
  SIN_ODD = 10,
  LEG = 11,
  LEG_EVEN = 12,
  LEG_ODD = 13,
  COSSIN_EVEN = 14,
  COSSIN_ODD = 15,
};

// 1-D operators.  OP_COEF/OP_COEF_I are the forward/inverse transforms; the
// others act on coefficients and may change the basis of the line.
enum Op1d : int {
  OP_COEF = 0,
  OP_COEF_I = 1,
  OP_DER = 2,
  OP_MULT_SIN = 3,
  OP_DIV_SIN = 4,
  OP_MULT_COS = 5,
  OP_DIV_COS = 6,
  OP_MULT_X = 7,
  OP_DIV_X = 8,
  OP_MULT_XM1 = 9,
  OP_DIV_XM1 = 10,
  OP_DIV_XP1 = 11,
  OP_DIV_1MX2 = 12,
  OP_IDENTITY = 13,
  // Coefficients of n_in terms -> values at the n_out standard collocation
  // points of the basis's grid (Scalar::val_point at those points, as the
  // FUKA regrid does it): the rows are summation_weights_1d there.
  OP_RESAMPLE = 14,
  OP_COUNT = 15,
};

const char* basis_name(int b);
const char* op_name(int op);

// Applies one 1-D operator to `tab` in place.  `tab` has max(n_in, n_out)
// entries; for OP_COEF the first n_in entries are collocation values and the
// first n_out entries on return are coefficients (and the reverse for
// OP_COEF_I).  Returns the output basis, or -1 when the reference has no
// implementation for (op, basis) (its *_pasprevu branch, which aborts).
int apply_1d(int op, int basis, std::vector<double>& tab, int n_in, int n_out);

struct Mat1d {
  int op = 0, basis = 0, n_in = 0, n_out = 0, out_basis = -1;
  std::vector<double> m;  // row-major n_out x n_in
  size_t pool_offset = 0; // offset (in doubles) inside the device matrix pool
};

// Builds the matrix of (op, basis) for a line of n_in inputs and n_out outputs.
// Returns false if the reference does not implement the pair.
bool build_matrix(int op, int basis, int n_in, int n_out, Mat1d& out);

// Weights of the evaluation of one coefficient line at x: the value of the
// line is sum_i w[i] * tab[i] (summation_1d_<basis>,
// src/Ope_1d/summation_1d.cpp:30-236).  false for an unknown basis.
bool summation_weights_1d(int basis, int n, double x, double* w);

// Host-side cache of every matrix a plan uses, uploaded as one device pool.
class MatrixBank {
 public:
  // Returns the index of the matrix in the bank (creating it if needed), or -1.
  int get(int op, int basis, int n_in, int n_out);
  const Mat1d& at(int idx) const { return mats_[idx]; }
  size_t pool_size() const { return pool_.size(); }
  const std::vector<double>& pool() const { return pool_; }
  size_t version() const { return version_; }

 private:
  std::map<std::tuple<int, int, int, int>, int> index_;
  std::vector<Mat1d> mats_;
  std::vector<double> pool_;
  size_t version_ = 0;
};

}  // namespace kd
