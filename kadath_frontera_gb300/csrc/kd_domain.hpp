// Spherical domains of Kadath: nucleus (r < R), shell (R1 < r < R2) and the
// compactified outer domain (r > R, 1/r mapped to [-1, 1]).  Geometry follows
// src/Domain/Spheric/domain_{nucleus,shell,compact}.cpp; the tau/Galerkin
// bookkeeping (which coefficients are unknowns, which residual coefficients
// become equations) is restated from the *_export_tau*, *_affecte_tau* and
// *_nbr_unknowns* files of the same directory and turned into sparse tables
// that the device gathers apply.
#pragma once
#include <string>
#include <utility>
#include <vector>

#include "kd_spectral.hpp"

namespace kd {

enum DomainType : int { DOM_NUCLEUS = 1, DOM_SHELL = 2, DOM_COMPACT = 3 };
enum Boundary : int { OUTER_BC = 0, INNER_BC = 1 };

// One sparse linear combination of coefficients: sum_e w_e * cf[idx_e].
struct SparseRow {
  std::vector<std::pair<int, double>> e;
  void add(int idx, double w) {
    for (auto& p : e)
      if (p.first == idx) {
        p.second += w;
        return;
      }
    e.emplace_back(idx, w);
  }
};

class Domain {
 public:
  Domain(int num, int type, const int npts[3], double a, double b, const double center[3]);

  int num;
  int type;
  int np[3];  // collocation points (r, theta, phi)
  int nc[3];  // coefficients (phi has two more)
  double alpha, beta;
  double center[3];
  std::vector<double> coloc[3];

  int npts() const { return np[0] * np[1] * np[2]; }
  int ncoefs() const { return nc[0] * nc[1] * nc[2]; }
  int cidx(int i, int j, int k) const { return (i * nc[1] + j) * nc[2] + k; }
  int pidx(int i, int j, int k) const { return (i * np[1] + j) * np[2] + k; }
  const char* type_name() const;

  // Radius and Cartesian coordinates at the collocation points (host copies).
  std::vector<double> radius_values() const;
  std::vector<double> cart_values(int c) const;  // c = 0 (x), 1 (y), 2 (z)
  double inner_radius() const;
  double outer_radius() const;

  // Bases (set_cheb_base, set_anti_cheb_base, Cartesian components).
  Base std_base() const;
  Base anti_base() const;
  Base cart_base(int c) const;  // std base of x/y/z components (c = 0, 1, 2)
  // Product rule of bases (Domain_*::mult).
  Base mult(const Base& a, const Base& b) const;

  // ---- tau / Galerkin tables (valence-0 values, mlim as in the reference)
  // Rows of export_tau_val_domain for an equation of given order.
  void export_tau_rows(const Base& b, int mlim, int order, std::vector<SparseRow>& rows) const;
  // Rows of export_tau_val_domain_boundary.
  void export_tau_boundary_rows(const Base& b, int mlim, int bound, std::vector<SparseRow>& rows) const;
  // Coefficient patterns of the unknowns (affecte_tau_one_coef_val_domain),
  // in the reference's unknown order.
  void unknown_patterns(const Base& b, int mlim, std::vector<SparseRow>& pats) const;
  // affecte_tau_val_domain as a map: coef[p] = sum_e w * x[first + e.idx];
  // returns the number of x values the reference consumes.
  int affecte_tau_map(const Base& b, int mlim, std::vector<SparseRow>& coef_rows) const;

  // val_boundary as a row over the r-coefficients of line (j, k).
  void val_boundary_row(int bound, int j, int k, double w, SparseRow& row) const;

  // Scalar::val_point as weights: the value at numerical coordinates
  // num = (xi, theta, phi) is sum_c w[c] cf[c] (Base_spectral::summation,
  // src/Ope_1d/summation_1d.cpp:272).
  void point_weights(const Base& b, const double num[3], std::vector<double>& w) const;

  // Domain_*::integ_volume (domain_{nucleus,shell,compact}_ope.cpp) as
  // weights on the coefficients of the integrand, i.e. of the field already
  // multiplied by r^2 sin(theta) alpha (nucleus, shell) or by
  // -r^4 sin(theta) alpha (compact): the k = 0 modes only, 2/(2j+1) per
  // SIN_ODD theta mode, integral_1d (src/Ope_1d/integral_1d.cpp) along r.
  void integ_volume_row(const Base& integrand, SparseRow& row) const;
  // Domain_compact::integ (domain_compact.cpp:89) at `bound`, as weights on
  // the coefficients of r^2 sin(theta) times the field.
  void integ_surface_row(const Base& integrand, int bound, SparseRow& row) const;

  bool has_boundary(int bound) const;
  void find_other_dom(int dom, int bound, int& other_dom, int& other_bound) const;
};

// Space_spheric (src/Space/Spheric/space_spheric.cpp:25): a nucleus, shells
// between the given radii, and optionally a compactified outer domain.
class Space {
 public:
  Space(const double center[3], const int npts[3], const std::vector<double>& bounds, bool withzec);
  explicit Space(std::vector<Domain> doms) : domains(std::move(doms)) {}
  std::vector<Domain> domains;
  int ndom() const { return static_cast<int>(domains.size()); }
  const Domain& dom(int d) const { return domains.at(d); }
  // Domain holding a Cartesian point and its numerical coordinates
  // (xi, theta, phi); -1 when no domain does.
  int locate(const double point[3], double num[3]) const;
  // Numerical coordinates of a Cartesian point in domain dd
  // (Domain_*::absol_to_num), whether or not the point lies in it.
  void absol_to_num(int dd, const double point[3], double num[3]) const;
};

}  // namespace kd
