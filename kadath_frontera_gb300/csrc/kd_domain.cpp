#include "kd_domain.hpp"

#include <cmath>
#include <sstream>

namespace kd {

namespace {
const double PI = 3.14159265358979323846;

inline double sgn_pow(int i) { return (i % 2 == 0) ? 1.0 : -1.0; }  // pow(-1, i)

// Parity signature of the theta bases used by the product rule:
// s1 = +1 for cosines, -1 for sines; s2 = parity of the harmonic family.
bool theta_sig(int b, int& s1, int& s2) {
  switch (b) {
    case COS_EVEN: s1 = 1; s2 = 1; return true;
    case COS_ODD: s1 = 1; s2 = -1; return true;
    case SIN_EVEN: s1 = -1; s2 = -1; return true;
    case SIN_ODD: s1 = -1; s2 = 1; return true;
    default: return false;
  }
}
int theta_from_sig(int s1, int s2) {
  if (s1 > 0) return s2 > 0 ? COS_EVEN : COS_ODD;
  return s2 > 0 ? SIN_ODD : SIN_EVEN;
}
}  // namespace

Domain::Domain(int num_, int type_, const int npts[3], double a, double b, const double c[3])
    : num(num_), type(type_), alpha(a), beta(b) {
  for (int d = 0; d < 3; d++) {
    np[d] = npts[d];
    nc[d] = npts[d];
    center[d] = c[d];
  }
  nc[2] += 2;  // do_coloc: nbr_coefs(2) += 2
  coloc[0].resize(np[0]);
  coloc[1].resize(np[1]);
  coloc[2].resize(np[2]);
  for (int i = 0; i < np[0]; i++)
    coloc[0][i] = (type == DOM_NUCLEUS) ? std::sin(PI / 2. * i / (np[0] - 1)) : -std::cos(PI * i / (np[0] - 1));
  for (int j = 0; j < np[1]; j++) coloc[1][j] = PI / 2. * j / (np[1] - 1);
  for (int k = 0; k < np[2]; k++) coloc[2][k] = PI * 2. * k / np[2];
}

const char* Domain::type_name() const {
  switch (type) {
    case DOM_NUCLEUS: return "nucleus";
    case DOM_SHELL: return "shell";
    default: return "compact";
  }
}

std::vector<double> Domain::radius_values() const {
  std::vector<double> r(npts());
  for (int i = 0; i < np[0]; i++) {
    double x = coloc[0][i];
    double rr;
    if (type == DOM_NUCLEUS) rr = alpha * x;
    else if (type == DOM_SHELL) rr = alpha * x + beta;
    else rr = 1. / alpha / (x - 1);  // infinite at x = 1, as in the reference
    for (int j = 0; j < np[1]; j++)
      for (int k = 0; k < np[2]; k++) r[pidx(i, j, k)] = rr;
  }
  return r;
}

std::vector<double> Domain::cart_values(int c) const {
  std::vector<double> v(npts());
  auto r = radius_values();
  for (int i = 0; i < np[0]; i++)
    for (int j = 0; j < np[1]; j++)
      for (int k = 0; k < np[2]; k++) {
        double rr = r[pidx(i, j, k)];
        double th = coloc[1][j], ph = coloc[2][k];
        double val;
        if (c == 0) val = rr * std::sin(th) * std::cos(ph) + center[0];
        else if (c == 1) val = rr * std::sin(th) * std::sin(ph) + center[1];
        else val = rr * std::cos(th) + center[2];
        v[pidx(i, j, k)] = val;
      }
  return v;
}

double Domain::inner_radius() const {
  if (type == DOM_NUCLEUS) return 0.0;
  if (type == DOM_SHELL) return beta - alpha;
  return -0.5 / alpha;
}

double Domain::outer_radius() const {
  if (type == DOM_NUCLEUS) return alpha;
  if (type == DOM_SHELL) return beta + alpha;
  return INFINITY;
}

Base Domain::std_base() const {
  Base b;
  b.allocate(nc[1], nc[2]);
  b.def = true;
  b.p = COSSIN;
  for (int k = 0; k < nc[2]; k++) {
    int m = (k % 2 == 0) ? k / 2 : (k - 1) / 2;
    b.t[k] = (m % 2 == 0) ? COS_EVEN : SIN_ODD;
    for (int j = 0; j < nc[1]; j++) {
      if (type == DOM_NUCLEUS) {
        int l = (m % 2 == 0) ? 2 * j : 2 * j + 1;
        b.rb(j, k) = (l % 2 == 0) ? CHEB_EVEN : CHEB_ODD;
      } else {
        b.rb(j, k) = CHEB;
      }
    }
  }
  return b;
}

Base Domain::anti_base() const {
  Base b;
  b.allocate(nc[1], nc[2]);
  b.def = true;
  b.p = COSSIN;
  for (int k = 0; k < nc[2]; k++) {
    int m = (k % 2 == 0) ? k / 2 : (k - 1) / 2;
    b.t[k] = (m % 2 == 0) ? COS_ODD : SIN_EVEN;
    for (int j = 0; j < nc[1]; j++) {
      if (type == DOM_NUCLEUS) {
        int l = (m % 2 == 0) ? 2 * j + 1 : 2 * j;
        b.rb(j, k) = (l % 2 == 1) ? CHEB_ODD : CHEB_EVEN;
      } else {
        b.rb(j, k) = CHEB;
      }
    }
  }
  return b;
}

Base Domain::cart_base(int c) const {
  // Domain::set_cheb_base_{x,y,z}_cart (src/Domain/domain.cpp:1258-1273),
  // not overridden by the spherical domains: x and y components take the
  // symmetric standard basis, z the antisymmetric one.
  return (c == 2) ? anti_base() : std_base();
}

// Domain_{shell,nucleus,compact}::mult (domain_shell.cpp:684, domain_nucleus.cpp:548):
// phi: COSSIN x COSSIN; theta and nucleus-r: parity rules that flip with the
// parity of m of the phi slot.
Base Domain::mult(const Base& a, const Base& b) const {
  Base res;
  if (!a.def || !b.def) return res;
  if (a.p != COSSIN || b.p != COSSIN) return res;
  res.allocate(a.n1c, a.n2c);
  res.p = COSSIN;
  for (int k = 0; k < a.n2c; k++) {
    int s1a, s2a, s1b, s2b;
    if (!theta_sig(a.t[k], s1a, s2a) || !theta_sig(b.t[k], s1b, s2b)) return Base();
    bool meven = (k % 4 < 2);
    int s1 = s1a * s1b * (meven ? 1 : -1);
    res.t[k] = theta_from_sig(s1, s2a * s2b);
  }
  for (int j = 0; j < a.n1c; j++)
    for (int k = 0; k < a.n2c; k++) {
      int ra = a.rb(j, k), rb = b.rb(j, k);
      if (type == DOM_NUCLEUS) {
        if ((ra != CHEB_EVEN && ra != CHEB_ODD) || (rb != CHEB_EVEN && rb != CHEB_ODD)) return Base();
        int pa = (ra == CHEB_EVEN) ? 1 : -1, pb = (rb == CHEB_EVEN) ? 1 : -1;
        bool meven = (k % 4 < 2);
        int p = pa * pb * (meven ? 1 : -1);
        res.rb(j, k) = (p > 0) ? CHEB_EVEN : CHEB_ODD;
      } else {
        if (ra != CHEB || rb != CHEB) return Base();
        res.rb(j, k) = CHEB;
      }
    }
  res.def = true;
  return res;
}

// ------------------------------------------------------------------ tau --
void Domain::val_boundary_row(int bound, int j, int k, double w, SparseRow& row) const {
  // Domain_*::val_boundary (domain_*_systems.cpp): sum of the radial
  // coefficients at x = 1, alternating sum at x = -1.
  for (int i = 0; i < nc[0]; i++) {
    double s = (bound == INNER_BC) ? sgn_pow(i) : 1.0;
    row.add(cidx(i, j, k), w * s);
  }
}

void Domain::integ_volume_row(const Base& b, SparseRow& row) const {
  row.e.clear();
  if (b.t.at(0) != SIN_ODD) throw KdError(KD_ERR_UNSUPPORTED, "integ_volume: theta basis of m = 0 is not SIN_ODD");
  const int want = (type == DOM_NUCLEUS) ? CHEB_EVEN : CHEB;
  for (int j = 0; j < nc[1]; j++) {
    if (b.rb(j, 0) != want) throw KdError(KD_ERR_UNSUPPORTED, "integ_volume: unexpected radial basis");
    const double wt = 2.0 / (2.0 * j + 1) * 2 * M_PI;
    for (int i = 0; i < nc[0]; i++) {
      double w1;
      if (want == CHEB_EVEN) {
        w1 = -1.0 / (4.0 * i * i - 1);  // integral_1d_cheb_even
      } else {
        if (i % 2 == 1) continue;
        w1 = -2.0 / (i * i - 1.0);  // integral_1d_cheb
      }
      row.add(cidx(i, j, 0), wt * w1);
    }
  }
}

void Domain::integ_surface_row(const Base& b, int bound, SparseRow& row) const {
  row.e.clear();
  if (type != DOM_COMPACT) throw KdError(KD_ERR_UNSUPPORTED, "integ() is only defined in the compactified domain");
  switch (b.t.at(0)) {
    case COS_ODD:
    case SIN_EVEN:
      break;
    case COS_EVEN:
      val_boundary_row(bound, 0, 0, M_PI * 2 * M_PI, row);
      break;
    case SIN_ODD:
      for (int j = 0; j < nc[1]; j++) val_boundary_row(bound, j, 0, 2.0 / (2 * double(j) + 1) * 2 * M_PI, row);
      break;
    default:
      throw KdError(KD_ERR_UNSUPPORTED, "integ: theta basis not handled");
  }
}

bool Domain::has_boundary(int bound) const {
  if (type == DOM_NUCLEUS) return bound == OUTER_BC;
  if (type == DOM_COMPACT) return true;
  return bound == INNER_BC || bound == OUTER_BC;
}

void Domain::find_other_dom(int dom, int bound, int& other_dom, int& other_bound) const {
  if (bound == INNER_BC) {
    if (type == DOM_NUCLEUS) throw KdError(KD_ERR_ARG, "nucleus has no inner boundary");
    other_dom = dom - 1;
    other_bound = OUTER_BC;
  } else {
    if (type == DOM_COMPACT) throw KdError(KD_ERR_ARG, "Domain_compact::find_other_dom: no outer neighbour");
    other_dom = dom + 1;
    other_bound = INNER_BC;
  }
}

void Domain::export_tau_rows(const Base& b, int mlim, int order, std::vector<SparseRow>& rows) const {
  const int kmin = 2 * mlim + 2;
  rows.clear();
  if (type != DOM_NUCLEUS) {
    // domain_shell_export_tau.cpp:27 (the compact domain has the same code)
    for (int k = 0; k < nc[2] - 1; k++) {
      if (k == 1) continue;
      int bt = b.t[k];
      for (int j = 0; j < nc[1]; j++)
        for (int i = 0; i < nc[0] - order; i++) {
          SparseRow r;
          switch (bt) {
            case COS_EVEN:
              if (k < kmin) r.add(cidx(i, j, k), 1.0);
              else if (j != 0) {
                r.add(cidx(i, j, k), 1.0);
                r.add(cidx(i, 0, k), -2.0);
              }
              break;
            case COS_ODD:
              if (j != nc[1] - 1) {
                if (k < kmin) r.add(cidx(i, j, k), 1.0);
                else if (j != 0) {
                  r.add(cidx(i, j, k), 1.0);
                  r.add(cidx(i, 0, k), -1.0);
                }
              }
              break;
            case SIN_EVEN:
              if (j != 0 && j != nc[1] - 1) {
                if (k < kmin + 2) r.add(cidx(i, j, k), 1.0);
                else if (j != 1) {
                  r.add(cidx(i, j, k), 1.0);
                  r.add(cidx(i, 1, k), -double(j));
                }
              }
              break;
            case SIN_ODD:
              if (j != nc[1] - 1) {
                if (k < kmin + 2) r.add(cidx(i, j, k), 1.0);
                else if (j != 0) {
                  r.add(cidx(i, j, k), 1.0);
                  r.add(cidx(i, 0, k), -double(2 * j + 1));
                }
              }
              break;
            default:
              throw KdError(KD_ERR_UNSUPPORTED, "Unknown theta basis in export_tau_val_domain");
          }
          if (!r.e.empty()) rows.push_back(std::move(r));
        }
    }
    return;
  }
  // domain_nucleus_export_tau.cpp:764 (standard case, CHEB parity bases)
  int rlim = (order == 0) ? 1 : 2;
  const int llim = 0;
  for (int k = 0; k < nc[2] - 1; k++) {
    if (k == 1) continue;
    int bt = b.t[k];
    for (int j = 0; j < nc[1]; j++) {
      int br = b.rb(j, k);
      for (int i = 0; i < nc[0]; i++) {
        SparseRow r;
        int lq;
        switch (bt) {
          case COS_EVEN:
            if (br != CHEB_EVEN) throw KdError(KD_ERR_UNSUPPORTED, "nucleus COS_EVEN needs CHEB_EVEN");
            lq = 2 * j;
            if (k < kmin && lq <= llim) {
              if (i != nc[0] - rlim + 1) r.add(cidx(i, j, k), 1.0);
            } else if (k < kmin) {
              if (i != 0 && i != nc[0] - rlim + 1) {
                r.add(cidx(i, j, k), 1.0);
                r.add(cidx(0, j, k), -2 * sgn_pow(i));
              }
            } else if (j != 0 && i != 0 && i != nc[0] - rlim + 1) {
              r.add(cidx(i, j, k), 1.0);
              r.add(cidx(0, j, k), -2 * sgn_pow(i));
              r.add(cidx(i, 0, k), -2.0);
              r.add(cidx(0, 0, k), 4 * sgn_pow(i));
            }
            break;
          case COS_ODD:
            if (br != CHEB_ODD) throw KdError(KD_ERR_UNSUPPORTED, "nucleus COS_ODD needs CHEB_ODD");
            lq = 2 * j + 1;
            if (j != nc[1] - 1 && i != nc[0] - rlim + 1 && i != nc[0] - rlim) {
              if (k < kmin && lq <= llim + 1) r.add(cidx(i, j, k), 1.0);
              else if (k < kmin && i != 0) {
                r.add(cidx(i, j, k), 1.0);
                r.add(cidx(0, j, k), -(2 * i + 1) * sgn_pow(i));
              } else if (j != 0 && i != 0) {
                r.add(cidx(i, j, k), 1.0);
                r.add(cidx(0, j, k), -sgn_pow(i) * (2 * i + 1));
                r.add(cidx(i, 0, k), -1.0);
                r.add(cidx(0, 0, k), sgn_pow(i) * (2 * i + 1));
              }
            }
            break;
          case SIN_EVEN:
            if (br != CHEB_EVEN) throw KdError(KD_ERR_UNSUPPORTED, "nucleus SIN_EVEN needs CHEB_EVEN");
            lq = 2 * j;
            if (j != 0 && j != nc[1] - 1 && i != nc[0] - rlim + 1) {
              if (k < kmin + 2 && lq <= llim) r.add(cidx(i, j, k), 1.0);
              else if (k < kmin + 2 && i != 0) {
                r.add(cidx(i, j, k), 1.0);
                r.add(cidx(0, j, k), -2 * sgn_pow(i));
              } else if (!(k < kmin + 2) && j != 1 && i != 0) {
                r.add(cidx(i, j, k), 1.0);
                r.add(cidx(0, j, k), -sgn_pow(i));
                r.add(cidx(i, 1, k), -double(j));
                r.add(cidx(0, 1, k), sgn_pow(i) * j);
              }
            }
            break;
          case SIN_ODD:
            if (br != CHEB_ODD) throw KdError(KD_ERR_UNSUPPORTED, "nucleus SIN_ODD needs CHEB_ODD");
            lq = 2 * j + 1;
            if (j != nc[1] - 1 && i != nc[0] - rlim + 1 && i != nc[0] - rlim) {
              if (k < kmin + 2 && lq <= llim + 1) r.add(cidx(i, j, k), 1.0);
              else if (k < kmin + 2 && i != 0) {
                r.add(cidx(i, j, k), 1.0);
                r.add(cidx(0, j, k), -(2 * i + 1) * sgn_pow(i));
              } else if (j != 0 && i != 0) {
                r.add(cidx(i, j, k), 1.0);
                r.add(cidx(0, j, k), -sgn_pow(i) * (2 * i + 1));
                r.add(cidx(i, 0, k), -double(2 * j + 1));
                r.add(cidx(0, 0, k), sgn_pow(i) * (2 * i + 1) * (2 * j + 1));
              }
            }
            break;
          default:
            throw KdError(KD_ERR_UNSUPPORTED, "Unknown theta basis in Domain_nucleus::export_tau_val_domain");
        }
        if (!r.e.empty()) rows.push_back(std::move(r));
      }
    }
  }
}

void Domain::export_tau_boundary_rows(const Base& b, int mlim, int bound, std::vector<SparseRow>& rows) const {
  // domain_shell_export_tau_boundary.cpp:27 and domain_nucleus_export_tau_boundary.cpp:262
  // (same angular structure; the radial sum is val_boundary).
  if (!has_boundary(bound)) throw KdError(KD_ERR_ARG, "unknown boundary for this domain");
  const int kmin = 2 * mlim + 2;
  rows.clear();
  for (int k = 0; k < nc[2] - 1; k++) {
    if (k == 1) continue;
    int bt = b.t[k];
    for (int j = 0; j < nc[1]; j++) {
      SparseRow r;
      switch (bt) {
        case COS_EVEN:
          if (k < kmin) val_boundary_row(bound, j, k, 1.0, r);
          else if (j != 0) {
            val_boundary_row(bound, j, k, 1.0, r);
            val_boundary_row(bound, 0, k, -2.0, r);
          }
          break;
        case COS_ODD:
          if (j != nc[1] - 1) {
            if (k < kmin) val_boundary_row(bound, j, k, 1.0, r);
            else if (j != 0) {
              val_boundary_row(bound, j, k, 1.0, r);
              val_boundary_row(bound, 0, k, -1.0, r);
            }
          }
          break;
        case SIN_EVEN:
          if (j != 0 && j != nc[1] - 1) {
            if (k < kmin + 2) val_boundary_row(bound, j, k, 1.0, r);
            else if (j != 1) {
              val_boundary_row(bound, j, k, 1.0, r);
              val_boundary_row(bound, 1, k, -double(j), r);
            }
          }
          break;
        case SIN_ODD:
          if (j != nc[1] - 1) {
            if (k < kmin + 2) val_boundary_row(bound, j, k, 1.0, r);
            else if (j != 0) {
              val_boundary_row(bound, j, k, 1.0, r);
              val_boundary_row(bound, 0, k, -double(2 * j + 1), r);
            }
          }
          break;
        default:
          throw KdError(KD_ERR_UNSUPPORTED, "Unknown theta basis in export_tau_val_domain_boundary");
      }
      bool counted = false;
      // A row is emitted whenever the reference increments pos_sec.
      switch (bt) {
        case COS_EVEN: counted = (k < kmin) || (j != 0); break;
        case COS_ODD: counted = (j != nc[1] - 1) && ((k < kmin) || (j != 0)); break;
        case SIN_EVEN: counted = (j != 0 && j != nc[1] - 1) && ((k < kmin + 2) || (j != 1)); break;
        case SIN_ODD: counted = (j != nc[1] - 1) && ((k < kmin + 2) || (j != 0)); break;
      }
      if (counted) rows.push_back(std::move(r));
    }
  }
}

void Domain::unknown_patterns(const Base& b, int mlim, std::vector<SparseRow>& pats) const {
  const int kmin = 2 * mlim + 2;
  pats.clear();
  if (type != DOM_NUCLEUS) {
    // domain_shell_affecte_tau_one_coef.cpp:26 (same in the compact domain)
    for (int k = 0; k < nc[2] - 1; k++) {
      if (k == 1) continue;
      int bt = b.t[k];
      for (int j = 0; j < nc[1]; j++) {
        bool tt = true;
        switch (bt) {
          case COS_EVEN: if (j == 0 && k >= kmin) tt = false; break;
          case COS_ODD: if (j == nc[1] - 1 || (j == 0 && k >= kmin)) tt = false; break;
          case SIN_EVEN: if ((j == 1 && k >= kmin + 2) || j == 0 || j == nc[1] - 1) tt = false; break;
          case SIN_ODD: if ((j == 0 && k >= kmin + 2) || j == nc[1] - 1) tt = false; break;
          default: throw KdError(KD_ERR_UNSUPPORTED, "Unknown theta basis in affecte_tau_one_coef");
        }
        if (!tt) continue;
        for (int i = 0; i < nc[0]; i++) {
          SparseRow p;
          p.add(cidx(i, j, k), 1.0);
          if ((bt == COS_EVEN || bt == COS_ODD) && k >= kmin) p.add(cidx(i, 0, k), -1.0);
          if (bt == SIN_EVEN && k >= kmin + 2) p.add(cidx(i, 1, k), -double(j));
          if (bt == SIN_ODD && k >= kmin + 2) p.add(cidx(i, 0, k), -double(2 * j + 1));
          pats.push_back(std::move(p));
        }
      }
    }
    return;
  }
  // domain_nucleus_affecte_tau_one_coef.cpp:853 (standard case, llim = 0)
  const int llim = 0;
  for (int k = 0; k < nc[2] - 1; k++) {
    if (k == 1) continue;
    int bt = b.t[k];
    for (int j = 0; j < nc[1]; j++) {
      for (int i = 0; i < nc[0]; i++) {
        SparseRow p;
        bool unk = false;
        int lq;
        switch (bt) {
          case COS_EVEN:
            lq = 2 * j;
            if (k < kmin && lq <= llim) {
              unk = true;
              p.add(cidx(i, j, k), 1.0);
            } else if (k < kmin) {
              if (i != 0) {
                unk = true;
                p.add(cidx(i, j, k), 1.0);
                p.add(cidx(0, j, k), -sgn_pow(i));
              }
            } else if (j != 0 && i != 0) {
              unk = true;
              p.add(cidx(i, j, k), 1.0);
              p.add(cidx(0, j, k), -sgn_pow(i));
              p.add(cidx(i, 0, k), -1.0);
              p.add(cidx(0, 0, k), sgn_pow(i));
            }
            break;
          case COS_ODD:
            lq = 2 * j + 1;
            if (j != nc[1] - 1 && i != nc[0] - 1) {
              if (k < kmin && lq <= llim + 1) {
                unk = true;
                p.add(cidx(i, j, k), 1.0);
              } else if (k < kmin && i != 0) {
                unk = true;
                p.add(cidx(i, j, k), 1.0);
                p.add(cidx(0, j, k), -(2 * i + 1) * sgn_pow(i));
              } else if (!(k < kmin) && j != 0 && i != 0) {
                unk = true;
                p.add(cidx(i, j, k), 1.0);
                p.add(cidx(0, j, k), -sgn_pow(i) * (2 * i + 1));
                p.add(cidx(i, 0, k), -1.0);
                p.add(cidx(0, 0, k), sgn_pow(i) * (2 * i + 1));
              }
            }
            break;
          case SIN_EVEN:
            lq = 2 * j;
            if (j != 0 && j != nc[1] - 1) {
              if (k < kmin + 2 && lq <= llim) {
                unk = true;
                p.add(cidx(i, j, k), 1.0);
              } else if (k < kmin + 2 && i != 0) {
                unk = true;
                p.add(cidx(i, j, k), 1.0);
                p.add(cidx(0, j, k), -sgn_pow(i));
              } else if (!(k < kmin + 2) && j != 1 && i != 0) {
                unk = true;
                p.add(cidx(i, j, k), 1.0);
                p.add(cidx(0, j, k), -sgn_pow(i));
                p.add(cidx(i, 1, k), -double(j));
                p.add(cidx(0, 1, k), sgn_pow(i) * j);
              }
            }
            break;
          case SIN_ODD:
            lq = 2 * j + 1;
            if (j != nc[1] - 1 && i != nc[0] - 1) {
              if (k < kmin + 2 && lq <= llim + 1) {
                unk = true;
                p.add(cidx(i, j, k), 1.0);
              } else if (k < kmin + 2 && i != 0) {
                unk = true;
                p.add(cidx(i, j, k), 1.0);
                p.add(cidx(0, j, k), -(2 * i + 1) * sgn_pow(i));
              } else if (!(k < kmin + 2) && j != 0 && i != 0) {
                unk = true;
                p.add(cidx(i, j, k), 1.0);
                p.add(cidx(0, j, k), -sgn_pow(i) * (2 * i + 1));
                p.add(cidx(i, 0, k), -double(2 * j + 1));
                p.add(cidx(0, 0, k), sgn_pow(i) * (2 * i + 1) * (2 * j + 1));
              }
            }
            break;
          default:
            throw KdError(KD_ERR_UNSUPPORTED, "Unknown theta basis in Domain_nucleus::affecte_tau_one_coef");
        }
        if (unk) pats.push_back(std::move(p));
      }
    }
  }
}

int Domain::affecte_tau_map(const Base& b, int mlim, std::vector<SparseRow>& coef_rows) const {
  coef_rows.assign(ncoefs(), SparseRow());
  if (type == DOM_NUCLEUS) {
    // domain_nucleus_affecte_tau.cpp:770 adds values(conte) times the same
    // patterns as affecte_tau_one_coef, in the same order.
    std::vector<SparseRow> pats;
    unknown_patterns(b, mlim, pats);
    for (size_t u = 0; u < pats.size(); u++)
      for (auto& e : pats[u].e) coef_rows[e.first].add(static_cast<int>(u), e.second);
    return static_cast<int>(pats.size());
  }
  // domain_shell_affecte_tau.cpp:26: true coefficients take the values, then
  // the Galerkin slots are set from the others ("regularisation").
  const int kmin = 2 * mlim + 2;
  int conte = 0;
  for (int k = 0; k < nc[2] - 1; k++) {
    if (k == 1) continue;
    int bt = b.t[k];
    for (int j = 0; j < nc[1]; j++) {
      bool tt = true;
      switch (bt) {
        case COS_EVEN: if (j == 0 && k >= kmin) tt = false; break;
        case COS_ODD: if (j == nc[1] - 1 || (j == 0 && k >= kmin)) tt = false; break;
        case SIN_EVEN: if ((j == 1 && k >= kmin + 2) || j == 0 || j == nc[1] - 1) tt = false; break;
        // the reference uses k > kmin+2 here (k >= kmin+2 elsewhere)
        case SIN_ODD: if ((j == 0 && k > kmin + 2) || j == nc[1] - 1) tt = false; break;
        default: throw KdError(KD_ERR_UNSUPPORTED, "Unknown theta basis in affecte_tau_val_domain");
      }
      if (!tt) continue;
      for (int i = 0; i < nc[0]; i++) coef_rows[cidx(i, j, k)].add(conte++, 1.0);
    }
  }
  for (int k = 0; k < nc[2] - 1; k++) {
    int bt = b.t[k];
    for (int i = 0; i < nc[0]; i++) {
      int gal_j = -1, jstart = 0;
      bool on = false;
      if ((bt == COS_EVEN || bt == COS_ODD) && k >= kmin) { on = true; gal_j = 0; jstart = 1; }
      if (bt == SIN_EVEN && k >= kmin + 2) { on = true; gal_j = 1; jstart = 2; }
      if (bt == SIN_ODD && k >= kmin + 2) { on = true; gal_j = 0; jstart = 1; }
      if (!on) continue;
      SparseRow sum;
      for (int j = jstart; j < nc[1]; j++) {
        double w = 1.0;
        if (bt == SIN_EVEN) w = j;
        if (bt == SIN_ODD) w = 2 * j + 1;
        for (auto& e : coef_rows[cidx(i, j, k)].e) sum.add(e.first, -w * e.second);
      }
      coef_rows[cidx(i, gal_j, k)] = sum;
    }
  }
  return conte;
}

Space::Space(const double center[3], const int npts[3], const std::vector<double>& bounds, bool withzec) {
  if (bounds.empty()) throw KdError(KD_ERR_ARG, "Space_spheric needs at least one radius");
  for (size_t i = 1; i < bounds.size(); i++)
    if (!(bounds[i] > bounds[i - 1])) throw KdError(KD_ERR_ARG, "radii must increase");
  int nd = withzec ? static_cast<int>(bounds.size()) + 1 : static_cast<int>(bounds.size());
  domains.emplace_back(0, DOM_NUCLEUS, npts, bounds[0], 0.0, center);
  int nshell = withzec ? nd - 1 : nd;
  for (int i = 1; i < nshell; i++)
    domains.emplace_back(i, DOM_SHELL, npts, (bounds[i] - bounds[i - 1]) / 2., (bounds[i] + bounds[i - 1]) / 2.,
                         center);
  if (withzec) domains.emplace_back(nd - 1, DOM_COMPACT, npts, -0.5 / bounds[nd - 2], 0.0, center);
}

void Domain::point_weights(const Base& b, const double num[3], std::vector<double>& w) const {
  if (!b.def) throw KdError(KD_ERR_STATE, "val_point of a field without a basis");
  w.assign(ncoefs(), 0.0);
  std::vector<double> wr(nc[0]), wt(nc[1]), wp(nc[2]);
  if (!summation_weights_1d(b.p, nc[2], num[2], wp.data())) throw KdError(KD_ERR_UNSUPPORTED, "val_point: basis");
  for (int k = 0; k < nc[2]; k++) {
    if (!summation_weights_1d(b.t[k], nc[1], num[1], wt.data())) throw KdError(KD_ERR_UNSUPPORTED, "val_point: basis");
    for (int j = 0; j < nc[1]; j++) {
      if (!summation_weights_1d(b.r[static_cast<size_t>(j) * b.n2c + k], nc[0], num[0], wr.data()))
        throw KdError(KD_ERR_UNSUPPORTED, "val_point: basis");
      for (int i = 0; i < nc[0]; i++) w[cidx(i, j, k)] = wr[i] * wt[j] * wp[k];
    }
  }
}

int Space::locate(const double point[3], double num[3]) const {
  const Domain& d0 = domains.at(0);
  const double x = point[0] - d0.center[0], y = point[1] - d0.center[1], z = point[2] - d0.center[2];
  const double r = std::sqrt(x * x + y * y + z * z);
  int dd = -1;
  for (const Domain& d : domains)
    if (d.inner_radius() - 1e-12 <= r && r <= d.outer_radius() + 1e-12) {
      dd = d.num;
      break;
    }
  if (dd < 0) return -1;
  absol_to_num(dd, point, num);
  return dd;
}

void Space::absol_to_num(int dd, const double point[3], double num[3]) const {
  const Domain& d0 = domains.at(0);
  const double x = point[0] - d0.center[0], y = point[1] - d0.center[1], z = point[2] - d0.center[2];
  const double r = std::sqrt(x * x + y * y + z * z);
  const Domain& d = domains.at(dd);
  if (d.type == DOM_NUCLEUS) num[0] = r / d.alpha;
  else if (d.type == DOM_SHELL) num[0] = (r - d.beta) / d.alpha;
  else num[0] = 1.0 + 1.0 / r / d.alpha;
  const double rho = std::sqrt(x * x + y * y);
  double th, ph;
  if (rho == 0.0) {
    th = (z >= 0) ? 0.0 : M_PI;
    ph = 0.0;
  } else {
    th = (z != 0.0) ? std::atan(rho / z) : M_PI / 2;
    ph = std::atan2(y, x);
  }
  if (th < 0) th += M_PI;
  num[1] = th;
  num[2] = ph;
}

}  // namespace kd
