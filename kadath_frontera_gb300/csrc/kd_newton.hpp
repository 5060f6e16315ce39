// One Newton-Raphson step with the semantics of System_of_eqs::do_newton
// (src_par/do_newton.cpp:65-430) and do_newton_seq (:519-572):
//   F = sec_member(); error = max|F|; if error < precision -> true, no update
//   else assemble J, solve J x = F, fields <- fields - x, return false.
#pragma once
#include <memory>

#include "kd_lu.hpp"
#include "kd_system.hpp"

namespace kd {

struct NewtonOpts {
  double precision = 1e-10;
  int lu_mode = LU_FP64;
  double gmres_tol = 1e-14;
  int max_refine = 50;
  int gmres_restarts = 4;
  int graph_capture = 0;
  int pivot_every_step = 0;
};

struct NewtonReport {
  double error = 0;
  int converged = 0;
  int n = 0;
  double t_residual_ms = 0, t_assembly_ms = 0, t_factor_ms = 0, t_solve_ms = 0, t_update_ms = 0;
  int refine_iters = 0;
  double refine_rel_residual = 0;
  long long kernel_launches = 0;
  int fp64_fallback = 0;
  int static_pivots = 0;
};

class Newton {
 public:
  explicit Newton(System* s);
  ~Newton();
  bool step(const NewtonOpts& o, NewtonReport& rep);
  // The Gauss-Newton variant (do_newton with SOLVER GAUSS_NEWTON,
  // src_par/do_newton.cpp:264-311): for nbr_conditions m >= nbr_unknowns n,
  // solve the normal equations (J^T J) x = J^T F (the m x n Jacobian,
  // J^T J and J^T F in FP64), then fields <- fields - x.
  bool step_gauss_newton(const NewtonOpts& o, NewtonReport& rep);
  // System_of_eqs::do_newton_with_linesearch (src_par/do_newton.cpp:454-516,
  // Numerical Recipes 2007 section 9.7.1): the Newton direction p = J^-1 F
  // (scaled so that max(p) <= stepmax), then fields = old - lambda p with
  // lambda backtracked (quadratic, then cubic model of f = sum F^2) until the
  // sufficient-decrease test holds, at most ntrymax tries.  rep.linesearch_lambda
  // gets the last lambda.
  bool step_linesearch(const NewtonOpts& o, int ntrymax, double stepmax, NewtonReport& rep, double* lambda_out);
  // Adjoint sensitivity at a converged state (implicit-function theorem):
  // F(u0 + A y, p) = 0 with A the unknown coefficient patterns, so
  // dQ/dp = dQ_explicit - lambda . dF/dp with J^T lambda = g, g = dQ/dy.
  // J is assembled at the current fields.  With reuse_factors and
  // mixed-precision factors from the last Newton step in hand, J^T lambda = g
  // is solved by GMRES on that J^T preconditioned by those factors
  // transposed (no new factorisation); otherwise, or when that refinement
  // does not converge, J is factored in FP64 and solved with the transposed
  // factors.  g and lambda_out (nullable) are host vectors of N.
  struct AdjointReport {
    int reused_factors = 0;
    int refine_iters = 0;
    double rel_residual = 0;
    double t_assembly_ms = 0, t_solve_ms = 0;
  };
  double adjoint(const double* g, int cst, double dq_explicit, double* lambda_out, bool reuse_factors = false,
                 AdjointReport* rep = nullptr);
  // Device buffers of the last step (valid until the next call).
  double* d_F = nullptr;
  double* d_J = nullptr;
  double* d_F0 = nullptr;  // copy of F kept for an FP64 re-solve when the mixed solve does not converge
  long long ld = 0;
  DenseLU& lu() { return *lu_; }
  void ensure(int N);

 private:
  System* sys_;
  std::unique_ptr<DenseLU> lu_;
  size_t capF_ = 0, capJ_ = 0;
  double* d_JtJ_ = nullptr;  // Gauss-Newton normal matrix and right-hand side
  double* d_JtF_ = nullptr;
  size_t capN_ = 0;
  cublasHandle_t blas_ = nullptr;
  DeviceArena ls_arena_{size_t(64) << 20};  // field snapshots of a line search
  double device_scalar(const double* d_x, long long n, int op);
  double residual_norm2();
};

}  // namespace kd
