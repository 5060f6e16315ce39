#include "kd_newton.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>

namespace kd {

namespace {
double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}
}  // namespace

Newton::Newton(System* s) : sys_(s), lu_(new DenseLU(s->ctx)) {}

Newton::~Newton() {
  cudaStreamSynchronize(sys_->ctx->stream());
  cudaFree(d_F);
  cudaFree(d_F0);
  cudaFree(d_J);
  cudaFree(d_JtJ_);
  cudaFree(d_JtF_);
  if (blas_) cublasDestroy(blas_);  cudaGetLastError();  // teardown status is not the next launch's error
}

void Newton::ensure(int N) {
  if (static_cast<size_t>(N) > capF_) {
    cudaFree(d_F);
    cudaFree(d_F0);
    d_F = d_F0 = nullptr;
    cuda_check(cudaMalloc(&d_F, sizeof(double) * N), "cudaMalloc(F)");
    cuda_check(cudaMalloc(&d_F0, sizeof(double) * N), "cudaMalloc(F copy)");
    capF_ = N;
  }
  size_t need = static_cast<size_t>(N) * N;
  if (need > capJ_) {
    cudaFree(d_J);
    cuda_check(cudaMalloc(&d_J, sizeof(double) * need), "cudaMalloc(J)");
    capJ_ = need;
  }
  ld = N;
}

bool Newton::step(const NewtonOpts& o, NewtonReport& rep) {
  Context* ctx = sys_->ctx;
  cudaStream_t s = ctx->stream();
  long long l0 = ctx->launches;
  rep = NewtonReport();
  sys_->set_residual_graph(o.graph_capture != 0);
  auto t0 = std::chrono::steady_clock::now();
  if (sys_->nbr_conditions() < 0) sys_->residual(nullptr);  // fixes nbr_conditions on the first call
  int N = sys_->nbr_conditions();
  ensure(N);
  sys_->residual(d_F, true);  // node values kept for the Jacobian
  double* d_err = ctx->scratch().alloc_doubles(1);
  cuda_check(launch_absmax(d_F, N, d_err, s), "absmax");
  double err = 0;
  cuda_check(cudaMemcpyAsync(&err, d_err, sizeof(double), cudaMemcpyDeviceToHost, s), "D2H err");
  cuda_check(cudaStreamSynchronize(s), "sync residual");
  rep.t_residual_ms = ms_since(t0);
  rep.error = err;
  rep.n = N;
  if (!std::isfinite(err))
    throw KdError(KD_ERR_ARG, "non-finite residual (the fields or constants hold NaN or Inf): no update made");
  if (err < o.precision) {
    rep.converged = 1;
    rep.kernel_launches = ctx->launches - l0;
    return true;
  }
  int nu = sys_->nbr_unknowns();
  if (nu != N)
    throw KdError(KD_ERR_STATE, "Number of unknowns (" + std::to_string(nu) +
                                    ") is different from the number of equations (" + std::to_string(N) + ")");
  auto t1 = std::chrono::steady_clock::now();
  sys_->jacobian(d_J, ld, true);
  cuda_check(cudaStreamSynchronize(s), "sync assembly");
  rep.t_assembly_ms = ms_since(t1);
  lu_->gmres_tol = o.gmres_tol;
  lu_->gmres_max_iter = o.max_refine;
  lu_->gmres_restarts = o.gmres_restarts;
  lu_->reuse_pivots = o.pivot_every_step == 0;
  const bool mixed = o.lu_mode != LU_FP64;
  if (mixed)
    cuda_check(cudaMemcpyAsync(d_F0, d_F, sizeof(double) * N, cudaMemcpyDeviceToDevice, s), "keep F");
  lu_->factor(d_J, ld, N, o.lu_mode);
  rep.t_factor_ms = lu_->stats.t_factor_ms;
  // the residual vector is solved in place
  try {
    lu_->solve(d_F, 0);
  } catch (const KdError& e) {
    if (!mixed || e.code != KD_ERR_NOCONV) throw;
    // the refinement did not reach the FP64 solution: factor the same
    // Jacobian (kept by the mixed modes) in FP64 and solve again
    rep.fp64_fallback = 1;
    lu_->factor(d_J, ld, N, LU_FP64);
    rep.t_factor_ms += lu_->stats.t_factor_ms;
    cuda_check(cudaMemcpyAsync(d_F, d_F0, sizeof(double) * N, cudaMemcpyDeviceToDevice, s), "restore F");
    lu_->solve(d_F, 0);
  }
  rep.t_solve_ms = lu_->stats.t_solve_ms;
  rep.static_pivots = lu_->stats.static_pivots && !lu_->stats.static_pivot_fallback;
  rep.refine_iters = lu_->stats.refine_iters;
  rep.refine_rel_residual = lu_->stats.final_rel_residual;
  auto t3 = std::chrono::steady_clock::now();
  sys_->update_from_x(d_F);
  rep.t_update_ms = ms_since(t3);
  rep.kernel_launches = ctx->launches - l0;
  return false;
}

bool Newton::step_gauss_newton(const NewtonOpts& o, NewtonReport& rep) {
  Context* ctx = sys_->ctx;
  cudaStream_t s = ctx->stream();
  long long l0 = ctx->launches;
  rep = NewtonReport();
  auto t0 = std::chrono::steady_clock::now();
  if (sys_->nbr_conditions() < 0) sys_->residual(nullptr);
  const int m = sys_->nbr_conditions();
  const int n = sys_->nbr_unknowns();
  if (m < n)
    throw KdError(KD_ERR_STATE, "Gauss-Newton needs at least as many conditions (" + std::to_string(m) +
                                    ") as unknowns (" + std::to_string(n) + ")");
  if (static_cast<size_t>(m) > capF_) {
    cudaFree(d_F);
    d_F = nullptr;
    cuda_check(cudaMalloc(&d_F, sizeof(double) * m), "cudaMalloc(F)");
    capF_ = m;
  }
  if (static_cast<size_t>(m) * n > capJ_) {
    cudaFree(d_J);
    d_J = nullptr;
    cuda_check(cudaMalloc(&d_J, sizeof(double) * static_cast<size_t>(m) * n), "cudaMalloc(J)");
    capJ_ = static_cast<size_t>(m) * n;
  }
  if (static_cast<size_t>(n) > capN_) {
    cudaFree(d_JtJ_);
    cudaFree(d_JtF_);
    d_JtJ_ = d_JtF_ = nullptr;
    cuda_check(cudaMalloc(&d_JtJ_, sizeof(double) * static_cast<size_t>(n) * n), "cudaMalloc(JtJ)");
    cuda_check(cudaMalloc(&d_JtF_, sizeof(double) * n), "cudaMalloc(JtF)");
    capN_ = n;
  }
  ld = m;
  sys_->residual(d_F, true);
  double* d_err = ctx->scratch().alloc_doubles(1);
  cuda_check(launch_absmax(d_F, m, d_err, s), "absmax");
  double err = 0;
  cuda_check(cudaMemcpyAsync(&err, d_err, sizeof(double), cudaMemcpyDeviceToHost, s), "D2H err");
  cuda_check(cudaStreamSynchronize(s), "sync residual");
  rep.t_residual_ms = ms_since(t0);
  rep.error = err;
  rep.n = n;
  if (err < o.precision) {
    rep.converged = 1;
    rep.kernel_launches = ctx->launches - l0;
    return true;
  }
  auto t1 = std::chrono::steady_clock::now();
  sys_->jacobian(d_J, m, true, true);
  // J^T F and J^T J (library FP64 products, as pdgemv / pdgemm)
  if (!blas_ && cublasCreate(&blas_) != CUBLAS_STATUS_SUCCESS) throw KdError(KD_ERR_CUDA, "cublasCreate failed");
  cublasSetStream(blas_, s);
  const double one = 1.0, zero = 0.0;
  if (cublasDgemv(blas_, CUBLAS_OP_T, m, n, &one, d_J, m, d_F, 1, &zero, d_JtF_, 1) != CUBLAS_STATUS_SUCCESS ||
      cublasDgemm(blas_, CUBLAS_OP_T, CUBLAS_OP_N, n, n, m, &one, d_J, m, d_J, m, &zero, d_JtJ_, n) !=
          CUBLAS_STATUS_SUCCESS)
    throw KdError(KD_ERR_CUDA, "normal equations (cuBLAS) failed");
  ctx->launches += 2;
  cuda_check(cudaStreamSynchronize(s), "sync assembly");
  rep.t_assembly_ms = ms_since(t1);
  lu_->gmres_tol = o.gmres_tol;
  lu_->gmres_max_iter = o.max_refine;
  lu_->gmres_restarts = o.gmres_restarts;
  lu_->reuse_pivots = o.pivot_every_step == 0;
  lu_->factor(d_JtJ_, n, n, o.lu_mode);
  rep.t_factor_ms = lu_->stats.t_factor_ms;
  lu_->solve(d_JtF_, 0);
  rep.t_solve_ms = lu_->stats.t_solve_ms;
  rep.refine_iters = lu_->stats.refine_iters;
  rep.refine_rel_residual = lu_->stats.final_rel_residual;
  auto t3 = std::chrono::steady_clock::now();
  sys_->update_from_x(d_JtF_);
  rep.t_update_ms = ms_since(t3);
  rep.kernel_launches = ctx->launches - l0;
  return false;
}

double Newton::device_scalar(const double* d_x, long long n, int op) {
  Context* ctx = sys_->ctx;
  double* d = ctx->scratch().alloc_doubles(1);
  cuda_check(launch_reduce1(d_x, n, op, d, ctx->stream()), "reduce");
  ctx->launches++;
  double h = 0;
  cuda_check(cudaMemcpyAsync(&h, d, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream()), "D2H");
  cuda_check(cudaStreamSynchronize(ctx->stream()), "sync");
  return h;
}

// compute_f (src_par/do_newton.cpp:594): sum of F^2 of a fresh sec_member.
double Newton::residual_norm2() {
  int N = sys_->nbr_conditions();
  sys_->residual(d_F);
  return device_scalar(d_F, N, 0);
}

bool Newton::step_linesearch(const NewtonOpts& o, int ntrymax, double stepmax, NewtonReport& rep,
                             double* lambda_out) {
  Context* ctx = sys_->ctx;
  cudaStream_t s = ctx->stream();
  long long l0 = ctx->launches;
  rep = NewtonReport();
  if (lambda_out) *lambda_out = 0.0;
  auto t0 = std::chrono::steady_clock::now();
  if (sys_->nbr_conditions() < 0) sys_->residual(nullptr);
  const int N = sys_->nbr_conditions();
  ensure(N);
  sys_->residual(d_F, true);
  double* d_err = ctx->scratch().alloc_doubles(1);
  cuda_check(launch_absmax(d_F, N, d_err, s), "absmax");
  double err = 0;
  cuda_check(cudaMemcpyAsync(&err, d_err, sizeof(double), cudaMemcpyDeviceToHost, s), "D2H err");
  cuda_check(cudaStreamSynchronize(s), "sync residual");
  rep.t_residual_ms = ms_since(t0);
  rep.error = err;
  rep.n = N;
  if (err < o.precision) {
    rep.converged = 1;
    rep.kernel_launches = ctx->launches - l0;
    return true;
  }
  if (sys_->nbr_unknowns() != N) throw KdError(KD_ERR_STATE, "Number of unknowns is different from the number of equations");
  const double fold = device_scalar(d_F, N, 0);
  const double slope = -2.0 * fold;
  if (!(slope < 0.0)) throw KdError(KD_ERR_NOCONV, "line search: the slope is not negative");  // check_negative
  // p = J^-1 F (compute_p)
  auto t1 = std::chrono::steady_clock::now();
  sys_->jacobian(d_J, ld, true);
  cuda_check(cudaStreamSynchronize(s), "sync assembly");
  rep.t_assembly_ms = ms_since(t1);
  lu_->gmres_tol = o.gmres_tol;
  lu_->gmres_max_iter = o.max_refine;
  lu_->gmres_restarts = o.gmres_restarts;
  lu_->reuse_pivots = o.pivot_every_step == 0;
  lu_->factor(d_J, ld, N, o.lu_mode);
  rep.t_factor_ms = lu_->stats.t_factor_ms;
  lu_->solve(d_F, 0);
  rep.t_solve_ms = lu_->stats.t_solve_ms;
  rep.refine_iters = lu_->stats.refine_iters;
  rep.refine_rel_residual = lu_->stats.final_rel_residual;
  auto t3 = std::chrono::steady_clock::now();
  const double pmax = device_scalar(d_F, N, 1);  // max(p), signed as in the reference
  ctx->scratch().reset();
  ls_arena_.reset();
  // old fields and the fields xx_to_vars(p) would give (compute_old_and_var)
  const int nvar = static_cast<int>(sys_->vars().size());
  const int nd = sys_->sp->ndom();
  std::vector<std::vector<DVal>> old(nvar), pv(nvar);
  std::vector<double> hp(N);
  cuda_check(cudaMemcpyAsync(hp.data(), d_F, sizeof(double) * N, cudaMemcpyDeviceToHost, s), "D2H p");
  cuda_check(cudaStreamSynchronize(s), "sync p");
  const double scale = (pmax > stepmax) ? stepmax / pmax : 1.0;  // rescale in case p is too large
  {
    DeviceArena* prev = ctx->redirect_scratch(&ls_arena_);
    try {
      for (int v = 0; v < nvar; v++) {
        Field* f = sys_->vars()[v].f;
        for (int dd = 0; dd < nd; dd++) {
          DVal ov = copy_to_arena(ctx, f->val(dd), ls_arena_);
          old[v].push_back(ov);
          if (dd < sys_->dom_min || dd > sys_->dom_max) {
            pv[v].push_back(ov);  // xx_to_vars leaves these domains as they are
          } else {
            DVal p = sys_->x_to_field(v, dd, d_F);
            pv[v].push_back(scale == 1.0 ? p : p * scale);
          }
        }
      }
    } catch (...) {
      ctx->redirect_scratch(prev);
      throw;
    }
    ctx->redirect_scratch(prev);
  }
  std::vector<double> old_d, p_d;
  for (int i = 0; i < sys_->n_var_doubles(); i++) {
    old_d.push_back(sys_->var_double(i));
    p_d.push_back(hp[i] * scale);
  }
  auto update_fields = [&](double lambda) {
    ctx->scratch().reset();
    for (int i = 0; i < static_cast<int>(old_d.size()); i++) sys_->set_var_double(i, old_d[i] - lambda * p_d[i]);
    for (int v = 0; v < nvar; v++) {
      Field* f = sys_->vars()[v].f;
      for (int dd = 0; dd < nd; dd++) {
        DVal nv = old[v][dd] - pv[v][dd] * lambda;
        f->assign(dd, nv);
      }
    }
    sys_->invalidate_values();
  };
  const double lambdamin = 1.0e-10, alpha = 1.0e-4;
  double lambda = 1.0, lambdatmp = 0.0, lambda2 = 0.0, f2 = 0.0;
  for (int itry = 1; itry <= ntrymax; ++itry) {
    update_fields(lambda);
    const double f = residual_norm2();
    if (f <= 5.0e-13) break;
    if (f <= fold + alpha * lambda * slope || lambda <= lambdamin) break;
    if (lambda == 1.0) {
      lambdatmp = -0.5 * slope / (f - fold - slope);
    } else {
      const double rhs1 = f - fold - lambda * slope;
      const double rhs2 = f2 - fold - lambda2 * slope;
      const double a = (rhs1 / (lambda * lambda) - rhs2 / (lambda2 * lambda2)) / (lambda - lambda2);
      const double b = (-lambda2 * rhs1 / (lambda * lambda) + lambda * rhs2 / (lambda2 * lambda2)) / (lambda - lambda2);
      if (a == 0.0) lambdatmp = -0.5 * slope / b;
      const double delta = b * b - 3.0 * a * slope;
      if (delta < 0.0) throw KdError(KD_ERR_NOCONV, "line search: negative discriminant");  // check_positive
      lambdatmp = (-b + std::sqrt(delta)) / (3.0 * a);
      if (lambdatmp > 0.5 * lambda) lambdatmp = 0.5 * lambda;
    }
    lambda2 = lambda;
    f2 = f;
    lambda = std::max(lambdatmp, 0.1 * lambda);
    if (itry == ntrymax) update_fields(lambda);
  }
  if (lambda_out) *lambda_out = lambda;
  rep.t_update_ms = ms_since(t3);
  rep.kernel_launches = ctx->launches - l0;
  return false;
}

double Newton::adjoint(const double* g, int cst, double dq_explicit, double* lambda_out, bool reuse_factors,
                       AdjointReport* rep) {
  Context* ctx = sys_->ctx;
  cudaStream_t s = ctx->stream();
  if (sys_->nbr_conditions() < 0) sys_->residual(nullptr);
  const int N = sys_->nbr_conditions();
  if (sys_->nbr_unknowns() != N) throw KdError(KD_ERR_STATE, "Number of unknowns is different from the number of equations");
  // mixed factors of the last Newton step of this size, whose refinement
  // operator is d_J (the buffer the assembly below overwrites with J at the
  // current fields)
  const bool have_mixed = lu_->mode() != LU_FP64 && lu_->n() == N && d_J != nullptr && lu_->op() == d_J &&
                          static_cast<size_t>(N) * static_cast<size_t>(ld) <= capJ_;
  ensure(N);
  AdjointReport r;
  auto t0 = std::chrono::steady_clock::now();
  sys_->residual(d_F, true);
  sys_->jacobian(d_J, ld, true);
  cuda_check(cudaStreamSynchronize(s), "sync adjoint assembly");
  r.t_assembly_ms = ms_since(t0);
  double* d = nullptr;
  cuda_check(cudaMalloc(&d, sizeof(double) * 2 * N), "cudaMalloc(adjoint)");
  struct Free {
    double* p;
    ~Free() { cudaFree(p); }
  } guard{d};
  double* d_lambda = d;
  double* d_fp = d + N;
  t0 = std::chrono::steady_clock::now();
  if (reuse_factors && have_mixed) {
    cuda_check(cudaMemcpyAsync(d_lambda, g, sizeof(double) * N, cudaMemcpyHostToDevice, s), "H2D g");
    try {
      lu_->solve(d_lambda, 1);  // GMRES on J^T, preconditioned by the step's factors transposed
      r.reused_factors = 1;
    } catch (const KdError& e) {
      if (e.code != KD_ERR_NOCONV) throw;
    }
  }
  if (!r.reused_factors) {
    lu_->factor(d_J, ld, N, LU_FP64);
    cuda_check(cudaMemcpyAsync(d_lambda, g, sizeof(double) * N, cudaMemcpyHostToDevice, s), "H2D g");
    lu_->solve(d_lambda, 1);  // J^T lambda = g with the FP64 factors
  }
  cuda_check(cudaStreamSynchronize(s), "sync adjoint solve");
  r.t_solve_ms = ms_since(t0);
  r.refine_iters = r.reused_factors ? lu_->stats.refine_iters : 0;
  r.rel_residual = r.reused_factors ? lu_->stats.final_rel_residual : 0.0;
  if (rep) *rep = r;
  sys_->dres_dcst(cst, d_fp);
  std::vector<double> lam(N), fp(N);
  cuda_check(cudaMemcpyAsync(lam.data(), d_lambda, sizeof(double) * N, cudaMemcpyDeviceToHost, s), "D2H lambda");
  cuda_check(cudaMemcpyAsync(fp.data(), d_fp, sizeof(double) * N, cudaMemcpyDeviceToHost, s), "D2H dF/dp");
  cuda_check(cudaStreamSynchronize(s), "sync adjoint");
  double dot = 0.0;
  for (int i = 0; i < N; i++) dot += lam[i] * fp[i];
  if (lambda_out) std::copy(lam.begin(), lam.end(), lambda_out);
  return dq_explicit - dot;
}

}  // namespace kd
