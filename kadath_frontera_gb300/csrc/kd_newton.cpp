#include "kd_newton.hpp"

#include <chrono>

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
  cudaFree(d_J);
}

void Newton::ensure(int N) {
  if (static_cast<size_t>(N) > capF_) {
    cudaFree(d_F);
    cuda_check(cudaMalloc(&d_F, sizeof(double) * N), "cudaMalloc(F)");
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
  lu_->factor(d_J, ld, N, o.lu_mode);
  rep.t_factor_ms = lu_->stats.t_factor_ms;
  // the residual vector is solved in place
  lu_->solve(d_F, 0);
  rep.t_solve_ms = lu_->stats.t_solve_ms;
  rep.refine_iters = lu_->stats.refine_iters;
  rep.refine_rel_residual = lu_->stats.final_rel_residual;
  auto t3 = std::chrono::steady_clock::now();
  sys_->update_from_x(d_F);
  rep.t_update_ms = ms_since(t3);
  rep.kernel_launches = ctx->launches - l0;
  return false;
}

}  // namespace kd
