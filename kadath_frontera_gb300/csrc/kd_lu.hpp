// Dense LU with partial pivoting on the GPU, replacing Matrice::set_lu /
// Matrice::solve (src/Matrice/matrice.cpp:192-249, LAPACK dgetrf/dgetrs)
// and the ScaLAPACK pdgesv of src_par/do_newton.cpp:317.
//
// Matrices are column-major with leading dimension ld.  Modes:
//   KD_LU_FP64      blocked right-looking LU, FP64 trailing updates
//   KD_LU_TF32_IR   FP32 working copy, trailing updates on tcgen05 tensor
//                   cores in TF32 with FP32 accumulation, then FP64 GMRES
//                   iterative refinement against the FP64 matrix
#pragma once
#include <cublas_v2.h>

#include "kd_context.hpp"

namespace kd {

enum LuMode : int { LU_FP64 = 0, LU_TF32_IR = 1, LU_FP32_IR = 2 };

struct LuStats {
  double t_factor_ms = 0, t_solve_ms = 0;
  int refine_iters = 0;
  double final_rel_residual = 0;
  long long flops = 0;
  int static_pivots = 0;          // the factors used a reused pivot order
  int static_pivot_fallback = 0;  // that order failed and partial pivoting was redone
};

class DenseLU {
 public:
  explicit DenseLU(Context* ctx);
  ~DenseLU();

  // Factors the N x N matrix A (device, FP64, column-major, ld).  For the
  // FP64 mode A is overwritten by its factors; for the mixed modes A is kept
  // (it is the refinement operator) and an FP32 copy is factored.
  void factor(double* A, long long ld, int N, int mode);
  // Solves A x = b in place (b on the device).  Mixed modes run GMRES-IR.
  void solve(double* b, int trans = 0);
  // Transposed solve with the same factors (A^T x = b), FP64 mode only.
  void solve_transposed(double* b) { solve(b, 1); }

  int mode() const { return mode_; }
  int n() const { return N_; }
  const double* op() const { return A_; }  // the FP64 matrix of the last factor() call
  LuStats stats;
  double gmres_tol = 1e-14;
  int gmres_max_iter = 50;   // GMRES iterations per cycle
  int gmres_restarts = 4;    // cycles (restarts) of GMRES(gmres_max_iter)
  int nb = 128;
  // TF32 mode: 3 = 3xTF32 trailing updates (about FP32 accurate factors,
  // fewer refinement iterations), 1 = plain TF32 products.
  int tf32_terms = 3;
  // Mixed modes: factor D_r A D_c (power-of-two row and column scales), the
  // refinement works on A itself.
  bool equilibrate = true;
  // Mixed modes: a factorisation of a matrix of the size of the last
  // partial-pivoting one reuses its pivot order (static pivoting: the rows
  // are gathered in that order and factored without row search; GMRES-IR
  // against the FP64 matrix restores the accuracy).  When the refinement
  // does not converge with those factors, the matrix is factored again with
  // partial pivoting; when it needs more than 4 iterations beyond the
  // pivoted factors' count, the next factorisation pivots again.
  bool reuse_pivots = false;
  // Triangular sweeps: 2 = three consecutive 64-row blocks per CTA chained
  // in shared memory, finished blocks pulled through a progress counter;
  // 1 = one block per CTA, pulled; 0 = one grid barrier per block.
  int sweep_kind = 2;
  // Forgets the pivot order: the next factorisation pivots.
  void forget_pivots() { perm_n_ = 0; }

 private:
  Context* ctx_;
  cublasHandle_t blas_ = nullptr;
  int mode_ = 0, N_ = 0;
  long long ld_ = 0;
  double* A_ = nullptr;        // FP64 matrix (factors in FP64 mode, operator in mixed modes)
  float* A32_ = nullptr;       // FP32 factors (mixed modes), leading dimension ld32_
  long long ld32_ = 0;
  size_t a32_cap_ = 0;
  int* ipiv_ = nullptr;        // device pivots
  size_t ipiv_cap_ = 0;
  int* d_info_ = nullptr;
  int nsm_ = 0;                // SM count (grid of the panel kernel)
  void* slot_mem_ = nullptr;   // panel exchange slots, barrier, row-move list
  int* swap_map_ = nullptr;
  int* panel_err_ = nullptr;   // set when a grid barrier wait runs out (panel or sweep)
  unsigned* tri_bar_ = nullptr;  // barrier counters of the two triangular sweeps
  unsigned* np_done_ = nullptr;  // CTAs of a static panel that have finished (the last one resets it)
  double* eq_buf_ = nullptr;   // row scales, column scales, row maxima (mixed modes)
  size_t eq_cap_ = 0;
  bool scaled_ = false;
  double* part_ = nullptr;     // split-K partial sums of the FP64 matvec
  size_t part_cap_ = 0;
  void gemv(const double* x, double* y, double alpha, double beta, const double* b, int trans = 0);
  double* work_ = nullptr;     // solver workspace
  size_t work_cap_ = 0;
  double* hproj_ = nullptr;    // pinned host copy of one GMRES step's projections and norm
  size_t hproj_cap_ = 0;
  float* work32_ = nullptr;
  size_t work32_cap_ = 0;

  void ensure_work(size_t n);
  void factor_fp64(double* A, long long ld, int N);
  void factor_f32(float* A, long long ld, int N, bool tf32);
  void solve_fp64(const double* LU, long long ld, int N, double* b, int trans);
  void solve_f32(double* b, int trans = 0);  // applies the FP32 factors to an FP64 vector
  template <class T>
  void tri_solve(const T* LU, long long ld, int N, double* b, int trans);
  template <class T>
  void prepare_solves(const T* LU, long long ld, int N, bool keep_perm);
  void factor_f32_nopiv(float* A, long long ld, int N, bool tf32);
  void factor_mixed(double* A, long long ld, int N, int mode, const int* perm);
  int read_info();
  void check_sweeps();
  void ensure_bsave();
  bool nopiv_ = false;        // the current factors are static-pivot ones
  int perm_n_ = 0;            // N of the pivot order in perm_ (0: none)
  int pivoted_iters_ = 1000;  // refinement iterations with the last pivoted factors
  double* bsave_ = nullptr;   // right-hand side kept for a re-solve
  size_t bsave_cap_ = 0;
  double* dinv_l_ = nullptr;  // inverses of the 64 x 64 diagonal blocks
  double* dinv_u_ = nullptr;
  float2* dinv2_l_ = nullptr;  // the same as (hi, lo) FP32 pairs (sweeps with FP32 factors)
  float2* dinv2_u_ = nullptr;
  size_t dinv_cap_ = 0;
  int* perm_ = nullptr;       // pivots as one permutation
  double* tri_work_ = nullptr;
  size_t perm_cap_ = 0;
  void gmres_ir(double* b, int trans = 0);
};

}  // namespace kd
