/*
 * kadath_gb300.h -- C ABI of the GB300 Newton-Raphson hot path for Kadath/FUKA.
 *
 * Every entry point returns an int status (KD_OK on success) and never
 * aborts; kd_last_error(ctx) gives the message of the last failure.  Pointers
 * are plain host pointers unless an argument says "device".  All arithmetic
 * behind these calls runs in CUDA kernels on the context's GPU; there is no
 * CPU fallback.
 *
 * Each declaration names the reference interface (path:line inside the
 * Kadath/FUKA tree) whose behaviour it reproduces.
 */
#ifndef KADATH_GB300_H
#define KADATH_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define KD_OK 0
#define KD_ERR_ARG 1
#define KD_ERR_CUDA 2
#define KD_ERR_SINGULAR 3
#define KD_ERR_NOCONV 4
#define KD_ERR_TIMEOUT 5
#define KD_ERR_UNSUPPORTED 6
#define KD_ERR_STATE 7

/* Spectral basis codes: include/base_spectral.hpp:27-42. */
#define KD_CHEB 1
#define KD_CHEB_EVEN 2
#define KD_CHEB_ODD 3
#define KD_COSSIN 4
#define KD_COS 5
#define KD_COS_EVEN 6
#define KD_COS_ODD 7
#define KD_SIN 8
#define KD_SIN_EVEN 9
#define KD_SIN_ODD 10
#define KD_COSSIN_EVEN 14
#define KD_COSSIN_ODD 15

/* Boundaries: include/headcpp.hpp (INNER_BC / OUTER_BC). */
#define KD_OUTER_BC 0
#define KD_INNER_BC 1

typedef struct kd_ctx kd_ctx;

/* ---- context ----------------------------------------------------------- */
int kd_ctx_create(kd_ctx** out, int device);
int kd_ctx_destroy(kd_ctx* ctx);
/* No reference counterpart (the reference runs one system per process):
 * at most `sms` SMs for this context's grid-wide solver kernels (0: all),
 * so that contexts driven side by side share the GPU. */
int kd_ctx_set_sm_budget(kd_ctx* ctx, int sms);
/* Failure detection (no reference counterpart: MPI ranks of the reference
 * block forever on a lost peer).  Every grid-barrier wait of the solver's
 * cooperative kernels (LU panel, triangular sweeps) gives up after
 * `seconds` (default 2); the kernel then sets an error flag and returns, the
 * call reports KD_ERR_TIMEOUT, and the context stays usable.
 * kd_ctx_stall_waits(ctx, 1) injects the failure for tests: every barrier
 * target is raised by one, so the waits run out;
 * kd_ctx_stall_waits(ctx, 0) restores normal operation. */
int kd_ctx_set_wait_limit(kd_ctx* ctx, double seconds);
int kd_ctx_stall_waits(kd_ctx* ctx, int on);
/* The project's autotuner (no reference counterpart): launch shapes of the
 * spectral line passes (one CTA of 64, 128 or 256 threads per field, or a
 * cluster of 2, 4 or 8 CTAs per field) per shape class of a launch (number
 * of fields, largest stage, passes).  mode 0: a fixed rule; 1: the shapes of
 * the JSON table at `path` (the fixed rule for classes it lacks); 2: as 1,
 * and a class met for the first time outside a graph capture is timed
 * (every candidate, CUDA events, outputs to a scratch buffer), its fastest
 * shape added and the table written back to `path`.  Shapes change no
 * result bit.  Stats: table entries, classes timed by this context, launches
 * that used a table entry.  A context starts in mode 1 with the table named
 * by the environment variable KD_TUNING_FILE when it is set. */
int kd_ctx_autotune(kd_ctx* ctx, const char* path, int mode);
int kd_ctx_autotune_stats(const kd_ctx* ctx, long long* entries, long long* tuned, long long* hits);
const char* kd_last_error(const kd_ctx* ctx);
int kd_ctx_synchronize(kd_ctx* ctx);
/* Number of kernels this context has launched so far. */
long long kd_ctx_launch_count(const kd_ctx* ctx);
/* Kernel timing by category with CUDA events on the context's stream
 * (no reference counterpart: the reference prints wall-clock phase times,
 * src_par/do_newton.cpp:257,333).  Categories, with the unit of `work`:
 * 0 separable transforms and 1-D operators (FP64 flops), 1 elementwise
 * (bytes), 2 tau gathers (bytes), 3 partial-pivoting LU panels (bytes: the
 * panel read and written once), 4 LU row swaps + U12 solve (bytes of A12
 * read and written), 5 LU trailing update (bytes of the tensor-core update;
 * flops of the FP64 GEMM), 6 one triangular sweep (bytes of the triangle
 * read), 7 refinement matvecs and vector operations (bytes), 8 static-pivot
 * LU panels (bytes).  While profiling is on, a short idle kernel is queued
 * ahead of a timed launch whenever the stream has drained, so each event
 * pair holds device time only; the residual is then not graph-captured. */
#define KD_PROF_NCAT 9
/* The CUDA stream (cudaStream_t) all of this context's work runs on, so a
 * caller can order its own work or record timing events on it. */
void* kd_ctx_stream(const kd_ctx* ctx);
int kd_ctx_profile_enable(kd_ctx* ctx, int on);
int kd_ctx_profile_read(kd_ctx* ctx, double* ms, long long* launches, double* work);

/* ---- spectral transforms (subsystem a) --------------------------------- */
/* One batch of fields of one domain shape.  base_r is the (nc1 x nc2)
 * radial basis table (row-major), base_t the nc2 theta bases, base_p the phi
 * basis -- Base_spectral::bases_1d[0..2].  Arrays are row-major (r, theta,
 * phi) with phi fastest; conf blocks have nbr_points dims, coef blocks
 * nbr_coefs dims. `in`/`out` are DEVICE pointers; `batch` fields follow each
 * other contiguously. */
typedef struct kd_transform_desc {
  int nbr_points[3];
  int nbr_coefs[3];
  const int* base_r;
  const int* base_t;
  int base_p;
  int batch;
  const double* in;
  double* out;
} kd_transform_desc;

/* Base_spectral::coef (src/Coef/coef.cpp:96) for n descriptors in one launch. */
int kd_coef_many(kd_ctx* ctx, int n, const kd_transform_desc* descs);
/* Base_spectral::coef_i (src/Coef/coef_i.cpp:96) for n descriptors. */
int kd_coef_i_many(kd_ctx* ctx, int n, const kd_transform_desc* descs);
/* Host-pointer forms of the two above for one domain: copies in, transforms,
 * copies out (the host<->device copies are part of the call). */
int kd_coef_host(kd_ctx* ctx, const kd_transform_desc* desc);
int kd_coef_i_host(kd_ctx* ctx, const kd_transform_desc* desc);

/* Same result as kd_coef_host, but the call allocates no device memory.
 * No counterpart in the reference (its transforms run on the host).
 *
 * For callers that cannot let a library allocate GPU memory: applications
 * that reserve their whole device memory budget up front and serve it from
 * their own pool -- e.g. an evolution code importing initial data -- where an
 * allocation by the library fails or breaks the budget, and code running
 * between the steps of such an application, where a cudaFree would also
 * synchronise the whole device.  The device staging buffers and basis tables
 * are fixed arrays compiled into the library (2 x KD_NOALLOC_MAX_DOUBLES
 * doubles and KD_NOALLOC_MAX_TABLE ints, about 16 MiB), held by every GPU that
 * loads the library until the process exits; the per-line matrices go into
 * the context's matrix pool, allocated once with the context.
 *
 * Limits: batch * nbr_points product and batch * nbr_coefs product must each
 * be at most KD_NOALLOC_MAX_DOUBLES (KD_ERR_ARG otherwise); the per-line basis
 * tables (1 + nc2 + nc1*nc2 entries) at most KD_NOALLOC_MAX_TABLE.
 * The first call on a device looks up the device addresses of those arrays
 * (cudaGetSymbolAddress, with that device current); make that first call
 * before any stream capture.
 * All calls share the arrays and leave the last call's data in them; calls
 * whose GPU work overlaps (several host threads or contexts on one device)
 * race.  desc->in and desc->out are HOST pointers. */
#define KD_NOALLOC_MAX_DOUBLES (1 << 20)
#define KD_NOALLOC_MAX_TABLE (1 << 14)
int kd_coef_host_noalloc(kd_ctx* ctx, const kd_transform_desc* desc);

/* Base_spectral::ope_1d (src/Ope_1d/ope_1d.cpp:25) with one of the 1-D
 * operators below along dimension `dim` (0=r, 1=theta, 2=phi) of coefficient
 * arrays.  The output basis table of that dimension is written to
 * base_out_{r,t,p} (same shapes as the inputs).  Device pointers. */
#define KD_OP_DER 2        /* src/Ope_1d/der_1d.cpp:290 */
#define KD_OP_MULT_SIN 3   /* src/Ope_1d/mult_sin_1d.cpp */
#define KD_OP_DIV_SIN 4    /* src/Ope_1d/div_sin_1d.cpp */
#define KD_OP_MULT_COS 5   /* src/Ope_1d/mult_cos_1d.cpp */
#define KD_OP_DIV_COS 6    /* src/Ope_1d/div_cos_1d.cpp */
#define KD_OP_MULT_X 7     /* src/Ope_1d/mult_x_1d.cpp */
#define KD_OP_DIV_X 8      /* src/Ope_1d/div_x_1d.cpp */
#define KD_OP_MULT_XM1 9   /* src/Ope_1d/mult_xm1_1d.cpp */
#define KD_OP_DIV_XM1 10   /* src/Ope_1d/div_xm1_1d.cpp */
#define KD_OP_DIV_XP1 11   /* src/Ope_1d/div_xp1_1d.cpp */
#define KD_OP_DIV_1MX2 12  /* src/Ope_1d/div_1mx2.cpp */
/* Coefficients -> values at the n_out collocation points of the basis's own
 * grid (Base_spectral::summation, src/Ope_1d/summation_1d.cpp, at those
 * points); the 1-D step of kd_field_regrid.  kd_matrix_1d only. */
#define KD_OP_RESAMPLE 14
int kd_ope_1d(kd_ctx* ctx, int op, int dim, const kd_transform_desc* desc, int* base_out_r,
              int* base_out_t, int* base_out_p);

/* Matrix of a 1-D operator for a line of n_in inputs and n_out outputs
 * (row-major n_out x n_in) and its output basis; host memory. */
int kd_matrix_1d(kd_ctx* ctx, int op, int basis, int n_in, int n_out, double* mat, int* out_basis);

/* ---- spaces and fields (API surface of Space / Scalar) ----------------- */
typedef struct kd_space kd_space;
typedef struct kd_field kd_field;
typedef struct kd_system kd_system;

/* Space_spheric(CHEB_TYPE, center, res, bounds, withzec)
 * (src/Space/Spheric/space_spheric.cpp:25): nucleus, shells, and a
 * compactified outer domain when withzec != 0. */
int kd_space_spheric_create(kd_ctx* ctx, const double center[3], const int res[3], const double* bounds,
                            int nbounds, int withzec, kd_space** out);
int kd_space_destroy(kd_space* sp);
int kd_space_nbr_domains(const kd_space* sp, int* n);
/* type: 1 nucleus, 2 shell, 3 compact (Domain_nucleus/_shell/_compact). */
int kd_space_domain_info(const kd_space* sp, int dom, int* type, int npts[3], int ncoefs[3], double* alpha,
                         double* beta);
/* Domain::get_radius() and get_cart(c) at the collocation points (host). */
int kd_space_radius(const kd_space* sp, int dom, double* out);
int kd_space_cart(const kd_space* sp, int dom, int c, double* out);
/* Standard bases of a domain (Domain_*::set_cheb_base): r table nc1*nc2,
 * theta table nc2, phi basis. */
int kd_space_std_base(const kd_space* sp, int dom, int* base_r, int* base_t, int* base_p);

/* Scalar(space): one Val_domain per domain (include/scalar.hpp:67). */
int kd_field_create(kd_space* sp, kd_field** out);
int kd_field_destroy(kd_field* f);
int kd_field_set_value(kd_field* f, double v);                 /* Scalar = v */
int kd_field_std_base(kd_field* f);                            /* Scalar::std_base */
/* Val_domain::std_base_{x,y,z}_cart on every domain, c = 0, 1, 2 (bases of
 * the Cartesian components of a vector, Tensor::std_base src/Tensor/tensor.cpp:609). */
int kd_field_cart_base(kd_field* f, int c);
int kd_field_set_conf(kd_field* f, int dom, const double* v);  /* values at collocation points */
int kd_field_get_conf(kd_field* f, int dom, double* out);      /* Val_domain::coef_i + copy */
int kd_field_get_coef(kd_field* f, int dom, double* out);      /* Val_domain::coef + copy */
int kd_field_get_base(const kd_field* f, int dom, int* base_r, int* base_t, int* base_p);
/* dst = src on every domain, device to device (Scalar copy assignment). */
int kd_field_copy(kd_field* dst, const kd_field* src);

/* ---- Save files (Kadath's binary format, every number big-endian) ------- */
/* The files Space_spheric::save, Scalar::save and Tensor::save write
 * (src/Space/Spheric/space_spheric.cpp:124, src/Scalar/scalar.cpp:64,
 * src/Tensor/tensor.cpp:361; fwrite_be, src/Utilities/fwrite_be.cpp), read
 * back as Space_spheric(FILE*, withzec), Scalar(space, FILE*) and
 * Tensor(space, FILE*) read them.  Items follow one another in the order
 * they are saved, as with the reference's FILE*. */
typedef struct kd_file kd_file;
int kd_file_open(const char* path, const char* mode, kd_file** out); /* mode "wb" or "rb" */
int kd_file_close(kd_file* f);
int kd_space_save(const kd_space* sp, kd_file* f);
int kd_space_load(kd_ctx* ctx, kd_file* f, int withzec, kd_space** out);
int kd_field_save(kd_field* fld, kd_file* f);
int kd_field_load(kd_field* fld, kd_file* f); /* into a field of the same space */
/* A Vector with the Cartesian basis: type_index CON (+1) or COV (-1). */
int kd_vector_save(kd_field* fx, kd_field* fy, kd_field* fz, int type_index, kd_file* f);
int kd_vector_load(kd_field* fx, kd_field* fy, kd_field* fz, int* type_index, kd_file* f);

/* ---- System_of_eqs (include/system_of_eqs.hpp:54) ----------------------- */
int kd_system_create(kd_space* sp, int dom_min, int dom_max, kd_system** out);
int kd_system_destroy(kd_system* s);
int kd_system_add_var(kd_system* s, const char* name, kd_field* f);        /* add_var(name, Tensor&) */
int kd_system_add_var_double(kd_system* s, const char* name, double v);    /* add_var(name, double&) */
int kd_system_get_var_double(const kd_system* s, const char* name, double* v);
int kd_system_add_cst(kd_system* s, const char* name, double v);           /* add_cst(name, double) */
int kd_system_add_cst_field(kd_system* s, const char* name, kd_field* f);  /* add_cst(name, Tensor) */
int kd_system_add_def(kd_system* s, int dom, const char* text);            /* add_def; dom < 0: all */
/* Cartesian vectors (add_var(name, Tensor&) / add_cst(name, const Tensor&)
 * with a Vector of CARTESIAN_BASIS, src/System_of_eqs/system_of_eqs.cpp:404
 * and :436): components x, y, z as three fields, each with its component's
 * basis (kd_field_cart_base).  Equations write the vector with one index
 * ("bet^i", "bet_j") or none.  Its unknowns follow xx_to_vars
 * (system_of_eqs.cpp:597): domain by domain, the three components inside
 * each domain. */
int kd_system_add_var_vector(kd_system* s, const char* name, kd_field* fx, kd_field* fy, kd_field* fz);
int kd_system_add_cst_vector(kd_system* s, const char* name, kd_field* fx, kd_field* fy, kd_field* fz);
/* Metric_flat::set_system (src/Metric/metric_flat.cpp:501) with a Cartesian
 * basis: D_i / D^i become the flat derivatives and `name` with two indices
 * ("g_ij") the metric tensor.  A second metric is an error. */
int kd_system_set_metric_flat(kd_system* s, const char* name);
int kd_system_add_eq_inside(kd_system* s, int dom, const char* eq);        /* add_eq_inside */
int kd_system_add_eq_bc(kd_system* s, int dom, int bound, const char* eq); /* add_eq_bc */
int kd_system_add_eq_matching(kd_system* s, int dom, int bound, const char* eq); /* add_eq_matching */
/* add_eq_order (src/System_of_eqs/add_eq.cpp:80, Eq_order): the tau export
 * drops `order` radial coefficients (0, 1 or 2; add_eq_inside is order 2).
 * add_eq_full (add_eq.cpp:291, Eq_full) is order 0: every coefficient. */
int kd_system_add_eq_order(kd_system* s, int dom, int order, const char* eq);
int kd_system_add_eq_full(kd_system* s, int dom, const char* eq);
/* add_eq_first_integral (add_eq.cpp:414, Eq_first_integral,
 * src/Equation/eq_first_integral.cpp): integ_part is constant over domains
 * dom_min..dom_max, with cst_part = 0 at the first collocation point of
 * dom_min.  Conditions: every coefficient of integ_part minus its value at
 * that point, in each domain; in dom_min the points of radial index 0 carry
 * cst_part's value there instead. */
int kd_system_add_eq_first_integral(kd_system* s, int dom_min, int dom_max, const char* integ_part,
                                    const char* cst_part);
/* Integral-type equations (Eq_int, include/system_of_eqs.hpp:1352): one
 * condition each, placed before all other equations (sec_member,
 * src/System_of_eqs/solver.cpp:49).
 * - int_volume: "integvolume(f) = c" over domains dom_min..dom_max
 *   (Space_spheric::add_eq_int_volume, src/Space/Spheric/spheric_add_eq.cpp:81);
 * - int_inf: "integ(f) = c" with integ() at the outer boundary of the
 *   compactified domain (Domain_compact::integ, domain_compact.cpp:89);
 * - val: the expression vanishes at collocation point pos = (i, j, k) of
 *   dom (System_of_eqs::add_eq_val, src/System_of_eqs/add_eq.cpp:343);
 * - point: the expression vanishes at a Cartesian point, summed in dom
 *   (System_of_eqs::add_eq_point, add_eq.cpp:355).
 * Double unknowns (kd_system_add_var_double) get their own Jacobian columns,
 * first in the unknown order (do_col_J, solver.cpp:120). */
int kd_system_add_eq_int_volume(kd_system* s, int dom_min, int dom_max, const char* eq);
int kd_system_add_eq_int_inf(kd_system* s, const char* eq);
int kd_system_add_eq_val(kd_system* s, int dom, const char* eq, const int pos[3]);
int kd_system_add_eq_point(kd_system* s, int dom, const char* eq, const double point[3]);
/* System_of_eqs::add_ope(name, &EOS<Cold_PWPoly, var>::action, ...)
 * (include/system_of_eqs.hpp:277, include/EOS/EOS.hh:235): registers
 * name(h) = var of a cold piecewise polytrope at the enthalpy h, with its
 * variation (include/EOS/EOS.hh:67-160).  var: KD_EOS_EPSILON, _PRESSURE,
 * _DENSITY, _DHDRHO.  The polytrope is given as Margherita's polytrope files
 * give it (eos/gam2.polytrope: npieces, rhomin, rhomax, ktab0, gamma_tab,
 * rho_tab), geometrised units; the other pieces' K, eps and h follow from
 * continuity as in Margherita_setup_polytrope. */
#define KD_EOS_EPSILON 0
#define KD_EOS_PRESSURE 1
#define KD_EOS_DENSITY 2
#define KD_EOS_DHDRHO 3
int kd_system_add_ope_eos(kd_system* s, const char* name, int var, int npieces, double rhomin, double rhomax,
                          double k0, const double* gamma_tab, const double* rho_tab);
int kd_system_sizes(kd_system* s, int* n_unknowns, int* n_conditions);
int kd_system_n_equations(kd_system* s, int* neq);
/* sec_member (src/System_of_eqs/solver.cpp:49): F(u) into host F. */
int kd_system_residual(kd_system* s, double* F);
/* check_equations (solver.cpp:24): per-equation max |F| into errors[neq]. */
int kd_system_check_equations(kd_system* s, double* errors);
/* All columns of do_col_J (solver.cpp:120) as one column-major N x N
 * host matrix (ld = N). */
int kd_system_jacobian(kd_system* s, double* J);
/* Same, into a device buffer of leading dimension ld (device pointer). */
/* Keeps, between Jacobian assemblies, the batched tangents of the subtrees
 * whose tangent does not depend on the iterate (Laplacians and derivatives
 * of unknowns, matching and boundary conditions, products with numbers):
 * later assemblies skip those subtrees.  On by default; 0 frees them.  No
 * reference counterpart: the reference recomputes every column of the
 * Jacobian at every step (do_col_J, src/System_of_eqs/solver.cpp:120). */
/* Captures and replays of the residual's value pass (kd_newton_opts.graph_capture). */
int kd_system_graph_stats(kd_system* s, long long* captures, long long* replays);
/* The same for the Jacobian's seed passes, which kd_newton_opts.graph_capture
 * also replays from CUDA graphs: a pass is captured the second time the
 * system is in the same state (the residual's state, the node values'
 * addresses, the output buffer, the tangent cache's contents), with the
 * tangent cache as the pass leaves it; systems with integral-type
 * equations or double unknowns are never captured. */
int kd_system_jacobian_graph_stats(kd_system* s, long long* captures, long long* replays);
int kd_system_cache_tangents(kd_system* s, int enable);
int kd_system_jacobian_device(kd_system* s, double* dJ, long long ld);
/* do_JX (src/System_of_eqs/solver.cpp:87-118): y = J x without forming J,
 * every unknown seeded by x through affecte_tau (xx_to_ders,
 * src/System_of_eqs/system_of_eqs.cpp:557) in one tangent pass.  Host
 * vectors of length nbr_unknowns; the _device form takes device vectors. */
int kd_system_jx(kd_system* s, const double* x, double* y);
int kd_system_jx_device(kd_system* s, const double* dx, double* dy);
/* xx_to_vars + var = old - x (src_par/do_newton.cpp:397-414), host x. */
int kd_system_update(kd_system* s, const double* x);

/* LU modes for the dense solve. */
#define KD_LU_FP64 0     /* blocked LU, FP64 trailing updates */
#define KD_LU_TF32_IR 1  /* TF32 tensor-core trailing updates + FP64 GMRES-IR */
#define KD_LU_FP32_IR 2  /* FP32 trailing updates + FP64 GMRES-IR */

typedef struct kd_newton_opts {
  double precision;  /* stop when max |F| < precision (do_newton's first argument) */
  int lu_mode;       /* KD_LU_* */
  double gmres_tol;  /* relative residual target of the refinement */
  int max_refine;    /* GMRES iterations per restart */
  int graph_capture; /* nonzero: the residual's value pass runs from a CUDA
                        graph captured the second time the fields are in
                        the same state (same representations, bases and
                        numbers); systems with integral-type equations are
                        never captured */
  int gmres_restarts; /* GMRES cycles of max_refine iterations (0: 4).  When
                         the mixed-precision solve stops above a relative
                         residual of 1e-10 (KD_ERR_NOCONV), the step factors
                         the same Jacobian in FP64 and solves again
                         (report.fp64_fallback = 1) */
  int pivot_every_step; /* 0 (default): a mixed-precision step reuses the
                           pivot order of the last partial-pivoting
                           factorisation of this system (static pivoting;
                           refinement against the FP64 Jacobian restores the
                           accuracy, and a refinement that does not converge
                           makes the step factor again with partial
                           pivoting); 1: partial pivoting at every step */
} kd_newton_opts;

typedef struct kd_newton_report {
  double error;      /* pre-step max |F| (do_newton's `error` output) */
  int converged;     /* do_newton's return value */
  int n;             /* N = number of unknowns */
  double t_residual_ms, t_assembly_ms, t_factor_ms, t_solve_ms, t_update_ms;
  int refine_iters;
  double refine_rel_residual;
  long long kernel_launches;
  int fp64_fallback; /* 1 when the mixed-precision solve did not converge
                        (KD_ERR_NOCONV) and the step was solved again with
                        the FP64 LU of the same Jacobian */
  int static_pivots; /* 1 when the step's factors used the reused pivot order */
} kd_newton_report;

/* System_of_eqs::do_newton (src_par/do_newton.cpp:65; decl
 * include/system_of_eqs.hpp:871).  Returns KD_OK and fills rep; the fields
 * registered with add_var are updated in place on the device. */
int kd_newton_step(kd_system* s, const kd_newton_opts* opts, kd_newton_report* rep);
/* One stage of a FUKA solver (the stage loops of
 * include/Solvers/ns_3d_xcts/ns_3d_xcts_stages.cpp, e.g. norot_stage :141-165,
 * and check_max_iter_exceeded in include/Solvers/solvers.hpp): Newton steps
 * (kd_newton_step with opts) until the pre-step error is below
 * opts->precision.  After every update, and once more at the end, the
 * space and the nfields scalars are written to `checkpoint` (NULL: no file)
 * in Kadath's save format (Space::save, then Scalar::save each).  More than
 * max_iter updates: accepted when the last error is below 10 precision,
 * else KD_ERR_NOCONV.  iterations/error (nullable): updates made and the
 * last pre-step error. */
int kd_stage_solve(kd_system* s, const kd_newton_opts* opts, int max_iter, const char* checkpoint, int nfields,
                   kd_field* const* fields, int* iterations, double* error);
/* The regrid of the FUKA solvers (include/Solvers/ns_3d_xcts/ns_3d_xcts_regrid.hpp):
 * dst = src evaluated at the collocation points of dst's space, which must
 * have the same domains as src's (kinds and radii) at any resolution; on the
 * GPU, as three separable passes from src's coefficients (the summation of
 * Base_spectral::summation at the new points).  dst gets the standard or
 * anti-symmetric basis, as src has. */
int kd_field_regrid(kd_field* dst, kd_field* src);
/* Forgets the pivot order kept for static pivoting: the next mixed-precision
 * step factors with partial pivoting (no reference counterpart). */
int kd_system_reset_pivot_order(kd_system* s);
/* do_newton(precision, error, GAUSS_NEWTON) (include/system_of_eqs.hpp:134,
 * src_par/do_newton.cpp:264-311): for a system with at least as many
 * conditions m as unknowns n, solves the normal equations
 * (J^T J) x = J^T F (J is m x n; J^T J and J^T F in FP64; J^T J factored in
 * opts->lu_mode) and updates fields <- fields - x.  rep->n is n. */
int kd_newton_step_gauss_newton(kd_system* s, const kd_newton_opts* opts, kd_newton_report* rep);
/* System_of_eqs::do_newton_with_linesearch (src_par/do_newton.cpp:454-516):
 * Newton direction p = J^-1 F, rescaled when max(p) > stepmax, then fields
 * = old - lambda p with lambda backtracked (quadratic, then cubic model of
 * f = sum F^2, sufficient decrease 1e-4) for at most ntrymax tries.  lambda
 * (may be NULL) receives the last lambda; rep->converged as do_newton. */
int kd_newton_step_linesearch(kd_system* s, const kd_newton_opts* opts, int ntrymax, double stepmax,
                              kd_newton_report* rep, double* lambda);

/* ---- evaluation at arbitrary points (exporters) ------------------------ */
/* Scalar::val_point (include/scalar.hpp:221) for many points and up to 8
 * fields of one space at once: the evaluation the reference's exporters
 * (src/Utilities/Exporters) do point by point, here one GPU thread per
 * point.  out[f * npts + p] = fields[f] at the Cartesian point
 * (xyz[3p], xyz[3p+1], xyz[3p+2]); NaN for a point in no domain.  Host
 * pointers, synchronous. */
int kd_fields_val_points(int nfields, kd_field* const* fields, long long npts, const double* xyz, double* out);
/* The same with device pointers (d_xyz, d_out) on the context's stream;
 * returns once the values are written. */
int kd_fields_val_points_device(int nfields, kd_field* const* fields, long long npts, const double* d_xyz,
                                double* d_out);

/* ---- adjoint sensitivities --------------------------------------------- */
/* No reference counterpart for the adjoint itself: the reference obtains
 * parameter derivatives by finite differences of full re-solves.  Pieces:
 *  kd_system_set_cst       changes a double constant of add_cst(name, double)
 *                          (src/System_of_eqs/system_of_eqs.cpp:340);
 *  kd_field_val_point      Scalar::val_point (include/scalar.hpp:221);
 *  kd_system_val_point_gradient
 *                          g = dQ/dy for Q = var's value at a point, y the
 *                          unknown vector (nbr_unknowns doubles, host);
 *  kd_system_dres_dcst     dF/dp for a double constant p (host vector);
 *  kd_system_integral_gradient
 *                          Q and g = dQ/dy for Q an integral observable:
 *                          kind 0, the sum over domains dmin..dmax of
 *                          `expr` (the left side of add_eq_int_volume,
 *                          e.g. "integvolume(psi^5)");
 *                          kind 1, the integral at infinity (the left side
 *                          of add_eq_int_inf, e.g. "integ(dn(P))" or
 *                          "integ(intMadm)" with intMadm = -dr(P)/2/PI
 *                          defined in the last domain, as FUKA's ADM mass,
 *                          include/Solvers/fuka_syst/fuka_syst_setup.hpp:62);
 *                          g is the row such an equation would add to J;
 *  kd_system_dres_dcst     dF/dp for a double constant p (host vector);
 *  kd_adjoint              dQ/dp = dq_explicit - lambda . dF/dp with
 *                          J^T lambda = g, J assembled at the current
 *                          (converged) fields and factored in FP64; lambda
 *                          (nullable) receives the adjoint vector;
 *  kd_adjoint_ex           the same; with reuse_factors = 1 and the
 *                          mixed-precision factors of the system's last
 *                          Newton step at hand, J^T lambda = g is solved by
 *                          FP64 GMRES on J^T (J at the current fields)
 *                          preconditioned by those factors transposed, with
 *                          no new factorisation; when that refinement does
 *                          not converge, or without such factors, J is
 *                          factored in FP64 as in kd_adjoint.  rep
 *                          (nullable) tells which ran. */
typedef struct {
  int reused_factors;  /* 1: the Newton step's mixed factors preconditioned the solve */
  int refine_iters;    /* GMRES iterations on J^T (reused factors only) */
  double rel_residual; /* final |g - J^T lambda| / |g| (reused factors only) */
  double t_assembly_ms, t_solve_ms;
} kd_adjoint_report;
int kd_system_set_cst(kd_system* s, const char* name, double v);
int kd_field_val_point(kd_field* f, const double point[3], double* value);
int kd_system_val_point_gradient(kd_system* s, const char* var, const double point[3], double* g);
int kd_system_integral_gradient(kd_system* s, int kind, int dmin, int dmax, const char* expr, double* q,
                                double* g);
int kd_system_dres_dcst(kd_system* s, const char* cst, double* fp);
int kd_adjoint(kd_system* s, const double* g, const char* cst, double dq_explicit, double* dqdp, double* lambda);
int kd_adjoint_ex(kd_system* s, const double* g, const char* cst, double dq_explicit, int reuse_factors,
                  double* dqdp, double* lambda, kd_adjoint_report* rep);

/* ---- dense LU (Matrice::set_lu / solve, src/Matrice/matrice.cpp:192-249) */
typedef struct kd_lu kd_lu;
int kd_lu_create(kd_ctx* ctx, kd_lu** out);
int kd_lu_destroy(kd_lu* lu);
/* Factors the device matrix dA (column-major, ld).  FP64 mode overwrites
 * dA with its factors; mixed modes keep dA as the refinement operator. */
int kd_lu_factor(kd_lu* lu, double* dA, long long ld, int n, int mode);
/* Solves in place on the device vector db; trans = 1 solves A^T x = b
 * with the same factors (FP64 mode: transposed triangular solves; mixed
 * modes: GMRES on A^T preconditioned by the transposed FP32 factors). */
int kd_lu_solve(kd_lu* lu, double* db, int trans);
/* Refinement of the mixed modes: GMRES(iters) restarted up to `restarts`
 * times until the relative residual is below tol (defaults 1e-14, 50, 4);
 * kd_lu_solve returns KD_ERR_NOCONV when it ends above 1e-10. */
int kd_lu_set_refinement(kd_lu* lu, double tol, int iters, int restarts);
/* Static pivoting for the mixed modes (off by default here, on for Newton
 * steps): with on = 1, a factorisation of a matrix of the size of the last
 * partial-pivoting one gathers the rows in that pivot order and factors
 * without row search; a zero pivot there, or a refinement that does not
 * converge with those factors, makes the call factor with partial pivoting
 * instead.  kd_lu_pivot_info reports, for the last factor/solve, whether
 * the reused order was used and whether it had to be replaced. */
int kd_lu_set_pivot_reuse(kd_lu* lu, int on);
int kd_lu_pivot_info(const kd_lu* lu, int* static_pivots, int* fallback);
int kd_lu_stats(const kd_lu* lu, double* t_factor_ms, double* t_solve_ms, int* refine_iters,
                double* rel_residual);
/* The LU's trailing update on its own: C -= A * B on the tcgen05 tensor
 * cores in TF32 with FP32 accumulation (replaces the pdgemm/dgemm inside
 * pdgesv/dgetrf, src_par/do_newton.cpp:317).  Column-major FP32 device
 * matrices: A is m x k (lda), B is k x n (ldb), C is m x n (ldc); k <= 128. */
int kd_tf32_gemm_update(kd_ctx* ctx, int m, int n, int k, const float* A, long long lda, const float* B,
                        long long ldb, float* C, long long ldc);
/* The same update with 3xTF32 products (A = Ah + Al, B = Bh + Bl in TF32,
 * C -= Al Bh + Ah Bl + Ah Bh), about FP32 accurate; the update the mixed LU
 * uses.  Needs k <= 192, C 16-byte aligned, ldc a multiple of 4 and m a
 * multiple of 4 (else KD_ERR_UNSUPPORTED). */
int kd_tf32x3_gemm_update(kd_ctx* ctx, int m, int n, int k, const float* A, long long lda, const float* B,
                          long long ldb, float* C, long long ldc);

#ifdef __cplusplus
}
#endif

#endif /* KADATH_GB300_H */
