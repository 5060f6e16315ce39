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
const char* kd_last_error(const kd_ctx* ctx);
int kd_ctx_synchronize(kd_ctx* ctx);
/* Number of kernels this context has launched so far. */
long long kd_ctx_launch_count(const kd_ctx* ctx);

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
int kd_ope_1d(kd_ctx* ctx, int op, int dim, const kd_transform_desc* desc, int* base_out_r,
              int* base_out_t, int* base_out_p);

/* Matrix of a 1-D operator for a line of n_in inputs and n_out outputs
 * (row-major n_out x n_in) and its output basis; host memory. */
int kd_matrix_1d(kd_ctx* ctx, int op, int basis, int n_in, int n_out, double* mat, int* out_basis);

#ifdef __cplusplus
}
#endif

#endif /* KADATH_GB300_H */
