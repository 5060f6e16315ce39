/* Stand-in for the subset of FFTW 3.3.8's public API that Kadath's transform
 * layer calls (src/Coef/coef_1d.cpp, src/Coef/coef_i_1d.cpp through
 * include/base_fftw.hpp:28-35): real-to-real plans of kind R2HC and HC2R.
 *
 * Test infrastructure only: it lets the reference's own sources be compiled
 * here as the oracle's pin.  The transforms are direct DFTs evaluated in long
 * double (ref_shims.cpp), following FFTW's published halfcomplex layout:
 *   R2HC: hc[k] = sum_j x_j cos(2 pi j k / n)        for 0 <= k <= n/2,
 *         hc[n-k] = -sum_j x_j sin(2 pi j k / n)     for 0 <  k <  (n+1)/2;
 *   HC2R: the unnormalised inverse of R2HC (HC2R(R2HC(x)) = n x). */
#ifndef KD_REF_SHIM_FFTW3_H
#define KD_REF_SHIM_FFTW3_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum { FFTW_R2HC = 0, FFTW_HC2R = 1 } fftw_r2r_kind;
typedef struct kd_shim_fftw_plan_s* fftw_plan;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

double* fftw_alloc_real(unsigned long n);
void fftw_free(void* p);
fftw_plan fftw_plan_r2r_1d(int n, double* in, double* out, fftw_r2r_kind kind, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif
#endif
