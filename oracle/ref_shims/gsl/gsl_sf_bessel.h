/* Stand-in for GSL's spherical Bessel functions j_l and y_l as used by the
 * reference (src/Term_eq/term_eq_bessel.cpp, src/Ope_eq/ope_fit_waves.cpp).
 * None of the oracle's drivers calls them; they exist so the reference links.
 * Implemented in ref_shims.cpp from the closed forms j_0, j_1, y_0, y_1 and the
 * three-term recurrence f_{l+1} = (2l+1)/x f_l - f_{l-1}. */
#ifndef KD_REF_SHIM_GSL_SF_BESSEL_H
#define KD_REF_SHIM_GSL_SF_BESSEL_H

#ifdef __cplusplus
extern "C" {
#endif

double gsl_sf_bessel_jl(int l, double x);
double gsl_sf_bessel_yl(int l, double x);

#ifdef __cplusplus
}
#endif
#endif
