/* Stand-in for GSL's permutation API as used by the reference
 * (src/Ope_eq/ope_inverse.cpp, ope_inverse_nodet.cpp, include/metric_tensor.hpp).
 * Test infrastructure for compiling the reference here; implemented in
 * ref_shims.cpp (lexicographic next permutation, as GSL documents). */
#ifndef KD_REF_SHIM_GSL_PERMUTATION_H
#define KD_REF_SHIM_GSL_PERMUTATION_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GSL_SUCCESS 0
#define GSL_FAILURE (-1)

typedef struct {
  size_t size;
  size_t* data;
} gsl_permutation;

gsl_permutation* gsl_permutation_calloc(size_t n);
void gsl_permutation_free(gsl_permutation* p);
size_t gsl_permutation_get(const gsl_permutation* p, size_t i);
size_t gsl_permutation_size(const gsl_permutation* p);
int gsl_permutation_next(gsl_permutation* p);

#ifdef __cplusplus
}
#endif
#endif
