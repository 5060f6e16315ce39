// Host-pointer forward transform that allocates no device memory (see
// kd_noalloc.cu for the fixed device arrays it stages through).
#pragma once
#include "kadath_gb300.h"  // KD_NOALLOC_MAX_DOUBLES, KD_NOALLOC_MAX_TABLE
#include "kd_spectral.hpp"

namespace kd {

void coef_host_noalloc(Context& ctx, const Base& base, const int np[3], const int nc[3], int batch,
                       const double* h_in, double* h_out);

}  // namespace kd
