// Fields evaluated at arbitrary Cartesian points on the GPU (the exporters'
// step: Scalar::val_point, include/scalar.hpp:221, for many points).
#pragma once
#include <vector>

#include "kd_system.hpp"

namespace kd {

constexpr int PT_MAX_DOM = 16;
constexpr int PT_MAX_FIELDS = 8;

// d_out[f * npts + p] = fields[f] at point p (d_xyz[3p .. 3p+2]), NaN for a
// point in no domain.  Device pointers, on the context's stream; returns
// after the kernel has run.
void fields_val_points(Context* ctx, const std::vector<const Field*>& fields, long long npts, const double* d_xyz,
                       double* d_out);

}  // namespace kd
