// Stage drivers: the Newton loop of one FUKA solver stage with checkpoints,
// and the regrid of a field onto a space of another resolution (kd_stages.cpp).
#pragma once
#include <vector>

#include "kd_newton.hpp"
#include "kd_system.hpp"

namespace kd {

void regrid(Field& dst, Field& src);
void stage_solve(System& sys, Newton& newton, const NewtonOpts& o, int max_iter, const char* checkpoint,
                 const std::vector<Field*>& fields, int& iterations, double& error);

}  // namespace kd
