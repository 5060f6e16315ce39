// Kadath's binary save format for Space_spheric, Scalar and Cartesian
// vectors: the files Space_spheric::save / Scalar::save / Tensor::save write
// (src/Space/Spheric/space_spheric.cpp:124, src/Scalar/scalar.cpp:64,
// src/Tensor/tensor.cpp:361), every number big-endian (fwrite_be,
// src/Utilities/fwrite_be.cpp).
#pragma once

#include <cstdio>
#include <memory>
#include <vector>

#include "kd_domain.hpp"
#include "kd_system.hpp"

namespace kd {

// Space_spheric::save: nbr_domains, ndim, type_base, then each domain
// (Domain_nucleus/shell/compact::save).
void save_space(const Space& sp, std::FILE* f);
// Space_spheric(FILE*, withzec): domain 0 a nucleus, then shells, the last
// one compactified when withzec.
std::unique_ptr<Space> load_space(std::FILE* f, bool withzec);

// Scalar::save: one Val_domain per domain (basis, zero flag, collocation
// values if held, coefficients if held).
void save_field(Field& fld, std::FILE* f);
// Scalar(space, FILE*), into an existing field of the same space.
void load_field(Field& fld, std::FILE* f);

// Tensor::save of a valence-1 tensor with the Cartesian basis in every
// domain: tensorial basis, index types, valence, number of components, then
// each component as a Scalar.  type_index: CON (+1) or COV (-1).
void save_vector(Field* const comps[3], int type_index, std::FILE* f);
void load_vector(Field* const comps[3], int* type_index, std::FILE* f);

}  // namespace kd
