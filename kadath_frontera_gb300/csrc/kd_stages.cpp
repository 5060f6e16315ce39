// Stage drivers of the FUKA solvers on the GPU path: the Newton loop of one
// stage with its checkpoints, and the regrid of a solution onto a space of
// another resolution.
//
// Reference: the stage loops of include/Solvers/ns_3d_xcts/ns_3d_xcts_stages.cpp
// (norot_stage, :141-165: `while (!endloop) { endloop = syst.do_newton(prec,
// conv); ... checkpoint(); ite++; check_max_iter_exceeded(...) }`, then the
// converged checkpoint), check_max_iter_exceeded in include/Solvers/solvers.hpp
// (a stage that ran out of iterations is accepted when its error is below ten
// times the precision), and the regrid of
// include/Solvers/ns_3d_xcts/ns_3d_xcts_regrid.hpp, which evaluates the old
// fields (Scalar::val_point) at the collocation points of a space with the
// same domains and a new resolution.
#include "kd_stages.hpp"

#include <cmath>
#include <cstdio>
#include <string>

#include "kadath_gb300.h"
#include "kd_device.hpp"
#include "kd_io.hpp"
#include "kd_spectral.hpp"

namespace kd {

namespace {

bool same_geometry(const Domain& a, const Domain& b) {
  auto close = [](double x, double y) { return std::fabs(x - y) <= 1e-12 * (std::fabs(x) + std::fabs(y) + 1.0); };
  return a.type == b.type && close(a.alpha, b.alpha) && close(a.beta, b.beta);
}

}  // namespace

// dst (on its own space) = src evaluated at dst's collocation points, on
// the GPU: three separable passes from src's coefficients through the
// OP_RESAMPLE matrices.  The spaces must have the same domains (kinds,
// radii); only the resolutions may differ.  dst gets the basis of the same
// kind as src's (standard or anti-symmetric; the Cartesian components are
// of one of the two).
void regrid(Field& dst, Field& src) {
  const Space& so = *src.sp;
  const Space& sn = *dst.sp;
  if (so.ndom() != sn.ndom()) throw KdError(KD_ERR_ARG, "regrid: the spaces have different numbers of domains");
  if (src.ctx != dst.ctx) throw KdError(KD_ERR_ARG, "regrid: the fields belong to different contexts");
  Context& ctx = *dst.ctx;
  for (int dd = 0; dd < so.ndom(); dd++) {
    const Domain& dmo = so.dom(dd);
    const Domain& dmn = sn.dom(dd);
    if (!same_geometry(dmo, dmn)) throw KdError(KD_ERR_ARG, "regrid: domain " + std::to_string(dd) + " differs");
    Field::PerDom& pn = dst.d[dd];
    const Field::PerDom& po = src.d[dd];
    if (!po.base.def && !po.zero) throw KdError(KD_ERR_STATE, "regrid: Base not defined");
    Base nb;
    if (po.base.def) {
      if (po.base == dmo.std_base())
        nb = dmn.std_base();
      else if (po.base == dmo.anti_base())
        nb = dmn.anti_base();
      else
        throw KdError(KD_ERR_UNSUPPORTED, "regrid: a basis other than the standard or anti-symmetric one");
    }
    pn.base = nb;
    if (po.zero) {
      pn.zero = true;
      pn.in_conf = pn.in_coef = false;
      continue;
    }
    const size_t mark = ctx.scratch().mark();
    DVal v = src.val(dd);
    v.coef();
    const int nco[3] = {dmo.nc[0], dmo.nc[1], dmo.nc[2]};
    const int npn[3] = {dmn.np[0], dmn.np[1], dmn.np[2]};
    std::vector<LinePassSpec> specs = resample_specs(ctx, po.base, nco, npn);
    KdItemList list{};
    list.nitems = 1;
    list.prefix[0] = 0;
    list.prefix[1] = 1;
    list.items[0] = make_item(ctx, specs, v.cf, pn.c, nco, dmo.ncoefs(), dmn.npts(), 1.0);
    int maxe = dmo.ncoefs();
    int d[3] = {nco[0], nco[1], nco[2]};
    for (const auto& sp : specs) {
      d[sp.dim] = sp.n_out;
      const int e = d[0] * d[1] * d[2];
      if (e > maxe) maxe = e;
    }
    cuda_check(launch_line_passes(list, maxe, ctx.pool(), ctx.stream()), "regrid line passes");
    ctx.launches++;
    cuda_check(cudaStreamSynchronize(ctx.stream()), "sync regrid");
    ctx.scratch().release_to(mark);
    pn.zero = false;
    pn.in_conf = true;
    pn.in_coef = false;
  }
}

// One stage of a FUKA solver: Newton steps until the pre-step error is
// below opts.precision.  After every update the space and `fields` are
// written to `checkpoint` (when given), and once more when converged.  A
// stage that exceeds max_iter updates is accepted when its last error is
// below ten times the precision, otherwise KD_ERR_NOCONV.
void stage_solve(System& sys, Newton& newton, const NewtonOpts& o, int max_iter, const char* checkpoint,
                 const std::vector<Field*>& fields, int& iterations, double& error) {
  auto save = [&]() {
    if (!checkpoint) return;
    std::FILE* f = std::fopen(checkpoint, "wb");
    if (!f) throw KdError(KD_ERR_ARG, std::string("cannot write checkpoint ") + checkpoint);
    try {
      save_space(*sys.sp, f);
      for (Field* fl : fields) save_field(*fl, f);
    } catch (...) {
      std::fclose(f);
      throw;
    }
    std::fclose(f);
  };
  iterations = 0;
  bool done = false;
  while (!done) {
    NewtonReport rep;
    done = newton.step(o, rep);
    error = rep.error;
    if (!done) {
      iterations++;
      save();
      if (iterations > max_iter) {
        if (error < 10.0 * o.precision) break;  // check_max_iter_exceeded's accepted branch
        throw KdError(KD_ERR_NOCONV, "stage: no convergence in " + std::to_string(max_iter) +
                                         " Newton updates (error " + std::to_string(error) + ")");
      }
    }
  }
  save();
}

}  // namespace kd
