"""The caller side of do_newton in the FUKA solvers: a sequence of stages at
increasing resolution, each a Newton loop with checkpoints, the converged
fields of one stage regridded onto the next stage's space.

Reference: the resolution sequences of the FUKA drivers
(include/Solvers/ns_3d_xcts/ns_3d_xcts_driver.cpp, ns_3d_xcts_sequence: a
solve at the initial resolution, then the same stages at the next
resolutions from the regridded solution), the stage loop
(include/Solvers/ns_3d_xcts/ns_3d_xcts_stages.cpp, norot_stage :141-165) and
the regrid (include/Solvers/ns_3d_xcts/ns_3d_xcts_regrid.hpp).  The loop and
the regrid run in the library (kd_stage_solve, kd_field_regrid); this module
only sequences them.  The stages here are the static TOV star of
``workloads.ns_tov`` (the fixed-radius branch of norot_stage on a
Space_spheric)."""
from __future__ import annotations

from pathlib import Path

from . import workloads


def tov_sequence(resolutions=((9, 5, 4), (13, 9, 4)), precision=1e-10, checkpoint_dir=None, lu_mode=None,
                 max_iter=20, ctx=None):
    """Solves the TOV stage at each resolution in turn.  The first stage
    starts from the workload's initial guess; each later one from the
    previous stage's converged H, P and N regridded onto its space.  With
    checkpoint_dir, stage k writes tov_<nr>_<nt>_<np>.dat there after every
    Newton update and when converged (Space::save, then H, P, N).  Returns
    one dict per stage: res, updates, error, checkpoint, workload."""
    stages = []
    prev = None
    for res in resolutions:
        wl = workloads.ns_tov(tuple(res), ctx=ctx)
        if prev is not None:
            for (_, new), (_, old) in zip(wl.unknowns, prev.unknowns):
                new.regrid_from(old)
        ck = None
        if checkpoint_dir is not None:
            ck = Path(checkpoint_dir) / f"tov_{res[0]}_{res[1]}_{res[2]}.dat"
        updates, err = wl.syst.stage_solve(precision, max_iter, ck, [f for _, f in wl.unknowns], lu_mode)
        stages.append({"res": tuple(res), "updates": updates, "error": err, "checkpoint": ck, "workload": wl})
        prev = wl
    return stages
