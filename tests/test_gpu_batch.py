"""Batched uneven solves: independent isolated stars (random central density,
nr in {9, ..., 17}) solved concurrently, one context (its own streams and
workspaces) per instance from a pool of host threads.

Concurrent solves reach the fields of one-at-a-time solves to rounding (1e-12
of their magnitude).  They are not bitwise equal: a context limited to a
share of the SMs picks its LU panel shape (width, cluster or grid panel)
from that share, so its first-step factors, and the pivot order the later
steps reuse, round differently; the FP64 path's trailing update is cuBLAS
DGEMM, which may pick another implementation while several streams are
active.  Both paths refine to the FP64 solution of each step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fields(wl):
    nd = wl.space.get_nbr_domains()
    return {(nm, d): f.get_coef(d) for nm, f in wl.unknowns for d in range(nd)}


def test_concurrent_mixed_solves_match_serial(ctx):
    from kadath_frontera_gb300 import workloads
    from kadath_frontera_gb300.kadath import KD_LU_TF32_IR
    cfgs = workloads.star_batch_configs(4, seed=3)
    assert len({c["res"] for c in cfgs}) > 1  # uneven sizes
    serial = workloads.solve_batch(cfgs, threads=1, lu_mode=KD_LU_TF32_IR)
    conc = workloads.solve_batch(cfgs, threads=4, lu_mode=KD_LU_TF32_IR)
    for a, b in zip(serial, conc):
        fa, fb = _fields(a), _fields(b)
        for key in fa:
            assert np.linalg.norm(fa[key] - fb[key]) <= 1e-12 * max(np.linalg.norm(fa[key]), 1.0), key
        assert np.abs(b.syst.sec_member()).max() < 1e-10


def test_concurrent_fp64_solves_match_serial(ctx):
    from kadath_frontera_gb300 import workloads
    from kadath_frontera_gb300.kadath import KD_LU_FP64
    cfgs = workloads.star_batch_configs(3, seed=5)
    serial = workloads.solve_batch(cfgs, threads=1, lu_mode=KD_LU_FP64)
    conc = workloads.solve_batch(cfgs, threads=3, lu_mode=KD_LU_FP64)
    for a, b in zip(serial, conc):
        fa, fb = _fields(a), _fields(b)
        scale = max(np.abs(v).max() for v in fa.values())
        for key in fa:
            assert np.abs(fa[key] - fb[key]).max() <= 1e-12 * scale, key
        assert np.abs(b.syst.sec_member()).max() < 1e-10


def test_batch_configs_are_seeded_and_uneven():
    from kadath_frontera_gb300 import workloads
    a = workloads.star_batch_configs(64, seed=0)
    assert a == workloads.star_batch_configs(64, seed=0)
    assert {c["res"][0] for c in a} == {9, 11, 13, 15, 17}
    assert all(8e-4 <= c["rho_c"] <= 2e-3 for c in a)
    assert all(c["res"][1] % 2 == 1 and c["res"][1] in (c["res"][0] // 2 + 1, c["res"][0] // 2 + 2)
               and c["res"][2] == 4 for c in a)
