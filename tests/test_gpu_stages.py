"""Stage drivers on the GPU path: the FUKA regrid (kd_field_regrid) and the
stage loop with checkpoints (kd_stage_solve), sequenced over resolutions as
the FUKA drivers do (kadath_frontera_gb300.stages)."""
import numpy as np
import pytest

from oracle import configs, kadath as K, kadath_io as KIO

pytestmark = pytest.mark.gpu

BOUNDS = (3.5, 7.0, 12.0)


def _values(kind):
    """A smooth field even in z (std) or odd in z (anti), vanishing at infinity."""
    def fn(x, y, z):
        with np.errstate(all="ignore"):
            r2 = x * x + y * y + z * z
            g = np.exp(-r2 / 40.0)
            v = g * (1.0 + 0.1 * x * y) if kind == "std" else z * g
        return np.where(np.isfinite(r2), v, 0.0)
    return fn


def _field(space, kind, fn):
    from kadath_frontera_gb300.kadath import Scalar
    f = Scalar(space)
    for d in range(space.get_nbr_domains()):
        x, y, z = (space.get_cart(d, c) for c in (1, 2, 3))
        f.set_domain(d, fn(x, y, z))
    if kind == "std":
        f.std_base()
    else:
        f.std_base_cart(3)
    return f


@pytest.mark.parametrize("kind", ["std", "anti"])
def test_regrid_up_and_back_reproduces_the_field(ctx, kind):
    """A field known at (9, 5, 4) is a spectral expansion the finer grid
    holds exactly: regridded to (13, 9, 8) and back, it comes back to
    round-off."""
    from kadath_frontera_gb300.kadath import CHEB_TYPE, Scalar, Space_spheric
    coarse = Space_spheric(CHEB_TYPE, (0, 0, 0), (9, 5, 4), BOUNDS)
    fine = Space_spheric(CHEB_TYPE, (0, 0, 0), (13, 9, 8), BOUNDS)
    f = _field(coarse, kind, _values(kind))
    g = Scalar(fine).regrid_from(f)
    h = Scalar(coarse).regrid_from(g)
    for d in range(coarse.get_nbr_domains()):
        a, b = h.get_domain(d), f.get_domain(d)
        assert np.abs(a - b).max() <= 1e-13 * max(1.0, np.abs(b).max()), (kind, d)
        rb, tb, pb = g.get_base(d)
        std = Scalar(fine).std_base() if kind == "std" else Scalar(fine).std_base_cart(3)
        r2, t2, p2 = std.get_base(d)
        assert np.array_equal(rb, r2) and np.array_equal(tb, t2) and pb == p2


@pytest.mark.parametrize("kind", ["std", "anti"])
def test_regrid_is_the_summation_at_the_new_points(ctx, kind):
    """Against the oracle's Base_spectral::summation (restated from
    src/Ope_1d/summation_1d.cpp) of the coarse field at every collocation
    point of the fine space, infinity included."""
    from kadath_frontera_gb300.kadath import CHEB_TYPE, Scalar, Space_spheric
    coarse = Space_spheric(CHEB_TYPE, (0, 0, 0), (9, 5, 4), BOUNDS)
    fine = Space_spheric(CHEB_TYPE, (0, 0, 0), (11, 7, 6), BOUNDS)
    f = _field(coarse, kind, _values(kind))
    g = Scalar(fine).regrid_from(f)
    odoms = K.space_spheric((9, 5, 4), list(BOUNDS))
    fdoms = K.space_spheric((11, 7, 6), list(BOUNDS))
    for dc, dn in zip(odoms, fdoms):
        base = dc.std_base() if kind == "std" else configs._anti(dc)
        vd = K.VD(dc, 1, c=f.get_domain(dc.num)[None].copy(), base=base)
        got = g.get_domain(dn.num)
        for i in range(dn.np[0]):
            for j in range(dn.np[1]):
                for k in range(dn.np[2]):
                    ref = K.summation(vd, (dn.x[i], dn.theta[j], dn.phi[k]))[0]
                    assert abs(got[i, j, k] - ref) <= 1e-12 * max(1.0, abs(ref)), (dn.num, i, j, k)


def test_tov_sequence_over_resolutions_with_checkpoints(ctx, tmp_path):
    """The TOV stage at (9, 5, 4), regridded to (13, 9, 4) and solved again:
    the second stage starts near the solution, converges to the same fields
    as a solve at (13, 9, 4) from the initial guess, and its checkpoint is a
    Kadath save file of the converged state."""
    from kadath_frontera_gb300 import stages, workloads
    seq = stages.tov_sequence(((9, 5, 4), (13, 9, 4)), checkpoint_dir=tmp_path)
    assert seq[0]["error"] < 1e-10 and seq[1]["error"] < 1e-10
    direct = workloads.ns_tov((13, 9, 4))
    n_direct = workloads.solve(direct)
    assert seq[1]["updates"] < n_direct
    wl = seq[1]["workload"]
    nd = wl.space.get_nbr_domains()
    for (_, a), (_, b) in zip(wl.unknowns, direct.unknowns):
        for d in range(nd):
            x, y = a.get_coef(d), b.get_coef(d)
            assert np.linalg.norm(x - y) <= 1e-10 * max(np.linalg.norm(y), 1e-300)
    with open(seq[1]["checkpoint"], "rb") as fp:
        sp = KIO.read_space(fp)
        assert len(sp) == nd and sp[0]["np"] == (13, 9, 4)
        for _, fld in wl.unknowns:
            vals = KIO.read_scalar(fp, sp)
            for dd, (base, zero, conf, coef) in enumerate(vals):
                if coef is not None:
                    assert np.array_equal(coef.reshape(-1), fld.get_coef(dd).reshape(-1))
                elif conf is not None:
                    assert np.array_equal(conf, fld.get_domain(dd))
        assert fp.read() == b""


def test_stage_that_cannot_converge_reports_noconv(ctx):
    from kadath_frontera_gb300 import KadathError, workloads
    from kadath_frontera_gb300._lib import KD_ERR_NOCONV
    wl = workloads.ns_tov((9, 5, 4))
    with pytest.raises(KadathError) as e:
        wl.syst.stage_solve(1e-10, max_iter=1)
    assert e.value.status == KD_ERR_NOCONV
