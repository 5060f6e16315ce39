"""Fields evaluated at arbitrary points on the GPU (kd_fields_val_points)
against the oracle's spectral summation (Scalar::val_point restated), in
every domain, on the axis, at the domain boundaries and at infinity, for
several fields with different bases at once."""
import math

import numpy as np
import pytest

from oracle import configs, kadath as K

pytestmark = pytest.mark.gpu


def _points(rng, n, rmax):
    # radii spread over all domains, directions uniform, plus special points
    r = rmax * rng.random(n) ** 2
    v = rng.standard_normal((n, 3))
    v /= np.linalg.norm(v, axis=1)[:, None]
    pts = v * r[:, None]
    special = np.array([[0, 0, 0], [0, 0, 0.7], [0, 0, -3.0], [1.0, 0, 0], [0, 2.0, 0], [0, 0, 12.0],
                        [1e6, 0, 0], [0.3, -0.2, 0.0]])
    return np.vstack([pts, special])


def test_star_fields_at_points_match_oracle(ctx):
    from kadath_frontera_gb300 import workloads
    from kadath_frontera_gb300.kadath import val_points
    wl = workloads.star(res=(9, 5, 4), ctx=ctx)
    for _ in range(2):
        wl.syst.do_newton(1e-10)
    # oracle copies of the GPU fields (coefficients and bases read back)
    doms = K.space_spheric((9, 5, 4), list(workloads.STAR_BOUNDS))
    fields = [f for _, f in wl.unknowns]
    pts = _points(np.random.default_rng(3), 400, 40.0)
    got = val_points(fields, pts)
    assert got.shape == (len(fields), len(pts))
    for fi, f in enumerate(fields):
        of = {}
        for d in range(len(doms)):
            cf = f.get_coef(d).reshape(doms[d].nc)
            br, bt, bp = f.get_base(d)
            base = K.OBase(np.asarray(br).reshape(doms[d].nc[1], doms[d].nc[2]), bt, bp)
            of[d] = K.VD(doms[d], 1, cf=cf[None].copy(), base=base)
        scale = max(np.abs(f.get_coef(d)).max() for d in range(len(doms)))
        for p in range(len(pts)):
            exp = K.val_point(doms, of, tuple(pts[p]))
            assert abs(got[fi, p] - exp) <= 1e-13 * max(scale, 1e-300) + 1e-15, (fi, p, pts[p])
    # the single-point entry point agrees too
    assert fields[0].val_point(tuple(pts[5])) == pytest.approx(got[0, 5], rel=1e-13, abs=1e-15)


def test_points_outside_every_domain_are_nan(ctx):
    from kadath_frontera_gb300.kadath import CHEB_TYPE, Scalar, Space_spheric, val_points
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), (9, 5, 4), (1.0, 2.0), withzec=False)
    f = Scalar(space, 1.0).std_base()
    got = val_points([f], np.array([[0.5, 0, 0], [3.0, 0, 0]]))
    assert got[0, 0] == pytest.approx(1.0)
    assert math.isnan(got[0, 1])


def test_analytic_field_at_points(ctx):
    """1 + (x y + z^2) / (1 + r^4): a field known in closed form, even in z
    as the symmetric spheric space requires, evaluated away from the
    collocation points (spectral accuracy of the summation itself)."""
    from kadath_frontera_gb300.kadath import CHEB_TYPE, Scalar, Space_spheric, val_points
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), (17, 9, 8), (1.0, 2.0, 4.0))
    f = Scalar(space)
    for d in range(space.get_nbr_domains()):
        x, y, z = (space.get_cart(d, c) for c in (1, 2, 3))
        r = space.get_radius(d)
        with np.errstate(invalid="ignore", divide="ignore"):
            v = np.where(np.isfinite(r), 1.0 + (x * y + z * z) / (1.0 + r ** 4), 1.0)
        f.set_domain(d, v)
    f.std_base()
    pts = _points(np.random.default_rng(5), 300, 30.0)[:-2]
    got = val_points([f], pts)[0]
    r = np.linalg.norm(pts, axis=1)
    exact = 1.0 + (pts[:, 0] * pts[:, 1] + pts[:, 2] ** 2) / (1.0 + r ** 4)
    assert np.abs(got - exact).max() < 1e-9
