"""Oracle restatement of the integral-type equations (Eq_int: integvolume,
integ at infinity, value at a collocation point) and of the double unknowns'
Jacobian columns: closed-form integrals, known-answer eigenvalue and
mass problems, and the Jacobian against finite differences."""
import math

import numpy as np
import pytest

from oracle import configs, kadath as K


def solve(sysm, prec, maxit=12):
    for it in range(maxit):
        done, err, F, J = sysm.newton_step(prec)
        if done:
            return it
    raise AssertionError("oracle Newton did not converge")


def _field(d, fn):
    r = d.radius()
    with np.errstate(divide="ignore", invalid="ignore"):
        v = np.where(np.isfinite(r), fn(np.where(np.isfinite(r), r, 1.0)), 0.0)
    return K.VD(d, 1, c=v[None].copy(), base=d.std_base())


def test_volume_and_surface_integrals_closed_forms():
    doms = K.space_spheric((11, 5, 4), [1.0, 2.0])
    assert K.integ_volume(_field(doms[0], lambda r: 1.0 + 0 * r))[0] == pytest.approx(4 * math.pi / 3, rel=1e-13)
    assert K.integ_volume(_field(doms[1], lambda r: 1.0 + 0 * r))[0] == pytest.approx(28 * math.pi / 3, rel=1e-13)
    # r^-4 outside r = 2: 4 pi / 2
    assert K.integ_volume(_field(doms[2], lambda r: r ** -4))[0] == pytest.approx(2 * math.pi, rel=1e-10)
    # r^2 weighted sphere at infinity of r^-2: 4 pi
    assert K.integ_surface(_field(doms[2], lambda r: r ** -2), K.OUTER_BC)[0] == pytest.approx(4 * math.pi, rel=1e-12)


@pytest.mark.parametrize("normalise", ["val", "integral"])
def test_eigenvalue_known_answer(normalise):
    doms, sysm, u = configs.eigen_nucleus((11, 5, 4), normalise)
    solve(sysm, 1e-12)
    lam = sysm.vdoubles[0][1]
    assert abs(lam - math.pi ** 2) < 1e-10
    v = K.val_point(doms, u, (0.3, 0.2, 0.25))
    r = math.sqrt(0.09 + 0.04 + 0.0625)
    exact = math.sin(math.pi * r) / (math.pi * r)
    assert abs(v - exact) < 1e-9


def test_mass_at_infinity_known_answer():
    doms, sysm, P = configs.mass_at_infinity((15, 5, 4))
    solve(sysm, 1e-10)
    assert abs(sysm.vdoubles[0][1] - 1.0) < 1e-8
    assert K.val_point(doms, P, (0.3, 1.2, 2.1)) == pytest.approx(1 + 1 / math.sqrt(5.94), rel=1e-8)


@pytest.mark.parametrize("which", ["eigen_val", "eigen_integral", "mass"])
def test_jacobian_with_doubles_matches_finite_differences(which):
    if which == "mass":
        doms, sysm, f = configs.mass_at_infinity((9, 5, 4))
        name, dmin, dmax = "P", 1, 3
    else:
        doms, sysm, f = configs.eigen_nucleus((9, 5, 4), which.split("_")[1])
        name, dmin, dmax = "u", 0, 0
    F0, J = sysm.jacobian()
    assert J.shape[0] == J.shape[1] == len(F0)
    # column of the double unknown: central difference of F in that number
    h = 1e-6
    v0 = sysm.vdoubles[0][1]
    sysm.vdoubles[0][1] = v0 + h
    Fp = sysm.residual()
    sysm.vdoubles[0][1] = v0 - h
    Fm = sysm.residual()
    sysm.vdoubles[0][1] = v0
    col = (Fp - Fm) / (2 * h)
    assert np.abs(col - J[:, 0]).max() < 1e-6 * max(1.0, np.abs(J[:, 0]).max())
    # the integral row against a random direction of the field unknowns
    layout, N = sysm.unknown_layout()
    rng = np.random.default_rng(0)
    x = np.zeros(N)
    x[1:] = rng.standard_normal(N - 1) * 1e-3
    jx = J @ x
    saved = {d: f[d] for d in range(len(doms))}
    for vi, dd, c0, pats in layout:
        d = doms[dd]
        M = d.affecte_tau_matrix(f[dd].base)
        cf = (M @ x[c0:c0 + M.shape[1]]).reshape((1,) + d.nc)
        f[dd] = saved[dd] + K.VD(d, 1, cf=cf, base=f[dd].base)
    F1 = sysm.residual()
    for dd in saved:
        f[dd] = saved[dd]
    # residuals are linear in the field for the integral rows
    assert abs((F1 - F0)[0] - jx[0]) < 1e-9 * max(1.0, abs(jx[0]))
