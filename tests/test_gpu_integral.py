"""GPU parity of the integral-type equations (Eq_int: integvolume, integ at
infinity, the value at a collocation point) and of the double unknowns'
Jacobian columns against the oracle, and the known answers: the Helmholtz
eigenvalue pi^2 of the unit nucleus, and the mass M = 1 of P = 1 + M/r read
from the surface integral at infinity."""
import math

import numpy as np
import pytest

from oracle import configs, kadath as K

pytestmark = pytest.mark.gpu

REL = 1e-12     # residual / Jacobian, normwise relative (FP64 both sides)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def build_eigen(res, normalise, lam0=9.0):
    from kadath_frontera_gb300.kadath import CHEB_TYPE, OUTER_BC, Scalar, Space_spheric, System_of_eqs
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), res, (1.0, 2.0))
    u = Scalar(space)
    for d in range(space.get_nbr_domains()):
        r = space.get_radius(d)
        u.set_domain(d, (1 - 0.9 * r ** 2) if d == 0 else np.zeros_like(r))
    u.std_base()
    syst = System_of_eqs(space, 0, 0)
    syst.add_var("u", u)
    syst.add_var("lam", lam0)
    syst.add_cst("pi", math.pi)
    syst.add_eq_inside(0, "Lap(u) + lam*u = 0")
    syst.add_eq_bc(0, OUTER_BC, "u = 0")
    if normalise == "val":
        space.add_eq_ori(syst, "u - 1")
    else:
        syst.add_eq_int_volume(0, 0, "integvolume(u) = 4/pi")
    return space, syst, u


def build_mass(res, m0=0.5):
    from kadath_frontera_gb300.kadath import CHEB_TYPE, INNER_BC, OUTER_BC, Scalar, Space_spheric, System_of_eqs
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), res, (1.0, 2.0, 4.0))
    P = Scalar(space, 1.0).std_base()
    syst = System_of_eqs(space, 1, 3)
    syst.add_var("P", P)
    syst.add_var("M", m0)
    syst.add_cst("pi", math.pi)
    for d in range(1, 4):
        syst.add_eq_inside(d, "Lap(P) = 0")
    syst.add_eq_bc(1, INNER_BC, "P = 2")
    for d in range(1, 3):
        syst.add_eq_matching(d, OUTER_BC, "P")
        syst.add_eq_matching(d, OUTER_BC, "dn(P)")
    syst.add_eq_bc(3, OUTER_BC, "P = 1")
    syst.add_eq_int_inf("integ(dn(P)) + 4*pi*M = 0")
    return space, syst, P


def _build(which, res):
    if which == "mass":
        return build_mass(res), configs.mass_at_infinity(res)
    normalise = which.split("_")[1]
    return build_eigen(res, normalise), configs.eigen_nucleus(res, normalise)


@pytest.mark.parametrize("which", ["eigen_val", "eigen_integral", "mass"])
def test_residual_and_jacobian_with_doubles_match_oracle(ctx, which):
    (space, syst, f), (doms, osys, of) = _build(which, (9, 5, 4))
    F = syst.sec_member()
    Fo = osys.residual()
    assert F.shape == Fo.shape
    J = syst.jacobian()
    _, Jo = osys.jacobian()
    scale = np.abs(Jo).max()
    assert np.abs(F - Fo).max() <= 1e-13 * scale
    assert rel(J, Jo) < REL
    # the double unknown's column and the integral row, on their own
    assert rel(J[:, 0], Jo[:, 0]) < REL
    assert rel(J[0, :], Jo[0, :]) < REL
    # do_JX through the same tangent rules
    x = np.random.default_rng(1).standard_normal(J.shape[0])
    assert rel(syst.do_JX(x), Jo @ x) < REL


@pytest.mark.parametrize("normalise", ["val", "integral"])
def test_eigenvalue_known_answer_gpu(ctx, normalise):
    space, syst, u = build_eigen((11, 5, 4), normalise)
    doms, osys, ou = configs.eigen_nucleus((11, 5, 4), normalise)
    for it in range(12):
        done, err = syst.do_newton(1e-12)
        odone, oerr, _, _ = osys.newton_step(1e-12)
        assert abs(err - oerr) <= 1e-10 * max(1.0, abs(oerr)) + 1e-13
        if done:
            break
    assert done
    lam = syst.get_var_double("lam")
    assert abs(lam - math.pi ** 2) < 1e-10
    assert abs(lam - osys.vdoubles[0][1]) < 1e-12
    r = math.sqrt(0.09 + 0.04 + 0.0625)
    assert abs(u.val_point((0.3, 0.2, 0.25)) - math.sin(math.pi * r) / (math.pi * r)) < 1e-9


def test_mass_at_infinity_known_answer_gpu(ctx):
    space, syst, P = build_mass((15, 5, 4))
    for it in range(12):
        done, err = syst.do_newton(1e-10)
        if done:
            break
    assert done
    assert abs(syst.get_var_double("M") - 1.0) < 1e-8
    assert P.val_point((0.3, 1.2, 2.1)) == pytest.approx(1 + 1 / math.sqrt(5.94), rel=1e-8)


def test_point_equation_matches_oracle(ctx):
    """add_eq_point: the value at an arbitrary point through the spectral
    summation, as the normalisation of the eigenproblem."""
    from kadath_frontera_gb300.kadath import CHEB_TYPE, OUTER_BC, Scalar, Space_spheric, System_of_eqs
    res = (9, 5, 4)
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), res, (1.0, 2.0))
    u = Scalar(space)
    for d in range(space.get_nbr_domains()):
        r = space.get_radius(d)
        u.set_domain(d, (1 - 0.9 * r ** 2) if d == 0 else np.zeros_like(r))
    u.std_base()
    syst = System_of_eqs(space, 0, 0)
    syst.add_var("u", u)
    syst.add_var("lam", 9.0)
    syst.add_eq_inside(0, "Lap(u) + lam*u = 0")
    syst.add_eq_bc(0, OUTER_BC, "u = 0")
    pt = (0.2, 0.1, 0.3)
    syst.add_eq_point(0, "u - 0.5", pt)

    doms, osys, ou = configs.eigen_nucleus(res, "val")
    osys.ieqs.clear()
    osys.add_eq_point(0, lambda T: T["u"] - 0.5, pt)
    F = syst.sec_member()
    Fo = osys.residual()
    J = syst.jacobian()
    _, Jo = osys.jacobian()
    assert np.abs(F - Fo).max() <= 1e-13 * np.abs(Jo).max()
    assert rel(J, Jo) < REL
    for it in range(12):
        done, err = syst.do_newton(1e-11)
        if done:
            break
    assert done
    assert abs(syst.get_var_double("lam") - math.pi ** 2) < 1e-9
    assert abs(u.val_point(pt) - 0.5) < 1e-10
