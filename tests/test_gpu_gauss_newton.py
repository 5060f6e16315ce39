"""The Gauss-Newton variant of do_newton (SOLVER GAUSS_NEWTON,
src_par/do_newton.cpp:264-311) on an overdetermined, consistent system:
the toy problem with its outer condition stated twice.  The rectangular
Jacobian is compared with the oracle's, and both Gauss-Newton iterations
converge to the same fields."""
import math

import numpy as np
import pytest

from oracle import configs, kadath as K

pytestmark = pytest.mark.gpu


def build_toy_redundant(res):
    from kadath_frontera_gb300.kadath import CHEB_TYPE, OUTER_BC, Scalar, Space_spheric, System_of_eqs
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), res, (1.0, 2.0))
    nd = space.get_nbr_domains()
    psi = Scalar(space, 1.0).std_base()
    rho = Scalar(space)
    doms = K.space_spheric(res, [1.0, 2.0])
    for d in range(nd):
        rho.set_domain(d, configs.toy_rho(doms[d]))
    rho.std_base()
    syst = System_of_eqs(space, 0, nd - 1)
    syst.add_var("psi", psi)
    syst.add_cst("pi", math.pi)
    syst.add_cst("rho", rho)
    for d in range(nd):
        syst.add_eq_inside(d, "Lap(psi) + 2*pi*rho*psi^5 = 0")
    for d in range(nd - 1):
        syst.add_eq_matching(d, OUTER_BC, "psi")
        syst.add_eq_matching(d, OUTER_BC, "dn(psi)")
    syst.add_eq_bc(nd - 1, OUTER_BC, "psi = 1")
    syst.add_eq_bc(nd - 1, OUTER_BC, "psi = 1")
    return space, syst, psi, rho


def test_gauss_newton_matches_oracle(ctx):
    from kadath_frontera_gb300.kadath import GAUSS_NEWTON, KD_LU_FP64
    res = (7, 5, 4)
    space, syst, psi, rho = build_toy_redundant(res)
    doms, osys, opsi, orho = configs.toy(res=res)
    nd = len(doms)
    osys.add_eq_bc(nd - 1, K.OUTER_BC, lambda T, b: T["psi"] - 1.0)
    F = syst.sec_member()
    nu, nc = syst.sizes()
    assert nc > nu
    Fo, Jo = osys.jacobian(rectangular=True)
    assert np.abs(F - Fo).max() <= 1e-13 * np.abs(Jo).max()
    for it in range(10):
        done, err = syst.do_newton(1e-10, lu_mode=KD_LU_FP64, solver=GAUSS_NEWTON)
        odone, oerr, _, _ = osys.newton_step(1e-10, gauss_newton=True)
        if it == 0:
            assert abs(err - oerr) <= 1e-12 * max(1.0, abs(oerr))
        if done and odone:
            break
    assert done and odone
    for d in range(nd):
        g = np.asarray(psi.get_coef(d)).ravel()
        o = opsi[d]
        o.coef()
        assert np.linalg.norm(g - o.cf[0].ravel()) <= 1e-9 * max(np.linalg.norm(o.cf[0]), 1e-12)


def test_gauss_newton_rejects_underdetermined(ctx):
    from kadath_frontera_gb300 import KadathError
    from kadath_frontera_gb300.kadath import CHEB_TYPE, OUTER_BC, GAUSS_NEWTON, Scalar, Space_spheric, System_of_eqs
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), (7, 5, 4), (1.0, 2.0))
    psi = Scalar(space, 1.0).std_base()
    syst = System_of_eqs(space, 0, space.get_nbr_domains() - 1)
    syst.add_var("psi", psi)
    for d in range(space.get_nbr_domains()):
        syst.add_eq_inside(d, "Lap(psi) = 0")
    with pytest.raises(KadathError):
        syst.do_newton(1e-10, solver=GAUSS_NEWTON)
