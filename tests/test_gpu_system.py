"""GPU parity of the Newton-Raphson path against the oracle: residual
(sec_member), dense Jacobian (all do_col_J columns), Newton updates and the
converged fields, on the toy configuration and the reference's known-answer
programs."""
import math

import numpy as np
import pytest

from oracle import configs, kadath as K

pytestmark = pytest.mark.gpu

REL = 1e-12     # residual / Jacobian, normwise relative (FP64 both sides)
FIELD = 1e-10   # converged fields: the bound the mixed-precision path must meet against the FP64 path


def build_toy(res=(13, 7, 4), bounds=(1.0, 2.0)):
    from kadath_frontera_gb300.kadath import CHEB_TYPE, OUTER_BC, Scalar, Space_spheric, System_of_eqs
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), res, bounds)
    nd = space.get_nbr_domains()
    psi = Scalar(space, 1.0).std_base()
    rho = Scalar(space)
    doms = K.space_spheric(res, list(bounds))
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
    return space, syst, psi, rho


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_toy_residual_and_jacobian_match_oracle(ctx):
    space, syst, psi, rho = build_toy()
    doms, osys, opsi, orho = configs.toy()
    F = syst.sec_member()
    Fo = osys.residual()
    assert F.shape == Fo.shape
    J = syst.jacobian()
    Fo2, Jo = osys.jacobian()
    assert J.shape == Jo.shape
    # F(u) at u = 1 is the roundoff of Lap(1) plus the source: compare on the
    # scale of the operator (both sides amplify eps through the derivatives).
    scale = np.abs(Jo).max()
    assert np.abs(F - Fo).max() <= 1e-13 * scale
    assert rel(J, Jo) < REL
    # do_col_J column access
    assert rel(syst.do_col_J(5), Jo[:, 5]) < REL


def test_toy_newton_iterates_match_oracle(ctx):
    space, syst, psi, rho = build_toy()
    doms, osys, opsi, orho = configs.toy()
    for it in range(8):
        done, err = syst.do_newton(1e-10)
        odone, oerr, _, _ = osys.newton_step(1e-10)
        assert done == odone
        assert abs(err - oerr) <= 1e-10 * max(1.0, abs(oerr)) + 1e-13
        for d in range(space.get_nbr_domains()):
            g = psi.get_coef(d)
            o = opsi[d]
            o.coef()
            assert rel(g, o.cf[0]) < FIELD
        if done:
            break
    assert done


def test_tuto5_known_answer_gpu(ctx):
    from kadath_frontera_gb300.kadath import CHEB_TYPE, INNER_BC, OUTER_BC, Scalar, Space_spheric, System_of_eqs
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), (13, 5, 4), (1, 2, 4))
    field = Scalar(space, 1.0).std_base()
    syst = System_of_eqs(space, 1, 3)
    syst.add_var("F", field)
    syst.add_cst("a", 1.0)
    for d in range(1, 4):
        syst.add_eq_inside(d, "Lap(F)=0")
    syst.add_eq_bc(1, INNER_BC, "dn(F) + 0.5*F/a = 0")
    syst.add_eq_bc(3, OUTER_BC, "F=1")
    for d in range(1, 3):
        syst.add_eq_matching(d, OUTER_BC, "F")
        syst.add_eq_matching(d, OUTER_BC, "dn(F)")
    n = 0
    while True:
        done, err = syst.do_newton(1e-8)
        if done:
            break
        n += 1
        assert n < 5
    assert n == 1
    doms = K.space_spheric((13, 5, 4), [1.0, 2.0, 4.0])
    of = {d.num: K.VD(d, 1, cf=field.get_coef(d.num)[None], base=d.std_base()) for d in doms}
    num = K.val_point(doms, of, configs.TUTO_POINT)
    rr = math.sqrt(sum(c * c for c in configs.TUTO_POINT))
    assert abs(num - (1 + 1 / rr)) / num < 1e-8
    # the nucleus (outside the system) is zeroed by the update, as in the reference
    assert np.all(field.get_domain(0) == 0.0)


def test_tuto6_grad_scal_definition(ctx):
    """tutorials/tuto6.cpp: add_def with scal(grad(P), grad(P)); analytic log(1+a/r)."""
    from kadath_frontera_gb300.kadath import CHEB_TYPE, INNER_BC, OUTER_BC, Scalar, Space_spheric, System_of_eqs
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), (13, 5, 4), (1, 2, 4))
    field = Scalar(space, 1.0).std_base()
    syst = System_of_eqs(space, 1, 3)
    syst.add_var("P", field)
    syst.add_def("dP2 = scal(grad(P), grad(P))")
    syst.add_cst("a", 1.0)
    for d in range(1, 4):
        syst.add_eq_inside(d, "Lap(P) + dP2 = 0")
    syst.add_eq_bc(1, INNER_BC, "dn(P) + 0.5/a = 0")
    syst.add_eq_bc(3, OUTER_BC, "P=0")
    for d in range(1, 3):
        syst.add_eq_matching(d, OUTER_BC, "P")
        syst.add_eq_matching(d, OUTER_BC, "dn(P)")
    for it in range(20):
        done, err = syst.do_newton(1e-8)
        if done:
            break
    assert done
    doms = K.space_spheric((13, 5, 4), [1.0, 2.0, 4.0])
    of = {d.num: K.VD(d, 1, cf=field.get_coef(d.num)[None], base=d.std_base()) for d in doms}
    num = K.val_point(doms, of, configs.TUTO_POINT)
    rr = math.sqrt(sum(c * c for c in configs.TUTO_POINT))
    ana = math.log(1 + 1 / rr)
    assert abs(num - ana) / abs(num) < 1e-6


def test_schwarz_matches_oracle_and_analytic(ctx):
    from kadath_frontera_gb300.kadath import CHEB_TYPE, Scalar, Space_spheric, System_of_eqs
    aa = 1.323
    bounds = (aa, 1.7557 * aa, 2.9861 * aa)
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), (13, 5, 4), bounds)
    conf = Scalar(space, 1.0).std_base()
    syst = System_of_eqs(space, 1, 3)
    syst.add_var("P", conf)
    syst.add_cst("a", aa)
    space.add_inner_bc(syst, "dn(P) + 0.5 / a * P = 0")
    space.add_eq(syst, "Lap(P) = 0", "P", "dn(P)")
    space.add_outer_bc(syst, "P=1")
    doms, osys, oP = configs.schwarz(aa=aa)
    while True:
        done, err = syst.do_newton(1e-8)
        odone, oerr, _, _ = osys.newton_step(1e-8)
        assert done == odone
        if done:
            break
    for d in range(1, 4):
        oP[d].coef()
        assert rel(conf.get_coef(d), oP[d].cf[0]) < FIELD


def test_unknown_variable_is_an_error(ctx):
    from kadath_frontera_gb300 import KadathError
    from kadath_frontera_gb300.kadath import CHEB_TYPE, Scalar, Space_spheric, System_of_eqs
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), (9, 5, 4), (1, 2))
    f = Scalar(space, 1.0).std_base()
    syst = System_of_eqs(space, 0, 2)
    syst.add_var("f", f)
    with pytest.raises(KadathError, match="Unknown operator"):
        syst.add_eq_inside(0, "Lap(g) = 0")


def test_star_workload_matches_oracle(ctx):
    """XCTS-shaped star (5 unknowns, vector Laplacian with Cartesian
    derivatives) at reduced resolution: residual, Jacobian and every Newton
    iterate against the oracle."""
    from kadath_frontera_gb300 import workloads
    res = (9, 5, 4)
    wl = workloads.star(res=res)
    doms, osys, ofields, _ = configs.star(res=res)
    F = wl.syst.sec_member()
    Fo = osys.residual()
    J = wl.syst.jacobian()
    _, Jo = osys.jacobian()
    assert np.abs(F - Fo).max() <= 1e-13 * np.abs(Jo).max()
    assert rel(J, Jo) < REL
    for it in range(6):
        done, err = wl.syst.do_newton(1e-10)
        odone, oerr, _, _ = osys.newton_step(1e-10)
        assert done == odone
        for (nm, f), of in zip(wl.unknowns, ofields):
            for d in range(len(doms)):
                of[d].coef()
                g = f.get_coef(d)
                scale = max(np.linalg.norm(of[d].cf[0]), 1e-12)
                assert np.linalg.norm(g - of[d].cf[0]) / scale < FIELD, (nm, d, it)
        if done:
            break
    assert done


def test_star_eight_phi_points_matter_in_shells_matches_oracle(ctx):
    """The large configuration's shape at small size: eight phi points,
    matter over the nucleus and three shells (r < 8), six domains."""
    from kadath_frontera_gb300 import workloads
    res, bounds = (7, 5, 8), (2.0, 4.0, 6.0, 8.0, 12.0)
    wl = workloads.star(res=res, bounds=bounds, matter_domains=4)
    doms, osys, ofields, _ = configs.star(res=res, bounds=bounds, matter_domains=4)
    F = wl.syst.sec_member()
    J = wl.syst.jacobian()
    Fo, Jo = osys.jacobian()
    assert F.shape == Fo.shape
    assert np.abs(F - Fo).max() <= 1e-13 * np.abs(Jo).max()
    assert rel(J, Jo) < REL
    done, err = wl.syst.do_newton(1e-10)
    odone, oerr, _, _ = osys.newton_step(1e-10)
    assert abs(err - oerr) <= 1e-12 * max(1.0, oerr)
    for (nm, f), of in zip(wl.unknowns, ofields):
        for d in range(len(doms)):
            of[d].coef()
            g = f.get_coef(d)
            scale = max(np.linalg.norm(of[d].cf[0]), 1e-12)
            assert np.linalg.norm(g - of[d].cf[0]) / scale < FIELD, (nm, d)


def test_star_mixed_precision_newton_matches_fp64(ctx):
    """The mixed-precision LU (TF32 trailing updates + FP64 GMRES-IR) gives the
    same Newton iterates as the FP64 LU to 1e-10."""
    from kadath_frontera_gb300 import workloads
    from kadath_frontera_gb300.kadath import KD_LU_FP64, KD_LU_TF32_IR
    res = (9, 5, 4)
    a = workloads.star(res=res)
    b = workloads.star(res=res)
    for it in range(6):
        da, ea = a.syst.do_newton(1e-10, lu_mode=KD_LU_FP64)
        db, eb = b.syst.do_newton(1e-10, lu_mode=KD_LU_TF32_IR)
        assert da == db
        if da:
            break
        for (nm, fa), (_, fb) in zip(a.unknowns, b.unknowns):
            for d in range(a.space.get_nbr_domains()):
                ga, gb = fa.get_coef(d), fb.get_coef(d)
                assert np.linalg.norm(ga - gb) <= 1e-10 * max(np.linalg.norm(ga), 1e-12)
    assert da


def test_star_tangent_cache_is_exact(ctx):
    """Tangents of iterate-independent subtrees kept from the first assembly
    give bitwise the same Jacobian, at a later iterate, as a system that
    recomputes every tangent; the iterates agree bitwise too."""
    from kadath_frontera_gb300 import workloads
    res = (9, 5, 4)
    a = workloads.star(res=res)
    b = workloads.star(res=res)
    b.syst.cache_tangents(False)
    for it in range(2):
        da, _ = a.syst.do_newton(1e-10)
        db, _ = b.syst.do_newton(1e-10)
        assert da == db
    Ja = a.syst.jacobian()
    Jb = b.syst.jacobian()
    assert np.array_equal(Ja, Jb)
    for (nm, fa), (_, fb) in zip(a.unknowns, b.unknowns):
        for d in range(a.space.get_nbr_domains()):
            assert np.array_equal(fa.get_coef(d), fb.get_coef(d)), (nm, d)


@pytest.mark.parametrize("which", ["toy", "star"])
def test_do_JX_matches_assembled_jacobian(ctx, which):
    """do_JX (matrix-free, all unknowns seeded by x through affecte_tau) equals
    J x with the assembled Jacobian, at the initial guess and after a step."""
    from kadath_frontera_gb300 import workloads
    wl = workloads.toy(res=(9, 5, 4)) if which == "toy" else workloads.star(res=(9, 5, 4))
    n = wl.syst.get_nbr_unknowns()
    rng = np.random.default_rng(3)
    for it in range(2):
        x = rng.standard_normal(n)
        J = wl.syst.jacobian()
        y = wl.syst.do_JX(x)
        ref = J @ x
        assert np.linalg.norm(y - ref) <= 1e-12 * np.linalg.norm(np.abs(J) @ np.abs(x))
        wl.syst.do_newton(1e-10)


def test_linesearch_newton_matches_oracle(ctx):
    """do_newton_with_linesearch from a far initial guess (psi = 3), where the
    full Newton step is rejected: the backtracked lambdas (quadratic, then
    cubic model, with the max(p) <= stepmax rescaling) and every iterate
    against the oracle's restatement."""
    from kadath_frontera_gb300 import workloads
    res = (9, 5, 4)
    wl = workloads.toy(res=res)
    psi = wl.unknowns[0][1]
    for d in range(wl.space.get_nbr_domains()):
        psi.set_domain(d, np.full(psi.get_domain(d).shape, 3.0))
    psi.std_base()
    doms, osys, opsi, _ = configs.toy(res=res)
    for d in opsi:
        opsi[d] = K.VD(doms[d], 1, c=np.full((1,) + tuple(doms[d].nc[:2]) + (doms[d].nc[2] - 2,), 3.0),
                       base=doms[d].std_base())
    lams = []
    for it in range(4):
        done, err, lam = wl.syst.do_newton_with_linesearch(1e-10, ntrymax=10, stepmax=1.0)
        odone, oerr, olam = K.newton_linesearch_step(osys, 1e-10, ntrymax=10, stepmax=1.0)
        assert done == odone
        assert abs(err - oerr) <= 1e-9 * abs(oerr)
        assert abs(lam - olam) <= 1e-8 * abs(olam), (it, lam, olam)
        lams.append(lam)
        for d in range(len(doms)):
            opsi[d].coef()
            assert rel(psi.get_coef(d), opsi[d].cf[0]) < 1e-9, (it, d)
    assert min(lams) < 1.0  # the backtracking branch ran


def test_eos_operators_match_oracle(ctx):
    """User EOS operators eps/press/rho/dHdlnrho (add_ope with
    EOS<Cold_PWPoly, var>::action) of the Gamma = 2, K = 100 polytrope inside
    an equation: residual, Jacobian and Newton iterates against the oracle."""
    from kadath_frontera_gb300.kadath import (CHEB_TYPE, OUTER_BC, KD_EOS_DENSITY, KD_EOS_DHDRHO, KD_EOS_EPSILON,
                                              KD_EOS_PRESSURE, Scalar, Space_spheric, System_of_eqs)
    res = (9, 5, 4)
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), res, (1.0, 2.0))
    nd = space.get_nbr_domains()
    psi = Scalar(space, 1.0).std_base()
    syst = System_of_eqs(space, 0, nd - 1)
    syst.add_var("psi", psi)
    for nm, v in (("eps", KD_EOS_EPSILON), ("press", KD_EOS_PRESSURE), ("rho", KD_EOS_DENSITY),
                  ("dHdlnrho", KD_EOS_DHDRHO)):
        syst.add_ope_eos(nm, v)
    eq = "Lap(psi) + 30*rho(1.001*psi^2) + 2*press(1.001*psi^2) - 3*eps(1.001*psi^2) + 0.1*dHdlnrho(1.001*psi^2) = 0"
    for d in range(nd):
        syst.add_eq_inside(d, eq)
    for d in range(nd - 1):
        syst.add_eq_matching(d, OUTER_BC, "psi")
        syst.add_eq_matching(d, OUTER_BC, "dn(psi)")
    syst.add_eq_bc(nd - 1, OUTER_BC, "psi = 1")

    doms = K.space_spheric(res, [1.0, 2.0])
    opsi = K.scalar_field(doms, lambda d: np.ones(d.np))
    osys = K.OSystem(doms, 0, nd - 1)
    osys.add_var("psi", opsi)
    E = K.polytrope()

    def oeq(T, b):
        p = T["psi"]
        c = lambda x: K.OTerm(p.dom, x, None if p.der is None else 0.0)  # noqa: E731
        h = c(1.001) * p ** 2
        return (p.lap() + c(30.0) * K.eos_term(h, E, 2) + c(2.0) * K.eos_term(h, E, 1)
                - c(3.0) * K.eos_term(h, E, 0) + c(0.1) * K.eos_term(h, E, 3))
    for d in range(nd):
        osys.add_eq_inside(d, oeq)
    for d in range(nd - 1):
        osys.add_eq_matching(d, K.OUTER_BC, lambda T, b: T["psi"])
        osys.add_eq_matching(d, K.OUTER_BC, lambda T, b: T["psi"].dn(b))
    osys.add_eq_bc(nd - 1, K.OUTER_BC, lambda T, b: T["psi"] - 1.0)

    F = syst.sec_member()
    J = syst.jacobian()
    Fo, Jo = osys.jacobian()
    assert np.abs(F - Fo).max() <= 1e-12 * max(np.abs(Fo).max(), 1.0)
    assert rel(J, Jo) < REL
    for it in range(5):
        done, err = syst.do_newton(1e-10)
        odone, oerr, _, _ = osys.newton_step(1e-10)
        assert done == odone
        for d in range(nd):
            opsi[d].coef()
            assert rel(psi.get_coef(d), opsi[d].cf[0]) < FIELD, (it, d)
        if done:
            break
