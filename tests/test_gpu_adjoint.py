"""Adjoint sensitivities dQ/dp of a converged solution (implicit-function
theorem), checked against central finite differences of full Newton re-solves
on the GPU and with the CPU oracle, and through the torch.autograd.Function.

Q is a field's value at a point, or an integral observable: the ADM-mass
form M = -1/(2 pi) * integral at infinity of dn(psi) (FUKA's intMadm,
include/Solvers/fuka_syst/fuka_syst_setup.hpp:62) and a volume integral.
J^T lambda = g is solved either with a new FP64 factorisation or by GMRES on
J^T preconditioned by the mixed-precision factors of the last Newton step,
transposed (no new factorisation)."""
import math

import numpy as np
import pytest

from oracle import configs, kadath as K

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

RES = (9, 5, 4)
POINTS = [(0.3, 0.2, 0.4), (1.2, -0.5, 0.7), (3.0, 1.0, -2.0)]  # nucleus, shell, compactified domain


def build(amp):
    from kadath_frontera_gb300.kadath import CHEB_TYPE, OUTER_BC, Scalar, Space_spheric, System_of_eqs
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), RES, (1.0, 2.0))
    nd = space.get_nbr_domains()
    psi = Scalar(space, 1.0).std_base()
    rho = Scalar(space)
    doms = K.space_spheric(RES, [1.0, 2.0])
    for d in range(nd):
        rho.set_domain(d, configs.toy_rho(doms[d]))
    rho.std_base()
    syst = System_of_eqs(space, 0, nd - 1)
    syst.add_var("psi", psi)
    syst.add_cst("pi", math.pi)
    syst.add_cst("amp", amp)
    syst.add_cst("rho", rho)
    for d in range(nd):
        syst.add_eq_inside(d, "Lap(psi) + 2*pi*amp*rho*psi^5 = 0")
    for d in range(nd - 1):
        syst.add_eq_matching(d, OUTER_BC, "psi")
        syst.add_eq_matching(d, OUTER_BC, "dn(psi)")
    syst.add_eq_bc(nd - 1, OUTER_BC, "psi = 1")
    return space, syst, psi, rho


def solve(syst, prec=1e-12):
    for _ in range(30):
        done, err = syst.do_newton(prec)
        if done:
            return
    raise AssertionError("no convergence")


def oracle_solve(amp):
    """The oracle's own Newton solve of the same problem (the CPU reference
    path); returns (domains, psi)."""
    doms = K.space_spheric(RES, [1.0, 2.0])
    psi = K.scalar_field(doms, lambda d: np.ones(d.np))
    nd = len(doms)
    sysm = K.OSystem(doms, 0, nd - 1)
    sysm.add_var("psi", psi)
    rho = K.scalar_field(doms, configs.toy_rho)
    for d in range(nd):
        rh = rho[d]

        # Lap(psi) + (((2*pi)*amp)*rho)*(psi^5), as the string is parsed
        def eq(T, b, rh=rh):
            p = T["psi"]
            rho_t = K.OTerm(p.dom, rh, None if p.der is None else K.VD.zeros(rh.dom, p.der.B))
            c = K.OTerm(p.dom, 2 * math.pi * amp, None if p.der is None else 0.0)
            return p.lap() + (c * rho_t) * p ** 5
        sysm.add_eq_inside(d, eq)
    for d in range(nd - 1):
        sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b: T["psi"])
        sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b: T["psi"].dn(b))
    sysm.add_eq_bc(nd - 1, K.OUTER_BC, lambda T, b: T["psi"] - 1.0)
    for _ in range(30):
        done, *_ = sysm.newton_step(1e-12)
        if done:
            break
    return doms, psi


def oracle_q(amp, point):
    doms, psi = oracle_solve(amp)
    return K.val_point(doms, psi, point)


def oracle_madm(amp):
    """-1/(2 pi) * the integral at infinity of dn(psi) (Domain_compact::integ)."""
    doms, psi = oracle_solve(amp)
    d = doms[-1]
    dn = K.OTerm(d, psi[d.num]).dn(K.OUTER_BC).val
    return float(-K.integ_surface(dn, K.OUTER_BC)[0] / (2 * math.pi))


def test_val_point_matches_oracle(ctx):
    space, syst, psi, rho = build(1.0)
    solve(syst)
    doms = K.space_spheric(RES, [1.0, 2.0])
    of = {d.num: K.VD(d, 1, cf=psi.get_coef(d.num)[None], base=d.std_base()) for d in doms}
    for p in POINTS:
        assert abs(psi.val_point(p) - K.val_point(doms, of, p)) <= 1e-13


def test_dres_dcst_matches_central_difference(ctx):
    space, syst, psi, rho = build(1.0)
    syst.do_newton(1e-12)  # a non-trivial iterate
    fp = syst.dres_dcst("amp")
    h = 1e-3
    syst.set_cst("amp", 1.0 + h)
    Fp = syst.sec_member()
    syst.set_cst("amp", 1.0 - h)
    Fm = syst.sec_member()
    syst.set_cst("amp", 1.0)
    fd = (Fp - Fm) / (2 * h)  # F is linear in amp: exact up to roundoff
    assert np.linalg.norm(fp - fd) <= 1e-9 * np.linalg.norm(fd)


@pytest.mark.parametrize("point", POINTS)
def test_adjoint_matches_finite_differences(ctx, point):
    space, syst, psi, rho = build(1.0)
    solve(syst)
    g = syst.val_point_gradient("psi", point)
    dqdp, lam = syst.adjoint(g, "amp")
    h = 1e-4
    qs = []
    for a in (1.0 + h, 1.0 - h):
        syst.set_cst("amp", a)
        solve(syst)
        qs.append(psi.val_point(point))
    fd = (qs[0] - qs[1]) / (2 * h)
    assert abs(dqdp - fd) <= 1e-6 * abs(fd), (dqdp, fd)
    # and against the CPU oracle's own finite difference of re-solves
    ofd = (oracle_q(1.0 + h, point) - oracle_q(1.0 - h, point)) / (2 * h)
    assert abs(dqdp - ofd) <= 1e-6 * abs(ofd), (dqdp, ofd)


def test_autograd_function(ctx):
    from kadath_frontera_gb300.adjoint import converged_observable
    space, syst, psi, rho = build(1.0)
    p = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    q = converged_observable(p, syst, psi, "psi", "amp", POINTS[0])
    q.backward()
    h = 1e-4
    qp = converged_observable(torch.tensor(1.0 + h, dtype=torch.float64), syst, psi, "psi", "amp", POINTS[0])
    qm = converged_observable(torch.tensor(1.0 - h, dtype=torch.float64), syst, psi, "psi", "amp", POINTS[0])
    fd = float(qp - qm) / (2 * h)
    assert abs(float(p.grad) - fd) <= 1e-6 * abs(fd)


MADM = "integ(dn(psi))"  # Q = -integ(dn(psi)) / (2 pi)


def test_integral_gradient_matches_central_differences(ctx):
    """dQ/dy of the ADM-mass integral (linear in the fields: the difference
    is exact up to rounding) and of a volume integral of psi^5 (second-order
    differences with a small step: along a random coefficient direction the
    quintic's third derivative is large), along a random direction of the
    unknown vector."""
    space, syst, psi, rho = build(1.0)
    syst.do_newton(1e-12)  # a non-trivial iterate
    n = syst.get_nbr_unknowns()
    dy = np.random.default_rng(3).standard_normal(n)
    # the update path u <- u - x rounds the coefficients (about 1e-11 in Q
    # after three updates), which bounds the differences' accuracy
    for expr, kind, doms, h, tol in ((MADM, "inf", None, 1e-1, 1e-8),
                                     ("integvolume(psi^5)", "volume", (0, 1), 1e-6, 1e-6)):
        q0, g = syst.integral_gradient(expr, kind, doms)
        syst.xx_to_vars_update(-h * dy)  # u + h dy
        qp, _ = syst.integral_gradient(expr, kind, doms)
        syst.xx_to_vars_update(2 * h * dy)  # u - h dy
        qm, _ = syst.integral_gradient(expr, kind, doms)
        syst.xx_to_vars_update(-h * dy)
        q1, _ = syst.integral_gradient(expr, kind, doms)
        assert abs(q1 - q0) <= 1e-10 * max(1.0, abs(q0))
        fd = (qp - qm) / (2 * h)
        assert abs(g @ dy - fd) <= tol * max(abs(fd), 1e-300), (expr, g @ dy, fd)


def test_integral_value_matches_oracle(ctx):
    space, syst, psi, rho = build(1.0)
    solve(syst)
    q, _ = syst.integral_gradient(MADM, "inf")
    doms = K.space_spheric(RES, [1.0, 2.0])
    d = doms[-1]
    v = K.VD(d, 1, cf=psi.get_coef(d.num)[None], base=d.std_base())
    ref = K.integ_surface(K.OTerm(d, v).dn(K.OUTER_BC).val, K.OUTER_BC)[0]
    assert abs(q - ref) <= 1e-12 * abs(ref)


def test_transposed_mixed_solve_matches_lapack(ctx):
    from kadath_frontera_gb300.kadath import DenseLU, KD_LU_TF32_IR
    n = 1500
    rng = np.random.default_rng(11)
    u, _ = np.linalg.qr(rng.standard_normal((n, n)))
    v, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = (u * np.logspace(0, -4, n)) @ v.T
    b = rng.standard_normal(n)
    lu = DenseLU(ctx)
    dA = torch.tensor(A.T.copy(), device="cuda")  # column-major A
    lu.factor(dA.data_ptr(), n, n, KD_LU_TF32_IR)
    db = torch.tensor(b, device="cuda")
    lu.solve(db.data_ptr(), trans=1)
    x = db.cpu().numpy()
    ref = np.linalg.solve(A.T, b)
    assert np.linalg.norm(x - ref) <= 1e-10 * np.linalg.norm(ref)
    assert np.linalg.norm(A.T @ x - b) <= 1e-12 * np.linalg.norm(b)


@pytest.mark.parametrize("reuse", [False, True])
def test_adm_mass_adjoint_matches_finite_differences(ctx, reuse):
    """dM/damp for the ADM-mass integral, by the adjoint with a new FP64
    factorisation or with the mixed factors of the last Newton step reused,
    against central differences of full re-solves on the GPU and with the
    oracle."""
    from kadath_frontera_gb300.kadath import KD_LU_FP64, KD_LU_TF32_IR
    space, syst, psi, rho = build(1.0)
    mode = KD_LU_TF32_IR if reuse else KD_LU_FP64
    for _ in range(30):
        done, _ = syst.do_newton(1e-12, lu_mode=mode)
        if done:
            break
    q, g = syst.integral_gradient(MADM, "inf")
    dqdp, lam = syst.adjoint(-g / (2 * math.pi), "amp", reuse_factors=reuse)
    assert syst.last_adjoint_report["reused_factors"] == int(reuse)
    if reuse:
        assert syst.last_adjoint_report["rel_residual"] < 1e-12
    h = 1e-4
    qs = []
    for a in (1.0 + h, 1.0 - h):
        syst.set_cst("amp", a)
        solve(syst)
        qs.append(-syst.integral_gradient(MADM, "inf")[0] / (2 * math.pi))
    syst.set_cst("amp", 1.0)
    fd = (qs[0] - qs[1]) / (2 * h)
    assert abs(dqdp - fd) <= 1e-6 * abs(fd), (dqdp, fd)
    ofd = (oracle_madm(1.0 + h) - oracle_madm(1.0 - h)) / (2 * h)
    assert abs(dqdp - ofd) <= 1e-6 * abs(ofd), (dqdp, ofd)


def test_reused_factors_give_the_fp64_adjoint(ctx):
    """lambda from GMRES on J^T with the mixed factors of the last step equals
    lambda from the FP64 factors of J at the converged fields."""
    from kadath_frontera_gb300.kadath import KD_LU_TF32_IR
    space, syst, psi, rho = build(1.0)
    for _ in range(30):
        done, _ = syst.do_newton(1e-12, lu_mode=KD_LU_TF32_IR)
        if done:
            break
    g = syst.val_point_gradient("psi", POINTS[1])
    d1, lam1 = syst.adjoint(g, "amp", reuse_factors=True)
    assert syst.last_adjoint_report["reused_factors"] == 1
    d0, lam0 = syst.adjoint(g, "amp", reuse_factors=False)
    assert syst.last_adjoint_report["reused_factors"] == 0
    assert np.linalg.norm(lam1 - lam0) <= 1e-10 * np.linalg.norm(lam0)
    assert abs(d1 - d0) <= 1e-10 * abs(d0)


def test_autograd_integral_with_reused_factors(ctx):
    from kadath_frontera_gb300.adjoint import converged_integral
    from kadath_frontera_gb300.kadath import KD_LU_TF32_IR
    space, syst, psi, rho = build(1.0)
    sc = -1.0 / (2 * math.pi)
    p = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    q = converged_integral(p, syst, MADM, "amp", scale=sc, lu_mode=KD_LU_TF32_IR, reuse_factors=True)
    q.backward()
    assert syst.last_adjoint_report["reused_factors"] == 1
    h = 1e-4
    qp = converged_integral(torch.tensor(1.0 + h, dtype=torch.float64), syst, MADM, "amp", scale=sc)
    qm = converged_integral(torch.tensor(1.0 - h, dtype=torch.float64), syst, MADM, "amp", scale=sc)
    fd = float(qp - qm) / (2 * h)
    assert abs(float(p.grad) - fd) <= 1e-6 * abs(fd)
