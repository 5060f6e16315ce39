"""Adjoint sensitivities dQ/dp of a converged solution (implicit-function
theorem, transposed solve with the FP64 factors), checked against central
finite differences of full Newton re-solves on the GPU and with the CPU
oracle, and through the torch.autograd.Function."""
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


def oracle_q(amp, point):
    """Q(amp) with the oracle's own Newton solver (the CPU reference path)."""
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
    return K.val_point(doms, psi, point)


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
