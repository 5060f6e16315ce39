"""Oracle builders for the reference's known-answer programs and the toy
configuration (TEST INFRASTRUCTURE ONLY; see oracle/kadath.py).

* tuto5   -- tutorials/tuto5.cpp: Lap F = 0 in three shells + compact,
             dn(F) + 0.5 F/a = 0 at r = a = 1, F = 1 at infinity;
             analytic F = 1 + a/r, checked at the point (1.3873, -0.827, 0.982).
* tuto6   -- tutorials/tuto6.cpp: Lap P + grad(P).grad(P) = 0,
             dn(P) + 0.5/a = 0, P = 0 at infinity; analytic P = log(1 + a/r).
* schwarz -- codes/Seq_version/schwarz.cpp: conformal factor of a
             Schwarzschild slice, a = 1.323, bounds a, 1.7557a, 2.9861a.
* toy     -- the CPU-runnable configuration: nucleus r<1, shell 1<r<2,
             compact r>2, (13, 7, 4) points, Lap psi = -2 pi rho psi^5 with
             rho = 0.05 exp(-r^2/0.25), psi -> 1 at infinity, continuity of
             psi and dn(psi) at r = 1, 2; initial guess psi = 1.
"""
from __future__ import annotations

import math

import numpy as np

from . import kadath as K

TUTO_POINT = (1.3873, -0.827, 0.982)


def tuto5(nr=13, nt=5, npp=4):
    doms = K.space_spheric((nr, nt, npp), [1.0, 2.0, 4.0])
    F = K.scalar_field(doms, lambda d: np.ones(d.np))
    sysm = K.OSystem(doms, 1, 3)
    sysm.add_var("F", F)
    a = 1.0
    for d in range(1, 4):
        sysm.add_eq_inside(d, lambda T, b: T["F"].lap())
    sysm.add_eq_bc(1, K.INNER_BC, lambda T, b: T["F"].dn(b) + 0.5 * T["F"] / a)
    sysm.add_eq_bc(3, K.OUTER_BC, lambda T, b: T["F"] - 1.0)
    for d in range(1, 3):
        sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b: T["F"])
        sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b: T["F"].dn(b))
    return doms, sysm, F


def schwarz(nbr=13, aa=1.323):
    bounds = [aa, 1.7557 * aa, 2.9861 * aa]
    doms = K.space_spheric((nbr, 5, 4), bounds)
    P = K.scalar_field(doms, lambda d: np.ones(d.np))
    sysm = K.OSystem(doms, 1, 3)
    sysm.add_var("P", P)
    sysm.add_eq_bc(1, K.INNER_BC, lambda T, b: T["P"].dn(b) + 0.5 / aa * T["P"])
    for d in range(1, 3):
        sysm.add_eq_inside(d, lambda T, b: T["P"].lap())
        sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b: T["P"])
        sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b: T["P"].dn(b))
    sysm.add_eq_inside(3, lambda T, b: T["P"].lap())
    sysm.add_eq_bc(3, K.OUTER_BC, lambda T, b: T["P"] - 1.0)
    return doms, sysm, P


def toy_rho(d):
    r = d.radius()
    with np.errstate(over="ignore", invalid="ignore"):
        v = 0.05 * np.exp(-r * r / 0.25)
    v[~np.isfinite(r)] = 0.0
    return v


def toy(res=(13, 7, 4), bounds=(1.0, 2.0)):
    doms = K.space_spheric(res, list(bounds))
    psi = K.scalar_field(doms, lambda d: np.ones(d.np))
    rho = K.scalar_field(doms, toy_rho)
    nd = len(doms)
    sysm = K.OSystem(doms, 0, nd - 1)
    sysm.add_var("psi", psi)
    two_pi = 2 * math.pi
    for d in range(nd):
        rh = rho[d]
        # parsed by Kadath as Lap(psi) + (((2*pi)*rho)*(psi^5))
        def eq(T, b, rh=rh):
            p = T["psi"]
            rho_t = K.OTerm(p.dom, rh, None if p.der is None else K.VD.zeros(rh.dom, p.der.B))
            c = K.OTerm(p.dom, two_pi, None if p.der is None else 0.0)
            return p.lap() + (c * rho_t) * p ** 5
        sysm.add_eq_inside(d, eq)
    for d in range(nd - 1):
        sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b: T["psi"])
        sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b: T["psi"].dn(b))
    sysm.add_eq_bc(nd - 1, K.OUTER_BC, lambda T, b: T["psi"] - 1.0)
    return doms, sysm, psi, rho


# The same systems as strings, for the product's parser (Kadath syntax).
TOY_EQUATIONS = {
    "inside": "Lap(psi) + 2*pi*rho*psi^5 = 0",
    "matching": ["psi", "dn(psi)"],
    "outer": "psi = 1",
}
