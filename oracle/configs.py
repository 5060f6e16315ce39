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


STAR_R = 8.0
STAR_RHOC = 1.28e-3
STAR_K = 100.0


def star_matter(d, matter_domains=1):
    """Frozen Gamma = 2 matter: Lane-Emden n = 1 density rho_c sinc(pi r/R)
    in the first matter_domains domains (the nucleus of radius R by default);
    E = rho (1 + K rho), S = 3 K rho^2."""
    r = d.radius()
    rho = np.zeros(d.np)
    if d.num < matter_domains:
        x = np.pi * r / STAR_R
        with np.errstate(invalid="ignore", divide="ignore"):
            rho = STAR_RHOC * np.where(x > 0, np.sin(x) / np.where(x > 0, x, 1.0), 1.0)
    E = rho * (1 + STAR_K * rho)
    S = 3 * STAR_K * rho * rho
    return E, S


def star(res=(13, 9, 4), bounds=(STAR_R, 12.0, 16.0, 24.0, 32.0), matter_domains=1):
    """XCTS-shaped static star (oracle side): unknowns P (conformal factor),
    NP (lapse times P) and the Cartesian shift components bx, by, bz."""
    doms = K.space_spheric(res, list(bounds))
    ones = lambda d: np.ones(d.np)
    P = K.scalar_field(doms, ones)
    NP = K.scalar_field(doms, ones)
    bx = K.scalar_field(doms, lambda d: np.zeros(d.np))
    by = K.scalar_field(doms, lambda d: np.zeros(d.np))
    bz = {d.num: K.VD(d, 1, c=np.zeros((1,) + d.np), base=_anti(d)) for d in doms}
    E = K.scalar_field(doms, lambda d: star_matter(d, matter_domains)[0])
    E2S = K.scalar_field(doms, lambda d: star_matter(d, matter_domains)[0] + 2 * star_matter(d, matter_domains)[1])
    nd = len(doms)
    sysm = K.OSystem(doms, 0, nd - 1)
    for name, f in (("P", P), ("NP", NP), ("bx", bx), ("by", by), ("bz", bz)):
        sysm.add_var(name, f)
    two_pi = 2 * math.pi

    def cst(T, v):
        p = T["P"]
        return K.OTerm(p.dom, v, None if p.der is None else K.VD.zeros(v.dom, p.der.B))

    def num(T, x):
        return K.OTerm(T["P"].dom, float(x), None if T["P"].der is None else 0.0)

    for d in range(nd):
        Ed, E2Sd = E[d], E2S[d]
        # parsed as Lap(P) + (2*pi)*(E/P) and Lap(NP) - ((2*pi)*NP)*(E2S/(P^2))
        sysm.add_eq_inside(d, lambda T, b, Ed=Ed: T["P"].lap() + num(T, two_pi) * (cst(T, Ed) / T["P"]))
        sysm.add_eq_inside(d, lambda T, b, E2Sd=E2Sd: T["NP"].lap() - (num(T, two_pi) * T["NP"]) *
                           (cst(T, E2Sd) / T["P"] ** 2))
        for c, name in ((1, "bx"), (2, "by"), (3, "bz")):
            def eqb(T, b, c=c, name=name):
                div = T["bx"].partial(1) + T["by"].partial(2) + T["bz"].partial(3)
                return T[name].lap() + div.partial(c) / num(T, 3.0)
            sysm.add_eq_inside(d, eqb)
    for d in range(nd - 1):
        for name in ("P", "NP", "bx", "by", "bz"):
            sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b, name=name: T[name])
            sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b, name=name: T[name].dn(b))
    sysm.add_eq_bc(nd - 1, K.OUTER_BC, lambda T, b: T["P"] - 1.0)
    sysm.add_eq_bc(nd - 1, K.OUTER_BC, lambda T, b: T["NP"] - 1.0)
    for name in ("bx", "by", "bz"):
        sysm.add_eq_bc(nd - 1, K.OUTER_BC, lambda T, b, name=name: T[name])
    return doms, sysm, (P, NP, bx, by, bz), (E, E2S)


def star_vector(res=(13, 9, 4), bounds=(STAR_R, 12.0, 16.0, 24.0, 32.0)):
    """The static star with the shift as one Cartesian vector unknown bet and
    its equations in index notation with the flat metric, as the product
    parses them:
      D_j D^j bet^i + D^i D_j bet^j / 3 = 0,  bet^i and dn(bet^i) matched,
      bet^i = 0 at infinity.
    D_j D^j X^i is sum_j d_j(d_j X^i) and D_j X^j is sum_j d_j X^j, each sum
    in the order j = 1, 2, 3 (Metric_flat::derive_partial_cart, then
    Tensor::do_summation_one_dom).  The unknowns of bet come domain by domain,
    x, y, z inside each domain (xx_to_vars)."""
    doms, _, (P, NP, bx, by, bz), (E, E2S) = star(res, bounds)
    nd = len(doms)
    sysm = K.OSystem(doms, 0, nd - 1)
    sysm.add_var("P", P)
    sysm.add_var("NP", NP)
    sysm.add_var_vector("bet", (bx, by, bz))
    two_pi = 2 * math.pi

    def cst(T, v):
        p = T["P"]
        return K.OTerm(p.dom, v, None if p.der is None else K.VD.zeros(v.dom, p.der.B))

    def num(T, x):
        return K.OTerm(T["P"].dom, float(x), None if T["P"].der is None else 0.0)

    def shift_eq(T, b):
        bet = T["bet"]
        div = bet[0].partial(1) + bet[1].partial(2) + bet[2].partial(3)
        out = []
        for i in range(3):
            d2 = [bet[i].partial(j).partial(j) for j in (1, 2, 3)]
            out.append((d2[0] + d2[1] + d2[2]) + div.partial(i + 1) / num(T, 3.0))
        return out

    for d in range(nd):
        Ed, E2Sd = E[d], E2S[d]
        sysm.add_eq_inside(d, lambda T, b, Ed=Ed: T["P"].lap() + num(T, two_pi) * (cst(T, Ed) / T["P"]))
        sysm.add_eq_inside(d, lambda T, b, E2Sd=E2Sd: T["NP"].lap() - (num(T, two_pi) * T["NP"]) *
                           (cst(T, E2Sd) / T["P"] ** 2))
        sysm.add_eq_inside(d, shift_eq)
    for d in range(nd - 1):
        for name in ("P", "NP"):
            sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b, name=name: T[name])
            sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b, name=name: T[name].dn(b))
        sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b: list(T["bet"]))
        sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b: [x.dn(b) for x in T["bet"]])
    sysm.add_eq_bc(nd - 1, K.OUTER_BC, lambda T, b: T["P"] - 1.0)
    sysm.add_eq_bc(nd - 1, K.OUTER_BC, lambda T, b: T["NP"] - 1.0)
    sysm.add_eq_bc(nd - 1, K.OUTER_BC, lambda T, b: list(T["bet"]))
    return doms, sysm, (P, NP, bx, by, bz), (E, E2S)


# Static TOV star with the log-enthalpy as unknown, in the shape of the
# reference's non-rotating NS stage (include/Solvers/ns_3d_xcts/
# ns_3d_xcts_stages.cpp:63-140, syst_init in ns_3d_xcts_solver_imp.cpp:89):
# the matter fills domains 0 and 1 and its outer radius is fixed (the
# "fixed" branch, here with a domain boundary that is not adapted).
NS_BOUNDS = (3.5, 7.0, 12.0, 18.0, 24.0)
NS_RHOC = 1.28e-3
NS_QPIG = 4 * math.pi


def ns_hc(rho_c=NS_RHOC, k=100.0):
    """log h at the centre of a Gamma = 2 polytrope: h = 1 + eps + p/rho = 1 + 2 K rho."""
    return math.log(1.0 + 2.0 * k * rho_c)


NS_DEFS_ALL = ["NP = P*N", "h = exp(H)", "rho = rho(h)", "eps = eps(h)", "press = press(h)",
               "delta = h - eps - 1."]
NS_DEFS_MATTER = ["Etilde = press * h - press * delta", "Stilde = 3 * press * delta",
                  "eqP = delta * D^i D_i P + 4piG / 2. * P^5 * Etilde",
                  "eqNP = delta * D^i D_i NP - 4piG / 2. * N * P^5 * (Etilde + 2. * Stilde)",
                  "firstint = H + log(N)"]
NS_DEFS_VACUUM = ["eqP = D^i D_i P", "eqNP = D^i D_i NP"]


def ns_tov(res=(9, 5, 4), bounds=NS_BOUNDS, rho_c=NS_RHOC):
    """Oracle side of the TOV system: unknowns H (log enthalpy), P, N in that
    order; H = 0 on every coefficient outside the matter (Eq_full); the first
    integral H + log(N) = const in domains 0..1 with H - Hc at the centre
    (Eq_first_integral); eqNP and eqP inside with N, dn(N), P, dn(P) matched
    (Space_spheric::add_eq); N = P = 1 at infinity.  Initial guess H = Hc in
    the matter and 0 outside, P = N = 1."""
    doms = K.space_spheric(res, list(bounds))
    nd = len(doms)
    eos = K.polytrope()
    hc = ns_hc(rho_c)
    H = K.scalar_field(doms, lambda d: np.full(d.np, hc) if d.num <= 1 else np.zeros(d.np))
    P = K.scalar_field(doms, lambda d: np.ones(d.np))
    N = K.scalar_field(doms, lambda d: np.ones(d.np))
    sysm = K.OSystem(doms, 0, nd - 1)
    sysm.add_var("H", H)
    sysm.add_var("P", P)
    sysm.add_var("N", N)

    def num(T, x):
        return K.OTerm(T["P"].dom, float(x), None if T["P"].der is None else 0.0)

    def matter(T):
        h = T["H"].exp()
        eps = K.eos_term(h, eos, K.EOS_EPSILON)
        press = K.eos_term(h, eos, K.EOS_PRESSURE)
        delta = (h - eps) - num(T, 1.0)
        Etilde = press * h - press * delta
        Stilde = (num(T, 3.0) * press) * delta
        return delta, Etilde, Stilde

    def lapD(t):
        # D^i D_i X: sum over i of d_i d_i X, in the order 1, 2, 3
        d2 = [t.partial(i).partial(i) for i in (1, 2, 3)]
        return K.OTerm(t.dom, (d2[0].val + d2[1].val) + d2[2].val,
                       None if t.der is None else (d2[0].der + d2[1].der) + d2[2].der)

    qpig2 = lambda T: num(T, NS_QPIG) / num(T, 2.0)

    def eqP(T, b):
        if T["P"].dom > 1:
            return lapD(T["P"])
        delta, Et, _ = matter(T)
        return delta * lapD(T["P"]) + (qpig2(T) * T["P"] ** 5) * Et

    def eqNP(T, b):
        NP = T["P"] * T["N"]
        if T["P"].dom > 1:
            return lapD(NP)
        delta, Et, St = matter(T)
        return delta * lapD(NP) - ((qpig2(T) * T["N"]) * T["P"] ** 5) * (Et + num(T, 2.0) * St)

    for d in range(2, nd):
        sysm.add_eq_full(d, lambda T, b: T["H"])
    for eq, rac in ((eqNP, "N"), (eqP, "P")):
        for d in range(nd - 1):
            sysm.add_eq_inside(d, eq)
            sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b, rac=rac: T[rac])
            sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b, rac=rac: T[rac].dn(b))
        sysm.add_eq_inside(nd - 1, eq)
    sysm.add_eq_bc(nd - 1, K.OUTER_BC, lambda T, b: T["N"] - 1.0)
    sysm.add_eq_bc(nd - 1, K.OUTER_BC, lambda T, b: T["P"] - 1.0)
    sysm.add_eq_first_integral(0, 1, lambda T, b: T["H"] + T["N"].log(),
                               lambda T, b: T["H"] - num(T, hc))
    return doms, sysm, (H, P, N), eos


# The vector star in Kadath's index notation (the product parses these).
STAR_VECTOR_EQUATIONS = {
    "P": "Lap(P) + 2*pi*E/P = 0",
    "NP": "Lap(NP) - 2*pi*NP*E2S/P^2 = 0",
    "bet": "D_j D^j bet^i + D^i D_j bet^j / 3 = 0",
}


def _anti(d):
    b = d.std_base()
    nc1, nc2 = d.nc[1], d.nc[2]
    for k in range(nc2):
        m = k // 2
        b.t[k] = S_COS_ODD if m % 2 == 0 else S_SIN_EVEN
        for j in range(nc1):
            if d.type == K.NUCLEUS:
                b.r[j, k] = S_CHEB_ODD if m % 2 == 0 else S_CHEB_EVEN
    return b


from .spectral import CHEB_EVEN as S_CHEB_EVEN, CHEB_ODD as S_CHEB_ODD, COS_ODD as S_COS_ODD, \
    SIN_EVEN as S_SIN_EVEN  # noqa: E402

# Kadath-syntax strings of the star system (the product parses these).
STAR_EQUATIONS = {
    "P": "Lap(P) + 2*pi*E/P = 0",
    "NP": "Lap(NP) - 2*pi*NP*E2S/P^2 = 0",
    "bx": "Lap(bx) + partial_x(partial_x(bx) + partial_y(by) + partial_z(bz))/3 = 0",
    "by": "Lap(by) + partial_y(partial_x(bx) + partial_y(by) + partial_z(bz))/3 = 0",
    "bz": "Lap(bz) + partial_z(partial_x(bx) + partial_y(by) + partial_z(bz))/3 = 0",
}

# The same systems as strings, for the product's parser (Kadath syntax).
TOY_EQUATIONS = {
    "inside": "Lap(psi) + 2*pi*rho*psi^5 = 0",
    "matching": ["psi", "dn(psi)"],
    "outer": "psi = 1",
}


def eigen_nucleus(res=(11, 5, 4), normalise="val", lam0=9.0):
    """Lap(u) + lam u = 0 in a nucleus of radius 1, u = 0 on its surface,
    with the eigenvalue lam a double unknown and one normalisation: u = 1 at
    the origin (add_eq_ori, "val") or integvolume(u) = 4/pi over the nucleus
    (add_eq_int_volume, "integral").  Known answer: u = sin(pi r)/(pi r),
    lam = pi^2.  Initial guess u = 1 - 0.9 r^2 in the nucleus, lam = lam0."""
    doms = K.space_spheric(res, [1.0, 2.0])
    u = K.scalar_field(doms, lambda d: (1 - 0.9 * d.radius() ** 2) if d.type == K.NUCLEUS else np.zeros(d.np))
    sysm = K.OSystem(doms, 0, 0)
    sysm.add_var("u", u)
    sysm.add_var_double("lam", lam0)
    sysm.add_eq_inside(0, lambda T, b: T["u"].lap() + T["lam"] * T["u"])
    sysm.add_eq_bc(0, K.OUTER_BC, lambda T, b: T["u"])
    if normalise == "val":
        sysm.add_eq_val(0, lambda T: T["u"] - 1.0, (0, 0, 0))
    else:
        sysm.add_eq_int_volume(0, 0, lambda T: T["u"], lambda T: K.OTerm(0, 4.0 / math.pi, 0.0))
    return doms, sysm, u


def mass_at_infinity(res=(11, 5, 4), m0=0.5, redundant=False):
    """Lap(P) = 0 in two shells and the compactified domain (bounds 1, 2, 4),
    P = 2 at r = 1, P = 1 at infinity, and a double unknown M fixed by the
    surface integral at infinity integ(dn(P)) + 4 pi M = 0.  Known answer:
    P = 1 + 1/r, M = 1.  Initial guess P = 1, M = m0."""
    doms = K.space_spheric(res, [1.0, 2.0, 4.0])
    P = K.scalar_field(doms, lambda d: np.ones(d.np))
    sysm = K.OSystem(doms, 1, 3)
    sysm.add_var("P", P)
    sysm.add_var_double("M", m0)
    for d in range(1, 4):
        sysm.add_eq_inside(d, lambda T, b: T["P"].lap())
    sysm.add_eq_bc(1, K.INNER_BC, lambda T, b: T["P"] - 2.0)
    for d in range(1, 3):
        sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b: T["P"])
        sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b: T["P"].dn(b))
    sysm.add_eq_bc(3, K.OUTER_BC, lambda T, b: T["P"] - 1.0)
    if redundant:  # the outer condition once more: an overdetermined, consistent system
        sysm.add_eq_bc(3, K.OUTER_BC, lambda T, b: T["P"] - 1.0)
    sysm.add_eq_int([(3, K.OUTER_BC, lambda T, b: T["P"].dn(b).integ(b) + 4 * math.pi * T["M"])])
    return doms, sysm, P
