"""Systems used by the benchmark and the smoke check, written with the same
public API and equation strings a Kadath user would write.

* ``toy``  -- nucleus r < 1, shell 1 < r < 2, compactified r > 2, (13, 7, 4)
  points: Lap(psi) = -2 pi rho psi^5 with rho = 0.05 exp(-r^2/0.25),
  psi = 1 at infinity, continuity of psi and dn(psi); initial guess 1.
* ``star`` -- XCTS-shaped static star at the isolated-star configuration's
  size: six domains (nucleus of radius R = 8 holding frozen Gamma = 2,
  K = 100 matter with rho_c = 1.28e-3, four shells, compactified exterior),
  (13, 9, 4) points, five unknowns: conformal factor P, lapse times P (NP)
  and the Cartesian shift components bx, by, bz with the flat vector
  Laplacian Lap(b^i) + d^i(div b)/3.  N is about 13k.
"""
from __future__ import annotations

import math

import numpy as np

from .kadath import CHEB_TYPE, OUTER_BC, Scalar, Space_spheric, System_of_eqs

STAR_R = 8.0
STAR_RHOC = 1.28e-3
STAR_K = 100.0
STAR_BOUNDS = (STAR_R, 12.0, 16.0, 24.0, 32.0)

STAR_EQUATIONS = {
    "P": "Lap(P) + 2*pi*E/P = 0",
    "NP": "Lap(NP) - 2*pi*NP*E2S/P^2 = 0",
    "bx": "Lap(bx) + partial_x(partial_x(bx) + partial_y(by) + partial_z(bz))/3 = 0",
    "by": "Lap(by) + partial_y(partial_x(bx) + partial_y(by) + partial_z(bz))/3 = 0",
    "bz": "Lap(bz) + partial_z(partial_x(bx) + partial_y(by) + partial_z(bz))/3 = 0",
}


def toy_rho_values(r):
    v = np.zeros_like(r)
    fin = np.isfinite(r)
    v[fin] = 0.05 * np.exp(-r[fin] ** 2 / 0.25)
    return v


def star_matter_values(r, nucleus: bool, rho_c=STAR_RHOC):
    rho = np.zeros_like(r)
    if nucleus:
        x = np.pi * r / STAR_R
        safe = np.where(x > 0, x, 1.0)
        rho = rho_c * np.where(x > 0, np.sin(x) / safe, 1.0)
    E = rho * (1 + STAR_K * rho)
    S = 3 * STAR_K * rho * rho
    return E, E + 2 * S


class Workload:
    def __init__(self, name, space, syst, unknowns, constants):
        self.name = name
        self.space = space
        self.syst = syst
        self.unknowns = unknowns        # list of (name, Scalar)
        self.constants = constants
        # device copies of the initial guess, for restarting a step
        self.initial = []
        for nm, f in unknowns:
            g = Scalar(space)
            g.copy_from(f)
            self.initial.append(g)
        # host copies of the initial guess at the collocation points (e2e input)
        nd = space.get_nbr_domains()
        self.initial_host = [[f.get_domain(d).copy() for d in range(nd)] for _, f in unknowns]

    def restore(self):
        for (nm, f), g in zip(self.unknowns, self.initial):
            f.copy_from(g)

    def upload_initial(self, host=None):
        """Host -> device copy of every unknown at every domain."""
        host = host or self.initial_host
        for (nm, f), per_dom in zip(self.unknowns, host):
            for d, v in enumerate(per_dom):
                f.set_domain(d, v)

    def download(self):
        nd = self.space.get_nbr_domains()
        return [[f.get_coef(d) for d in range(nd)] for _, f in self.unknowns]

    def bytes_in(self):
        return sum(v.nbytes for per in self.initial_host for v in per)


def toy(res=(13, 7, 4), bounds=(1.0, 2.0), ctx=None, rho_values=None) -> Workload:
    """rho_values: optional per-domain arrays of rho at the collocation points."""
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), res, bounds, ctx=ctx)
    nd = space.get_nbr_domains()
    psi = Scalar(space, 1.0).std_base()
    rho = Scalar(space)
    for d in range(nd):
        rho.set_domain(d, toy_rho_values(space.get_radius(d)) if rho_values is None else rho_values[d])
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
    return Workload("toy", space, syst, [("psi", psi)], [rho])


def star(res=(13, 9, 4), bounds=STAR_BOUNDS, ctx=None, rho_c=STAR_RHOC, matter_domains=1, matter=None) -> Workload:
    """matter: optional (E, E2S), each a list of per-domain value arrays at the
    collocation points, used instead of the Lane-Emden profile."""
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), res, bounds, ctx=ctx)
    nd = space.get_nbr_domains()
    P = Scalar(space, 1.0).std_base()
    NP = Scalar(space, 1.0).std_base()
    bx = Scalar(space, 0.0).std_base_cart(1)
    by = Scalar(space, 0.0).std_base_cart(2)
    bz = Scalar(space, 0.0).std_base_cart(3)
    # explicit zeros (not the zero flag) so that every operator carries its
    # basis through the first residual evaluation
    for f in (bx, by, bz):
        for d in range(nd):
            f.set_domain(d, np.zeros(space.domain_info(d)["nbr_points"]))
    E = Scalar(space)
    E2S = Scalar(space)
    for d in range(nd):
        if matter is None:
            e, e2s = star_matter_values(space.get_radius(d), d < matter_domains, rho_c)
        else:
            e, e2s = matter[0][d], matter[1][d]
        E.set_domain(d, e)
        E2S.set_domain(d, e2s)
    E.std_base()
    E2S.std_base()
    syst = System_of_eqs(space, 0, nd - 1)
    unknowns = [("P", P), ("NP", NP), ("bx", bx), ("by", by), ("bz", bz)]
    for nm, f in unknowns:
        syst.add_var(nm, f)
    syst.add_cst("pi", math.pi)
    syst.add_cst("E", E)
    syst.add_cst("E2S", E2S)
    for d in range(nd):
        for nm, _ in unknowns:
            syst.add_eq_inside(d, STAR_EQUATIONS[nm])
    for d in range(nd - 1):
        for nm, _ in unknowns:
            syst.add_eq_matching(d, OUTER_BC, nm)
            syst.add_eq_matching(d, OUTER_BC, f"dn({nm})")
    syst.add_eq_bc(nd - 1, OUTER_BC, "P = 1")
    syst.add_eq_bc(nd - 1, OUTER_BC, "NP = 1")
    for nm in ("bx", "by", "bz"):
        syst.add_eq_bc(nd - 1, OUTER_BC, f"{nm} = 0")
    return Workload("star", space, syst, unknowns, [E, E2S])


# The binary-BH configuration's size on a spherical space: twelve domains
# (nucleus, ten shells, compactified exterior) at (11, 9, 8), the star's
# five unknowns, matter in the four domains inside r = 8: N = 40,081.
LARGE_RES = (11, 9, 8)
LARGE_BOUNDS = (2.0, 4.0, 6.0, 8.0, 10.0, 12.0, 16.0, 20.0, 24.0, 28.0, 32.0)


def star_large(ctx=None) -> Workload:
    return star(LARGE_RES, LARGE_BOUNDS, ctx=ctx, matter_domains=4)


STAR_VECTOR_EQUATIONS = {
    "P": "Lap(P) + 2*pi*E/P = 0",
    "NP": "Lap(NP) - 2*pi*NP*E2S/P^2 = 0",
    "bet": "D_j D^j bet^i + D^i D_j bet^j / 3 = 0",
}


def star_vector(res=(13, 9, 4), bounds=STAR_BOUNDS, ctx=None, rho_c=STAR_RHOC, matter=None) -> Workload:
    """The star with the shift as one Cartesian vector unknown ``bet`` and its
    equation in index notation with the flat metric: the form Kadath codes
    write.  Same fields and matter as ``star``; the unknowns of bet come
    domain by domain, x, y, z inside each domain."""
    from .kadath import Metric_flat, Vector
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), res, bounds, ctx=ctx)
    nd = space.get_nbr_domains()
    P = Scalar(space, 1.0).std_base()
    NP = Scalar(space, 1.0).std_base()
    bet = Vector(space).std_base()
    for c in (1, 2, 3):
        for d in range(nd):
            bet(c).set_domain(d, np.zeros(space.domain_info(d)["nbr_points"]))
    E = Scalar(space)
    E2S = Scalar(space)
    for d in range(nd):
        if matter is None:
            e, e2s = star_matter_values(space.get_radius(d), space.domain_info(d)["type"] == 1, rho_c)
        else:
            e, e2s = matter[0][d], matter[1][d]
        E.set_domain(d, e)
        E2S.set_domain(d, e2s)
    E.std_base()
    E2S.std_base()
    syst = System_of_eqs(space, 0, nd - 1)
    Metric_flat(space).set_system(syst, "f")
    syst.add_var("P", P)
    syst.add_var("NP", NP)
    syst.add_var("bet", bet)
    syst.add_cst("pi", math.pi)
    syst.add_cst("E", E)
    syst.add_cst("E2S", E2S)
    for d in range(nd):
        for nm in ("P", "NP", "bet"):
            syst.add_eq_inside(d, STAR_VECTOR_EQUATIONS[nm])
    for d in range(nd - 1):
        for nm in ("P", "NP", "bet^i"):
            syst.add_eq_matching(d, OUTER_BC, nm)
            syst.add_eq_matching(d, OUTER_BC, f"dn({nm})")
    syst.add_eq_bc(nd - 1, OUTER_BC, "P = 1")
    syst.add_eq_bc(nd - 1, OUTER_BC, "NP = 1")
    syst.add_eq_bc(nd - 1, OUTER_BC, "bet^i = 0")
    unknowns = [("P", P), ("NP", NP), ("bet_x", bet(1)), ("bet_y", bet(2)), ("bet_z", bet(3))]
    return Workload("star_vector", space, syst, unknowns, [E, E2S])


NS_BOUNDS = (3.5, 7.0, 12.0, 18.0, 24.0)
NS_RHOC = 1.28e-3
NS_DEFS_ALL = ["NP = P*N", "h = exp(H)", "rho = rho(h)", "eps = eps(h)", "press = press(h)",
               "delta = h - eps - 1."]
NS_DEFS_MATTER = ["Etilde = press * h - press * delta", "Stilde = 3 * press * delta",
                  "eqP = delta * D^i D_i P + 4piG / 2. * P^5 * Etilde",
                  "eqNP = delta * D^i D_i NP - 4piG / 2. * N * P^5 * (Etilde + 2. * Stilde)",
                  "firstint = H + log(N)"]
NS_DEFS_VACUUM = ["eqP = D^i D_i P", "eqNP = D^i D_i NP"]


def ns_tov(res=(13, 9, 4), bounds=NS_BOUNDS, ctx=None, rho_c=NS_RHOC) -> Workload:
    """Static TOV star with the log-enthalpy H as unknown, in the shape of
    the non-rotating stage of Kadath's NS solver: the Gamma = 2, K = 100
    polytrope through the EOS operators, lapse N and conformal factor P,
    matter in domains 0 and 1 whose outer radius is fixed (7), H = 0 on every
    coefficient outside (add_eq_full), the first integral H + log(N) =
    const in the matter with H = Hc at the centre (add_eq_first_integral).
    The equations are the solver's strings.  Initial guess H = Hc in the
    matter, P = N = 1."""
    from .kadath import KD_EOS_DENSITY, KD_EOS_DHDRHO, KD_EOS_EPSILON, KD_EOS_PRESSURE, Metric_flat
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), res, bounds, ctx=ctx)
    nd = space.get_nbr_domains()
    hc = math.log(1.0 + 2.0 * 100.0 * rho_c)
    H = Scalar(space)
    for d in range(nd):
        H.set_domain(d, np.full(space.domain_info(d)["nbr_points"], hc if d <= 1 else 0.0))
    H.std_base()
    P = Scalar(space, 1.0).std_base()
    N = Scalar(space, 1.0).std_base()
    syst = System_of_eqs(space, 0, nd - 1)
    syst.add_var("H", H)
    Metric_flat(space).set_system(syst, "f")
    syst.add_cst("4piG", 4 * math.pi)
    syst.add_var("P", P)
    syst.add_var("N", N)
    syst.add_cst("Hc", hc)
    for name, var in (("eps", KD_EOS_EPSILON), ("press", KD_EOS_PRESSURE), ("rho", KD_EOS_DENSITY),
                      ("dHdlnrho", KD_EOS_DHDRHO)):
        syst.add_ope_eos(name, var)
    for df in NS_DEFS_ALL:
        syst.add_def(df)
    for d in range(nd):
        if d <= 1:
            for df in NS_DEFS_MATTER:
                syst.add_def(d, df)
        else:
            syst.add_eq_full(d, "H = 0")
            for df in NS_DEFS_VACUUM:
                syst.add_def(d, df)
    space.add_eq(syst, "eqNP= 0", "N", "dn(N)")
    space.add_eq(syst, "eqP = 0", "P", "dn(P)")
    syst.add_eq_bc(nd - 1, OUTER_BC, "N=1")
    syst.add_eq_bc(nd - 1, OUTER_BC, "P=1")
    syst.add_eq_first_integral(0, 1, "firstint", "H - Hc")
    return Workload("ns_tov", space, syst, [("H", H), ("P", P), ("N", N)], [])


WORKLOADS = {"toy": toy, "star": star, "star_vector": star_vector, "ns_tov": ns_tov, "star_large": star_large}


def solve(wl: Workload, precision=1e-10, lu_mode=None, max_steps=20) -> int:
    """Newton steps from the current fields until |F| < precision; returns the
    number of updates made."""
    err = math.inf
    for it in range(max_steps):
        done, err = wl.syst.do_newton(precision, lu_mode=lu_mode)
        if done:
            return it
    raise RuntimeError(f"{wl.name}: no convergence in {max_steps} steps (|F| = {err:.3e})")


def batch_ntheta(nr):
    """ntheta of a batch instance: nr // 2 + 1, raised to the next odd number.
    With an even number of theta points the nucleus's Galerkin/tau system is
    singular (the oracle's Jacobian of the toy problem has condition number
    ~1e22 at (9, 6, 4) against ~1e9 at (9, 5, 4); shells alone are regular),
    and Kadath's own codes use odd theta resolutions."""
    nt = nr // 2 + 1
    return nt if nt % 2 == 1 else nt + 1


def star_batch_configs(n, seed=0):
    """Independent isolated stars with central densities uniform in
    [8e-4, 2e-3] and nr in {9, 11, 13, 15, 17} per instance
    (ntheta = batch_ntheta(nr), nphi = 4), from a fixed seed."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nr = int(rng.choice([9, 11, 13, 15, 17]))
        out.append({"res": (nr, batch_ntheta(nr), 4), "rho_c": float(rng.uniform(8e-4, 2e-3))})
    return out


def solve_batch(configs, threads, precision=1e-10, lu_mode=None, device=0, keep=True, sm_share=None):
    """Builds and solves every configuration, each instance on its own
    context (its own CUDA streams and workspaces) from a pool of `threads`
    host threads, so that instances overlap on the GPU.  Returns the
    converged workloads in configuration order, or with keep=False only
    their numbers of Newton updates (each instance's device memory is then
    released as soon as it has converged).  With several threads each
    context's grid-wide solver kernels get sm_share SMs (default: the
    device's SMs divided by the number of threads, at least 16), so that the
    instances' factorisations and sweeps run side by side."""
    from concurrent.futures import ThreadPoolExecutor

    if sm_share is None and threads > 1:
        import torch
        nsm = torch.cuda.get_device_properties(device).multi_processor_count
        sm_share = max(16, nsm // threads)

    from ._lib import Context

    def one(cfg):
        ctx = Context(device)
        if threads > 1 and sm_share:
            ctx.set_sm_budget(sm_share)
        wl = star(res=cfg["res"], rho_c=cfg["rho_c"], ctx=ctx)
        updates = solve(wl, precision, lu_mode)
        return wl if keep else updates

    if threads <= 1:
        return [one(c) for c in configs]
    with ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(one, configs))


def main(argv=None) -> int:
    """Runs Newton steps of a workload from its initial guess: the command a
    profiler wraps (`python -m kadath_frontera_gb300.workloads --steps 1`).
    With --solves K it runs K complete solves instead (initial guess to
    |F| <= precision, as the benchmark times them, residual graph-captured),
    each inside an NVTX range "solve<i>", so that a profiler can select one
    (`ncu --nvtx --nvtx-include "solve1/" ...`)."""
    import argparse

    from . import kadath as KD
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--workload", default="star", choices=sorted(WORKLOADS))
    ap.add_argument("--mode", default="mixed", choices=["mixed", "fp64", "fp32"])
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--solves", type=int, default=0)
    ap.add_argument("--precision", type=float, default=1e-10)
    args = ap.parse_args(argv)
    mode = {"mixed": KD.KD_LU_TF32_IR, "fp64": KD.KD_LU_FP64, "fp32": KD.KD_LU_FP32_IR}[args.mode]
    wl = WORKLOADS[args.workload]()
    if args.solves > 0:
        import torch
        wl.syst.graph_capture = True
        for i in range(args.solves):
            wl.restore()
            wl.syst.cache_tangents(False)
            wl.syst.cache_tangents(True)
            wl.syst.reset_pivot_order()
            torch.cuda.nvtx.range_push(f"solve{i}")
            steps = []
            for _ in range(20):
                done, err = wl.syst.do_newton(args.precision, lu_mode=mode)
                steps.append(wl.syst.last_report)
                if done:
                    break
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_pop()
            print(f"solve {i}: {len(steps) - 1} updates, |F| = {err:.3e}, factor "
                  + ", ".join(f"{r['t_factor_ms']:.1f}" for r in steps[:-1]) + " ms", flush=True)
        return 0
    for i in range(args.warmup + args.steps):
        wl.restore()
        done, err = wl.syst.do_newton(args.precision, lu_mode=mode)
        rep = wl.syst.last_report
        print(f"step {i}: |F| = {err:.3e}, factor {rep['t_factor_ms']:.1f} ms, assembly {rep['t_assembly_ms']:.1f} ms",
              flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
