"""Index notation with the flat metric on the GPU: Cartesian vector unknowns,
D_i / D^i / partial_i, contraction of repeated indices, tensor definitions
and the metric tensor (Metric_flat, src/Metric/metric_flat.cpp:150,
give_ope.cpp:385-520, name_tools.cpp:187).

* the vector star against the oracle's vector star;
* the vector star against the component star run through the same library
  (identical operations: the numbers agree to the last bit up to the order
  of rows and columns);
* Newton on the vector star converges to the component star's solution;
* identities between index expressions and the errors the parser raises."""
import math

import numpy as np
import pytest

from oracle import configs

pytestmark = pytest.mark.gpu

RES = (7, 5, 4)
REL = 1e-12


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def component_star_in_vector_order(res, ctx=None):
    """The component star with its matching equations in the vector form's
    order (per boundary P, dn(P), NP, dn(NP), bx, by, bz, then their dn)."""
    from kadath_frontera_gb300 import workloads as W
    from kadath_frontera_gb300.kadath import CHEB_TYPE, OUTER_BC, Scalar, Space_spheric, System_of_eqs
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), res, W.STAR_BOUNDS, ctx=ctx)
    nd = space.get_nbr_domains()
    P = Scalar(space, 1.0).std_base()
    NP = Scalar(space, 1.0).std_base()
    b = [Scalar(space, 0.0).std_base_cart(c) for c in (1, 2, 3)]
    for f in b:
        for d in range(nd):
            f.set_domain(d, np.zeros(space.domain_info(d)["nbr_points"]))
    E, E2S = Scalar(space), Scalar(space)
    for d in range(nd):
        e, e2s = W.star_matter_values(space.get_radius(d), space.domain_info(d)["type"] == 1)
        E.set_domain(d, e)
        E2S.set_domain(d, e2s)
    E.std_base()
    E2S.std_base()
    syst = System_of_eqs(space, 0, nd - 1)
    names = ["P", "NP", "bx", "by", "bz"]
    for nm, f in zip(names, [P, NP] + b):
        syst.add_var(nm, f)
    syst.add_cst("pi", math.pi)
    syst.add_cst("E", E)
    syst.add_cst("E2S", E2S)
    for d in range(nd):
        for nm in names:
            syst.add_eq_inside(d, W.STAR_EQUATIONS[nm])
    for d in range(nd - 1):
        for nm in ("P", "NP"):
            syst.add_eq_matching(d, OUTER_BC, nm)
            syst.add_eq_matching(d, OUTER_BC, f"dn({nm})")
        for nm in ("bx", "by", "bz"):
            syst.add_eq_matching(d, OUTER_BC, nm)
        for nm in ("bx", "by", "bz"):
            syst.add_eq_matching(d, OUTER_BC, f"dn({nm})")
    syst.add_eq_bc(nd - 1, OUTER_BC, "P = 1")
    syst.add_eq_bc(nd - 1, OUTER_BC, "NP = 1")
    for nm in ("bx", "by", "bz"):
        syst.add_eq_bc(nd - 1, OUTER_BC, f"{nm} = 0")
    return space, syst, [P, NP] + b, (E, E2S)


def vector_columns(nd, ncols_of):
    """Column permutation component form -> vector form: ncols_of(var, dom)
    gives the number of unknowns of (var, dom); vars 0..4 = P, NP, x, y, z."""
    col0, c = {}, 0
    for v in range(5):
        for d in range(nd):
            col0[(v, d)] = c
            c += ncols_of(v, d)
    perm = []
    for v in (0, 1):
        for d in range(nd):
            perm += range(col0[(v, d)], col0[(v, d)] + ncols_of(v, d))
    for d in range(nd):
        for v in (2, 3, 4):
            perm += range(col0[(v, d)], col0[(v, d)] + ncols_of(v, d))
    return np.array(perm)


def oracle_ncols(osys):
    layout, _ = osys.unknown_layout()
    return {(vi, dd): len(p) for vi, dd, _, p in layout}


def test_vector_star_matches_oracle(ctx):
    from kadath_frontera_gb300 import workloads as W
    wl = W.star_vector(RES, ctx=ctx)
    doms, osys, _, _ = configs.star_vector(RES)
    F = wl.syst.sec_member()
    J = wl.syst.jacobian()
    Fo, Jo = osys.jacobian()
    assert F.shape == Fo.shape and J.shape == Jo.shape
    scale = np.abs(Jo).max()
    assert np.abs(F - Fo).max() <= 1e-13 * scale
    assert rel(J, Jo) < REL
    x = np.random.default_rng(3).standard_normal(J.shape[0])
    assert rel(wl.syst.do_JX(x), Jo @ x) < REL


def test_vector_star_equals_component_star(ctx):
    from kadath_frontera_gb300 import workloads as W
    wl = W.star_vector(RES, ctx=ctx)
    _, sc, _, _ = component_star_in_vector_order(RES, ctx=ctx)
    doms, osys, _, _ = configs.star(RES)
    n = oracle_ncols(osys)
    perm = vector_columns(len(doms), lambda v, d: n[(v, d)])
    Fv, Jv = wl.syst.sec_member(), wl.syst.jacobian()
    Fc, Jc = sc.sec_member(), sc.jacobian()
    assert Fv.shape == Fc.shape
    scale = np.abs(Jc).max()
    # the same kernels on the same operands in the same order
    assert np.abs(Fv - Fc).max() <= 1e-15 * scale
    assert np.abs(Jv - Jc[:, perm]).max() <= 1e-15 * scale


def test_vector_star_newton_converges_to_component_solution(ctx):
    from kadath_frontera_gb300 import workloads as W
    res = (9, 5, 4)
    wl = W.star_vector(res, ctx=ctx)
    space, sc, comps, _ = component_star_in_vector_order(res, ctx=ctx)
    nv = W.solve(wl, 1e-10)
    nc = 0
    for it in range(20):
        done, err = sc.do_newton(1e-10)
        if done:
            break
        nc += 1
    assert done and abs(nv - nc) <= 1
    for (_, f), g in zip(wl.unknowns, comps):
        for d in range(space.get_nbr_domains()):
            a, b = f.get_coef(d), g.get_coef(d)
            assert np.abs(a - b).max() <= 1e-10 * max(1.0, np.abs(b).max())


def _toy_with(eq_inside, metric=True, extra=None):
    from kadath_frontera_gb300.kadath import CHEB_TYPE, OUTER_BC, Metric_flat, Scalar, Space_spheric, \
        System_of_eqs, Vector
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), (9, 5, 4), (1.0, 2.0))
    nd = space.get_nbr_domains()
    P = Scalar(space)
    v = Vector(space)
    for d in range(nd):
        x, y, z = (space.get_cart(d, c) for c in (1, 2, 3))
        r2 = x * x + y * y + z * z
        fin = np.isfinite(r2)
        p = np.zeros_like(r2)
        p[fin] = 1.0 + 0.3 * x[fin] * y[fin] / (1 + r2[fin] ** 2)
        P.set_domain(d, p)
        for c, comp in enumerate((x, y, z)):
            w = np.zeros_like(r2)
            w[fin] = comp[fin] / (1 + r2[fin] ** 2) * (1 + 0.1 * c)
            v(c + 1).set_domain(d, w)
    P.std_base()
    v.std_base()
    syst = System_of_eqs(space, 0, nd - 1)
    if metric:
        Metric_flat(space).set_system(syst, "g")
    syst.add_var("P", P)
    syst.add_var("v", v)
    if extra:
        extra(syst)
    for d in range(nd):
        for eq in eq_inside:
            syst.add_eq_inside(d, eq)
    for d in range(nd - 1):
        syst.add_eq_matching(d, OUTER_BC, "P")
        syst.add_eq_matching(d, OUTER_BC, "dn(P)")
        syst.add_eq_matching(d, OUTER_BC, "v^i")
        syst.add_eq_matching(d, OUTER_BC, "dn(v^i)")
    syst.add_eq_bc(nd - 1, OUTER_BC, "P = 1")
    syst.add_eq_bc(nd - 1, OUTER_BC, "v^i = 0")
    return syst


def _FJ(eqs, **kw):
    s = _toy_with(eqs, **kw)
    return s.sec_member(), s.jacobian()


def test_contracted_second_derivative_is_the_laplacian(ctx):
    """D_i D^i P and partial_i partial_i P are Lap(P) with the same sum, term
    by term: identical numbers."""
    vec = "Lap(v^i) = 0"
    F0, J0 = _FJ(["Lap(P) = 0", vec])
    for form in ("D_i D^i P = 0", "D^i D_i P = 0", "partial_i partial_i P = 0"):
        F, J = _FJ([form, vec])
        assert np.array_equal(F, F0) and np.array_equal(J, J0), form
    F, J = _FJ(["Lap(P) = 0", "D_j D^j v^i = 0"])
    assert np.array_equal(F, F0) and np.array_equal(J, J0)


def test_index_identities(ctx):
    """Tensor definitions, positional renaming, traces, the metric and sums
    of differently ordered indices."""
    base = ["Lap(P) = 0", "Lap(v^i) + D^i D_j v^j = 0"]
    F0, J0 = _FJ(base)
    tol = 1e-13 * np.abs(J0).max()

    def defs(s):
        s.add_def("A_ij = D_i v_j + D_j v_i")
        s.add_def("B_ij = D_i v_j")
        s.add_def("C_ij = D_j v_i")

    # a definition is its expression: D^j B_ij is D^j D_i v_j, operation
    # for operation; C_ij is stored in its left side's index order, so
    # C_ji (renamed by position) is B_ij again
    Fi, Ji = _FJ(["Lap(P) = 0", "D^j D_i v_j = 0"])
    for form in ("D^j B_ij = 0", "D^j C_ji = 0"):
        F, J = _FJ(["Lap(P) = 0", form], extra=defs)
        assert np.array_equal(F, Fi) and np.array_equal(J, Ji), form
    # a sum of tensors with their indices in another order is aligned by name
    F1, J1 = _FJ(["Lap(P) = 0", "D^j A_ij = 0"], extra=defs)
    F2, J2 = _FJ(["Lap(P) = 0", "D^j (D_i v_j + D_j v_i) = 0"])
    assert np.array_equal(F1, F2) and np.array_equal(J1, J2)
    F3, J3 = _FJ(["Lap(P) = 0", "D^j (B_ij + C_ij) = 0"], extra=defs)
    assert np.array_equal(F1, F3) and np.array_equal(J1, J3)
    # metric contraction: g_ij v^j is v_i; trace A_ii is 2 div v
    Fm, Jm = _FJ(["Lap(P) = 0", "Lap(g_ij * v^j) + D^i D_j v^j = 0"])
    assert np.abs(Fm - F0).max() <= tol and np.abs(Jm - J0).max() <= tol
    F1, J1 = _FJ(["Lap(P) + A_ii = 0", "Lap(v^i) + D^i D_j v^j = 0"], extra=defs)
    F2, J2 = _FJ(["Lap(P) + 2*D_j v^j = 0", "Lap(v^i) + D^i D_j v^j = 0"])
    assert np.abs(F1 - F2).max() <= tol and np.abs(J1 - J2).max() <= tol
    # scal() of a vector written without indices is the contraction v_i v^i
    F1, J1 = _FJ(["Lap(P) + scal(v, v) = 0", base[1]])
    F2, J2 = _FJ(["Lap(P) + v_i * v^i = 0", base[1]])
    assert np.array_equal(F1, F2) and np.array_equal(J1, J2)


def test_index_errors(ctx):
    from kadath_frontera_gb300.kadath import KadathError
    with pytest.raises(KadathError):
        _toy_with(["D_i D^i P = 0", "Lap(v^i) = 0"], metric=False)
    with pytest.raises(KadathError):
        _FJ(["Lap(P) = 0", "Lap(v^i) + D^j P = 0"])
    with pytest.raises(KadathError):
        _FJ(["Lap(P) = 0", "Lap(v^ij) = 0"])
