"""The oracle's Cartesian vector unknowns and vector equations (CPU).

The vector form of the star (one unknown bet, the shift equation in index
notation) must give exactly the component form's residual and Jacobian once
the component form's equations and unknowns are put in the vector form's
order: the rows of a vector equation come component by component, and the
unknowns of a vector domain by domain with x, y, z inside each domain
(xx_to_vars, src/System_of_eqs/system_of_eqs.cpp:597)."""
import numpy as np

from oracle import configs, kadath as K

RES = (7, 5, 4)


def reorder_component_form(sysm, nd):
    """The component star's equations in the vector form's order: per
    boundary P, dn(P), NP, dn(NP), then bx, by, bz, then their dn."""
    inside = [e for e in sysm.eqs if e[0] == "inside"]
    bc = [e for e in sysm.eqs if e[0] == "bc"]
    match = [e for e in sysm.eqs if e[0] == "matching"]
    new = []
    for d in range(nd - 1):
        m = [e for e in match if e[1] == d]
        new += m[:4] + [m[4], m[6], m[8], m[5], m[7], m[9]]
    sysm.eqs = inside + new + bc


def column_permutation(s_comp, s_vec):
    L1, _ = s_comp.unknown_layout()
    L2, _ = s_vec.unknown_layout()
    cols1 = {(vi, dd): (c, len(p)) for vi, dd, c, p in L1}
    perm = []
    for vi, dd, c, p in L2:
        c1, n = cols1[(vi, dd)]
        perm += list(range(c1, c1 + n))
    return np.array(perm)


def test_vector_unknown_layout_is_domain_major():
    doms, s2, *_ = configs.star_vector(RES)
    layout, N = s2.unknown_layout()
    nd = len(doms)
    # P over every domain, NP over every domain, then bet: (dom, x y z)
    order = [(vi, dd) for vi, dd, _, _ in layout]
    expect = [(0, d) for d in range(nd)] + [(1, d) for d in range(nd)]
    expect += [(2 + c, d) for d in range(nd) for c in range(3)]
    assert order == expect
    cols = [c for _, _, c, _ in layout]
    assert cols == sorted(cols) and N == layout[-1][2] + len(layout[-1][3])


def test_vector_form_equals_component_form():
    doms, s1, *_ = configs.star(RES)
    _, s2, *_ = configs.star_vector(RES)
    reorder_component_form(s1, len(doms))
    F1, J1 = s1.jacobian()
    F2, J2 = s2.jacobian()
    perm = column_permutation(s1, s2)
    assert F1.shape == F2.shape
    # same operations in the same order: identical numbers
    assert np.array_equal(F1, F2)
    assert np.array_equal(J1[:, perm], J2)


def test_vector_form_newton_step_equals_component_form():
    doms, s1, f1, _ = configs.star(RES)
    _, s2, f2, _ = configs.star_vector(RES)
    reorder_component_form(s1, len(doms))
    s1.newton_step(1e-12)
    s2.newton_step(1e-12)
    for a, b in zip(f1, f2):
        for d in range(len(doms)):
            va, vb = a[d], b[d]
            va.coef_i()
            vb.coef_i()
            assert np.abs(va.c - vb.c).max() <= 1e-12 * max(1.0, np.abs(va.c).max())
