"""Pins the spectral oracle with known answers from the reference's own
evaluation routine (src/Ope_1d/summation_1d.cpp) on the collocation grids of
src/Domain/Spheric/domain_{shell,nucleus,compact}.cpp (do_coloc)."""
import math

import numpy as np
import pytest

from oracle import spectral as S


def grid(base, n):
    """Collocation points each basis is used with."""
    if base == S.CHEB:
        return [-math.cos(math.pi * i / (n - 1)) for i in range(n)]
    if base in (S.CHEB_EVEN, S.CHEB_ODD):
        return [math.sin(math.pi / 2. * i / (n - 1)) for i in range(n)]
    if base in (S.COS_EVEN, S.COS_ODD, S.SIN_EVEN, S.SIN_ODD):
        return [math.pi / 2. * j / (n - 1) for j in range(n)]
    if base in (S.COS, S.SIN):
        return [math.pi * j / (n - 1) for j in range(n)]
    raise ValueError(base)


def active_slots(base, n):
    """Coefficient slots that carry information on the grid."""
    if base in (S.CHEB, S.CHEB_EVEN, S.COS, S.COS_EVEN):
        return list(range(n))
    if base in (S.CHEB_ODD, S.COS_ODD):
        return list(range(n - 1))
    if base == S.SIN_ODD:
        return list(range(n - 1))
    if base in (S.SIN_EVEN, S.SIN):
        return list(range(1, n - 1))
    raise ValueError(base)


@pytest.mark.parametrize("base", [S.CHEB, S.CHEB_EVEN, S.CHEB_ODD, S.COS, S.SIN, S.COS_EVEN, S.COS_ODD,
                                  S.SIN_EVEN, S.SIN_ODD])
@pytest.mark.parametrize("n", [5, 7, 9, 11, 13, 17])
def test_basis_functions_give_unit_coefficients(base, n):
    pts = grid(base, n)
    for k in active_slots(base, n):
        e = np.zeros(n)
        e[k] = 1.0
        vals = np.array([S.summation_1d(base, x, e) for x in pts])
        cf = S.COEF_1D[base](vals.copy())
        assert np.allclose(cf, e, atol=1e-12), (S.BASE_NAMES[base], n, k, cf)
        back = S.COEF_I_1D[base](e.copy())
        assert np.allclose(back, vals, atol=1e-12), (S.BASE_NAMES[base], n, k)


@pytest.mark.parametrize("nphi", [4, 6, 8, 12])
def test_cossin_known_answers(nphi):
    nbr = nphi + 2
    pts = [2 * math.pi * k / nphi for k in range(nphi)]
    for slot in range(nbr):
        if slot == 1 or slot == nbr - 1:
            continue  # sin(0) and sin(nphi/2 phi) vanish on the grid
        e = np.zeros(nbr)
        e[slot] = 1.0
        vals = np.array([S.summation_1d(S.COSSIN, p, e) for p in pts])
        t = np.zeros(nbr)
        t[:nphi] = vals
        cf = S.COEF_1D[S.COSSIN](t)
        assert np.allclose(cf, e, atol=1e-12), (nphi, slot, cf)
        back = S.COEF_I_1D[S.COSSIN](e.copy())[:nphi]
        assert np.allclose(back, vals, atol=1e-12)


def test_derivative_known_answer_cheb():
    # d/dx of T_k, evaluated with summation_1d on the output basis
    n = 9
    xs = np.linspace(-0.9, 0.9, 7)
    for k in range(n):
        e = np.zeros(n)
        e[k] = 1.0
        ob, d = S.der_1d(S.CHEB, e)
        assert ob == S.CHEB
        for x in xs:
            exact = k * math.sin(k * math.acos(x)) / math.sqrt(1 - x * x)
            assert abs(S.summation_1d(S.CHEB, x, d) - exact) < 1e-11


def test_mult_div_sin_roundtrip():
    # div_sin(mult_sin(f)) == f for COS_EVEN lines whose top mode is empty
    rng = np.random.default_rng(1)
    for n in (5, 7, 9):
        f = rng.standard_normal(n)
        f[-1] = 0.0
        b1, g = S.mult_sin_1d(S.COS_EVEN, f)
        b2, h = S.div_sin_1d(b1, g)
        assert b1 == S.SIN_ODD and b2 == S.COS_EVEN
        assert np.allclose(h, f, atol=1e-12)


def test_3d_roundtrip_shell_std_base():
    n0, n1, n2 = 9, 5, 4
    nc = (n0, n1, n2 + 2)
    base_t = [S.COS_EVEN if ((k // 2) % 2 == 0) else S.SIN_ODD for k in range(nc[2])]
    base_r = [[S.CHEB] * nc[2] for _ in range(nc[1])]
    rng = np.random.default_rng(0)
    # A smooth symmetric field: values from random coefficients.
    cf = rng.standard_normal(nc)
    cf[:, :, 1] = 0
    cf[:, :, -1] = 0
    for k in range(nc[2]):
        if base_t[k] == S.SIN_ODD:
            cf[:, -1, k] = 0
    vals = S.coef_i_3d(cf, base_r, base_t, S.COSSIN, (n0, n1, n2))
    back = S.coef_3d(vals, base_r, base_t, S.COSSIN, nc)
    assert np.allclose(back, cf, atol=1e-11)
