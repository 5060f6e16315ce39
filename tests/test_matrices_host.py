"""The C++ restatement of every 1-D operator (host code inside the CUDA
library, exported as kd_matrix_1d) against the numpy oracle.  Host-only
calls: no GPU needed."""
import ctypes as C

import numpy as np
import pytest

from kadath_frontera_gb300 import _lib
from oracle import spectral as S

THETA = [S.COS_EVEN, S.COS_ODD, S.SIN_EVEN, S.SIN_ODD]
FULL = [S.COS, S.SIN]
RADIAL = [S.CHEB, S.CHEB_EVEN, S.CHEB_ODD]

CASES = []
for n in (5, 7, 9, 11, 13, 17):
    for b in RADIAL + THETA + FULL:
        CASES.append((S.OP_COEF, b, n, n))
        CASES.append((S.OP_COEF_I, b, n, n))
        CASES.append((S.OP_DER, b, n, n))
    for b in THETA + FULL:
        CASES += [(S.OP_MULT_SIN, b, n, n), (S.OP_DIV_SIN, b, n, n), (S.OP_MULT_COS, b, n, n)]
    for b in THETA:
        CASES.append((S.OP_DIV_COS, b, n, n))
    for b in RADIAL:
        CASES += [(S.OP_MULT_X, b, n, n), (S.OP_DIV_1MX2, b, n, n)]
    for b in (S.CHEB_EVEN, S.CHEB_ODD):
        CASES.append((S.OP_DIV_X, b, n, n))
    CASES += [(S.OP_MULT_XM1, S.CHEB, n, n), (S.OP_DIV_XM1, S.CHEB, n, n), (S.OP_DIV_XP1, S.CHEB, n, n)]
for nphi in (1, 4, 6, 8, 12):
    CASES.append((S.OP_COEF, S.COSSIN, nphi, nphi + 2))
    CASES.append((S.OP_COEF_I, S.COSSIN, nphi + 2, nphi))
    if nphi >= 4:
        CASES += [(S.OP_DER, S.COSSIN, nphi + 2, nphi + 2), (S.OP_MULT_SIN, S.COSSIN, nphi + 2, nphi + 2),
                  (S.OP_MULT_COS, S.COSSIN, nphi + 2, nphi + 2)]
for nphi in (4, 8):
    for b in (S.COSSIN_EVEN, S.COSSIN_ODD):
        CASES.append((S.OP_COEF, b, nphi, nphi + 2))
        CASES.append((S.OP_COEF_I, b, nphi + 2, nphi))
        CASES.append((S.OP_DER, b, nphi + 2, nphi + 2))


def product_matrix(op, base, n_in, n_out):
    lib = _lib.load()
    m = (C.c_double * (n_in * n_out))()
    ob = C.c_int()
    st = lib.kd_matrix_1d(None, op, base, n_in, n_out, m, C.byref(ob))
    assert st == 0
    return ob.value, np.frombuffer(m, dtype=np.float64).reshape(n_out, n_in).copy()


@pytest.mark.parametrize("op,base,n_in,n_out", CASES)
def test_product_matrix_matches_oracle(op, base, n_in, n_out):
    ob, mp = product_matrix(op, base, n_in, n_out)
    if op == S.OP_COEF and base in (S.COSSIN, S.COSSIN_EVEN, S.COSSIN_ODD):
        # the oracle's forward line has nbr = n_out slots, of which the first n_in are values
        mo = np.zeros((n_out, n_in))
        for c in range(n_in):
            t = np.zeros(n_out)
            t[c] = 1.0
            mo[:, c] = S.COEF_1D[base](t)[:n_out]
        obo = base
    elif op == S.OP_COEF_I and base in (S.COSSIN, S.COSSIN_EVEN, S.COSSIN_ODD):
        mo = np.zeros((n_out, n_in))
        for c in range(n_in):
            t = np.zeros(n_in)
            t[c] = 1.0
            mo[:, c] = S.COEF_I_1D[base](t)[:n_out]
        obo = base
    else:
        obo, mo = S.matrix_1d(op, base, n_in, n_out)
    assert ob == obo
    scale = max(1.0, np.abs(mo).max())
    assert np.abs(mp - mo).max() <= 1e-13 * scale, np.abs(mp - mo).max()


def test_unsupported_pair_reports_status():
    lib = _lib.load()
    m = (C.c_double * 25)()
    ob = C.c_int()
    # div_x is defined only for the parity Chebyshev bases
    assert lib.kd_matrix_1d(None, S.OP_DIV_X, S.CHEB, 5, 5, m, C.byref(ob)) == _lib.KD_ERR_UNSUPPORTED


def _reference_cases():
    from pathlib import Path
    z = np.load(Path(__file__).resolve().parent / "golden" / "ref_spectral_1d.npz")
    out = []
    for key in z.files:
        if key.endswith("_base"):
            continue
        op, base, nin, nout = (int(t[1:] if t[0] in "bnm" else t[2:]) for t in key.split("_"))
        out.append((op, base, nin, nout, z[key], int(z[key + "_base"])))
    return out


def test_product_matrices_match_the_reference():
    """Every 1-D matrix the GPU applies, against the reference's own coef_1d,
    coef_i_1d and src/Ope_1d routines (tests/golden/ref_spectral_1d.npz,
    written by tests/golden/make_ref_vectors.py from the reference compiled
    here)."""
    cases = _reference_cases()
    assert len(cases) > 300
    checked = 0
    for op, base, nin, nout, ref, ref_base in cases:
        lib = _lib.load()
        m = (C.c_double * (nin * nout))()
        ob = C.c_int()
        st = lib.kd_matrix_1d(None, op, base, nin, nout, m, C.byref(ob))
        if st == _lib.KD_ERR_UNSUPPORTED:
            continue  # pairs the product does not build (none of the configurations' bases)
        assert st == 0
        mp = np.frombuffer(m, dtype=np.float64).reshape(nout, nin)
        scale = max(1.0, np.abs(ref).max())
        assert np.abs(mp - ref).max() <= 1e-13 * scale, (op, base, nin, nout, np.abs(mp - ref).max())
        if op not in (S.OP_COEF, S.OP_COEF_I):
            assert ob.value == ref_base, (op, base, nin)
        checked += 1
    print(f"{checked} of {len(cases)} reference matrices checked")
    assert checked >= 0.8 * len(cases)


def _grid(base, n):
    if base == S.CHEB:
        return [-np.cos(np.pi * i / (n - 1)) for i in range(n)]
    if base in (S.CHEB_EVEN, S.CHEB_ODD):
        return [np.sin(np.pi / 2 * i / (n - 1)) for i in range(n)]
    if base in (S.COS_EVEN, S.COS_ODD, S.SIN_EVEN, S.SIN_ODD):
        return [np.pi / 2 * i / (n - 1) for i in range(n)]
    return [2 * np.pi * k / n for k in range(n)]


RESAMPLE_OP = 14  # KD_OP_RESAMPLE


@pytest.mark.parametrize("base", RADIAL + THETA + [S.COSSIN])
@pytest.mark.parametrize("n_in,n_out", [(9, 13), (13, 9), (7, 7), (5, 17)])
def test_resample_matrix_is_the_reference_summation_at_the_new_grid(base, n_in, n_out):
    """kd_field_regrid's 1-D step: row r is the oracle's summation_1d (the
    restatement of src/Ope_1d/summation_1d.cpp) at the r-th point of the
    n_out-point grid of the basis."""
    if base == S.COSSIN:
        n_in, n_out = n_in + 1 - n_in % 2 + 2, n_out + 1 - n_out % 2  # phi: even point counts, 2 more coefs
    ob, mp = product_matrix(RESAMPLE_OP, base, n_in, n_out)
    assert ob == base
    pts = _grid(base, n_out)
    for c in range(n_in):
        e = np.zeros(n_in)
        e[c] = 1.0
        col = np.array([S.summation_1d(base, x, e) for x in pts])
        assert np.abs(mp[:, c] - col).max() <= 1e-13 * max(1.0, np.abs(col).max())


@pytest.mark.parametrize("base", RADIAL + THETA)
@pytest.mark.parametrize("n", [5, 9, 13])
def test_resample_onto_the_same_grid_is_the_inverse_transform(base, n):
    """On the field's own grid the resampling is coef_i, whose matrices are
    pinned to the reference (ref_spectral_1d.npz), on every coefficient slot
    that carries information on that grid (the reference's coef_i ignores
    the last slot of the odd bases)."""
    from tests.test_oracle_spectral import active_slots
    _, mr = product_matrix(RESAMPLE_OP, base, n, n)
    _, mi = product_matrix(S.OP_COEF_I, base, n, n)
    act = active_slots(base, n)  # the slots that carry information on the grid
    assert np.abs(mr[:, act] - mi[:, act]).max() <= 1e-13 * max(1.0, np.abs(mi).max())
