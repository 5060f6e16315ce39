"""CPU oracle for the spectral layer of Kadath (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module, and only as the checker.  The product
path (``kadath_frontera_gb300``) never imports it.

This is a line-by-line numpy restatement of the reference's 1-D routines:

* forward transforms  -- src/Coef/coef_1d.cpp  (coef_1d_<basis>, dispatch :607)
* inverse transforms  -- src/Coef/coef_i_1d.cpp (coef_i_1d_<basis>, dispatch :527)
* separable 3-D drivers -- src/Coef/coef.cpp:28-104, src/Coef/coef_i.cpp:28-104
* coefficient-space operators -- src/Ope_1d/*.cpp
* evaluation of a coefficient line -- src/Ope_1d/summation_1d.cpp

The reference calls FFTW 3.3.8 (not vendored, Cmake/CMakeLocal.cmake:14-16)
for its length-(n-1) real DFTs in FFTW_R2HC / FFTW_HC2R mode.  FFTW's
published halfcomplex layout is restated in ``r2hc``/``hc2r`` below on top
of numpy's FFT.

Pinning: no test of the reference holds coefficient values, so the
transforms are pinned by known answers derived from the reference's own
evaluation routine (summation_1d): sampling each basis function at the
collocation points of src/Domain/Spheric/domain_*.cpp (do_coloc) must give
the unit coefficient vector, and coef_i must reproduce the samples.  The
system-level restatement (oracle/kadath.py) is pinned by the analytic
solutions printed by tutorials/tuto5.cpp and codes/Seq_version/schwarz.cpp.
"""
from __future__ import annotations

import math

import numpy as np

CHEB, CHEB_EVEN, CHEB_ODD, COSSIN, COS, COS_EVEN, COS_ODD, SIN, SIN_EVEN, SIN_ODD = 1, 2, 3, 4, 5, 6, 7, 8, 9, 10
LEG, LEG_EVEN, LEG_ODD, COSSIN_EVEN, COSSIN_ODD = 11, 12, 13, 14, 15

ALL_BASES = (CHEB, CHEB_EVEN, CHEB_ODD, COSSIN, COS, COS_EVEN, COS_ODD, SIN, SIN_EVEN, SIN_ODD,
             COSSIN_EVEN, COSSIN_ODD)
BASE_NAMES = {CHEB: "CHEB", CHEB_EVEN: "CHEB_EVEN", CHEB_ODD: "CHEB_ODD", COSSIN: "COSSIN", COS: "COS",
              COS_EVEN: "COS_EVEN", COS_ODD: "COS_ODD", SIN: "SIN", SIN_EVEN: "SIN_EVEN", SIN_ODD: "SIN_ODD",
              COSSIN_EVEN: "COSSIN_EVEN", COSSIN_ODD: "COSSIN_ODD"}

# Operator codes (same numbering as include/kadath_gb300.h KD_OP_*).
OP_COEF, OP_COEF_I, OP_DER, OP_MULT_SIN, OP_DIV_SIN, OP_MULT_COS, OP_DIV_COS = 0, 1, 2, 3, 4, 5, 6
OP_MULT_X, OP_DIV_X, OP_MULT_XM1, OP_DIV_XM1, OP_DIV_XP1, OP_DIV_1MX2 = 7, 8, 9, 10, 11, 12


# --------------------------------------------------------------- FFTW r2r --
def r2hc(x: np.ndarray) -> np.ndarray:
    """FFTW_R2HC: h[k]=Re Y_k (k<=n/2), h[n-k]=Im Y_k (0<k<(n+1)/2)."""
    n = len(x)
    y = np.fft.rfft(x)
    h = np.zeros(n)
    h[: n // 2 + 1] = y.real[: n // 2 + 1]
    for k in range(1, (n + 1) // 2):
        h[n - k] = y.imag[k]
    return h


def hc2r(h: np.ndarray) -> np.ndarray:
    """FFTW_HC2R (unnormalised inverse of r2hc)."""
    n = len(h)
    y = np.zeros(n // 2 + 1, dtype=complex)
    y.real[: n // 2 + 1] = h[: n // 2 + 1]
    for k in range(1, (n + 1) // 2):
        y.imag[k] = h[n - k]
    return np.fft.irfft(y, n) * n


# ----------------------------------------------------------------- coef_1d --
def _cheb_like_forward(tab, nr, sym_sign, cheb_style):
    """Shared body of coef_1d_cheb (cheb_style) and coef_1d_cheb_even/cos/..."""
    aux = np.zeros(nr - 1)
    for i in range(1, (nr - 1) // 2):
        fp = 0.5 * (tab[i] + tab[nr - 1 - i])
        if sym_sign > 0:
            fms = 0.5 * (tab[i] - tab[nr - 1 - i]) * math.sin(math.pi * i / (nr - 1))
        else:
            fms = 0.5 * (-tab[i] + tab[nr - 1 - i]) * math.sin(math.pi * i / (nr - 1))
        aux[i] = fp + fms
        aux[nr - 1 - i] = fp - fms
    aux[0] = 0.5 * (tab[0] + tab[nr - 1])
    aux[(nr - 1) // 2] = tab[(nr - 1) // 2]
    return r2hc(aux)


def coef_1d_cheb(tab):
    nr = len(tab)
    fmoins0 = 0.5 * (tab[0] - tab[nr - 1])
    aux = _cheb_like_forward(tab, nr, +1, True)
    out = np.zeros(nr)
    out[0] = aux[0] / (nr - 1)
    for i in range(2, nr - 1, 2):
        out[i] = 2 * aux[i // 2] / (nr - 1)
    out[nr - 1] = aux[(nr - 1) // 2] / (nr - 1)
    out[1] = 0
    som = 0.0
    for i in range(3, nr, 2):
        out[i] = out[i - 2] - 4 * aux[nr - 1 - (i - 1) // 2] / (nr - 1)
        som += out[i]
    c1 = -(fmoins0 + som) / ((nr - 1) // 2)
    out[1] = c1
    for i in range(3, nr, 2):
        out[i] += c1
    return out


def _even_unscramble(aux, nr, fmoins0):
    out = np.zeros(nr)
    out[0] = aux[0] / (nr - 1)
    for i in range(2, nr - 1, 2):
        out[i] = 2 * aux[i // 2] / (nr - 1)
    out[nr - 1] = aux[(nr - 1) // 2] / (nr - 1)
    out[1] = 0
    som = 0.0
    for i in range(3, nr, 2):
        out[i] = out[i - 2] + 4 * aux[nr - 1 - i // 2] / (nr - 1)
        som += out[i]
    c1 = (fmoins0 - som) / ((nr - 1) // 2)
    out[1] = c1
    for i in range(3, nr, 2):
        out[i] += c1
    return out


def coef_1d_cheb_even(tab):
    nr = len(tab)
    fmoins0 = -0.5 * (tab[0] - tab[nr - 1])
    aux = _cheb_like_forward(tab, nr, -1, False)
    return _even_unscramble(aux, nr, fmoins0)


def coef_1d_cheb_odd(tab):
    nr = len(tab)
    cf = np.array([tab[i] * math.sin(math.pi / 2. * i / (nr - 1)) for i in range(nr)])
    fmoins0 = -0.5 * (cf[0] - cf[nr - 1])
    aux = _cheb_like_forward(cf, nr, -1, False)
    cf = _even_unscramble(aux, nr, fmoins0)
    cf[0] = 2 * cf[0]
    for i in range(1, nr - 1):
        cf[i] = 2 * cf[i] - cf[i - 1]
    cf[nr - 1] = 0
    return cf


def coef_1d_cossin(tab):
    nbr = len(tab)
    out = np.array(tab, dtype=float)
    if nbr > 3:
        h = r2hc(np.array(tab[: nbr - 2], dtype=float))
        idx, pc, ps = 0, 0, nbr - 3
        out[idx] = h[pc] / (nbr - 2); idx += 1; pc += 1
        out[idx] = 0; idx += 1
        for _ in range(1, nbr // 2 - 1):
            out[idx] = 2. * h[pc] / (nbr - 2); idx += 1; pc += 1
            out[idx] = -2. * h[ps] / (nbr - 2); idx += 1; ps -= 1
        out[idx] = h[pc] / (nbr - 2); idx += 1
        out[idx] = 0
    else:
        out[1] = 0
        out[2] = 0
    return out


def coef_1d_cos(tab):
    nbr = len(tab)
    fmoins0 = 0.5 * (tab[0] - tab[nbr - 1])
    aux = _cheb_like_forward(tab, nbr, +1, False)
    return _even_unscramble(aux, nbr, fmoins0)


def _sin_forward(tab, nbr, minus0):
    aux = np.zeros(nbr - 1)
    for i in range(1, (nbr - 1) // 2):
        fp = 0.5 * (tab[i] + tab[nbr - 1 - i]) * math.sin(math.pi * i / (nbr - 1))
        fms = 0.5 * (tab[i] - tab[nbr - 1 - i])
        aux[i] = fp + fms
        aux[nbr - 1 - i] = fp - fms
    aux[0] = 0.5 * (tab[0] - tab[nbr - 1]) if minus0 else 0.5 * (tab[0] + tab[nbr - 1])
    aux[(nbr - 1) // 2] = tab[(nbr - 1) // 2]
    aux = r2hc(aux)
    out = np.zeros(nbr)
    for i in range(2, nbr - 1, 2):
        out[i] = -2 * aux[nbr - 1 - i // 2] / (nbr - 1)
    out[1] = 2 * aux[0] / (nbr - 1)
    for i in range(3, nbr, 2):
        out[i] = out[i - 2] + 4 * aux[i // 2] / (nbr - 1)
    return out


def coef_1d_sin(tab):
    return _sin_forward(tab, len(tab), False)


def coef_1d_cos_even(tab):
    return coef_1d_cos(tab) if len(tab) > 3 else np.array(tab, dtype=float)


def coef_1d_cos_odd(tab):
    nbr = len(tab)
    if nbr <= 3:
        return np.array(tab, dtype=float)
    cf = np.zeros(nbr)
    for i in range(nbr - 1):
        cf[i] = tab[i] * math.sin(math.pi * (nbr - 1 - i) / 2. / (nbr - 1))
    cf[nbr - 1] = 0
    fmoins0 = 0.5 * (cf[0] - cf[nbr - 1])
    aux = _cheb_like_forward(cf, nbr, +1, False)
    cf = _even_unscramble(aux, nbr, fmoins0)
    cf[0] = 2 * cf[0]
    for i in range(1, nbr - 1):
        cf[i] = 2 * cf[i] - cf[i - 1]
    cf[nbr - 1] = 0
    return cf


def coef_1d_sin_even(tab):
    if len(tab) <= 3:
        return np.array(tab, dtype=float)
    return _sin_forward(tab, len(tab), True)


def coef_1d_sin_odd(tab):
    nbr = len(tab)
    if nbr <= 3:
        return np.array(tab, dtype=float)
    cf = np.zeros(nbr)
    for i in range(1, nbr):
        cf[i] = tab[i] * math.sin(math.pi * i / 2. / (nbr - 1))
    fmoins0 = 0.5 * (cf[0] - cf[nbr - 1])
    aux = _cheb_like_forward(cf, nbr, +1, False)
    cf = _even_unscramble(aux, nbr, fmoins0)
    cf[0] = 2 * cf[0]
    for i in range(1, nbr - 1):
        cf[i] = 2 * cf[i] + cf[i - 1]
    cf[nbr - 1] = 0
    return cf


def coef_1d_cossin_even(tab):
    nbr = len(tab)
    tab2 = np.zeros(2 * nbr - 2)
    for i in range(nbr - 2):
        tab2[i] = tab[i]
        tab2[i + nbr - 2] = tab[i]
    tab2 = coef_1d_cossin(tab2)
    out = np.array(tab, dtype=float)
    c = 0
    for k in range(0, nbr - 1, 2):
        out[k] = tab2[c]
        out[k + 1] = tab2[c + 1]
        c += 4
    return out


def coef_1d_cossin_odd(tab):
    nbr = len(tab)
    tab2 = np.zeros(2 * nbr - 2)
    for i in range(nbr - 2):
        tab2[i] = tab[i]
        tab2[i + nbr - 2] = -tab[i]
    tab2 = coef_1d_cossin(tab2)
    out = np.array(tab, dtype=float)
    c = 2
    for k in range(0, nbr - 3, 2):
        out[k] = tab2[c]
        out[k + 1] = tab2[c + 1]
        c += 4
    out[nbr - 2] = 0.
    out[nbr - 1] = 0.
    return out


COEF_1D = {CHEB: coef_1d_cheb, CHEB_EVEN: coef_1d_cheb_even, CHEB_ODD: coef_1d_cheb_odd, COSSIN: coef_1d_cossin,
           COS: coef_1d_cos, SIN: coef_1d_sin, COS_EVEN: coef_1d_cos_even, COS_ODD: coef_1d_cos_odd,
           SIN_EVEN: coef_1d_sin_even, SIN_ODD: coef_1d_sin_odd, COSSIN_EVEN: coef_1d_cossin_even,
           COSSIN_ODD: coef_1d_cossin_odd}


# --------------------------------------------------------------- coef_i_1d --
def _hc_from_cheb_coefs(tab, nbr, sign):
    cf = np.zeros(nbr)
    c1 = tab[1]
    somme = 0.0
    for i in range(3, nbr, 2):
        cf[i] = tab[i] - c1
        somme += cf[i]
    half = (nbr - 1) // 2
    fmoins0 = sign * (half * c1 + somme)
    aux = np.zeros(nbr - 1)
    for i in range(3, nbr, 2):
        aux[nbr - 1 - i // 2] = sign * 0.25 * (cf[i] - cf[i - 2])
    aux[0] = tab[0]
    for i in range(1, (nbr - 1) // 2):
        aux[i] = 0.5 * tab[2 * i]
    aux[(nbr - 1) // 2] = tab[nbr - 1]
    return hc2r(aux), fmoins0


def coef_i_1d_cheb(tab):
    nbr = len(tab)
    out = np.array(tab, dtype=float)
    if nbr > 3:
        aux, fmoins0 = _hc_from_cheb_coefs(tab, nbr, -1.0)
        for i in range(1, (nbr - 1) // 2):
            fp = 0.5 * (aux[i] + aux[nbr - 1 - i])
            fm = 0.5 * (aux[i] - aux[nbr - 1 - i]) / math.sin(math.pi * i / (nbr - 1))
            out[i] = fp + fm
            out[nbr - i - 1] = fp - fm
        out[0] = aux[0] + fmoins0
        out[nbr - 1] = aux[0] - fmoins0
        out[(nbr - 1) // 2] = aux[(nbr - 1) // 2]
    return out


def coef_i_1d_cheb_even(tab):
    nbr = len(tab)
    out = np.array(tab, dtype=float)
    aux, fmoins0 = _hc_from_cheb_coefs(tab, nbr, +1.0)
    for i in range(1, (nbr - 1) // 2):
        fp = 0.5 * (aux[i] + aux[nbr - 1 - i])
        fm = 0.5 * (aux[i] - aux[nbr - 1 - i]) / math.sin(math.pi * i / (nbr - 1))
        out[nbr - 1 - i] = fp + fm
        out[i] = fp - fm
    out[0] = aux[0] - fmoins0
    out[nbr - 1] = aux[0] + fmoins0
    out[(nbr - 1) // 2] = aux[(nbr - 1) // 2]
    return out


def _ti(tab, nbr, sign):
    ti = np.zeros(nbr)
    ti[0] = 0.5 * tab[0]
    for i in range(1, nbr - 1):
        ti[i] = 0.5 * (tab[i] + sign * tab[i - 1])
    ti[nbr - 1] = sign * 0.5 * tab[nbr - 2]
    return ti


def coef_i_1d_cheb_odd(tab):
    nbr = len(tab)
    out = np.array(tab, dtype=float)
    ti = _ti(tab, nbr, +1)
    aux, fmoins0 = _hc_from_cheb_coefs(ti, nbr, +1.0)
    for i in range(1, (nbr - 1) // 2):
        fp = 0.5 * (aux[i] + aux[nbr - 1 - i])
        fm = 0.5 * (aux[i] - aux[nbr - 1 - i]) / math.sin(math.pi * i / (nbr - 1))
        out[nbr - 1 - i] = (fp + fm) / math.sin(math.pi * (nbr - 1 - i) / 2 / (nbr - 1))
        out[i] = (fp - fm) / math.sin(math.pi * i / 2 / (nbr - 1))
    out[0] = 0
    out[nbr - 1] = aux[0] + fmoins0
    out[(nbr - 1) // 2] = aux[(nbr - 1) // 2] / math.sin(math.pi * (nbr - 1) / 4 / (nbr - 1))
    return out


def coef_i_1d_cossin(tab):
    nbr = len(tab)
    out = np.array(tab, dtype=float)
    np_ = nbr - 2
    if np_ > 1:
        cf = np.zeros(np_)
        cf[0] = tab[0]
        for i in range(1, np_ // 2):
            cf[i] = 0.5 * tab[2 * i]
            cf[np_ - i] = -0.5 * tab[2 * i + 1]
        cf[np_ // 2] = tab[np_]
        x = hc2r(cf)
        out[:np_] = x
    return out


def coef_i_1d_cos(tab):
    nbr = len(tab)
    out = np.array(tab, dtype=float)
    aux, fmoins0 = _hc_from_cheb_coefs(tab, nbr, +1.0)
    for i in range(1, (nbr - 1) // 2):
        fp = 0.5 * (aux[i] + aux[nbr - 1 - i])
        fm = 0.5 * (aux[i] - aux[nbr - 1 - i]) / math.sin(math.pi * i / (nbr - 1))
        out[i] = fp + fm
        out[nbr - i - 1] = fp - fm
    out[0] = aux[0] + fmoins0
    out[nbr - 1] = aux[0] - fmoins0
    out[(nbr - 1) // 2] = aux[(nbr - 1) // 2]
    return out


def _sin_inverse(tab, nbr, even_variant):
    aux = np.zeros(nbr - 1)
    for i in range(2, nbr - 1, 2):
        aux[nbr - 1 - i // 2] = -0.5 * tab[i]
    aux[0] = 0.5 * tab[1]
    if even_variant:
        for i in range(1, (nbr - 1) // 2):
            aux[i] = 0.25 * (tab[2 * i + 1] - tab[2 * i - 1])
    else:
        for i in range(3, nbr, 2):
            aux[i // 2] = 0.25 * (tab[i] - tab[i - 2])
    aux[(nbr - 1) // 2] = -0.5 * tab[nbr - 2]
    aux = hc2r(aux)
    out = np.array(tab, dtype=float)
    for i in range(1, (nbr - 1) // 2):
        fp = 0.5 * (aux[i] + aux[nbr - 1 - i]) / math.sin(math.pi * i / (nbr - 1))
        fm = 0.5 * (aux[i] - aux[nbr - 1 - i])
        out[i] = fp + fm
        out[nbr - i - 1] = fp - fm
    out[0] = 0
    out[nbr - 1] = -2 * aux[0]
    out[(nbr - 1) // 2] = aux[(nbr - 1) // 2]
    return out


def coef_i_1d_sin(tab):
    return _sin_inverse(tab, len(tab), False)


def coef_i_1d_cos_even(tab):
    return coef_i_1d_cos(tab) if len(tab) > 3 else np.array(tab, dtype=float)


def coef_i_1d_cos_odd(tab):
    nbr = len(tab)
    out = np.array(tab, dtype=float)
    if nbr <= 3:
        return out
    ti = _ti(tab, nbr, +1)
    aux, fmoins0 = _hc_from_cheb_coefs(ti, nbr, +1.0)
    for i in range(1, (nbr - 1) // 2):
        fp = 0.5 * (aux[i] + aux[nbr - 1 - i])
        fm = 0.5 * (aux[i] - aux[nbr - 1 - i]) / math.sin(math.pi * i / (nbr - 1))
        out[i] = (fp + fm) / math.sin(math.pi * (nbr - 1 - i) / 2 / (nbr - 1))
        out[nbr - i - 1] = (fp - fm) / math.sin(math.pi * i / 2 / (nbr - 1))
    out[0] = aux[0] + fmoins0
    out[nbr - 1] = 0
    out[(nbr - 1) // 2] = aux[(nbr - 1) // 2] / math.sin(math.pi * (nbr - 1) / 4 / (nbr - 1))
    return out


def coef_i_1d_sin_even(tab):
    if len(tab) <= 3:
        return np.array(tab, dtype=float)
    return _sin_inverse(tab, len(tab), True)


def coef_i_1d_sin_odd(tab):
    nbr = len(tab)
    out = np.array(tab, dtype=float)
    if nbr <= 3:
        return out
    ti = _ti(tab, nbr, -1)
    aux, fmoins0 = _hc_from_cheb_coefs(ti, nbr, +1.0)
    for i in range(1, (nbr - 1) // 2):
        fp = 0.5 * (aux[i] + aux[nbr - 1 - i])
        fm = 0.5 * (aux[i] - aux[nbr - 1 - i]) / math.sin(math.pi * i / (nbr - 1))
        out[i] = (fp + fm) / math.sin(math.pi * i / 2 / (nbr - 1))
        out[nbr - i - 1] = (fp - fm) / math.sin(math.pi * (nbr - 1 - i) / 2 / (nbr - 1))
    out[0] = 0
    out[nbr - 1] = aux[0] - fmoins0
    out[(nbr - 1) // 2] = aux[(nbr - 1) // 2] / math.sin(math.pi * (nbr - 1) / 4 / (nbr - 1))
    return out


def coef_i_1d_cossin_even(tab):
    nbr = len(tab)
    tab2 = np.zeros(2 * nbr - 2)
    c = 0
    for i in range(0, nbr - 2, 2):
        tab2[c], tab2[c + 1], tab2[c + 2], tab2[c + 3] = tab[i], tab[i + 1], 0., 0.
        c += 4
    tab2[c], tab2[c + 1] = tab[nbr - 2], tab[nbr - 1]
    tab2 = coef_i_1d_cossin(tab2)
    out = np.array(tab, dtype=float)
    out[: nbr - 2] = tab2[: nbr - 2]
    out[nbr - 2] = 0
    out[nbr - 1] = 0
    return out


def coef_i_1d_cossin_odd(tab):
    nbr = len(tab)
    tab2 = np.zeros(2 * nbr - 2)
    c = 0
    for i in range(0, nbr - 2, 2):
        tab2[c], tab2[c + 1], tab2[c + 2], tab2[c + 3] = 0., 0., tab[i], tab[i + 1]
        c += 4
    tab2[c], tab2[c + 1] = tab[nbr - 2], tab[nbr - 1]
    tab2 = coef_i_1d_cossin(tab2)
    out = np.array(tab, dtype=float)
    out[: nbr - 2] = tab2[: nbr - 2]
    out[nbr - 2] = 0
    out[nbr - 1] = 0
    return out


COEF_I_1D = {CHEB: coef_i_1d_cheb, CHEB_EVEN: coef_i_1d_cheb_even, CHEB_ODD: coef_i_1d_cheb_odd,
             COSSIN: coef_i_1d_cossin, COS: coef_i_1d_cos, SIN: coef_i_1d_sin, COS_EVEN: coef_i_1d_cos_even,
             COS_ODD: coef_i_1d_cos_odd, SIN_EVEN: coef_i_1d_sin_even, SIN_ODD: coef_i_1d_sin_odd,
             COSSIN_EVEN: coef_i_1d_cossin_even, COSSIN_ODD: coef_i_1d_cossin_odd}


# ------------------------------------------------------------ summation_1d --
def summation_1d(base: int, xx: float, tab) -> float:
    """Evaluation of one coefficient line at xx (src/Ope_1d/summation_1d.cpp)."""
    nr = len(tab)
    if base == CHEB:
        tm2, tm1 = 1.0, xx
        res = tab[0] * tm2 + (tab[1] * tm1 if nr > 1 else 0.0)
        for i in range(2, nr):
            tm = 2 * xx * tm1 - tm2
            res += tab[i] * tm
            tm2, tm1 = tm1, tm
        return res
    if base == CHEB_EVEN:
        return sum(tab[i] * math.cos(2 * i * math.acos(max(-1.0, min(1.0, xx)))) for i in range(nr))
    if base == CHEB_ODD:
        return sum(tab[i] * math.cos((2 * i + 1) * math.acos(max(-1.0, min(1.0, xx)))) for i in range(nr))
    if base == COSSIN:
        return sum(tab[i] * math.cos((i // 2) * xx) if i % 2 == 0 else tab[i] * math.sin(((i - 1) // 2) * xx)
                   for i in range(nr))
    if base == COSSIN_EVEN:
        return sum(tab[i] * math.cos(i * xx) if i % 2 == 0 else tab[i] * math.sin((i - 1) * xx) for i in range(nr))
    if base == COSSIN_ODD:
        return sum(tab[i] * math.cos((i + 1) * xx) if i % 2 == 0 else tab[i] * math.sin(i * xx) for i in range(nr))
    if base == COS:
        return sum(tab[i] * math.cos(i * xx) for i in range(nr))
    if base == SIN:
        return sum(tab[i] * math.sin(i * xx) for i in range(1, nr))
    if base == COS_EVEN:
        return sum(tab[i] * math.cos(2 * i * xx) for i in range(nr))
    if base == COS_ODD:
        return sum(tab[i] * math.cos((2 * i + 1) * xx) for i in range(nr))
    if base == SIN_EVEN:
        return sum(tab[i] * math.sin(2 * i * xx) for i in range(1, nr))
    if base == SIN_ODD:
        return sum(tab[i] * math.sin((2 * i + 1) * xx) for i in range(nr))
    raise ValueError(f"summation_1d: basis {base}")


# ------------------------------------------------------------- ope_1d ops --
def der_1d(base, tab):
    """src/Ope_1d/der_1d.cpp:31-289; returns (output basis, line)."""
    t = np.asarray(tab, dtype=float)
    nr = len(t)
    res = np.zeros(nr)
    if base == CHEB:
        for i in range(nr):
            for p in range(i + 1, nr, 2):
                res[i] += p * t[p]
        res *= 2
        res[0] /= 2
        return CHEB, res
    if base == CHEB_EVEN:
        for i in range(nr):
            for p in range(i + 1, nr):
                res[i] += 2 * p * t[p]
        res[nr - 1] = 0
        return CHEB_ODD, 2 * res
    if base == CHEB_ODD:
        for i in range(nr):
            for p in range(i, nr):
                res[i] += (2 * p + 1) * t[p]
        res *= 2
        res[0] /= 2
        return CHEB_EVEN, res
    if base in (COSSIN, COSSIN_EVEN, COSSIN_ODD):
        for i in range(0, nr - 1, 2):
            m = {COSSIN: i // 2, COSSIN_EVEN: i, COSSIN_ODD: i + 1}[base]
            res[i + 1] = -m * t[i]
        for i in range(1, nr, 2):
            m = {COSSIN: (i - 1) // 2, COSSIN_EVEN: i - 1, COSSIN_ODD: i}[base]
            res[i - 1] = m * t[i]
        if base == COSSIN:
            res[nr - 1] = 0
        return base, res
    k = np.arange(nr)
    if base == COS:
        return SIN, -k * t
    if base == SIN:
        return COS, k * t
    if base == COS_EVEN:
        res = -2 * k * t
        res[nr - 1] = 0
        return SIN_EVEN, res
    if base == COS_ODD:
        return SIN_ODD, -(2 * k + 1) * t
    if base == SIN_EVEN:
        return COS_EVEN, 2 * k * t
    if base == SIN_ODD:
        res = (2 * k + 1) * t
        res[nr - 1] = 0
        return COS_ODD, res
    raise ValueError(base)


def mult_sin_1d(base, tab):
    """src/Ope_1d/mult_sin_1d.cpp"""
    t = np.asarray(tab, dtype=float)
    nr = len(t)
    r = np.zeros(nr)
    if base == COSSIN:
        r[0] = 0.5 * t[3]; r[1] = 0; r[2] = 0.5 * t[5]; r[3] = t[0] - 0.5 * t[4]
        for k in range(4, nr - 2, 2):
            r[k] = 0.5 * (t[3 + k] - t[k - 1])
            r[k + 1] = 0.5 * (t[k - 2] - t[k + 2])
        r[nr - 2] = -0.5 * t[nr - 3]; r[nr - 1] = 0
        return COSSIN, r
    if base == COS:
        r[1] = t[0] - 0.5 * t[2]
        for k in range(2, nr - 1):
            r[k] = 0.5 * (t[k - 1] - t[k + 1])
        return SIN, r
    if base == SIN:
        r[0] = 0.5 * t[1]; r[1] = 0.5 * t[2]
        for k in range(2, nr - 1):
            r[k] = 0.5 * (-t[k - 1] + t[k + 1])
        return COS, r
    if base == COS_EVEN:
        r[0] = t[0] - 0.5 * t[1]
        for k in range(1, nr - 1):
            r[k] = 0.5 * (t[k] - t[k + 1])
        return SIN_ODD, r
    if base == COS_ODD:
        for k in range(1, nr):
            r[k] = 0.5 * (t[k - 1] - t[k])
        return SIN_EVEN, r
    if base == SIN_EVEN:
        r[0] = 0.5 * t[1]
        for k in range(1, nr - 1):
            r[k] = 0.5 * (-t[k] + t[k + 1])
        return COS_ODD, r
    if base == SIN_ODD:
        r[0] = 0.5 * t[0]
        for k in range(1, nr):
            r[k] = 0.5 * (-t[k - 1] + t[k])
        return COS_EVEN, r
    raise ValueError(base)


def mult_cos_1d(base, tab):
    """src/Ope_1d/mult_cos_1d.cpp"""
    t = np.asarray(tab, dtype=float)
    nr = len(t)
    r = np.zeros(nr)
    if base == COSSIN:
        r[0] = 0.5 * t[2]; r[2] = t[0] + 0.5 * t[4]; r[3] = 0.5 * t[5]
        for k in range(4, nr - 2):
            r[k] = 0.5 * (t[2 + k] + t[k - 2])
        r[nr - 2] = 0.5 * t[nr - 4]
        return COSSIN, r
    if base == COS:
        r[0] = 0.5 * t[1]; r[1] = t[0] + 0.5 * t[2]
        for k in range(2, nr - 1):
            r[k] = 0.5 * (t[k - 1] + t[k + 1])
        return COS, r
    if base == SIN:
        r[1] = 0.5 * t[2]
        for k in range(2, nr - 1):
            r[k] = 0.5 * (t[k - 1] + t[k + 1])
        return SIN, r
    if base == COS_EVEN:
        r[0] = t[0] + 0.5 * t[1]
        for k in range(1, nr - 1):
            r[k] = 0.5 * (t[k] + t[k + 1])
        return COS_ODD, r
    if base == COS_ODD:
        r[0] = 0.5 * t[0]
        for k in range(1, nr):
            r[k] = 0.5 * (t[k - 1] + t[k])
        return COS_EVEN, r
    if base == SIN_EVEN:
        r[0] = 0.5 * t[1]
        for k in range(1, nr - 1):
            r[k] = 0.5 * (t[k] + t[k + 1])
        return SIN_ODD, r
    if base == SIN_ODD:
        for k in range(1, nr):
            r[k] = 0.5 * (t[k - 1] + t[k])
        return SIN_EVEN, r
    raise ValueError(base)


def div_sin_1d(base, tab):
    """src/Ope_1d/div_sin_1d.cpp"""
    t = np.asarray(tab, dtype=float)
    nr = len(t)
    r = np.zeros(nr)
    s = 0.0
    if base in (COS, SIN):
        sg = -1.0 if base == COS else 1.0
        for k in range(nr - 2, -1, -2):
            s += sg * 2 * t[k]
            if k - 1 >= 0:
                r[k - 1] = s
        s = 0.0
        for k in range(nr - 3, -1, -2):
            s += sg * 2 * t[k + 2]
            r[k + 1] = s
        if base == COS:
            r[0] = 0
            return SIN, r
        r[0] *= 0.5
        return COS, r
    if base == COS_EVEN:
        for k in range(nr - 2, -1, -1):
            s -= 2 * t[k + 1]; r[k] = s
        return SIN_ODD, r
    if base == COS_ODD:
        for k in range(nr - 2, -1, -1):
            s -= 2 * t[k]; r[k] = s
        return SIN_EVEN, r
    if base == SIN_EVEN:
        for k in range(nr - 2, -1, -1):
            s += 2 * t[k + 1]; r[k] = s
        return COS_ODD, r
    if base == SIN_ODD:
        for k in range(nr - 2, -1, -1):
            s += 2 * t[k]; r[k] = s
        r[0] *= 0.5
        return COS_EVEN, r
    raise ValueError(base)


def div_cos_1d(base, tab):
    """src/Ope_1d/div_cos_1d.cpp"""
    t = np.asarray(tab, dtype=float)
    nr = len(t)
    r = np.zeros(nr)
    s = 0.0
    if base == COS_EVEN:
        sg = 1
        for k in range(nr - 2, -1, -1):
            s -= 2 * sg * t[k + 1]; sg = -sg
            r[k] = s if k % 2 == 0 else -s
        return COS_ODD, r
    if base == SIN_ODD:
        sg = -1
        for k in range(nr - 2, 0, -1):
            s -= 2 * sg * t[k]; sg = -sg
            r[k] = -s if k % 2 == 0 else s
        return SIN_EVEN, r
    if base == COS_ODD:
        sg = -1
        for k in range(nr - 2, -1, -1):
            s += 2 * t[k] * sg
            r[k] = s if k % 2 == 0 else -s
            sg = -sg
        r[0] *= 0.5
        return COS_EVEN, r
    if base == SIN_EVEN:
        sg = -1
        for k in range(nr - 2, -1, -1):
            s -= 2 * t[k + 1] * sg; sg = -sg
            r[k] = -s if k % 2 == 0 else s
        return SIN_ODD, r
    raise ValueError(base)


def mult_x_1d(base, tab):
    """src/Ope_1d/mult_x_1d.cpp"""
    t = np.asarray(tab, dtype=float)
    nr = len(t)
    r = np.zeros(nr)
    if base == CHEB:
        r[0] = 0.5 * t[1]; r[1] = t[0] + 0.5 * t[2]
        for i in range(2, nr - 1):
            r[i] = 0.5 * (t[i + 1] + t[i - 1])
        r[nr - 1] = 0.5 * t[nr - 2]
        return CHEB, r
    if base == CHEB_EVEN:
        r[0] = t[0] + 0.5 * t[1]
        for i in range(1, nr - 1):
            r[i] = 0.5 * (t[i] + t[i + 1])
        return CHEB_ODD, r
    if base == CHEB_ODD:
        r[0] = 0.5 * t[0]
        for i in range(1, nr - 1):
            r[i] = 0.5 * (t[i] + t[i - 1])
        r[nr - 1] = 0.5 * t[nr - 2]
        return CHEB_EVEN, r
    raise ValueError(base)


def div_x_1d(base, tab):
    """src/Ope_1d/div_x_1d.cpp"""
    t = np.asarray(tab, dtype=float)
    nr = len(t)
    r = np.zeros(nr)
    sgn = 1
    if base == CHEB_EVEN:
        s = 2 * sgn * t[nr - 1]
        r[nr - 2] = s
        for i in range(nr - 3, -1, -1):
            sgn = -sgn; s += 2 * sgn * t[i + 1]; r[i] = s
        r[0::2] *= -1
        return CHEB_ODD, r
    if base == CHEB_ODD:
        s = 2 * sgn * t[nr - 2]
        r[nr - 2] = s
        for i in range(nr - 3, -1, -1):
            sgn = -sgn; s += 2 * sgn * t[i]; r[i] = s
        r[0::2] *= -1
        r[0] *= 0.5
        return CHEB_EVEN, r
    raise ValueError(base)


def mult_xm1_1d(base, tab):
    """src/Ope_1d/mult_xm1_1d.cpp:26"""
    if base != CHEB:
        raise ValueError(base)
    t = np.asarray(tab, dtype=float)
    nr = len(t)
    r = np.zeros(nr)
    r[0] = -t[0] + 0.5 * t[1]
    r[1] = t[0] - t[1] + 0.5 * t[2]
    for i in range(2, nr - 1):
        r[i] = 0.5 * t[i - 1] - t[i] + 0.5 * t[i + 1]
    r[nr - 1] = 0.5 * t[nr - 2] - t[nr - 1]
    return CHEB, r


def div_xm1_1d(base, tab):
    """src/Ope_1d/div_xm1_1d.cpp:27"""
    if base != CHEB:
        raise ValueError(base)
    t = np.asarray(tab, dtype=float)
    nr = len(t)
    r = np.zeros(nr)
    for i in range(nr - 1):
        for j in range(i + 1, nr):
            r[i] += 2 * (j - i) * t[j]
    r[0] *= 0.5
    return CHEB, r


def div_xp1_1d(base, tab):
    """src/Ope_1d/div_xp1_1d.cpp:25"""
    if base != CHEB:
        raise ValueError(base)
    t = np.asarray(tab, dtype=float)
    nr = len(t)
    r = np.zeros(nr)
    r[nr - 2] = 2 * t[nr - 1]
    for i in range(nr - 3, 0, -1):
        r[i] = 2 * t[i + 1] - 2 * r[i + 1] - r[i + 2]
    s = sum(t[i] if i % 2 == 0 else -t[i] for i in range(nr))
    r[0] = t[0] - r[1] / 2. - s
    return CHEB, r


def div_1mx2_1d(base, tab):
    """src/Ope_1d/div_1mx2.cpp"""
    t = np.asarray(tab, dtype=float)
    nr = len(t)
    r = np.zeros(nr)
    if base == CHEB:
        for n in range(nr):
            for p in range(n + 2, nr, 2):
                r[n] += -2 * (p - n) * t[p]
        r[0] *= 0.5
        return CHEB, r
    if base in (CHEB_EVEN, CHEB_ODD):
        for n in range(nr):
            for p in range(n + 1, nr):
                r[n] += -4 * (p - n) * t[p]
        if base == CHEB_EVEN:
            r[0] *= 0.5
        return base, r
    raise ValueError(base)


OPE_1D = {OP_DER: der_1d, OP_MULT_SIN: mult_sin_1d, OP_DIV_SIN: div_sin_1d, OP_MULT_COS: mult_cos_1d,
          OP_DIV_COS: div_cos_1d, OP_MULT_X: mult_x_1d, OP_DIV_X: div_x_1d, OP_MULT_XM1: mult_xm1_1d,
          OP_DIV_XM1: div_xm1_1d, OP_DIV_XP1: div_xp1_1d, OP_DIV_1MX2: div_1mx2_1d}


def apply_1d(op: int, base: int, tab, n_out: int | None = None):
    """Applies one operator to a line; returns (out_basis, line)."""
    if op == OP_COEF:
        nin = len(tab)
        n = max(nin, n_out or nin)
        t = np.zeros(n)
        t[:nin] = tab
        return base, COEF_1D[base](t)[: (n_out or nin)]
    if op == OP_COEF_I:
        return base, COEF_I_1D[base](np.asarray(tab, dtype=float))[: (n_out or len(tab))]
    return OPE_1D[op](base, tab)


def matrix_1d(op: int, base: int, n_in: int, n_out: int | None = None):
    """Matrix (n_out x n_in) of a 1-D operator, column by column."""
    n_out = n_out or n_in
    m = np.zeros((n_out, n_in))
    ob = None
    for c in range(n_in):
        e = np.zeros(n_in)
        e[c] = 1.0
        ob, col = apply_1d(op, base, e, n_out)
        m[:, c] = col[:n_out]
    return ob, m


# -------------------------------------------------- 3-D separable drivers --
def coef_3d(values: np.ndarray, base_r, base_t, base_p, nbr_coefs):
    """Base_spectral::coef (src/Coef/coef.cpp:96): phi, then theta, then r.

    values: (n0, n1, n2) collocation block.  base_r: (nc1, nc2) ints;
    base_t: (nc2,) ints; base_p: int.
    """
    x = np.array(values, dtype=float)
    n0, n1, n2 = x.shape
    nc0, nc1, nc2 = nbr_coefs
    # phi (dim 2): the 1-D work line has max(n_conf, n_coef) slots
    y = np.zeros((n0, n1, nc2))
    for i in range(n0):
        for j in range(n1):
            t = np.zeros(max(n2, nc2))
            t[:n2] = x[i, j, :]
            y[i, j, :] = COEF_1D[base_p](t)[:nc2]
    # theta (dim 1): basis by phi-coefficient index k
    z = np.zeros((n0, nc1, nc2))
    for k in range(nc2):
        for i in range(n0):
            z[i, :, k] = COEF_1D[base_t[k]](y[i, :, k].copy())[:nc1]
    # r (dim 0): basis by (j, k)
    w = np.zeros((nc0, nc1, nc2))
    for j in range(nc1):
        for k in range(nc2):
            w[:, j, k] = COEF_1D[base_r[j][k]](z[:, j, k].copy())[:nc0]
    return w


def coef_i_3d(coefs: np.ndarray, base_r, base_t, base_p, nbr_points):
    """Base_spectral::coef_i (src/Coef/coef_i.cpp:96): r, then theta, then phi."""
    w = np.array(coefs, dtype=float)
    nc0, nc1, nc2 = w.shape
    n0, n1, n2 = nbr_points
    z = np.zeros((n0, nc1, nc2))
    for j in range(nc1):
        for k in range(nc2):
            z[:, j, k] = COEF_I_1D[base_r[j][k]](w[:, j, k].copy())[:n0]
    y = np.zeros((n0, n1, nc2))
    for k in range(nc2):
        for i in range(n0):
            y[i, :, k] = COEF_I_1D[base_t[k]](z[i, :, k].copy())[:n1]
    x = np.zeros((n0, n1, n2))
    for i in range(n0):
        for j in range(n1):
            x[i, j, :] = COEF_I_1D[base_p](y[i, j, :].copy())[:n2]
    return x


def ope_1d_3d(op, dim, coefs, base_r, base_t, base_p):
    """Base_spectral::ope_1d (src/Ope_1d/ope_1d.cpp:25) on a coefficient block.

    Returns (result, new basis table of `dim`)."""
    w = np.array(coefs, dtype=float)
    n0, n1, n2 = w.shape
    out = np.zeros_like(w)
    if dim == 0:
        nb = np.array(base_r).copy()
        for j in range(n1):
            for k in range(n2):
                nb[j][k], out[:, j, k] = apply_1d(op, base_r[j][k], w[:, j, k])
        return out, nb
    if dim == 1:
        nb = np.array(base_t).copy()
        for k in range(n2):
            for i in range(n0):
                nb[k], out[i, :, k] = apply_1d(op, base_t[k], w[i, :, k])
        return out, nb
    nb = base_p
    for i in range(n0):
        for j in range(n1):
            nb, out[i, j, :] = apply_1d(op, base_p, w[i, j, :])
    return out, nb
