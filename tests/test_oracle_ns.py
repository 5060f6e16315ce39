"""The oracle's TOV star with the log-enthalpy as unknown (CPU): the
vectorised EOS against the point-by-point restatement, the first-integral
and Eq_full rows, and Newton's quadratic convergence to H = Hc at the
centre."""
import math

import numpy as np

from oracle import configs, kadath as K


def test_eos_array_matches_pointwise():
    rng = np.random.default_rng(0)
    for e in (K.polytrope(), K.polytrope(3, gamma_tab=(1.5, 2.5, 3.0), rho_tab=(0.0, 1e-4, 1e-3))):
        h = np.concatenate([np.linspace(0.9, 1.6, 701), [1.0, 1.0 + 1e-9]])
        dh = rng.standard_normal(h.shape)
        for var in range(4):
            a = np.array([K._eos_point(e, var, x) for x in h])
            b = K._eos_array(e, var, h)
            assert np.allclose(b, a, rtol=1e-14, atol=0.0)
            c = np.array([K._eos_point(e, var, x, y) for x, y in zip(h, dh)])
            d = K._eos_array(e, var, h, dh)
            assert np.allclose(d, c, rtol=1e-14, atol=0.0)


def test_first_integral_rows():
    """At the initial guess H = Hc, N = 1 the first integral H + log N is Hc
    everywhere and its value at the centre equals the constant part's: all
    first-integral rows vanish, while the Eq_full rows of H = 0 outside the
    matter vanish too."""
    doms, s, (H, P, N), _ = configs.ns_tov((7, 5, 4))
    F = s.residual()
    layout_rows = []
    r = 0
    for eq in s.eqs:
        if eq[0] == "first_integral":
            _, ns = s._first_integral(eq)
        else:
            _, ns = s._value_rows(eq[0], eq[3](s._terms(eq[1]), eq[2]), eq[1], eq[2])
        layout_rows.append((eq[0], r, sum(ns)))
        r += sum(ns)
    assert r == len(F)
    for kind, r0, n in layout_rows:
        if kind in ("first_integral", "order"):
            assert np.abs(F[r0:r0 + n]).max() < 1e-14
    # the system is square
    _, N_unk = s.unknown_layout()
    assert N_unk == len(F)


def test_tov_newton_converges():
    doms, s, (H, P, N), _ = configs.ns_tov((7, 5, 4))
    errs = []
    for it in range(12):
        done, err, F, J = s.newton_step(1e-11)
        errs.append(err)
        if done:
            break
    assert done
    # quadratic convergence at the end
    assert errs[-2] < 1e-6 and errs[-1] < 1e-11
    H[0].coef_i()
    assert abs(H[0].c[0, 0, 0, 0] - configs.ns_hc()) < 1e-12
    # N and P regular and bounded at the centre; H vanishes outside the matter
    N[0].coef_i()
    P[0].coef_i()
    assert 0.5 < N[0].c[0, 0, 0, 0] < 1.0 and 1.0 < P[0].c[0, 0, 0, 0] < 1.5
    for d in range(2, len(doms)):
        H[d].coef_i()
        assert H[d].zero or np.abs(H[d].c).max() < 1e-12
