"""Pins the system-level oracle on the reference's known-answer programs
(tutorials/tuto5.cpp, codes/Seq_version/schwarz.cpp) and checks its
Jacobian against finite differences of its residual."""
import math

import numpy as np
import pytest

from oracle import configs, kadath as K


def solve(sysm, prec=1e-8, maxit=20):
    for it in range(maxit):
        done, err, F, J = sysm.newton_step(prec)
        if done:
            return it, err
    raise AssertionError("oracle Newton did not converge")


def test_tuto5_known_answer():
    doms, sysm, F = configs.tuto5()
    it, err = solve(sysm)
    assert it == 1  # linear problem: one update, converged at the second call
    num = K.val_point(doms, F, configs.TUTO_POINT)
    rr = math.sqrt(sum(c * c for c in configs.TUTO_POINT))
    ana = 1 + 1.0 / rr
    assert abs(num - ana) / abs(num) < 1e-8


def test_schwarz_known_answer():
    aa = 1.323
    doms, sysm, P = configs.schwarz(aa=aa)
    solve(sysm)
    # schwarz.cpp:66-86: 100 points on a ray in the equatorial plane
    resol, tet, phi = 100, math.pi / 2., -2.349
    xxmin, xxmax = aa * 1.01, 2.9861 * aa * 5
    step = (xxmax - xxmin) / resol
    xx = xxmin + step
    err_max = 0.0
    for _ in range(resol - 1):
        M = (xx * math.sin(tet) * math.cos(phi), xx * math.sin(tet) * math.sin(phi), xx * math.cos(tet))
        err_max = max(err_max, abs(1. + aa / xx - K.val_point(doms, P, M)))
        xx += step
    assert err_max < 1e-8


def test_toy_jacobian_matches_finite_differences():
    doms, sysm, psi, rho = configs.toy(res=(9, 5, 4))
    F0, J = sysm.jacobian()
    layout, N = sysm.unknown_layout()
    rng = np.random.default_rng(0)
    x = rng.standard_normal(N) * 1e-6
    # F(u - x) ~ F(u) - J x
    import copy
    saved = {d: (psi[d].c, psi[d].cf, psi[d].base) for d in psi}
    sysm.update(x)
    F1 = sysm.residual()
    for d, (c, cf, b) in saved.items():
        psi[d] = K.VD(doms[d], 1, c=c, cf=cf, base=b)
    lin = F0 - J @ x
    assert np.linalg.norm(F1 - lin) < 1e-3 * np.linalg.norm(J @ x)


def test_toy_newton_converges():
    doms, sysm, psi, rho = configs.toy()
    errs = []
    for it in range(10):
        done, err, F, J = sysm.newton_step(1e-10)
        errs.append(err)
        if done:
            break
    assert done, errs
    assert errs[-1] < 1e-10
    assert len(F) == J.shape[0] == J.shape[1]
