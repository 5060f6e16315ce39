"""The oracle and the GPU path against the committed analytic known answers
of the reference's programs (tests/golden/known_answers.json, written by
tests/golden/make_known_answers.py)."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import configs, kadath as K

GOLD = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())


def solve(sysm, prec=1e-8, maxit=20):
    for _ in range(maxit):
        done, *_ = sysm.newton_step(prec)
        if done:
            return
    raise AssertionError("oracle Newton did not converge")


def test_oracle_tuto5_golden():
    g = GOLD["tuto5"]
    doms, sysm, F = configs.tuto5()
    solve(sysm)
    num = K.val_point(doms, F, tuple(g["point"]))
    assert abs(num - g["value"]) / abs(g["value"]) < 1e-8


def test_oracle_schwarz_golden():
    g = GOLD["schwarz"]
    doms, sysm, P = configs.schwarz(aa=g["aa"])
    solve(sysm)
    err = max(abs(K.val_point(doms, P, tuple(p)) - v) for p, v in zip(g["points"], g["values"]))
    assert err < g["max_error"]


@pytest.mark.gpu
def test_gpu_schwarz_golden(ctx):
    from kadath_frontera_gb300.kadath import CHEB_TYPE, Scalar, Space_spheric, System_of_eqs
    g = GOLD["schwarz"]
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), tuple(g["res"]), tuple(g["bounds"]))
    conf = Scalar(space, 1.0).std_base()
    syst = System_of_eqs(space, 1, 3)
    syst.add_var("P", conf)
    syst.add_cst("a", g["aa"])
    space.add_inner_bc(syst, "dn(P) + 0.5 / a * P = 0")
    space.add_eq(syst, "Lap(P) = 0", "P", "dn(P)")
    space.add_outer_bc(syst, "P=1")
    for _ in range(10):
        done, _ = syst.do_newton(1e-8)
        if done:
            break
    assert done
    doms = K.space_spheric(tuple(g["res"]), list(g["bounds"]))
    of = {d.num: K.VD(d, 1, cf=conf.get_coef(d.num)[None], base=d.std_base()) for d in doms}
    err = max(abs(K.val_point(doms, of, tuple(p)) - v) for p, v in zip(g["points"], g["values"]))
    assert err < g["max_error"]
