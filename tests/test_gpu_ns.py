"""GPU parity of the TOV star with the log-enthalpy as unknown: Eq_full
(add_eq_full), Eq_first_integral (add_eq_first_integral), the EOS operators,
exp/log and index-notation definitions, written with the strings of Kadath's
NS solver, against the oracle's restatement of the same system."""
import numpy as np
import pytest

from oracle import configs

pytestmark = pytest.mark.gpu

RES = (9, 5, 4)
REL = 1e-12


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_tov_residual_and_jacobian_match_oracle(ctx):
    from kadath_frontera_gb300 import workloads as W
    wl = W.ns_tov(RES, ctx=ctx)
    doms, osys, _, _ = configs.ns_tov(RES)
    F = wl.syst.sec_member()
    J = wl.syst.jacobian()
    Fo, Jo = osys.jacobian()
    assert F.shape == Fo.shape and J.shape == Jo.shape
    scale = np.abs(Jo).max()
    assert np.abs(F - Fo).max() <= 1e-13 * scale
    assert rel(J, Jo) < REL
    x = np.random.default_rng(5).standard_normal(J.shape[0])
    assert rel(wl.syst.do_JX(x), Jo @ x) < REL


def test_tov_newton_iterates_match_oracle(ctx):
    from kadath_frontera_gb300 import workloads as W
    wl = W.ns_tov(RES, ctx=ctx)
    doms, osys, ofields, _ = configs.ns_tov(RES)
    for it in range(12):
        done, err = wl.syst.do_newton(1e-11)
        odone, oerr, _, _ = osys.newton_step(1e-11)
        assert abs(err - oerr) <= 1e-10 * max(1.0, abs(oerr)) + 1e-14
        assert done == odone
        if done:
            break
    assert done
    for (_, f), of in zip(wl.unknowns, ofields):
        for d in range(len(doms)):
            a = f.get_coef(d).reshape(-1)
            v = of[d]
            if v.zero:
                assert np.abs(a).max() < 1e-12
                continue
            v.coef()
            b = v.cf.reshape(-1)
            assert np.abs(a - b).max() <= 1e-10 * max(1.0, np.abs(b).max())
    H = dict(wl.unknowns)["H"]
    assert abs(H.val_point((0.0, 0.0, 0.0)) - configs.ns_hc()) < 1e-10


def test_tov_mixed_precision_matches_fp64(ctx):
    """The mixed LU reaches the FP64 solution of the coupled system."""
    from kadath_frontera_gb300 import kadath as KK
    from kadath_frontera_gb300 import workloads as W
    res = (11, 7, 4)
    a = W.ns_tov(res, ctx=ctx)
    b = W.ns_tov(res, ctx=ctx)
    W.solve(a, 1e-10, lu_mode=KK.KD_LU_FP64)
    W.solve(b, 1e-10, lu_mode=KK.KD_LU_TF32_IR)
    for (_, f), (_, g) in zip(a.unknowns, b.unknowns):
        for d in range(a.space.get_nbr_domains()):
            x, y = f.get_coef(d), g.get_coef(d)
            assert np.abs(x - y).max() <= 1e-10 * max(1.0, np.abs(x).max())
