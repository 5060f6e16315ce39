"""Pins the oracle to the reference's own outputs.

The fixtures tests/golden/ref_*.npz were produced by the reference's sources
compiled here (oracle/Makefile.ref) and run through the drivers in
oracle/ref_drivers/ (tests/golden/make_ref_vectors.py): the 1-D transforms
and operators of src/Coef and src/Ope_1d, Base_spectral::coef/coef_i, and
sec_member / do_col_J / do_JX / do_newton_seq of the toy configuration and
of the isolated star.  The numpy oracle must reproduce them."""
from pathlib import Path

import numpy as np
import pytest

from oracle import configs as CF
from oracle import kadath as K
from oracle import spectral as S

GOLD = Path(__file__).resolve().parent / "golden"


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


def test_spectral_1d_matrices_match_the_reference():
    z = np.load(GOLD / "ref_spectral_1d.npz")
    keys = [k for k in z.files if not k.endswith("_base")]
    assert len(keys) > 300
    worst = 0.0
    for key in keys:
        op, base, nin, nout = (int(t[1:] if t[0] in "bnm" else t[2:]) for t in key.split("_"))
        ob, m = S.matrix_1d(op, base, nin, nout)
        ref = z[key]
        scale = max(np.abs(ref).max(), 1.0)
        err = np.abs(m - ref).max() / scale
        worst = max(worst, err)
        assert err < 1e-13, (key, err)
        if op not in (S.OP_COEF, S.OP_COEF_I):
            assert ob == int(z[key + "_base"]), key
    print("worst 1-D difference", worst)


def _domain_base(d, kind):
    b = d.std_base()
    if kind in ("anti", "zcart"):
        return CF._anti(d)
    return b


@pytest.mark.parametrize("kind", ["std", "anti", "xcart", "ycart", "zcart"])
def test_coef_3d_matches_the_reference(kind):
    z = np.load(GOLD / "ref_coef3d.npz")
    doms = K.space_spheric(tuple(z["res"]), list(z["bounds"]))
    x, c = z[f"values_{kind}"], z[f"coefs_in_{kind}"]
    cf_ref, v_ref = z[f"coef_{kind}"], z[f"coef_i_{kind}"]
    ip = ic = 0
    for d in doms:
        b = _domain_base(d, kind)
        npt, ncf = int(np.prod(d.np)), int(np.prod(d.nc))
        got = S.coef_3d(x[ip:ip + npt].reshape(d.np), b.r, b.t, b.p, d.nc)
        assert _rel(got, cf_ref[ic:ic + ncf]) < 1e-13, (kind, d.num)
        back = S.coef_i_3d(c[ic:ic + ncf].reshape(d.nc), b.r, b.t, b.p, d.np)
        assert _rel(back, v_ref[ip:ip + npt]) < 1e-13, (kind, d.num)
        ip += npt
        ic += ncf


def field_coefs(fields, doms):
    """Coefficients in the order the reference driver dumps them: field by
    field (vector components in turn), domain by domain."""
    out = []
    for f in fields:
        for d in doms:
            v = f[d.num]
            if v.zero:
                out.append(np.zeros(int(np.prod(d.nc))))
                continue
            v.coef()
            out.append(np.asarray(v.cf).ravel())
    return np.concatenate(out)


def _check_system(sysm, fields, doms, z, newton=True):
    F, J = sysm.jacobian()
    scale = np.abs(J).max()
    assert len(F) == len(z["F0"])
    assert np.abs(F - z["F0"]).max() < 1e-13 * scale
    if "cols" in z.files:
        for k, c in enumerate(z["cols"]):
            assert np.abs(J[:, c] - z["J_cols"][k]).max() < 1e-13 * scale, c
        assert _rel(J @ z["x"], z["Jx"]) < 1e-12
    if not newton:
        return
    errs = z["errors"]
    for k in range(len(errs)):
        done, err, _, _ = sysm.newton_step(1e-10)
        if k < len(errs) - 1:
            assert not done
            # max|F| carries the residual's round-off (~1e-12 absolute here)
            assert abs(err - errs[k]) <= 1e-9 * errs[k] + 1e-11, (k, err, errs[k])
            got = field_coefs(fields, doms)
            ref = z["iterates"][k]
            assert _rel(got, ref) < 1e-12, (k, _rel(got, ref))
        else:
            assert done and err < 1e-10


def test_toy_newton_matches_the_reference_do_newton_seq():
    z = np.load(GOLD / "ref_toy.npz")
    doms, sysm, psi, rho = CF.toy(tuple(z["res"]))
    got_rho = np.concatenate([np.asarray(rho[d.num].c).ravel() for d in doms])
    assert np.array_equal(got_rho, z["rho"])
    _check_system(sysm, [psi], doms, z)


@pytest.mark.parametrize("name", ["ref_star_954.npz"])
def test_vector_star_matches_the_reference(name):
    z = np.load(GOLD / name)
    doms, sysm, (P, NP, bx, by, bz), (E, E2S) = _star_vector(tuple(z["res"]))
    got_E = np.concatenate([np.asarray(E[d.num].c).ravel() for d in doms])
    assert np.array_equal(got_E, z["E"])
    _check_system(sysm, [P, NP, bx, by, bz], doms, z)


def _star_vector(res):
    doms, sysm, fields, matter = CF.star_vector(res)
    return doms, sysm, fields, matter


def test_star_residual_at_the_timed_size_matches_the_reference():
    """The isolated star at (13, 9, 4), N = 12,331: the oracle's residual at
    the initial guess against the reference's sec_member (the iterates at this
    size are compared on the GPU, tests/test_gpu_ref_pinned.py)."""
    z = np.load(GOLD / "ref_star_1394.npz")
    doms, sysm, _, (E, E2S) = _star_vector(tuple(z["res"]))
    got_E = np.concatenate([np.asarray(E[d.num].c).ravel() for d in doms])
    assert np.array_equal(got_E, z["E"])
    F = sysm.residual()
    assert len(F) == len(z["F0"]) == 12331
    # absolute round-off of the residual (about 1e-14 here, amplified by the
    # spectral second derivatives); the other tests compare at 1e-13 max|J|
    # and max|J| is far above 1 at this resolution
    assert np.abs(F - z["F0"]).max() < 1e-13


def test_trig_atanh_ddr_match_the_reference():
    """cos/sin/cosh/sinh of a number, atanh of the field and ddr in the toy
    system (tests/golden/ref_funcs.npz, made by the reference): F, Jacobian
    columns, J x and every Newton iterate."""
    import math
    z = np.load(GOLD / "ref_funcs.npz")
    res = tuple(int(v) for v in z["res"])
    amp = float(z["cst_amp"])
    doms = K.space_spheric(res, [1.0, 2.0])
    nd = len(doms)
    psi = K.scalar_field(doms, lambda d: np.ones(d.np))
    rho = K.scalar_field(doms, CF.toy_rho)
    got_rho = np.concatenate([np.asarray(rho[d.num].c).ravel() for d in doms])
    assert np.array_equal(got_rho, z["rho"])
    sysm = K.OSystem(doms, 0, nd - 1)
    sysm.add_var("psi", psi)
    for d in range(nd):
        rh = rho[d]

        # Lap(psi) + 2*pi*rho*psi^5*cos(amp) + rho*atanh(psi/4)*sinh(amp)
        #   + 0.01*sin(amp)*cosh(amp)*ddr(psi), in the parser's order
        def eq(T, b, rh=rh):
            p = T["psi"]
            zero = None if p.der is None else K.VD.zeros(rh.dom, p.der.B)
            rho_t = K.OTerm(p.dom, rh, zero)
            c = K.OTerm(p.dom, 2 * math.pi, None if p.der is None else 0.0)
            t1 = ((c * rho_t) * p ** 5) * math.cos(amp)
            t2 = (rho_t * (p / 4.0).atanh()) * math.sinh(amp)
            t3 = ((0.01 * math.sin(amp)) * math.cosh(amp)) * p.ddr()
            return ((p.lap() + t1) + t2) + t3
        sysm.add_eq_inside(d, eq)
    for d in range(nd - 1):
        sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b: T["psi"])
        sysm.add_eq_matching(d, K.OUTER_BC, lambda T, b: T["psi"].dn(b))
    sysm.add_eq_bc(nd - 1, K.OUTER_BC, lambda T, b: T["psi"] - 1.0)
    _check_system(sysm, [psi], doms, z)


@pytest.mark.parametrize("case", ["bispheric_std", "bispheric_anti", "cossin_even", "cossin_odd"])
def test_coef_3d_with_bispheric_and_cossin_parity_bases_matches_the_reference(case):
    """Base_spectral::coef / coef_i with the bispheric domains' bases and the
    COSSIN_EVEN / COSSIN_ODD phi bases (tests/golden/ref_coef3_bases.npz)."""
    z = np.load(GOLD / "ref_coef3_bases.npz")
    np_, nc = tuple(int(v) for v in z[f"{case}_np"]), tuple(int(v) for v in z[f"{case}_nc"])
    br, bt, bp = np.asarray(z[f"{case}_br"]), np.asarray(z[f"{case}_bt"]), int(z[f"{case}_bp"])
    got = S.coef_3d(z[f"{case}_values"].reshape(np_), br, bt, bp, nc)
    assert _rel(got, z[f"{case}_coef"]) < 1e-13
    back = S.coef_i_3d(z[f"{case}_coefs_in"].reshape(nc), br, bt, bp, np_)
    assert _rel(back, z[f"{case}_coef_i"]) < 1e-13
