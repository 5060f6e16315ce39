"""The CUDA path against vectors produced by the reference's own code.

tests/golden/ref_*.npz hold what the reference's sources, compiled here
against stand-ins for FFTW/LAPACK/GSL/MPI (oracle/Makefile.ref), compute for
Base_spectral::coef/coef_i (src/Coef/coef.cpp:96, coef_i.cpp:96),
sec_member / do_col_J / do_JX (src/System_of_eqs/solver.cpp:49-214) and
do_newton_seq (src_par/do_newton.cpp:519-572).  These tests feed the product
the same inputs through its C ABI and compare:

* coefficients and collocation values at 1e-13 (normwise relative);
* the residual at 1e-13 of max|J|, Jacobian columns at 1e-13 of max|J|,
  J x at 1e-12;
* every Newton iterate at 1e-10 relative (the bound the converged fields must
  meet), with the FP64 LU and with the mixed-precision LU;
* at the isolated star's timed size, (13, 9, 4) with N = 12,331, every
  iterate of the component-form star (the benchmark's workload) and of the
  index-notation star, and the mixed-LU fields against the FP64-LU fields."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from tests.spectral_cases import std_base

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
TOL_T = 1e-13     # transforms, normwise relative
FIELD = 1e-10     # Newton iterates and converged fields, relative


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


def split(flat, shapes):
    out, at = [], 0
    for sh in shapes:
        n = int(np.prod(sh))
        out.append(np.asarray(flat[at:at + n]).reshape(sh))
        at += n
    assert at == len(flat)
    return out


def _shapes(space):
    nd = space.get_nbr_domains()
    info = [space.domain_info(d) for d in range(nd)]
    return [tuple(i["nbr_points"]) for i in info], [tuple(i["nbr_coefs"]) for i in info], info


@pytest.mark.parametrize("kind", ["std", "anti", "xcart", "ycart", "zcart"])
def test_transforms_match_the_reference(ctx, kind):
    from kadath_frontera_gb300._lib import TransformDesc
    from kadath_frontera_gb300.kadath import CHEB_TYPE, Space_spheric
    z = np.load(GOLD / "ref_coef3d.npz")
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), tuple(int(v) for v in z["res"]), list(z["bounds"]))
    pts, cfs, info = _shapes(space)
    kinds = {1: "nucleus", 2: "shell", 3: "compact"}
    xs = split(z[f"values_{kind}"], pts)
    cs = split(z[f"coefs_in_{kind}"], cfs)
    ref_cf = split(z[f"coef_{kind}"], cfs)
    ref_v = split(z[f"coef_i_{kind}"], pts)
    anti = kind in ("anti", "zcart")
    for d in range(len(pts)):
        br, bt, bp = std_base(kinds[info[d]["type"]], cfs[d][1], cfs[d][2], anti)
        r = (C.c_int * (cfs[d][1] * cfs[d][2]))(*[b for row in br for b in row])
        t = (C.c_int * cfs[d][2])(*bt)
        for fn, src, n_out, ref in ((ctx.lib.kd_coef_host, xs[d], cfs[d], ref_cf[d]),
                                    (ctx.lib.kd_coef_i_host, cs[d], pts[d], ref_v[d])):
            x = np.ascontiguousarray(src, dtype=np.float64)
            y = np.zeros(n_out)
            desc = TransformDesc()
            desc.nbr_points[:] = pts[d]
            desc.nbr_coefs[:] = cfs[d]
            desc.base_r = C.cast(r, C.POINTER(C.c_int))
            desc.base_t = C.cast(t, C.POINTER(C.c_int))
            desc.base_p = bp
            desc.batch = 1
            desc.in_ = x.ctypes.data
            desc.out = y.ctypes.data
            ctx.check(fn(ctx.h, C.byref(desc)))
            assert rel(y, ref) < TOL_T, (kind, d, fn.__name__, rel(y, ref))


def field_coefs(fields, nd):
    return np.concatenate([f.get_coef(d).ravel() for f in fields for d in range(nd)])


def check_system(wl, z, lu_mode):
    syst = wl.syst
    nd = wl.space.get_nbr_domains()
    fields = [f for _, f in wl.unknowns]
    if "cols" in z.files:
        F = syst.sec_member()
        J = syst.jacobian()
        scale = np.abs(J).max()
        assert np.abs(F - z["F0"]).max() <= 1e-13 * scale
        for k, c in enumerate(z["cols"]):
            assert np.abs(J[:, c] - z["J_cols"][k]).max() <= 1e-13 * scale, c
        assert rel(J @ z["x"], z["Jx"]) < 1e-12
        assert rel(syst.do_JX(z["x"]), z["Jx"]) < 1e-12
    errs = z["errors"]
    worst = 0.0
    for k in range(len(errs)):
        done, err = syst.do_newton(1e-10, lu_mode=lu_mode)
        if k < len(errs) - 1:
            assert not done, k
            assert abs(err - errs[k]) <= 1e-9 * errs[k] + 1e-11, (k, err, errs[k])
            e = rel(field_coefs(fields, nd), z["iterates"][k])
            worst = max(worst, e)
            assert e < FIELD, (k, e)
        else:
            assert done and err < 1e-10
    return worst


def _lu(mode):
    from kadath_frontera_gb300 import kadath as KD
    return {"fp64": KD.KD_LU_FP64, "mixed": KD.KD_LU_TF32_IR}[mode]


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_toy_matches_the_reference_newton(ctx, mode):
    from kadath_frontera_gb300 import workloads
    z = np.load(GOLD / "ref_toy.npz")
    from kadath_frontera_gb300.kadath import CHEB_TYPE, Space_spheric
    res = tuple(int(v) for v in z["res"])
    pts, _, _ = _shapes(Space_spheric(CHEB_TYPE, (0, 0, 0), res, (1.0, 2.0)))
    wl = workloads.toy(res, rho_values=split(z["rho"], pts))
    check_system(wl, z, _lu(mode))


def _star(form, z):
    from kadath_frontera_gb300 import workloads
    res = tuple(int(v) for v in z["res"])
    build = workloads.star if form == "components" else workloads.star_vector
    from kadath_frontera_gb300.kadath import CHEB_TYPE, Space_spheric
    pts, _, _ = _shapes(Space_spheric(CHEB_TYPE, (0, 0, 0), res, workloads.STAR_BOUNDS))
    return build(res, matter=(split(z["E"], pts), split(z["E2S"], pts)))


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_vector_star_954_matches_the_reference(ctx, mode):
    z = np.load(GOLD / "ref_star_954.npz")
    check_system(_star("vector", z), z, _lu(mode))


def test_component_star_954_matches_the_reference_iterates(ctx):
    # the component form orders rows and columns differently, so only the
    # iterates (fields) are compared
    z = np.load(GOLD / "ref_star_954.npz")
    zz = {k: z[k] for k in ("errors", "iterates")}
    check_system(_star("components", z), _NoCols(zz), _lu("mixed"))


class _NoCols(dict):
    @property
    def files(self):
        return list(self.keys())


@pytest.mark.parametrize("form", ["components", "vector"])
def test_timed_star_1394_matches_the_reference(ctx, form):
    """The benchmark's configuration, N = 12,331: every Newton iterate of the
    mixed-precision path and of the FP64-LU path against the reference's
    do_newton_seq, and the two paths' converged fields against each other."""
    z = np.load(GOLD / "ref_star_1394.npz")
    zz = _NoCols({k: z[k] for k in ("errors", "iterates")})
    wl64 = _star(form, z)
    w64 = check_system(wl64, zz, _lu("fp64"))
    wlmx = _star(form, z)
    wmx = check_system(wlmx, zz, _lu("mixed"))
    nd = wl64.space.get_nbr_domains()
    f64 = field_coefs([f for _, f in wl64.unknowns], nd)
    fmx = field_coefs([f for _, f in wlmx.unknowns], nd)
    diff = rel(fmx, f64)
    print(f"{form}: worst iterate vs reference fp64 {w64:.2e} mixed {wmx:.2e}; mixed vs fp64 {diff:.2e}")
    assert diff < FIELD


def _funcs_system(z):
    """The toy system with cos, sin, cosh, sinh of a double constant, atanh of
    the field and ddr, as tests/golden/make_ref_vectors.py gives it to the
    reference."""
    import math
    from types import SimpleNamespace
    from kadath_frontera_gb300.kadath import CHEB_TYPE, OUTER_BC, Scalar, Space_spheric, System_of_eqs
    res = tuple(int(v) for v in z["res"])
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), res, (1.0, 2.0))
    pts, _, _ = _shapes(space)
    nd = space.get_nbr_domains()
    psi = Scalar(space, 1.0).std_base()
    rho = Scalar(space)
    for d, v in enumerate(split(z["rho"], pts)):
        rho.set_domain(d, v)
    rho.std_base()
    syst = System_of_eqs(space, 0, nd - 1)
    syst.add_var("psi", psi)
    syst.add_cst("rho", rho)
    syst.add_cst("pi", math.pi)
    syst.add_cst("amp", float(z["cst_amp"]))
    for d in range(nd):
        syst.add_eq_inside(d, str(z["equation"]))
    for d in range(nd - 1):
        syst.add_eq_matching(d, OUTER_BC, "psi")
        syst.add_eq_matching(d, OUTER_BC, "dn(psi)")
    syst.add_eq_bc(nd - 1, OUTER_BC, "psi = 1")
    return SimpleNamespace(space=space, syst=syst, unknowns=[("psi", psi)])


@pytest.mark.parametrize("fixture", ["ref_funcs.npz", "ref_funcs2.npz"])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_more_operators_match_the_reference(ctx, mode, fixture):
    """cos/sin/cosh/sinh of a number, atanh of a field and ddr (Ope_cos,
    Ope_sin, Ope_cosh, Ope_sinh, Ope_atanh, Ope_ddr); lap2, multrsint and
    divrsint (Ope_lap2, Ope_mult_rsint, Ope_div_rsint): F, Jacobian columns,
    J x and every Newton iterate against the reference's own."""
    z = np.load(GOLD / fixture)
    check_system(_funcs_system(z), z, _lu(mode))


def test_trig_of_a_field_has_no_basis(ctx):
    """cos of a field gives values without a basis (Val_domain cos,
    src/Val_domain/val_domain_math.cpp:75): an equation that needs their
    coefficients is refused with KD_ERR_STATE, where the reference stops."""
    from kadath_frontera_gb300 import KadathError
    from kadath_frontera_gb300._lib import KD_ERR_STATE
    z = dict(np.load(GOLD / "ref_funcs.npz"))
    z["equation"] = np.array("Lap(psi) + rho*cos(psi) = 0")
    wl = _funcs_system(z)
    with pytest.raises(KadathError) as e:
        wl.syst.do_newton(1e-10)
    assert e.value.status == KD_ERR_STATE


@pytest.mark.parametrize("case", ["bispheric_std", "bispheric_anti", "cossin_even", "cossin_odd"])
def test_transforms_with_bispheric_and_cossin_parity_bases_match_the_reference(ctx, case):
    """The GPU line passes with the bispheric domains' bases (COS / SIN in
    phi, CHEB_EVEN / CHEB_ODD in chi, CHEB in eta) and with the COSSIN_EVEN /
    COSSIN_ODD phi bases, against Base_spectral::coef / coef_i of the
    reference (tests/golden/ref_coef3_bases.npz)."""
    from kadath_frontera_gb300._lib import TransformDesc
    z = np.load(GOLD / "ref_coef3_bases.npz")
    np_, nc = [int(v) for v in z[f"{case}_np"]], [int(v) for v in z[f"{case}_nc"]]
    br, bt, bp = np.asarray(z[f"{case}_br"]), [int(v) for v in z[f"{case}_bt"]], int(z[f"{case}_bp"])
    r = (C.c_int * (nc[1] * nc[2]))(*[int(br[j][k]) for j in range(nc[1]) for k in range(nc[2])])
    t = (C.c_int * nc[2])(*bt)
    for fn, src, n_out, ref in ((ctx.lib.kd_coef_host, z[f"{case}_values"], nc, z[f"{case}_coef"]),
                                (ctx.lib.kd_coef_i_host, z[f"{case}_coefs_in"], np_, z[f"{case}_coef_i"])):
        x = np.ascontiguousarray(src, dtype=np.float64)
        y = np.zeros(int(np.prod(n_out)))
        desc = TransformDesc()
        desc.nbr_points[:] = np_
        desc.nbr_coefs[:] = nc
        desc.base_r = C.cast(r, C.POINTER(C.c_int))
        desc.base_t = C.cast(t, C.POINTER(C.c_int))
        desc.base_p = bp
        desc.batch = 1
        desc.in_ = x.ctypes.data
        desc.out = y.ctypes.data
        ctx.check(fn(ctx.h, C.byref(desc)))
        assert rel(y, ref) < TOL_T, (case, fn.__name__, rel(y, ref))
