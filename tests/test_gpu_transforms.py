"""GPU parity of the batched 3-D transforms and of ope_1d against the oracle
(src/Coef/coef.cpp, src/Coef/coef_i.cpp, src/Ope_1d/ope_1d.cpp)."""
import ctypes as C

import numpy as np
import pytest

from oracle import spectral as S
from tests.spectral_cases import SHAPES, std_base

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu
TOL = 1e-13  # normwise relative, FP64 on both sides


def desc_for(kind, shape, batch, din, dout, anti=False):
    from kadath_frontera_gb300._lib import TransformDesc
    n0, n1, n2 = shape
    nc = (n0, n1, n2 + 2)
    br, bt, bp = std_base(kind, nc[1], nc[2], anti)
    r = (C.c_int * (nc[1] * nc[2]))(*[b for row in br for b in row])
    t = (C.c_int * nc[2])(*bt)
    d = TransformDesc()
    d.nbr_points[:] = shape
    d.nbr_coefs[:] = nc
    d.base_r = C.cast(r, C.POINTER(C.c_int))
    d.base_t = C.cast(t, C.POINTER(C.c_int))
    d.base_p = bp
    d.batch = batch
    d.in_ = din.data_ptr()
    d.out = dout.data_ptr()
    return d, (r, t), (br, bt, bp)


def relerr(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("kind,shape", SHAPES)
@pytest.mark.parametrize("anti", [False, True])
def test_coef_and_coef_i_match_oracle(ctx, kind, shape, anti):
    rng = np.random.default_rng(hash((kind, shape, anti)) % 2**32)
    batch = 3
    n0, n1, n2 = shape
    nc = (n0, n1, n2 + 2)
    x = rng.standard_normal((batch,) + shape)
    xd = torch.tensor(x, device="cuda", dtype=torch.float64)
    yd = torch.zeros((batch,) + nc, device="cuda", dtype=torch.float64)
    d, keep, (br, bt, bp) = desc_for(kind, shape, batch, xd, yd, anti)
    ctx.check(ctx.lib.kd_coef_many(ctx.h, 1, C.byref(d)))
    ctx.synchronize()
    y = yd.cpu().numpy()
    for b in range(batch):
        ref = S.coef_3d(x[b], br, bt, bp, nc)
        assert relerr(y[b], ref) < TOL
    # inverse on the oracle's coefficients
    cd = torch.tensor(y, device="cuda")
    zd = torch.zeros((batch,) + shape, device="cuda", dtype=torch.float64)
    d2, keep2, _ = desc_for(kind, shape, batch, cd, zd, anti)
    ctx.check(ctx.lib.kd_coef_i_many(ctx.h, 1, C.byref(d2)))
    ctx.synchronize()
    z = zd.cpu().numpy()
    for b in range(batch):
        ref = S.coef_i_3d(y[b], br, bt, bp, shape)
        assert relerr(z[b], ref) < TOL


def test_packed_uneven_domains_one_launch(ctx):
    """Fields of all config domains (uneven shapes) in a single launch."""
    from kadath_frontera_gb300._lib import TransformDesc
    rng = np.random.default_rng(7)
    descs, keeps, refs, outs = [], [], [], []
    for kind, shape in SHAPES:
        nc = (shape[0], shape[1], shape[2] + 2)
        x = rng.standard_normal((2,) + shape)
        xd = torch.tensor(x, device="cuda")
        yd = torch.zeros((2,) + nc, device="cuda", dtype=torch.float64)
        d, keep, (br, bt, bp) = desc_for(kind, shape, 2, xd, yd)
        descs.append(d)
        keeps.append((keep, xd))
        outs.append(yd)
        refs.append([S.coef_3d(x[b], br, bt, bp, nc) for b in range(2)])
    arr = (TransformDesc * len(descs))(*descs)
    before = ctx.launches
    ctx.check(ctx.lib.kd_coef_many(ctx.h, len(descs), arr))
    ctx.synchronize()
    assert ctx.launches - before == 1
    for yd, rr in zip(outs, refs):
        y = yd.cpu().numpy()
        for b in range(2):
            assert relerr(y[b], rr[b]) < TOL


@pytest.mark.parametrize("op,dim,kind", [(S.OP_DER, 0, "shell"), (S.OP_DER, 0, "nucleus"), (S.OP_DER, 1, "shell"),
                                         (S.OP_DER, 2, "shell"), (S.OP_MULT_SIN, 1, "shell"),
                                         (S.OP_DIV_SIN, 1, "nucleus"), (S.OP_MULT_COS, 2, "shell"),
                                         (S.OP_MULT_SIN, 2, "compact"), (S.OP_DIV_X, 0, "nucleus"),
                                         (S.OP_MULT_XM1, 0, "compact"), (S.OP_DIV_XM1, 0, "compact")])
def test_ope_1d_matches_oracle(ctx, op, dim, kind):
    shape = (13, 7, 4)
    nc = (13, 7, 6)
    rng = np.random.default_rng(op * 10 + dim)
    w = rng.standard_normal((2,) + nc)
    wd = torch.tensor(w, device="cuda")
    od = torch.zeros_like(wd)
    d, keep, (br, bt, bp) = desc_for(kind, shape, 2, wd, od)
    rout = (C.c_int * (nc[1] * nc[2]))()
    tout = (C.c_int * nc[2])()
    pout = C.c_int()
    ctx.check(ctx.lib.kd_ope_1d(ctx.h, op, dim, C.byref(d), rout, tout, C.byref(pout)))
    ctx.synchronize()
    o = od.cpu().numpy()
    for b in range(2):
        ref, nb = S.ope_1d_3d(op, dim, w[b], br, bt, bp)
        assert relerr(o[b], ref) < TOL
    if dim == 0:
        assert list(rout) == [int(v) for row in nb for v in row]
    elif dim == 1:
        assert list(tout) == [int(v) for v in nb]
    else:
        assert pout.value == nb


def test_host_pointer_transform(ctx):
    from kadath_frontera_gb300._lib import TransformDesc
    shape = (13, 7, 4)
    nc = (13, 7, 6)
    rng = np.random.default_rng(3)
    x = rng.standard_normal(shape)
    y = np.zeros(nc)
    br, bt, bp = std_base("shell", nc[1], nc[2])
    r = (C.c_int * (nc[1] * nc[2]))(*[b for row in br for b in row])
    t = (C.c_int * nc[2])(*bt)
    d = TransformDesc()
    d.nbr_points[:] = shape
    d.nbr_coefs[:] = nc
    d.base_r = C.cast(r, C.POINTER(C.c_int))
    d.base_t = C.cast(t, C.POINTER(C.c_int))
    d.base_p = bp
    d.batch = 1
    d.in_ = x.ctypes.data
    d.out = y.ctypes.data
    ctx.check(ctx.lib.kd_coef_host(ctx.h, C.byref(d)))
    assert relerr(y, S.coef_3d(x, br, bt, bp, nc)) < TOL
