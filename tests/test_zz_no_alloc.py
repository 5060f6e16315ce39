"""kd_coef_host_noalloc: the host-pointer forward transform for callers that
cannot let a library allocate GPU memory (an application that serves its whole
device budget from its own pool, or code between its steps where a cudaFree
would synchronise the device).  It must give the same coefficients as
kd_coef_host, call after call, while staging through the library's fixed
device arrays, and a call must leave the device's free memory unchanged.

This file is collected last on purpose (tests/test_zz_*), so that a run that
stops at the first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from tests.spectral_cases import std_base

pytestmark = pytest.mark.gpu

TOL = 1e-13  # normwise relative, the transform tests' tolerance


def _desc(kind, shape, batch, x, y, anti=False):
    from kadath_frontera_gb300._lib import TransformDesc
    nc = (shape[0], shape[1], shape[2] + 2)
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
    d.in_ = x.ctypes.data
    d.out = y.ctypes.data
    return d, (r, t)


def _run(ctx, fn, kind, shape, batch, x, anti=False):
    nc = (shape[0], shape[1], shape[2] + 2)
    y = np.zeros((batch,) + nc)
    d, keep = _desc(kind, shape, batch, x, y, anti)
    ctx.check(fn(ctx.h, C.byref(d)))
    return y


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_noalloc_matches_allocating_entry_point_twice(ctx):
    lib = ctx.lib
    lib.kd_coef_host_noalloc.restype = C.c_int
    lib.kd_coef_host_noalloc.argtypes = lib.kd_coef_host.argtypes
    rng = np.random.default_rng(11)
    cases = [("nucleus", (13, 9, 4), 5, False), ("shell", (11, 9, 8), 3, True)]
    for kind, shape, batch, anti in cases:  # two calls in a row, different shapes
        x = rng.standard_normal((batch,) + shape)
        ref = _run(ctx, lib.kd_coef_host, kind, shape, batch, x, anti)
        got = _run(ctx, lib.kd_coef_host_noalloc, kind, shape, batch, x, anti)
        assert _rel(got, ref) < TOL, (kind, _rel(got, ref))


def test_noalloc_rejects_sizes_beyond_its_arrays(ctx):
    lib = ctx.lib
    lib.kd_coef_host_noalloc.restype = C.c_int
    lib.kd_coef_host_noalloc.argtypes = lib.kd_coef_host.argtypes
    shape = (13, 9, 4)
    per_field = 13 * 9 * 6
    batch = (1 << 20) // per_field + 1  # one field more than the staging array holds
    x = np.zeros((1,) + shape)  # never read: the call is rejected before any copy
    y = np.zeros((1, 13, 9, 6))
    d, keep = _desc("shell", shape, 1, x, y)
    d.batch = batch
    st = lib.kd_coef_host_noalloc(ctx.h, C.byref(d))
    assert st == 1  # KD_ERR_ARG
    assert b"KD_NOALLOC_MAX_DOUBLES" in lib.kd_last_error(ctx.h)


def _declare(lib):
    lib.kd_coef_host_noalloc.restype = C.c_int
    lib.kd_coef_host_noalloc.argtypes = lib.kd_coef_host.argtypes


def test_noalloc_first_call_on_a_fresh_context(ctx):
    """The very first transform of a new context goes through the no-alloc
    entry point, with a basis and size nothing has used before: its matrices
    enter the context's pool during that call."""
    from kadath_frontera_gb300._lib import Context
    _declare(ctx.lib)
    fresh = Context(0)
    rng = np.random.default_rng(23)
    shape = (15, 11, 6)
    x = rng.standard_normal((2,) + shape)
    got = _run(fresh, fresh.lib.kd_coef_host_noalloc, "compact", shape, 2, x, True)
    ref = _run(fresh, fresh.lib.kd_coef_host, "compact", shape, 2, x, True)
    assert _rel(got, ref) < TOL
    again = _run(fresh, fresh.lib.kd_coef_host_noalloc, "compact", shape, 2, x, True)
    assert np.array_equal(again, got)


def test_noalloc_call_leaves_device_memory_unchanged(ctx):
    """After a first call of each launch form (few fields: the cluster kernel;
    many fields: the plain kernel), a call with a new shape and basis takes no
    device memory."""
    import torch
    _declare(ctx.lib)
    rng = np.random.default_rng(29)
    for kind, shape, batch in (("shell", (9, 5, 4), 1), ("shell", (9, 5, 4), 300)):
        x = rng.standard_normal((batch,) + shape)
        _run(ctx, ctx.lib.kd_coef_host_noalloc, kind, shape, batch, x)
    torch.cuda.synchronize()
    shape, batch = (17, 13, 8), 3
    x = rng.standard_normal((batch,) + shape)
    free_before, _ = torch.cuda.mem_get_info()
    got = _run(ctx, ctx.lib.kd_coef_host_noalloc, "nucleus", shape, batch, x, True)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before, (free_before, free_after)
    ref = _run(ctx, ctx.lib.kd_coef_host, "nucleus", shape, batch, x, True)
    assert _rel(got, ref) < TOL
