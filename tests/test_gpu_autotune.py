"""The autotuner of the line passes' launch shapes: a solve with shape
classes timed as they are met (mode 2) writes a JSON table; a new context
reading the table (mode 1) uses its entries; and every shape gives the fields
of the fixed rule to the bit (each output value is summed in the same
order whatever the shape)."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solve(ctx, res=(9, 5, 4)):
    from kadath_frontera_gb300 import workloads as W
    from kadath_frontera_gb300.kadath import KD_LU_TF32_IR
    wl = W.star(res, ctx=ctx)
    W.solve(wl, lu_mode=KD_LU_TF32_IR)
    return wl.download()


def test_tuned_shapes_give_the_same_fields(tmp_path):
    from kadath_frontera_gb300._lib import Context
    table = tmp_path / "lp.json"
    fixed = _solve(Context(0))
    tctx = Context(0)
    tctx.autotune(table, mode=2)
    tuned = _solve(tctx)
    st = tctx.autotune_stats()
    assert st["tuned"] >= 3 and st["entries"] == st["tuned"]
    doc = json.loads(table.read_text())
    assert len(doc["line_passes"]) == st["entries"]
    for shape in doc["line_passes"].values():
        assert shape["cluster"] in (1, 2, 4, 8) and shape["threads"] in (64, 128, 256) and shape["us"] > 0
    rctx = Context(0)
    rctx.autotune(table, mode=1)
    again = _solve(rctx)
    rs = rctx.autotune_stats()
    assert rs["entries"] == st["entries"] and rs["tuned"] == 0 and rs["hits"] > 0
    for a, b, c in zip(fixed, tuned, again):
        for x, y, z in zip(a, b, c):
            assert np.array_equal(x, y) and np.array_equal(x, z)


def test_bad_mode_is_refused(ctx):
    from kadath_frontera_gb300 import KadathError
    with pytest.raises(KadathError):
        ctx.autotune(None, mode=3)
