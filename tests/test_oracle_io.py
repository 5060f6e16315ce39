"""The oracle's restatement of Kadath's save format (CPU): header bytes of a
Space_spheric file, and write -> read round trips of a space and a scalar."""
import io

import numpy as np

from oracle import kadath as K, kadath_io as KIO


def test_space_header_bytes():
    doms = K.space_spheric((13, 7, 4), [1.0, 2.0])
    buf = io.BytesIO()
    KIO.write_space(buf, doms)
    b = buf.getvalue()
    # nbr_domains 3, ndim 3, CHEB_TYPE 1, then the nucleus: Dim_array(3) of
    # points (13, 7, 4) and of coefficients (13, 7, 6), all big-endian
    assert b[:12] == bytes([0, 0, 0, 3, 0, 0, 0, 3, 0, 0, 0, 1])
    assert b[12:28] == bytes([0, 0, 0, 3, 0, 0, 0, 13, 0, 0, 0, 7, 0, 0, 0, 4])
    assert b[28:44] == bytes([0, 0, 0, 3, 0, 0, 0, 13, 0, 0, 0, 7, 0, 0, 0, 6])
    # nucleus record: 2 Dim_arrays (32 B), ndim, type (8 B), Point (4 + 24 B), alpha (8 B)
    nucleus = 32 + 8 + 28 + 8
    shell = nucleus + 8
    assert len(b) == 12 + nucleus + shell + nucleus
    sp = KIO.read_space(io.BytesIO(b))
    assert [d["type"] for d in sp] == [K.NUCLEUS, K.SHELL, K.COMPACT]
    assert sp[1]["alpha"] == 0.5 and sp[1]["beta"] == 1.5 and sp[2]["alpha"] == -0.25


def test_scalar_round_trip():
    doms = K.space_spheric((7, 5, 4), [1.0, 2.0])
    f = K.scalar_field(doms, lambda d: np.cos(d.radius() * 0.3) if d.type != K.COMPACT else np.zeros(d.np))
    for d in doms:
        f[d.num].coef()
    buf = io.BytesIO()
    KIO.write_scalar(buf, doms, f)
    buf.seek(0)
    sp = [dict(np=d.np, nc=d.nc) for d in doms]
    back = KIO.read_scalar(buf, sp)
    for d, (base, zero, conf, coef) in zip(doms, back):
        assert not zero
        assert np.array_equal(base[0], f[d.num].base.r) and np.array_equal(base[1], f[d.num].base.t)
        assert np.array_equal(conf, f[d.num].c[0]) and np.array_equal(coef, f[d.num].cf[0])
