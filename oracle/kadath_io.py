"""Test infrastructure: Kadath's binary save format restated in Python, to
check the product's save files byte by byte.

Follows Space_spheric::save / Space_spheric(FILE*, withzec)
(src/Space/Spheric/space_spheric.cpp:99-129), Domain_nucleus/shell/compact
::save (src/Domain/Spheric/domain_nucleus.cpp:52, domain_shell.cpp:53,
domain_compact.cpp:58), Scalar::save (src/Scalar/scalar.cpp:64),
Val_domain::save (src/Val_domain/val_domain.cpp:83), Base_spectral::save
(src/Base_spectral/base_spectral.cpp:70), Array<T>::save
(include/implementation/array.cpp:83), Dim_array::save and Point::save
(include/implementation/dim_array.cpp:73, point.cpp:51), Tensor::save
(src/Tensor/tensor.cpp:361); every number big-endian (fwrite_be,
src/Utilities/fwrite_be.cpp:30-100)."""
import struct

import numpy as np

from . import kadath as K

CHEB_TYPE = 1
CARTESIAN_BASIS = 0


class Writer:
    def __init__(self, fp):
        self.fp = fp

    def ints(self, *v):
        self.fp.write(struct.pack(">%di" % len(v), *v))

    def doubles(self, v):
        v = np.asarray(v, dtype=">f8").reshape(-1)
        self.fp.write(v.tobytes())

    def dims(self, d):
        self.ints(len(d), *d)

    def int_array(self, dims, data):
        self.dims(dims)
        data = [int(x) for x in np.asarray(data).reshape(-1)]
        self.ints(len(data), *data)

    def double_array(self, dims, data):
        self.dims(dims)
        data = np.asarray(data, dtype=np.float64).reshape(-1)
        self.ints(len(data))
        self.doubles(data)


class Reader:
    def __init__(self, fp):
        self.fp = fp

    def ints(self, n):
        b = self.fp.read(4 * n)
        assert len(b) == 4 * n, "unexpected end of file"
        return list(struct.unpack(">%di" % n, b))

    def doubles(self, n):
        b = self.fp.read(8 * n)
        assert len(b) == 8 * n, "unexpected end of file"
        return np.frombuffer(b, dtype=">f8").astype(np.float64)

    def dims(self):
        n = self.ints(1)[0]
        return self.ints(n)

    def int_array(self):
        d = self.dims()
        n = self.ints(1)[0]
        assert n == int(np.prod(d))
        return d, self.ints(n)

    def double_array(self):
        d = self.dims()
        n = self.ints(1)[0]
        assert n == int(np.prod(d))
        return d, self.doubles(n).reshape(d)


def write_space(fp, doms):
    w = Writer(fp)
    w.ints(len(doms), 3, CHEB_TYPE)
    for d in doms:
        w.dims(d.np)
        w.dims(d.nc)
        w.ints(3, CHEB_TYPE)
        w.ints(3)
        w.doubles([0.0, 0.0, 0.0])
        w.doubles([d.alpha])
        if d.type == K.SHELL:
            w.doubles([d.beta])


def read_space(fp, withzec=True):
    """Domains as dicts: type, np, nc, center, alpha, beta."""
    r = Reader(fp)
    nd, ndim, tb = r.ints(3)
    assert ndim == 3 and tb == CHEB_TYPE
    out = []
    for i in range(nd):
        typ = K.NUCLEUS if i == 0 else (K.COMPACT if (withzec and i == nd - 1) else K.SHELL)
        npts, nc = r.dims(), r.dims()
        ndim_d, tb_d = r.ints(2)
        assert ndim_d == 3 and tb_d == CHEB_TYPE
        assert r.ints(1)[0] == 3
        center = r.doubles(3)
        alpha = r.doubles(1)[0]
        beta = r.doubles(1)[0] if typ == K.SHELL else 0.0
        out.append(dict(type=typ, np=tuple(npts), nc=tuple(nc), center=center, alpha=alpha, beta=beta))
    return out


def write_val_domain(w, d, vd):
    """vd: a VD with B = 1 (values at the collocation points and/or coefficients)."""
    b = vd.base
    if b.defined:
        w.ints(0, 3)
        w.int_array([d.nc[1], d.nc[2]], b.r)
        w.int_array([d.nc[2]], b.t)
        w.int_array([1], [b.p])
    else:
        w.ints(1, 3)
    w.ints(1 if vd.zero else 0)
    conf = (not vd.zero) and vd.c is not None
    w.ints(0 if conf else 1)
    if conf:
        w.double_array(list(d.np), vd.c[0])
    coef = (not vd.zero) and vd.cf is not None
    w.ints(0 if coef else 1)
    if coef:
        w.double_array(list(d.nc), vd.cf[0])


def read_val_domain(r, d):
    """(base (r, t, p) or None, zero, conf array or None, coef array or None)."""
    undefined, ndim = r.ints(2)
    assert ndim == 3
    base = None
    if not undefined:
        dr, br = r.int_array()
        dt, bt = r.int_array()
        dp, bp = r.int_array()
        assert dr == [d["nc"][1], d["nc"][2]] and dt == [d["nc"][2]] and dp == [1]
        base = (np.array(br).reshape(dr), np.array(bt), bp[0])
    zero = r.ints(1)[0] != 0
    conf = coef = None
    if r.ints(1)[0] == 0:
        dd, conf = r.double_array()
        assert tuple(dd) == d["np"]
    if r.ints(1)[0] == 0:
        dd, coef = r.double_array()
        assert tuple(dd) == d["nc"]
    return base, zero, conf, coef


def write_scalar(fp, doms, field):
    w = Writer(fp)
    for d in doms:
        write_val_domain(w, d, field[d.num])


def read_scalar(fp, domains):
    r = Reader(fp)
    return [read_val_domain(r, d) for d in domains]


def read_vector(fp, domains):
    """(type_index, three components as read_scalar lists)."""
    r = Reader(fp)
    db, basis = r.int_array()
    assert db == [len(domains)] and all(b == CARTESIAN_BASIS for b in basis)
    _, ti = r.int_array()
    valence, ncomp = r.ints(2)
    assert valence == 1 and ncomp == 3 and len(ti) == 1
    return ti[0], [read_scalar(fp, domains) for _ in range(3)]
