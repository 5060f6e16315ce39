"""CPU oracle for the Newton-Raphson path of Kadath (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module, and only as the checker or as the timed
CPU baseline.  The product path never imports it.

A numpy restatement of the reference's CPU solver for spherical spaces:

* Val_domain with its lazy conf/coef state (src/Val_domain/val_domain.cpp,
  val_domain_math.cpp), batched over Jacobian seeds;
* Domain_{nucleus,shell,compact} geometry, basis product rules and operators
  (src/Domain/Spheric/domain_*.cpp, domain_*_ope.cpp), Cartesian derivatives
  by the chain rule (do_der_abs_from_der_var) and the flat Laplacian
  (src/Domain/domain.cpp:155);
* tau/Galerkin tables: export_tau (domain_*_export_tau.cpp), boundary export
  (domain_*_export_tau_boundary.cpp + val_boundary, domain_*_systems.cpp),
  unknown patterns (domain_*_affecte_tau_one_coef.cpp) and the x -> fields
  map (domain_*_affecte_tau.cpp);
* Term_eq forward-mode rules (src/Term_eq/term_eq_math.cpp);
* the serial Newton step do_newton_seq (src_par/do_newton.cpp:519-572) with
  the Jacobian built column by column as do_col_J (solver.cpp:120) would,
  here vectorised over columns, and LAPACK getrf/getrs through scipy.

Equations are given as Python callables on ``OTerm`` objects instead of
strings (the string parser is product code under test).

Pinning: the analytic solutions printed by tutorials/tuto5.cpp
(F = 1 + a/r), codes/Seq_version/schwarz.cpp (conformal factor 1 + a/r,
max error over 100 points) and tutorials/tuto6.cpp (P = log(1 + a/r)) are
reproduced by this oracle in tests/test_oracle_newton.py.
"""
from __future__ import annotations

import math

import numpy as np

from . import spectral as S

NUCLEUS, SHELL, COMPACT = 1, 2, 3
OUTER_BC, INNER_BC = 0, 1

_MAT_CACHE: dict = {}


def mat(op, base, n_in, n_out=None):
    key = (op, int(base), n_in, n_out or n_in)
    if key not in _MAT_CACHE:
        _MAT_CACHE[key] = S.matrix_1d(op, int(base), n_in, n_out or n_in)
    return _MAT_CACHE[key]


class OBase:
    def __init__(self, r=None, t=None, p=None):
        self.r = None if r is None else np.array(r, dtype=int)
        self.t = None if t is None else np.array(t, dtype=int)
        self.p = p

    @property
    def defined(self):
        return self.r is not None

    def copy(self):
        return OBase(None if self.r is None else self.r.copy(), None if self.t is None else self.t.copy(), self.p)

    def key(self):
        return (tuple(self.r.ravel()), tuple(self.t), self.p)


def _apply_dim(x, dim, op, base_table, n_in, n_out):
    """Applies per-line matrices along `dim` of a batch x[B, n0, n1, n2].

    base_table: for dim 0 an (n1, n2) table, dim 1 an (n2,) table, dim 2 a
    scalar.  Returns (result, output basis table)."""
    B, n0, n1, n2 = x.shape
    shape = [B, n0, n1, n2]
    shape[dim + 1] = n_out
    y = np.zeros(shape)
    if dim == 2:
        ob, m = mat(op, base_table, n_in, n_out)
        y[:] = np.einsum("ok,bijk->bijo", m, x)
        return y, ob
    if dim == 1:
        out_t = np.array(base_table).copy()
        for k in range(n2):
            ob, m = mat(op, base_table[k], n_in, n_out)
            y[:, :, :, k] = np.einsum("oj,bij->bio", m, x[:, :, :, k])
            out_t[k] = ob
        return y, out_t
    out_r = np.array(base_table).copy()
    for j in range(n1):
        for k in range(n2):
            ob, m = mat(op, base_table[j][k], n_in, n_out)
            y[:, :, j, k] = np.einsum("oi,bi->bo", m, x[:, :, j, k])
            out_r[j][k] = ob
    return y, out_r


class ODomain:
    """Domain_nucleus / Domain_shell / Domain_compact (CHEB_TYPE)."""

    def __init__(self, num, dtype, res, alpha, beta):
        self.num, self.type = num, dtype
        self.np = tuple(res)
        self.nc = (res[0], res[1], res[2] + 2)
        self.alpha, self.beta = alpha, beta
        n0, n1, n2 = res
        if dtype == NUCLEUS:
            self.x = np.array([math.sin(math.pi / 2. * i / (n0 - 1)) for i in range(n0)])
        else:
            self.x = np.array([-math.cos(math.pi * i / (n0 - 1)) for i in range(n0)])
        self.theta = np.array([math.pi / 2. * j / (n1 - 1) for j in range(n1)])
        self.phi = np.array([math.pi * 2. * k / n2 for k in range(n2)])

    # geometry --------------------------------------------------------------
    def radius_1d(self):
        if self.type == NUCLEUS:
            return self.alpha * self.x
        if self.type == SHELL:
            return self.alpha * self.x + self.beta
        with np.errstate(divide="ignore"):
            return 1. / self.alpha / (self.x - 1)

    def radius(self):
        r = self.radius_1d()
        return np.broadcast_to(r[:, None, None], self.np).copy()

    def cart(self, c):
        r = self.radius()
        th = self.theta[None, :, None]
        ph = self.phi[None, None, :]
        if c == 0:
            return r * np.sin(th) * np.cos(ph)
        if c == 1:
            return r * np.sin(th) * np.sin(ph)
        return r * np.cos(th) * np.ones_like(ph)

    # bases -----------------------------------------------------------------
    def std_base(self):
        nc1, nc2 = self.nc[1], self.nc[2]
        t = np.zeros(nc2, dtype=int)
        r = np.zeros((nc1, nc2), dtype=int)
        for k in range(nc2):
            m = k // 2
            t[k] = S.COS_EVEN if m % 2 == 0 else S.SIN_ODD
            for j in range(nc1):
                if self.type == NUCLEUS:
                    l = 2 * j if m % 2 == 0 else 2 * j + 1
                    r[j, k] = S.CHEB_EVEN if l % 2 == 0 else S.CHEB_ODD
                else:
                    r[j, k] = S.CHEB
        return OBase(r, t, S.COSSIN)

    def mult(self, a, b):
        """Domain_*::mult: basis of a product."""
        if not (a.defined and b.defined):
            return OBase()
        sig = {S.COS_EVEN: (1, 1), S.COS_ODD: (1, -1), S.SIN_EVEN: (-1, -1), S.SIN_ODD: (-1, 1)}
        inv = {v: k for k, v in sig.items()}
        t = np.zeros_like(a.t)
        for k in range(len(a.t)):
            s1a, s2a = sig[int(a.t[k])]
            s1b, s2b = sig[int(b.t[k])]
            flip = 1 if k % 4 < 2 else -1
            t[k] = inv[(s1a * s1b * flip, s2a * s2b)]
        r = np.zeros_like(a.r)
        for j in range(a.r.shape[0]):
            for k in range(a.r.shape[1]):
                if self.type == NUCLEUS:
                    pa = 1 if a.r[j, k] == S.CHEB_EVEN else -1
                    pb = 1 if b.r[j, k] == S.CHEB_EVEN else -1
                    flip = 1 if k % 4 < 2 else -1
                    r[j, k] = S.CHEB_EVEN if pa * pb * flip > 0 else S.CHEB_ODD
                else:
                    r[j, k] = S.CHEB
        return OBase(r, t, S.COSSIN)

    # tau tables ------------------------------------------------------------
    def cidx(self, i, j, k):
        return (i * self.nc[1] + j) * self.nc[2] + k

    def export_tau(self, base, order):
        """export_tau_val_domain (mlim = 0): list of rows [(idx, w), ...]."""
        nc0, nc1, nc2 = self.nc
        kmin = 2
        rows = []
        ci = self.cidx
        if self.type != NUCLEUS:
            for k in range(nc2 - 1):
                if k == 1:
                    continue
                bt = base.t[k]
                for j in range(nc1):
                    for i in range(nc0 - order):
                        if bt == S.COS_EVEN:
                            if k < kmin:
                                rows.append([(ci(i, j, k), 1.0)])
                            elif j != 0:
                                rows.append([(ci(i, j, k), 1.0), (ci(i, 0, k), -2.0)])
                        elif bt == S.COS_ODD:
                            if j != nc1 - 1:
                                if k < kmin:
                                    rows.append([(ci(i, j, k), 1.0)])
                                elif j != 0:
                                    rows.append([(ci(i, j, k), 1.0), (ci(i, 0, k), -1.0)])
                        elif bt == S.SIN_EVEN:
                            if j != 0 and j != nc1 - 1:
                                if k < kmin + 2:
                                    rows.append([(ci(i, j, k), 1.0)])
                                elif j != 1:
                                    rows.append([(ci(i, j, k), 1.0), (ci(i, 1, k), -float(j))])
                        elif bt == S.SIN_ODD:
                            if j != nc1 - 1:
                                if k < kmin + 2:
                                    rows.append([(ci(i, j, k), 1.0)])
                                elif j != 0:
                                    rows.append([(ci(i, j, k), 1.0), (ci(i, 0, k), -float(2 * j + 1))])
            return rows
        rlim = 1 if order == 0 else 2
        llim = 0
        sg = lambda i: 1.0 if i % 2 == 0 else -1.0
        for k in range(nc2 - 1):
            if k == 1:
                continue
            bt = base.t[k]
            for j in range(nc1):
                for i in range(nc0):
                    if bt == S.COS_EVEN:
                        lq = 2 * j
                        if k < kmin and lq <= llim:
                            if i != nc0 - rlim + 1:
                                rows.append([(ci(i, j, k), 1.0)])
                        elif k < kmin:
                            if i != 0 and i != nc0 - rlim + 1:
                                rows.append([(ci(i, j, k), 1.0), (ci(0, j, k), -2 * sg(i))])
                        elif j != 0 and i != 0 and i != nc0 - rlim + 1:
                            rows.append([(ci(i, j, k), 1.0), (ci(0, j, k), -2 * sg(i)), (ci(i, 0, k), -2.0),
                                         (ci(0, 0, k), 4 * sg(i))])
                    elif bt == S.COS_ODD:
                        lq = 2 * j + 1
                        if j != nc1 - 1 and i != nc0 - rlim + 1 and i != nc0 - rlim:
                            if k < kmin and lq <= llim + 1:
                                rows.append([(ci(i, j, k), 1.0)])
                            elif k < kmin and i != 0:
                                rows.append([(ci(i, j, k), 1.0), (ci(0, j, k), -(2 * i + 1) * sg(i))])
                            elif j != 0 and i != 0:
                                rows.append([(ci(i, j, k), 1.0), (ci(0, j, k), -sg(i) * (2 * i + 1)),
                                             (ci(i, 0, k), -1.0), (ci(0, 0, k), sg(i) * (2 * i + 1))])
                    elif bt == S.SIN_EVEN:
                        lq = 2 * j
                        if j != 0 and j != nc1 - 1 and i != nc0 - rlim + 1:
                            if k < kmin + 2 and lq <= llim:
                                rows.append([(ci(i, j, k), 1.0)])
                            elif k < kmin + 2 and i != 0:
                                rows.append([(ci(i, j, k), 1.0), (ci(0, j, k), -2 * sg(i))])
                            elif k >= kmin + 2 and j != 1 and i != 0:
                                rows.append([(ci(i, j, k), 1.0), (ci(0, j, k), -sg(i)), (ci(i, 1, k), -float(j)),
                                             (ci(0, 1, k), sg(i) * j)])
                    elif bt == S.SIN_ODD:
                        lq = 2 * j + 1
                        if j != nc1 - 1 and i != nc0 - rlim + 1 and i != nc0 - rlim:
                            if k < kmin + 2 and lq <= llim + 1:
                                rows.append([(ci(i, j, k), 1.0)])
                            elif k < kmin + 2 and i != 0:
                                rows.append([(ci(i, j, k), 1.0), (ci(0, j, k), -(2 * i + 1) * sg(i))])
                            elif j != 0 and i != 0:
                                rows.append([(ci(i, j, k), 1.0), (ci(0, j, k), -sg(i) * (2 * i + 1)),
                                             (ci(i, 0, k), -float(2 * j + 1)),
                                             (ci(0, 0, k), sg(i) * (2 * i + 1) * (2 * j + 1))])
        return rows

    def val_boundary(self, bound, j, k, w):
        """val_boundary as (idx, w) terms."""
        out = []
        for i in range(self.nc[0]):
            s = (1.0 if i % 2 == 0 else -1.0) if bound == INNER_BC else 1.0
            out.append((self.cidx(i, j, k), w * s))
        return out

    def export_tau_boundary(self, base, bound):
        nc0, nc1, nc2 = self.nc
        kmin = 2
        rows = []
        vb = self.val_boundary
        for k in range(nc2 - 1):
            if k == 1:
                continue
            bt = base.t[k]
            for j in range(nc1):
                if bt == S.COS_EVEN:
                    if k < kmin:
                        rows.append(vb(bound, j, k, 1.0))
                    elif j != 0:
                        rows.append(vb(bound, j, k, 1.0) + vb(bound, 0, k, -2.0))
                elif bt == S.COS_ODD:
                    if j != nc1 - 1:
                        if k < kmin:
                            rows.append(vb(bound, j, k, 1.0))
                        elif j != 0:
                            rows.append(vb(bound, j, k, 1.0) + vb(bound, 0, k, -1.0))
                elif bt == S.SIN_EVEN:
                    if j != 0 and j != nc1 - 1:
                        if k < kmin + 2:
                            rows.append(vb(bound, j, k, 1.0))
                        elif j != 1:
                            rows.append(vb(bound, j, k, 1.0) + vb(bound, 1, k, -float(j)))
                elif bt == S.SIN_ODD:
                    if j != nc1 - 1:
                        if k < kmin + 2:
                            rows.append(vb(bound, j, k, 1.0))
                        elif j != 0:
                            rows.append(vb(bound, j, k, 1.0) + vb(bound, 0, k, -float(2 * j + 1)))
        return rows

    def unknown_patterns(self, base):
        """affecte_tau_one_coef_val_domain (mlim = llim = 0)."""
        nc0, nc1, nc2 = self.nc
        kmin = 2
        pats = []
        ci = self.cidx
        if self.type != NUCLEUS:
            for k in range(nc2 - 1):
                if k == 1:
                    continue
                bt = base.t[k]
                for j in range(nc1):
                    if bt == S.COS_EVEN:
                        true_t = not (j == 0 and k >= kmin)
                    elif bt == S.COS_ODD:
                        true_t = not (j == nc1 - 1 or (j == 0 and k >= kmin))
                    elif bt == S.SIN_EVEN:
                        true_t = not ((j == 1 and k >= kmin + 2) or j == 0 or j == nc1 - 1)
                    else:
                        true_t = not ((j == 0 and k >= kmin + 2) or j == nc1 - 1)
                    if not true_t:
                        continue
                    for i in range(nc0):
                        p = [(ci(i, j, k), 1.0)]
                        if bt in (S.COS_EVEN, S.COS_ODD) and k >= kmin:
                            p.append((ci(i, 0, k), -1.0))
                        if bt == S.SIN_EVEN and k >= kmin + 2:
                            p.append((ci(i, 1, k), -float(j)))
                        if bt == S.SIN_ODD and k >= kmin + 2:
                            p.append((ci(i, 0, k), -float(2 * j + 1)))
                        pats.append(p)
            return pats
        llim = 0
        sg = lambda i: 1.0 if i % 2 == 0 else -1.0
        for k in range(nc2 - 1):
            if k == 1:
                continue
            bt = base.t[k]
            for j in range(nc1):
                for i in range(nc0):
                    p = None
                    if bt == S.COS_EVEN:
                        lq = 2 * j
                        if k < kmin and lq <= llim:
                            p = [(ci(i, j, k), 1.0)]
                        elif k < kmin:
                            if i != 0:
                                p = [(ci(i, j, k), 1.0), (ci(0, j, k), -sg(i))]
                        elif j != 0 and i != 0:
                            p = [(ci(i, j, k), 1.0), (ci(0, j, k), -sg(i)), (ci(i, 0, k), -1.0), (ci(0, 0, k), sg(i))]
                    elif bt == S.COS_ODD:
                        lq = 2 * j + 1
                        if j != nc1 - 1 and i != nc0 - 1:
                            if k < kmin and lq <= llim + 1:
                                p = [(ci(i, j, k), 1.0)]
                            elif k < kmin and i != 0:
                                p = [(ci(i, j, k), 1.0), (ci(0, j, k), -(2 * i + 1) * sg(i))]
                            elif j != 0 and i != 0:
                                p = [(ci(i, j, k), 1.0), (ci(0, j, k), -sg(i) * (2 * i + 1)), (ci(i, 0, k), -1.0),
                                     (ci(0, 0, k), sg(i) * (2 * i + 1))]
                    elif bt == S.SIN_EVEN:
                        lq = 2 * j
                        if j != 0 and j != nc1 - 1:
                            if k < kmin + 2 and lq <= llim:
                                p = [(ci(i, j, k), 1.0)]
                            elif k < kmin + 2 and i != 0:
                                p = [(ci(i, j, k), 1.0), (ci(0, j, k), -sg(i))]
                            elif k >= kmin + 2 and j != 1 and i != 0:
                                p = [(ci(i, j, k), 1.0), (ci(0, j, k), -sg(i)), (ci(i, 1, k), -float(j)),
                                     (ci(0, 1, k), sg(i) * j)]
                    elif bt == S.SIN_ODD:
                        lq = 2 * j + 1
                        if j != nc1 - 1 and i != nc0 - 1:
                            if k < kmin + 2 and lq <= llim + 1:
                                p = [(ci(i, j, k), 1.0)]
                            elif k < kmin + 2 and i != 0:
                                p = [(ci(i, j, k), 1.0), (ci(0, j, k), -(2 * i + 1) * sg(i))]
                            elif j != 0 and i != 0:
                                p = [(ci(i, j, k), 1.0), (ci(0, j, k), -sg(i) * (2 * i + 1)),
                                     (ci(i, 0, k), -float(2 * j + 1)), (ci(0, 0, k), sg(i) * (2 * i + 1) * (2 * j + 1))]
                    if p is not None:
                        pats.append(p)
        return pats

    def affecte_tau_matrix(self, base):
        """x -> coefficients (affecte_tau_val_domain) as a dense matrix."""
        nc0, nc1, nc2 = self.nc
        ncf = nc0 * nc1 * nc2
        if self.type == NUCLEUS:
            pats = self.unknown_patterns(base)
            M = np.zeros((ncf, len(pats)))
            for u, p in enumerate(pats):
                for idx, w in p:
                    M[idx, u] += w
            return M
        kmin = 2
        cols = []
        M = np.zeros((ncf, ncf))
        conte = 0
        ci = self.cidx
        for k in range(nc2 - 1):
            if k == 1:
                continue
            bt = base.t[k]
            for j in range(nc1):
                if bt == S.COS_EVEN:
                    tt = not (j == 0 and k >= kmin)
                elif bt == S.COS_ODD:
                    tt = not (j == nc1 - 1 or (j == 0 and k >= kmin))
                elif bt == S.SIN_EVEN:
                    tt = not ((j == 1 and k >= kmin + 2) or j == 0 or j == nc1 - 1)
                else:
                    tt = not ((j == 0 and k > kmin + 2) or j == nc1 - 1)
                if not tt:
                    continue
                for i in range(nc0):
                    M[ci(i, j, k), conte] = 1.0
                    conte += 1
        for k in range(nc2 - 1):
            bt = base.t[k]
            for i in range(nc0):
                if bt in (S.COS_EVEN, S.COS_ODD) and k >= kmin:
                    M[ci(i, 0, k), :] = -sum(M[ci(i, j, k), :] for j in range(1, nc1))
                elif bt == S.SIN_EVEN and k >= kmin + 2:
                    M[ci(i, 1, k), :] = -sum(j * M[ci(i, j, k), :] for j in range(2, nc1))
                elif bt == S.SIN_ODD and k >= kmin + 2:
                    M[ci(i, 0, k), :] = -sum((2 * j + 1) * M[ci(i, j, k), :] for j in range(1, nc1))
        return M[:, :conte]

    def has_boundary(self, bound):
        if self.type == NUCLEUS:
            return bound == OUTER_BC
        return True


def space_spheric(res, bounds, withzec=True):
    """Space_spheric (src/Space/Spheric/space_spheric.cpp:25)."""
    doms = [ODomain(0, NUCLEUS, res, bounds[0], 0.0)]
    nd = len(bounds) + 1 if withzec else len(bounds)
    nshell = nd - 1 if withzec else nd
    for i in range(1, nshell):
        doms.append(ODomain(i, SHELL, res, (bounds[i] - bounds[i - 1]) / 2., (bounds[i] + bounds[i - 1]) / 2.))
    if withzec:
        doms.append(ODomain(nd - 1, COMPACT, res, -0.5 / bounds[nd - 2], 0.0))
    return doms


# ------------------------------------------------------------- Val_domain --
class VD:
    """Val_domain batch: c has shape (B,)+np, cf (B,)+nc."""

    def __init__(self, dom, B=1, c=None, cf=None, base=None, zero=False):
        self.dom, self.B = dom, B
        self.c, self.cf = c, cf
        self.base = base if base is not None else OBase()
        self.zero = zero
        self._dvar = None
        self._dabs = None

    @staticmethod
    def zeros(dom, B=1):
        return VD(dom, B, zero=True)

    def coef(self):
        if self.zero or self.cf is not None:
            return
        b = self.base
        d = self.dom
        x, _ = _apply_dim(self.c, 2, S.OP_COEF, b.p, d.np[2], d.nc[2])
        x, _ = _apply_dim(x, 1, S.OP_COEF, b.t, d.np[1], d.nc[1])
        x, _ = _apply_dim(x, 0, S.OP_COEF, b.r, d.np[0], d.nc[0])
        self.cf = x

    def coef_i(self):
        if self.zero or self.c is not None:
            return
        b = self.base
        d = self.dom
        x, _ = _apply_dim(self.cf, 0, S.OP_COEF_I, b.r, d.nc[0], d.np[0])
        x, _ = _apply_dim(x, 1, S.OP_COEF_I, b.t, d.nc[1], d.np[1])
        x, _ = _apply_dim(x, 2, S.OP_COEF_I, b.p, d.nc[2], d.np[2])
        self.c = x

    def ope(self, op, dim):
        self.coef()
        b = self.base.copy()
        d = self.dom
        table = [b.r, b.t, b.p][dim]
        y, ob = _apply_dim(self.cf, dim, op, table, d.nc[dim], d.nc[dim])
        if dim == 0:
            b.r = ob
        elif dim == 1:
            b.t = ob
        else:
            b.p = ob
        return VD(d, self.B, cf=y, base=b)

    def der_var(self, var):
        if self.zero:
            return self
        if self._dvar is None:
            self._dvar = [self.ope(S.OP_DER, v) for v in range(3)]
        return self._dvar[var - 1]

    def der_abs(self, var):
        if self.zero:
            return self
        if self._dabs is None:
            self._dabs = der_abs_from_der_var(self.dom, [self.der_var(v) for v in (1, 2, 3)])
        return self._dabs[var - 1]

    # algebra (val_domain_math.cpp) ------------------------------------------
    def _bc(self, other):
        return max(self.B, other.B)

    def __add__(self, o):
        if isinstance(o, (int, float)):
            if self.zero:
                return VD(self.dom, 1, c=np.full((1,) + self.dom.np, float(o)), base=self.dom.std_base())
            self.coef_i()
            return VD(self.dom, self.B, c=self.c + o, base=self.base)
        if self.zero:
            return o
        if o.zero:
            return self
        if self.c is not None or o.c is not None:
            self.coef_i(); o.coef_i()
            res = VD(self.dom, self._bc(o), c=self.c + o.c)
        else:
            res = VD(self.dom, self._bc(o), cf=self.cf + o.cf)
        if self.base.defined and o.base.defined:
            res.base = self.base
        return res

    def __neg__(self):
        if self.zero:
            return self
        return self.scale(-1.0)

    def __sub__(self, o):
        if isinstance(o, (int, float)):
            return self + (-o)
        if self.zero:
            return -o
        if o.zero:
            return self
        if self.c is not None or o.c is not None:
            self.coef_i(); o.coef_i()
            res = VD(self.dom, self._bc(o), c=self.c - o.c)
        else:
            res = VD(self.dom, self._bc(o), cf=self.cf - o.cf)
        if self.base.defined and o.base.defined:
            res.base = self.base
        return res

    def rsub(self, x):
        """x - self (double minus Val_domain)."""
        if self.zero:
            return VD(self.dom, 1, c=np.full((1,) + self.dom.np, float(x)), base=self.dom.std_base())
        self.coef_i()
        return VD(self.dom, self.B, c=x - self.c, base=self.base)

    def scale(self, x):
        if self.zero:
            return self
        return VD(self.dom, self.B, c=None if self.c is None else self.c * x,
                  cf=None if self.cf is None else self.cf * x, base=self.base)

    def __mul__(self, o):
        if isinstance(o, (int, float)):
            return self.scale(float(o))
        if self.zero:
            return self
        if o.zero:
            return o
        self.coef_i(); o.coef_i()
        return VD(self.dom, self._bc(o), c=self.c * o.c, base=self.dom.mult(self.base, o.base))

    def __truediv__(self, o):
        if isinstance(o, (int, float)):
            if self.zero:
                return self
            return VD(self.dom, self.B, c=None if self.c is None else self.c / o,
                      cf=None if self.cf is None else self.cf / o, base=self.base)
        if self.zero:
            return self
        self.coef_i(); o.coef_i()
        return VD(self.dom, self._bc(o), c=self.c / o.c, base=self.dom.mult(self.base, o.base))

    def rdiv(self, x):
        self.coef_i()
        return VD(self.dom, self.B, c=x / self.c, base=self.dom.std_base())

    def exp(self):
        """exp(Val_domain) (val_domain_math.cpp): at the collocation points,
        the basis kept; exp(0) is 1 with no basis."""
        if self.zero:
            return VD(self.dom, self.B, c=np.ones((self.B,) + self.dom.np))
        self.coef_i()
        return VD(self.dom, self.B, c=np.exp(self.c), base=self.base)

    def log(self):
        self.coef_i()
        return VD(self.dom, self.B, c=np.log(self.c), base=self.base)

    def atanh(self):
        """atanh(Val_domain) (val_domain_math.cpp:506): at the collocation
        points, the basis kept."""
        if self.zero:
            return self
        self.coef_i()
        return VD(self.dom, self.B, c=np.arctanh(self.c), base=self.base)


def radius_vd(dom):
    return VD(dom, 1, c=dom.radius()[None])


def _swap_t(b):
    return {S.COS_EVEN: S.SIN_ODD, S.COS_ODD: S.SIN_EVEN, S.SIN_EVEN: S.COS_ODD, S.SIN_ODD: S.COS_EVEN}[int(b)]


def mult_trig_phi(so, op):
    if so.zero:
        return so
    so.coef()
    nb = so.base.copy()
    nb.t = np.array([_swap_t(b) for b in so.base.t])
    if so.dom.type == NUCLEUS:
        nb.r = np.where(so.base.r == S.CHEB_EVEN, S.CHEB_ODD, S.CHEB_EVEN)
    y, ob = _apply_dim(so.cf, 2, op, so.base.p, so.dom.nc[2], so.dom.nc[2])
    nb.p = ob
    return VD(so.dom, so.B, cf=y, base=nb)


def opc(so, op, dim):
    return so if so.zero else so.ope(op, dim)


def der_abs_from_der_var(dom, dv):
    a = dom.alpha
    if dom.type == SHELL:
        sintdr = opc(dv[0], S.OP_MULT_SIN, 1) / a
        rad = radius_vd(dom)
        dtsr = dv[1] / rad
        dtsr.base = dv[1].base
        dpsr = dv[2] / rad
        dpsr.base = dv[2].base
        costdtsr = opc(dtsr, S.OP_MULT_COS, 1)
        dpsrssint = opc(dpsr, S.OP_DIV_SIN, 1)
        s = sintdr + costdtsr
        dx = mult_trig_phi(s, S.OP_MULT_COS) - mult_trig_phi(dpsrssint, S.OP_MULT_SIN)
        dy = mult_trig_phi(s, S.OP_MULT_SIN) + mult_trig_phi(dpsrssint, S.OP_MULT_COS)
        dz = opc(dv[0], S.OP_MULT_COS, 1) / a - opc(dtsr, S.OP_MULT_SIN, 1)
        return [dx, dy, dz]
    if dom.type == NUCLEUS:
        sintdr = opc(dv[0], S.OP_MULT_SIN, 1) / a
        dtsr = opc(dv[1], S.OP_DIV_X, 0) / a
        dpsr = opc(dv[2], S.OP_DIV_X, 0) / a
        costdtsr = opc(dtsr, S.OP_MULT_COS, 1)
        dpsrssint = opc(dpsr, S.OP_DIV_SIN, 1)
        s = sintdr + costdtsr
        dx = mult_trig_phi(s, S.OP_MULT_COS) - mult_trig_phi(dpsrssint, S.OP_MULT_SIN)
        dy = mult_trig_phi(s, S.OP_MULT_SIN) + mult_trig_phi(dpsrssint, S.OP_MULT_COS)
        dz = opc(dv[0], S.OP_MULT_COS, 1) / a - opc(dtsr, S.OP_MULT_SIN, 1)
        return [dx, dy, dz]
    dr = -opc(dv[0], S.OP_MULT_XM1, 0)
    sintdr = opc(dr, S.OP_MULT_SIN, 1)
    costdt = opc(dv[1], S.OP_MULT_COS, 1)
    dpssint = opc(dv[2], S.OP_DIV_SIN, 1)
    s = sintdr + costdt
    ax = mult_trig_phi(s, S.OP_MULT_COS) - mult_trig_phi(dpssint, S.OP_MULT_SIN)
    ay = mult_trig_phi(s, S.OP_MULT_SIN) + mult_trig_phi(dpssint, S.OP_MULT_COS)
    az = opc(dr, S.OP_MULT_COS, 1) - opc(dv[1], S.OP_MULT_SIN, 1)
    return [opc(ax, S.OP_MULT_XM1, 0) * a, opc(ay, S.OP_MULT_XM1, 0) * a, opc(az, S.OP_MULT_XM1, 0) * a]


def laplacian(so):
    res = so.der_abs(1).der_abs(1)
    for j in (2, 3):
        res = res + so.der_abs(j).der_abs(j)
    return res


def der_normal(so, bound):
    d = so.dom
    if d.type == COMPACT:
        r = opc(opc(so.der_var(1), S.OP_MULT_XM1, 0), S.OP_MULT_XM1, 0)
        return r * (-d.alpha)
    return so.der_var(1) / d.alpha


def der_r(so):
    """Domain_nucleus::der_r and Domain_shell::der_r (domain_nucleus_ope.cpp:238,
    domain_shell_ope.cpp:218): der_var(1) / alpha; Domain_compact::der_r
    (domain_compact_ope.cpp:187): -alpha (x - 1)^2 der_var(1).  In these
    domains that is der_normal at either boundary."""
    if so.zero:
        return so
    return der_normal(so, OUTER_BC)


def mult_r(so):
    """Domain_*::mult_r (domain_nucleus_ope.cpp:214, domain_shell_ope.cpp:156,
    domain_compact_ope.cpp:173)."""
    if so.zero:
        return so
    d = so.dom
    if d.type == NUCLEUS:
        return opc(so, S.OP_MULT_X, 0) * d.alpha
    if d.type == SHELL:
        so.coef()
        mx = opc(so, S.OP_MULT_X, 0)
        return VD(d, so.B, cf=mx.cf * d.alpha + so.cf * d.beta, base=mx.base)
    return opc(so, S.OP_DIV_XM1, 0) / d.alpha


def integral_1d(base, cf):
    """integral_1d (src/Ope_1d/integral_1d.cpp) of coefficient rows cf[..., i]."""
    n = cf.shape[-1]
    res = np.zeros(cf.shape[:-1])
    if base == S.CHEB_EVEN:
        for i in range(n):
            res = res + -cf[..., i] / (4. * i * i - 1)
    elif base == S.CHEB:
        for i in range(0, n, 2):
            res = res + -2 * cf[..., i] / (i * i - 1.)
    else:
        raise NotImplementedError(f"integral_1d of basis {base}")
    return res


def integ_volume(so):
    """Domain_*::integ_volume (domain_nucleus_ope.cpp:260,
    domain_shell_ope.cpp:281, domain_compact_ope.cpp:228), per batch member."""
    if so.zero:
        return np.zeros(so.B)
    d = so.dom
    w = mult_r(mult_r(opc(so, S.OP_MULT_SIN, 1)))
    if d.type == COMPACT:
        w = -mult_r(mult_r(w)) * d.alpha
    else:
        w = w * d.alpha
    w.coef()
    assert int(w.base.t[0]) == S.SIN_ODD
    val = np.zeros(so.B)
    for j in range(d.nc[1]):
        baser = int(w.base.r[j, 0])
        assert baser == (S.CHEB_EVEN if d.type == NUCLEUS else S.CHEB)
        val = val + 2. / (2. * j + 1) * integral_1d(baser, w.cf[:, :, j, 0])
    return val * 2 * math.pi


def integ_surface(so, bound):
    """Domain_compact::integ (domain_compact.cpp:89), per batch member."""
    d = so.dom
    assert d.type == COMPACT
    if so.zero:
        return np.zeros(so.B)
    rr = mult_r(mult_r(opc(so, S.OP_MULT_SIN, 1)))
    rr.coef()

    def vb(j):
        sg = np.array([(1.0 if i % 2 == 0 else -1.0) if bound == INNER_BC else 1.0 for i in range(d.nc[0])])
        return rr.cf[:, :, j, 0] @ sg

    res = np.zeros(so.B)
    bt = int(rr.base.t[0])
    if bt == S.COS_EVEN:
        res = res + math.pi * vb(0)
    elif bt == S.SIN_ODD:
        for j in range(d.nc[1]):
            res = res + 2. / (2 * j + 1) * vb(j)
    elif bt not in (S.COS_ODD, S.SIN_EVEN):
        raise NotImplementedError("integ: theta basis")
    return res * 2 * math.pi


def value_at(so, pos):
    """Ope_val (src/Ope_eq/ope_val.cpp): the value at collocation point pos."""
    if so.zero:
        return np.zeros(so.B)
    so.coef_i()
    i, j, k = pos
    return so.c[:, i, j, k].copy()


def summation(so, num):
    """Base_spectral::summation at numerical coordinates num, per batch member."""
    if so.zero:
        return np.zeros(so.B)
    so.coef()
    d, b = so.dom, so.base
    xi, th, ph = num
    nc0, nc1, nc2 = d.nc
    out = np.zeros(so.B)
    for m in range(so.B):
        cf = so.cf[m]
        lines = np.zeros((nc1, nc2))
        for j in range(nc1):
            for k in range(nc2):
                lines[j, k] = S.summation_1d(int(b.r[j, k]), xi, cf[:, j, k])
        tvals = np.array([S.summation_1d(int(b.t[k]), th, lines[:, k]) for k in range(nc2)])
        out[m] = S.summation_1d(int(b.p), ph, tvals)
    return out


def absol_to_num(d, point):
    """Domain_*::absol_to_num for a spheric domain centred at the origin."""
    x, y, z = point
    r = math.sqrt(x * x + y * y + z * z)
    if d.type == NUCLEUS:
        xi = r / d.alpha
    elif d.type == SHELL:
        xi = (r - d.beta) / d.alpha
    else:
        xi = 1. + 1. / r / d.alpha
    rho = math.sqrt(x * x + y * y)
    if rho == 0:
        th, ph = (0.0 if z >= 0 else math.pi), 0.0
    else:
        th = math.atan(rho / z) if z != 0 else math.pi / 2
        ph = math.atan2(y, x)
    if th < 0:
        th += math.pi
    return xi, th, ph


def _zero_der(x):
    return not isinstance(x, np.ndarray) and x == 0.0


def _no_seed_der(d):
    if isinstance(d.der, np.ndarray):
        raise NotImplementedError("a double depending on the seeded fields combined with a field")


# ----------------------------------------------------------------- Term_eq --
class OTerm:
    """Scalar Term_eq: value (VD or float) and optional batched tangent."""

    def __init__(self, dom, val, der=None):
        self.dom, self.val, self.der = dom, val, der

    @property
    def is_double(self):
        return isinstance(self.val, float)

    def _coerce(self, o):
        if isinstance(o, OTerm):
            return o
        return OTerm(self.dom, float(o), 0.0 if self.der is not None else None)

    def __add__(self, o):
        o = self._coerce(o)
        do = self.der is not None and o.der is not None
        if self.is_double and o.is_double:
            return OTerm(self.dom, self.val + o.val, self.der + o.der if do else None)
        if self.is_double or o.is_double:
            t, dd = (o, self) if self.is_double else (self, o)
            der = None
            if do:
                _no_seed_der(dd)
                der = t.der if dd.der == 0.0 else t.der + dd.der
            return OTerm(self.dom, t.val + dd.val, der)
        return OTerm(self.dom, self.val + o.val, self.der + o.der if do else None)

    __radd__ = __add__

    def __sub__(self, o):
        o = self._coerce(o)
        do = self.der is not None and o.der is not None
        if self.is_double and o.is_double:
            return OTerm(self.dom, self.val - o.val, self.der - o.der if do else None)
        if o.is_double:
            if do:
                _no_seed_der(o)
            return OTerm(self.dom, self.val - o.val, (self.der if o.der == 0.0 else self.der - o.der) if do else None)
        if self.is_double:
            der = None
            if do:
                _no_seed_der(self)
                der = -o.der if self.der == 0.0 else o.der.rsub(self.der)
            return OTerm(self.dom, o.val.rsub(self.val), der)
        return OTerm(self.dom, self.val - o.val, self.der - o.der if do else None)

    def __rsub__(self, o):
        return self._coerce(o) - self

    def __neg__(self):
        if self.is_double:
            return OTerm(self.dom, -self.val, None if self.der is None else -self.der)
        return OTerm(self.dom, self.val * -1.0, None if self.der is None else self.der * -1.0)

    def __mul__(self, o):
        o = self._coerce(o)
        do = self.der is not None and o.der is not None
        if self.is_double and o.is_double:
            return OTerm(self.dom, self.val * o.val, self.der * o.val + self.val * o.der if do else None)
        if self.is_double or o.is_double:
            t, dd = (o, self) if self.is_double else (self, o)
            der = None
            if do:
                _no_seed_der(dd)
                der = t.der * dd.val
                if dd.der != 0.0:
                    der = der + t.val * dd.der
            return OTerm(self.dom, t.val * dd.val, der)
        return OTerm(self.dom, self.val * o.val, self.der * o.val + self.val * o.der if do else None)

    __rmul__ = __mul__

    def __truediv__(self, o):
        o = self._coerce(o)
        do = self.der is not None and o.der is not None
        if o.is_double:
            der = None
            if do:
                if self.is_double:
                    der = (self.der * o.val - self.val * o.der) / (o.val * o.val)
                else:
                    _no_seed_der(o)
                    num = self.der * o.val
                    if not _zero_der(o.der):
                        num = num - self.val * o.der
                    der = num / (o.val * o.val)
            return OTerm(self.dom, self.val / o.val, der)
        if self.is_double:
            raise NotImplementedError("double divided by a field term")
        der = None
        if do:
            der = (self.der * o.val - self.val * o.der) / (o.val * o.val)
        return OTerm(self.dom, self.val / o.val, der)

    def __pow__(self, n):
        assert isinstance(n, int) and n > 0
        r = self
        for _ in range(1, n):
            r = r * self
        return r

    def lap(self):
        return OTerm(self.dom, laplacian(self.val), None if self.der is None else laplacian(self.der))

    def exp(self):
        """Ope_exp (src/Ope_eq/ope_exp.cpp), term_eq_math.cpp exp: der = u' exp(u)."""
        v = self.val.exp()
        return OTerm(self.dom, v, None if self.der is None else self.der * v)

    def log(self):
        """Ope_log: der = u' / u."""
        v = self.val.log()
        return OTerm(self.dom, v, None if self.der is None else self.der / self.val)

    def atanh(self):
        """Ope_atanh (src/Ope_eq/ope_atanh.cpp): der = u' / (1 - u u)."""
        v = self.val.atanh()
        return OTerm(self.dom, v, None if self.der is None else self.der / (self.val * self.val).rsub(1.0))

    def ddr(self):
        """Ope_ddr (src/Ope_eq/ope_ddr.cpp, Domain::ddr in domain.cpp:1522):
        der_r twice, value and tangent."""
        return OTerm(self.dom, der_r(der_r(self.val)), None if self.der is None else der_r(der_r(self.der)))

    def dn(self, bound):
        return OTerm(self.dom, der_normal(self.val, bound), None if self.der is None else
                     (self.der if self.der.zero else der_normal(self.der, bound)))

    def partial(self, i):
        """Cartesian derivative d/dx_i (Val_domain::der_abs, i = 1, 2, 3)."""
        return OTerm(self.dom, self.val.der_abs(i), None if self.der is None else self.der.der_abs(i))

    def _functional(self, f):
        val = 0.0 if self.val.zero else float(f(self.val)[0])
        der = None
        if self.der is not None:
            der = 0.0 if self.der.zero else f(self.der)
        return OTerm(self.dom, val, der)

    def integvolume(self):
        """Ope_int_volume (src/Ope_eq/ope_int_volume.cpp)."""
        return self._functional(integ_volume)

    def integ(self, bound):
        """Ope_int (src/Ope_eq/ope_int.cpp) in the compactified domain."""
        return self._functional(lambda v: integ_surface(v, bound))

    def val_at(self, pos):
        """Ope_val (src/Ope_eq/ope_val.cpp)."""
        return self._functional(lambda v: value_at(v, pos))

    def val_point(self, num):
        """Ope_point (src/Ope_eq/ope_point.cpp)."""
        return self._functional(lambda v: summation(v, num))


# -------------------------------------------------------------- the system --
class OSystem:
    """System_of_eqs with scalar and Cartesian vector unknowns and the
    equation kinds Eq_inside (order 2), Eq_bc and Eq_matching.  An equation
    function returns one OTerm, or a list of OTerms for a vector equation
    (its rows component by component, Eq_inside::export_val)."""

    def __init__(self, doms, dom_min, dom_max):
        self.doms, self.dmin, self.dmax = doms, dom_min, dom_max
        self.vars = []       # (name, dict dom -> VD with B=1)
        self.vectors = {}    # name -> index in vars of its x component
        self.vdoubles = []   # [name, value]: unknowns that are numbers
        self.eqs = []        # (kind, dom, bound, fn_lhs, other_dom, other_bound, fn_rhs)
        self.ieqs = []       # integral-type equations: lists of parts (dom, bound, fn -> double OTerm)
        self.nbr_conditions = None

    def add_var(self, name, fields):
        self.vars.append((name, fields))

    def add_var_vector(self, name, comps):
        """add_var(name, Tensor&) with a Cartesian Vector (system_of_eqs.cpp:404):
        T[name] is the list of its three component OTerms."""
        self.vectors[name] = len(self.vars)
        for c in range(3):
            self.vars.append((f"{name}#{c + 1}", comps[c]))

    def add_var_double(self, name, value):
        """add_var(name, double&) (system_of_eqs.cpp:284)."""
        self.vdoubles.append([name, float(value)])

    def add_eq_int(self, parts):
        """An Eq_int (eq_int.cpp): its value is the sum of its parts, each a
        (dom, bound, fn(T, bound) -> double OTerm); one condition, placed
        before every other equation (sec_member, solver.cpp:49)."""
        self.ieqs.append(list(parts))

    def add_eq_int_volume(self, dmin, dmax, fn_integrand, fn_const):
        """Space_spheric::add_eq_int_volume (spheric_add_eq.cpp:81):
        sum_d integvolume(f) in every domain, minus the constant side."""
        parts = [(d, None, (lambda T, b, fn=fn_integrand: fn(T).integvolume())) for d in range(dmin, dmax + 1)]
        parts.append((dmin, None, lambda T, b: -fn_const(T)))
        self.add_eq_int(parts)

    def add_eq_val(self, dom, fn, pos):
        """add_eq_val (add_eq.cpp:343): fn vanishes at collocation point pos."""
        self.add_eq_int([(dom, None, lambda T, b: fn(T).val_at(pos))])

    def add_eq_point(self, dom, fn, point):
        """add_eq_point (add_eq.cpp:355): fn vanishes at a Cartesian point."""
        num = absol_to_num(self.doms[dom], point)
        self.add_eq_int([(dom, None, lambda T, b: fn(T).val_point(num))])

    def add_eq_inside(self, dom, fn):
        self.eqs.append(("inside", dom, None, fn, None, None, None))

    def add_eq_order(self, dom, order, fn):
        """add_eq_order (add_eq.cpp:80): Eq_order, the tau export dropping
        `order` radial coefficients; order 0 is add_eq_full (Eq_full,
        eq_full.cpp: every coefficient)."""
        self.eqs.append(("order", dom, order, fn, None, None, None))

    def add_eq_full(self, dom, fn):
        self.add_eq_order(dom, 0, fn)

    def add_eq_first_integral(self, dom_min, dom_max, fn_integ, fn_cst):
        """add_eq_first_integral (add_eq.cpp:414), Eq_first_integral
        (eq_first_integral.cpp): fn_integ minus its value at the first
        collocation point of dom_min, in every domain dom_min..dom_max, all
        coefficients; in dom_min the points of radial index 0 carry fn_cst's
        value at that first point instead."""
        self.eqs.append(("first_integral", dom_min, dom_max, fn_integ, None, None, fn_cst))

    def add_eq_bc(self, dom, bound, fn):
        self.eqs.append(("bc", dom, bound, fn, None, None, None))

    def add_eq_matching(self, dom, bound, fn_lhs, fn_rhs=None):
        other = dom + 1 if bound == OUTER_BC else dom - 1
        other_bound = INNER_BC if bound == OUTER_BC else OUTER_BC
        self.eqs.append(("matching", dom, bound, fn_lhs, other, other_bound, fn_rhs or fn_lhs))

    def _terms(self, dom, seed=None):
        """Unknowns as Term_eqs; seed = (var, dom, batch seed VD) for a field
        block, or ("double", i) for the column of double unknown i."""
        out = {}
        dseed = seed is not None and seed[0] == "double"
        for vi, (name, f) in enumerate(self.vars):
            val = f[dom]
            der = None
            if seed is not None:
                if dseed:
                    der = VD.zeros(self.doms[dom], 1)
                else:
                    sv, sd, sb = seed
                    der = sb if (vi == sv and dom == sd) else VD.zeros(self.doms[dom], sb.B)
            out[name] = OTerm(dom, val, der)
        for i, (name, v) in enumerate(self.vdoubles):
            der = None
            if seed is not None:
                der = 1.0 if (dseed and seed[1] == i) else 0.0
            out[name] = OTerm(dom, float(v), der)
        for name, first in self.vectors.items():
            out[name] = [out[self.vars[first + c][0]] for c in range(3)]
        return out

    def _value_rows(self, kind, t, dom, bound):
        """Value rows of an equation's term and the row count of each component."""
        blocks, ns = [], []
        for c in (t if isinstance(t, list) else [t]):
            v, n = self._export(kind, c.val, dom, bound)
            blocks.append(np.zeros(n) if v is None else v[0].copy())
            ns.append(len(blocks[-1]))
        return np.concatenate(blocks), ns

    def _der_rows(self, kind, t, dom, bound, ns):
        """(row offset, B x n tangent rows) of each component whose tangent is not zero."""
        off = 0
        for c, n in zip((t if isinstance(t, list) else [t]), ns):
            v, _ = self._export(kind, c.der, dom, bound)
            if v is not None:
                yield off, v
            off += n

    def _int_rows(self, seed=None, only_dom=None):
        """Values (seed None) or tangents of the integral equations."""
        out = []
        for parts in self.ieqs:
            acc = 0.0
            for (d, b, fn) in parts:
                if only_dom is not None and d != only_dom:
                    continue
                t = fn(self._terms(d, seed), b)
                acc = acc + (t.val if seed is None else t.der)
            out.append(acc)
        return out

    def _rows(self, kind, dom, base, bound):
        d = self.doms[dom]
        if kind == "inside":
            return d.export_tau(base, 2)
        if kind in ("order", "first_integral"):
            return d.export_tau(base, bound)
        return d.export_tau_boundary(base, bound)

    def _export(self, kind, vd, dom, bound, nrows_expected=None):
        d = self.doms[dom]
        if vd.zero:
            # Equation::export_der of a zero tangent skips the block (pos += ncond)
            return None, nrows_expected
        rows = self._rows(kind, dom, vd.base, bound)
        vd.coef()
        cf = vd.cf.reshape(vd.B, -1)
        M = np.zeros((len(rows), cf.shape[1]))
        for r, row in enumerate(rows):
            for idx, w in row:
                M[r, idx] += w
        return cf @ M.T, len(rows)

    def _first_integral(self, eq, seed=None):
        """Eq_first_integral::export_val (seed None) / export_der
        (eq_first_integral.cpp:44-120): per domain dom_min..dom_max, the
        B x rows block (None: exactly zero) and the row count of the value."""
        _, dmin, dmax, fn_integ, _, _, fn_cst = eq
        use_der = seed is not None
        Tmin = self._terms(dmin, seed)
        cst = fn_cst(Tmin, None)
        integ = {d: fn_integ(Tmin if d == dmin else self._terms(d, seed), None) for d in range(dmin, dmax + 1)}

        def part(t):
            return t.der if use_der else t.val

        def point0(vd):
            if vd is None or vd.zero:
                return None
            vd.coef_i()
            return vd.c[:, 0, 0, 0].copy()
        val_cst = point0(part(cst))
        val_ori = point0(part(integ[dmin]))
        blocks, ns = [], []
        for d in range(dmin, dmax + 1):
            dm = self.doms[d]
            val = integ[d].val
            nrow = len(dm.export_tau(val.base, 0))
            ns.append(nrow)
            v = part(integ[d])
            inject = d == dmin
            if v.zero and val_ori is None and not (inject and val_cst is not None):
                blocks.append(None)
                continue
            B = max(1 if v.zero else v.B, 1 if val_ori is None else len(val_ori),
                    1 if val_cst is None else len(val_cst))
            if v.zero:
                c = np.zeros((B,) + dm.np)
            else:
                v.coef_i()
                c = np.broadcast_to(v.c, (B,) + dm.np).copy()
            if val_ori is not None:
                c = c - val_ori.reshape((-1, 1, 1, 1))
            if inject:
                c[:, 0, :, :] = 0.0 if val_cst is None else val_cst.reshape((-1, 1, 1))
            base = v.base if (not v.zero and v.base.defined) else val.base
            out, n = self._export("first_integral", VD(dm, B, c=c, base=base), d, 0)
            assert n == nrow
            blocks.append(out)
        return blocks, ns

    def residual(self):
        F = [np.array([v]) for v in self._int_rows()]
        for eq in self.eqs:
            if eq[0] == "first_integral":
                blocks, ns = self._first_integral(eq)
                F.append(np.concatenate([np.zeros(n) if b is None else b[0] for b, n in zip(blocks, ns)]))
                continue
            (kind, dom, bound, fn, odom, obound, fnr) = eq
            block, _ = self._value_rows(kind, fn(self._terms(dom), bound), dom, bound)
            if kind == "matching":
                v2, _ = self._value_rows(kind, fnr(self._terms(odom), obound), odom, obound)
                block = block - v2
            F.append(block)
        F = np.concatenate(F)
        self.nbr_conditions = len(F)
        return F

    def unknown_layout(self):
        """xx_to_vars (system_of_eqs.cpp:597): variable by variable, domain by
        domain; a vector's three components inside each domain."""
        layout = []
        col = len(self.vdoubles)
        firsts = set(self.vectors.values())
        vi = 0
        while vi < len(self.vars):
            ncmp = 3 if vi in firsts else 1
            for dd in range(self.dmin, self.dmax + 1):
                for c in range(ncmp):
                    f = self.vars[vi + c][1]
                    pats = self.doms[dd].unknown_patterns(f[dd].base)
                    layout.append((vi + c, dd, col, pats))
                    col += len(pats)
            vi += ncmp
        return layout, col

    def jacobian(self, rectangular=False):
        F = self.residual()
        layout, N = self.unknown_layout()
        assert (len(F) >= N) if rectangular else (N == len(F)), (N, len(F))
        J = np.zeros((len(F), N))
        row0 = []
        nint = len(self.ieqs)
        r = nint
        for eq in self.eqs:
            kind, dom, bound, fn, odom, obound, fnr = eq
            if kind == "first_integral":
                _, ns = self._first_integral(eq)
            else:
                _, ns = self._value_rows(kind, fn(self._terms(dom), bound), dom, bound)
            row0.append((r, ns))
            r += sum(ns)

        def add_fi(e, seed, cols, sign=1.0):
            r0, ns = row0[e]
            blocks, _ = self._first_integral(self.eqs[e], seed)
            off = r0
            for b, n in zip(blocks, ns):
                if b is not None:
                    J[off:off + n, cols] += sign * (b[0] if isinstance(cols, int) else b.T)
                off += n
        # columns of the double unknowns: every equation (do_col_J, is_var_double)
        for i in range(len(self.vdoubles)):
            seed = ("double", i)
            for e, (kind, dom, bound, fn, odom, obound, fnr) in enumerate(self.eqs):
                r0, ns = row0[e]
                if kind == "first_integral":
                    add_fi(e, seed, i)
                    continue
                for off, v in self._der_rows(kind, fn(self._terms(dom, seed), bound), dom, bound, ns):
                    J[r0 + off:r0 + off + v.shape[1], i] += v[0]
                if kind == "matching":
                    for off, v in self._der_rows(kind, fnr(self._terms(odom, seed), obound), odom, obound, ns):
                        J[r0 + off:r0 + off + v.shape[1], i] -= v[0]
            for k, dv in enumerate(self._int_rows(seed)):
                J[k, i] = float(np.asarray(dv).reshape(-1)[0]) if isinstance(dv, np.ndarray) else dv
        for vi, dd, col, pats in layout:
            d = self.doms[dd]
            B = len(pats)
            seed = np.zeros((B, d.nc[0] * d.nc[1] * d.nc[2]))
            for s, p in enumerate(pats):
                for idx, w in p:
                    seed[s, idx] = w
            base = self.vars[vi][1][dd].base
            sb = VD(d, B, cf=seed.reshape((B,) + d.nc), base=base)
            for e, (kind, dom, bound, fn, odom, obound, fnr) in enumerate(self.eqs):
                r0, ns = row0[e]
                if kind == "first_integral":
                    if dom <= dd <= bound:
                        add_fi(e, (vi, dd, sb), slice(col, col + B))
                    continue
                if dom == dd:
                    t = fn(self._terms(dom, (vi, dd, sb)), bound)
                    for off, v in self._der_rows(kind, t, dom, bound, ns):
                        J[r0 + off:r0 + off + v.shape[1], col:col + B] += v.T
                if kind == "matching" and odom == dd:
                    t = fnr(self._terms(odom, (vi, dd, sb)), obound)
                    for off, v in self._der_rows(kind, t, odom, obound, ns):
                        J[r0 + off:r0 + off + v.shape[1], col:col + B] -= v.T
            for k, dv in enumerate(self._int_rows((vi, dd, sb), only_dom=dd)):
                J[k, col:col + B] += dv
        return F, J

    def update(self, x):
        """xx_to_vars then var = old - new (do_newton_seq, src_par/do_newton.cpp:558-566)."""
        layout, N = self.unknown_layout()
        for i in range(len(self.vdoubles)):
            self.vdoubles[i][1] -= x[i]
        for vi, dd, col, pats in layout:
            name, f = self.vars[vi]
            d = self.doms[dd]
            M = d.affecte_tau_matrix(f[dd].base)
            cf = (M @ x[col:col + M.shape[1]]).reshape((1,) + d.nc)
            new = VD(d, 1, cf=cf, base=f[dd].base)
            f[dd] = f[dd] - new
        for vi, (name, f) in enumerate(self.vars):
            for dd in range(len(self.doms)):
                if dd < self.dmin or dd > self.dmax:
                    if not f[dd].zero:
                        f[dd] = f[dd] - f[dd]

    def newton_step(self, precision, solve=None, gauss_newton=False):
        """One step of do_newton; gauss_newton: the SOLVER GAUSS_NEWTON branch
        (src_par/do_newton.cpp:264-311), x = (J^T J)^-1 J^T F."""
        import scipy.linalg as sla
        F, J = self.jacobian(rectangular=gauss_newton)
        err = float(np.max(np.abs(F)))
        if err < precision:
            return True, err, F, J
        if gauss_newton:
            x = sla.lu_solve(sla.lu_factor(J.T @ J), J.T @ F)
        elif solve is None:
            x = sla.lu_solve(sla.lu_factor(J), F)
        else:
            x = solve(J, F)
        self.update(x)
        return False, err, F, J


# ---------------------------------------------------------------- EOS ops --
# EOS variables (Margherita's EPSILON, PRESSURE, DENSITY, DHDRHO)
EOS_EPSILON, EOS_PRESSURE, EOS_DENSITY, EOS_DHDRHO = 0, 1, 2, 3


def polytrope(npieces=1, rhomin=1e-19, rhomax=1.0, k0=100.0, gamma_tab=(2.0,), rho_tab=(0.0,)):
    """Cold piecewise polytrope tables as Margherita_setup_polytrope builds
    them (include/EOS/standalone/setup_polytrope.cc), geometrised units."""
    g = list(gamma_tab)
    r = list(rho_tab)
    k = [k0] + [0.0] * (npieces - 1)
    eps = [0.0] * npieces
    h = [0.0] * npieces
    for i in range(1, npieces):
        k[i] = k[i - 1] * r[i] ** (g[i - 1] - g[i])
        eps[i] = eps[i - 1] + k[i - 1] * r[i] ** (g[i - 1] - 1.0) / (g[i - 1] - 1.0) - k[i] * r[i] ** (g[i] - 1.0) / (g[i] - 1.0)
        P = k[i] * r[i] ** g[i]
        e = eps[i] + P / r[i] / (g[i] - 1.0)
        h[i] = 1.0 + e + P / r[i]
    return dict(n=npieces, rhomin=rhomin, rhomax=rhomax, k=k, gamma=g, rho=r, eps=eps, h=h)


def _eos_point(e, var, hv, dh=None):
    """EOS::term_by_term / term_by_term_variation at one point
    (include/EOS/EOS.hh:67-160, cold_pwpoly_implementation.hh)."""
    def clamp(x):
        return min(max(x, e["rhomin"]), e["rhomax"])

    def piece_rho(x):
        for nn in range(1, e["n"]):
            if e["rho"][nn - 1] < x <= e["rho"][nn]:
                return nn - 1
        return e["n"] - 1
    if hv <= 1.0:
        rho, hh = e["rho"][0], 1.0
    else:
        hh = hv
        idx = e["n"] - 1
        for nn in range(1, e["n"]):
            if e["h"][nn - 1] < hv <= e["h"][nn]:
                idx = nn - 1
                break
        gm1 = e["gamma"][idx] - 1.0
        rho = (gm1 * (hv - 1.0 - e["eps"][idx]) / (e["gamma"][idx] * e["k"][idx])) ** (1.0 / gm1)
    rho = clamp(rho)
    i = piece_rho(rho)
    P = e["k"][i] * rho ** e["gamma"][i]
    epsc = e["eps"][i] + P / (rho * (e["gamma"][i] - 1.0))
    dpdrho = e["gamma"][i] * P / rho
    if dh is None:
        return [epsc, P, rho, 1.0 / hh * dpdrho][var]
    drho = rho * 1.0 / dpdrho * dh
    return [P / rho ** 2 * drho, dpdrho * drho, drho, 0.0][var]


def _eos_array(e, var, hv, dh=None):
    """_eos_point over arrays (the same branches, element by element);
    dh broadcasts against hv."""
    hv = np.asarray(hv, dtype=np.float64)
    n = e["n"]
    gam, kk, ee, hh_t, rr = (np.array(e[x], dtype=np.float64) for x in ("gamma", "k", "eps", "h", "rho"))
    above = hv > 1.0
    hh = np.where(above, hv, 1.0)
    idx = np.full(hv.shape, n - 1)
    found = np.zeros(hv.shape, bool)
    for nn in range(1, n):
        m = (~found) & (hh_t[nn - 1] < hv) & (hv <= hh_t[nn])
        idx = np.where(m, nn - 1, idx)
        found |= m
    gm1 = gam[idx] - 1.0
    with np.errstate(invalid="ignore", divide="ignore"):
        rho_a = (gm1 * (hv - 1.0 - ee[idx]) / (gam[idx] * kk[idx])) ** (1.0 / gm1)
    rho = np.where(above, rho_a, rr[0])
    rho = np.minimum(np.maximum(rho, e["rhomin"]), e["rhomax"])
    i = np.full(hv.shape, n - 1)
    found = np.zeros(hv.shape, bool)
    for nn in range(1, n):
        m = (~found) & (rr[nn - 1] < rho) & (rho <= rr[nn])
        i = np.where(m, nn - 1, i)
        found |= m
    P = kk[i] * rho ** gam[i]
    epsc = ee[i] + P / (rho * (gam[i] - 1.0))
    dpdrho = gam[i] * P / rho
    if dh is None:
        return [epsc, P, rho, 1.0 / hh * dpdrho][var]
    drho = rho * 1.0 / dpdrho * dh
    return [P / rho ** 2 * drho, dpdrho * drho, drho, np.zeros_like(drho)][var]


def eos_term(t, e, var):
    """Ope_user with EOS<eos, var>::action on an OTerm (value and tangent)."""
    v = t.val
    if v.zero:
        val = v
    else:
        v.coef_i()
        val = VD(v.dom, 1, c=_eos_array(e, var, v.c), base=v.base)
    der = None
    if t.der is not None:
        d = t.der
        if d.zero or v.zero:
            der = VD.zeros(d.dom, d.B)
        else:
            d.coef_i()
            der = VD(d.dom, d.B, c=_eos_array(e, var, v.c[0][None], d.c), base=d.base)
    return OTerm(t.dom, val, der)


def newton_linesearch_step(sysm, precision, ntrymax=10, stepmax=1.0):
    """do_newton_with_linesearch (src_par/do_newton.cpp:454-516; compute_f
    :594, update_fields :667, compute_old_and_var :676), restated on OSystem.
    Returns (converged, error, last lambda)."""
    import scipy.linalg as sla
    F, J = sysm.jacobian()
    err = float(np.max(np.abs(F)))
    if err < precision:
        return True, err, 0.0
    fold = float(np.sum(F * F))
    slope = -2.0 * fold
    assert slope < 0.0
    p = sla.lu_solve(sla.lu_factor(J), F)
    pmax = float(np.max(p))
    if pmax > stepmax:
        p = p * (stepmax / pmax)
    layout, N = sysm.unknown_layout()
    old = {vi: {dd: f[dd] for dd in range(len(sysm.doms))} for vi, (name, f) in enumerate(sysm.vars)}
    pv = {vi: dict(old[vi]) for vi in old}  # xx_to_vars leaves the other domains as they are
    for vi, dd, col, pats in layout:
        name, f = sysm.vars[vi]
        d = sysm.doms[dd]
        M = d.affecte_tau_matrix(f[dd].base)
        cf = (M @ p[col:col + M.shape[1]]).reshape((1,) + d.nc)
        pv[vi][dd] = VD(d, 1, cf=cf, base=f[dd].base)

    def update_fields(lam):
        for vi, (name, f) in enumerate(sysm.vars):
            for dd in range(len(sysm.doms)):
                f[dd] = old[vi][dd] - pv[vi][dd] * lam

    lambdamin, alpha = 1.0e-10, 1.0e-4
    lam, lamtmp, lam2, f2 = 1.0, 0.0, 0.0, 0.0
    for itry in range(1, ntrymax + 1):
        update_fields(lam)
        Fn = sysm.residual()
        f = float(np.sum(Fn * Fn))
        if f <= 5.0e-13:
            break
        if f <= fold + alpha * lam * slope or lam <= lambdamin:
            break
        if lam == 1.0:
            lamtmp = -0.5 * slope / (f - fold - slope)
        else:
            rhs1 = f - fold - lam * slope
            rhs2 = f2 - fold - lam2 * slope
            a = (rhs1 / lam ** 2 - rhs2 / lam2 ** 2) / (lam - lam2)
            b = (-lam2 * rhs1 / lam ** 2 + lam * rhs2 / lam2 ** 2) / (lam - lam2)
            delta = b * b - 3.0 * a * slope
            assert delta >= 0.0
            lamtmp = (-b + math.sqrt(delta)) / (3.0 * a)
            if lamtmp > 0.5 * lam:
                lamtmp = 0.5 * lam
        lam2, f2 = lam, f
        lam = max(lamtmp, 0.1 * lam)
        if itry == ntrymax:
            update_fields(lam)
    return False, err, lam


def scalar_field(doms, value_fn):
    """A Scalar with std_base, values from value_fn(dom) -> (n0,n1,n2) array."""
    out = {}
    for d in doms:
        out[d.num] = VD(d, 1, c=np.asarray(value_fn(d), dtype=float)[None].copy(), base=d.std_base())
    return out


def val_point(doms, field, point):
    """Scalar::val_point: evaluate the spectral expansion at a Cartesian point."""
    x, y, z = point
    r = math.sqrt(x * x + y * y + z * z)
    for d in doms:
        rin = 0.0 if d.type == NUCLEUS else (d.beta - d.alpha if d.type == SHELL else -0.5 / d.alpha)
        rout = d.alpha if d.type == NUCLEUS else (d.beta + d.alpha if d.type == SHELL else math.inf)
        if rin - 1e-12 <= r <= rout + 1e-12:
            break
    if d.type == NUCLEUS:
        xi = r / d.alpha
    elif d.type == SHELL:
        xi = (r - d.beta) / d.alpha
    else:
        xi = 1. + 1. / r / d.alpha
    rho = math.sqrt(x * x + y * y)
    if rho == 0:
        th, ph = (0.0 if z >= 0 else math.pi), 0.0
    else:
        th = math.atan(rho / z) if z != 0 else math.pi / 2
        ph = math.atan2(y, x)
    if th < 0:
        th += math.pi
    v = field[d.num]
    v.coef()
    cf = v.cf[0]
    b = v.base
    nc0, nc1, nc2 = d.nc
    # Base_spectral::summation: r first, then theta, then phi
    lines = np.zeros((nc1, nc2))
    for j in range(nc1):
        for k in range(nc2):
            lines[j, k] = S.summation_1d(int(b.r[j, k]), xi, cf[:, j, k])
    tvals = np.array([S.summation_1d(int(b.t[k]), th, lines[:, k]) for k in range(nc2)])
    return S.summation_1d(int(b.p), ph, tvals)
