"""Python mirror of Kadath's user-facing classes, driving the GB300 library.

Names, argument meaning and error behaviour follow the reference:

* ``Space_spheric``  -- src/Space/Spheric/space_spheric.cpp:25 (plus the
  add_eq / add_inner_bc / add_outer_bc / add_matching helpers of
  src/Space/Spheric/spheric_add_eq.cpp)
* ``Scalar``         -- include/scalar.hpp:67 (one Val_domain per domain)
* ``System_of_eqs``  -- include/system_of_eqs.hpp:54 (add_var, add_cst,
  add_def, add_eq_inside, add_eq_bc, add_eq_matching, sec_member,
  check_equations, do_col_J, do_newton)

Every numerical operation runs in the CUDA library through the C ABI.
Where the reference aborts, these raise ``KadathError`` with the same message.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import KadathError, default_context

CHEB_TYPE = 1
OUTER_BC, INNER_BC = 0, 1
NEWTON_RAPHSON, GAUSS_NEWTON = 0, 1  # System_of_eqs::SOLVER (include/system_of_eqs.hpp:134)

KD_LU_FP64, KD_LU_TF32_IR, KD_LU_FP32_IR = 0, 1, 2
KD_EOS_EPSILON, KD_EOS_PRESSURE, KD_EOS_DENSITY, KD_EOS_DHDRHO = 0, 1, 2, 3


class NewtonOpts(C.Structure):
    _fields_ = [("precision", C.c_double), ("lu_mode", C.c_int), ("gmres_tol", C.c_double), ("max_refine", C.c_int),
                ("graph_capture", C.c_int), ("gmres_restarts", C.c_int), ("pivot_every_step", C.c_int)]


class AdjointReport(C.Structure):
    _fields_ = [("reused_factors", C.c_int), ("refine_iters", C.c_int), ("rel_residual", C.c_double),
                ("t_assembly_ms", C.c_double), ("t_solve_ms", C.c_double)]


class NewtonReport(C.Structure):
    _fields_ = [("error", C.c_double), ("converged", C.c_int), ("n", C.c_int), ("t_residual_ms", C.c_double),
                ("t_assembly_ms", C.c_double), ("t_factor_ms", C.c_double), ("t_solve_ms", C.c_double),
                ("t_update_ms", C.c_double), ("refine_iters", C.c_int), ("refine_rel_residual", C.c_double),
                ("kernel_launches", C.c_longlong), ("fp64_fallback", C.c_int), ("static_pivots", C.c_int)]

    def as_dict(self):
        return {f[0]: getattr(self, f[0]) for f in self._fields_}


def _declare_system(lib):
    P, I, D = C.c_void_p, C.c_int, C.c_double
    IP, DP = C.POINTER(C.c_int), C.POINTER(C.c_double)
    sig = {
        "kd_space_spheric_create": (I, [P, DP, IP, DP, I, I, C.POINTER(P)]),
        "kd_space_destroy": (I, [P]),
        "kd_space_nbr_domains": (I, [P, IP]),
        "kd_space_domain_info": (I, [P, I, IP, IP, IP, DP, DP]),
        "kd_space_radius": (I, [P, I, DP]),
        "kd_space_cart": (I, [P, I, I, DP]),
        "kd_space_std_base": (I, [P, I, IP, IP, IP]),
        "kd_field_create": (I, [P, C.POINTER(P)]),
        "kd_field_destroy": (I, [P]),
        "kd_field_set_value": (I, [P, D]),
        "kd_field_std_base": (I, [P]),
        "kd_field_set_conf": (I, [P, I, DP]),
        "kd_field_cart_base": (I, [P, I]),
        "kd_field_copy": (I, [P, P]),
        "kd_ctx_profile_enable": (I, [P, I]),
        "kd_ctx_profile_read": (I, [P, DP, C.POINTER(C.c_longlong), DP]),
        "kd_field_get_conf": (I, [P, I, DP]),
        "kd_field_get_coef": (I, [P, I, DP]),
        "kd_field_get_base": (I, [P, I, IP, IP, IP]),
        "kd_system_create": (I, [P, I, I, C.POINTER(P)]),
        "kd_system_destroy": (I, [P]),
        "kd_system_add_var": (I, [P, C.c_char_p, P]),
        "kd_system_add_var_double": (I, [P, C.c_char_p, D]),
        "kd_system_get_var_double": (I, [P, C.c_char_p, DP]),
        "kd_system_add_cst": (I, [P, C.c_char_p, D]),
        "kd_system_add_cst_field": (I, [P, C.c_char_p, P]),
        "kd_system_add_def": (I, [P, I, C.c_char_p]),
        "kd_system_add_var_vector": (I, [P, C.c_char_p, P, P, P]),
        "kd_file_open": (I, [C.c_char_p, C.c_char_p, C.POINTER(P)]),
        "kd_file_close": (I, [P]),
        "kd_space_save": (I, [P, P]),
        "kd_space_load": (I, [P, P, I, C.POINTER(P)]),
        "kd_field_save": (I, [P, P]),
        "kd_field_load": (I, [P, P]),
        "kd_vector_save": (I, [P, P, P, I, P]),
        "kd_vector_load": (I, [P, P, P, C.POINTER(C.c_int), P]),
        "kd_system_add_eq_order": (I, [P, I, I, C.c_char_p]),
        "kd_system_add_eq_full": (I, [P, I, C.c_char_p]),
        "kd_system_add_eq_first_integral": (I, [P, I, I, C.c_char_p, C.c_char_p]),
        "kd_system_add_cst_vector": (I, [P, C.c_char_p, P, P, P]),
        "kd_system_set_metric_flat": (I, [P, C.c_char_p]),
        "kd_system_add_eq_inside": (I, [P, I, C.c_char_p]),
        "kd_system_add_eq_bc": (I, [P, I, I, C.c_char_p]),
        "kd_system_add_eq_matching": (I, [P, I, I, C.c_char_p]),
        "kd_system_add_eq_int_volume": (I, [P, I, I, C.c_char_p]),
        "kd_system_add_eq_int_inf": (I, [P, C.c_char_p]),
        "kd_system_add_eq_val": (I, [P, I, C.c_char_p, IP]),
        "kd_system_add_eq_point": (I, [P, I, C.c_char_p, DP]),
        "kd_system_sizes": (I, [P, IP, IP]),
        "kd_system_n_equations": (I, [P, IP]),
        "kd_system_residual": (I, [P, DP]),
        "kd_system_check_equations": (I, [P, DP]),
        "kd_system_jacobian": (I, [P, DP]),
        "kd_system_cache_tangents": (I, [P, I]),
        "kd_system_graph_stats": (I, [P, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
        "kd_system_jacobian_graph_stats": (I, [P, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
        "kd_system_jx": (I, [P, DP, DP]),
        "kd_system_jacobian_device": (I, [P, P, C.c_longlong]),
        "kd_system_update": (I, [P, DP]),
        "kd_newton_step": (I, [P, C.POINTER(NewtonOpts), C.POINTER(NewtonReport)]),
        "kd_system_reset_pivot_order": (I, [P]),
        "kd_stage_solve": (I, [P, C.POINTER(NewtonOpts), I, C.c_char_p, I, C.POINTER(P), IP, DP]),
        "kd_field_regrid": (I, [P, P]),
        "kd_newton_step_gauss_newton": (I, [P, C.POINTER(NewtonOpts), C.POINTER(NewtonReport)]),
        "kd_newton_step_linesearch": (I, [P, C.POINTER(NewtonOpts), I, D, C.POINTER(NewtonReport), DP]),
        "kd_system_set_cst": (I, [P, C.c_char_p, D]),
        "kd_system_add_ope_eos": (I, [P, C.c_char_p, I, I, D, D, D, DP, DP]),
        "kd_field_val_point": (I, [P, DP, DP]),
        "kd_fields_val_points": (I, [I, C.POINTER(P), C.c_longlong, DP, DP]),
        "kd_fields_val_points_device": (I, [I, C.POINTER(P), C.c_longlong, P, P]),
        "kd_system_val_point_gradient": (I, [P, C.c_char_p, DP, DP]),
        "kd_system_dres_dcst": (I, [P, C.c_char_p, DP]),
        "kd_adjoint": (I, [P, DP, C.c_char_p, D, DP, DP]),
        "kd_adjoint_ex": (I, [P, DP, C.c_char_p, D, I, DP, DP, P]),
        "kd_system_integral_gradient": (I, [P, I, I, I, C.c_char_p, DP, DP]),
        "kd_lu_create": (I, [P, C.POINTER(P)]),
        "kd_lu_destroy": (I, [P]),
        "kd_lu_factor": (I, [P, P, C.c_longlong, I, I]),
        "kd_lu_solve": (I, [P, P, I]),
        "kd_lu_stats": (I, [P, DP, DP, IP, DP]),
        "kd_lu_set_refinement": (I, [P, D, I, I]),
        "kd_lu_set_pivot_reuse": (I, [P, I]),
        "kd_lu_pivot_info": (I, [P, IP, IP]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args


_declared = False


def _L():
    global _declared
    lib = _lib.load()
    if not _declared:
        _declare_system(lib)
        _declared = True
    return lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class KadathFile:
    """A save file in Kadath's binary format, written or read item by item
    in order, as with the reference's FILE* (fopen(name, "w") / "r")."""

    def __init__(self, path, mode="r"):
        m = {"r": "rb", "w": "wb", "rb": "rb", "wb": "wb"}[mode]
        h = C.c_void_p()
        st = _L().kd_file_open(str(path).encode(), m.encode(), C.byref(h))
        if st != 0:
            raise KadathError(st, f"cannot open {path}")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            _L().kd_file_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


CON, COV = 1, -1


class Space_spheric:
    """Space_spheric(type_coloc, center, res, bounds, withzec=True)."""

    def __init__(self, type_coloc, center, res, bounds, withzec=True, ctx=None):
        if type_coloc != CHEB_TYPE:
            raise KadathError(_lib.KD_ERR_UNSUPPORTED, "only CHEB_TYPE collocation is supported")
        self.ctx = ctx or default_context()
        lib = _L()
        c = np.asarray(center, dtype=np.float64)
        r = np.asarray(res, dtype=np.int32)
        b = np.asarray(bounds, dtype=np.float64)
        h = C.c_void_p()
        self.ctx.check(lib.kd_space_spheric_create(self.ctx.h, _dp(c), _ip(r), _dp(b), len(b), int(withzec), C.byref(h)))
        self.h = h
        self.res = tuple(int(v) for v in res)
        self.bounds = tuple(float(v) for v in bounds)

    @classmethod
    def from_file(cls, f: "KadathFile", withzec=True, ctx=None):
        """Space_spheric(FILE*, withzec)."""
        self = cls.__new__(cls)
        self.ctx = ctx or default_context()
        h = C.c_void_p()
        self.ctx.check(_L().kd_space_load(self.ctx.h, f.h, 1 if withzec else 0, C.byref(h)))
        self.h = h
        info = [self.domain_info(d) for d in range(self.get_nbr_domains())]
        self.res = tuple(int(v) for v in info[0]["nbr_points"])
        bounds = [info[0]["alpha"]]
        for d in info[1:]:
            if d["type"] == 2:  # shell: beta + alpha
                bounds.append(d["beta"] + d["alpha"])
        self.bounds = tuple(bounds)
        return self

    def save(self, f: "KadathFile"):
        """Space_spheric::save."""
        self.ctx.check(_L().kd_space_save(self.h, f.h))

    def get_nbr_domains(self):
        n = C.c_int()
        _L().kd_space_nbr_domains(self.h, C.byref(n))
        return n.value

    def domain_info(self, dom):
        t = C.c_int()
        npts = np.zeros(3, np.int32)
        nc = np.zeros(3, np.int32)
        a, b = C.c_double(), C.c_double()
        self.ctx.check(_L().kd_space_domain_info(self.h, dom, C.byref(t), _ip(npts), _ip(nc), C.byref(a), C.byref(b)))
        return {"type": t.value, "nbr_points": tuple(npts), "nbr_coefs": tuple(nc), "alpha": a.value, "beta": b.value}

    def get_radius(self, dom):
        info = self.domain_info(dom)
        out = np.zeros(info["nbr_points"])
        self.ctx.check(_L().kd_space_radius(self.h, dom, _dp(out)))
        return out

    def get_cart(self, dom, c):
        info = self.domain_info(dom)
        out = np.zeros(info["nbr_points"])
        self.ctx.check(_L().kd_space_cart(self.h, dom, c - 1, _dp(out)))
        return out

    # spheric_add_eq.cpp helpers
    def add_inner_bc(self, syst, eq):
        syst.add_eq_bc(syst.dom_min, INNER_BC, eq)

    def add_outer_bc(self, syst, eq):
        syst.add_eq_bc(syst.dom_max, OUTER_BC, eq)

    def add_matching(self, syst, eq):
        for dd in range(syst.dom_min, syst.dom_max):
            syst.add_eq_matching(dd, OUTER_BC, eq)

    def add_eq_int_volume(self, syst, eq):
        """Space_spheric::add_eq_int_volume: "integvolume(f) = c" over every
        domain of the space."""
        syst.add_eq_int_volume(0, self.get_nbr_domains() - 1, eq)

    def add_eq_full(self, syst, eq):
        """Space_spheric::add_eq_full: Eq_full in every domain of the system."""
        for dd in range(syst.dom_min, syst.dom_max + 1):
            syst.add_eq_full(dd, eq)

    def add_eq_ori(self, syst, eq):
        """Space_spheric::add_eq_ori: eq vanishes at the origin (the first
        collocation point of the nucleus)."""
        syst.add_eq_val(0, eq, (0, 0, 0))

    def add_eq(self, syst, eq, rac=None, rac_der=None):
        if rac is None:
            for dd in range(syst.dom_min, syst.dom_max + 1):
                syst.add_eq_inside(dd, eq)
            return
        for dd in range(syst.dom_min, syst.dom_max):
            syst.add_eq_inside(dd, eq)
            syst.add_eq_matching(dd, OUTER_BC, rac)
            syst.add_eq_matching(dd, OUTER_BC, rac_der)
        syst.add_eq_inside(syst.dom_max, eq)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                _L().kd_space_destroy(self.h)
        except Exception:
            pass


def val_points(fields, xyz):
    """Values of one or several Scalars of one space at Cartesian points
    xyz (array (n, 3)), evaluated on the GPU: an array (nfields, n), NaN for
    points in no domain (Scalar::val_point for many points)."""
    fields = list(fields)
    pts = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).reshape(-1, 3))
    out = np.zeros((len(fields), pts.shape[0]))
    arr = (C.c_void_p * len(fields))(*[f.h for f in fields])
    fields[0].space.ctx.check(_L().kd_fields_val_points(len(fields), arr, pts.shape[0], _dp(pts), _dp(out)))
    return out


def val_points_device(fields, d_xyz, d_out, npts):
    """val_points with device pointers (d_xyz: 3 npts doubles, d_out:
    nfields npts doubles), on the fields' context stream."""
    fields = list(fields)
    arr = (C.c_void_p * len(fields))(*[f.h for f in fields])
    fields[0].space.ctx.check(_L().kd_fields_val_points_device(len(fields), arr, int(npts), C.c_void_p(d_xyz), C.c_void_p(d_out)))


class Scalar:
    """Scalar(space); ``field = v`` is ``set_value(v)``."""

    def __init__(self, space: Space_spheric, value=None):
        self.space = space
        h = C.c_void_p()
        space.ctx.check(_L().kd_field_create(space.h, C.byref(h)))
        self.h = h
        if value is not None:
            self.set_value(value)

    def set_value(self, v):
        self.space.ctx.check(_L().kd_field_set_value(self.h, float(v)))
        return self

    def std_base(self):
        self.space.ctx.check(_L().kd_field_std_base(self.h))
        return self

    def copy_from(self, other: "Scalar"):
        """Scalar assignment (device to device)."""
        self.space.ctx.check(_L().kd_field_copy(self.h, other.h))
        return self

    def val_point(self, point):
        """Scalar::val_point: the value at a Cartesian point."""
        pt = np.ascontiguousarray(point, dtype=np.float64)
        out = C.c_double()
        self.space.ctx.check(_L().kd_field_val_point(self.h, _dp(pt), C.byref(out)))
        return out.value

    @classmethod
    def from_file(cls, space: "Space_spheric", f: "KadathFile"):
        """Scalar(space, FILE*)."""
        s = cls(space)
        space.ctx.check(_L().kd_field_load(s.h, f.h))
        return s

    def save(self, f: "KadathFile"):
        """Scalar::save."""
        self.space.ctx.check(_L().kd_field_save(self.h, f.h))

    def regrid_from(self, src: "Scalar"):
        """This field = src evaluated at the collocation points of this
        field's space (same domains, other resolution): the FUKA regrid,
        on the GPU.  The basis follows src's kind (standard or
        anti-symmetric)."""
        self.space.ctx.check(_L().kd_field_regrid(self.h, src.h))
        return self

    def std_base_cart(self, c):
        """Basis of the Cartesian component c = 1, 2, 3 (x, y, z) of a vector."""
        self.space.ctx.check(_L().kd_field_cart_base(self.h, int(c) - 1))
        return self

    def set_domain(self, dom, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        info = self.space.domain_info(dom)
        if v.shape != tuple(info["nbr_points"]):
            raise KadathError(_lib.KD_ERR_ARG, f"expected shape {info['nbr_points']}")
        self.space.ctx.check(_L().kd_field_set_conf(self.h, dom, _dp(v)))

    def get_domain(self, dom):
        """Values at the collocation points of domain dom."""
        info = self.space.domain_info(dom)
        out = np.zeros(info["nbr_points"])
        self.space.ctx.check(_L().kd_field_get_conf(self.h, dom, _dp(out)))
        return out

    def get_coef(self, dom):
        info = self.space.domain_info(dom)
        out = np.zeros(info["nbr_coefs"])
        self.space.ctx.check(_L().kd_field_get_coef(self.h, dom, _dp(out)))
        return out

    def get_base(self, dom):
        info = self.space.domain_info(dom)
        nc = info["nbr_coefs"]
        r = np.zeros(nc[1] * nc[2], np.int32)
        t = np.zeros(nc[2], np.int32)
        p = C.c_int()
        self.space.ctx.check(_L().kd_field_get_base(self.h, dom, _ip(r), _ip(t), C.byref(p)))
        return r.reshape(nc[1], nc[2]), t, p.value

    def __del__(self):
        try:
            if getattr(self, "h", None):
                _L().kd_field_destroy(self.h)
        except Exception:
            pass


CARTESIAN_BASIS = 0


class Vector:
    """Vector(space, CARTESIAN_BASIS): three Scalar components, v(1) = x,
    v(2) = y, v(3) = z (Tensor with valence 1, include/tensor.hpp)."""

    def __init__(self, space: Space_spheric, type_tensor=None, basis=CARTESIAN_BASIS):
        if basis != CARTESIAN_BASIS:
            raise KadathError(_lib.KD_ERR_UNSUPPORTED, "only the Cartesian tensorial basis is supported")
        self.space = space
        self.cmp = [Scalar(space) for _ in range(3)]

    def __call__(self, i):
        return self.cmp[i - 1]

    def set(self, i):
        return self.cmp[i - 1]

    def std_base(self):
        """Each component gets the basis of its Cartesian component."""
        for c in range(3):
            self.cmp[c].std_base_cart(c + 1)
        return self

    def set_value(self, v):
        for c in self.cmp:
            c.set_value(v)
        return self

    def save(self, f: "KadathFile", type_index=CON):
        """Tensor::save of the vector (Cartesian basis)."""
        self.space.ctx.check(_L().kd_vector_save(*[c.h for c in self.cmp], int(type_index), f.h))

    @classmethod
    def from_file(cls, space: "Space_spheric", f: "KadathFile"):
        """Vector(space, FILE*); the index type read is kept in type_index."""
        v = cls(space)
        ti = C.c_int()
        space.ctx.check(_L().kd_vector_load(*[c.h for c in v.cmp], C.byref(ti), f.h))
        v.type_index = ti.value
        return v

    def copy_from(self, other: "Vector"):
        for a, b in zip(self.cmp, other.cmp):
            a.copy_from(b)
        return self


class Metric_flat:
    """Metric_flat(space, basis) with a Cartesian basis; set_system(syst,
    name) gives the system its covariant derivatives D_i / D^i and the
    metric tensor `name` (src/Metric/metric_flat.cpp:501)."""

    def __init__(self, space: Space_spheric, basis=CARTESIAN_BASIS):
        if basis != CARTESIAN_BASIS:
            raise KadathError(_lib.KD_ERR_UNSUPPORTED, "only the Cartesian tensorial basis is supported")
        self.space = space

    def set_system(self, syst: "System_of_eqs", name):
        syst.ctx.check(_L().kd_system_set_metric_flat(syst.h, name.encode()))


class System_of_eqs:
    """System_of_eqs(space, dom_min, dom_max)."""

    def __init__(self, space: Space_spheric, dom_min=None, dom_max=None):
        if dom_min is None:
            dom_min, dom_max = 0, space.get_nbr_domains() - 1
        elif dom_max is None:
            dom_max = dom_min
        self.space = space
        self.ctx = space.ctx
        self.dom_min, self.dom_max = dom_min, dom_max
        h = C.c_void_p()
        self.ctx.check(_L().kd_system_create(space.h, dom_min, dom_max, C.byref(h)))
        self.h = h
        self._keep = []
        self.lu_mode = KD_LU_FP64
        self.graph_capture = False
        self.last_report = None
        self._J = None

    def get_dom_min(self):
        return self.dom_min

    def get_dom_max(self):
        return self.dom_max

    def add_var(self, name, field):
        if isinstance(field, Scalar):
            self._keep.append(field)
            self.ctx.check(_L().kd_system_add_var(self.h, name.encode(), field.h))
        elif isinstance(field, Vector):
            self._keep.append(field)
            self.ctx.check(_L().kd_system_add_var_vector(self.h, name.encode(), *[c.h for c in field.cmp]))
        else:
            self.ctx.check(_L().kd_system_add_var_double(self.h, name.encode(), float(field)))

    def get_var_double(self, name):
        v = C.c_double()
        self.ctx.check(_L().kd_system_get_var_double(self.h, name.encode(), C.byref(v)))
        return v.value

    def add_cst(self, name, value):
        if isinstance(value, Scalar):
            self._keep.append(value)
            self.ctx.check(_L().kd_system_add_cst_field(self.h, name.encode(), value.h))
        elif isinstance(value, Vector):
            self._keep.append(value)
            self.ctx.check(_L().kd_system_add_cst_vector(self.h, name.encode(), *[c.h for c in value.cmp]))
        else:
            self.ctx.check(_L().kd_system_add_cst(self.h, name.encode(), float(value)))

    def add_def(self, *args):
        dom, text = (-1, args[0]) if len(args) == 1 else args
        self.ctx.check(_L().kd_system_add_def(self.h, int(dom), text.encode()))

    def add_eq_inside(self, dom, eq):
        self.ctx.check(_L().kd_system_add_eq_inside(self.h, dom, eq.encode()))

    def add_eq_bc(self, dom, bound, eq):
        self.ctx.check(_L().kd_system_add_eq_bc(self.h, dom, bound, eq.encode()))

    def add_eq_order(self, dom, order, eq):
        self.ctx.check(_L().kd_system_add_eq_order(self.h, dom, int(order), eq.encode()))

    def add_eq_full(self, dom, eq):
        self.ctx.check(_L().kd_system_add_eq_full(self.h, dom, eq.encode()))

    def add_eq_first_integral(self, dom_min, dom_max, integ_part, cst_part):
        self.ctx.check(_L().kd_system_add_eq_first_integral(self.h, dom_min, dom_max, integ_part.encode(),
                                                             cst_part.encode()))

    def add_eq_matching(self, dom, bound, eq):
        self.ctx.check(_L().kd_system_add_eq_matching(self.h, dom, bound, eq.encode()))

    def add_eq_int_volume(self, dom_min, dom_max, eq):
        """Integral equation "integvolume(f) = c" over domains dom_min..dom_max."""
        self.ctx.check(_L().kd_system_add_eq_int_volume(self.h, dom_min, dom_max, eq.encode()))

    def add_eq_int_inf(self, eq):
        """Integral equation "integ(f) = c", integ() at infinity."""
        self.ctx.check(_L().kd_system_add_eq_int_inf(self.h, eq.encode()))

    def add_eq_val(self, dom, eq, pos):
        """eq vanishes at collocation point pos = (i, j, k) of dom."""
        p = (C.c_int * 3)(*[int(v) for v in pos])
        self.ctx.check(_L().kd_system_add_eq_val(self.h, dom, eq.encode(), p))

    def add_eq_point(self, dom, eq, point):
        """eq vanishes at a Cartesian point, evaluated in domain dom."""
        p = (C.c_double * 3)(*[float(v) for v in point])
        self.ctx.check(_L().kd_system_add_eq_point(self.h, dom, eq.encode(), p))

    def sizes(self):
        nu, nc = C.c_int(), C.c_int()
        self.ctx.check(_L().kd_system_sizes(self.h, C.byref(nu), C.byref(nc)))
        return nu.value, nc.value

    def get_nbr_unknowns(self):
        return self.sizes()[0]

    def get_nbr_conditions(self):
        return self.sizes()[1]

    def sec_member(self):
        n = self.get_nbr_conditions()
        out = np.zeros(n)
        self.ctx.check(_L().kd_system_residual(self.h, _dp(out)))
        return out

    def check_equations(self):
        neq = C.c_int()
        self.ctx.check(_L().kd_system_n_equations(self.h, C.byref(neq)))
        out = np.zeros(neq.value)
        self.ctx.check(_L().kd_system_check_equations(self.h, _dp(out)))
        return out

    def jacobian(self):
        """All do_col_J columns at once: the dense N x N Jacobian."""
        n = self.get_nbr_unknowns()
        out = np.zeros((n, n), order="F")
        self.ctx.check(_L().kd_system_jacobian(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return np.asfortranarray(out.reshape((n, n), order="F"))

    def do_JX(self, x):
        """System_of_eqs::do_JX: J x without forming J."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.get_nbr_unknowns())
        self.ctx.check(_L().kd_system_jx(self.h, _dp(x), _dp(y)))
        return y

    def add_ope_eos(self, name, var, gamma_tab=(2.0,), rho_tab=(0.0,), k0=100.0, rhomin=1e-19, rhomax=1.0):
        """add_ope(name, &EOS<Cold_PWPoly, var>::action): name(h) in equations.
        var: KD_EOS_EPSILON / PRESSURE / DENSITY / DHDRHO.  Defaults: the
        Gamma = 2, K = 100 polytrope of eos/gam2.polytrope."""
        g = np.ascontiguousarray(gamma_tab, dtype=np.float64)
        r = np.ascontiguousarray(rho_tab, dtype=np.float64)
        self.ctx.check(_L().kd_system_add_ope_eos(self.h, name.encode(), int(var), len(g), float(rhomin),
                                                  float(rhomax), float(k0), _dp(g), _dp(r)))

    def set_cst(self, name, value):
        """Changes a double constant registered with add_cst(name, double)."""
        self.ctx.check(_L().kd_system_set_cst(self.h, name.encode(), float(value)))

    def val_point_gradient(self, var, point):
        """dQ/dy for Q = var's value at a point, y the unknown vector."""
        pt = np.ascontiguousarray(point, dtype=np.float64)
        g = np.zeros(self.get_nbr_unknowns())
        self.ctx.check(_L().kd_system_val_point_gradient(self.h, var.encode(), _dp(pt), _dp(g)))
        return g

    def dres_dcst(self, name):
        """dF/dp for the double constant p = name."""
        fp = np.zeros(self.get_nbr_unknowns())
        self.ctx.check(_L().kd_system_dres_dcst(self.h, name.encode(), _dp(fp)))
        return fp

    def integral_gradient(self, expr, kind="inf", domains=None):
        """(Q, dQ/dy) for an integral observable: kind "inf", the integral at
        infinity of expr (the left side of add_eq_int_inf, e.g.
        "integ(dn(P))"); kind "volume", expr summed over domains
        (dmin, dmax) (the left side of add_eq_int_volume, e.g.
        "integvolume(psi^5)")."""
        k = {"volume": 0, "inf": 1}[kind]
        dmin, dmax = domains if domains is not None else (0, 0)
        g = np.zeros(self.get_nbr_unknowns())
        q = C.c_double()
        self.ctx.check(_L().kd_system_integral_gradient(self.h, k, int(dmin), int(dmax), expr.encode(), C.byref(q),
                                                        _dp(g)))
        return q.value, g

    def adjoint(self, g, cst, dq_explicit=0.0, reuse_factors=False):
        """dQ/dp at the current (converged) fields: dq_explicit - lambda.dF/dp
        with J^T lambda = g.  Returns (dQ/dp, lambda).  With reuse_factors,
        the mixed-precision factors of the last Newton step precondition
        GMRES on J^T instead of a new FP64 factorisation (last_adjoint_report
        says which ran)."""
        g = np.ascontiguousarray(g, dtype=np.float64)
        lam = np.zeros(self.get_nbr_unknowns())
        out = C.c_double()
        rep = AdjointReport()
        self.ctx.check(_L().kd_adjoint_ex(self.h, _dp(g), cst.encode(), float(dq_explicit), 1 if reuse_factors else 0,
                                          C.byref(out), _dp(lam), C.byref(rep)))
        self.last_adjoint_report = {f: getattr(rep, f) for f, _ in AdjointReport._fields_}
        return out.value, lam

    def cache_tangents(self, on=True):
        """Keep the tangents of iterate-independent subtrees between Jacobian
        assemblies (on by default); off frees them."""
        self.ctx.check(_L().kd_system_cache_tangents(self.h, 1 if on else 0))

    def do_col_J(self, cc):
        """One column of the Jacobian (System_of_eqs::do_col_J)."""
        if self._J is None:
            self._J = self.jacobian()
        return self._J[:, cc].copy()

    def xx_to_vars_update(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        self.ctx.check(_L().kd_system_update(self.h, _dp(x)))
        self._J = None

    def do_newton(self, precision, lu_mode=None, gmres_tol=1e-14, max_refine=50, solver=None, graph=None,
                  gmres_restarts=4, pivot_every_step=False):
        """System_of_eqs::do_newton(precision, error, solver): returns
        (converged, error); solver NEWTON_RAPHSON (default) or GAUSS_NEWTON.
        graph: replay the residual's value pass from a CUDA graph (default:
        the system's graph_capture attribute).  A mixed-precision solve that
        ends above a relative residual of 1e-10 is redone with the FP64 LU
        (last_report["fp64_fallback"]).  Later mixed-precision steps reuse the
        pivot order of the last pivoted factorisation unless pivot_every_step
        (last_report["static_pivots"])."""
        g = self.graph_capture if graph is None else graph
        opts = NewtonOpts(precision, self.lu_mode if lu_mode is None else lu_mode, gmres_tol, max_refine,
                          1 if g else 0, gmres_restarts, 1 if pivot_every_step else 0)
        rep = NewtonReport()
        fn = _L().kd_newton_step_gauss_newton if solver == GAUSS_NEWTON else _L().kd_newton_step
        self.ctx.check(fn(self.h, C.byref(opts), C.byref(rep)))
        self.last_report = rep.as_dict()
        self._J = None
        return bool(rep.converged), rep.error

    def stage_solve(self, precision, max_iter=20, checkpoint=None, fields=(), lu_mode=None, gmres_tol=1e-14,
                    max_refine=50):
        """One stage of a FUKA solver: do_newton until converged, the space
        and `fields` (Scalars) written to `checkpoint` after every update and
        at the end.  Returns (updates made, last pre-step error)."""
        opts = NewtonOpts(precision, self.lu_mode if lu_mode is None else lu_mode, gmres_tol, max_refine,
                          1 if self.graph_capture else 0, 4, 0)
        handles = [f.h.value if isinstance(f.h, C.c_void_p) else f.h for f in fields]
        arr = (C.c_void_p * max(len(handles), 1))(*handles)
        it = C.c_int()
        err = C.c_double()
        path = str(checkpoint).encode() if checkpoint else None
        self.ctx.check(_L().kd_stage_solve(self.h, C.byref(opts), int(max_iter), path, len(handles),
                                           C.cast(arr, C.POINTER(C.c_void_p)), C.byref(it), C.byref(err)))
        self._J = None
        return it.value, err.value

    def reset_pivot_order(self):
        """The next mixed-precision step factors with partial pivoting."""
        self.ctx.check(_L().kd_system_reset_pivot_order(self.h))

    def graph_stats(self):
        """(captures, replays) of the residual's value pass."""
        c, r = C.c_longlong(), C.c_longlong()
        self.ctx.check(_L().kd_system_graph_stats(self.h, C.byref(c), C.byref(r)))
        return c.value, r.value

    def jacobian_graph_stats(self):
        """(captures, replays) of the Jacobian's seed passes."""
        c, r = C.c_longlong(), C.c_longlong()
        self.ctx.check(_L().kd_system_jacobian_graph_stats(self.h, C.byref(c), C.byref(r)))
        return c.value, r.value

    def do_newton_with_linesearch(self, precision, ntrymax=10, stepmax=1.0, lu_mode=None, gmres_tol=1e-14,
                                  max_refine=50):
        """System_of_eqs::do_newton_with_linesearch: returns (converged, error,
        last lambda)."""
        opts = NewtonOpts(precision, self.lu_mode if lu_mode is None else lu_mode, gmres_tol, max_refine, 0, 4, 0)
        rep = NewtonReport()
        lam = C.c_double()
        self.ctx.check(_L().kd_newton_step_linesearch(self.h, C.byref(opts), ntrymax, stepmax, C.byref(rep),
                                                      C.byref(lam)))
        self.last_report = rep.as_dict()
        self._J = None
        return bool(rep.converged), rep.error, lam.value

    def __del__(self):
        try:
            if getattr(self, "h", None):
                _L().kd_system_destroy(self.h)
        except Exception:
            pass


class DenseLU:
    """GPU LU of a device matrix (torch tensor, float64, column-major view)."""

    def __init__(self, ctx=None):
        self.ctx = ctx or default_context()
        h = C.c_void_p()
        self.ctx.check(_L().kd_lu_create(self.ctx.h, C.byref(h)))
        self.h = h

    def factor(self, dA_ptr, ld, n, mode=KD_LU_FP64):
        self.ctx.check(_L().kd_lu_factor(self.h, C.c_void_p(dA_ptr), ld, n, mode))

    def solve(self, db_ptr, trans=0):
        self.ctx.check(_L().kd_lu_solve(self.h, C.c_void_p(db_ptr), trans))

    def set_pivot_reuse(self, on=True):
        """Static pivoting: later factorisations reuse the last pivot order."""
        self.ctx.check(_L().kd_lu_set_pivot_reuse(self.h, 1 if on else 0))

    def pivot_info(self):
        """(static pivots used, fallback to partial pivoting) of the last call."""
        a, b = C.c_int(), C.c_int()
        self.ctx.check(_L().kd_lu_pivot_info(self.h, C.byref(a), C.byref(b)))
        return bool(a.value), bool(b.value)

    def set_refinement(self, tol=1e-14, iters=50, restarts=4):
        """GMRES(iters) with at most `restarts` cycles down to tol (mixed modes)."""
        self.ctx.check(_L().kd_lu_set_refinement(self.h, float(tol), int(iters), int(restarts)))

    def stats(self):
        a, b, r = C.c_double(), C.c_double(), C.c_double()
        it = C.c_int()
        _L().kd_lu_stats(self.h, C.byref(a), C.byref(b), C.byref(it), C.byref(r))
        return {"t_factor_ms": a.value, "t_solve_ms": b.value, "refine_iters": it.value, "rel_residual": r.value}

    def __del__(self):
        try:
            if getattr(self, "h", None):
                _L().kd_lu_destroy(self.h)
        except Exception:
            pass


PROFILE_CATEGORIES = ("transform", "elementwise", "tau_gather", "lu_panel", "lu_swap_trsm", "lu_gemm", "lu_solve",
                      "refine_matvec", "lu_panel_static")


def profile_enable(ctx, on=True):
    ctx.check(_L().kd_ctx_profile_enable(ctx.h, int(on)))


def profile_read(ctx):
    """Per-category (ms, launches, work) of the launches since profile_enable."""
    n = len(PROFILE_CATEGORIES)
    ms = np.zeros(n)
    cnt = np.zeros(n, dtype=np.int64)
    work = np.zeros(n)
    ctx.check(_L().kd_ctx_profile_read(ctx.h, _dp(ms), cnt.ctypes.data_as(C.POINTER(C.c_longlong)), _dp(work)))
    return {name: {"ms": float(ms[i]), "launches": int(cnt[i]), "work": float(work[i])}
            for i, name in enumerate(PROFILE_CATEGORIES)}
