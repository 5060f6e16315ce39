"""ctypes binding of ``libkadath_gb300.so`` (the C ABI in include/kadath_gb300.h).

The shared library is the product: every numeric call goes through it to
CUDA kernels.  If it cannot be loaded this module raises -- there is no
Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libkadath_gb300.so"

KD_OK, KD_ERR_ARG, KD_ERR_CUDA, KD_ERR_SINGULAR, KD_ERR_NOCONV, KD_ERR_TIMEOUT, KD_ERR_UNSUPPORTED, KD_ERR_STATE = range(8)

STATUS_NAMES = {0: "KD_OK", 1: "KD_ERR_ARG", 2: "KD_ERR_CUDA", 3: "KD_ERR_SINGULAR", 4: "KD_ERR_NOCONV",
                5: "KD_ERR_TIMEOUT", 6: "KD_ERR_UNSUPPORTED", 7: "KD_ERR_STATE"}


class KadathError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class TransformDesc(C.Structure):
    _fields_ = [("nbr_points", C.c_int * 3), ("nbr_coefs", C.c_int * 3), ("base_r", C.POINTER(C.c_int)),
                ("base_t", C.POINTER(C.c_int)), ("base_p", C.c_int), ("batch", C.c_int),
                ("in_", C.c_void_p), ("out", C.c_void_p)]


_lib = None


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads the library (building it in-tree first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        if not build_if_missing:
            raise KadathError(KD_ERR_STATE, f"{LIB_PATH} missing; run kadath_frontera_gb300.build.build()")
        from . import build as _build
        _build.build()
    lib = C.CDLL(str(LIB_PATH))
    _declare(lib)
    _lib = lib
    return lib


def _declare(lib: C.CDLL) -> None:
    P, I, D, V = C.c_void_p, C.c_int, C.c_double, None
    IP, DP = C.POINTER(C.c_int), C.POINTER(C.c_double)
    sig = {
        "kd_ctx_create": (I, [C.POINTER(P), I]),
        "kd_ctx_destroy": (I, [P]),
        "kd_ctx_set_sm_budget": (I, [P, I]),
        "kd_ctx_set_wait_limit": (I, [P, C.c_double]),
        "kd_ctx_stall_waits": (I, [P, I]),
        "kd_ctx_autotune": (I, [P, C.c_char_p, I]),
        "kd_ctx_autotune_stats": (I, [P, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
        "kd_last_error": (C.c_char_p, [P]),
        "kd_ctx_synchronize": (I, [P]),
        "kd_ctx_launch_count": (C.c_longlong, [P]),
        "kd_coef_many": (I, [P, I, C.POINTER(TransformDesc)]),
        "kd_coef_i_many": (I, [P, I, C.POINTER(TransformDesc)]),
        "kd_coef_host": (I, [P, C.POINTER(TransformDesc)]),
        "kd_coef_i_host": (I, [P, C.POINTER(TransformDesc)]),
        "kd_ope_1d": (I, [P, I, I, C.POINTER(TransformDesc), IP, IP, IP]),
        "kd_matrix_1d": (I, [P, I, I, I, I, DP, IP]),
        "kd_ctx_stream": (P, [P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _declare_more(lib)


def _declare_more(lib: C.CDLL) -> None:
    """Signatures of the system/solver entry points (added as they exist)."""
    for name, (res, args) in EXTRA_SIGNATURES.items():
        if hasattr(lib, name):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args


EXTRA_SIGNATURES: dict = {}


def check(status: int, ctx=None) -> None:
    if status != KD_OK:
        msg = load().kd_last_error(ctx).decode() if ctx is not None else ""
        raise KadathError(status, msg)


class Context:
    """Owns one kd_ctx (one GPU, one CUDA stream)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        st = self.lib.kd_ctx_create(C.byref(h), device)
        self.h = h
        if st != KD_OK:
            msg = self.lib.kd_last_error(h).decode() if h else ""
            raise KadathError(st, f"cannot create GPU context on device {device}: {msg}")

    def check(self, st: int) -> None:
        if st != KD_OK:
            raise KadathError(st, self.lib.kd_last_error(self.h).decode())

    def synchronize(self) -> None:
        self.check(self.lib.kd_ctx_synchronize(self.h))

    def set_sm_budget(self, sms: int) -> None:
        """At most `sms` SMs for this context's grid-wide solver kernels
        (0: all of them), for contexts that run side by side."""
        self.check(self.lib.kd_ctx_set_sm_budget(self.h, int(sms)))

    def set_wait_limit(self, seconds: float) -> None:
        """Limit of one grid-barrier wait of the solver's cooperative kernels
        (KD_ERR_TIMEOUT when it runs out)."""
        self.check(self.lib.kd_ctx_set_wait_limit(self.h, float(seconds)))

    def stall_waits(self, on: bool) -> None:
        """Failure injection for tests: no grid barrier completes while on."""
        self.check(self.lib.kd_ctx_stall_waits(self.h, 1 if on else 0))

    def autotune(self, path=None, mode: int = 1) -> None:
        """Launch shapes of the spectral line passes from the JSON table at
        `path` (mode 1), also timing the shape classes it lacks and saving it
        (mode 2), or the fixed rule (mode 0)."""
        p = None if path is None else str(path).encode()
        self.check(self.lib.kd_ctx_autotune(self.h, p, int(mode)))

    def autotune_stats(self) -> dict:
        e, t, h = C.c_longlong(), C.c_longlong(), C.c_longlong()
        self.check(self.lib.kd_ctx_autotune_stats(self.h, C.byref(e), C.byref(t), C.byref(h)))
        return {"entries": e.value, "tuned": t.value, "hits": h.value}

    @property
    def launches(self) -> int:
        return int(self.lib.kd_ctx_launch_count(self.h))

    @property
    def stream_ptr(self) -> int:
        """cudaStream_t of this context (as an integer handle)."""
        return int(self.lib.kd_ctx_stream(self.h) or 0)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.kd_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(int(os.environ.get("KD_DEVICE", "0")))
    return _default_ctx
