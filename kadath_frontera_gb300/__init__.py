"""GB300-native Newton-Raphson hot path for Kadath/FUKA.

The numeric work runs in the in-tree CUDA library ``libkadath_gb300.so``
(C ABI: include/kadath_gb300.h).  This package holds the Python mirror of
the reference's user-facing classes on top of that ABI.
"""
from ._lib import Context, KadathError, default_context, load  # noqa: F401

__all__ = ["Context", "KadathError", "default_context", "load"]
