"""The C-ABI library loads and exports every entry point declared in
include/kadath_gb300.h (no GPU needed: nothing is called)."""
import re
from pathlib import Path

from kadath_frontera_gb300 import _lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "kadath_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(kd_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
