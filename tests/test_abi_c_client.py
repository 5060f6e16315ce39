"""A plain C client of the C ABI: include/kadath_gb300.h compiles as strict
C99 (no C++ constructs leak into the header) and every function it declares
links against libkadath_gb300.so.  The client takes the address of each
entry point and runs without calling any of them, so no GPU is needed --
this is the check a reference-side binding (cgo, a C shim beside
do_newton.cpp) relies on."""
import os
import shutil
import subprocess

import pytest

from kadath_frontera_gb300 import _lib
from test_abi_symbols import HEADER, declared_functions


def test_header_compiles_as_c99_and_every_entry_point_links(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    lib = _lib.LIB_PATH
    if not lib.exists():
        _lib.load()
    names = declared_functions()
    assert len(names) > 40
    src = ['#include "kadath_gb300.h"', "#include <stdio.h>", "typedef void (*fp)(void);",
           "static const fp table[] = {"]
    src += ["  (fp)%s," % n for n in names]
    src += ["};", "int main(void) {", "  size_t n = 0, i;",
            "  for (i = 0; i < sizeof table / sizeof table[0]; i++) n += table[i] != 0;",
            '  printf("%lu\\n", (unsigned long)n);', "  return 0;", "}"]
    c_file = tmp_path / "client.c"
    c_file.write_text("\n".join(src) + "\n")
    exe = tmp_path / "client"
    cmd = ["gcc", "-std=c99", "-Wall", "-Werror", "-Wno-pedantic", "-I", str(HEADER.parent), str(c_file),
           "-o", str(exe), "-L", str(lib.parent), "-lkadath_gb300", "-Wl,-rpath," + str(lib.parent)]
    out = subprocess.run(cmd, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, env=dict(os.environ))
    assert run.returncode == 0, run.stderr
    assert int(run.stdout.strip()) == len(names)


def test_header_is_self_contained_c(tmp_path):
    """The header alone, first in a translation unit, compiles as C99 with
    pedantic warnings as errors (its own includes, no C++ keywords)."""
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    c_file = tmp_path / "only_header.c"
    c_file.write_text('#include "kadath_gb300.h"\nint kd_client_unused;\n')
    out = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only", "-I",
                          str(HEADER.parent), str(c_file)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
