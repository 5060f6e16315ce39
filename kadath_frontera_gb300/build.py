"""Builds the in-tree shared library ``libkadath_gb300.so`` for sm_103a.

Every translation unit under ``csrc/`` is compiled in parallel with nvcc
(``-gencode arch=compute_103a,code=sm_103a -lineinfo``) and linked into one
shared library next to this file.  Objects go to ``_build/`` (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libkadath_gb300.so"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo", f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build kadath_frontera_gb300")
    return cand


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _obj(src: Path) -> Path:
    return BUILD / (src.name + ".o")


def _stamp() -> str:
    h = hashlib.sha256()
    for p in sorted(list(CSRC.glob("*")) + list(INCLUDE.glob("*.h"))):
        if p.is_file():
            h.update(p.name.encode())
            h.update(p.read_bytes())
    h.update(" ".join(ARCH + COMMON).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compiles (if sources changed) and returns the path of the library."""
    stamp_file = BUILD / "stamp"
    stamp = _stamp()
    if not force and LIB.exists() and stamp_file.exists() and stamp_file.read_text() == stamp:
        return LIB
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    srcs = _sources()

    def compile_one(src: Path) -> None:
        cmd = [nvcc, *ARCH, *COMMON, "-c", str(src), "-o", str(_obj(src))]
        if src.suffix == ".cu" and verbose:
            cmd += ["-Xptxas", "-v"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
        if verbose and res.stderr:
            sys.stderr.write(res.stderr)

    workers = min(len(srcs), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *[str(_obj(s)) for s in srcs], "-lcublas", "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    stamp_file.write_text(stamp)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
