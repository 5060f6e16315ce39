"""Builds oracle/_ref: the reference's own sources compiled where they lie
against this project's FFTW/GSL/LAPACK/MPI stand-ins (oracle/Makefile.ref),
with the golden-vector drivers of oracle/ref_drivers/.  Test infrastructure:
the reference's sources exist only on the machine that generates the
fixtures, so elsewhere this does nothing and returns False."""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF = Path(os.environ.get("REF", "/root/reference"))


def build(quiet: bool = True) -> bool:
    if not (REF / "src" / "Coef" / "coef_1d.cpp").exists():
        return False
    cmd = ["make", "-f", str(HERE / "Makefile.ref"), "-j", str(os.cpu_count() or 4), f"REF={REF}"]
    subprocess.run(cmd, check=True, cwd=HERE.parent, stdout=subprocess.DEVNULL if quiet else None)
    return True


if __name__ == "__main__":
    print("built oracle/_ref" if build(quiet=False) else "reference sources absent: nothing to build")
