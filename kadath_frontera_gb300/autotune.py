"""Builds the autotuner's table of line-pass launch shapes on this GPU.

    python -m kadath_frontera_gb300.autotune [--out PATH]

Solves the workloads the benchmark runs (the star in component and index
form, the toy, the TOV star, and one star at each resolution of the batched
solves) with the context's autotuner in mode 2: every shape class of a
line-pass launch met outside a graph capture is timed once, and the table is
written to PATH (default: tuning/line_passes_gb300.json in this package, the
table `bench.py` loads).  Shapes change no result bit, so the table only
changes times.
"""
from __future__ import annotations

import argparse
from pathlib import Path

DEFAULT_TABLE = Path(__file__).resolve().parent / "tuning" / "line_passes_gb300.json"


def build_table(out: Path = DEFAULT_TABLE, device: int = 0) -> dict:
    from . import workloads
    from ._lib import Context
    out = Path(out)
    out.parent.mkdir(parents=True, exist_ok=True)
    if out.exists():
        out.unlink()
    ctx = Context(device)
    ctx.autotune(out, mode=2)
    cases = [workloads.star(ctx=ctx), workloads.star_vector(ctx=ctx), workloads.toy(ctx=ctx),
             workloads.ns_tov(ctx=ctx)]
    for nr in (9, 11, 13, 15, 17):
        cases.append(workloads.star(res=(nr, workloads.batch_ntheta(nr), 4), ctx=ctx))
    from .kadath import KD_LU_TF32_IR
    for wl in cases:
        workloads.solve(wl, lu_mode=KD_LU_TF32_IR)
    return ctx.autotune_stats()


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--out", default=str(DEFAULT_TABLE))
    args = ap.parse_args(argv)
    stats = build_table(Path(args.out))
    print(f"{stats['entries']} shape classes in {args.out} ({stats['tuned']} timed)")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
