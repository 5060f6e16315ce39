"""Writes known_answers.json: the analytic solutions that the reference's own
programs print, evaluated in closed form at the points those programs use.

* tutorials/tuto5.cpp: Lap(F) = 0, dn(F) + F/(2a) = 0 at r = 1, F = 1 at
  infinity, a = 1  ->  F = 1 + a/r, printed at one point.
* tutorials/tuto6.cpp: Lap(P) + grad(P).grad(P) = 0, dn(P) + 1/(2a) = 0 at
  r = 1, P = 0 at infinity  ->  P = log(1 + a/r).
* codes/Seq_version/schwarz.cpp:45-90: conformal factor of a Schwarzschild
  slice, P = 1 + aa/r with aa = 1.323, checked on 99 points of a ray in the
  equatorial plane (phi = -2.349) from 1.01 aa to 5 x 2.9861 aa.

Nothing of the reference is run: the values come from the closed forms.
Run:  python tests/golden/make_known_answers.py
"""
import json
import math
from pathlib import Path

POINT = (1.3873, -0.827, 0.982)  # the evaluation point used by the tutorials' checks


def main():
    r = math.sqrt(sum(c * c for c in POINT))
    out = {
        "tuto5": {"a": 1.0, "bounds": [1.0, 2.0, 4.0], "res": [13, 5, 4], "point": list(POINT),
                  "value": 1.0 + 1.0 / r},
        "tuto6": {"a": 1.0, "bounds": [1.0, 2.0, 4.0], "res": [13, 5, 4], "point": list(POINT),
                  "value": math.log(1.0 + 1.0 / r)},
    }
    aa = 1.323
    resol, tet, phi = 100, math.pi / 2.0, -2.349
    xxmin, xxmax = aa * 1.01, 2.9861 * aa * 5
    step = (xxmax - xxmin) / resol
    pts, vals = [], []
    xx = xxmin + step
    for _ in range(resol - 1):
        pts.append([xx * math.sin(tet) * math.cos(phi), xx * math.sin(tet) * math.sin(phi), xx * math.cos(tet)])
        vals.append(1.0 + aa / xx)
        xx += step
    out["schwarz"] = {"aa": aa, "bounds": [aa, 1.7557 * aa, 2.9861 * aa], "res": [13, 5, 4], "points": pts,
                      "values": vals, "max_error": 1e-8}
    path = Path(__file__).with_name("known_answers.json")
    path.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {path}")


if __name__ == "__main__":
    main()
