"""Writes the golden vectors produced by the reference's OWN code.

The reference's sources (src/** and src_par/do_newton.cpp) are compiled where
they lie by oracle/Makefile.ref against this project's stand-ins for FFTW,
GSL, LAPACK and single-rank MPI (oracle/ref_shims/), together with two
drivers written against the reference's public API (oracle/ref_drivers/).
This script runs those drivers and stores what the reference computes as
small .npz fixtures next to it:

* ref_spectral_1d.npz -- matrices of coef_1d / coef_i_1d (src/Coef) and of the
  eleven src/Ope_1d operators for every basis and several line lengths, with
  the output basis each operator returns;
* ref_coef3d.npz -- Base_spectral::coef / coef_i (src/Coef/coef.cpp:96,
  coef_i.cpp:96) of seeded fields in the nucleus, shell and compactified
  domain, for the standard, anti-symmetric and Cartesian-component bases;
* ref_coef3_bases.npz -- Base_spectral::coef / coef_i with the bispheric
  domains' bases (COS / SIN in phi, CHEB_EVEN / CHEB_ODD in chi, CHEB in eta)
  and with the COSSIN_EVEN / COSSIN_ODD phi bases (oracle/ref_drivers/
  ref_coef3.cpp);
* ref_toy.npz -- the CPU-runnable configuration (nucleus, shell, compact,
  (13, 7, 4); Lap(psi) + 2 pi rho psi^5 = 0): sec_member at the initial
  guess, Jacobian columns from do_col_J, do_JX of a seeded vector, and every
  do_newton_seq iterate with its pre-step error;
* ref_funcs.npz, ref_funcs2.npz -- the same system at (9, 5, 4) with cos,
  sin, cosh, sinh of a double constant, atanh of the field and ddr
  (FUNCS_EQUATION), and with lap2, multrsint and divrsint (FUNCS2_EQUATION);
* ref_star_<nr><nt><np>.npz -- the isolated star with the shift as a
  Cartesian vector in index notation (the equations of
  kadath_frontera_gb300.workloads.STAR_VECTOR_EQUATIONS), at (9, 5, 4) with
  columns and J x, and at the timed size (13, 9, 4), N = 12,331, with the
  residual and every Newton iterate.

The inputs that are not constants (rho, and the frozen matter E, E + 2S) are
evaluated here on the oracle's collocation radii and stored in the fixtures,
so that the product's tests feed bit-identical inputs.

Needs the reference's sources (REF, default /root/reference) and g++; the
fixtures it writes are committed, so tests never need either.

    python tests/golden/make_ref_vectors.py [--only toy,star954,...]
"""
from __future__ import annotations

import argparse
import math
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import kadath as K  # noqa: E402
from oracle import spectral as S  # noqa: E402

REF = os.environ.get("REF", "/root/reference")
REF_BIN = ROOT / "oracle" / "_ref"

STAR_R, STAR_K, STAR_RHOC = 8.0, 100.0, 1.28e-3
STAR_BOUNDS = (STAR_R, 12.0, 16.0, 24.0, 32.0)
STAR_VECTOR_EQUATIONS = {  # the product's workloads.STAR_VECTOR_EQUATIONS
    "P": "Lap(P) + 2*pi*E/P = 0",
    "NP": "Lap(NP) - 2*pi*NP*E2S/P^2 = 0",
    "bet": "D_j D^j bet^i + D^i D_j bet^j / 3 = 0",
}
TOY_EQUATION = "Lap(psi) + 2*pi*rho*psi^5 = 0"


def build():
    from oracle import build_ref
    if not build_ref.build():
        raise SystemExit(f"the reference's sources are not at {REF}")


def run_spec(spec: str, workdir: Path):
    """Runs the driver; returns the reference's own printed timings of each
    Newton step (do_newton_seq's "Loading the matrix" and "Inverting the
    matrix" lines, seconds) as an array of (assembly, LU) pairs."""
    (workdir / "case.spec").write_text(spec)
    t = time.time()
    r = subprocess.run([str(REF_BIN / "ref_newton"), "case.spec"], cwd=workdir, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"ref_newton failed ({r.returncode}):\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    print(f"  ref_newton: {time.time() - t:.1f} s", flush=True)
    load = [float(ln.split(":")[1].split()[0]) for ln in r.stdout.splitlines() if ln.startswith("Loading the matrix")]
    inv = [float(ln.split(":")[1].split()[0]) for ln in r.stdout.splitlines() if ln.startswith("Inverting the matrix")]
    return np.array(list(zip(load, inv)))


def load(workdir: Path, name: str) -> np.ndarray:
    return np.fromfile(workdir / name, dtype="<f8")


# ------------------------------------------------------------------ 1-D --

OPS = [S.OP_COEF, S.OP_COEF_I, S.OP_DER, S.OP_MULT_SIN, S.OP_DIV_SIN, S.OP_MULT_COS, S.OP_DIV_COS, S.OP_MULT_X,
       S.OP_DIV_X, S.OP_MULT_XM1, S.OP_DIV_XM1, S.OP_DIV_XP1, S.OP_DIV_1MX2]
PHI_BASES = (S.COSSIN, S.COSSIN_EVEN, S.COSSIN_ODD)


def spectral_requests():
    """(op, base, line, n_in, n_out) for every pair the oracle accepts."""
    out = []
    for base in S.ALL_BASES:
        # phi lines hold an even number of points (with an odd number the
        # reference's coef_i_1d_cossin leaves one DFT input slot unset,
        # src/Coef/coef_i_1d.cpp:229-233); r and theta lines an odd number
        sizes = (4, 6, 8, 12, 16) if base in PHI_BASES else (5, 7, 9, 13, 17)
        for n in sizes:
            for op in OPS:
                if base in PHI_BASES:
                    if op == S.OP_COEF:
                        req = (op, base, n + 2, n, n + 2)
                    elif op == S.OP_COEF_I:
                        req = (op, base, n + 2, n + 2, n)
                    else:
                        req = (op, base, n + 2, n + 2, n + 2)
                else:
                    req = (op, base, n, n, n)
                try:  # only what the oracle restates (the reference aborts on the rest)
                    S.matrix_1d(op, base, req[3], req[4])
                except Exception:
                    continue
                out.append(req)
    return out


def make_spectral(dest: Path):
    reqs = spectral_requests()
    arrays = {}
    skipped = []
    for req in reqs:
        r = subprocess.run([str(REF_BIN / "ref_spectral")], input=" ".join(map(str, req)) + "\n",
                           capture_output=True, text=True)
        if r.returncode != 0 or not r.stdout.strip():
            skipped.append(req)  # the reference rejects this (operator, basis) pair
            continue
        vals = r.stdout.split()
        op, base, line, nin, nout = req
        key = f"op{op}_b{base}_n{nin}_m{nout}"
        arrays[key] = np.array([float(v) for v in vals[1:]]).reshape(nout, nin)
        arrays[key + "_base"] = np.array(int(vals[0]))
    np.savez_compressed(dest, **arrays)
    print(f"  {len(arrays) // 2} matrices; the reference rejects {skipped}")


# ------------------------------------------------------------------ 3-D --

def base_kind_list():
    return ["std", "anti", "xcart", "ycart", "zcart"]


def make_coef3d(dest: Path, res=(13, 7, 4), bounds=(1.0, 2.0)):
    rng = np.random.default_rng(20260)
    doms = K.space_spheric(res, list(bounds))
    npts = [int(np.prod(d.np)) for d in doms]
    ncfs = [int(np.prod(d.nc)) for d in doms]
    arrays = {"res": np.array(res), "bounds": np.array(bounds)}
    head = f"space {res[0]} {res[1]} {res[2]} {len(bounds)} " + " ".join(map(repr, bounds)) + "\n"
    with tempfile.TemporaryDirectory() as tmp:
        w = Path(tmp)
        spec = head
        for kind in base_kind_list():
            x = rng.standard_normal(sum(npts))
            c = rng.standard_normal(sum(ncfs))
            x.astype("<f8").tofile(w / f"x_{kind}.bin")
            c.astype("<f8").tofile(w / f"c_{kind}.bin")
            arrays[f"values_{kind}"] = x
            arrays[f"coefs_in_{kind}"] = c
            spec += f"scalar f_{kind} {kind} x_{kind}.bin\n"
            spec += f"dump_coefs f_{kind} cf_{kind}.bin\n"
            spec += f"scalar_c g_{kind} {kind} c_{kind}.bin\n"
            spec += f"dump_conf g_{kind} v_{kind}.bin\n"
        run_spec(spec, w)
        for kind in base_kind_list():
            arrays[f"coef_{kind}"] = load(w, f"cf_{kind}.bin")
            arrays[f"coef_i_{kind}"] = load(w, f"v_{kind}.bin")
    np.savez_compressed(dest, **arrays)


# ------------------------------------------------------------- systems --

def toy_rho(doms):
    vals = []
    for d in doms:
        r = d.radius()
        v = np.zeros_like(r)
        fin = np.isfinite(r)
        v[fin] = 0.05 * np.exp(-r[fin] ** 2 / 0.25)
        vals.append(v.ravel())
    return vals


def star_matter(doms, rho_c=STAR_RHOC):
    E, E2S = [], []
    for d in doms:
        r = d.radius()
        rho = np.zeros_like(r)
        if d.num == 0:
            x = np.pi * r / STAR_R
            safe = np.where(x > 0, x, 1.0)
            rho = rho_c * np.where(x > 0, np.sin(x) / safe, 1.0)
        e = rho * (1 + STAR_K * rho)
        s = 3 * STAR_K * rho * rho
        E.append(e.ravel())
        E2S.append((e + 2 * s).ravel())
    return E, E2S


def system_dumps(spec_body, w: Path, n_unknowns, cols, seed, newton=True):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(n_unknowns)
    x.astype("<f8").tofile(w / "x.bin")
    spec = spec_body + "dump_residual F0.bin\n"
    if cols is not None:
        spec += "dump_cols cols.bin " + " ".join(map(str, cols)) + "\n"
        spec += "dump_jx x.bin jx.bin\n"
    if newton:
        spec += "newton 1e-10 12 it\n"
    timings = run_spec(spec, w)
    out = {"F0": load(w, "F0.bin")}
    if newton:
        # seconds per step as the reference prints them, on the machine that
        # made the fixture (assembly on one core; LU through the stand-in)
        out["ref_step_seconds"] = timings
    if cols is not None:
        out["cols"] = np.array(cols)
        out["J_cols"] = load(w, "cols.bin").reshape(len(cols), -1)
        out["x"] = x
        out["Jx"] = load(w, "jx.bin")
    if newton:
        errs = load(w, "it_errors.bin")
        out["errors"] = errs
        out["iterates"] = np.stack([load(w, f"it_step{k}.bin") for k in range(len(errs) - 1)])
    return out


def make_toy(dest: Path, res=(13, 7, 4), equation=TOY_EQUATION, extra_csts=()):
    doms = K.space_spheric(res, [1.0, 2.0])
    rho = toy_rho(doms)
    nd = len(doms)
    N = 941 if res == (13, 7, 4) else None
    with tempfile.TemporaryDirectory() as tmp:
        w = Path(tmp)
        np.concatenate(rho).astype("<f8").tofile(w / "rho.bin")
        body = f"space {res[0]} {res[1]} {res[2]} 2 1.0 2.0\nsystem 0 {nd - 1}\n"
        body += "scalar psi std 1\nscalar rho std rho.bin\nvar psi\ncst rho\n"
        body += f"cstd pi {math.pi!r}\n"
        for name, value in extra_csts:
            body += f"cstd {name} {value!r}\n"
        for d in range(nd):
            body += f"inside {d} | {equation}\n"
        for d in range(nd - 1):
            body += f"matching {d} 1 | psi\nmatching {d} 1 | dn(psi)\n"
        body += f"bc {nd - 1} 1 | psi = 1\n"
        # size of the system from a first residual
        (w / "case.spec").write_text(body + "dump_residual F0.bin\n")
        run_spec(body + "dump_residual F0.bin\n", w)
        N = len(load(w, "F0.bin"))
        cols = sorted(set(np.linspace(0, N - 1, 24).astype(int).tolist()))
        out = system_dumps(body, w, N, cols, seed=7)
    out["res"] = np.array(res)
    out["rho"] = np.concatenate(rho)
    out["equation"] = np.array(equation)
    for name, value in extra_csts:
        out["cst_" + name] = np.array(value)
    np.savez_compressed(dest, **out)
    print(f"  N = {N}, errors {out['errors']}")


# cos, sin, cosh, sinh of a double constant, atanh of a field and ddr
# (src/Ope_eq/ope_cos.cpp, ope_sin.cpp, ope_cosh.cpp, ope_sinh.cpp,
# ope_atanh.cpp, ope_ddr.cpp).  With a field argument the reference's cos,
# sin, cosh and sinh give a value without a basis, which its equations
# cannot use, so those appear here on numbers only.
FUNCS_EQUATION = "Lap(psi) + 2*pi*rho*psi^5*cos(amp) + rho*atanh(psi/4)*sinh(amp) + 0.01*sin(amp)*cosh(amp)*ddr(psi) = 0"
# lap2 (Ope_lap2, Domain_*::laplacian2 with m = 0), multrsint, divrsint
FUNCS2_EQUATION = "Lap(psi) + 2*pi*rho*psi^5 + 0.01*lap2(psi)*cos(amp) + 0.01*divrsint(multrsint(psi)) = 0"


def make_star(dest: Path, res, with_cols):
    doms = K.space_spheric(res, list(STAR_BOUNDS))
    nd = len(doms)
    E, E2S = star_matter(doms)
    with tempfile.TemporaryDirectory() as tmp:
        w = Path(tmp)
        np.concatenate(E).astype("<f8").tofile(w / "E.bin")
        np.concatenate(E2S).astype("<f8").tofile(w / "E2S.bin")
        body = f"space {res[0]} {res[1]} {res[2]} {len(STAR_BOUNDS)} " + " ".join(map(repr, STAR_BOUNDS)) + "\n"
        body += f"system 0 {nd - 1}\nmetric_flat f\n"
        body += "scalar P std 1\nscalar NP std 1\nvector bet 0\nscalar E std E.bin\nscalar E2S std E2S.bin\n"
        body += "var P\nvar NP\nvar bet\n"
        body += f"cstd pi {math.pi!r}\ncst E\ncst E2S\n"
        for d in range(nd):
            for nm in ("P", "NP", "bet"):
                body += f"inside {d} | {STAR_VECTOR_EQUATIONS[nm]}\n"
        for d in range(nd - 1):
            for nm in ("P", "NP", "bet^i"):
                body += f"matching {d} 1 | {nm}\nmatching {d} 1 | dn({nm})\n"
        body += f"bc {nd - 1} 1 | P = 1\nbc {nd - 1} 1 | NP = 1\nbc {nd - 1} 1 | bet^i = 0\n"
        run_spec(body + "dump_residual F0.bin\n", w)
        N = len(load(w, "F0.bin"))
        cols = sorted(set(np.linspace(0, N - 1, 32).astype(int).tolist())) if with_cols else None
        out = system_dumps(body, w, N, cols, seed=11)
    out["res"] = np.array(res)
    out["E"] = np.concatenate(E)
    out["E2S"] = np.concatenate(E2S)
    np.savez_compressed(dest, **out)
    print(f"  N = {N}, errors {out['errors']}")


# Base_spectral::coef / coef_i with the bases of the bispheric domains
# (domain_bispheric_rect.cpp:466-500: COS or SIN in phi, CHEB_EVEN / CHEB_ODD
# in chi by the parity of the phi index, CHEB in eta; points = coefficients)
# and with the COSSIN_EVEN / COSSIN_ODD phi bases, through oracle/ref_drivers/
# ref_coef3.cpp.
def coef3_cases():
    cases = []
    n = 9
    for name, bp in (("bispheric_std", S.COS), ("bispheric_anti", S.SIN)):
        bt = [S.CHEB_EVEN if k % 2 == 0 else S.CHEB_ODD for k in range(n)]
        br = [[S.CHEB] * n for _ in range(n)]
        cases.append((name, (n, n, n), (n, n, n), bp, bt, br))
    for name, bp in (("cossin_even", S.COSSIN_EVEN), ("cossin_odd", S.COSSIN_ODD)):
        np_, nc = (9, 7, 8), (9, 7, 10)
        bt = [S.COS_EVEN if k % 2 == 0 else S.SIN_EVEN for k in range(nc[2])]
        br = [[S.CHEB] * nc[2] for _ in range(nc[1])]
        cases.append((name, np_, nc, bp, bt, br))
    return cases


def make_coef3(dest: Path):
    rng = np.random.default_rng(31)
    out = {}
    for name, np_, nc, bp, bt, br in coef3_cases():
        vals = rng.standard_normal(int(np.prod(np_)))
        cfs = rng.standard_normal(int(np.prod(nc)))
        lines = [" ".join(map(str, np_ + nc)), str(bp), " ".join(map(str, bt))]
        lines.append(" ".join(str(br[j][k]) for k in range(nc[2]) for j in range(nc[1])))
        lines.append(" ".join(repr(float(v)) for v in vals))
        lines.append(" ".join(repr(float(v)) for v in cfs))
        r = subprocess.run([str(REF_BIN / "ref_coef3")], input="\n".join(lines) + "\n", capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(f"ref_coef3 failed ({r.returncode}) on {name}: {r.stderr[-500:]}")
        nums = [float(t) for t in r.stdout.split()[1:]]
        ncf = int(np.prod(nc))
        out[f"{name}_np"] = np.array(np_)
        out[f"{name}_nc"] = np.array(nc)
        out[f"{name}_bp"] = np.array(bp)
        out[f"{name}_bt"] = np.array(bt)
        out[f"{name}_br"] = np.array(br)
        out[f"{name}_values"] = vals
        out[f"{name}_coefs_in"] = cfs
        out[f"{name}_coef"] = np.array(nums[:ncf])
        out[f"{name}_coef_i"] = np.array(nums[ncf:])
    np.savez_compressed(dest, **out)
    print(f"  {len(out) // 9} cases")


CASES = {
    "spectral": lambda: make_spectral(HERE / "ref_spectral_1d.npz"),
    "coef3d": lambda: make_coef3d(HERE / "ref_coef3d.npz"),
    "coef3bases": lambda: make_coef3(HERE / "ref_coef3_bases.npz"),
    "toy": lambda: make_toy(HERE / "ref_toy.npz"),
    "funcs": lambda: make_toy(HERE / "ref_funcs.npz", (9, 5, 4), FUNCS_EQUATION, (("amp", 0.3),)),
    "funcs2": lambda: make_toy(HERE / "ref_funcs2.npz", (9, 5, 4), FUNCS2_EQUATION, (("amp", 0.3),)),
    "star954": lambda: make_star(HERE / "ref_star_954.npz", (9, 5, 4), True),
    "star1394": lambda: make_star(HERE / "ref_star_1394.npz", (13, 9, 4), False),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default=",".join(CASES))
    args = ap.parse_args()
    build()
    for name in args.only.split(","):
        print(name, flush=True)
        CASES[name]()


if __name__ == "__main__":
    main()
