"""Newton-step benchmark of the GB300 Kadath path.

    python bench.py --gpus N --steps K --warmup W [--impl reference] [--workload star|toy]

A step is one System_of_eqs::do_newton update (residual, Jacobian assembly,
dense LU, solve, field update) of the workload from its initial guess.  The
headline `value` is the mixed-precision step (TF32 tensor-core LU + FP64
GMRES-IR); the plain FP64 step is reported beside it.  `e2e` times the same
step through the C ABI with the fields uploaded from pinned host memory and
the converged coefficients read back inside the timed region.

With --gpus N > 1 (launched by torch.distributed.run) every rank solves its
own replica of the problem on its own GPU ("replicas only": the dense Newton
step has no data-parallel split in this design); value is the slowest rank's
step time.

--impl reference times the reference's CPU algorithm on the host cores: the
oracle's restatement of do_newton_seq (oracle/, pinned to the reference's own
outputs by tests/golden/ref_*.npz), one complete Newton step of the same
workload per timed step.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Newton-step time (assemble+LU+solve) at 1e-10 residual: FP64 vs mixed-prec"
TUNING_TABLE = ROOT / "kadath_frontera_gb300" / "tuning" / "line_passes_gb300.json"
PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(backend=None):
    """Replicas: one process per GPU (torchrun environment).  The path itself
    has no collective; the process group only carries the barrier and the
    max-over-ranks timing.  backend: "nccl" on GPUs, "gloo" for CPU tests."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        if backend is None:
            backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------- CPU side --
def cpu_full_step(workload):
    """One complete Newton step of the oracle (the numpy restatement of the
    reference's do_newton_seq, src_par/do_newton.cpp:519-572) from the
    workload's initial guess, timed on the host cores: the residual
    (sec_member), every Jacobian column (do_col_J, vectorised per seed
    block), LAPACK getrf/getrs on that Jacobian (scipy, all host cores) and
    the field update.  Nothing is sampled or extrapolated."""
    import scipy.linalg as sla
    from oracle import configs

    if workload == "toy":
        doms, sysm, *_ = configs.toy()
    else:
        doms, sysm, *_ = configs.star()
    t0 = time.perf_counter()
    F = sysm.residual()
    t_res = time.perf_counter() - t0
    t0 = time.perf_counter()
    _, J = sysm.jacobian()
    t_asm = time.perf_counter() - t0
    t0 = time.perf_counter()
    lu = sla.lu_factor(J, overwrite_a=True, check_finite=False)
    x = sla.lu_solve(lu, F, check_finite=False)
    t_lu = time.perf_counter() - t0
    t0 = time.perf_counter()
    sysm.update(x)
    t_upd = time.perf_counter() - t0
    total = t_res + t_asm + t_lu + t_upd
    N = len(F)
    return {"ms": 1e3 * total, "residual_ms": 1e3 * t_res, "assembly_ms": 1e3 * t_asm, "lu_solve_ms": 1e3 * t_lu,
            "update_ms": 1e3 * t_upd, "N": N,
            "sample": f"one complete Newton step from the initial guess: residual, all {N} Jacobian columns, "
                      f"LAPACK getrf/getrs of that {N}x{N} Jacobian, update (no extrapolation)"}


def cpu_warmup(workload):
    """Untimed warm-up of the CPU arm: imports and one residual."""
    from oracle import configs
    doms, sysm, *_ = configs.toy() if workload == "toy" else configs.star()
    sysm.residual()


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_warmup(args.workload)
    times = []
    info = None
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        info = cpu_full_step(args.workload)
        times.append(info["ms"])
    wall = time.perf_counter() - t_wall
    ms = statistics.mean(times)
    phases = ("residual_ms", "assembly_ms", "lu_solve_ms", "update_ms")
    line = {"impl": "reference", "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_label(args.workload), "N": info["N"],
                       "timed_wall_s": wall, "warmup": "one residual evaluation per warm-up step"},
            "cpu_baseline": {"value": ms, "unit": "ms", "cores": cores, "kind": "port", "sample": info["sample"],
                             "phases_ms": {k: info[k] for k in phases}},
            "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def workload_label(name):
    if name == "toy":
        return "toy: Space_spheric 3 domains (13,7,4), Lap(psi) = -2 pi rho psi^5"
    return ("star: XCTS-shaped static star, Space_spheric 6 domains (13,9,4), unknowns P, NP, bx, by, bz, "
            "frozen Gamma=2 K=100 rho_c=1.28e-3 matter in the nucleus")


# --------------------------------------------------------------- GPU side --
def run_gpu(args, ws, rank, local):
    import numpy as np
    import torch

    # the autotuner's table of line-pass launch shapes for this GPU, for
    # every context this process makes (shapes change no result bit)
    if TUNING_TABLE.exists() and not args.no_tuning:
        os.environ["KD_TUNING_FILE"] = str(TUNING_TABLE)

    from kadath_frontera_gb300 import Context
    from kadath_frontera_gb300 import kadath as KD
    from kadath_frontera_gb300 import workloads

    ctx = Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream_ptr, device=f"cuda:{local}")
    wl = workloads.WORKLOADS[args.workload](ctx=ctx)
    syst = wl.syst
    syst.graph_capture = not args.no_graph
    N = syst.get_nbr_unknowns()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB > L2

    def one_solve(mode):
        """A complete Newton solve from the initial guess to |F| <= precision,
        with every cache that outlives a step (the tangents of
        iterate-independent subtrees) cleared first: the first step pays for
        building it.  Returns (ms, number of updates, per-call reports)."""
        wl.restore()
        syst.cache_tangents(False)
        syst.cache_tangents(True)
        syst.reset_pivot_order()  # the first step of every solve pivots
        flush.zero_()
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        reps = []
        for _ in range(20):
            done, err = syst.do_newton(args.precision, lu_mode=mode)
            reps.append(dict(syst.last_report))
            if done:
                break
        ev1.record(stream)
        ev1.synchronize()
        if not done:
            raise RuntimeError(f"Newton did not converge (mode {mode}, |F| = {err:.3e})")
        return ev0.elapsed_time(ev1), len(reps) - 1, reps

    modes = {"mixed": KD.KD_LU_TF32_IR, "fp64": KD.KD_LU_FP64}
    # warm-up: builds matrices, tables, seeds, cuBLAS handles
    for _ in range(args.warmup):
        for m in modes.values():
            one_solve(m)
    results = {}
    barrier(ws)
    solutions = {}
    with ClockSampler(local) as clk:
        for name, m in modes.items():
            runs = [one_solve(m) for _ in range(args.steps if name == "mixed" else max(1, args.fp64_steps))]
            results[name] = runs
            solutions[name] = wl.download()
    barrier(ws)
    # the error of the mixed-precision solution against the FP64-LU solution
    # of the same solve (coefficients of every unknown in every domain)
    num = den = 0.0
    for fa, fb in zip(solutions["mixed"], solutions["fp64"]):
        for a, b in zip(fa, fb):
            num = max(num, float(np.abs(a - b).max()))
            den = max(den, float(np.abs(b).max()))
    mixed_vs_fp64 = num / den if den > 0 else 0.0

    def per_step(runs):
        return statistics.mean(ms / max(upd, 1) for ms, upd, _ in runs)

    def step_split(runs):
        """(first step of a solve, later steps) wall times from the reports."""
        first, later = [], []
        for _, _, reps in runs:
            upd = [r for r in reps if not r["converged"]]
            tot = [r["t_residual_ms"] + r["t_assembly_ms"] + r["t_factor_ms"] + r["t_solve_ms"] + r["t_update_ms"]
                   for r in upd]
            if tot:
                first.append(tot[0])
                later.extend(tot[1:])
        return (statistics.mean(first) if first else None, statistics.mean(later) if later else None)

    mixed_ms = max_over_ranks(ws, per_step(results["mixed"]))
    fp64_ms = max_over_ranks(ws, per_step(results["fp64"]))
    updates = results["mixed"][0][1]
    launches_mixed = statistics.mean(sum(r["kernel_launches"] for r in reps) / max(upd, 1)
                                     for _, upd, reps in results["mixed"])

    # end-to-end through the C ABI with host buffers (pinned), mixed LU:
    # upload of the initial guess, the solve, download of the solution
    host = [[torch.from_numpy(v).pin_memory().numpy() for v in per] for per in wl.initial_host]
    h2d = sum(v.nbytes for per in host for v in per)
    e2e_times = []
    d2h = 0
    for _ in range(args.steps):
        syst.cache_tangents(False)
        syst.cache_tangents(True)
        syst.reset_pivot_order()
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        wl.upload_initial(host)
        n_upd = 0
        for _ in range(20):
            done, _ = syst.do_newton(args.precision, lu_mode=modes["mixed"])
            if done:
                break
            n_upd += 1
        out = wl.download()
        e2e_times.append(1e3 * (time.perf_counter() - t0) / max(n_upd, 1))
        d2h = sum(v.nbytes for per in out for v in per)
    e2e_ms = max_over_ranks(ws, statistics.mean(e2e_times))

    # one instrumented step per mode: per-category kernel time and work
    prof = {}
    for name, m in modes.items():
        KD.profile_enable(ctx, True)
        one_solve(m)
        prof[name] = KD.profile_read(ctx)
        KD.profile_enable(ctx, False)

    exporter = run_exporter(args, ctx, wl, stream, local) if args.export_points > 0 else None
    batch = run_batch(args, local) if args.batch > 0 else None

    if rank != 0:
        return 0
    peaks, peak_kind = load_peaks()
    fp64_tflops = measure_fp64_peak(f"cuda:{local}")
    # The dominant kernel: the most wall time of a solve.  Each phase's wall
    # time (mean over the timed mixed solves) is charged to the kernels that
    # run in it, in proportion to their device time in the instrumented
    # solve: the transforms, elementwise kernels and gathers run side by side
    # on per-domain and per-seed-block streams (their device times add up to
    # several times the phases' wall time), the trailing update beside the
    # next panel.
    pm = prof["mixed"]
    wall = {"residual+assembly": 0.0, "factor": 0.0, "solve": 0.0}
    for _, _, reps in results["mixed"]:
        for r in reps:
            wall["residual+assembly"] += r["t_residual_ms"] + r["t_assembly_ms"]
            wall["factor"] += r["t_factor_ms"]
            wall["solve"] += r["t_solve_ms"]
    wall = {k: v / len(results["mixed"]) for k, v in wall.items()}
    groups = {"residual+assembly": ("transform", "elementwise", "tau_gather"),
              "factor": ("lu_panel", "lu_panel_static", "lu_swap_trsm", "lu_gemm"),
              "solve": ("lu_solve", "refine_matvec")}
    charged = {}
    for ph, cats in groups.items():
        dev = sum(pm[c]["ms"] for c in cats if c in pm)
        for c in cats:
            if c in pm and pm[c]["launches"]:
                charged[c] = pm[c]["ms"] * (wall[ph] / dev if dev > wall[ph] else 1.0)
    ranked = sorted(charged.items(), key=lambda kv: -kv[1])
    solve_wall = sum(wall.values())
    roof = roofline_for(ranked[0][0], pm[ranked[0][0]], peaks, peak_kind, fp64_tflops)
    roof["wall_ms_per_solve"] = ranked[0][1]
    roof["share_of_solve_wall_time"] = ranked[0][1] / solve_wall if solve_wall else None
    dev_total = sum(v["ms"] for v in pm.values())
    rooflines = {ROOF_KERNELS[k][0]: roofline_for(k, pm[k], peaks, peak_kind, fp64_tflops)
                 for k in ("lu_solve", "lu_gemm", "lu_panel", "lu_panel_static", "lu_swap_trsm", "transform")
                 if pm.get(k, {}).get("launches")}
    rep0 = results["mixed"][-1][2][0]
    rep64 = results["fp64"][-1][2][0]
    first_m, later_m = step_split(results["mixed"])
    first_f, later_f = step_split(results["fp64"])
    line = {
        "metric": METRIC, "value": mixed_ms, "unit": "ms", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": mixed_ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 (LU trailing update tf32, refined to f64)", "data": "synthetic",
        "config": {"workload": workload_label(args.workload), "N": N, "precision": args.precision,
                   "step": "mean Newton step of complete solves from the initial guess to |F| <= precision "
                           "(one timed unit = one solve; caches that outlive a step cleared per solve)",
                   "newton_updates_per_solve": updates, "solves_timed": args.steps,
                   "l2": "flushed between solves (256 MB write); the 1.2 GB Jacobian exceeds L2 within a solve",
                   "residual_graph": {"on": not args.no_graph,
                                      "captures_replays": list(syst.graph_stats())},
                   "jacobian_graph": {"on": not args.no_graph,
                                      "captures_replays": list(syst.jacobian_graph_stats())},
                   "autotuner": dict(ctx.autotune_stats(),
                                     table=str(TUNING_TABLE.relative_to(ROOT)) if TUNING_TABLE.exists()
                                     and not args.no_tuning else None),
                   "parallelism": "replicas" if ws > 1 else "single"},
        "fp64_ms_per_step": fp64_ms, "mixed_speedup_vs_fp64": fp64_ms / mixed_ms if mixed_ms > 0 else None,
        "first_step_ms": {"mixed": first_m, "fp64": first_f},
        "later_step_ms": {"mixed": later_m, "fp64": later_f},
        "phases_ms_first_step": {
            "mixed": {k: rep0[k] for k in ("t_residual_ms", "t_assembly_ms", "t_factor_ms", "t_solve_ms",
                                           "t_update_ms")},
            "fp64": {k: rep64[k] for k in ("t_residual_ms", "t_assembly_ms", "t_factor_ms", "t_solve_ms",
                                          "t_update_ms")}},
        "phases_ms_later_step": {
            "mixed": {k: results["mixed"][-1][2][1][k] for k in ("t_residual_ms", "t_assembly_ms", "t_factor_ms",
                                                                 "t_solve_ms", "t_update_ms")}}
        if len(results["mixed"][-1][2]) > 2 else None,
        "refine": {"iters": rep0["refine_iters"], "rel_residual": rep0["refine_rel_residual"],
                   "iters_later_steps": [r["refine_iters"] for r in results["mixed"][-1][2][1:] if not r["converged"]],
                   "static_pivots_later_steps": [r["static_pivots"] for r in results["mixed"][-1][2][1:]
                                                 if not r["converged"]]},
        "mixed_vs_fp64_solution_max_rel_diff": mixed_vs_fp64,
        "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches_mixed),
        "kernel_profile_ms": {name: {k: round(v["ms"], 3) for k, v in p.items()} for name, p in prof.items()},
        "device_time_share": {k: round(v["ms"] / dev_total, 4) for k, v in pm.items() if v["launches"]}
        if dev_total else None,
        "wall_ms_per_solve": {"phases": {k: round(v, 3) for k, v in wall.items()},
                              "charged_to_kernels": {k: round(v, 3) for k, v in ranked}},
        "roofline": roof,
        "rooflines": rooflines,
        "fp64_peak_tflops_measured": fp64_tflops,
        "clocks": clk.summary(),
        "batch": batch,
        "exporter": exporter,
    }
    if exporter:
        exporter["frac_of_fp64_peak"] = exporter["achieved_tflops_fp64"] / fp64_tflops if fp64_tflops else None
    if not args.no_cpu:
        cb = cpu_full_step(args.workload)
        line["cpu_baseline"] = {"value": cb["ms"], "unit": "ms", "cores": os.cpu_count(), "kind": "port",
                                "sample": cb["sample"],
                                "phases_ms": {k: cb[k] for k in ("residual_ms", "assembly_ms", "lu_solve_ms",
                                                                 "update_ms")}}
    print(json.dumps(line), flush=True)
    return 0


def run_exporter(args, ctx, wl, stream, local):
    """The converged fields evaluated at --export-points random Cartesian
    points (radii up to 4x the outer shell, every domain including the
    compactified one) on the GPU: kd_fields_val_points_device, all unknown
    fields at once, points already resident in HBM.  Work per point and
    field: 2 flops per coefficient of the domain holding the point."""
    import numpy as np
    import torch

    from kadath_frontera_gb300 import kadath as KD

    n = args.export_points
    fields = [f for _, f in wl.unknowns]
    g = torch.Generator(device=f"cuda:{local}").manual_seed(0)
    r = 128.0 * torch.rand(n, device=f"cuda:{local}", dtype=torch.float64, generator=g) ** 2
    v = torch.randn(n, 3, device=f"cuda:{local}", dtype=torch.float64, generator=g)
    xyz = (v / v.norm(dim=1, keepdim=True) * r[:, None]).contiguous()
    out = torch.empty(len(fields), n, device=f"cuda:{local}", dtype=torch.float64)
    torch.cuda.synchronize()
    for _ in range(2):
        KD.val_points_device(fields, xyz.data_ptr(), out.data_ptr(), n)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    reps = 5
    ev0.record(stream)
    for _ in range(reps):
        KD.val_points_device(fields, xyz.data_ptr(), out.data_ptr(), n)
    ev1.record(stream)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1) / reps
    # algorithmic flops: 2 per coefficient of the point's domain, per field
    space = wl.space
    radii = r.cpu().numpy()
    ncoef = []
    for d in range(space.get_nbr_domains()):
        info = space.domain_info(d)
        nc = info["nbr_coefs"]
        ncoef.append(int(nc[0] * nc[1] * nc[2]))
    edges = list(workloads_bounds(wl))
    dom_of = np.searchsorted(np.asarray(edges), radii, side="left")
    flops = 2.0 * len(fields) * float(np.sum(np.asarray(ncoef)[np.minimum(dom_of, len(ncoef) - 1)]))
    achieved = flops / (ms * 1e-3) / 1e12
    return {"points": n, "fields": len(fields), "ms": ms, "points_per_s": n / (ms * 1e-3),
            "kernel": "pt_classify + pt_scatter + val_points_sorted_kernel", "achieved_tflops_fp64": achieved,
            "work": "2 flops per coefficient of the point's domain per field (spectral summation)"}


def workloads_bounds(wl):
    """Outer radii of the star workload's domains (the last one infinite)."""
    from kadath_frontera_gb300 import workloads
    return list(workloads.STAR_BOUNDS) if wl.name == "star" else [1.0, 2.0]


def run_batch(args, local):
    """Batched uneven solves: `--batch` independent isolated stars (central
    density uniform in [8e-4, 2e-3], nr in {9, ..., 17}) solved from scratch
    (context, space, system, Newton to the precision), one at a time and
    then concurrently, one context per instance from `--batch-threads` host
    threads.  Returns solves/s of both and the concurrent speed-up."""
    import gc

    import torch

    from kadath_frontera_gb300 import kadath as KD
    from kadath_frontera_gb300 import workloads

    cfgs = workloads.star_batch_configs(args.batch, seed=0)
    # warm-up: one instance of every resolution (module load, kernel attributes)
    seen = {}
    for c in cfgs:
        seen.setdefault(c["res"], c)
    workloads.solve_batch(list(seen.values()), 1, args.precision, KD.KD_LU_TF32_IR, local, keep=False)
    gc.collect()
    out = {"instances": args.batch, "threads": args.batch_threads,
           "res": sorted({c["res"] for c in cfgs}), "unit": "solves/s",
           "lu": "mixed (tf32 trailing update, f64 GMRES-IR)",
           "includes": "per instance: context, space and system set-up, Newton solve to |F| <= precision"}
    for name, threads in (("serial", 1), ("concurrent", args.batch_threads)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        upd = workloads.solve_batch(cfgs, threads, args.precision, KD.KD_LU_TF32_IR, local, keep=False)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        gc.collect()
        out[name] = {"s": dt, "solves_per_s": len(cfgs) / dt, "newton_updates": int(sum(upd))}
    out["concurrent_speedup"] = out["serial"]["s"] / out["concurrent"]["s"]
    return out


def measure_fp64_peak(device):
    """FP64 arithmetic peak of this GPU, measured here: cuBLAS DGEMM
    throughput (torch.matmul, float64, 4096^3, best of 3).  GB300's FP64 rate
    is the bound of the spectral transforms; the driver's peak file has no
    FP64 entry."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=device)
    b = torch.randn(n, n, dtype=torch.float64, device=device)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = None
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


# The kernel behind each profile category of the mixed-precision step, and
# the resource that bounds it.  `work` of every category but the transforms
# is algorithmic bytes (include/kadath_gb300.h, kd_ctx_profile_read).
ROOF_KERNELS = {
    "lu_solve": ("trsv_chain<float>", "one triangular sweep over the FP32 factors (forward L or backward U)"),
    "lu_gemm": ("tf32_update_persistent", "3xTF32 tcgen05 trailing update"),
    "lu_panel": ("panel_cluster16_kernel", "partial-pivoting panel, one 16-CTA cluster"),
    "lu_panel_static": ("panel_nopiv_kernel", "static-pivot panel"),
    "lu_swap_trsm": ("trsm_chunk_f32", "U12 triangular solve (and row swaps after a pivoting panel)"),
    "refine_matvec": ("gemv_partial", "FP64 refinement matvec b - J x and GMRES vector work"),
    "elementwise": ("ew_kernel", "pointwise algebra at collocation points"),
    "tau_gather": ("gather_csr_kernel", "tau / Galerkin row gathers"),
    "transform": ("line_passes_kernel", "separable spectral transforms and 1-D operators (FP64)"),
}

# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) over the
# algorithmic bytes of one ncu-captured launch of each kernel on the star
# workload (N = 12,331); the summaries under profiles/ give the launches and
# the commands.  traffic per launch = ratio x algorithmic bytes per launch.
NCU_TRAFFIC_RATIO = {
    "lu_solve": (1.032, "profiles/trsv_chain_star_N12331.md"),
    "lu_gemm": (0.955, "profiles/tf32_update_persistent_star_N12331.md"),
    "lu_panel": (0.51, "profiles/panel_cluster16_kernel_star_N12331.md"),
    "lu_panel_static": (0.52, "profiles/panel_nopiv_kernel_star_N12331.md"),
    "lu_swap_trsm": (0.51, "profiles/trsm_chunk_f32_star_N12331.md"),
}


def roofline_for(cat, st, peaks, peak_kind, fp64_tflops=None):
    """Roofline of one profile category of the mixed step: algorithmic work
    per launch over the mean launch duration (CUDA events on the launching
    stream, profile mode), against HBM (measured copy bandwidth) for the
    byte-bound kernels and against the in-run DGEMM rate for the FP64
    transforms."""
    if not st or not st["launches"]:
        return None
    kernel, what = ROOF_KERNELS[cat]
    per_launch_ms = st["ms"] / st["launches"]
    work_per_launch = st["work"] / st["launches"]
    out = {"kernel": kernel, "what": what, "launches": st["launches"], "avg_launch_ms": per_launch_ms,
           "device_ms_per_solve": st["ms"]}
    if cat == "transform":
        achieved = work_per_launch / (per_launch_ms * 1e-3) / 1e12
        out.update({"bound": "fp64", "achieved": achieved, "peak": fp64_tflops, "unit": "TFLOP/s",
                    "frac": (achieved / fp64_tflops) if fp64_tflops else None, "traffic": None,
                    "work_per_launch": work_per_launch,
                    "peak_note": "FP64 DGEMM throughput measured in this run; work = algorithmic FP64 flops"})
        return out
    achieved = work_per_launch / (per_launch_ms * 1e-3) / 1e9
    peak = peaks.get("hbm_gbs", PEAKS_FALLBACK["hbm_gbs"])
    ratio = NCU_TRAFFIC_RATIO.get(cat)
    out.update({"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "algorithmic_bytes_per_launch": work_per_launch,
                "traffic": ratio[0] * work_per_launch if ratio else None,
                "traffic_source": ratio[1] if ratio else None,
                "peak_note": f"{peak_kind} copy bandwidth (of {peak_kind})"})
    return out


def run_large(args, local):
    """The binary-BH configuration's size (twelve domains at (11, 9, 8),
    N = 40,081, a 12.9 GB FP64 Jacobian) on a spherical space: complete
    Newton solves with the mixed LU and with the FP64 LU from the same
    initial guess, timed per step with CUDA events, and the difference of
    the two converged solutions."""
    import numpy as np
    import torch

    from kadath_frontera_gb300 import Context
    from kadath_frontera_gb300 import kadath as KD
    from kadath_frontera_gb300 import workloads

    ctx = Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream_ptr, device=f"cuda:{local}")
    wl = workloads.star_large(ctx=ctx)
    syst = wl.syst
    syst.graph_capture = not args.no_graph
    N = syst.get_nbr_unknowns()

    def solve(mode):
        wl.restore()
        syst.cache_tangents(False)
        syst.cache_tangents(True)
        syst.reset_pivot_order()
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        reps = []
        for _ in range(12):
            done, err = syst.do_newton(args.precision, lu_mode=mode)
            reps.append(dict(syst.last_report))
            if done:
                break
        ev1.record(stream)
        ev1.synchronize()
        if not done:
            raise RuntimeError(f"large: no convergence (|F| = {err:.3e})")
        return ev0.elapsed_time(ev1) / max(len(reps) - 1, 1), len(reps) - 1, reps

    solve(KD.KD_LU_TF32_IR)  # warm-up: matrices, tables, seeds, workspaces
    with ClockSampler(local) as clk:
        mixed = [solve(KD.KD_LU_TF32_IR) for _ in range(max(1, args.steps))]
        sol_mixed = wl.download()
        fp64 = solve(KD.KD_LU_FP64) if args.fp64_steps > 0 else None
        sol_fp64 = wl.download() if fp64 else sol_mixed
    # one instrumented mixed solve: kernel time and work per category
    KD.profile_enable(ctx, True)
    solve(KD.KD_LU_TF32_IR)
    prof = KD.profile_read(ctx)
    KD.profile_enable(ctx, False)
    diff = 0.0
    for fa, fb in zip(sol_mixed, sol_fp64):
        for a, b in zip(fa, fb):
            diff = max(diff, float(np.abs(a - b).max() / max(1.0, np.abs(b).max())))

    def phases(rep):
        return {k: rep[k] for k in ("t_residual_ms", "t_assembly_ms", "t_factor_ms", "t_solve_ms", "t_update_ms")}
    mixed_ms = statistics.mean(m[0] for m in mixed)
    line = {
        "metric": METRIC + " (binary-BH size, spherical space)", "value": mixed_ms, "unit": "ms",
        "n_gpus": 1, "steps": len(mixed), "higher_is_better": False, "data": "synthetic",
        "config": {"workload": "star, 12 domains at (11,9,8), matter inside r = 8", "N": N,
                   "jacobian_gb_fp64": 8.0 * N * N / 1e9, "precision": args.precision,
                   "step": "mean Newton step of complete solves (CUDA events)"},
        "fp64_ms_per_step": fp64[0] if fp64 else None,
        "mixed_speedup_vs_fp64": fp64[0] / mixed_ms if fp64 else None,
        "updates": {"mixed": mixed[0][1], "fp64": fp64[1] if fp64 else None},
        "phases_ms_first_step": {"mixed": phases(mixed[-1][2][0]), "fp64": phases(fp64[2][0]) if fp64 else None},
        "refine": {"iters": mixed[-1][2][0]["refine_iters"],
                   "rel_residual": mixed[-1][2][0]["refine_rel_residual"]},
        "mixed_vs_fp64_solution_max_rel_diff": diff if fp64 else None,
        "kernel_profile_ms": {k: round(v["ms"], 3) for k, v in prof.items()},
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gemm(args, local):
    """The tensor-core trailing update C -= A B alone (kd_tf32x3_gemm_update,
    3xTF32) at m x n x k, C column-major FP32: median of --steps timed calls
    after --warmup, CUDA events on the library's stream."""
    import ctypes as C

    import torch

    from kadath_frontera_gb300 import Context, _lib

    m, n, k = (int(x) for x in args.gemm.split(","))
    ctx = Context(local)
    lib = _lib.load()
    f = lib.kd_tf32x3_gemm_update
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong,
                  C.c_void_p, C.c_longlong]
    dev = f"cuda:{local}"
    g = torch.Generator(device=dev).manual_seed(0)
    A = torch.randn(k * m, device=dev, generator=g)   # m x k, lda = m
    B = torch.randn(n * k, device=dev, generator=g)   # k x n, ldb = k
    Cm = torch.randn(n * m, device=dev, generator=g)  # m x n, ldc = m
    stream = torch.cuda.ExternalStream(ctx.stream_ptr, device=dev)

    def call():
        ctx.check(f(ctx.h, m, n, k, A.data_ptr(), m, B.data_ptr(), k, Cm.data_ptr(), m))
    for _ in range(max(args.warmup, 1)):
        call()
    torch.cuda.synchronize()
    ms = []
    for _ in range(max(args.steps, 1)):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    med = statistics.median(ms)
    cbytes = 8.0 * m * n
    print(json.dumps({"kernel": "tf32_update_persistent (3xTF32)", "m": m, "n": n, "k": k, "ms_median": med,
                      "c_bytes": cbytes, "c_traffic_TBps": cbytes / med / 1e9,
                      "useful_tflops": 2.0 * m * n * k / med / 1e9}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="star", choices=["star", "toy"])
    ap.add_argument("--precision", type=float, default=1e-10)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--batch", type=int, default=64, help="instances of the batched-solve measurement (0: skip)")
    ap.add_argument("--export-points", type=int, default=1 << 20,
                    help="points of the exporter measurement (0: skip)")
    ap.add_argument("--batch-threads", type=int, default=8)
    ap.add_argument("--gemm", default=None, metavar="M,N,K",
                    help="only the tensor-core trailing update at this shape")
    ap.add_argument("--no-tuning", action="store_true",
                    help="line passes with the fixed launch-shape rule instead of the autotuner's table")
    ap.add_argument("--no-graph", action="store_true",
                    help="run the residual's value pass without CUDA-graph replay")
    ap.add_argument("--large", action="store_true",
                    help="only the binary-BH-size measurement (N = 40,081): mixed and FP64 solves")
    args = ap.parse_args()
    if args.impl == "reference":
        # rank 0 alone runs the CPU reference; other ranks exit without work
        rank = int(os.environ.get("RANK", "0"))
        return run_reference(args, int(os.environ.get("WORLD_SIZE", "1")), rank)
    ws, rank, local = dist_setup()
    if args.large:
        return run_large(args, local)
    if args.gemm:
        return run_gemm(args, local)
    return run_gpu(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
