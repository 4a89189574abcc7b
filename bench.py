#!/usr/bin/env python
"""Benchmark of the spaND factorization + PCG hot path on GB300.

Metric: seconds for factorize + preconditioned CG to an FP64 relative residual of 1e-10
on the 3D 7-point Laplacian 64^3 (n = 262,144), 12 nested-dissection levels,
eps = 1e-2, one N(0,1) right-hand side -- the mixed-precision path (FP32 factor, FP64
CG).  The plain FP64 path is timed beside it.  A step = one factorization (from the
assembled blocks, resident in HBM) + one CG solve.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  Under torchrun (N > 1) every rank runs an independent replica on
its own GPU (the path has no data exchange) and the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "factor+PCG seconds to 1e-10 FP64 rel. residual (3D 7-pt Laplacian 64^3, eps=1e-2)"


PROBLEMS = {
    "lap2d": "2D 5-pt Laplacian {n}^2",
    "lap3d": "3D 7-pt Laplacian {n}^3",
    "fv2d": "2D 5-pt finite-volume diffusion {n}^2, coefficients 10^U(-3,3) on 8x8 tiles",
    "aniso3d": "3D anisotropic diffusion {n}^3, face conductivities exp(0.5 z), axis scaling (1,1,0.01)",
    "batch": "{systems} systems -Laplacian + cI on m^3 grids, m ~ U{{16..40}}, c ~ U(0,1)",
}


def metric(args):
    """The headline metric string; other problems, grids, tolerances and right-hand-side
    counts say so."""
    if (args.problem, args.n, args.eps, args.nrhs) == ("lap3d", 64, 1e-2, 1):
        return METRIC
    if args.problem == "batch":
        return (f"seconds to factor and PCG-solve every system to {args.tol:g} FP64 rel. residual "
                f"({PROBLEMS['batch'].format(systems=args.systems)}, eps={args.eps:g})")
    return (f"factor+PCG seconds to {args.tol:g} FP64 rel. residual ({PROBLEMS[args.problem].format(n=args.n)}, "
            f"eps={args.eps:g}, {args.nrhs} RHS)")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--problem", default="lap3d", choices=sorted(PROBLEMS))
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--levels", type=int, default=12)
    ap.add_argument("--eps", type=float, default=1e-2)
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--maxit", type=int, default=200)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--nrhs", type=int, default=1, help="right-hand sides solved together (independent CGs)")
    ap.add_argument("--systems", type=int, default=256, help="independent systems of --problem batch")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def workload(args):
    from spand_public_gb300 import problems as P

    if args.problem == "lap3d":
        A, X = P.neglapl(args.n, 3), P.linspace_nd(args.n, 3)
    elif args.problem == "lap2d":
        A, X = P.neglapl(args.n, 2), P.linspace_nd(args.n, 2)
    elif args.problem == "fv2d":
        A, X = P.high_contrast_fv2d(args.n, 8, seed=0), P.linspace_nd(args.n, 2)
    else:
        A, X = P.anisotropic3d(args.n, P.anisotropic_theta(args.n, seed=0)), P.linspace_nd(args.n, 3)
    B = np.asfortranarray(P.rhs(A.shape[0], args.nrhs, seed=0))  # n x nrhs, column j = RHS j
    return A, X, B


def config(args, extra=None):
    dim = 2 if args.problem in ("fv2d", "lap2d") else 3
    c = {"workload": f"{PROBLEMS[args.problem].format(n=args.n)} (n={args.n ** dim}), {args.levels} ND levels, "
                     f"eps={args.eps:g}, {args.nrhs} RHS N(0,1) seed 0, PCG to {args.tol:g}",
         "problem": args.problem, "grid": args.n, "levels": args.levels, "eps": args.eps, "nrhs": args.nrhs, "pcg_tol": args.tol,
         "ordering": "geometric modified nested dissection",
         "l2": "working set larger than L2 (factor arena of several GB)"}
    if extra:
        c.update(extra)
    return c


# --------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p.get("hbm_gbs", 6800.0), p.get("bf16_tflops", 1900.0), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def ncu_traffic(cls: str, bytes_per_launch: float):
    """DRAM bytes per launch of a kernel class: the DRAM-to-algorithmic byte ratio of its
    committed ncu capture (profiles/ncu_traffic.json, measured on a smaller case of the same
    kernel) times this launch's algorithmic bytes, or None without a capture."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(path) as f:
            e = json.load(f).get(cls)
    except Exception:
        return None
    if isinstance(e, dict) and "dram_per_algorithmic" in e:
        return round(e["dram_per_algorithmic"] * bytes_per_launch)
    return None


# --------------------------------------------------------------------------------------
def make_tree(A, X, args, fp32: bool):
    import spand_public_gb300 as pkg

    t = pkg.Tree(args.levels)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(X)
    t.set_tol(args.eps)
    t.set_fp32(fp32)
    t.partition(A)
    t.assemble(A)
    return t


def oracle_mode(threads: int = 1):
    """Dense kernels of the timed oracle: the CBLAS / LAPACKE of scipy's bundled OpenBLAS
    where it can be loaded (dgemm, dsyrk, dtrsm, dpotrf, dgeqp3 -- the calls the reference
    makes, util.cpp:122-394), on `threads` OpenBLAS threads (1: like the reference's build,
    sequential MKL, tests/Makefile:29); else the oracle's restated kernels on one thread.
    Returns a description."""
    from oracle import oracle as O

    path = O.use_lapack(int(threads))
    if path:
        return (f"dense kernels through {os.path.basename(path)} (CBLAS/LAPACKE as the reference calls them), "
                f"{threads} OpenBLAS thread(s)")
    return "dense kernels restated in plain C++ (no CBLAS/LAPACKE library found), one thread"


def host_info():
    import platform

    return {"nproc": os.cpu_count(), "machine": platform.machine(), "processor": platform.processor() or None}


def cpu_oracle_solve(A, X, B, args, threads: int = 1):
    """The oracle (C++ restatement of the reference; its dense kernels on `threads` OpenBLAS
    threads): factorize + CG of the first right-hand side.  Returns (factor s, CG s,
    iterations, true relative residual)."""
    from oracle.oracle import OracleTree

    oracle_mode(threads)
    o = OracleTree(args.levels)
    o.set_Xcoo(X)
    o.set_tol(args.eps)
    o.partition(A)
    o.assemble(A)
    b = np.ascontiguousarray(B[:, 0])
    t0 = time.perf_counter()
    o.factorize()
    t1 = time.perf_counter()
    x, it = o.cg(b, args.maxit, args.tol)
    t2 = time.perf_counter()
    rel = float(np.linalg.norm(A @ x - b) / np.linalg.norm(b))
    return t1 - t0, t2 - t1, it, rel


def cpu_thread_choice(A, X, B, args):
    """One factor + CG on one OpenBLAS thread and one on every host core; the faster of the
    two is the CPU configuration to report.  Returns (threads, {threads: (factor s, CG s,
    iterations, relres)})."""
    n = max(1, os.cpu_count() or 1)
    runs = {1: cpu_oracle_solve(A, X, B, args, 1)}
    if n > 1:
        runs[n] = cpu_oracle_solve(A, X, B, args, n)
    k = args.nrhs
    best = min(runs, key=lambda t: runs[t][0] + k * runs[t][1])
    return best, runs


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    A, X, b = workload(args)
    # one step is one full factor + CG of the 64^3 problem (~10 s on one core); the first
    # two steps time one OpenBLAS thread and every host core, the rest use the faster; the
    # run is capped at about three minutes
    k = args.nrhs
    budget = 180.0
    t_start = time.perf_counter()
    threads, probe = cpu_thread_choice(A, X, b, args)
    its = [probe[threads][2]]
    rels = [probe[threads][3]]
    best_times = [probe[threads][0] + k * probe[threads][1]]
    while len(best_times) + len(probe) - 1 < args.steps:
        if time.perf_counter() - t_start + best_times[-1] > budget:
            break
        f, g, it, rel = cpu_oracle_solve(A, X, b, args, threads)
        best_times.append(f + k * g)
        its.append(it)
        rels.append(rel)
    v = float(np.mean(best_times))
    by_threads = {t: round(probe[t][0] + k * probe[t][1], 3) for t in probe}
    line = {"impl": "reference", "metric": metric(args), "value": v, "unit": "s", "n_gpus": world,
            "steps": len(best_times), "warmup": 0, "ms_per_step": v * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config(args, {"pcg_iterations": its[-1], "true_relres": rels[-1]}),
            "cpu_baseline": {"value": v, "unit": "s", "cores": threads, "kind": "port", "host": host_info(),
                             "seconds_by_openblas_threads": by_threads,
                             "sample": f"{len(best_times)} factorization(s) + CG of the first RHS of the {args.n}^3 "
                                       f"problem (CG time x {k} RHS) with the faster of 1 and {os.cpu_count()} "
                                       "OpenBLAS threads; the reference cannot be built here (no "
                                       "Eigen/METIS/LAPACKE), so its C++ restatement runs: " + oracle_mode(threads)},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    from oracle import oracle as O

    O.use_restated()
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args, rank, world, local_rank):
    import torch

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

    A, X, b = workload(args)
    N = A.shape[0]
    t_analysis0 = time.perf_counter()
    t32 = make_tree(A, X, args, fp32=True)
    t_analysis = time.perf_counter() - t_analysis0
    k = args.nrhs
    b_dev = torch.from_numpy(np.ascontiguousarray(b.T)).to(dev)  # k x n: column j of B contiguous
    x_dev = torch.zeros_like(b_dev)

    def true_relres(xd):
        xh = xd.cpu().numpy().T
        return max(float(np.linalg.norm(A @ xh[:, j] - b[:, j]) / np.linalg.norm(b[:, j])) for j in range(k))

    def step(tree):
        return tree.bench_step(b_dev.data_ptr(), x_dev.data_ptr(), args.maxit, args.tol, nrhs=k)
    # a fresh tree's first factorization (launches sized from capacity bounds: what a
    # one-shot caller pays) and its second (times the candidate QRCP launches of every
    # wave); every later one replays the tuned factorization graph
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    t32.factorize()
    cold_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    t32.factorize()
    tuning_ms = (time.perf_counter() - t0) * 1e3
    for _ in range(args.warmup):
        step(t32)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t32.launches(reset=True)
    clocks = ClockSampler(local_rank)
    clocks.start()
    steps = []
    for _ in range(args.steps):
        steps.append(step(t32))
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = t32.launches(reset=True) / max(args.steps, 1)
    step_s = [(s["factor_ms"] + s["pcg_ms"]) / 1e3 for s in steps]
    value = float(np.mean(step_s))
    if dist:
        tv = torch.tensor([value], device=dev, dtype=torch.float64)
        dist.all_reduce(tv, op=dist.ReduceOp.MAX)
        value = float(tv.item())
    true_rel = true_relres(x_dev)
    factor_ms = float(np.mean([s["factor_ms"] for s in steps]))
    pcg_ms = float(np.mean([s["pcg_ms"] for s in steps]))
    iters = steps[-1]["iterations"]

    # profiled step (CUDA events around every launch): per-kernel-class time
    t32.set_profiling(True)
    prof_step = step(t32)
    prof = t32.profile()
    t32.set_profiling(False)
    wf = t32.work("factor")
    ws = t32.work("solve")
    n_solves = prof.get("perm", {}).get("launches", 0) // 2
    hbm, bf16, peak_kind = peaks()
    kernels = {}
    for cls, p in prof.items():
        if cls in wf:
            by, fl = wf[cls]["bytes"], wf[cls]["flops"]
        elif cls in ws:
            by, fl = ws[cls]["bytes"] * n_solves, ws[cls]["flops"] * n_solves
        else:
            by, fl = None, None
        e = {"launches": p["launches"], "ms": round(p["ms"], 4)}
        if by is not None and p["ms"] > 0:
            e["gbs"] = round(by / (p["ms"] * 1e-3) / 1e9, 1)
            e["gflops"] = round(fl / (p["ms"] * 1e-3) / 1e9, 1)
        kernels[cls] = e
    total_prof = sum(p["ms"] for p in prof.values())
    dom = max((c for c in prof if c != "restore"), key=lambda c: prof[c]["ms"])
    dom_by = wf[dom]["bytes"] if dom in wf else ws.get(dom, {}).get("bytes", 0) * n_solves
    dom_launches = prof[dom]["launches"]
    dom_avg_ms = prof[dom]["ms"] / max(dom_launches, 1)
    achieved = (dom_by / max(dom_launches, 1)) / (dom_avg_ms * 1e-3) / 1e9 if dom_avg_ms > 0 else 0.0
    traffic = ncu_traffic(dom, dom_by / max(dom_launches, 1))
    roofline = {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 4), "peak_source": peak_kind,
                "traffic": traffic, "bytes_per_launch": dom_by / max(dom_launches, 1),
                "avg_launch_ms": dom_avg_ms, "share_of_step": round(prof[dom]["ms"] / max(total_prof, 1e-9), 3)}
    if dom == "qrcp":
        # what bounds it in practice (from its ncu section set: DRAM 0.1%, FMA pipe 7%)
        roofline["note"] = ("latency-bound per pivot step (dependent shared-memory passes and one "
                            "cluster barrier per column); DRAM and FMA pipes both near idle")

    # plain FP64 path, same workload
    fp64 = None
    if args.fp64_steps > 0:
        t64 = make_tree(A, X, args, fp32=False)
        # the same warm state as the FP32 tree: cold, launch-measuring and graph-capturing
        # factorizations before the timed ones
        for _ in range(3):
            step(t64)
        s64 = [step(t64) for _ in range(args.fp64_steps)]
        fp64 = {"seconds": float(np.mean([(s["factor_ms"] + s["pcg_ms"]) / 1e3 for s in s64])),
                "factor_ms": float(np.mean([s["factor_ms"] for s in s64])),
                "pcg_ms": float(np.mean([s["pcg_ms"] for s in s64])),
                "pcg_iterations": s64[-1]["iterations"],
                "true_relres": true_relres(x_dev)}
        t64.close()

    # end to end through the C ABI with host buffers: values upload (assemble on the
    # cached plan), factorize, CG with host b -> host x
    e2e_t = []
    for _ in range(max(args.steps, 1)):
        t0 = time.perf_counter()
        t32.assemble(A)
        t32.factorize()
        if k == 1:
            xh, it_h, _ = t32.cg(b[:, 0], args.maxit, args.tol)
            xh = xh[:, None]
        else:
            xh, its_h, _ = t32.cg(b, args.maxit, args.tol)
            it_h = int(its_h.max())
        e2e_t.append(time.perf_counter() - t0)
    h2d = t32.assembled_bytes() + b.nbytes * 2  # values of A (scattered into blocks and CSR on the device), B, X0
    d2h = xh.nbytes
    e2e = {"value": float(np.mean(e2e_t)), "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
           "pcg_iterations": it_h,
           "true_relres": max(float(np.linalg.norm(A @ xh[:, j] - b[:, j]) / np.linalg.norm(b[:, j])) for j in range(k))}

    # the differentiable solve (anisotropic workload): loss 0.5 |x - x*|^2 through
    # spand_public_gb300.autograd.solve, forward (re-assembly of the values on the device,
    # factorization, PCG) and backward (the adjoint PCG with the same factor and the
    # -lambda x^T scatter onto the pattern), timed with CUDA events
    adjoint = None
    if args.problem == "aniso3d" and k == 1:
        from spand_public_gb300.autograd import Pattern, solve

        pat = Pattern(A)
        vals = torch.as_tensor(A.data, device=dev).requires_grad_(True)
        bb = torch.as_tensor(b[:, 0], device=dev).requires_grad_(True)
        xstar = torch.as_tensor(np.random.default_rng(1).standard_normal(N), device=dev)

        def fwd_bwd():
            vals.grad = None
            bb.grad = None
            xx = solve(vals, bb, t32, pat, iters=args.maxit, tol=args.tol)
            (0.5 * torch.sum((xx - xstar) ** 2)).backward()

        for _ in range(2):
            fwd_bwd()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()
        nadj = max(1, min(args.steps, 5))
        for _ in range(nadj):
            fwd_bwd()
        ev[1].record()
        torch.cuda.synchronize()
        adjoint = {"forward_backward_ms": ev[0].elapsed_time(ev[1]) / nadj, "steps": nadj,
                   "what": "values -> factor + PCG (forward) -> loss 0.5|x - x*|^2 -> adjoint PCG + pattern "
                           "scatter (backward), FP32 factor, FP64 PCG to the metric's tolerance"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads, runs = cpu_thread_choice(A, X, b, args)
        f_c, g_c, it_c, rel_c = runs[threads]
        cpu = {"value": f_c + k * g_c, "unit": "s", "cores": threads, "kind": "port", "host": host_info(),
               "seconds_by_openblas_threads": {t: round(r[0] + k * r[1], 3) for t, r in runs.items()},
               "sample": f"one factorization + the CG of the first right-hand side of the same {PROBLEMS[args.problem].format(n=args.n)} problem "
                         f"by the oracle (C++ restatement of the reference; CG time x {k} RHS; the faster of 1 and "
                         f"{os.cpu_count()} OpenBLAS threads: {oracle_mode(threads)}): "
                         f"{it_c} CG iterations, true relres {rel_c:.2e}"}
        from oracle import oracle as O

        O.use_restated()

    if rank == 0:
        extra = {"pcg_iterations": iters, "true_relres": true_rel, "factor_ms": factor_ms, "pcg_ms": pcg_ms,
                 "analysis_s": t_analysis, "cold_factor_ms": cold_ms, "tuning_factor_ms": tuning_ms,
                 "precision": "FP32 factor (SIMT), FP64 CG/SpMV/dots",
                 "plain_fp64": fp64, "adjoint": adjoint,
                 "speedup_vs_plain_fp64": (fp64["seconds"] / value) if fp64 else None,
                 "kernels": kernels, "profiled_step_ms": prof_step["factor_ms"] + prof_step["pcg_ms"],
                 "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"}
        line = {"metric": metric(args), "value": value, "unit": "s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config(args, extra),
                "e2e": e2e, "gpu_launches": int(round(launches)), "roofline": roofline, "cpu_baseline": cpu,
                "clocks": clk}
        print(json.dumps(line), flush=True)
    t32.close()
    return 0


def max_over_ranks(value, device=None):
    """The largest of a per-rank number over the process group (the number itself without
    one): the whole-job time of replicas or shards is the slowest rank's."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def batch_workload(args, rank=0):
    """args.systems systems -Laplacian + cI on m^3 grids, m ~ U{16..40}, c ~ U(0,1), one
    N(0,1) right-hand side each, ceil(log2(m^3/64)) levels; generator seeded with the rank
    (rank r of N takes its own args.systems systems: weak scaling, no data exchange)."""
    from spand_public_gb300 import problems as P

    rng = np.random.default_rng(rank)
    out = []
    for _ in range(args.systems):
        m = int(rng.integers(16, 41))
        c = float(rng.uniform(0.0, 1.0))
        levels = max(2, int(np.ceil(np.log2(m ** 3 / 64))))
        out.append((m, P.reaction_diffusion3d(m, c), P.linspace_nd(m, 3), levels, rng.standard_normal(m ** 3)))
    return out


def run_batch(args, rank, world, local_rank):
    import torch

    import spand_public_gb300 as pkg

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    systems = batch_workload(args, rank)

    def trees(fp32):
        out = []
        for m, A, X, levels, _ in systems:
            t = pkg.Tree(levels)
            t.set_verb(False)
            t.set_use_geo(True)
            t.set_Xcoo(X)
            t.set_tol(args.eps)
            t.set_fp32(fp32)
            t.partition(A)
            t.assemble(A)
            out.append(t)
        return out

    t_an = time.perf_counter()
    T32 = trees(True)
    F32 = pkg.Forest(T32)
    t_an = time.perf_counter() - t_an
    bs = [b for *_, b in systems]
    bd = torch.from_numpy(F32.stack(bs)).to(dev)
    xd = torch.zeros_like(bd)

    def step(f):
        xd.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f.factorize()
        t1 = time.perf_counter()
        its, rr = f.cg_device(bd.data_ptr(), xd.data_ptr(), args.maxit, args.tol)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        return t1 - t0, t2 - t1, its, rr

    for _ in range(args.warmup):
        step(F32)
    if world > 1:
        torch.distributed.barrier()
    F32.launches(reset=True)
    clocks = ClockSampler(local_rank)
    clocks.start()
    res = [step(F32) for _ in range(args.steps)]
    clk = clocks.stop()
    launches = F32.launches(reset=True) / max(args.steps, 1)
    value = max_over_ranks(float(np.mean([f + g for f, g, _, _ in res])), dev)
    its = res[-1][2]
    xs = F32.split(xd.cpu().numpy())
    true_rel = max(float(np.linalg.norm(A @ x - b) / np.linalg.norm(b)) for (m, A, X, levels, b), x in zip(systems, xs))
    fp64 = None
    if args.fp64_steps > 0:
        T64 = trees(False)
        F64 = pkg.Forest(T64)
        for t in T64:
            t.close()
        step(F64)
        r64 = [step(F64) for _ in range(args.fp64_steps)]
        fp64 = {"seconds": float(np.mean([f + g for f, g, _, _ in r64])), "pcg_iterations_max": int(r64[-1][2].max())}
        F64.close()
    # the same systems as 256 trees on their own streams (batch_factorize + batch_cg_device)
    bl = [torch.from_numpy(b).to(dev) for b in bs]
    xl = [torch.zeros_like(b) for b in bl]
    pkg.batch_factorize(T32)
    pkg.batch_cg_device(T32, [b.data_ptr() for b in bl], [x.data_ptr() for x in xl], args.maxit, args.tol)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pkg.batch_factorize(T32)
    pkg.batch_cg_device(T32, [b.data_ptr() for b in bl], [x.data_ptr() for x in xl], args.maxit, args.tol)
    torch.cuda.synchronize()
    streams_s = time.perf_counter() - t0
    # end to end through the C ABI with host buffers: stacked values upload, factor, CG
    vals = np.concatenate([A.data for _, A, _, _, _ in systems])
    b_st = F32.stack(bs)
    e2e_t = []
    for _ in range(max(args.steps, 1)):
        t0 = time.perf_counter()
        F32.assemble_values(vals)
        F32.factorize()
        xs_h, its_h, _ = F32.cg(b_st, args.maxit, args.tol)
        e2e_t.append(time.perf_counter() - t0)
    h2d = vals.nbytes + 2 * b_st.nbytes
    d2h = b_st.nbytes
    e2e = {"value": float(np.mean(e2e_t)), "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
           "pcg_iterations_max": int(its_h.max())}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle.oracle import OracleTree

        oracle_mode()
        sample = systems[:8]
        ts = 0.0
        for m, A, X, levels, b in sample:
            o = OracleTree(levels)
            o.set_Xcoo(X)
            o.set_tol(args.eps)
            o.partition(A)
            o.assemble(A)
            t0 = time.perf_counter()
            o.factorize()
            o.cg(b, args.maxit, args.tol)
            ts += time.perf_counter() - t0
        frac = sum(s[0] ** 3 for s in sample) / sum(s[0] ** 3 for s in systems)
        cpu = {"value": ts / frac, "unit": "s", "cores": 1, "kind": "port",
               "sample": f"factor+CG of the first {len(sample)} systems by the oracle ({oracle_mode()}), scaled to "
                         f"all {args.systems} by unknown count ({frac:.3f} of the dofs)"}
    line = {"metric": metric(args), "value": value, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": PROBLEMS["batch"].format(systems=args.systems) + f", eps={args.eps:g}, "
                                   f"PCG to {args.tol:g} per system", "systems": args.systems,
                       "dofs": int(sum(s[0] ** 3 for s in systems)), "eps": args.eps, "pcg_tol": args.tol,
                       "factor_s": float(np.mean([f for f, _, _, _ in res])),
                       "pcg_s": float(np.mean([g for _, g, _, _ in res])),
                       "pcg_iterations_max": int(its.max()), "pcg_iterations_mean": float(its.mean()),
                       "true_relres_max": true_rel, "analysis_s": t_an, "plain_fp64": fp64,
                       "design": "one Forest: every system's ordering and hierarchy side by side in one plan; each "
                                 "launch carries all systems' work; segmented CG (per-system scalars)",
                       "streams_s": streams_s,
                       "streams": "the same step as 256 trees on 256 streams (batch_factorize + batch_cg_device)",
                       "timing": "host wall clock between device-wide synchronisations",
                       "precision": "FP32 factor (SIMT), FP64 CG/SpMV/dots", "parallelism": "1 GPU"},
            "e2e": e2e, "gpu_launches": int(round(launches)), "roofline": None, "cpu_baseline": cpu, "clocks": clk}
    if world > 1:
        line["config"]["systems_all_ranks"] = args.systems * world
        line["config"]["sharding"] = "each rank factors and solves its own systems (seeded by rank); no collective"
    if rank == 0:
        print(json.dumps(line), flush=True)
    F32.close()
    for t in T32:
        t.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.problem == "batch":
        return run_batch(args, rank, world, local_rank)
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    try:
        return run_gb300(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
