"""Measured QRCP launch choices against every forced configuration, wave by wave.

    python -m spand_public_gb300.tune_report [--grid 64] [--levels 12] [--eps 1e-2]
                                             [--fp64] [--repeats 3] [--out FILE]

Problem: the 3D 7-point negative Laplacian on a grid^3 mesh with geometric nested
dissection (the benchmark's matrix).  First a tuned tree: its first factorization sizes the
sparsification waves, the second times the tuner's candidate launch configurations of every
wave on the same inputs and keeps the fastest.  Then, per forced configuration (CTAs per
cluster x threads per CTA x vectorised trailing update, through SPAND_QC_CS,
SPAND_QC_THREADS and SPAND_QC_VEC with the measuring factorization off), a fresh tree with
the same waves.  Every wave's QRCP launch is timed with CUDA events by the tree's profiler,
median over `repeats` factorizations.  A forced run counts for a wave only where that wave
really launched the forced configuration (a configuration whose shared memory does not fit
a wave's matrices is not launched for it).  Per wave the report gives the tuned choice and
its time, the fastest forced configuration and its time, their ratio, and what the tuner
itself measured.
"""
import argparse
import itertools
import os
import statistics
import sys

FORCE_KEYS = ("SPAND_QC_CS", "SPAND_QC_THREADS", "SPAND_QC_VEC", "SPAND_QC_TUNE")


def _conf_name(c):
    vec = "v" if c["vec_rows"] < (1 << 30) else "s"
    blk = f" b{c['rpl']}" if c["rpl"] else ""
    return f"{c['cs']}x{c['threads']}{vec}{blk}"


def _tree(A, X, levels, eps, fp32):
    import spand_public_gb300 as pkg

    t = pkg.Tree(levels)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(X)
    t.set_tol(eps)
    t.set_fp32(fp32)
    t.partition(A)
    t.assemble(A)
    return t


def _wave_times(t, repeats):
    """Median per-wave QRCP time (ms) over `repeats` profiled factorizations."""
    runs = []
    for _ in range(repeats):
        t.set_profiling(True)
        t.factorize()
        prof = t.profile()
        t.set_profiling(False)
        runs.append({k[len("qrcp@"):]: v["ms"] for k, v in prof.items() if k.startswith("qrcp@")})
    return {k: statistics.median(r.get(k, 0.0) for r in runs) for k in runs[0]}


def study(grid=64, levels=12, eps=1e-2, fp32=True, repeats=3, log=sys.stderr):
    from spand_public_gb300 import problems as P

    saved = {k: os.environ.get(k) for k in FORCE_KEYS}
    os.environ["SPAND_PROFILE_LEVELS"] = "2"  # per-wave launch names
    A, X = P.neglapl(grid, 3), P.linspace_nd(grid, 3)
    try:
        for k in FORCE_KEYS:
            os.environ.pop(k, None)
        t = _tree(A, X, levels, eps, fp32)
        t.factorize()  # sizes the waves
        t.factorize()  # times the candidates
        waves = t.qrcp_waves()
        tuned = _wave_times(t, repeats)
        del t
        forced = {}  # wave key -> {conf name: ms}
        for cs, th, vec in itertools.product((1, 2, 4, 8, 16), (64, 128, 256, 512), (0, 1)):
            os.environ.update(SPAND_QC_CS=str(cs), SPAND_QC_THREADS=str(th), SPAND_QC_VEC=str(vec),
                              SPAND_QC_TUNE="0")
            t = _tree(A, X, levels, eps, fp32)
            t.factorize()
            got = t.qrcp_waves()
            times = _wave_times(t, repeats)
            del t
            n = 0
            for w in got:
                if w["cs"] != cs or w["threads"] != th or (vec == 0 and w["vec_rows"] < (1 << 30)):
                    continue
                key = f"L{w['level']}w{w['wave']}"
                if key in times:
                    forced.setdefault(key, {})[_conf_name(w)] = times[key]
                    n += 1
            print(f"forced {cs}x{th} vec={vec}: {n} waves", file=log, flush=True)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
        os.environ.pop("SPAND_PROFILE_LEVELS", None)
    rows = []
    for w in waves:
        key = f"L{w['level']}w{w['wave']}"
        f = forced.get(key, {})
        best = min(f.items(), key=lambda kv: kv[1]) if f else (None, float("nan"))
        rows.append(dict(key=key, items=w["items"], cap=w["cap_rows"], tuned=_conf_name(w),
                         tuned_ms=tuned.get(key, float("nan")), best=best[0], best_ms=best[1],
                         nforced=len(f), timed=[(_conf_name(c), ms) for c, ms in w["timed"]]))
    return rows


def report(rows, grid, levels, eps, fp32, repeats):
    ok = [r for r in rows if r["best"] is not None and r["best_ms"] > 0]
    tot_t = sum(r["tuned_ms"] for r in ok)
    tot_b = sum(r["best_ms"] for r in ok)
    within = sum(r["tuned_ms"] <= 1.02 * r["best_ms"] for r in ok)
    worst = max(ok, key=lambda r: r["tuned_ms"] / r["best_ms"]) if ok else None
    out = [f"QRCP launch choice per wave, 3D 7-pt Laplacian {grid}^3, {levels} levels, eps={eps:g}, "
           f"{'FP32' if fp32 else 'FP64'} factor; median of {repeats} profiled factorizations per run",
           "",
           f"waves compared: {len(ok)} of {len(rows)}; tuned within 2% of the best forced: {within}; "
           f"sum tuned {tot_t:.3f} ms, sum best forced {tot_b:.3f} ms (ratio {tot_t / max(tot_b, 1e-9):.3f})",
           ]
    if worst:
        out.append(f"largest ratio: {worst['key']} {worst['tuned_ms'] / worst['best_ms']:.3f}")
    out += ["",
            "config: CTAs per cluster x threads per CTA, v = vectorised trailing update, s = scalar",
            "",
            "| wave | items | cap rows | tuned | tuned ms | best forced | best ms | ratio | forced runs | tuner measured (ms) |",
            "|---|---|---|---|---|---|---|---|---|---|"]
    for r in rows:
        ratio = r["tuned_ms"] / r["best_ms"] if r["best"] is not None and r["best_ms"] > 0 else float("nan")
        meas = ", ".join(f"{n} {ms:.3f}" for n, ms in r["timed"]) or "cached / single"
        out.append(f"| {r['key']} | {r['items']} | {r['cap']} | {r['tuned']} | {r['tuned_ms']:.4f} | "
                   f"{r['best'] or '-'} | {r['best_ms']:.4f} | {ratio:.3f} | {r['nforced']} | {meas} |")
    return "\n".join(out) + "\n"


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--grid", type=int, default=64)
    ap.add_argument("--levels", type=int, default=12)
    ap.add_argument("--eps", type=float, default=1e-2)
    ap.add_argument("--fp64", action="store_true")
    ap.add_argument("--repeats", type=int, default=3)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    rows = study(a.grid, a.levels, a.eps, not a.fp64, a.repeats)
    text = report(rows, a.grid, a.levels, a.eps, not a.fp64, a.repeats)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text)
    print(text)


if __name__ == "__main__":
    main()
