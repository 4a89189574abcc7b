"""How far the deterministic QRCP tie rule moves the factorization from LAPACK's dgeqp3.

Test and documentation infrastructure (it drives the CPU oracle only).  The reference calls
LAPACK's dgeqp3 (src/util.cpp:383-394, from src/tree.cpp:1309), whose pivot is idamax's
first exact maximum of the partial column norms; the oracle and the device take the first
column within a relative 1e-7 of the maximum instead, so that columns whose norms are equal
in exact arithmetic pivot the same way whatever the summation order.  This script factors
the same problem twice with the oracle -- restated kernels (the tie rule; the device path
matches these ranks exactly) and the reference's BLAS / LAPACK calls through scipy's
OpenBLAS (LAPACK's own dgeqp3, no tie rule) -- and prints per level the sparsified
clusters, the rank sums, how many clusters' ranks differ and by how much, and the CG
iteration counts to 1e-10 on the same right-hand side.

    python oracle/lapack_deviation.py [--n 64] [--levels 12] [--eps 1e-2 1e-3]
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# run as a script, this folder would shadow the oracle package with oracle.py
sys.path[:] = [ROOT] + [p for p in sys.path if os.path.abspath(p or ".") != HERE]


def factor(A, X, levels, eps, lapack):
    from oracle import oracle as O

    if lapack:
        if O.use_lapack(1) is None:
            raise SystemExit("no CBLAS / LAPACKE library found next to scipy")
    else:
        O.use_restated()
    try:
        t = O.OracleTree(levels)
        t.set_Xcoo(X)
        t.set_tol(eps)
        t.partition(A)
        t.assemble(A)
        t.factorize()
        return t
    finally:
        O.use_restated()


def table(n, levels, eps, seed=0):
    from spand_public_gb300 import problems as P

    A, X = P.neglapl(n, 3), P.linspace_nd(n, 3)
    b = P.rhs(A.shape[0], 1, seed=seed)[:, 0]
    tr = factor(A, X, levels, eps, lapack=False)
    rr = tr.ranks()
    _, it_r = tr.cg(b, 200, 1e-10)[:2]
    del tr
    tl = factor(A, X, levels, eps, lapack=True)
    rl = tl.ranks()
    from oracle import oracle as O

    O.use_lapack(1)
    try:
        _, it_l = tl.cg(b, 200, 1e-10)[:2]
    finally:
        O.use_restated()
    assert np.array_equal(rr[:, :2], rl[:, :2])  # same clusters in the same order; sizes follow earlier ranks
    lines = [f"3D 7-point -Laplacian {n}^3, {levels} levels, eps = {eps:g}: CG iterations to 1e-10 (b = N(0,1), "
             f"seed {seed}): tie rule {it_r}, LAPACK dgeqp3 {it_l}",
             "",
             "| level | sparsified clusters | rows (tie rule) | rows (LAPACK) | rank sum (tie rule) | rank sum (LAPACK) | "
             "clusters with another rank | largest rank difference |",
             "|---:|---:|---:|---:|---:|---:|---:|---:|"]
    for lvl in np.unique(rr[:, 0]):
        m = rr[:, 0] == lvl
        d = rr[m, 3] - rl[m, 3]
        lines.append(f"| {lvl} | {int(m.sum())} | {int(rr[m, 2].sum())} | {int(rl[m, 2].sum())} | "
                     f"{int(rr[m, 3].sum())} | {int(rl[m, 3].sum())} | "
                     f"{int(np.count_nonzero(d))} | {int(np.abs(d).max()) if d.size else 0} |")
    return "\n".join(lines), it_r, it_l


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--levels", type=int, default=12)
    ap.add_argument("--eps", type=float, nargs="+", default=[1e-2, 1e-3])
    a = ap.parse_args()
    from oracle import oracle as O

    O.build()
    for eps in a.eps:
        print(table(a.n, a.levels, eps)[0])
        print()


if __name__ == "__main__":
    main()
