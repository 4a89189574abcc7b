"""Generate tests/golden/reference_golden.json from a checkout of leopoldcambier/spaND_public.

Reads, as data: the golden vectors of the reference's gtest suite (tests/tests.cpp:
Util.ChooseRank :254-262, PartitionTest.Square :378-412, Util.swap2perm :349-357,
Util.LinspaceNd :301-310) and checksums of its Matrix Market fixtures (mats/*.mm), so the
tests can pin the oracle and the generators without the reference tree at run time.

usage: python tests/golden/make_golden.py /path/to/spaND_public
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import sys

import numpy as np


def parse_mm(path):
    """Coordinate Matrix Market -> full (symmetrised when 'symmetric'/'hermitian') triplets."""
    with open(path) as f:
        header = f.readline().lower()
        line = f.readline()
        while line.startswith("%"):
            line = f.readline()
        m, n, nnz = map(int, line.split())
        data = np.loadtxt(f, ndmin=2)
    rows = data[:, 0].astype(np.int64) - 1
    cols = data[:, 1].astype(np.int64) - 1
    vals = data[:, 2]
    if "symmetric" in header or "hermitian" in header:
        off = rows != cols
        rows, cols, vals = (np.concatenate([rows, cols[off]]), np.concatenate([cols, rows[off]]),
                            np.concatenate([vals, vals[off]]))
    order = np.lexsort((rows, cols))
    return m, n, rows[order], cols[order], vals[order]


def triplet_hash(rows, cols, vals):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(rows, dtype=np.int64).tobytes())
    h.update(np.ascontiguousarray(cols, dtype=np.int64).tobytes())
    h.update(np.ascontiguousarray(vals, dtype=np.float64).tobytes())
    return h.hexdigest()


def sepids(block):
    return [[int(a), int(b)] for a, b in re.findall(r"SepID\((\d+)\s*,\s*(\d+)\)", block)]


def main(ref):
    out = {"source": "leopoldcambier/spaND_public tests/tests.cpp and mats/*.mm"}
    src = open(os.path.join(ref, "tests", "tests.cpp")).read()
    # PartitionTest.Square: three vectors of 25 SepIDs
    sq = src[src.index("TEST(PartitionTest, Square)"):src.index("TEST(PartitionTest, Consistency)")]
    vecs = {}
    for name in ("sepidref", "leftref", "rightref"):
        body = sq[sq.index(name):]
        body = body[: body.index("}")]
        vecs[name] = sepids(body)
    out["partition_square"] = {"n": 5, "dim": 2, "nlevels": 3, **vecs}
    # Util.ChooseRank
    cr = src[src.index("TEST(Util, ChooseRank)"):src.index("TEST(Util, Block2Dense)")]
    errs = [float(v) for v in re.search(r"errs <<([^;]+);", cr).group(1).split(",")]
    cases = [[float(t), int(r)] for t, r in re.findall(r"choose_rank\(errs,\s*([0-9.e+-]+)\),\s*(\d+)\)", cr)]
    out["choose_rank"] = {"s": errs, "cases": cases}
    # Util.swap2perm
    sw = src[src.index("TEST(Util, swap2perm)"):]
    swap = [int(v) for v in re.search(r"swap <<([^;]+);", sw).group(1).split(",")]
    pref = [int(v) for v in re.search(r"permRef <<([^;]+);", sw).group(1).split(",")]
    out["swap2perm"] = {"swap": swap, "perm": pref}
    # Util.LinspaceNd
    ls = src[src.index("TEST(Util, LinspaceNd)"):src.index("TEST(Util, SymmPerm)")]
    x2 = [float(v) for v in re.search(r"X2ref <<([^;]+);", ls).group(1).split(",")]
    x3 = [float(v) for v in re.search(r"X3ref <<([^;]+);", ls).group(1).split(",")]
    out["linspace_nd"] = {"n3d2_rowmajor": x2, "n2d3_rowmajor": x3}
    # fixtures
    mats = {}
    mdir = os.path.join(ref, "mats")
    for fn in sorted(os.listdir(mdir)):
        m = re.match(r"neglapl_(\d)_(\d+)\.mm$", fn)
        if not m:
            continue
        M, N, r, c, v = parse_mm(os.path.join(mdir, fn))
        mats[fn] = {"dim": int(m.group(1)), "n": int(m.group(2)), "N": M, "nnz": int(len(v)),
                    "sha256": triplet_hash(r, c, v)}
    out["neglapl"] = mats
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
