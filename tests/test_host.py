"""Host side of the product (no GPU needed): ordering vs the oracle, the C ABI surface,
argument and state errors, and the symbolic plan's invariants."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import spand_public_gb300 as pkg
from oracle.oracle import OracleTree
from spand_public_gb300 import problems as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built():
    from spand_public_gb300 import build

    build.build()
    return pkg.lib()


def test_header_symbols_exported():
    """Every function declared in include/spand_gb300.h is exported by the library."""
    hdr = open(os.path.join(ROOT, "include", "spand_gb300.h")).read()
    declared = set(re.findall(r"^\s*(?:int|const char\*)\s+(spand_\w+)\s*\(", hdr, re.M))
    out = subprocess.run(["nm", "-D", "--defined-only", pkg.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if l.strip())
    assert declared, "no declarations parsed"
    assert declared <= exported, declared - exported
    assert declared == set(pkg.exported_symbols())


@pytest.mark.parametrize("n,dim,nlevels", [(5, 2, 3), (20, 2, 4), (64, 2, 7), (16, 3, 6), (32, 3, 8)])
def test_partition_matches_oracle(n, dim, nlevels):
    A = P.neglapl(n, dim)
    X = P.linspace_nd(n, dim)
    o = OracleTree(nlevels)
    o.set_Xcoo(X)
    po = o.partition(A)
    t = pkg.Tree(nlevels)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(X)
    pt = t.partition(A)
    assert np.array_equal(po, pt)
    assert np.array_equal(o.get_assembly_perm(), t.get_assembly_perm())


@pytest.mark.parametrize("n,dim", [(5, 2), (20, 2), (64, 2), (10, 3), (17, 3)])
def test_partition_lorasp_matches_oracle(n, dim):
    """LoRaSp ordering (partition_lorasp, tree.cpp:421-503): the recursive-bisection parts and
    the assembly permutation equal the oracle's."""
    A = P.neglapl(n, dim)
    X = P.linspace_nd(n, dim)
    for nlevels in (2, 3, 5, 7):
        t = pkg.Tree(nlevels)
        t.set_verb(False)
        t.set_use_geo(True)
        t.set_Xcoo(X)
        pt = t.partition_lorasp(A)
        o = OracleTree(nlevels)
        o.set_Xcoo(X)
        po = o.partition_lorasp(A)
        assert np.array_equal(pt, po)
        assert np.array_equal(t.get_assembly_perm(), o.get_assembly_perm())


def test_partition_square_golden(golden):
    g = golden["partition_square"]
    t = pkg.Tree(3)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(P.linspace_nd(5, 2))
    part = t.partition(P.neglapl(5, 2))
    assert part[:, 0:2].tolist() == g["sepidref"]
    assert part[:, 2:4].tolist() == g["leftref"]
    assert part[:, 4:6].tolist() == g["rightref"]


def test_state_and_argument_errors():
    t = pkg.Tree(3)
    with pytest.raises(pkg.SpandError) as e:
        t.factorize()
    assert e.value.status == 2  # SPAND_ERR_STATE
    with pytest.raises(pkg.SpandError) as e:
        t.set_scaling_kind(9)
    assert e.value.status == 1
    with pytest.raises(pkg.SpandError) as e:
        pkg.Tree(0)
    assert e.value.status == 1
    # algebraic ordering needs METIS: reported, not crashed
    t2 = pkg.Tree(3)
    t2.set_verb(False)
    with pytest.raises(pkg.SpandError):
        t2.partition(P.neglapl(5, 2))
    # unsorted CSC rejected
    L = pkg.lib()
    cp = np.array([0, 2, 3], dtype=np.int32)
    rv = np.array([1, 0, 1], dtype=np.int32)
    t3 = pkg.Tree(2)
    rc = L.spand_tree_partition(t3.h, 2, cp.ctypes.data_as(ctypes.c_void_p), rv.ctypes.data_as(ctypes.c_void_p), None)
    assert rc == 1


def test_empty_and_tiny_inputs():
    """1x1 and 2x2 systems partition without error (ragged edge cases)."""
    import scipy.sparse as sp

    for n in (1, 2, 3):
        A = sp.csc_matrix(np.diag(np.full(n, 2.0)))
        X = np.arange(n, dtype=float)[None, :]
        t = pkg.Tree(2)
        t.set_verb(False)
        t.set_use_geo(True)
        t.set_Xcoo(X)
        part = t.partition(A)
        o = OracleTree(2)
        o.set_Xcoo(X)
        assert np.array_equal(part, o.partition(A))
