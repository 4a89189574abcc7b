"""The allocation-free solve entry point against the regular device solve.

spand_tree_solve_device_noalloc serves callers that cannot call cudaMalloc when they
solve: code that runs inside a fixed, preallocated device-memory budget, and frameworks
whose own allocator owns the GPU's memory and must not be bypassed.  It keeps the
per-cluster solve vectors and their scratch copy in a fixed array inside the library
instead of memory the tree allocates on its first solve.  Here both entry points are
called through the C ABI on the same inputs, twice in a row for the allocation-free one
(the shared array keeps the previous call's contents), and the results must agree to the
FP64 solve tolerance of the parity tests.  Covered: the few-right-hand-side sweeps
(nrhs = 3) and the many-right-hand-side sweeps (nrhs = 20, 16 or more), SPD, LDLT and
PLU trees, FP64 and FP32 factors, the size limit at its exact edge, and one right-hand
side of a 64^3 problem.  This file is collected last on purpose.
"""
import ctypes
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, as for M^{-1}b in the FP64 parity tests
SCRATCH_BYTES = 16 << 20  # the fixed array's size, as documented in include/spand_gb300.h


def _tree(kind="spd", fp32=False, n=32, dim=2, nlevels=5):
    import spand_public_gb300 as pkg
    from spand_public_gb300 import problems as P

    if kind == "gen":
        A = P.neglapl_unsym(n, dim, seed=3)
    else:
        A = P.neglapl(n, dim)
    t = pkg.Tree(nlevels)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(P.linspace_nd(n, dim))
    t.set_tol(1e-2)
    t.set_fp32(fp32)
    if kind == "ldlt":
        t.set_symm_kind(pkg.SYM)
        t.set_scaling_kind(pkg.LDLT)
    elif kind == "gen":
        t.set_symm_kind(pkg.GEN)
        t.set_scaling_kind(pkg.PLU)
    t.partition(A)
    t.assemble(A)
    t.factorize()
    return t, A.shape[0]


def _compare(t, n, nrhs, calls=2, seed=21):
    import torch

    import spand_public_gb300 as pkg
    from spand_public_gb300 import problems as P

    L = pkg.lib()
    b = P.rhs(n, nrhs, seed=seed)
    src = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()  # (nrhs, n) row-major = n x nrhs column-major
    ref = src.clone()
    torch.cuda.synchronize()
    assert L.spand_tree_solve_device(t.h, ctypes.c_void_p(ref.data_ptr()), nrhs, n) == 0
    torch.cuda.synchronize()
    expect = ref.cpu().numpy()
    for _ in range(calls):
        out = src.clone()
        torch.cuda.synchronize()
        rc = L.spand_tree_solve_device_noalloc(t.h, ctypes.c_void_p(out.data_ptr()), nrhs, n)
        assert rc == 0, L.spand_last_error().decode()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        err = np.linalg.norm(got - expect) / np.linalg.norm(expect)
        assert err <= TOL, err


@pytest.mark.parametrize("nrhs", [3, 20])
@pytest.mark.parametrize("fp32", [False, True])
def test_noalloc_solve_matches_device_solve(fp32, nrhs):
    t, n = _tree("spd", fp32)
    _compare(t, n, nrhs)


@pytest.mark.parametrize("kind", ["ldlt", "gen"])
@pytest.mark.parametrize("nrhs", [3, 20])
def test_noalloc_solve_other_pivot_kinds(kind, nrhs):
    t, n = _tree(kind)
    _compare(t, n, nrhs)


def _x_len(L, t, n):
    """Per-right-hand-side length of the solve vectors, read from the rejection message of a
    request far beyond the limit (the message states 2 x x_len x nrhs x element size)."""
    import torch

    x = torch.zeros((1, n), dtype=torch.float64, device="cuda")
    rc = L.spand_tree_solve_device_noalloc(t.h, ctypes.c_void_p(x.data_ptr()), 1 << 20, n)
    assert rc == 1  # SPAND_ERR_ARG, before touching x
    msg = L.spand_last_error().decode()
    assert "scratch" in msg
    m = re.search(r"\(2 x (\d+) x (\d+) x (\d+)\)", msg)
    assert m, msg
    return int(m.group(1)), int(m.group(3))


@pytest.mark.parametrize("fp32", [False, True])
def test_noalloc_solve_limit_edge(fp32):
    import torch

    import spand_public_gb300 as pkg

    L = pkg.lib()
    t, n = _tree("spd", fp32)
    xlen, elem = _x_len(L, t, n)
    assert elem == (4 if fp32 else 8)
    assert xlen >= n
    nmax = SCRATCH_BYTES // (2 * xlen * elem)
    assert nmax >= 1
    # nrhs = nmax fits exactly: accepted and equal to the regular solve
    _compare(t, n, nmax, calls=1, seed=5)
    # one more right-hand side is rejected before anything is touched
    x = torch.full((nmax + 1, n), 7.0, dtype=torch.float64, device="cuda")
    rc = L.spand_tree_solve_device_noalloc(t.h, ctypes.c_void_p(x.data_ptr()), nmax + 1, n)
    assert rc == 1, rc
    torch.cuda.synchronize()
    assert bool(torch.all(x == 7.0))


def test_noalloc_solve_one_rhs_of_64cubed():
    """The documented capacity: one right-hand side of a 3D 64^3 problem (FP64 factor)."""
    t, n = _tree("spd", False, n=64, dim=3, nlevels=12)
    _compare(t, n, 1)
