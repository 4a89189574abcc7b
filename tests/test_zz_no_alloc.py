"""The allocation-free solve entry point against the regular device solve.

spand_tree_solve_device_noalloc serves callers that cannot allocate device memory when
they solve: code being captured into a CUDA graph, where cudaMalloc is not allowed, code
running under a fixed, preallocated memory budget, or a framework that owns the device
allocator.  It keeps the per-cluster solve vectors in a fixed array inside the library
instead of memory the tree allocates on first use.  Here both entry points are called
through the C ABI on the same inputs, twice in a row for the allocation-free one (the
shared array keeps the previous call's contents), and the results must agree to the FP64
solve tolerance of the parity tests.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, as for M^{-1}b in the FP64 parity tests


def _tree(fp32):
    import spand_public_gb300 as pkg
    from spand_public_gb300 import problems as P

    A = P.neglapl(32, 2)
    t = pkg.Tree(5)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(P.linspace_nd(32, 2))
    t.set_tol(1e-2)
    t.set_fp32(fp32)
    t.partition(A)
    t.assemble(A)
    t.factorize()
    return t, A.shape[0]


@pytest.mark.parametrize("fp32", [False, True])
def test_noalloc_solve_matches_device_solve(fp32):
    import torch

    import spand_public_gb300 as pkg
    from spand_public_gb300 import problems as P

    L = pkg.lib()
    t, n = _tree(fp32)
    nrhs = 3
    b = P.rhs(n, nrhs, seed=21)
    src = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()  # (nrhs, n) row-major = n x nrhs column-major
    ref = src.clone()
    torch.cuda.synchronize()
    assert L.spand_tree_solve_device(t.h, ctypes.c_void_p(ref.data_ptr()), nrhs, n) == 0
    torch.cuda.synchronize()
    expect = ref.cpu().numpy()
    for _ in range(2):
        out = src.clone()
        torch.cuda.synchronize()
        rc = L.spand_tree_solve_device_noalloc(t.h, ctypes.c_void_p(out.data_ptr()), nrhs, n)
        assert rc == 0, L.spand_last_error().decode()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        err = np.linalg.norm(got - expect) / np.linalg.norm(expect)
        assert err <= TOL, err


def test_noalloc_solve_rejects_oversized_request():
    import torch

    import spand_public_gb300 as pkg

    L = pkg.lib()
    t, n = _tree(False)
    nrhs = 4096  # solve vectors of ~3N x 4096 doubles, far beyond the fixed scratch
    x = torch.zeros((1, n), dtype=torch.float64, device="cuda")
    rc = L.spand_tree_solve_device_noalloc(t.h, ctypes.c_void_p(x.data_ptr()), nrhs, n)
    assert rc == 1  # SPAND_ERR_ARG, before touching x
    assert "scratch" in L.spand_last_error().decode()
