"""Device path vs the CPU oracle (plain FP64 and mixed FP32 factor).

Bars: partition and permutation identical; per-cluster ranks identical; every recorded
factor block (ScalingLLT lower triangles, Gemm panels, Householder reflectors) within
1e-12 relative (Frobenius, per block) of the oracle; M^{-1}b within 1e-12 relative; CG
iteration count equal.  The FP32 factor must reach the same FP64 residual with at most
15% more CG iterations.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_BLOCK = 1e-12   # relative Frobenius error per factor block, FP64 path
TOL_SOLVE = 1e-12   # relative error of M^{-1} b, FP64 path


def _build(n, dim, nlevels, tol, skip=0, fp32=False, A=None, factorizations=1):
    import spand_public_gb300 as pkg
    from oracle.oracle import OracleTree
    from spand_public_gb300 import problems as P

    A = P.neglapl(n, dim) if A is None else A
    X = P.linspace_nd(n, dim)
    t = pkg.Tree(nlevels)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(X)
    t.set_tol(tol)
    t.set_skip(skip)
    t.set_fp32(fp32)
    pt = t.partition(A)
    t.assemble(A)
    for _ in range(factorizations):
        t.factorize()
    o = OracleTree(nlevels)
    o.set_Xcoo(X)
    o.set_tol(tol)
    o.set_skip(skip)
    po = o.partition(A)
    o.assemble(A)
    o.factorize()
    assert np.array_equal(pt, po)
    return A, t, o


CASES = [
    (5, 2, 3, 1e-2, 0),
    (20, 2, 4, 1e-14, 0),
    (32, 2, 5, 1e-2, 0),
    (64, 2, 7, 1e-2, 0),    # 2D 5-point -Laplacian 64x64, 7 levels, eps = 1e-2
    (64, 2, 7, 1e-2, 2),
    (10, 3, 4, 1e-2, 0),
    (16, 3, 6, 1e-2, 0),
    (16, 3, 6, 0.0, 0),
    (20, 2, 4, 10.0, 0),    # tol >= 1: every sparsified cluster drops to rank 0
]


# (n, dim, levels, tol, skip, factorizations): the second factorization of a tree runs
# with the launch configuration tuned from the first one's sizes (for 3D 32^3 the
# largest pivots, 224-256 rows, take the thread-block-cluster Cholesky)
CASES_F = [c + (1,) for c in CASES] + [(32, 3, 8, 1e-2, 0, 2)]


@pytest.mark.parametrize("n,dim,nlevels,tol,skip,nf", CASES_F)
def test_factor_parity_fp64(n, dim, nlevels, tol, skip, nf):
    _check_parity(n, dim, nlevels, tol, skip, nf)


@pytest.mark.parametrize("n,dim,nlevels,tol", [(16, 3, 6, 1e-2), (64, 2, 7, 1e-2)])
def test_factor_parity_fp64_global_qrcp(n, dim, nlevels, tol, monkeypatch):
    """Every sparsification matrix through the QRCP variant whose column slabs live in
    global memory (the path of matrices too large for a cluster's shared memory), on
    full clusters."""
    monkeypatch.setenv("SPAND_QC_GLOBAL", "1")
    _check_parity(n, dim, nlevels, tol, 0, 2)


@pytest.mark.parametrize("threads", [64, 128, 512])
def test_factor_parity_fp64_narrow_qrcp(threads, monkeypatch):
    """Every shared-memory QRCP launch with 64 or 128 threads per CTA (the configurations
    the launch model picks for the many small matrices of the lower levels), or with the
    wide 512-thread instantiation (for waves held at one CTA per SM)."""
    monkeypatch.setenv("SPAND_QC_THREADS", str(threads))
    _check_parity(16, 3, 6, 1e-2, 0, 2)
    _check_parity(64, 2, 7, 1e-2, 0, 1)


@pytest.mark.parametrize("mode", ["0", "1"])
def test_factor_parity_fp64_qrcp_vectorised(mode, monkeypatch):
    """Every shared-memory QRCP launch with the scalar trailing update (0) or with the
    vectorised one on the slabs of 128 rows or more (1)."""
    monkeypatch.setenv("SPAND_QC_VEC", mode)
    for case in [(32, 3, 8, 1e-2, 0, 2), (24, 3, 7, 1e-3, 0, 2), (16, 3, 6, 0.0, 0, 2), (64, 2, 7, 1e-2, 0, 2)]:
        _check_parity(*case)


@pytest.mark.parametrize("mode", ["0", "1"])
def test_factor_parity_fp64_qrcp_kind(mode, monkeypatch):
    """Every shared-memory QRCP launch through the unblocked kernel (0) or through the
    blocked panel kernel (1, wherever the matrices fit it): the same bars, so the panel
    scheme reproduces the unblocked pivots, ranks and factors."""
    monkeypatch.setenv("SPAND_QC_BLOCKED", mode)
    for case in [(16, 3, 6, 1e-2, 0, 2), (64, 2, 7, 1e-2, 0, 1), (20, 2, 4, 1e-14, 0, 1), (16, 3, 6, 0.0, 0, 1),
                 (32, 3, 8, 1e-2, 0, 2), (24, 3, 7, 1e-3, 0, 2)]:
        _check_parity(*case)


@pytest.mark.parametrize("threads", [64, 128])
def test_factor_parity_fp64_blocked_narrow(threads, monkeypatch):
    """The blocked QRCP with 64- and 128-thread CTAs (fewer warps than slab columns)."""
    monkeypatch.setenv("SPAND_QC_BLOCKED", "1")
    monkeypatch.setenv("SPAND_QC_THREADS", str(threads))
    _check_parity(16, 3, 6, 1e-2, 0, 2)
    _check_parity(64, 2, 7, 1e-2, 0, 1)


def _check_parity(n, dim, nlevels, tol, skip, nf):
    A, t, o = _build(n, dim, nlevels, tol, skip, factorizations=nf)
    assert np.array_equal(t.get_assembly_perm(), o.get_assembly_perm())
    # ranks
    rt, ro = t.ranks(), o.ranks()
    assert np.array_equal(rt, ro), "per-cluster ranks differ"
    # op structure (kind, level, self, nbr, sizes)
    opt, opo = t.ops(), o.ops()
    assert opt.shape == opo.shape
    assert np.array_equal(opt[:, :6], opo[:, :6])
    # factor blocks
    worst = 0.0
    for k in range(opt.shape[0]):
        kind, rows, cols = opt[k, 0], opt[k, 6], opt[k, 7]
        if kind not in (0, 1, 2, 3) or rows * cols == 0:
            continue
        mt = t.op_matrix(k, rows, cols)
        mo = o.op_matrix(k, opo[k, 6], opo[k, 7])
        if kind == 0:
            mt, mo = np.tril(mt), np.tril(mo)
        if kind == 3:
            mt, mo = np.tril(mt, -1), np.tril(mo, -1)
            ht, ho = t.op_tau(k, cols), o.op_tau(k, cols)
            worst = max(worst, np.linalg.norm(ht - ho) / max(np.linalg.norm(ho), 1e-300))
        den = max(np.linalg.norm(mo), 1e-300)
        worst = max(worst, np.linalg.norm(mt - mo) / den)
    assert worst < TOL_BLOCK, worst
    # per-level log
    lt, lo = t.level_log(), o.level_log()
    for a, b in zip(lt, lo):
        for key in ("dofs_nd", "dofs_left_nd", "dofs_left_elim", "dofs_left_spars", "rank_before_sum",
                    "rank_after_sum", "rank_after_count", "ignored", "nbrs_sum", "fact_nnz"):
            assert a[key] == b[key], (key, a[key], b[key])
    assert t.nnz() == o.nnz()
    assert t.get_stop() == o.get_stop()
    # solve
    from spand_public_gb300 import problems as P
    b = P.rhs(A.shape[0], 2, seed=3)
    xt, xo = t.solve(b), o.solve(b)
    assert np.linalg.norm(xt - xo) / np.linalg.norm(xo) < TOL_SOLVE


@pytest.mark.parametrize("n,dim,nlevels,tol", [(64, 2, 7, 1e-2), (16, 3, 6, 1e-2), (24, 3, 7, 1e-3)])
def test_pcg_iterations_match(n, dim, nlevels, tol):
    from spand_public_gb300 import problems as P
    A, t, o = _build(n, dim, nlevels, tol)
    b = P.rhs(A.shape[0], 1, seed=11)[:, 0]
    xt, it, rel = t.cg(b, iters=200, tol=1e-12)
    xo, ito = o.cg(b, iters=200, tol=1e-12)
    assert it == ito, (it, ito)
    res = np.linalg.norm(A @ xt - b) / np.linalg.norm(b)
    assert res < 1e-11
    assert np.linalg.norm(xt - xo) / np.linalg.norm(xo) < 1e-9


@pytest.mark.parametrize("n,dim,nlevels,tol,nf", [(64, 2, 7, 1e-2, 1), (16, 3, 6, 1e-2, 1), (24, 3, 7, 1e-3, 1),
                                                   (32, 3, 8, 1e-2, 2)])
def test_mixed_precision_pcg(n, dim, nlevels, tol, nf):
    """FP32 factor + FP64 PCG reaches 1e-10 with <= 15% more iterations than FP64."""
    from spand_public_gb300 import problems as P
    A, t64, o = _build(n, dim, nlevels, tol, factorizations=nf)
    _, t32, _ = _build(n, dim, nlevels, tol, fp32=True, factorizations=nf)
    b = P.rhs(A.shape[0], 1, seed=5)[:, 0]
    x64, it64, _ = t64.cg(b, iters=200, tol=1e-10)
    x32, it32, _ = t32.cg(b, iters=200, tol=1e-10)
    assert np.linalg.norm(A @ x32 - b) / np.linalg.norm(b) < 1e-9
    assert it32 <= max(it64 + 1, int(np.ceil(1.15 * it64))), (it32, it64)
    # the FP32 preconditioner against the FP64 oracle's (error stated: ~FP32 epsilon x conditioning)
    xt = t32.solve(b)
    xo = o.solve(b)
    assert np.linalg.norm(xt - xo) / np.linalg.norm(xo) < 1e-3


def test_reproducible():
    """Bit-identical results across runs (tests/tests.cpp:917-994)."""
    from spand_public_gb300 import problems as P
    A, t, _ = _build(32, 2, 5, 1e-5, skip=1)
    b = P.rhs(A.shape[0], 1, seed=1)[:, 0]
    x0 = t.solve(b)
    for _ in range(3):
        _, t2, _ = _build(32, 2, 5, 1e-5, skip=1)
        assert np.array_equal(t2.solve(b), x0)


def test_not_spd_error():
    """A non-SPD pivot is reported as an error (tree.cpp:587-590), not a crash."""
    import spand_public_gb300 as pkg
    from spand_public_gb300 import problems as P
    A = -P.neglapl(10, 2)
    X = P.linspace_nd(10, 2)
    t = pkg.Tree(3)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(X)
    t.partition(A)
    t.assemble(A)
    with pytest.raises(pkg.SpandError) as e:
        t.factorize()
    assert e.value.status == 4
    # the context is still usable
    t2 = pkg.Tree(3)
    t2.set_use_geo(True)
    t2.set_Xcoo(X)
    t2.set_verb(False)
    t2.partition(-A)
    t2.assemble(-A)
    t2.factorize()


def test_reassemble_same_pattern():
    """assemble() again with new values on the same pattern reuses the plan and the
    device work lists (values scattered on the device) and factors the new matrix."""
    import spand_public_gb300 as pkg
    from oracle.oracle import OracleTree
    from spand_public_gb300 import problems as P

    n, dim, nl, tol = 16, 3, 6, 1e-2
    A1 = P.neglapl(n, dim)
    A2 = P.reaction_diffusion3d(n, 0.37)
    assert np.array_equal(A1.indptr, A2.indptr) and np.array_equal(A1.indices, A2.indices)
    X = P.linspace_nd(n, dim)
    t = pkg.Tree(nl)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(X)
    t.set_tol(tol)
    t.partition(A1)
    t.assemble(A1)
    t.factorize()
    t.assemble(A2)
    t.factorize()
    o = OracleTree(nl)
    o.set_Xcoo(X)
    o.set_tol(tol)
    o.partition(A2)
    o.assemble(A2)
    o.factorize()
    assert np.array_equal(t.ranks(), o.ranks())
    b = P.rhs(A2.shape[0], 1, seed=4)[:, 0]
    xt, xo = t.solve(b), o.solve(b)
    assert np.linalg.norm(xt - xo) / np.linalg.norm(xo) < TOL_SOLVE


def test_reassemble_new_pattern():
    """assemble() with a different pattern after a first assemble() rebuilds the plan
    (the same-pattern shortcut of the C ABI must not take it): the result equals a fresh
    tree's, bit for bit, and going back to the first pattern does too."""
    import scipy.sparse as sp
    import spand_public_gb300 as pkg
    from spand_public_gb300 import problems as P

    n, dim, nl, tol = 12, 3, 5, 1e-2
    A1 = P.neglapl(n, dim)
    N = A1.shape[0]
    # second pattern: A1 without the couplings (i, i+1) for i = 0 mod 3 (fewer edges keep the
    # separators of A1's partition; the diagonal still dominates)
    C = A1.tocoo()
    keep = ~((np.abs(C.row - C.col) == 1) & (np.minimum(C.row, C.col) % 3 == 0))
    A2 = sp.csc_matrix((C.data[keep], (C.row[keep], C.col[keep])), shape=(N, N))
    A2.sort_indices()
    assert A2.nnz < A1.nnz
    X = P.linspace_nd(n, dim)

    def fresh(A):
        u = pkg.Tree(nl)
        u.set_verb(False)
        u.set_use_geo(True)
        u.set_Xcoo(X)
        u.set_tol(tol)
        u.partition(A1)
        u.assemble(A)
        u.factorize()
        return u

    t = fresh(A1)
    b = P.rhs(N, 1, seed=5)[:, 0]
    for A in (A2, A1):
        t.assemble(A)
        t.factorize()
        ref = fresh(A)
        assert np.array_equal(t.ranks(), ref.ranks())
        assert np.array_equal(t.solve(b), ref.solve(b))
        x, it, _ = t.cg(b, iters=100, tol=1e-10)
        assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-9


@pytest.mark.parametrize("fp32,k", [(False, 5), (True, 5), (False, 20), (True, 20)])
def test_cg_multi_matches_single(fp32, k):
    """Several right-hand sides at once: every column takes the iterations and reaches the
    solution of its own single-right-hand-side CG (the columns share the preconditioner
    applications only); a zero column stays zero after 0 iterations.  20 columns take the
    many-right-hand-side solve kernels (one block of 32, 20 lanes live)."""
    from spand_public_gb300 import problems as P
    A, t, o = _build(16, 3, 6, 1e-2, fp32=fp32)
    B = P.rhs(A.shape[0], k, seed=7)
    B[:, 3] = 0.0
    X, its, rr = t.cg(B, iters=200, tol=1e-10)
    assert X.shape == B.shape and its.shape == (k,)
    for j in range(k):
        if j == 3:
            assert its[j] == 0 and not np.any(X[:, j])
            continue
        xj, itj, rj = t.cg(B[:, j], iters=200, tol=1e-10)
        if k < 16:  # the same kernels: the same arithmetic as one column at a time
            assert its[j] == itj, (j, its[j], itj)
            assert np.linalg.norm(X[:, j] - xj) <= 1e-12 * np.linalg.norm(xj)
            assert abs(rr[j] - rj) <= 1e-12 + 1e-9 * rj
        else:  # chunked sums: rounding may move the stopping test by one iteration
            assert abs(int(its[j]) - itj) <= 1, (j, its[j], itj)
            assert np.linalg.norm(X[:, j] - xj) <= 1e-8 * np.linalg.norm(xj)
        assert np.linalg.norm(A @ X[:, j] - B[:, j]) / np.linalg.norm(B[:, j]) < 1e-9
        if not fp32 and k < 16:
            _, ito = o.cg(B[:, j], 200, 1e-10)
            assert its[j] == ito


@pytest.mark.parametrize("fp32", [False, True])
def test_solve_many_rhs(fp32):
    """The preconditioner on 40 right-hand sides at once (the many-right-hand-side kernels:
    one full block of 32 and one of 8) against the columns solved one at a time and, for
    the FP64 factor, against the oracle."""
    from spand_public_gb300 import problems as P
    A, t, o = _build(16, 3, 6, 1e-2, fp32=fp32)
    B = P.rhs(A.shape[0], 40, seed=9)
    X = t.solve(B)
    tol = 1e-5 if fp32 else 1e-12
    for j in range(0, 40, 7):
        xj = t.solve(B[:, j])
        assert np.linalg.norm(X[:, j] - xj) <= tol * np.linalg.norm(xj)
    if not fp32:
        Xo = o.solve(B)
        assert np.linalg.norm(X - Xo) <= TOL_SOLVE * np.linalg.norm(Xo)


def test_factor_graph_replay(monkeypatch):
    """factorize() replayed from its CUDA graph (captured on the second factorization,
    replayed from the third on) gives bit-identical factors to the launch-by-launch path."""
    from spand_public_gb300 import problems as P
    A = P.neglapl(16, 3)
    b = P.rhs(A.shape[0], 2, seed=9)
    monkeypatch.setenv("SPAND_FACTOR_GRAPH", "0")
    _, t0, _ = _build(16, 3, 6, 1e-2, factorizations=3)
    x0 = t0.solve(b)
    monkeypatch.delenv("SPAND_FACTOR_GRAPH")
    _, t1, o = _build(16, 3, 6, 1e-2, factorizations=3)
    assert np.array_equal(t1.ranks(), o.ranks())
    assert np.array_equal(t1.solve(b), x0)
    t1.launches(reset=True)
    t1.factorize()
    assert t1.launches(reset=True) > 0  # the replay still counts its kernels
    assert np.array_equal(t1.solve(b), x0)


@pytest.mark.parametrize("graph", ["0", "1"])
def test_tolerance_change_after_tuning(graph, monkeypatch):
    """A tree tuned at eps = 1e-2 factored again at 1e-3 (larger ranks, pivots and panels
    than its launches were sized for: the kernels take their fallback paths, then tune
    again), with and without the factorization graph: oracle parity at each tolerance."""
    from oracle.oracle import OracleTree
    from spand_public_gb300 import problems as P
    monkeypatch.setenv("SPAND_FACTOR_GRAPH", graph)
    A = P.neglapl(16, 3)
    b = P.rhs(A.shape[0], 2, seed=9)
    _, t, _ = _build(16, 3, 6, 1e-2, factorizations=3)
    o3 = OracleTree(6)
    o3.set_Xcoo(P.linspace_nd(16, 3))
    o3.set_tol(1e-3)
    o3.partition(A)
    o3.assemble(A)
    o3.factorize()
    t.set_tol(1e-3)
    for _ in range(4):  # fallback paths, re-tune, measure, graph
        t.factorize()
        assert np.array_equal(t.ranks(), o3.ranks())
        xt, xo = t.solve(b), o3.solve(b)
        assert np.linalg.norm(xt - xo) / np.linalg.norm(xo) < TOL_SOLVE


def test_relayered_waves(monkeypatch):
    """The sparsification waves re-layered after the first factorization (list scheduling
    over the dependency graph, bounded by the co-resident clusters) against the plan's
    waves: the same ranks and op list, M^{-1}b within 1e-12, and the oracle's parity."""
    from spand_public_gb300 import problems as P
    monkeypatch.setenv("SPAND_QC_RELAYER", "0")
    A, t0, o = _build(32, 3, 8, 1e-2, factorizations=3)
    monkeypatch.delenv("SPAND_QC_RELAYER")
    _, t1, _ = _build(32, 3, 8, 1e-2, factorizations=3)
    assert np.array_equal(t0.ranks(), t1.ranks())
    assert np.array_equal(t1.ranks(), o.ranks())
    assert np.array_equal(t0.ops(), t1.ops())
    b = P.rhs(A.shape[0], 2, seed=4)
    x0, x1, xo = t0.solve(b), t1.solve(b), o.solve(b)
    assert np.linalg.norm(x1 - x0) / np.linalg.norm(x0) < TOL_SOLVE
    assert np.linalg.norm(x1 - xo) / np.linalg.norm(xo) < TOL_SOLVE


@pytest.mark.parametrize("n,dim,nlevels", [(64, 2, 7), (32, 3, 8)])
def test_tensor_cores_fp32(monkeypatch, n, dim, nlevels):
    """The FP32 panel products and Schur updates on the tensor cores (TF32 head/tail
    split, FP32 accumulation) against the SIMT kernels.  Without sparsification (every
    level skipped) the factorization has no pivot decisions, and both FP32 factorizations
    are compared with the FP64 oracle's: the tensor-core blocks (ScalingLLT and Gemm) and
    M^{-1}b are within 8x the SIMT kernels' own FP32 error (plus 1e-6) -- a head/tail TF32
    product carries about 22 of FP32's 24 significand bits (measured: 1-4x).  With sparsification at eps = 1e-2 the two FP32 factorizations
    may take different (equally valid) QRCP pivots where two column norms sit at the edge
    of the FP32 tie window, so there the bar is the mixed path's own: CG to 1e-10 within
    the iteration budget of the FP64 factor."""
    from spand_public_gb300 import problems as P

    def pair(skip, tol):
        monkeypatch.setenv("SPAND_TRSM_TC", "0")
        monkeypatch.setenv("SPAND_SCHUR_TC", "0")
        A, t0, o = _build(n, dim, nlevels, tol, skip=skip, fp32=True, factorizations=2)
        monkeypatch.delenv("SPAND_TRSM_TC")
        monkeypatch.delenv("SPAND_SCHUR_TC")
        _, t1, _ = _build(n, dim, nlevels, tol, skip=skip, fp32=True, factorizations=2)
        return A, t0, t1, o

    def rel(a, b):
        return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)

    A, t0, t1, o = pair(nlevels, 1e-2)
    ops0, ops1, opo = t0.ops(), t1.ops(), o.ops()
    assert np.array_equal(ops0, ops1)
    assert np.array_equal(ops0[:, :8], opo[:, :8])
    e_simt, e_tc = 0.0, 0.0
    for k in range(ops0.shape[0]):
        kind, rows, cols = ops0[k, 0], ops0[k, 6], ops0[k, 7]
        if kind not in (0, 1, 2) or rows * cols == 0:
            continue
        a, b, c = t1.op_matrix(k, rows, cols), t0.op_matrix(k, rows, cols), o.op_matrix(k, rows, cols)
        if kind == 0:
            a, b, c = np.tril(a), np.tril(b), np.tril(c)
        e_tc, e_simt = max(e_tc, rel(a, c)), max(e_simt, rel(b, c))
    assert e_tc <= 8 * e_simt + 1e-6, (e_tc, e_simt)
    b = P.rhs(A.shape[0], 1, seed=5)[:, 0]
    x0, x1, xo = t0.solve(b), t1.solve(b), o.solve(b)
    assert rel(x1, xo) <= 8 * rel(x0, xo) + 1e-6, (rel(x1, xo), rel(x0, xo))

    A, t0, t1, _ = pair(0, 1e-2)
    _, t64, _ = _build(n, dim, nlevels, 1e-2, factorizations=1)
    _, it64, _ = t64.cg(b, iters=200, tol=1e-10)
    x1, it1, _ = t1.cg(b, iters=200, tol=1e-10)
    assert np.linalg.norm(A @ x1 - b) / np.linalg.norm(b) < 1e-9
    assert it1 <= max(it64 + 1, int(np.ceil(1.15 * it64))), (it1, it64)


@pytest.mark.parametrize("form", [{"SPAND_ORTHO_FULL": "0"}, {"SPAND_ORTHO_CLUSTER": "0"}, {}])
def test_orthogonal_op_forms(monkeypatch, form):
    """The one-right-hand-side Orthogonal op in each of its forms (blocked WY, whole-T on one
    CTA, whole-T on a thread-block cluster for the large clusters; the same for the
    triangular products with and without the warp kernel): M^{-1}b against the oracle's
    within 1e-12 relative, 3D (large top-level clusters) and 2D."""
    from spand_public_gb300 import problems as P
    for k, v in form.items():
        monkeypatch.setenv(k, v)
    if not form:
        monkeypatch.setenv("SPAND_TRSV_SMALL", "0")
    for n, dim, nlevels in ((32, 3, 8), (64, 2, 7)):
        A, t, o = _build(n, dim, nlevels, 1e-2, factorizations=2)
        b = P.rhs(A.shape[0], 2, seed=9)
        xt, xo = t.solve(b), o.solve(b)
        assert np.linalg.norm(xt - xo) / np.linalg.norm(xo) < TOL_SOLVE


def test_outgrown_launches_refactor():
    """A tree tuned at eps = 1e-2 (its waves' global-memory QRCP passes no longer queued)
    factored at eps = 1e-8: the sparsification matrices outgrow the tuned launches, the
    device status reports it, and the factorization runs again with every pass queued --
    ranks and M^{-1}b equal to the oracle's at the new tolerance, then again once re-tuned."""
    from oracle.oracle import OracleTree
    from spand_public_gb300 import problems as P
    A = P.neglapl(16, 3)
    b = P.rhs(A.shape[0], 2, seed=10)
    _, t, _ = _build(16, 3, 6, 1e-2, factorizations=3)
    o = OracleTree(6)
    o.set_Xcoo(P.linspace_nd(16, 3))
    o.set_tol(1e-8)
    o.partition(A)
    o.assemble(A)
    o.factorize()
    t.set_tol(1e-8)
    for _ in range(3):
        t.factorize()
        assert np.array_equal(t.ranks(), o.ranks())
        xt, xo = t.solve(b), o.solve(b)
        assert np.linalg.norm(xt - xo) / np.linalg.norm(xo) < TOL_SOLVE


def test_trsv_fused_identical(monkeypatch):
    """A solve phase's small-cluster and row-tile triangular products in one launch give
    bit for bit the solve of the two separate launches (the two sets of clusters are
    disjoint and each cluster runs the same code), direct and inside the CG's graph."""
    from spand_public_gb300 import problems as P
    monkeypatch.setenv("SPAND_TRSV_FUSE", "0")
    A, t0, _ = _build(32, 3, 8, 1e-2, factorizations=2)
    monkeypatch.delenv("SPAND_TRSV_FUSE")
    _, t1, _ = _build(32, 3, 8, 1e-2, factorizations=2)
    b = P.rhs(A.shape[0], 2, seed=13)
    assert np.array_equal(t0.solve(b), t1.solve(b))
    x0, it0, _ = t0.cg(b[:, 0], iters=200, tol=1e-10)
    x1, it1, _ = t1.cg(b[:, 0], iters=200, tol=1e-10)
    assert it0 == it1
    assert np.array_equal(x0, x1)


def test_pdl_sweep_identical(monkeypatch):
    """The solve sweep's kernels launched as programmatic dependents (each waits for its
    predecessor inside the kernel) give bit for bit the solve of plain stream order, direct
    and inside the CG's captured graph."""
    from spand_public_gb300 import problems as P
    monkeypatch.setenv("SPAND_PDL", "0")
    A, t0, _ = _build(32, 3, 8, 1e-2, factorizations=2)
    monkeypatch.delenv("SPAND_PDL")
    _, t1, _ = _build(32, 3, 8, 1e-2, factorizations=2)
    b = P.rhs(A.shape[0], 2, seed=12)
    assert np.array_equal(t0.solve(b), t1.solve(b))
    x0, it0, _ = t0.cg(b[:, 0], iters=200, tol=1e-10)
    x1, it1, _ = t1.cg(b[:, 0], iters=200, tol=1e-10)
    assert it0 == it1
    assert np.array_equal(x0, x1)
