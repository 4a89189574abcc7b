"""LoRaSp (partition_lorasp tree.cpp:421-503, factorize_lorasp tree.cpp:1553-1608) on the
device against the CPU oracle, SPD / LLT: ordering identical; per-cluster ranks, op list
(kinds, levels, clusters, sizes) and per-level log identical; every factor block (the
scaled pivots, the siblings' Gemm blocks, the reflectors and tau) and M^{-1}b within
max(1e-12, 100 x the oracle's own rounding sensitivity), measured per block as the
difference between the oracle and the oracle run on A with its values moved by one unit in
the last place (pattern and symmetry kept); CG iterations equal; exact at tol 0.  At tol
1e-2 the bar is 1e-12 almost everywhere; at 1e-4 the QRCPs keep columns down to 1e-4 of
the largest, whose reflectors the reference's own algorithm fixes only to ~1e-9.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_BLOCK = 1e-12


def _oracle(A, X, nlevels, tol):
    from oracle.oracle import OracleTree
    o = OracleTree(nlevels)
    o.set_Xcoo(X)
    o.set_tol(tol)
    po = o.partition_lorasp(A)
    o.assemble(A)
    o.factorize_lorasp()
    return o, po


def _ulp_moved(A, seed=1):
    """A with every stored value moved by one unit in the last place, symmetrically."""
    import scipy.sparse as sp
    C = sp.triu(A).tocoo()
    d = C.data + np.spacing(np.abs(C.data)) * np.random.default_rng(seed).choice([-1.0, 1.0], C.data.shape)
    U = sp.coo_matrix((d, (C.row, C.col)), shape=A.shape)
    B = (U + sp.triu(U, 1).T).tocsc()
    B.sort_indices()
    assert np.array_equal(B.indptr, A.indptr) and np.array_equal(B.indices, A.indices)
    return B


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _blocks(t, ops, k):
    kind, rows, cols = ops[k, 0], ops[k, 6], ops[k, 7]
    m = t.op_matrix(k, rows, cols)
    if kind == 0:
        return [np.tril(m)]
    if kind == 3:
        return [np.tril(m, -1), t.op_tau(k, cols)]
    return [m]


def _trees(n, dim, nlevels, tol, fp32=False):
    import spand_public_gb300 as pkg
    from spand_public_gb300 import problems as P
    A = P.neglapl(n, dim)
    X = P.linspace_nd(n, dim)
    t = pkg.Tree(nlevels)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(X)
    t.set_tol(tol)
    t.set_fp32(fp32)
    pt = t.partition_lorasp(A)
    t.assemble(A)
    t.factorize_lorasp()
    o, po = _oracle(A, X, nlevels, tol)
    assert np.array_equal(pt, po)
    assert np.array_equal(t.get_assembly_perm(), o.get_assembly_perm())
    return A, t, o


CASES = [
    (10, 2, 3, 1e-2),
    (20, 2, 4, 1e-2),
    (32, 2, 5, 1e-2),
    (32, 2, 5, 1e-4),
    (64, 2, 6, 1e-3),
    (10, 3, 4, 1e-2),
    (16, 3, 6, 1e-2),
    (16, 3, 5, 1e-4),
]


@pytest.mark.parametrize("n,dim,nlevels,tol", CASES)
def test_lorasp_parity_fp64(n, dim, nlevels, tol):
    from spand_public_gb300 import problems as P
    A, t, o = _trees(n, dim, nlevels, tol)
    o2, _ = _oracle(_ulp_moved(A), P.linspace_nd(n, dim), nlevels, tol)
    assert np.array_equal(t.ranks(), o.ranks()), "per-cluster ranks differ"
    assert np.array_equal(o2.ranks(), o.ranks())
    opt, opo = t.ops(), o.ops()
    assert opt.shape == opo.shape
    assert np.array_equal(opt[:, :6], opo[:, :6])
    tight = 0
    for k in range(opt.shape[0]):
        kind, rows, cols = opt[k, 0], opt[k, 6], opt[k, 7]
        if kind not in (0, 2, 3) or rows * cols == 0:
            continue
        for a, b, c in zip(_blocks(t, opt, k), _blocks(o, opo, k), _blocks(o2, opo, k)):
            bar = max(TOL_BLOCK, 100.0 * _rel(c, b))
            assert _rel(a, b) <= bar, (k, kind, opt[k, 1], _rel(a, b), bar)
            tight += bar == TOL_BLOCK
    assert tight > 0
    lt, lo = t.level_log(), o.level_log()
    for a, b in zip(lt, lo):
        for key in ("dofs_left_spars", "rank_before_sum", "rank_after_sum", "rank_after_count", "fact_nnz"):
            assert a[key] == b[key], (key, a[key], b[key])
    assert t.nnz() == o.nnz()
    b = P.rhs(A.shape[0], 3, seed=7)
    xt, xo, x2 = t.solve(b), o.solve(b), o2.solve(b)
    assert _rel(xt, xo) <= max(1e-12, 100.0 * _rel(x2, xo))
    b1 = b[:, 0].copy()
    _, it, _ = t.cg(b1, iters=100, tol=1e-10)
    _, ito = o.cg(b1, 100, 1e-10)[:2]
    assert it == ito, (it, ito)


@pytest.mark.parametrize("n,dim,nlevels", [(20, 2, 4), (32, 2, 5), (10, 3, 4)])
def test_lorasp_exact(n, dim, nlevels):
    """tol 0: an exact factorization (ApproxTest.Exact's bar, 1e-10), as the oracle's."""
    from spand_public_gb300 import problems as P
    A, t, o = _trees(n, dim, nlevels, 0.0)
    b = P.rhs(A.shape[0], 1, seed=3)[:, 0]
    x = t.solve(b)
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-10
    xo = o.solve(b)
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-10


def test_lorasp_fp32_cg():
    """FP32 factor: PCG to 1e-10 with at most 15% more iterations than with the FP64 factor."""
    from spand_public_gb300 import problems as P
    A, t64, _ = _trees(16, 3, 6, 1e-2)
    _, t32, _ = _trees(16, 3, 6, 1e-2, fp32=True)
    b = P.rhs(A.shape[0], 1, seed=2)[:, 0]
    x64, it64, _ = t64.cg(b, iters=200, tol=1e-10)
    x32, it32, _ = t32.cg(b, iters=200, tol=1e-10)
    for x in (x64, x32):
        assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-9
    assert it32 <= int(np.floor(1.15 * it64)) + 1, (it32, it64)


def test_lorasp_api_errors():
    """factorize() on a LoRaSp-partitioned tree and factorize_lorasp() on a spaND one are
    refused; LoRaSp is SPD / LLT only."""
    import spand_public_gb300 as pkg
    from spand_public_gb300 import problems as P
    A = P.neglapl(10, 2)
    X = P.linspace_nd(10, 2)

    def tree():
        t = pkg.Tree(3)
        t.set_verb(False)
        t.set_use_geo(True)
        t.set_Xcoo(X)
        return t

    t = tree()
    t.partition_lorasp(A)
    t.assemble(A)
    with pytest.raises(pkg.SpandError):
        t.factorize()
    t.factorize_lorasp()
    u = tree()
    u.partition(A)
    u.assemble(A)
    with pytest.raises(pkg.SpandError):
        u.factorize_lorasp()
    v = tree()
    v.set_symm_kind(pkg.SYM)
    v.set_scaling_kind(pkg.LDLT)
    v.partition_lorasp(A)
    with pytest.raises(pkg.SpandError):
        v.assemble(-A)
