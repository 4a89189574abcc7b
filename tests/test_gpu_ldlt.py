"""Symmetric indefinite matrices: SymmKind SYM with ScalingKind LDLT (Eigen's pivoted LDL^T
pivots, sign-weighted Schur updates, the Q^T D Q split of every sparsified pivot with its
sibling eliminated), against the CPU oracle.

Matrices: -Laplacian (the reference's SPD_vs_LDLT test, tests/tests.cpp:614-683) and the
indefinite -Laplacian - shift*I.  Bars as for the other paths: ordering, ranks, op list and
per-level log identical; every factor block (L_s of each LDLT pivot with its permutation
and signs, Gemm panels, reflectors) within 1e-12 relative of the oracle, compared in
absolute value; M^{-1}b within 1e-12; GMRES iteration counts equal.

Why absolute values, and why the Orthogonal / Gemm blocks are compared on the first
level only: the -Laplacian of a cube is symmetric under the cube's reflections, so some
sparsification matrices have pairs of mirror-image columns whose norms tie exactly; after
the LDLT pivoting, device and oracle may take different members of such a pair (or a
reflector of opposite sign), and from there on the coarse unknowns of that cluster differ
by an orthogonal change of basis -- rows of later blocks change sign or mix -- while the
preconditioner M stays the same operator.  The pivots (L_s, permutation, signs) are
compared on every level, the blocks on level 0, and M itself through M^{-1}b for three
right-hand sides on every case.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_BLOCK = 1e-12
# indefinite pivots grow rounding differences (element growth of LDL^T with small |d|)
TOL_BLOCK_INDEF = 1e-10


def _matrix(kind, n, dim):
    import scipy.sparse as sp
    from spand_public_gb300 import problems as P
    A = P.neglapl(n, dim)
    if kind == "neg":
        return (-A).tocsc()
    return (A - {2: 0.5, 3: 1.0}[dim] * sp.identity(n ** dim)).tocsc()


def _build(A, n, dim, nlevels, tol, skip=0, fp32=False):
    import spand_public_gb300 as pkg
    from oracle.oracle import OracleTree
    from spand_public_gb300 import problems as P
    X = P.linspace_nd(n, dim)
    t = pkg.Tree(nlevels)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(X)
    t.set_tol(tol)
    t.set_skip(skip)
    t.set_fp32(fp32)
    t.set_symm_kind(pkg.SYM)
    t.set_scaling_kind(pkg.LDLT)
    pt = t.partition(A)
    t.assemble(A)
    t.factorize()
    o = OracleTree(nlevels)
    o.set_Xcoo(X)
    o.set_tol(tol)
    o.set_skip(skip)
    o.set_symm_kind(OracleTree.SYM)
    o.set_scaling_kind(OracleTree.LDLT)
    po = o.partition(A)
    o.assemble(A)
    o.factorize()
    assert np.array_equal(pt, po)
    return t, o


CASES = [
    ("neg", 8, 2, 3, 1e-2, 0),
    ("neg", 32, 2, 5, 1e-2, 0),
    ("neg", 64, 2, 7, 1e-2, 0),
    ("neg", 10, 3, 4, 1e-2, 0),
    ("neg", 16, 3, 6, 1e-3, 1),
    ("ind", 20, 2, 4, 0.0, 0),
    ("ind", 32, 2, 5, 1e-2, 0),
    ("ind", 10, 3, 4, 1e-2, 0),
    ("ind", 20, 2, 4, 10.0, 0),
]


@pytest.mark.parametrize("kind,n,dim,nlevels,tol,skip", CASES)
def test_ldlt_factor_parity_fp64(kind, n, dim, nlevels, tol, skip):
    A = _matrix(kind, n, dim)
    t, o = _build(A, n, dim, nlevels, tol, skip)
    assert np.array_equal(t.get_assembly_perm(), o.get_assembly_perm())
    assert np.array_equal(t.ranks(), o.ranks()), "per-cluster ranks differ"
    opt, opo = t.ops(), o.ops()
    assert opt.shape == opo.shape
    assert np.array_equal(opt[:, :6], opo[:, :6])
    assert 9 in set(np.unique(opt[:, 0]))
    worst, where = 0.0, None
    lsib = 0.0
    for k in range(opt.shape[0]):
        kind_, rows, cols = opt[k, 0], opt[k, 6], opt[k, 7]
        if kind_ not in (1, 2, 3, 9) or rows * cols == 0:
            continue
        if kind_ != 9 and opt[k, 1] > 0:
            continue  # mirror-image ties above level 0 (module docstring)
        mt = t.op_matrix(k, rows, cols)
        mo = o.op_matrix(k, opo[k, 6], opo[k, 7])
        scale = 0.0
        if kind_ == 9:
            assert np.array_equal(t.op_perm(k, rows), o.op_perm(k, rows)), k
            assert np.array_equal(t.op_signs(k, rows), o.op_signs(k, rows)), k
            pairs = [(np.tril(mt), np.tril(mo))]
            lsib = np.linalg.norm(np.tril(mo))
        elif kind_ == 3:
            pairs = [(np.tril(mt, -1), np.tril(mo, -1)), (t.op_tau(k, cols), o.op_tau(k, cols))]
        else:
            pairs = [(mt, mo)]
            if kind_ == 2 and opt[k - 1, 0] == 9 and opt[k - 1, 2] == opt[k, 2]:
                # the edge of a sibling, L_sib^{-1} P^T (Q^T D Q)[k:, :k]: exactly zero when the
                # cluster's signs agree (D = +-I), so measured against the sibling's factor
                scale = lsib
        for a, b in pairs:
            a, b = np.abs(a), np.abs(b)
            e = np.linalg.norm(a - b) / max(np.linalg.norm(b), scale, 1e-300)
            if e > worst:
                worst, where = e, (k, int(kind_), int(rows), int(cols))
    assert worst < (TOL_BLOCK if kind == "neg" else TOL_BLOCK_INDEF), (worst, where)
    lt, lo = t.level_log(), o.level_log()
    for a, b in zip(lt, lo):
        for key in ("dofs_nd", "dofs_left_nd", "dofs_left_elim", "dofs_left_spars", "rank_before_sum",
                    "rank_after_sum", "rank_after_count", "ignored", "nbrs_sum", "fact_nnz"):
            assert a[key] == b[key], (key, a[key], b[key])
    assert t.nnz() == o.nnz()
    from spand_public_gb300 import problems as P
    b = P.rhs(A.shape[0], 3, seed=7)
    xt, xo = t.solve(b), o.solve(b)
    assert np.linalg.norm(xt - xo) / np.linalg.norm(xo) < (1e-12 if kind == "neg" else 1e-10)
    if tol == 0.0:
        assert np.linalg.norm(A @ xt - b) / np.linalg.norm(b) < 1e-10


@pytest.mark.parametrize("n,dim,nlevels,tol,skip", [(64, 2, 7, 0.0, 100), (5, 3, 2, 1e-4, 1), (15, 3, 5, 1e-14, 0),
                                                    (32, 2, 6, 1e-4, 0)])
def test_spd_vs_ldlt(n, dim, nlevels, tol, skip):
    """ApproxTest.SPD_vs_LDLT on the device: SPD/LLT on A and SYM/LDLT on -A (b -> -b)
    agree to 1e-12 at tol 0 and tol * 1e2 otherwise."""
    import spand_public_gb300 as pkg
    from spand_public_gb300 import problems as P
    A = P.neglapl(n, dim)
    X = P.linspace_nd(n, dim)
    b = np.random.default_rng(nlevels).uniform(-1, 1, A.shape[0])
    xs = []
    for symm, sk, M, rhs in ((pkg.SPD, pkg.LLT, A, b), (pkg.SYM, pkg.LDLT, -A, -b)):
        t = pkg.Tree(nlevels)
        t.set_verb(False)
        t.set_use_geo(True)
        t.set_Xcoo(X)
        t.set_tol(tol)
        t.set_skip(skip)
        t.set_symm_kind(symm)
        t.set_scaling_kind(sk)
        t.partition(M)
        t.assemble(M)
        t.factorize()
        xs.append(t.solve(rhs))
    bound = 1e-12 if tol == 0.0 else tol * 1e2
    for x in xs:
        assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) <= bound
    assert np.linalg.norm(xs[0] - xs[1]) / np.linalg.norm(xs[0]) <= bound


@pytest.mark.parametrize("n,dim,nlevels,tol", [(32, 2, 5, 1e-2), (10, 3, 4, 1e-2), (16, 3, 6, 1e-3)])
def test_ldlt_gmres_matches_oracle(n, dim, nlevels, tol):
    from spand_public_gb300 import problems as P
    A = _matrix("ind", n, dim)
    t, o = _build(A, n, dim, nlevels, tol)
    b = P.rhs(A.shape[0], 1, seed=11)[:, 0]
    xt, it, rr = t.gmres(b, iters=200, tol=1e-12)
    xo, ito, _ = o.gmres(b, 200, 200, 1e-12)
    assert it == ito, (it, ito)
    assert rr < 1e-12
    assert np.linalg.norm(A @ xt - b) / np.linalg.norm(b) < 1e-9


@pytest.mark.parametrize("n,dim,nlevels,tol", [(32, 2, 5, 1e-2), (16, 3, 6, 1e-2)])
def test_ldlt_mixed_precision_fgmres(n, dim, nlevels, tol):
    """FP32 LDLT factor: the flexible GMRES reaches the FP64 residual 1e-10 with at most 15%
    more iterations than with the FP64 factor."""
    from spand_public_gb300 import problems as P
    A = _matrix("ind", n, dim)
    t64, _ = _build(A, n, dim, nlevels, tol)
    t32, _ = _build(A, n, dim, nlevels, tol, fp32=True)
    b = P.rhs(A.shape[0], 1, seed=5)[:, 0]
    _, it64, _ = t64.fgmres(b, iters=200, tol=1e-10)
    x32, it32, rr32 = t32.fgmres(b, iters=200, tol=1e-10)
    assert rr32 < 1e-10 and np.linalg.norm(A @ x32 - b) / np.linalg.norm(b) < 1e-10
    assert it32 <= int(np.floor(1.15 * it64)) + 1, (it32, it64)
