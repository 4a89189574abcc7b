"""The CPU oracle pinned against the reference's own tests and fixtures.

Golden vectors come from tests/golden/reference_golden.json (generated from the
reference's tests/tests.cpp and mats/*.mm by tests/golden/make_golden.py).  Tolerances
and loops follow the reference's gtest cases, cited per test.  The reference runs its
end-to-end cases with algebraic (METIS) ordering; METIS is not restated, so those cases
run here with the geometric ordering on the grid coordinates, which the reference test
PartitionTest.Consistency exercises in the same loops.
"""
import numpy as np
import pytest
import scipy.linalg as sla
import scipy.sparse as sp

from oracle import oracle as O
from spand_public_gb300 import problems as P


def test_choose_rank(golden):
    """Util.ChooseRank (tests/tests.cpp:254-262)."""
    g = golden["choose_rank"]
    for tol, rank in g["cases"]:
        assert O.choose_rank(g["s"], tol) == rank


def test_linspace_nd(golden):
    """Util.LinspaceNd (tests/tests.cpp:301-310)."""
    g = golden["linspace_nd"]
    assert np.array_equal(P.linspace_nd(3, 2), np.array(g["n3d2_rowmajor"]).reshape(2, 9))
    assert np.array_equal(P.linspace_nd(2, 3), np.array(g["n2d3_rowmajor"]).reshape(3, 8))


def test_neglapl_fixtures(golden):
    """The generators reproduce mats/neglapl_{d}_{n}.mm bit for bit."""
    import hashlib

    for fn, m in golden["neglapl"].items():
        A = P.neglapl(m["n"], m["dim"]).tocoo()
        o = np.lexsort((A.row, A.col))
        h = hashlib.sha256()
        h.update(A.row[o].astype(np.int64).tobytes())
        h.update(A.col[o].astype(np.int64).tobytes())
        h.update(A.data[o].astype(np.float64).tobytes())
        assert A.shape[0] == m["N"] and A.nnz == m["nnz"] and h.hexdigest() == m["sha256"], fn


def _sep(a):
    return [list(map(int, r)) for r in a]


def test_partition_square(golden):
    """PartitionTest.Square (tests/tests.cpp:378-412): exact (self, left, right) SepIDs."""
    g = golden["partition_square"]
    A = P.neglapl(5, 2)
    t = O.OracleTree(3)
    t.set_Xcoo(P.linspace_nd(5, 2))
    part = t.partition(A)
    assert _sep(part[:, 0:2]) == g["sepidref"]
    assert _sep(part[:, 2:4]) == g["leftref"]
    assert _sep(part[:, 4:6]) == g["rightref"]


def _disconnected(l1, l2, s1, s2):
    # should_be_disconnected, src/util.cpp:26-42
    while l2 > l1:
        l1 += 1
        s1 //= 2
    while l1 > l2:
        l2 += 1
        s2 //= 2
    return s1 != s2


@pytest.mark.parametrize("dim,n", [(2, 5), (2, 20), (2, 100), (3, 5), (3, 15)])
def test_partition_consistency(dim, n):
    """PartitionTest.Consistency (tests/tests.cpp:417-481), geometric MND, levels 1..7."""
    A = P.neglapl(n, dim).tocsc()
    X = P.linspace_nd(n, dim)
    for nlevels in range(1, 8):
        t = O.OracleTree(nlevels)
        t.set_Xcoo(X)
        part = t.partition(A)
        assert part.shape[0] == n ** dim
        for j in range(A.shape[0]):
            for i in A.indices[A.indptr[j]:A.indptr[j + 1]]:
                assert not _disconnected(part[j, 0], part[i, 0], part[j, 1], part[i, 1])
        for k in range(part.shape[0]):
            pl, ps, ll, ls, rl, rs = part[k]
            if pl == 0:
                assert (ll, ls) == (pl, ps) and (rl, rs) == (pl, ps)
            else:
                assert pl > ll and pl > rl
                while ll < pl - 1:
                    ll, ls = ll + 1, ls // 2
                while rl < pl - 1:
                    rl, rs = rl + 1, rs // 2
                assert (ll, ls) == (pl - 1, 2 * ps) and (rl, rs) == (pl - 1, 2 * ps + 1)


@pytest.mark.parametrize("dim,n", [(2, 5), (2, 10), (2, 20), (3, 5), (3, 10)])
def test_assembly_consistency(dim, n):
    """Assembly.Consistency (tests/tests.cpp:488-547): trailing matrix == P^T A P exactly."""
    A = P.neglapl(n, dim)
    X = P.linspace_nd(n, dim)
    for nlevels in range(2, 5):
        for lorasp in (False, True):  # the reference loops over partition / partition_lorasp
            t = O.OracleTree(nlevels)
            t.set_Xcoo(X)
            if lorasp:
                t.partition_lorasp(A)
            else:
                t.partition(A)
            t.assemble(A)
            p = t.get_assembly_perm()
            ref = A[p][:, p]
            assert abs(ref - t.trailing()).max() == 0.0


def test_swap2perm_via_getf(golden):
    """The LU pivot vector of the restated dgetrf follows swap2perm (tests/tests.cpp:349-357):
    perm^T x <=> x[perm]."""
    rng = np.random.default_rng(0)
    M = rng.standard_normal((7, 7))
    LU, perm, info = O.dense_getf(M)
    assert info == 0
    L = np.tril(LU, -1) + np.eye(7)
    U = np.triu(LU)
    assert np.allclose(M[perm], L @ U, atol=1e-12)


def test_dense_kernels_vs_lapack():
    """Restated dpotrf / dgeqp3 / dgetrf agree with LAPACK (scipy) on random inputs."""
    rng = np.random.default_rng(1)
    for n in (1, 5, 17, 64):
        B = rng.standard_normal((n, n))
        S = B @ B.T + n * np.eye(n)
        L, info = O.dense_potf(S)
        assert info == 0
        assert np.allclose(L, np.linalg.cholesky(S), rtol=1e-12, atol=1e-12)
    for m, n in ((5, 9), (20, 20), (17, 130), (64, 300)):
        A = rng.standard_normal((m, n)) * np.logspace(0, -6, n)[None, :]
        QR, jp, tau = O.dense_geqp3(A)
        qr_l, jp_l, tau_l, _, _ = sla.lapack.dgeqp3(np.asfortranarray(A.copy()))
        assert np.array_equal(jp, jp_l - 1)
        assert np.allclose(np.triu(QR[: min(m, n)]), np.triu(qr_l[: min(m, n)]), rtol=1e-10, atol=1e-12)
        assert np.allclose(tau, tau_l, rtol=1e-10, atol=1e-12)
    _, info = O.dense_potf(-np.eye(3))
    assert info == 1


def _solve_err(A, t, seed):
    b = np.random.default_rng(seed).uniform(-1, 1, A.shape[0])
    x = t.solve(b)
    return np.linalg.norm(A @ x - b) / np.linalg.norm(b)


@pytest.mark.parametrize("dim,n", [(2, 5), (2, 10), (2, 20), (3, 5), (3, 15)])
def test_approx_exact(dim, n):
    """ApproxTest.Exact (tests/tests.cpp:562-609), SPD/LLT: tol 1e-14 (skip 0, 4) and 0
    (skip 1000) give |Ax-b|/|b| <= 1e-10."""
    A = P.neglapl(n, dim)
    X = P.linspace_nd(n, dim)
    N = A.shape[0]
    lmin = 1 if N < 1000 else 8
    for nlevels in range(lmin, lmin + 5):
        for tol, skip in ((1e-14, 0), (1e-14, 4), (0.0, 1000)):
            t = O.OracleTree(nlevels)
            t.set_Xcoo(X)
            t.partition(A)
            t.assemble(A)
            t.set_tol(tol)
            t.set_skip(skip)
            t.factorize()
            assert _solve_err(A, t, nlevels) <= 1e-10


@pytest.mark.parametrize("dim,n", [(2, 5), (2, 10), (2, 20), (2, 128), (3, 5), (3, 15)])
def test_approx(dim, n):
    """ApproxTest.Approx (tests/tests.cpp:799-856), SPD/LLT: err <= tol * 2e2, and
    <= 5e-12 at tol 0; skip 0..2."""
    A = P.neglapl(n, dim)
    X = P.linspace_nd(n, dim)
    N = A.shape[0]
    lmin = 1 if N < 1000 else 8
    levels = range(lmin, lmin + 5) if N < 5000 else (lmin, lmin + 2, lmin + 4)
    for nlevels in levels:
        for tol in (0.0, 1e-10, 1e-6, 1e-2, 10.0):
            for skip in range(3):
                t = O.OracleTree(nlevels)
                t.set_Xcoo(X)
                t.partition(A)
                t.assemble(A)
                t.set_tol(tol)
                t.set_skip(skip)
                t.factorize()
                err = _solve_err(A, t, nlevels + skip)
                assert err <= (5e-12 if tol == 0.0 else tol * 2e2), (nlevels, tol, skip, err)


def test_repro():
    """ApproxTest.Repro (tests/tests.cpp:917-994): identical x over repeated runs."""
    A = P.neglapl(20, 2)
    X = P.linspace_nd(20, 2)
    b = np.random.default_rng(3).uniform(-1, 1, A.shape[0])
    for tol, skip in ((1e-5, 1), (10.0, 2), (1e-8, 0), (0.1, 1)):
        xs = []
        for _ in range(3):
            t = O.OracleTree(5)
            t.set_Xcoo(X)
            t.partition(A)
            t.assemble(A)
            t.set_tol(tol)
            t.set_skip(skip)
            t.factorize()
            xs.append(t.solve(b))
        assert all(np.array_equal(xs[0], x) for x in xs[1:])


def test_not_spd_raises():
    """Non-SPD pivot raises (src/tree.cpp:587-590)."""
    A = -P.neglapl(6, 2)
    t = O.OracleTree(3)
    t.set_Xcoo(P.linspace_nd(6, 2))
    t.partition(A)
    t.assemble(A)
    with pytest.raises(RuntimeError, match="Non-SPD"):
        t.factorize()


def test_cg_converges():
    """CG driver (src/is.cpp:39-121) reaches the tolerance on a 64x64 grid."""
    A = P.neglapl(64, 2)
    t = O.OracleTree(7)
    t.set_Xcoo(P.linspace_nd(64, 2))
    t.partition(A)
    t.assemble(A)
    t.set_tol(1e-2)
    t.factorize()
    b = P.rhs(A.shape[0], 1, 0)[:, 0]
    x, it = t.cg(b, 100, 1e-12)
    assert it < 20
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-11


@pytest.mark.parametrize("dim,n", [(2, 128), (3, 5), (3, 15)])
def test_spd_vs_ldlt(dim, n):
    """ApproxTest.SPD_vs_LDLT (tests/tests.cpp:614-683): SPD/LLT on A and SYM/LDLT on -A
    (b -> -b) agree; errors and difference <= 1e-12 at tol 0, <= tol * 1e2 otherwise."""
    A = P.neglapl(n, dim)
    X = P.linspace_nd(n, dim)
    N = A.shape[0]
    lmin = 1 if N < 1000 else 8
    levels = range(lmin, lmin + 5) if N < 5000 else (lmin, lmin + 2, lmin + 4)
    for nlevels in levels:
        for tol, skip in ((0.0, 100), (1e-4, 1), (1e-14, 0)):
            b = np.random.default_rng(nlevels).uniform(-1, 1, N)
            t = O.OracleTree(nlevels)
            t.set_Xcoo(X)
            t.set_tol(tol)
            t.set_skip(skip)
            t.partition(A)
            t.assemble(A)
            t.factorize()
            xl = t.solve(b)
            u = O.OracleTree(nlevels)
            u.set_Xcoo(X)
            u.set_tol(tol)
            u.set_skip(skip)
            u.set_symm_kind(O.OracleTree.SYM)
            u.set_scaling_kind(O.OracleTree.LDLT)
            u.partition(-A)
            u.assemble(-A)
            u.factorize()
            xd = u.solve(-b)
            bound = 1e-12 if tol == 0.0 else tol * 1e2
            for x in (xl, xd):
                assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) <= bound
            assert np.linalg.norm(xl - xd) / np.linalg.norm(xl) <= bound


@pytest.mark.parametrize("dim,n,shift", [(2, 20, 0.5), (3, 10, 1.0)])
def test_ldlt_indefinite(dim, n, shift):
    """SYM/LDLT on the indefinite -Laplacian - shift*I (a few negative eigenvalues, the
    smallest |eigenvalue| near 0.05): exact at tol 0 (<= 1e-10, ApproxTest.Exact); at tol
    1e-6 the error is amplified by the conditioning (<= 1e-2) and GMRES converges fast."""
    A = (P.neglapl(n, dim) - shift * sp.identity(n ** dim)).tocsc()
    X = P.linspace_nd(n, dim)
    b = np.random.default_rng(1).uniform(-1, 1, A.shape[0])
    for nlevels in (3, 5):
        for tol in (0.0, 1e-6):
            u = O.OracleTree(nlevels)
            u.set_Xcoo(X)
            u.set_tol(tol)
            u.set_symm_kind(O.OracleTree.SYM)
            u.set_scaling_kind(O.OracleTree.LDLT)
            u.partition(A)
            u.assemble(A)
            u.factorize()
            x = u.solve(b)
            err = np.linalg.norm(A @ x - b) / np.linalg.norm(b)
            assert err <= (1e-10 if tol == 0.0 else 1e-2), (nlevels, tol, err)
    x, it, rr = u.gmres(b, 50, 50, 1e-12)
    assert rr < 1e-12 and it < 20
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-10


def test_plu_exact_and_gmres():
    """GEN/PLU (ApproxTest.Exact with neglapl_unsym): exact at tol 0; restarted GMRES
    converges with every restart length."""
    A = P.neglapl_unsym(20, 2, seed=3)
    X = P.linspace_nd(20, 2)
    b = np.random.default_rng(2).uniform(-1, 1, A.shape[0])
    for tol in (0.0, 1e-2):
        u = O.OracleTree(5)
        u.set_Xcoo(X)
        u.set_tol(tol)
        u.set_symm_kind(O.OracleTree.GEN)
        u.set_scaling_kind(O.OracleTree.PLU)
        u.partition(A)
        u.assemble(A)
        u.factorize()
        if tol == 0.0:
            assert np.linalg.norm(A @ u.solve(b) - b) / np.linalg.norm(b) <= 1e-10
    for restart in (1, 3, 100):
        x, it, rr = u.gmres(b, 200, restart, 1e-12)
        assert rr < 1e-12 and np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-10


def _preserved(t, A, phi):
    """max over the columns of phi of |A x - A phi| / |A phi| and |x - phi| / |phi|, x = M^{-1} A phi."""
    e = 0.0
    for c in range(phi.shape[1]):
        b = A @ phi[:, c]
        x = t.solve(b)
        e = max(e, np.linalg.norm(A @ x - b) / np.linalg.norm(b),
                np.linalg.norm(x - phi[:, c]) / np.linalg.norm(phi[:, c]))
    return e


@pytest.mark.parametrize("dim,n", [(2, 5), (2, 10), (2, 20), (3, 5), (3, 10)])
def test_preservation(dim, n):
    """ApproxTest.Preservation (tests/tests.cpp:686-797): with preservation on, the
    preconditioner reproduces phi (the ones vector, and 5 random vectors) to 1e-12 for A
    (SPD / LLT) and -A (SYM / LDLT); a random b is solved to tol * 1e2 (1e-12 at tol 0).
    Tolerance 10 takes the preserve-only branch (tree.cpp:1257-1287), the others the
    preserve + RRQR branch (tree.cpp:1350-1409).  Levels and skips are a subset of the
    reference's loops (it runs nlevels..nlevels+4 and skip 0..2)."""
    A_spd = P.neglapl(n, dim)
    X = P.linspace_nd(n, dim)
    N = A_spd.shape[0]
    lmin = 1 if N < 1000 else 8
    for nlevels in (lmin, lmin + 2, lmin + 4):
        for tol in (10.0, 1e-2, 1e-4, 0.0):
            for skip in (0, 2):
                for symm in (0, 1):
                    A = A_spd if symm == 0 else -A_spd
                    for phi in (np.ones((N, 1)),
                                np.random.default_rng(nlevels + skip + 2019).uniform(-1, 1, (N, 5))):
                        t = O.OracleTree(nlevels)
                        t.set_Xcoo(X)
                        if symm:
                            t.set_symm_kind(O.OracleTree.SYM)
                            t.set_scaling_kind(O.OracleTree.LDLT)
                        t.partition(A)
                        t.assemble(A)
                        t.set_tol(tol)
                        t.set_skip(skip)
                        t.set_preserve(True)
                        t.set_phi(phi)
                        t.factorize()
                        assert _preserved(t, A, phi) < 1e-12, (nlevels, tol, skip, symm)
                        b = np.random.default_rng(nlevels + skip + 2019).uniform(-1, 1, N)
                        x = t.solve(b)
                        err = np.linalg.norm(A @ x - b) / np.linalg.norm(b)
                        assert err < (1e-12 if tol == 0.0 else tol * 1e2), (nlevels, tol, skip, symm, err)


@pytest.mark.parametrize("dim,n", [(2, 5), (2, 10), (2, 20), (2, 64), (3, 5), (3, 15)])
def test_lorasp(dim, n):
    """ApproxTest.ApproxLoRaSp (tests/tests.cpp:858-912), SPD / LLT configuration:
    partition_lorasp + factorize_lorasp for nlevels, ..., nlevels + 4 and tol in
    {0, 1e-10, 1e-6, 1e-4}; |Ax - b| / |b| <= 5e-12 at tol 0, <= tol * 2e2 otherwise (the
    reference's b is a seeded uniform vector, restated here with numpy's generator).  Also:
    2^(nlevels-1) parts, and PCG converges."""
    A = P.neglapl(n, dim)
    X = P.linspace_nd(n, dim)
    N = A.shape[0]
    lmin = 1 if N < 1000 else 8
    for nlevels in range(lmin, lmin + 5):
        for tol in (0.0, 1e-10, 1e-6, 1e-4):
            t = O.OracleTree(nlevels)
            t.set_Xcoo(X)
            t.set_tol(tol)
            parts = t.partition_lorasp(A)
            assert np.bincount(parts, minlength=2 ** (nlevels - 1)).size == 2 ** (nlevels - 1)
            t.assemble(A)
            t.factorize_lorasp()
            b = np.random.default_rng(nlevels + 2019).uniform(-1, 1, N)
            x = t.solve(b)
            err = np.linalg.norm(A @ x - b) / np.linalg.norm(b)
            assert err <= (5e-12 if tol == 0.0 else tol * 2e2), (nlevels, tol, err)
            x, it = t.cg(b, 100, 1e-10)[:2]
            assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-9


def test_lapack_mode_baseline():
    """The timed CPU baseline (bench.py) runs the oracle with the reference's BLAS / LAPACK
    calls (scipy's OpenBLAS: dgemm, dsyrk, dtrsm, dpotrf, and LAPACK's own dgeqp3 without the
    tie rule).  It must compute the same preconditioner up to pivot ties: CG to 1e-10 with
    at most one iteration more or less than the restated oracle, every cluster's rank within
    one of the restated oracle's (equal on this case)."""
    A = P.neglapl(16, 3)
    X = P.linspace_nd(16, 3)
    b = np.random.default_rng(0).uniform(-1, 1, A.shape[0])
    res = {}
    try:
        for mode in ("restated", "lapack"):
            if mode == "lapack" and O.use_lapack(1) is None:
                pytest.skip("no CBLAS / LAPACKE library found next to scipy")
            t = O.OracleTree(6)
            t.set_Xcoo(X)
            t.set_tol(1e-2)
            t.partition(A)
            t.assemble(A)
            t.factorize()
            x, it = t.cg(b, 100, 1e-10)[:2]
            assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-9
            res[mode] = (it, t.ranks())
    finally:
        O.use_restated()
    assert abs(res["restated"][0] - res["lapack"][0]) <= 1
    ra, rb = res["restated"][1], res["lapack"][1]
    assert np.array_equal(ra[:, :3], rb[:, :3])
    assert np.abs(ra[:, 3] - rb[:, 3]).max() <= 1
