"""Edge cases on the device for the three factorization kinds (SPD/LLT, SYM/LDLT, GEN/PLU)
against the oracle: 1x1 to 3x3 systems, one and two levels, every level skipped, a
tolerance at which every sparsified cluster keeps no row, and exact factorizations; plus a
1-D chain (a tridiagonal matrix: clusters with a single neighbour on each side)."""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

KINDS = {"spd": (0, 4, 0, 0), "sym": (1, 5, 1, 5), "gen": (2, 1, 2, 3)}  # pkg symm, pkg scaling, oracle symm, oracle scaling


def _pair(kind, A, X, nlevels, tol, skip=0):
    import spand_public_gb300 as pkg
    from oracle.oracle import OracleTree
    ps, pk, os_, ok = KINDS[kind]
    t = pkg.Tree(nlevels)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(X)
    t.set_tol(tol)
    t.set_skip(skip)
    t.set_symm_kind(ps)
    t.set_scaling_kind(pk)
    t.partition(A)
    t.assemble(A)
    t.factorize()
    o = OracleTree(nlevels)
    o.set_Xcoo(X)
    o.set_tol(tol)
    o.set_skip(skip)
    o.set_symm_kind(os_)
    o.set_scaling_kind(ok)
    o.partition(A)
    o.assemble(A)
    o.factorize()
    return t, o


def _matrix(kind, n, dim):
    from spand_public_gb300 import problems as P
    if kind == "spd":
        return P.neglapl(n, dim)
    if kind == "sym":
        return (-P.neglapl(n, dim)).tocsc()
    return P.neglapl_unsym(n, dim, seed=1)


@pytest.mark.parametrize("kind", sorted(KINDS))
@pytest.mark.parametrize("n", [1, 2, 3])
def test_tiny_systems(kind, n):
    A = sp.csc_matrix(np.diag(np.full(n, 2.0 if kind != "sym" else -2.0)) + (0.1 * np.eye(n, k=1) if kind == "gen" else 0))
    X = np.arange(n, dtype=float)[None, :]
    b = np.arange(1.0, n + 1)
    for nlevels in (1, 2):
        t, o = _pair(kind, A, X, nlevels, 1e-2)
        x = t.solve(b)
        assert np.allclose(x, o.solve(b), rtol=1e-13, atol=0)
        assert np.linalg.norm(A @ x - b) <= 1e-12 * np.linalg.norm(b)


@pytest.mark.parametrize("kind", sorted(KINDS))
@pytest.mark.parametrize("tol,skip", [(0.0, 0), (1e-2, 100), (10.0, 0), (1e-2, 1)])
def test_levels_skip_and_tolerance(kind, tol, skip):
    """skip >= levels: no scaling / sparsification at all (exact); tol >= 1: every
    sparsified cluster keeps no row; tol 0: exact."""
    from spand_public_gb300 import problems as P
    A = _matrix(kind, 12, 2)
    X = P.linspace_nd(12, 2)
    t, o = _pair(kind, A, X, 4, tol, skip)
    assert np.array_equal(t.ranks(), o.ranks())
    b = np.random.default_rng(0).standard_normal(A.shape[0])
    x = t.solve(b)
    assert np.linalg.norm(x - o.solve(b)) <= 1e-11 * np.linalg.norm(x)
    if tol == 0.0 or skip >= 4:
        assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)


@pytest.mark.parametrize("kind", sorted(KINDS))
def test_one_dimensional_chain(kind):
    n = 200
    A = sp.diags([-1.0, 2.0, -1.0], [-1, 0, 1], shape=(n, n), format="csc")
    if kind == "sym":
        A = (-A).tocsc()
    elif kind == "gen":
        A = (A + sp.diags([0.05], [1], shape=(n, n))).tocsc()
    X = np.arange(n, dtype=float)[None, :]
    t, o = _pair(kind, A, X, 5, 1e-3)
    assert np.array_equal(t.ranks(), o.ranks())
    b = np.random.default_rng(1).standard_normal(n)
    x = t.solve(b)
    assert np.linalg.norm(x - o.solve(b)) <= 1e-11 * np.linalg.norm(x)
