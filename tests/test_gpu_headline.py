"""Parity at the benchmark's own configurations, device against the CPU oracle.

* 3D 7-point -Laplacian on 64^3 (n = 262,144), 12 nested-dissection levels, eps = 1e-2
  (the timed workload) and eps = 1e-3: ordering and permutation identical, per-cluster
  ranks identical, op list identical, every recorded factor block (ScalingLLT lower
  triangles, Gemm panels, reflectors and tau) within 1e-12 relative, per-level log
  identical, M^{-1}b within 1e-12 relative, and the CG iteration count to 1e-10 equal to
  the oracle's on the same right-hand side -- the plain FP64 path.  The FP32 factor then
  reaches the same 1e-10 true residual with at most 15% more iterations.
* Many-systems sample: -Laplacian + cI on grids with sides 16, 28 and 40 (the extremes
  and middle of the batch workload's U{16..40}), levels ceil(log2(n/64)), eps = 1e-2:
  ranks and CG iterations equal to the oracle's per system, and the forest (all systems
  in one plan) equal to the systems factored one at a time.
* High-contrast finite-volume diffusion reduced to 256^2 (coefficients 10^U(-3,3) on 8x8
  tiles), 12 levels, eps = 1e-3: ranks, op list, log and CG iterations identical; blocks
  and M^{-1}b within max(1e-12, 100 x the oracle's own one-ulp sensitivity).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_BLOCK = 1e-12
TOL_SOLVE = 1e-12


def _pair(A, X, nlevels, tol, fp32=False):
    import spand_public_gb300 as pkg
    from oracle.oracle import OracleTree

    t = pkg.Tree(nlevels)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(X)
    t.set_tol(tol)
    t.set_fp32(fp32)
    pt = t.partition(A)
    t.assemble(A)
    t.factorize()
    t.factorize()  # the timed configuration: launches tuned from the first factorization
    if fp32:
        return t, None
    o = OracleTree(nlevels)
    o.set_Xcoo(X)
    o.set_tol(tol)
    po = o.partition(A)
    o.assemble(A)
    o.factorize()
    assert np.array_equal(pt, po)
    return t, o


def _blocks(tree, ops, k):
    kind, rows, cols = ops[k, 0], ops[k, 6], ops[k, 7]
    m = tree.op_matrix(k, rows, cols)
    if kind == 0:
        return [np.tril(m)]
    if kind == 3:
        return [np.tril(m, -1), tree.op_tau(k, cols)]
    return [m]


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _blocks_worst(t, o, o2=None):
    """Largest relative error of a device factor block against the oracle's; with o2 (the
    oracle on the matrix moved by one unit in the last place) every block must instead stay
    within max(1e-12, 100 x the oracle's own change), and the error scaled to that bar (as
    if the bar were 1e-12) is returned."""
    opt, opo = t.ops(), o.ops()
    assert opt.shape == opo.shape
    assert np.array_equal(opt[:, :8], opo[:, :8])
    worst, tight = 0.0, 0
    for k in range(opt.shape[0]):
        kind, rows, cols = opt[k, 0], opt[k, 6], opt[k, 7]
        if kind not in (0, 1, 2, 3) or rows * cols == 0:
            continue
        if o2 is None:
            for a, b in zip(_blocks(t, opt, k), _blocks(o, opo, k)):
                worst = max(worst, _rel(a, b))
        else:
            for a, b, c in zip(_blocks(t, opt, k), _blocks(o, opo, k), _blocks(o2, opo, k)):
                bar = max(TOL_BLOCK, 100.0 * _rel(c, b))
                worst = max(worst, _rel(a, b) / bar * TOL_BLOCK)
                tight += bar == TOL_BLOCK
    if o2 is not None:
        assert tight > 0
    return worst


def _ulp_moved(A, seed=1):
    """A with every stored value moved by one unit in the last place (symmetrically)."""
    import scipy.sparse as sp

    rng = np.random.default_rng(seed)
    L = sp.tril(A, -1).tocoo()
    d = A.diagonal()
    ld = L.data + np.spacing(np.abs(L.data)) * rng.choice([-1.0, 1.0], L.data.shape)
    dd = d + np.spacing(np.abs(d)) * rng.choice([-1.0, 1.0], d.shape)
    L2 = sp.coo_matrix((ld, (L.row, L.col)), shape=A.shape)
    return (L2 + L2.T + sp.diags(dd)).tocsc()


def _full_parity(A, t, o, cg_tol, seed=0, o2=None):
    from spand_public_gb300 import problems as P

    assert np.array_equal(t.get_assembly_perm(), o.get_assembly_perm())
    assert np.array_equal(t.ranks(), o.ranks()), "per-cluster ranks differ"
    worst = _blocks_worst(t, o, o2)
    assert worst < TOL_BLOCK, worst
    for a, b in zip(t.level_log(), o.level_log()):
        for key in ("dofs_nd", "dofs_left_nd", "dofs_left_elim", "dofs_left_spars", "rank_before_sum",
                    "rank_after_sum", "rank_after_count", "ignored", "nbrs_sum", "fact_nnz"):
            assert a[key] == b[key], (key, a[key], b[key])
    b = P.rhs(A.shape[0], 2, seed=3)
    xt, xo = t.solve(b), o.solve(b)
    bar = TOL_SOLVE if o2 is None else max(TOL_SOLVE, 100.0 * _rel(o2.solve(b), xo))
    assert _rel(xt, xo) < bar
    b1 = P.rhs(A.shape[0], 1, seed=seed)[:, 0]
    xs, it, _ = t.cg(b1, iters=200, tol=cg_tol)
    _, ito = o.cg(b1, iters=200, tol=cg_tol)
    assert it == ito, (it, ito)
    assert np.linalg.norm(A @ xs - b1) / np.linalg.norm(b1) < 10 * cg_tol
    return it


@pytest.mark.parametrize("eps", [1e-2, 1e-3])
def test_headline_64cubed(eps):
    from spand_public_gb300 import problems as P

    n = 64
    A, X = P.neglapl(n, 3), P.linspace_nd(n, 3)
    t, o = _pair(A, X, 12, eps)
    it64 = _full_parity(A, t, o, 1e-10, seed=0)
    del o
    t32, _ = _pair(A, X, 12, eps, fp32=True)
    b = P.rhs(A.shape[0], 1, seed=0)[:, 0]
    x32, it32, _ = t32.cg(b, iters=200, tol=1e-10)
    assert np.linalg.norm(A @ x32 - b) / np.linalg.norm(b) < 1e-9
    assert it32 <= max(it64 + 1, int(np.ceil(1.15 * it64))), (it32, it64)


def test_many_systems_sample_to_side_40():
    import spand_public_gb300 as pkg
    from spand_public_gb300 import problems as P

    rng = np.random.default_rng(4)
    trees, rhs, iters_one = [], [], []
    for n in (16, 28, 40):
        A = P.reaction_diffusion3d(n, float(rng.uniform(0.0, 1.0)))
        X = P.linspace_nd(n, 3)
        levels = max(2, int(np.ceil(np.log2(n ** 3 / 64))))
        t, o = _pair(A, X, levels, 1e-2)
        assert np.array_equal(t.ranks(), o.ranks())
        b = P.rhs(n ** 3, 1, seed=int(rng.integers(1 << 30)))[:, 0]
        _, it, _ = t.cg(b, iters=200, tol=1e-10)
        _, ito = o.cg(b, 200, 1e-10)
        assert it == ito, (n, it, ito)
        trees.append(t)
        rhs.append(b)
        iters_one.append(it)
    f = pkg.Forest(trees)
    f.factorize()
    xs, its, _ = f.cg(rhs, iters=200, tol=1e-10)
    assert list(its) == iters_one


def test_high_contrast_fv_256():
    """Coefficients spanning six orders of magnitude make some factor blocks sensitive to
    rounding beyond 1e-12 in the reference's own algorithm: the bar per block is
    max(1e-12, 100 x the oracle's change when every value of A moves by one unit in the
    last place) -- 1e-12 for the well-conditioned blocks, which are most of them."""
    from oracle.oracle import OracleTree
    from spand_public_gb300 import problems as P

    n = 256
    A, X = P.high_contrast_fv2d(n, 8, seed=0), P.linspace_nd(n, 2)
    t, o = _pair(A, X, 12, 1e-3)
    o2 = OracleTree(12)
    o2.set_Xcoo(X)
    o2.set_tol(1e-3)
    o2.partition(A)
    o2.assemble(_ulp_moved(A))
    o2.factorize()
    assert np.array_equal(o2.ranks(), o.ranks())
    _full_parity(A, t, o, 1e-10, seed=1, o2=o2)
