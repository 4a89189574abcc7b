"""Many independent systems at once (batch_factorize / batch_cg): the same factors,
iterations and solutions as each system run alone, and the oracle's iteration counts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _systems(fp32, sides, seed=0):
    import spand_public_gb300 as pkg
    from spand_public_gb300 import problems as P
    rng = np.random.default_rng(seed)
    out = []
    for n in sides:
        A = P.reaction_diffusion3d(n, float(rng.uniform(0.0, 1.0)))
        X = P.linspace_nd(n, 3)
        levels = max(2, int(np.ceil(np.log2(n ** 3 / 64))))
        t = pkg.Tree(levels)
        t.set_verb(False)
        t.set_use_geo(True)
        t.set_Xcoo(X)
        t.set_tol(1e-2)
        t.set_fp32(fp32)
        t.partition(A)
        t.assemble(A)
        out.append((A, X, levels, t, P.rhs(n ** 3, 1, seed=int(rng.integers(1 << 30)))[:, 0].copy()))
    return out


@pytest.mark.parametrize("fp32", [False, True])
def test_batch_matches_one_at_a_time(fp32):
    import spand_public_gb300 as pkg
    from oracle.oracle import OracleTree
    sides = [8, 11, 14, 9, 12, 10]
    sysb = _systems(fp32, sides)
    st = pkg.batch_factorize([s[3] for s in sysb])
    assert not np.any(st)
    xs, its, rr = pkg.batch_cg([s[3] for s in sysb], [s[4] for s in sysb], iters=200, tol=1e-10)
    sys1 = _systems(fp32, sides)
    for k, (A, X, levels, t, b) in enumerate(sys1):
        t.factorize()
        x1, it1, r1 = t.cg(b, iters=200, tol=1e-10)
        assert its[k] == it1, (k, its[k], it1)
        assert np.linalg.norm(xs[k] - x1) <= 1e-12 * np.linalg.norm(x1)
        assert np.linalg.norm(A @ xs[k] - b) / np.linalg.norm(b) < 1e-9
        if not fp32:
            o = OracleTree(levels)
            o.set_Xcoo(X)
            o.set_tol(1e-2)
            o.partition(A)
            o.assemble(A)
            o.factorize()
            _, ito = o.cg(b, 200, 1e-10)
            assert its[k] == ito


def test_batch_reports_a_failing_system():
    """A non-SPD system is reported by status; the others are factored."""
    import spand_public_gb300 as pkg
    sysb = _systems(False, [8, 9, 10])
    A, X, levels, t, b = sysb[1]
    t.assemble(-A)
    st = pkg.batch_factorize([s[3] for s in sysb])
    assert st[0] == 0 and st[2] == 0 and st[1] == 4
    xs, its, _ = pkg.batch_cg([sysb[0][3], sysb[2][3]], [sysb[0][4], sysb[2][4]], iters=200, tol=1e-10)
    for (A2, _, _, _, b2), x in zip([sysb[0], sysb[2]], xs):
        assert np.linalg.norm(A2 @ x - b2) / np.linalg.norm(b2) < 1e-9


def test_batch_cg_device_matches_host():
    """batch_cg_device on torch device vectors: the iterations and solutions of batch_cg."""
    torch = pytest.importorskip("torch")
    import spand_public_gb300 as pkg
    sysb = _systems(True, [9, 13, 10, 16])
    trees = [s[3] for s in sysb]
    assert not np.any(pkg.batch_factorize(trees))
    xs, its, rr = pkg.batch_cg(trees, [s[4] for s in sysb], iters=200, tol=1e-10)
    bd = [torch.from_numpy(s[4]).cuda() for s in sysb]
    xd = [torch.zeros_like(b) for b in bd]  # x holds the initial guess
    torch.cuda.synchronize()
    itd, rrd = pkg.batch_cg_device(trees, [b.data_ptr() for b in bd], [x.data_ptr() for x in xd], 200, 1e-10)
    assert np.array_equal(its, itd)
    assert np.allclose(rr, rrd, rtol=1e-12, atol=0)
    for x, xh in zip(xd, xs):
        assert np.linalg.norm(x.cpu().numpy() - xh) <= 1e-13 * np.linalg.norm(xh)


@pytest.mark.parametrize("fp32", [False, True])
def test_forest_matches_one_at_a_time(fp32):
    """One plan for all systems (Forest): per-system ranks equal to each tree's, M^{-1}b
    within 1e-12 (FP64) of each tree's solve, CG iteration counts equal and solutions
    within 1e-10; systems of different depths (3..6 levels)."""
    import spand_public_gb300 as pkg
    sides = [8, 11, 14, 9, 12, 10, 16]
    sysb = _systems(fp32, sides)
    trees = [s[3] for s in sysb]
    f = pkg.Forest(trees)
    f.factorize()
    for t in trees:
        t.factorize()
    fr = f.ranks()
    for k, t in enumerate(trees):
        mine = fr[fr[:, 0] == k][:, 1:]
        assert np.array_equal(mine, t.ranks()), k
    rng = np.random.default_rng(4)
    bs = [rng.standard_normal(s[0].shape[0]) for s in sysb]
    xs, its, rr = f.cg(bs, iters=200, tol=1e-10)
    for k, (A, X, levels, t, _) in enumerate(sysb):
        x1, it1, _ = t.cg(bs[k], iters=200, tol=1e-10)
        assert its[k] == it1, (k, its[k], it1)
        assert np.linalg.norm(A @ xs[k] - bs[k]) / np.linalg.norm(bs[k]) < 1e-9
        assert np.linalg.norm(xs[k] - x1) <= 1e-10 * np.linalg.norm(x1)
    if not fp32:
        torch = pytest.importorskip("torch")
        xd = torch.from_numpy(f.stack(bs)).cuda()
        torch.cuda.synchronize()
        f.solve_device(xd.data_ptr())
        torch.cuda.synchronize()
        for k, (b, x) in enumerate(zip(bs, f.split(xd.cpu().numpy()))):
            ref = trees[k].solve(b)
            assert np.linalg.norm(x - ref) <= 1e-12 * np.linalg.norm(ref), k
    f.close()


def test_forest_device_vectors_and_new_values():
    """cg_device on stacked device vectors equals cg on host vectors; new stacked values
    (each system scaled by its own factor) give the scaled systems' solutions."""
    torch = pytest.importorskip("torch")
    import spand_public_gb300 as pkg
    sysb = _systems(True, [10, 13, 9])
    f = pkg.Forest([s[3] for s in sysb])
    f.factorize()
    rng = np.random.default_rng(8)
    bs = [rng.standard_normal(s[0].shape[0]) for s in sysb]
    xs, its, _ = f.cg(bs, iters=200, tol=1e-10)
    bd = torch.from_numpy(f.stack(bs)).cuda()
    xd = torch.zeros_like(bd)
    torch.cuda.synchronize()
    itd, _ = f.cg_device(bd.data_ptr(), xd.data_ptr(), iters=200, tol=1e-10)
    assert np.array_equal(its, itd)
    assert np.array_equal(np.concatenate(xs), xd.cpu().numpy())
    scale = [2.0, 0.5, 3.0]
    vals = np.concatenate([s[0].tocsc().data * c for s, c in zip(sysb, scale)])
    f.assemble_values(vals)
    f.factorize()
    xs2, _, _ = f.cg(bs, iters=200, tol=1e-10)
    for (A, *_), x, b, c in zip(sysb, xs2, bs, scale):
        assert np.linalg.norm(c * (A @ x) - b) / np.linalg.norm(b) < 1e-9
    f.close()


def test_forest_reports_the_failing_system():
    import spand_public_gb300 as pkg
    sysb = _systems(False, [8, 9, 10])
    A, X, levels, t, b = sysb[2]
    t.assemble(-A)
    f = pkg.Forest([s[3] for s in sysb])
    with pytest.raises(pkg.SpandError, match="Non-SPD Pivot"):
        f.factorize()
    assert f.failed_system == 2
    f.close()
