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
