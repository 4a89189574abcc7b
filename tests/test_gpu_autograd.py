"""Differentiable solve (spand_public_gb300.autograd) on the 3D anisotropic diffusion
problem A(θ) (per-face conductivities scaling·θ, scaling (1, 1, 0.01)): the gradients of
loss = ½‖x(θ, b) − x*‖² with respect to θ and b against a dense FP64 solve and against
central finite differences."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCALING = (1.0, 1.0, 0.01)


def _problem(n, levels, fp32):
    torch = pytest.importorskip("torch")
    import spand_public_gb300 as pkg
    from spand_public_gb300 import problems as P
    from spand_public_gb300.autograd import Pattern

    th = P.anisotropic_theta(n, seed=1)
    A0 = P.anisotropic3d(n, th, SCALING)
    pat, pos, face, coef = P.face_diffusion_map(n, 3)
    assert np.array_equal(pat.indptr, A0.indptr) and np.array_equal(pat.indices, A0.indices)
    t = pkg.Tree(levels)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(P.linspace_nd(n, 3))
    t.set_tol(1e-2)
    t.set_fp32(fp32)
    t.partition(A0)
    t.assemble(A0)
    dev = torch.device("cuda")
    scale = torch.as_tensor(np.concatenate([np.full(np.asarray(x).size, s) for x, s in zip(th, SCALING)]),
                            device=dev)
    theta = torch.as_tensor(np.concatenate([np.asarray(x).reshape(-1) for x in th]), device=dev)
    pos_t = torch.as_tensor(pos, device=dev)
    face_t = torch.as_tensor(face, device=dev)
    coef_t = torch.as_tensor(coef, device=dev)

    def values(theta_):
        w = scale * theta_
        return torch.zeros(pat.nnz, dtype=torch.float64, device=dev).index_add(0, pos_t, coef_t * w[face_t])

    rng = np.random.default_rng(2)
    b = torch.as_tensor(rng.standard_normal(n ** 3), device=dev)
    xstar = torch.as_tensor(rng.standard_normal(n ** 3), device=dev)
    return torch, t, Pattern(A0), values, theta, b, xstar


@pytest.mark.parametrize("fp32", [False, True])
def test_gradient_against_dense_fp64(fp32):
    """16^3 instance: x, dL/dtheta and dL/db against torch's dense FP64 solve and its autograd."""
    torch, t, pat, values, theta0, b0, xstar = _problem(16, 6, fp32)
    from spand_public_gb300.autograd import solve

    theta = theta0.clone().requires_grad_(True)
    b = b0.clone().requires_grad_(True)
    x = solve(values(theta), b, t, pat)
    loss = 0.5 * torch.sum((x - xstar) ** 2)
    loss.backward()

    thd = theta0.clone().requires_grad_(True)
    bd = b0.clone().requires_grad_(True)
    v = values(thd)
    Ad = torch.sparse_coo_tensor(torch.stack([pat.rows, pat.cols]), v, (pat.n, pat.n)).to_dense()
    xd = torch.linalg.solve(Ad, bd)
    lossd = 0.5 * torch.sum((xd - xstar) ** 2)
    lossd.backward()

    assert torch.linalg.norm(x - xd) <= 1e-9 * torch.linalg.norm(xd)
    assert torch.linalg.norm(theta.grad - thd.grad) <= 1e-7 * torch.linalg.norm(thd.grad)
    assert torch.linalg.norm(b.grad - bd.grad) <= 1e-7 * torch.linalg.norm(bd.grad)


def test_adjoint_scatter_matches_pattern_outer_product():
    """spand_adjoint_device: lambda solves A lambda = g and grad_vals = -lambda[row] x[col]."""
    torch, t, pat, values, theta0, b0, xstar = _problem(12, 5, True)
    from spand_public_gb300.autograd import solve

    with torch.no_grad():
        v = values(theta0)
        x = solve(v, b0, t, pat)
        g = x - xstar
        lam = torch.zeros_like(g)
        grad = torch.full((pat.nnz,), float("nan"), dtype=torch.float64, device=g.device)
        torch.cuda.synchronize()
        it, rr = t.adjoint_device(g.data_ptr(), x.data_ptr(), lam.data_ptr(), grad.data_ptr(), 200, 1e-12)
        assert rr < 1e-12 and it > 0
        A = torch.sparse_coo_tensor(torch.stack([pat.rows, pat.cols]), v, (pat.n, pat.n))
        assert torch.linalg.norm(A @ lam - g) <= 1e-10 * torch.linalg.norm(g)
        assert torch.equal(grad, -(lam[pat.rows] * x[pat.cols]))


def test_gradient_against_finite_differences():
    """dL/dtheta on 64 random face conductivities against 4-point central differences
    (truncation O(h^4)) of the loss through the same solver, to 1e-6 relative."""
    torch, t, pat, values, theta0, b0, xstar = _problem(10, 5, False)
    from spand_public_gb300.autograd import solve

    tol = 1e-14
    theta = theta0.clone().requires_grad_(True)
    x = solve(values(theta), b0, t, pat, tol=tol)
    (0.5 * torch.sum((x - xstar) ** 2)).backward()

    def loss(th):
        with torch.no_grad():
            xx = solve(values(th), b0, t, pat, tol=tol)
            return float(0.5 * torch.sum((xx - xstar) ** 2))

    rng = np.random.default_rng(5)
    idx = rng.choice(theta0.numel(), size=64, replace=False)
    fd = np.zeros(64)
    for i, k in enumerate(idx):
        h = 1e-3 * float(theta0[k])
        f = {}
        for m in (-2, -1, 1, 2):
            tt = theta0.clone()
            tt[k] += m * h
            f[m] = loss(tt)
        fd[i] = (f[-2] - 8 * f[-1] + 8 * f[1] - f[2]) / (12 * h)
    g = theta.grad[torch.as_tensor(idx, device=theta.grad.device)].cpu().numpy()
    assert np.linalg.norm(fd - g) <= 1e-6 * np.linalg.norm(g), np.abs(fd - g).max()
    assert np.all(np.abs(fd - g) <= 1e-5 * np.maximum(np.abs(g), 1e-2 * np.abs(g).max()))


def test_gradient_fd_fp32_factor():
    """The differentiable-solve workload's own precision: an FP32 factor inside FP64 PCG
    (the adjoint reuses the same factor), on a 24^3 anisotropic instance, 8 levels.
    dL/dtheta on 64 random face conductivities against 4-point central differences of the
    loss through the same solver, to 1e-6 relative."""
    torch, t, pat, values, theta0, b0, xstar = _problem(24, 8, True)
    from spand_public_gb300.autograd import solve

    tol = 1e-13
    theta = theta0.clone().requires_grad_(True)
    x = solve(values(theta), b0, t, pat, tol=tol)
    (0.5 * torch.sum((x - xstar) ** 2)).backward()

    def loss(th):
        with torch.no_grad():
            xx = solve(values(th), b0, t, pat, tol=tol)
            return float(0.5 * torch.sum((xx - xstar) ** 2))

    rng = np.random.default_rng(6)
    idx = rng.choice(theta0.numel(), size=64, replace=False)
    fd = np.zeros(64)
    for i, k in enumerate(idx):
        h = 1e-3 * float(theta0[k])
        f = {}
        for m in (-2, -1, 1, 2):
            tt = theta0.clone()
            tt[k] += m * h
            f[m] = loss(tt)
        fd[i] = (f[-2] - 8 * f[-1] + 8 * f[1] - f[2]) / (12 * h)
    g = theta.grad[torch.as_tensor(idx, device=theta.grad.device)].cpu().numpy()
    assert np.linalg.norm(fd - g) <= 1e-6 * np.linalg.norm(g), np.abs(fd - g).max()
