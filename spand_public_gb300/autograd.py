"""Differentiable sparse solve x = A(values)^{-1} b for torch autograd, with the spaND
factorization as the preconditioner of a device CG.

The reference has no counterpart: its solve (`Tree::solve` inside `cg`, src/is.cpp:39-121)
is not differentiated.  A is SPD, so the adjoint of x = A^{-1} b is the system A λ = g
with the same operator and preconditioner, and

    dL/db          = λ
    dL/dvalues[k]  = -λ[row_k] · x[col_k]     for every stored entry k of A

(the −λxᵀ outer product restricted to the sparsity pattern).  Both come from one call,
`Tree.adjoint_device` (C ABI `spand_adjoint_device`): the PCG for λ and the pattern
scatter kernel.  Gradients with respect to
parameters that A's values depend on (face conductivities, shifts) follow from torch
autograd through the code that forms the values.

    tree = Tree(levels); tree.set_use_geo(True); tree.set_Xcoo(X); tree.set_tol(eps)
    tree.partition(A0); tree.assemble(A0)          # fixes the pattern (CSC) and the plan
    pat = Pattern(A0)
    x = solve(values, b, tree, pat)                # values: (nnz,) in A0's CSC order
"""
from __future__ import annotations

import numpy as np
import torch

__all__ = ["Pattern", "SpandSolve", "solve"]


class Pattern:
    """Row and column of every stored entry of a CSC matrix, as CUDA index tensors."""

    def __init__(self, A, device="cuda"):
        A = A.tocsc()
        n = A.shape[0]
        cols = np.repeat(np.arange(n, dtype=np.int64), np.diff(A.indptr))
        self.rows = torch.as_tensor(A.indices.astype(np.int64), device=device)
        self.cols = torch.as_tensor(cols, device=device)
        self.nnz = int(A.nnz)
        self.n = int(n)


def _refactor(tree, vals: torch.Tensor):
    """Assemble `vals` (device, float64, CSC order) on the tree's pattern and factorize."""
    torch.cuda.synchronize()
    tree.assemble_values((vals.data_ptr(), vals.numel()), on_device=True)
    tree.factorize()
    tree._autograd_values = vals


def _pcg(tree, rhs: torch.Tensor, iters: int, tol: float) -> torch.Tensor:
    out = torch.zeros_like(rhs)
    torch.cuda.synchronize()  # the tree runs on its own stream
    it, rr = tree.cg_device(rhs.data_ptr(), out.data_ptr(), iters, tol)
    if not rr < tol:
        raise RuntimeError(f"CG did not converge: |r|/|b| = {rr:.3e} after {it} iterations")
    return out


class SpandSolve(torch.autograd.Function):
    """x = A(values)^{-1} b; values on the pattern the tree was assembled with."""

    @staticmethod
    def forward(ctx, values, b, tree, pattern, iters, tol):
        if values.numel() != pattern.nnz or b.numel() != pattern.n:
            raise ValueError("values / right-hand side do not match the pattern")
        vals = values.detach().to(device="cuda", dtype=torch.float64).contiguous()
        _refactor(tree, vals)
        bb = b.detach().to(device="cuda", dtype=torch.float64).contiguous()
        x = _pcg(tree, bb, iters, tol)
        ctx.tree, ctx.pattern, ctx.iters, ctx.tol = tree, pattern, iters, tol
        ctx.vdev, ctx.bdev = values.device, b.device
        ctx.save_for_backward(vals, x)
        return x.to(device=b.device, dtype=b.dtype)

    @staticmethod
    def backward(ctx, g):
        vals, x = ctx.saved_tensors
        tree, pat = ctx.tree, ctx.pattern
        if getattr(tree, "_autograd_values", None) is not vals:
            _refactor(tree, vals)  # the tree was re-assembled since this forward
        gg = g.detach().to(device="cuda", dtype=torch.float64).contiguous()
        lam = torch.zeros_like(gg)
        grad_vals = torch.empty(pat.nnz, dtype=torch.float64, device=gg.device)
        torch.cuda.synchronize()  # the tree runs on its own stream
        it, rr = tree.adjoint_device(gg.data_ptr(), x.data_ptr(), lam.data_ptr(), grad_vals.data_ptr(), ctx.iters,
                                     ctx.tol)
        if not rr < ctx.tol:
            raise RuntimeError(f"adjoint CG did not converge: |r|/|g| = {rr:.3e} after {it} iterations")
        return grad_vals.to(ctx.vdev), lam.to(ctx.bdev), None, None, None, None


def solve(values: torch.Tensor, b: torch.Tensor, tree, pattern: Pattern, iters: int = 500,
          tol: float = 1e-12) -> torch.Tensor:
    """x = A(values)^{-1} b by CG with the spaND preconditioner, differentiable in values and b."""
    return SpandSolve.apply(values, b, tree, pattern, iters, tol)
