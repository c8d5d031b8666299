"""Differentiable sparse triangular solve: x = L^{-1} b as a torch.autograd.Function.

Forward runs the row-driven sync-free solve.  Backward is hand-written: the
same row kernels over the solver's transposed copy of the structure (built
once, its entries pointing back into the CSR values) solve L^T y = g
(grad_b = y), then one pass writes grad_val[k] = -sum_r y[row_k, r] *
x[col_k, r] for every stored entry k, each sum over the right-hand sides an
FMA chain in one thread.  A solver set to "syncfree_csc" runs the backward
column-driven on the CSR arrays instead, with grad_val fused into the sweep.
"""
from __future__ import annotations

import torch

from .solver import TriangularSolver

__all__ = ["SparseTriangularSolve", "sptrsv", "DifferentiableTriangular"]


class SparseTriangularSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, val: torch.Tensor, b: torch.Tensor, solver: TriangularSolver):
        # values may have changed in place (optimiser steps, .data writes):
        # re-point and recompute 1/diag on the stream, no synchronisation
        solver.refresh_values(val.detach())
        x = solver.solve(b.detach())
        ctx.solver = solver
        ctx.save_for_backward(val, x)
        return x

    @staticmethod
    def backward(ctx, gx: torch.Tensor):
        val, x = ctx.saved_tensors
        solver: TriangularSolver = ctx.solver
        # the forward's values, unless another forward re-bound the solver
        # since (autograd rejects a saved tensor modified in place, so the
        # same tensor at the same version holds the same values)
        solver.refresh_values_if_rebound(val.detach())
        gx = gx.contiguous()
        need_val, need_b = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        if need_val:
            y, gval = solver.solve_transpose_grad(gx, x)
        else:
            y, gval = solver.solve_transpose(gx), None
        return gval, (y if need_b else None), None


def sptrsv(solver: TriangularSolver, val: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """x = L(val)^{-1} b, differentiable in val and b."""
    return SparseTriangularSolve.apply(val, b, solver)


class DifferentiableTriangular(torch.nn.Module):
    """A lower-triangular CSR operator with learnable values (a torch.nn.Parameter)."""

    def __init__(self, rowptr: torch.Tensor, colidx: torch.Tensor, val: torch.Tensor, **solver_kwargs):
        super().__init__()
        self.val = torch.nn.Parameter(val.detach().clone())
        self.solver = TriangularSolver(rowptr, colidx, self.val.detach(), **solver_kwargs)

    def forward(self, b: torch.Tensor) -> torch.Tensor:
        return sptrsv(self.solver, self.val, b)
