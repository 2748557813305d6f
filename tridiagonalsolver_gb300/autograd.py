"""torch.autograd wrapper of the pivoted solve and its adjoint kernel.

``x = solve_ad(a, b, c, d)`` solves the batch of tridiagonal systems
A x = d with partial pivoting: the partitioned solve (``tridiag_pge_*``)
where it applies (contiguous layout, 65 <= n <= its size limit), else the
thread-per-system sweep (``tridiag_gtsv_*``) keeping its pivot record.
``x.backward(xbar)`` solves A^T lambda = xbar -- with the partitioned solve
on the transposed coefficients (``tridiag_pge_adjoint_*``), or with the
sweep's factorisation and pivots (``tridiag_gtsv_adjoint_*``) -- and returns

    grad_d = lambda,  grad_a[i] = -lambda[i] x[i-1],  grad_b[i] = -lambda[i] x[i],
    grad_c[i] = -lambda[i] x[i+1]

(grad_a[0] = grad_c[n-1] = 0: those entries are outside the matrix).  Both
directions are the library's CUDA kernels; this module only owns the
bookkeeping between them.
"""
from __future__ import annotations

import torch

from . import ops
from ._lib import ERR_NOT_SUPPORTED as NOT_SUPPORTED
from ._lib import TridiagError


class TridiagonalSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a, b, c, d, n, layout, pivoting=True):
        a, b, c, d = (t.contiguous() for t in (a, b, c, d))
        if not pivoting and layout == "contiguous" and ops.partition_supported(a, n):
            # the unpivoted partition method forward and adjoint (systems that
            # need no pivoting, e.g. diagonally dominant)
            method = "partition"
        else:
            method = "pge" if layout == "contiguous" else "gtsv"
        x = None
        if method == "partition":
            x = ops.solve_out(a, b, c, d, n, algo="partition")
            ctx.save_for_backward(a, b, c, x)
        if method == "pge":
            # the partitioned solve: no pivot record, its adjoint is the same
            # solver on A^T
            try:
                x = ops.pge(a, b, c, d, n, layout=layout)
            except TridiagError as e:
                if e.status != NOT_SUPPORTED:
                    raise
                method = "gtsv"
        if method == "pge":
            ctx.save_for_backward(a, b, c, x)
        elif method == "gtsv":
            piv = ops.pivot_record(a, n, layout)
            work = ops.gtsv_workspace(a, n, layout)
            x = ops.gtsv(a, b, c, d, n, layout=layout, pivots=piv, work=work)
            ctx.save_for_backward(a, b, c, x, piv, work)
        ctx.n, ctx.layout, ctx.method = n, layout, method
        return x

    @staticmethod
    def backward(ctx, xbar):
        if ctx.method == "partition":
            a, b, c, x = ctx.saved_tensors
            ga, gb, gc, gd = ops.partition_adjoint(a, b, c, x, xbar.contiguous(), ctx.n)
        elif ctx.method == "pge":
            a, b, c, x = ctx.saved_tensors
            ga, gb, gc, gd = ops.pge_adjoint(a, b, c, x, xbar.contiguous(), ctx.n, layout=ctx.layout)
        else:
            a, b, c, x, piv, work = ctx.saved_tensors
            ga, gb, gc, gd = ops.gtsv_adjoint(a, b, c, x, piv, xbar.contiguous(), ctx.n, layout=ctx.layout,
                                              work=work)
        need = ctx.needs_input_grad
        return (ga if need[0] else None, gb if need[1] else None, gc if need[2] else None,
                gd if need[3] else None, None, None, None)


def solve_ad(a: torch.Tensor, b: torch.Tensor, c: torch.Tensor, d: torch.Tensor, n: int | None = None,
             layout: str = "contiguous", pivoting: bool = True) -> torch.Tensor:
    """Differentiable batched solve.  ``a, b, c, d`` share one shape: (batch, n)
    for layout "contiguous" or (n, batch) for "interleaved"; ``n`` defaults to
    the matching dimension.  ``pivoting=False`` selects the unpivoted
    partition method (forward and adjoint) where it covers the shape -- for
    systems that need no pivoting, such as diagonally dominant ones."""
    if layout not in ("contiguous", "interleaved"):
        raise ValueError("solve_ad supports the contiguous and interleaved layouts")
    if not (a.shape == b.shape == c.shape == d.shape):
        raise ValueError("a, b, c, d must have the same shape")
    if n is None:
        if a.dim() != 2:
            raise ValueError("pass n for flat tensors")
        n = a.shape[1] if layout == "contiguous" else a.shape[0]
    return TridiagonalSolve.apply(a, b, c, d, n, layout, pivoting)
