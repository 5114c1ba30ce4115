"""Differentiable sparse products: Y = A X as a torch.autograd.Function over
the C ABI, with hand-written adjoint kernels.

    forward   Y = A X                       sblas_batch_spmm_xy (A's plan)
    backward  dX = A^T G                    sblas_batch_spmm_xy (A^T's plan: rows
                                            without entries left out, values read
                                            through the transpose permutation)
              dval[p] = G[row(p)] . X[col(p)]  sblas_batch_sddmm (A's plan)

A^T's structure (row pointer, columns and the value permutation) is built
once on the device by sblas_csr_transpose when the operator is created; its
empty rows are compacted away (the plan lists the rows it writes, the others
of dX are zeroed).
The reference has no differentiable form; the forward is its SpMV
(test/dspmv_test_smt.cu:39-52 is the arithmetic) with k right-hand sides.
Values are FP64 or FP32 (dval then rounded to FP32); products and sums are
FP64.  There is no CPU path: CPU tensors raise.
"""
from __future__ import annotations

import torch

from . import ops, tune


class CsrOperator:
    """A CSR pattern (int32 rowptr, col) of an m x n matrix, prepared for
    differentiable products with k right-hand sides (k in 1, 2, 4, 8, 16).
    value_dtype: torch.float64, torch.float32, or None for a pattern-only
    matrix (every stored entry 1, nothing to differentiate but X).
    s: nonzeros per lane of the forward and transposed plans; None picks
    each by measurement (tune.spmm_s), 0 takes the library default."""

    def __init__(self, rowptr: torch.Tensor, col: torch.Tensor, n: int, k: int,
                 value_dtype: torch.dtype | None = torch.float64, s: int | None = 0):
        self.m = rowptr.numel() - 1
        self.n = int(n)
        self.k = int(k)
        self.nnz = col.numel()
        self.value_dtype = value_dtype
        dev = rowptr.device
        proto = None if value_dtype is None else torch.zeros(self.nnz, dtype=value_dtype,
                                                               device=dev)
        self.rowptr, self.col = rowptr, col
        self.t_rowptr, self.t_col, self.perm = ops.csr_transpose(self.m, self.n, rowptr, col)
        # A^T without its empty rows (columns of A that hold no entry): the
        # transposed plan writes only the listed rows of dX, the rest are
        # zeroed first (setup-time compaction of the row pointer)
        nonempty = (self.t_rowptr[1:] > self.t_rowptr[:-1]).nonzero().flatten()
        self.t_rows = nonempty.to(torch.int32)
        self.t_rowptr_c = torch.cat([self.t_rowptr[nonempty],
                                     self.t_rowptr[-1:]]).to(torch.int32).contiguous()
        # A^T's values are read through the permutation: val[perm[q]]
        vperm = None if proto is None else self.perm
        s_f = s_b = s
        if s is None:
            s_f, _ = tune.spmm_s(rowptr, col, proto, self.n, self.k)
            s_b, _ = tune.spmm_s(self.t_rowptr_c, self.t_col, proto, self.m, self.k,
                                 row_ids=self.t_rows, m_out=self.n, val_perm=vperm)
        self.fwd = ops.SpmmPlan(rowptr, col, proto, n=self.n, k=self.k, s=s_f)
        self.bwd = ops.SpmmPlan(self.t_rowptr_c, self.t_col, proto, n=self.m, k=self.k,
                                s=s_b, row_ids=self.t_rows, m_out=self.n, val_perm=vperm)

    def _shape(self, rows: int, like: torch.Tensor) -> tuple:
        return (rows,) if like.dim() == 1 else (rows, self.k)

    def forward(self, val: torch.Tensor | None, x: torch.Tensor) -> torch.Tensor:
        y = torch.empty(self._shape(self.m, x), dtype=torch.float64, device=x.device)
        return self.fwd(x.contiguous(), y, val=val)

    def grad_x(self, val: torch.Tensor | None, g: torch.Tensor) -> torch.Tensor:
        dx = ops.zero_(torch.empty(self._shape(self.n, g), dtype=torch.float64, device=g.device))
        return self.bwd(g.contiguous(), dx, val=val)

    def grad_val(self, g: torch.Tensor, x: torch.Tensor) -> torch.Tensor:
        dval = torch.empty(self.nnz, dtype=self.value_dtype, device=g.device)
        return self.fwd.sddmm(g.contiguous(), x.contiguous(), dval)


class SpmmFunction(torch.autograd.Function):
    """Y = A(val) X; gradients for val and X."""

    @staticmethod
    def forward(ctx, val, x, op: CsrOperator):
        ctx.op = op
        ctx.save_for_backward(val, x)
        return op.forward(val, x)

    @staticmethod
    def backward(ctx, gy):
        val, x = ctx.saved_tensors
        op = ctx.op
        dval = dx = None
        if ctx.needs_input_grad[1]:
            dx = op.grad_x(val, gy)
        if ctx.needs_input_grad[0] and val is not None:
            dval = op.grad_val(gy, x)
        return dval, dx, None


def spmm(op: CsrOperator, val: torch.Tensor | None, x: torch.Tensor) -> torch.Tensor:
    """Y = A X with A = (op's pattern, val); differentiable in val and x."""
    if val is not None and val.dtype != op.value_dtype:
        raise TypeError("val dtype differs from the operator's value dtype")
    if x.dtype != torch.float64:
        raise TypeError("x must be float64")
    return SpmmFunction.apply(val, x, op)


__all__ = ["CsrOperator", "SpmmFunction", "spmm"]
