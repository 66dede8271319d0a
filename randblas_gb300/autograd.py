"""Differentiation path: sketch_general (RandBLAS/skge.hh:756-1199, dense operator) as a
``torch.autograd.Function``, differentiable in the data matrix A.

Forward and backward both run the library's own kernels, which generate the operator's
entries from its RNGState counter inside the GEMM; the backward pass regenerates op(submat(S))
instead of saving it:

* left:  Y = alpha * op(submat(S)) @ A   ->  dA = alpha * op(submat(S))^T @ dY
* right: Y = alpha * A @ op(submat(S))   ->  dA = alpha * dY @ op(submat(S))^T

The transposed operator is the same operator with ``opS`` flipped, so the backward call is an
ordinary sketch with the flipped op (RandBLAS/skge.hh:154-202 and 307-355 resolve opS the same
way).  ``precision=None`` runs the plain FP32 / FP64 path (the reference's arithmetic);
``precision="bf16"`` runs the tensor-core path with A (FP32 or BF16) and the operator rounded
to BF16 and FP32 accumulation, in both directions.  Matrices are row-major CUDA tensors.
"""
from __future__ import annotations

from typing import Optional

import torch

from . import lowp
from ._lib import ERROR_INVALID_ARGUMENT, RandBLASError
from .api import DenseSkOp, Layout, Op, sketch_general

_PRECISIONS = {None: None, "bf16": lowp.BF16}


def _flip(op: Op) -> Op:
    return Op.Trans if Op(op) == Op.NoTrans else Op.NoTrans


def _op_dims(S: DenseSkOp, opS: Op, ro_s: int, co_s: int, rows: Optional[int],
             cols: Optional[int]):
    """(rows, cols) of op(submat(S)); without offsets the whole operator is used."""
    if ro_s == 0 and co_s == 0 and rows is None and cols is None:
        r, c = S.n_rows, S.n_cols
        return (r, c) if Op(opS) == Op.NoTrans else (c, r)
    if rows is None or cols is None:
        raise RandBLASError(ERROR_INVALID_ARGUMENT,
                            "a submatrix of S needs its op(submat(S)) dimensions")
    return rows, cols


def _left(S, opS, d, n, m, alpha, ro_s, co_s, X, out, prec):
    """out (d x n) = alpha * op(submat(S)) (d x m) @ X (m x n), row-major."""
    if prec is None:
        sketch_general(Layout.RowMajor, opS, Op.NoTrans, d, n, m, alpha, S, ro_s, co_s, X, n,
                       0.0, out, n)
    else:
        lowp.sketch_lowp(Layout.RowMajor, opS, Op.NoTrans, d, n, m, alpha, S, ro_s, co_s, X, n,
                         0.0, out, n, precision=prec)


def _right(S, opS, r, d, m, alpha, ro_s, co_s, X, out, prec):
    """out (r x d) = alpha * X (r x m) @ op(submat(S)) (m x d), row-major."""
    if prec is None:
        sketch_general(Layout.RowMajor, Op.NoTrans, opS, r, d, m, alpha, X, m, S, ro_s, co_s,
                       0.0, out, d)
    else:
        # out^T (d x r) = op(submat(S))^T @ X^T: the same memory read column-major
        lowp.sketch_lowp(Layout.ColMajor, _flip(opS), Op.NoTrans, d, r, m, alpha, S, ro_s, co_s,
                         X, m, 0.0, out, d, precision=prec)


class SketchGeneral(torch.autograd.Function):
    """Y = alpha * op(submat(S)) @ A (side "left") or alpha * A @ op(submat(S)) (side "right")."""

    @staticmethod
    def forward(ctx, A, S, side, opS, alpha, ro_s, co_s, op_rows, op_cols, precision):
        prec = _PRECISIONS[precision]
        if prec is None and A.dtype not in (torch.float32, torch.float64):
            raise RandBLASError(ERROR_INVALID_ARGUMENT, "the plain path takes FP32 or FP64 A")
        if prec is not None and A.dtype not in (torch.float32, torch.bfloat16):
            raise RandBLASError(ERROR_INVALID_ARGUMENT, "the BF16 path takes FP32 or BF16 A")
        if A.dim() != 2:
            raise RandBLASError(ERROR_INVALID_ARGUMENT, "A must be a matrix")
        A = A.contiguous()
        out_dtype = A.dtype if prec is None else torch.float32
        pr, pc = _op_dims(S, opS, ro_s, co_s, op_rows, op_cols)
        if side == "left":
            m, n = A.shape
            if pc != m:
                raise RandBLASError(ERROR_INVALID_ARGUMENT,
                                    f"op(submat(S)) has {pc} columns, A has {m} rows")
            Y = torch.empty(pr, n, device=A.device, dtype=out_dtype)
            _left(S, opS, pr, n, m, alpha, ro_s, co_s, A, Y, prec)
        elif side == "right":
            r, m = A.shape
            if pr != m:
                raise RandBLASError(ERROR_INVALID_ARGUMENT,
                                    f"op(submat(S)) has {pr} rows, A has {m} columns")
            Y = torch.empty(r, pc, device=A.device, dtype=out_dtype)
            _right(S, opS, r, pc, m, alpha, ro_s, co_s, A, Y, prec)
        else:
            raise RandBLASError(ERROR_INVALID_ARGUMENT, "side must be 'left' or 'right'")
        ctx.S, ctx.side, ctx.opS, ctx.alpha = S, side, Op(opS), float(alpha)
        ctx.ro_s, ctx.co_s, ctx.pr, ctx.pc, ctx.prec = ro_s, co_s, pr, pc, prec
        ctx.a_shape, ctx.a_dtype = tuple(A.shape), A.dtype
        return Y

    @staticmethod
    def backward(ctx, dY):
        S, prec = ctx.S, ctx.prec
        gdtype = ctx.a_dtype if prec is None else torch.float32
        dY = dY.to(gdtype if prec is None else torch.float32).contiguous()
        dA = torch.empty(ctx.a_shape, device=dY.device, dtype=gdtype)
        flipped = _flip(ctx.opS)
        # op(submat(S))^T is submat(S) with the op flipped: (pc x pr)
        if ctx.side == "left":
            m, n = ctx.a_shape
            _left(S, flipped, m, n, ctx.pr, ctx.alpha, ctx.ro_s, ctx.co_s, dY, dA, prec)
        else:
            r, m = ctx.a_shape
            _right(S, flipped, r, m, ctx.pc, ctx.alpha, ctx.ro_s, ctx.co_s, dY, dA, prec)
        if dA.dtype != ctx.a_dtype:
            dA = dA.to(ctx.a_dtype)
        return dA, None, None, None, None, None, None, None, None, None


def sketch(S: DenseSkOp, A: torch.Tensor, *, side: str = "left", opS: Op = Op.NoTrans,
           alpha: float = 1.0, ro_s: int = 0, co_s: int = 0, op_rows: Optional[int] = None,
           op_cols: Optional[int] = None, precision: Optional[str] = None) -> torch.Tensor:
    """Differentiable sketch of A with the dense operator S (see the module docstring).
    With offsets (ro_s, co_s) give the dimensions (op_rows, op_cols) of op(submat(S))."""
    if precision not in _PRECISIONS:
        raise RandBLASError(ERROR_INVALID_ARGUMENT, "precision must be None or 'bf16'")
    if S.buff is not None:
        raise RandBLASError(ERROR_INVALID_ARGUMENT,
                            "the differentiation path regenerates S; pass an unfilled operator")
    return SketchGeneral.apply(A, S, side, Op(opS), float(alpha), int(ro_s), int(co_s), op_rows,
                               op_cols, precision)
