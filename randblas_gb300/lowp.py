"""Tensor-core precision path (rbg_lskge3_lowp): the left dense sketch with the operator's
entries generated in-kernel and rounded, together with A, to BF16 or FP8 e4m3 (A with one
power-of-two scale per column and K slice), FP32 accumulation on tcgen05 tensor cores.  No
reference counterpart; same argument meaning as sketch_general's left form with T = float."""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from ._lib import call
from .api import DenseSkOp, Layout, Op, _ptr, _ptr_device_or_pinned, _stream

BF16 = _lib.PREC_BF16
FP8_E4M3 = _lib.PREC_FP8_E4M3


def available(precision: int = BF16) -> bool:
    nbytes = C.c_size_t()
    rc = _lib.lib().rbg_lskge3_lowp_workspace(precision, 128, 128, 128, C.byref(nbytes))
    return rc == _lib.SUCCESS


def workspace_bytes(precision: int, d: int, n: int, m: int) -> int:
    nbytes = C.c_size_t()
    call("rbg_lskge3_lowp_workspace", precision, d, n, m, C.byref(nbytes))
    return nbytes.value


def sketch_lowp(layout: Layout, opS: Op, opA: Op, d: int, n: int, m: int, alpha: float,
                S: DenseSkOp, ro_s: int, co_s: int, A: torch.Tensor, lda: int, beta: float,
                B: torch.Tensor, ldb: int, precision: int = BF16,
                workspace: torch.Tensor | None = None) -> None:
    """B = alpha * op(submat(S)) * op(A) + beta * B on the tensor cores.  A is FP32 or BF16
    (BF16 data enters the tensor cores unchanged); B is FP32.  A and B may be CUDA tensors or
    pinned CPU tensors (A is then read over the host link by the conversion pass, B written in
    place).  A workspace, if given, is a CUDA tensor on the current device."""
    if workspace is not None and (not workspace.is_cuda or
                                  workspace.device.index != torch.cuda.current_device()):
        raise _lib.RandBLASError(_lib.ERROR_INVALID_ARGUMENT,
                                 "workspace must be device memory of the current GPU")
    ws = _ptr(workspace) if workspace is not None else None
    wbytes = workspace.numel() * workspace.element_size() if workspace is not None else 0
    a_dtype = {torch.float32: _lib.F32, torch.bfloat16: _lib.BF16}.get(A.dtype)
    if a_dtype is None:
        raise _lib.RandBLASError(_lib.ERROR_INVALID_ARGUMENT,
                                 "the precision path takes FP32 or BF16 A")
    call("rbg_lskge3_lowp_ex", precision, a_dtype, int(layout), int(opS), int(opA), d, n, m,
         float(alpha), C.byref(S._c()), ro_s, co_s, _ptr_device_or_pinned(A), lda,
         float(beta), _ptr_device_or_pinned(B), ldb, ws,
         wbytes, _stream())


def status() -> int:
    """Device-side status of the tensor-core kernels since the last call (0 = fine,
    4 = a bounded wait timed out); synchronises the device."""
    code = C.c_int32()
    call("rbg_lowp_status", C.byref(code))
    return code.value
