"""Host-side argument handling of the differentiation path (no GPU needed: every case is
rejected before a kernel would launch)."""
import pytest


def test_rejects_bad_arguments(rb_host):
    rb = rb_host
    import torch
    from randblas_gb300 import autograd
    S = rb.DenseSkOp(rb.DenseDist(8, 40), rb.RNGState(1))
    A = torch.zeros(40, 3)
    with pytest.raises(rb.RandBLASError, match="precision"):
        autograd.sketch(S, A, precision="fp16")
    with pytest.raises(rb.RandBLASError, match="side"):
        autograd.sketch(S, A, side="middle")
    with pytest.raises(rb.RandBLASError, match="columns"):
        autograd.sketch(S, torch.zeros(39, 3))
    with pytest.raises(rb.RandBLASError, match="rows"):
        autograd.sketch(S, torch.zeros(3, 9), side="right")
    with pytest.raises(rb.RandBLASError, match="submatrix"):
        autograd.sketch(S, A, ro_s=1)
    with pytest.raises(rb.RandBLASError, match="plain path"):
        autograd.sketch(S, A.to(torch.bfloat16))
    S.buff = torch.zeros(8 * 40)
    with pytest.raises(rb.RandBLASError, match="unfilled"):
        autograd.sketch(S, A)


def test_op_dims(rb_host):
    rb = rb_host
    from randblas_gb300 import autograd
    S = rb.DenseSkOp(rb.DenseDist(8, 40), rb.RNGState(1))
    assert autograd._op_dims(S, rb.Op.NoTrans, 0, 0, None, None) == (8, 40)
    assert autograd._op_dims(S, rb.Op.Trans, 0, 0, None, None) == (40, 8)
    assert autograd._op_dims(S, rb.Op.Trans, 2, 3, 5, 6) == (5, 6)
