"""Empty dimensions through the public entry points, as the reference treats them
(RandBLAS/skge.hh:154-202, skve.hh:140-246, sksp.hh:132-539): with d = 0 or n = 0 nothing is
written; with m = 0 (an empty product) B becomes beta * B, for the plain dense path, the
tensor-core precision path, a SASO operator and sketch_vector."""
import pytest

pytestmark = pytest.mark.gpu


def _dense(rb):
    return rb.DenseSkOp(rb.DenseDist(64, 96, rb.ScalarDist.Gaussian), rb.RNGState(2))


def _saso(rb):
    return rb.SparseSkOp(rb.SparseDist(64, 96, 4), rb.RNGState(2))


def _run(rb, path, S, d, n, m, A, B, beta):
    from randblas_gb300 import lowp
    if path == "lowp":
        lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 1.0, S, 3,
                         5, A, max(n, 1), beta, B, max(n, 1))
    else:
        rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 1.0, S,
                          3, 5, A, max(n, 1), beta, B, max(n, 1))


@pytest.mark.parametrize("path", ["plain", "lowp", "saso"])
def test_empty_product_scales_by_beta(rb, path):
    import torch
    S = _saso(rb) if path == "saso" else _dense(rb)
    g = torch.Generator(device="cuda").manual_seed(1)
    d, n = 20, 12
    A = torch.randn(4, n, device="cuda", generator=g)  # never read: m = 0
    B0 = torch.randn(d, n, device="cuda", generator=g)
    for beta in (0.5, 0.0):
        B = B0.clone()
        _run(rb, path, S, d, n, 0, A, B, beta)
        torch.cuda.synchronize()
        assert torch.equal(B, B0 * beta), (path, beta)


@pytest.mark.parametrize("path", ["plain", "lowp", "saso"])
@pytest.mark.parametrize("dn", [(0, 12), (20, 0)])
def test_empty_output_writes_nothing(rb, path, dn):
    import torch
    S = _saso(rb) if path == "saso" else _dense(rb)
    d, n = dn
    g = torch.Generator(device="cuda").manual_seed(2)
    A = torch.randn(30, max(n, 1), device="cuda", generator=g)
    B = torch.full((8, 13), 7.0, device="cuda")  # a guard buffer: nothing may change
    _run(rb, path, S, d, n, 30, A, B, 0.5)
    torch.cuda.synchronize()
    assert bool((B == 7.0).all()), (path, dn)


def test_sketch_vector_empty(rb):
    import torch
    S = _dense(rb)
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(8, device="cuda", generator=g)
    y0 = torch.randn(20, device="cuda", generator=g)
    y = y0.clone()
    rb.sketch_vector(rb.Op.NoTrans, 20, 0, 1.0, S, 0, 0, x, 1, 0.25, y, 1)  # m = 0
    torch.cuda.synchronize()
    assert torch.equal(y, y0 * 0.25)
    y = y0.clone()
    rb.sketch_vector(rb.Op.NoTrans, 0, 8, 1.0, S, 0, 0, x, 1, 0.25, y, 1)  # d = 0
    torch.cuda.synchronize()
    assert torch.equal(y, y0)
