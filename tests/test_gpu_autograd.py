"""The differentiation path (randblas_gb300.autograd): sketch_general as an autograd Function
whose backward regenerates the operator from its RNGState.

1. torch.autograd.gradcheck in FP64 (central finite differences, step 1e-6) on small left and
   right sketches, with and without submatrix offsets and transposed operators.
2. The loss ||S A - B||_F^2 in FP64: finite differences with step 1e-6 on 32 seeded entries of
   A and along 4 seeded random directions, against the autograd gradient.
3. Gaussian d=2048 x m=2^18, A 2^18 x 512 (FP32): the autograd gradient equals the explicit
   dense-S gradient 2 S^T (S A - B), S materialised with fill_dense, to FP32 accuracy.
4. The same problem on the BF16 tensor-core path (A in FP32 and in BF16): forward and gradient
   within 1e-2 relative Frobenius error of the FP64 values.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _skop(rb, d, m, seed, family=0):
    return rb.DenseSkOp(rb.DenseDist(d, m, rb.ScalarDist(family)), rb.RNGState(seed),
                        dtype=__import__("torch").float64)


@pytest.mark.parametrize("side,opS,offs", [("left", 0, None), ("left", 1, None),
                                           ("right", 0, None), ("right", 1, None),
                                           ("left", 0, (3, 5)), ("right", 1, (2, 7))])
def test_gradcheck_fp64(rb, side, opS, offs):
    import torch
    from randblas_gb300 import autograd
    torch.manual_seed(1)
    d, m, n = 12, 150, 4
    if offs is None:
        rows, cols = (d, m) if opS == 0 else (m, d)
        S = _skop(rb, rows, cols, 11)
        kw = {}
    else:
        ro, co = offs
        rows, cols = (d, m) if opS == 0 else (m, d)
        S = _skop(rb, rows + ro + 4, cols + co + 2, 11)
        kw = dict(ro_s=ro, co_s=co, op_rows=d, op_cols=m)
    if side == "left":
        A = torch.randn(m, n, device="cuda", dtype=torch.float64, requires_grad=True)
        f = lambda X: autograd.sketch(S, X, side="left", opS=rb.Op(opS), alpha=0.5, **kw)
    else:
        # right: A (n x d') @ op(submat(S)) with op(submat(S)) of shape (d x m) here
        A = torch.randn(n, d, device="cuda", dtype=torch.float64, requires_grad=True)
        f = lambda X: autograd.sketch(S, X, side="right", opS=rb.Op(opS), alpha=0.5, **kw)
    assert torch.autograd.gradcheck(f, (A,), eps=1e-6, atol=1e-6, rtol=1e-5)


def test_loss_finite_differences_fp64(rb):
    import torch
    from randblas_gb300 import autograd
    d, m, n = 256, 1 << 14, 64
    S = _skop(rb, d, m, 5)
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn(m, n, device="cuda", dtype=torch.float64, generator=g) / np.sqrt(m)
    B = torch.randn(d, n, device="cuda", dtype=torch.float64, generator=g)
    A.requires_grad_(True)

    def loss(X):
        return ((autograd.sketch(S, X) - B) ** 2).sum()

    L = loss(A)
    L.backward()
    G = A.grad.detach()
    h = 1e-6
    scale = float(G.abs().max())
    rng = np.random.default_rng(5)
    with torch.no_grad():
        for _ in range(32):
            i, j = int(rng.integers(m)), int(rng.integers(n))
            E = torch.zeros_like(A)
            E[i, j] = 1.0
            fd = (float(loss(A + h * E)) - float(loss(A - h * E))) / (2 * h)
            assert abs(fd - float(G[i, j])) <= 1e-5 * scale + 1e-6 * abs(fd), (i, j, fd,
                                                                               float(G[i, j]))
        for _ in range(4):
            V = torch.randn(m, n, device="cuda", dtype=torch.float64, generator=g)
            V /= V.norm()
            fd = (float(loss(A + h * V)) - float(loss(A - h * V))) / (2 * h)
            an = float((G * V).sum())
            assert abs(fd - an) <= 1e-5 * float(G.norm()), (fd, an)


def _dense_s(rb, d, m, seed, dtype):
    import torch
    D = rb.DenseDist(d, m, rb.ScalarDist.Gaussian)
    buf = torch.empty(d * m, device="cuda", dtype=dtype)
    rb.fill_dense(D, buf, rb.RNGState(seed))
    assert D.natural_layout == rb.Layout.RowMajor
    return buf.view(d, m)


def test_dense_s_gradient_fp32_full_size(rb):
    import torch
    from randblas_gb300 import autograd
    d, m, n = 2048, 1 << 18, 512
    S = rb.DenseSkOp(rb.DenseDist(d, m, rb.ScalarDist.Gaussian), rb.RNGState(5))
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn(m, n, device="cuda", generator=g)
    B = torch.randn(d, n, device="cuda", generator=g)
    A.requires_grad_(True)
    L = ((autograd.sketch(S, A) - B) ** 2).sum()
    L.backward()
    G = A.grad.detach().double()
    Sd = _dense_s(rb, d, m, 5, torch.float32).double()
    with torch.no_grad():
        R = Sd @ A.detach().double() - B.double()
        Gref = 2.0 * (Sd.T @ R)
    rel = float((G - Gref).norm() / Gref.norm())
    assert rel < 1e-5, rel


@pytest.mark.parametrize("adtype", ["float32", "bfloat16"])
def test_bf16_path_full_size(rb, adtype):
    import torch
    from randblas_gb300 import autograd
    d, m, n = 2048, 1 << 18, 512
    S = rb.DenseSkOp(rb.DenseDist(d, m, rb.ScalarDist.Gaussian), rb.RNGState(5))
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn(m, n, device="cuda", generator=g).to(getattr(torch, adtype))
    B = torch.randn(d, n, device="cuda", generator=g)
    A.requires_grad_(True)
    Y = autograd.sketch(S, A, precision="bf16")
    L = ((Y - B) ** 2).sum()
    L.backward()
    assert A.grad.dtype == A.dtype
    Sd = _dense_s(rb, d, m, 5, torch.float32).double()
    with torch.no_grad():
        Yref = Sd @ A.detach().double()
        Gref = 2.0 * (Sd.T @ (Yref - B.double()))
    ry = float((Y.detach().double() - Yref).norm() / Yref.norm())
    rg = float((A.grad.double() - Gref).norm() / Gref.norm())
    assert ry < 1e-2 and rg < 1e-2, (ry, rg)


def test_bf16_step_replays_from_cuda_graph(rb):
    """Forward + backward on the tensor-core path captured once in a CUDA graph: replays give
    the eager gradient bit for bit (the kernels launch stream-ordered work only, and every sum
    has a fixed order), including after the data changes in place."""
    import torch
    from randblas_gb300 import autograd
    d, m, n = 256, 8192, 96
    S = rb.DenseSkOp(rb.DenseDist(d, m, rb.ScalarDist.Gaussian), rb.RNGState(8))
    g = torch.Generator(device="cuda").manual_seed(8)
    A = torch.randn(m, n, device="cuda", generator=g).requires_grad_(True)
    B = torch.randn(d, n, device="cuda", generator=g)

    def step():
        ((autograd.sketch(S, A, precision="bf16") - B) ** 2).sum().backward()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(2):
            A.grad = None
            step()
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    A.grad = None
    with torch.cuda.graph(graph, capture_error_mode="relaxed"):
        step()
    static_grad = A.grad
    for _ in range(2):
        graph.replay()
        with torch.no_grad():
            A.mul_(1.5)  # new data in the captured input
        graph.replay()
        torch.cuda.synchronize()
        replayed = static_grad.clone()
        A.grad = None
        step()
        assert torch.equal(replayed, A.grad)
