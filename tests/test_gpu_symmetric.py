"""sketch_symmetric (RandBLAS/sksy.hh:158-529) and require_symmetric (RandBLAS/util.hh:128-146).

1. For a symmetric A, every overload (left / right, submatrix / whole operator, dense / sparse
   operator, FP32 / FP64, both layouts) gives exactly what sketch_general gives on the same data,
   and a case matches the oracle.
2. A non-symmetric A raises with the reference's message naming the first failing pair in the
   reference's loop order; a negative tolerance skips the check; a violation inside the
   tolerance passes."""
import numpy as np
import pytest

from gpu_helpers import to_host

pytestmark = pytest.mark.gpu


def _sym(n, dtype, seed):
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    X = torch.randn(n, n, device="cuda", dtype=dtype, generator=g)
    return (X + X.T).contiguous()


@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("layout", [0, 1])
@pytest.mark.parametrize("sparse", [False, True])
def test_symmetric_matches_general(rb, dtype, layout, sparse):
    import torch
    rb.set_deterministic(True)  # bitwise comparisons across calls (the fused SASO path is not)
    try:
        _matches_general(rb, dtype, layout, sparse)
    finally:
        rb.set_deterministic(False)


def _matches_general(rb, dtype, layout, sparse):
    import torch
    dt = getattr(torch, dtype)
    n, d = 300, 40
    A = _sym(n, dt, 1)  # symmetric: the same memory in either layout
    lay = rb.Layout(layout)
    row = lay == rb.Layout.RowMajor
    if sparse:
        S_left = rb.SparseSkOp(rb.SparseDist(d + 3, n + 5, 4), rb.RNGState(3), dtype=dt)
        S_right = rb.SparseSkOp(rb.SparseDist(n + 5, d + 3, 4), rb.RNGState(4), dtype=dt)
    else:
        S_left = rb.DenseSkOp(rb.DenseDist(d + 3, n + 5), rb.RNGState(3), dtype=dt)
        S_right = rb.DenseSkOp(rb.DenseDist(n + 5, d + 3), rb.RNGState(4), dtype=dt)
    # left, submatrix at (2, 5): B = 0.5 * submat(S) * A + 0 * B, d x n
    B1 = torch.empty(d, n, device="cuda", dtype=dt)
    B2 = torch.empty(d, n, device="cuda", dtype=dt)
    ldb = n if row else d
    rb.sketch_symmetric(lay, d, n, 0.5, S_left, 2, 5, A, n, 0.0, B1, ldb)
    rb.sketch_general(lay, rb.Op.NoTrans, rb.Op.NoTrans, d, n, n, 0.5, S_left, 2, 5, A, n, 0.0,
                      B2, ldb)
    assert torch.equal(B1, B2)
    # right, submatrix at (5, 2): B = A * submat(S), n x d
    C1 = torch.empty(n, d, device="cuda", dtype=dt)
    C2 = torch.empty(n, d, device="cuda", dtype=dt)
    ldc = d if row else n
    rb.sketch_symmetric(lay, n, d, 1.0, A, n, S_right, 5, 2, 0.0, C1, ldc)
    rb.sketch_general(lay, rb.Op.NoTrans, rb.Op.NoTrans, n, d, n, 1.0, A, n, S_right, 5, 2, 0.0,
                      C2, ldc)
    assert torch.equal(C1, C2)


def test_symmetric_whole_operator_vs_oracle(rb, oracle):
    import torch
    from oracle.oracle import State
    n, d = 257, 33
    A = _sym(n, torch.float64, 2)
    # uniform entries are bit-identical to the oracle's, so FP64 sums agree to rounding
    S = rb.DenseSkOp(rb.DenseDist(d, n, rb.ScalarDist.Uniform), rb.RNGState(7),
                     dtype=torch.float64)
    B = torch.empty(d, n, device="cuda", dtype=torch.float64)
    rb.sketch_symmetric(rb.Layout.RowMajor, 1.0, S, A, n, 0.0, B, n)
    Sm = oracle.dense_matrix(1, d, n, 1, 1, State.make((0, 0, 0, 0), (7, 0)))
    ref = Sm @ to_host(A)
    rel = np.linalg.norm(to_host(B) - ref) / np.linalg.norm(ref)
    assert rel < 1e-12, rel


def test_symmetry_check(rb):
    import torch
    n, d = 64, 8
    A = _sym(n, torch.float32, 5)
    A[3, 10] += 1.0   # first violation in (i, j) loop order
    A[20, 7] += 1.0
    S = rb.DenseSkOp(rb.DenseDist(d, n), rb.RNGState(1))
    B = torch.empty(d, n, device="cuda")
    with pytest.raises(rb.RandBLASError, match=r"Symmetry check failed\. \|A\(3,10\) - A\(10,3\)\|"):
        rb.sketch_symmetric(rb.Layout.RowMajor, 1.0, S, A, n, 0.0, B, n)
    # column-major reading: A(i, j) is memory (j, i); the pair (3, 10) still fails first
    with pytest.raises(rb.RandBLASError, match=r"\|A\(3,10\) - A\(10,3\)\|"):
        rb.require_symmetric(rb.Layout.ColMajor, A, n, n, 0.0)
    rb.sketch_symmetric(rb.Layout.RowMajor, 1.0, S, A, n, 0.0, B, n, -1.0)  # no check
    A2 = _sym(n, torch.float32, 6)
    A2[1, 2] += 1e-3 * (abs(float(A2[1, 2])) * 2 + 1)
    rb.require_symmetric(rb.Layout.RowMajor, A2, n, n, 2e-3)  # inside the tolerance
