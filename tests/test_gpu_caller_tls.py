"""A caller of the drop-in: the reference's total-least-squares examples
(examples/total-least-squares/tls_dense_skop.cc, tls_sparse_skop.cc) on the GPU.

Noisy data [A | B] (m x (n+1), column-major; A Gaussian from fill_dense with RNGState(0),
B = A * ones + Gaussian noise from RNGState(1)), a 2(n+1) x m sketching operator (dense
Gaussian, and a SASO with 8 nonzeros per column), SAB = S [A | B] through sketch_general in
column-major layout, then TLS on the small sketch via its SVD.  Checks: the sketch equals the
FP64 product with the operator materialised by fill_dense (dense) / fill_sparse (SASO), and the
sketched TLS solution is close to the TLS solution of the full data and to the target x = 1."""
import pytest

pytestmark = pytest.mark.gpu


def _noisy_data(rb, m, n):
    import torch
    A = torch.empty(m * n, dtype=torch.float64, device="cuda")
    rb.fill_dense(rb.DenseDist(m, n), A, rb.RNGState(0))
    eps = torch.empty(m, dtype=torch.float64, device="cuda")
    rb.fill_dense(rb.DenseDist(m, 1), eps, rb.RNGState(1))
    # DenseDist(m, n) is tall with a long major axis: natural layout column-major, as the
    # example's buffer is read
    Am = A.view(n, m).T
    AB = torch.empty(m, n + 1, dtype=torch.float64, device="cuda")
    AB[:, :n] = Am
    AB[:, n] = Am @ torch.ones(n, dtype=torch.float64, device="cuda") + eps
    return AB.T.contiguous()  # column-major storage of [A | B]: (n+1) x m row-major


def _tls(X):
    """TLS solution from an (k x (n+1)) matrix [A | B]: x = -V[:n, n] / V[n, n]."""
    import torch
    _, _, Vh = torch.linalg.svd(X, full_matrices=False)
    v = Vh[-1]
    return -v[:-1] / v[-1]


@pytest.mark.parametrize("kind", ["dense", "saso"])
def test_sketched_tls(rb, kind):
    import torch
    m, n = 10000, 500
    sk = 2 * (n + 1)
    ABc = _noisy_data(rb, m, n)  # memory of the column-major m x (n+1) matrix
    SAB = torch.empty((n + 1) * sk, dtype=torch.float64, device="cuda")
    if kind == "dense":
        S = rb.DenseSkOp(rb.DenseDist(sk, m), rb.RNGState(1997), dtype=torch.float64)
    else:
        S = rb.SparseSkOp(rb.SparseDist(sk, m, 8, rb.Axis.Short), rb.RNGState(1997),
                          dtype=torch.float64)
    rb.sketch_general(rb.Layout.ColMajor, rb.Op.NoTrans, rb.Op.NoTrans, sk, n + 1, m, 1.0, S,
                      ABc, m, 0.0, SAB, sk)
    SABm = SAB.view(n + 1, sk).T  # sk x (n+1)
    ABm = ABc.view(n + 1, m).T     # m x (n+1)
    # the sketch against the FP64 product with the materialised operator
    if kind == "dense":
        Sm = torch.empty(sk * m, dtype=torch.float64, device="cuda")
        rb.fill_dense(S.dist, Sm, S.seed_state)
        Sd = Sm.view(sk, m)  # wide, long axis: row-major natural layout
    else:
        Sf = rb.SparseSkOp(S.dist, S.seed_state, dtype=torch.float64)
        rb.fill_sparse(Sf)
        Sd = torch.sparse_coo_tensor(torch.stack([Sf.rows, Sf.cols]), Sf.vals, (sk, m)).to_dense()
    ref = Sd @ ABm
    assert float((SABm - ref).norm() / ref.norm()) < 1e-12
    x_sk = _tls(SABm)
    x_true = _tls(ABm)
    ones = torch.ones(n, dtype=torch.float64, device="cuda")
    rel_true = float((x_true - ones).norm() / ones.norm())
    rel_sk = float((x_sk - ones).norm() / ones.norm())
    assert rel_true < 0.1, rel_true
    assert rel_sk < 0.5, rel_sk   # a 2(n+1)-row sketch: coarser, as in the reference example
