"""Dense sketching on the GPU (LSKGE3 / RSKGE3 / sketch_vector) against the reference's own
outputs (tests/golden) and the oracle, every layout / op / side / submatrix combination.

Criterion: the reference's componentwise bound (test/test_matmul_cores/linop_common.hh:260-266)
|B - B_ref| <= |alpha| * c * eps * (|op(S)| |op(A)|) + 2 eps |beta| |B_in| with c = 2m + 16,
plus 8 float ulps of |op(S)| |op(A)| when S is Gaussian (Box-Muller entries may differ from the
reference's glibc-based ones by a few ulp)."""
import numpy as np
import pytest

from conftest import load_golden
from gpu_helpers import as_matrix, check_bound, state_of, to_dev, to_host

pytestmark = pytest.mark.gpu

F32_GAUSS = 8 * 2.0**-24


def _eps(dt):
    return np.finfo(np.float32 if dt == 0 else np.float64).eps


def _explicit_sub(oracle, c, rows, cols, family):
    from oracle.oracle import State
    return oracle.dense_matrix(1, c["D_rows"], c["D_cols"], family, 1,
                               State.make(c["ctr"], c["key"]), rows, cols, c["ro"], c["co"])


def test_sketch_general_dense_golden(rb, oracle):
    import torch
    meta, z = load_golden("sketch_dense")
    for i, c in enumerate(meta):
        dt = torch.float32 if c["dtype"] == 0 else torch.float64
        D = rb.DenseDist(c["D_rows"], c["D_cols"], rb.ScalarDist(c["family"]), rb.Axis.Long)
        S = rb.DenseSkOp(D, state_of([c["ctr"], c["key"]]), dtype=dt)
        if c["prefill"]:
            rb.fill_dense(S)
        A, B0 = z[f"A{i}"], z[f"B{i}"]
        B = to_dev(B0)
        d, n, m, lay = c["d"], c["n"], c["m"], c["layout"]
        if c["side"] == 0:
            rb.sketch_general(rb.Layout(lay), rb.Op(c["opS"]), rb.Op(c["opA"]), d, n, m,
                              c["alpha"], S, c["ro"], c["co"], to_dev(A), c["lda"], c["beta"], B,
                              c["ldb"])
            srows, scols = (d, m) if c["opS"] == 0 else (m, d)
            ar, ac = (m, n) if c["opA"] == 0 else (n, m)
            Ssub = _explicit_sub(oracle, c, srows, scols, c["family"])
            opS = Ssub if c["opS"] == 0 else Ssub.T
            Am = as_matrix(A, ar, ac, lay, c["lda"])
            opA = Am if c["opA"] == 0 else Am.T
            prod = np.abs(opS) @ np.abs(opA)
            br, bc, K = d, n, m
        else:
            # reference right overload (m, d, n) = (rows of B, d, inner)
            mm, dd, nn = m, d, n
            rb.sketch_general(rb.Layout(lay), rb.Op(c["opA"]), rb.Op(c["opS"]), mm, dd, nn,
                              c["alpha"], to_dev(A), c["lda"], S, c["ro"], c["co"], c["beta"], B,
                              c["ldb"])
            srows, scols = (nn, dd) if c["opS"] == 0 else (dd, nn)
            ar, ac = (mm, nn) if c["opA"] == 0 else (nn, mm)
            Ssub = _explicit_sub(oracle, c, srows, scols, c["family"])
            opS = Ssub if c["opS"] == 0 else Ssub.T
            Am = as_matrix(A, ar, ac, lay, c["lda"])
            opA = Am if c["opA"] == 0 else Am.T
            prod = np.abs(opA) @ np.abs(opS)
            br, bc, K = mm, dd, nn
        got = as_matrix(to_host(B), br, bc, lay, c["ldb"])
        ref = as_matrix(z[f"O{i}"], br, bc, lay, c["ldb"])
        bin_ = as_matrix(B0, br, bc, lay, c["ldb"])
        eps = _eps(c["dtype"])
        slack = (2 * K + 16) * eps + (F32_GAUSS if c["family"] == 0 else 0.0)
        bound = abs(c["alpha"]) * slack * prod + 2 * eps * abs(c["beta"]) * np.abs(bin_) + 1e-300
        check_bound(got, ref, bound, c)
        # untouched padding rows / columns of B stay as they were
        assert np.array_equal(to_host(B).size, B0.size)


def test_sketch_vector_golden(rb, oracle):
    import torch
    meta, z = load_golden("sketch_vector")
    for i, c in enumerate(meta):
        dt = torch.float32 if c["dtype"] == 0 else torch.float64
        D = rb.DenseDist(c["D_rows"], c["D_cols"], rb.ScalarDist(c["family"]), rb.Axis.Long)
        S = rb.DenseSkOp(D, state_of([c["ctr"], c["key"]]), dtype=dt)
        x, y0 = z[f"x{i}"], z[f"y{i}"]
        y = to_dev(y0)
        rb.sketch_vector(rb.Op(c["opS"]), c["d"], c["m"], c["alpha"], S, c["ro"], c["co"],
                         to_dev(x), c["incx"], c["beta"], y, c["incy"])
        Ssub = _explicit_sub(oracle, c, c["d"], c["m"], c["family"])
        opS = Ssub if c["opS"] == 0 else Ssub.T
        xs = x[::c["incx"]][:opS.shape[1]]
        ys = to_host(y)[::c["incy"]][:opS.shape[0]]
        ref = z[f"o{i}"][::c["incy"]][:opS.shape[0]]
        eps = _eps(c["dtype"])
        slack = (2 * opS.shape[1] + 16) * eps + (F32_GAUSS if c["family"] == 0 else 0.0)
        bound = abs(c["alpha"]) * slack * (np.abs(opS) @ np.abs(xs)) + \
            2 * eps * abs(c["beta"]) * np.abs(y0[::c["incy"]][:opS.shape[0]]) + 1e-300
        check_bound(ys, ref, bound, c)
        # entries between the strides are untouched
        if c["incy"] > 1:
            mask = np.ones(y0.size, bool)
            mask[::c["incy"]] = False
            assert np.array_equal(to_host(y)[mask], y0[mask])


@pytest.mark.parametrize("opS,co,incx", [(0, 0, 1), (0, 3, 1), (0, 4, 2), (1, 0, 1)])
def test_sketch_vector_large(rb, opS, co, incx):
    """sketch_vector with a uniform 512 x 2^18 operator (many K ranges, the interior fast path
    with vector loads when x is contiguous and aligned, scalar loads otherwise, and the
    transposed orientation), against the FP64 product of the filled operator."""
    import torch
    d, m = 512, 1 << 18
    D = rb.DenseDist(d, m + co + 5, rb.ScalarDist.Uniform)
    S = rb.DenseSkOp(D, rb.RNGState(21))
    g = torch.Generator(device="cuda").manual_seed(21)
    rows, cols = (d, m) if opS == 0 else (m, d)  # op(submat(S)); submat(S) is d x m
    full = torch.empty(D.n_rows * D.n_cols, device="cuda")
    rb.fill_dense(D, full, rb.RNGState(21))
    Sfull = full.view(D.n_rows, D.n_cols) if D.natural_layout == rb.Layout.RowMajor else \
        full.view(D.n_cols, D.n_rows).T
    Ssub = Sfull[:d, co:co + m]
    opSm = Ssub if opS == 0 else Ssub.T
    x = torch.randn(cols * incx, device="cuda", generator=g)
    y = torch.zeros(rows, device="cuda")
    rb.sketch_vector(rb.Op(opS), d, m, 1.0, S, 0, co, x, incx, 0.0, y, 1)
    ref = opSm.double() @ x[::incx].double()
    rel = float((y.double() - ref).norm() / ref.norm())
    # FP32 sums of up to 2^18 terms: about 6e-7 expected; a wrong entry or index gives O(1)
    assert rel <= 2e-6, rel


def test_gaussian_fp64_200x10000_left_sketch(rb, oracle):
    """The 200 x 10000 Gaussian FP64 left sketch of a 10000 x 50 column-major uniform[-1,1]
    matrix (Philox key 0, counter 0; the operator is seeded at the data's next state).  The
    GEMM itself is held to 1e-12 relative against an FP64 product of the operator the GPU
    generated; that operator is held to the reference's entries within a few ulp
    (test_gpu_fill)."""
    import torch
    from oracle.oracle import State
    # data: raw uneg11 values, 50 rows x 10000 row-major == 10000 x 50 col-major
    A, anext = oracle.fill_dense_submat(1, 1, 10000, 50, 10000, 0,
                                        State.make((0, 0, 0, 0), (0, 0)))
    assert list(anext.counter) == [125000, 0, 0, 0]
    seed = rb.RNGState(0, counter=(125000, 0, 0, 0))
    D = rb.DenseDist(200, 10000)
    S = rb.DenseSkOp(D, seed, dtype=torch.float64)
    B = torch.zeros(200 * 50, dtype=torch.float64, device="cuda")
    rb.sketch_general(rb.Layout.ColMajor, rb.Op.NoTrans, rb.Op.NoTrans, 200, 50, 10000, 1.0, S,
                      to_dev(A), 10000, 0.0, B, 200)
    Sbuf = torch.empty(200 * 10000, dtype=torch.float64, device="cuda")
    rb.fill_dense(D, Sbuf, seed)
    Sg = to_host(Sbuf).reshape(200, 10000)
    Acm = A.reshape(50, 10000).T
    ref = Sg @ Acm
    got = to_host(B).reshape(50, 200).T
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel <= 1e-12, rel


def test_fp32_larger_against_fp64_oracle(rb, oracle):
    """FP32 sketches with offsets, both sides: normwise relative error <= 1e-6 against FP64."""
    import torch
    from oracle.oracle import State
    rng = np.random.default_rng(1)
    for fam in (0, 1):
        d, n, m = 300, 130, 20000
        D = rb.DenseDist(d + 7, m + 11, rb.ScalarDist(fam))
        seed = rb.RNGState(77, counter=(3, 0, 0, 0))
        S = rb.DenseSkOp(D, seed)
        A = rng.standard_normal((m, n)).astype(np.float32)  # row-major m x n
        B = torch.zeros(d * n, dtype=torch.float32, device="cuda")
        rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 1.0, S, 5,
                          9, to_dev(A), n, 0.0, B, n)
        Ssub = oracle.dense_matrix(1, d + 7, m + 11, fam, 1, State.make((3, 0, 0, 0), (77, 0)),
                                   d, m, 5, 9)
        ref = Ssub @ A.astype(np.float64)
        got = to_host(B).reshape(d, n)
        rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert rel <= 1e-6, (fam, rel)
        # right sketch: A2 (n x m) * S^T-shaped submatrix
        A2 = rng.standard_normal((n, m)).astype(np.float32)
        B2 = torch.zeros(n * d, dtype=torch.float32, device="cuda")
        S2 = rb.DenseSkOp(rb.DenseDist(m + 11, d + 7, rb.ScalarDist(fam)), seed)
        rb.sketch_general(rb.Layout.ColMajor, rb.Op.NoTrans, rb.Op.NoTrans, n, d, m, 1.0,
                          to_dev(A2.T.copy()), n, S2, 9, 5, 0.0, B2, n)
        S2sub = oracle.dense_matrix(1, m + 11, d + 7, fam, 1, State.make((3, 0, 0, 0), (77, 0)),
                                    m, d, 9, 5)
        ref2 = A2.astype(np.float64) @ S2sub
        got2 = to_host(B2).reshape(d, n).T
        rel2 = np.linalg.norm(got2 - ref2) / np.linalg.norm(ref2)
        assert rel2 <= 1e-6, (fam, rel2)


def test_alpha_zero_and_beta_zero_semantics(rb):
    """alpha == 0 leaves beta * B and never reads A; beta == 0 overwrites NaNs in B."""
    import torch
    D = rb.DenseDist(20, 300)
    S = rb.DenseSkOp(D, rb.RNGState(1))
    B = torch.full((20 * 4,), float("nan"), device="cuda")
    A = torch.randn(300 * 4, device="cuda")
    rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, 20, 4, 300, 1.0, S, A, 4,
                      0.0, B, 4)
    assert torch.isfinite(B).all()
    B2 = torch.ones(20 * 4, device="cuda")
    rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, 20, 4, 300, 0.0, S, A, 4,
                      3.0, B2, 4)
    assert torch.equal(B2, torch.full_like(B2, 3.0))


@pytest.mark.parametrize("family,axis", [("Uniform", "Long"), ("Gaussian", "Long"),
                                         ("Uniform", "Short"), ("Gaussian", "Short")])
def test_cluster_shared_operator_tiles_bitwise(rb, family, axis):
    """Sketches whose data spans several 128-column tiles share each generated operator tile
    across a thread-block cluster (each CTA generates part of it).  The result must be the same
    bits as sketching each 128-column block alone (no cluster); K = 240 keeps both unsplit.
    Both natural layouts of S (rows of S per output row, or per k), and a partial last row
    block (d = 300)."""
    import torch
    d, n, m = 300, 512, 240
    D = rb.DenseDist(d, m, getattr(rb.ScalarDist, family), getattr(rb.Axis, axis))
    S = rb.DenseSkOp(D, rb.RNGState(77))
    A = torch.randn(m, n, device="cuda", generator=torch.Generator(device="cuda").manual_seed(2))
    B = torch.empty(d, n, device="cuda")
    rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 1.0, S,
                      A.view(-1), n, 0.0, B.view(-1), n)
    for c in range(0, n, 128):
        Ab = A[:, c:c + 128].contiguous()
        Bb = torch.empty(d, 128, device="cuda")
        rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, 128, m, 1.0, S,
                          Ab.view(-1), 128, 0.0, Bb.view(-1), 128)
        assert torch.equal(B[:, c:c + 128], Bb), c
