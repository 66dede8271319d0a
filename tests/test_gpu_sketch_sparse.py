"""Sparse sketching on the GPU (LSKGES / RSKGES with SASO and LASO operators, sketch_sparse
with COO / CSR / CSC data) against the reference's outputs (tests/golden) and, at the full
1024 x 2^20 SASO size, against an FP64 product of the bit-exact operator.

Criterion: the reference's componentwise bound (test/test_matmul_cores/linop_common.hh:
260-266), |B - B_ref| <= |alpha| (2K + 16) eps (|op(S)| |op(A)|) + 2 eps |beta| |B_in|."""
import numpy as np
import pytest

from conftest import load_golden
from gpu_helpers import as_matrix, check_bound, state_of, to_dev, to_host

pytestmark = pytest.mark.gpu

F32_GAUSS = 8 * 2.0**-24


def _eps(dt):
    return np.finfo(np.float32 if dt == 0 else np.float64).eps


def test_sparse_operator_sketch_golden(rb, oracle):
    import torch
    from oracle.oracle import State
    meta, z = load_golden("sketch_saso")
    for i, c in enumerate(meta):
        dt = torch.float32 if c["dtype"] == 0 else torch.float64
        D = rb.SparseDist(c["D_rows"], c["D_cols"], c["vec_nnz"], rb.Axis(c["axis"]))
        S = rb.SparseSkOp(D, state_of([c["ctr"], c["key"]]), dtype=dt)
        A, B0 = z[f"A{i}"], z[f"B{i}"]
        B = to_dev(B0)
        d, n, m, lay = c["d"], c["n"], c["m"], c["layout"]
        full = oracle.sparse_dense_matrix(1, c["D_rows"], c["D_cols"], c["vec_nnz"], c["axis"],
                                          State.make(c["ctr"], c["key"]))
        if c["side"] == 0:
            rb.sketch_general(rb.Layout(lay), rb.Op(c["opS"]), rb.Op(c["opA"]), d, n, m,
                              c["alpha"], S, c["ro"], c["co"], to_dev(A), c["lda"], c["beta"], B,
                              c["ldb"])
            sr, sc = (d, m) if c["opS"] == 0 else (m, d)
            Ssub = full[c["ro"]:c["ro"] + sr, c["co"]:c["co"] + sc]
            opS = Ssub if c["opS"] == 0 else Ssub.T
            ar, ac = (m, n) if c["opA"] == 0 else (n, m)
            Am = as_matrix(A, ar, ac, lay, c["lda"])
            prod = np.abs(opS) @ np.abs(Am if c["opA"] == 0 else Am.T)
            br, bc, K = d, n, m
        else:
            # reference right overload: B (n x d) = op(A) (n x m) op(S) (m x d)
            rb.sketch_general(rb.Layout(lay), rb.Op(c["opA"]), rb.Op(c["opS"]), n, d, m,
                              c["alpha"], to_dev(A), c["lda"], S, c["ro"], c["co"], c["beta"], B,
                              c["ldb"])
            sr, sc = (m, d) if c["opS"] == 0 else (d, m)
            Ssub = full[c["ro"]:c["ro"] + sr, c["co"]:c["co"] + sc]
            opS = Ssub if c["opS"] == 0 else Ssub.T
            ar, ac = (n, m) if c["opA"] == 0 else (m, n)
            Am = as_matrix(A, ar, ac, lay, c["lda"])
            prod = np.abs(Am if c["opA"] == 0 else Am.T) @ np.abs(opS)
            br, bc, K = n, d, m
        got = as_matrix(to_host(B), br, bc, lay, c["ldb"])
        ref = as_matrix(z[f"O{i}"], br, bc, lay, c["ldb"])
        bin_ = as_matrix(B0, br, bc, lay, c["ldb"])
        eps = _eps(c["dtype"])
        bound = abs(c["alpha"]) * (2 * K + 16) * eps * prod + \
            2 * eps * abs(c["beta"]) * np.abs(bin_) + 1e-300
        check_bound(got, ref, bound, c)


def test_prefilled_sparse_operator_matches_unsampled(rb):
    """Sampling inside the sketch and sketching with fill_sparse's COO give the same B: bitwise
    in deterministic mode (both through fixed-order row lists), to FP32 rounding with the fused
    SASO scatter (the default for short-axis operators)."""
    import torch
    for ax in (rb.Axis.Short, rb.Axis.Long):
        D = rb.SparseDist(64, 5000, 5, ax)
        A = torch.randn(5000 * 33, device="cuda")
        S1 = rb.SparseSkOp(D, rb.RNGState(21))
        S2 = rb.SparseSkOp(D, rb.RNGState(21))
        rb.fill_sparse(S2)
        out = {}
        for det in (True, False):
            rb.set_deterministic(det)
            try:
                for name, S in (("sampled", S1), ("filled", S2)):
                    B = torch.zeros(64 * 33, device="cuda")
                    rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, 64, 33,
                                      5000, 1.0, S, A, 33, 0.0, B, 33)
                    out[(det, name)] = B
            finally:
                rb.set_deterministic(False)
        assert torch.equal(out[(True, "sampled")], out[(True, "filled")])
        ref = out[(True, "filled")].double()
        rel = float((out[(False, "sampled")].double() - ref).norm() / ref.norm())
        assert rel <= 1e-6, (ax, rel)


def test_sketch_sparse_data_golden(rb, oracle):
    import torch
    from oracle.oracle import State
    meta, z = load_golden("sketch_sparse")
    for i, c in enumerate(meta):
        dt = torch.float32 if c["dtype"] == 0 else torch.float64
        D = rb.DenseDist(c["D_rows"], c["D_cols"], rb.ScalarDist.Gaussian, rb.Axis.Long)
        S = rb.DenseSkOp(D, state_of([c["ctr"], c["key"]]), dtype=dt)
        v, a, b = z[f"v{i}"], z[f"a{i}"], z[f"b{i}"]
        Ar, Ac = c["Ar"], c["Ac"]
        if c["fmt"] == 0:
            Amat = rb.COOMatrix(Ar, Ac, to_dev(v), to_dev(a), to_dev(b))
            dense = np.zeros((Ar, Ac))
            np.add.at(dense, (a, b), v.astype(np.float64))
        elif c["fmt"] == 1:
            Amat = rb.CSRMatrix(Ar, Ac, to_dev(v), to_dev(a), to_dev(b))
            rows = np.repeat(np.arange(Ar), np.diff(a))
            dense = np.zeros((Ar, Ac))
            np.add.at(dense, (rows, b), v.astype(np.float64))
        else:
            Amat = rb.CSCMatrix(Ar, Ac, to_dev(v), to_dev(b), to_dev(a))
            cols = np.repeat(np.arange(Ac), np.diff(a))
            dense = np.zeros((Ar, Ac))
            np.add.at(dense, (b, cols), v.astype(np.float64))
        B0 = z[f"B{i}"]
        B = to_dev(B0)
        d, n, m, lay = c["d"], c["n"], c["m"], c["layout"]
        opA = dense if c["opA"] == 0 else dense.T
        if c["side"] == 0:
            rb.sketch_sparse(rb.Layout(lay), rb.Op(c["opS"]), rb.Op(c["opA"]), d, n, m,
                             c["alpha"], S, c["ro"], c["co"], Amat, c["beta"], B, c["ldb"])
            sr, sc = (d, m) if c["opS"] == 0 else (m, d)
            Ssub = oracle.dense_matrix(1, c["D_rows"], c["D_cols"], 0, 1,
                                       State.make(c["ctr"], c["key"]), sr, sc, c["ro"], c["co"])
            prod = np.abs(Ssub if c["opS"] == 0 else Ssub.T) @ np.abs(opA)
            br, bc, K = d, n, m
        else:
            rb.sketch_sparse(rb.Layout(lay), rb.Op(c["opA"]), rb.Op(c["opS"]), n, d, m,
                             c["alpha"], Amat, S, c["ro"], c["co"], c["beta"], B, c["ldb"])
            sr, sc = (m, d) if c["opS"] == 0 else (d, m)
            Ssub = oracle.dense_matrix(1, c["D_rows"], c["D_cols"], 0, 1,
                                       State.make(c["ctr"], c["key"]), sr, sc, c["ro"], c["co"])
            prod = np.abs(opA) @ np.abs(Ssub if c["opS"] == 0 else Ssub.T)
            br, bc, K = n, d, m
        got = as_matrix(to_host(B), br, bc, lay, c["ldb"])
        ref = as_matrix(z[f"O{i}"], br, bc, lay, c["ldb"])
        bin_ = as_matrix(B0, br, bc, lay, c["ldb"])
        eps = _eps(c["dtype"])
        bound = abs(c["alpha"]) * ((2 * K + 16) * eps + F32_GAUSS) * prod + \
            2 * eps * abs(c["beta"]) * np.abs(bin_) + 1e-300
        check_bound(got, ref, bound, c)


def _kernels(rb, fn):
    """Run fn() with the library's kernel timing on; return (result, names of timed kernels)."""
    rb.profile.enable(True)
    try:
        out = fn()
        names = set(rb.profile.read())
    finally:
        rb.profile.enable(False)
    return out, names


def test_full_size_saso_sketch(rb):
    """1024 x 2^20 SASO (8 nonzeros per column) times a 2^20 x 256 N(0,1) FP32 matrix through
    each of the three SASO paths: row-major A takes the row-bucketed kernels (deterministic, so
    the default and deterministic modes agree bitwise), column-major A the shared-memory
    scatter by default and the row lists in deterministic mode.  Each: relative Frobenius error
    <= 1e-6 against an FP64 product of the same operator; the deterministic paths bitwise
    reproducible."""
    import torch
    m, d, n = 1 << 20, 1024, 256
    A = torch.empty(m * n, dtype=torch.float32, device="cuda")
    nxt = rb.fill_dense(rb.DenseDist(m, n, rb.ScalarDist.Gaussian, rb.Axis.Short), A,
                        rb.RNGState(0))
    S = rb.SparseSkOp(rb.SparseDist(d, m, 8), nxt)
    A_cm = A.view(m, n).t().contiguous().view(-1)  # the same matrix, column-major

    def sketch(layout, det):
        def go():
            B = torch.empty(d * n, dtype=torch.float32, device="cuda")
            if layout == rb.Layout.RowMajor:
                rb.sketch_general(layout, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 1.0, S, A, n,
                                  0.0, B, n)
                return B.view(d, n)
            rb.sketch_general(layout, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 1.0, S, A_cm, m,
                              0.0, B, d)
            return B.view(n, d).t()
        rb.set_deterministic(det)
        try:
            return _kernels(rb, go)
        finally:
            rb.set_deterministic(False)

    rows_fast, k1 = sketch(rb.Layout.RowMajor, False)
    rows_det, k2 = sketch(rb.Layout.RowMajor, True)
    scatter, k3 = sketch(rb.Layout.ColMajor, False)
    lists, k4 = sketch(rb.Layout.ColMajor, True)
    lists2, _ = sketch(rb.Layout.ColMajor, True)
    assert "saso_rows" in k1 and "saso_rows" in k2, (k1, k2)
    assert "saso_scatter" in k3 and "spmm_rows" in k4, (k3, k4)
    assert torch.equal(rows_fast, rows_det)
    assert torch.equal(lists, lists2)
    Sf = rb.SparseSkOp(rb.SparseDist(d, m, 8), nxt)
    rb.fill_sparse(Sf)
    idx = torch.stack([Sf.rows, Sf.cols])
    Ssp = torch.sparse_coo_tensor(idx, Sf.vals.double(), (d, m)).coalesce()
    ref = torch.sparse.mm(Ssp, A.view(m, n).double())
    for name, B in (("rows", rows_fast), ("scatter", scatter), ("lists", lists)):
        rel = (torch.linalg.norm(B.double() - ref) / torch.linalg.norm(ref)).item()
        assert rel <= 1e-6, (name, rel)


@pytest.mark.parametrize("M,N,K,k,ro,co,alpha,beta", [
    (700, 100, 100003, 5, 3, 7, 0.5, 2.0),    # ragged rows, columns and sub-chunks; beta != 0
    (2048, 64, 4096, 16, 0, 0, 1.0, 0.0),     # largest row count, 16 nonzeros per column
    (1, 64, 256, 1, 2, 0, -1.5, 0.0),         # one row, one sub-chunk (written directly)
    (513, 2560, 20000, 8, 0, 300, 1.0, 1.0),  # 40 column slices x 2 row blocks
])
def test_saso_row_bucketed(rb, M, N, K, k, ro, co, alpha, beta):
    """The row-bucketed SASO kernels on ragged shapes and submatrices of a larger operator:
    the reference's componentwise bound and relative error <= 1e-6 against an FP64 product of
    the operator from fill_sparse, and bitwise-identical repeated runs."""
    import torch
    D = rb.SparseDist(M + ro + 5, K + co + 11, k)
    st = rb.RNGState(M + 7 * K)
    lda = (N + 3) // 4 * 4 + 4   # 16-byte aligned rows with padding
    ldb = N + 1
    g = torch.Generator(device="cuda").manual_seed(K)
    A = torch.randn(K * lda, device="cuda", generator=g)
    B0 = torch.randn(M * ldb, device="cuda", generator=g)

    def go():
        S = rb.SparseSkOp(D, st)
        B = B0.clone()
        rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, M, N, K, alpha, S,
                          ro, co, A, lda, beta, B, ldb)
        return B

    B1, names = _kernels(rb, go)
    assert "saso_rows" in names and "saso_bucket" in names, names
    assert torch.equal(B1, go())
    Sf = rb.SparseSkOp(D, st)
    rb.fill_sparse(Sf)
    full = torch.zeros(D.n_rows, D.n_cols, dtype=torch.float64, device="cuda")
    full.index_put_((Sf.rows.long(), Sf.cols.long()), Sf.vals.double(), accumulate=True)
    Ssub = full[ro:ro + M, co:co + K]
    Am = A.view(K, lda)[:, :N].double()
    Bin = B0.view(M, ldb)[:, :N].double()
    ref = alpha * (Ssub @ Am) + beta * Bin
    got = B1.view(M, ldb)[:, :N].double()
    eps = 2.0**-23
    bound = abs(alpha) * (2 * K + 16) * eps * (Ssub.abs() @ Am.abs()) + \
        2 * eps * abs(beta) * Bin.abs() + 1e-300
    assert bool(((got - ref).abs() <= bound).all())
    rel = (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item()
    assert rel <= 1e-6, rel
    # padding columns of B untouched
    assert torch.equal(B1.view(M, ldb)[:, N:], B0.view(M, ldb)[:, N:])


@pytest.mark.parametrize("itype", ["int64", "int32"])
def test_saso_prefilled_row_bucketed(rb, itype):
    """A filled SASO operator (fill_sparse's COO arrays) goes through the row-bucketed kernels,
    which read the values from the arrays (here rescaled) and add entries that are no longer
    where fill_sparse put them (here 1000 positions shuffled across columns and 50 entries
    moved to other rows and columns) with atomics.  Checked against an FP64 product of the
    arrays as they are, on a submatrix; in deterministic mode the row-list path is used and
    repeats bitwise."""
    import torch
    M, N, K, k, ro, co = 700, 96, 50021, 6, 2, 3
    D = rb.SparseDist(M + 5, K + 9, k)
    idt = torch.int64 if itype == "int64" else torch.int32
    S = rb.SparseSkOp(D, rb.RNGState(11), index_dtype=idt)
    rb.fill_sparse(S)
    g = torch.Generator(device="cuda").manual_seed(3)
    S.vals.mul_(0.37)
    src = torch.randperm(1000, generator=g, device="cuda") + 5000
    dst = torch.arange(5000, 6000, device="cuda")
    for arr in (S.rows, S.cols, S.vals):
        arr[dst] = arr[src].clone()
    moved = torch.randint(0, D.full_nnz, (50,), generator=g, device="cuda")
    S.rows[moved] = torch.randint(0, D.n_rows, (50,), generator=g, device="cuda").to(idt)
    S.cols[moved] = torch.randint(0, D.n_cols, (50,), generator=g, device="cuda").to(idt)
    A = torch.randn(K * N, device="cuda", generator=g)

    def go():
        B = torch.zeros(M * N, device="cuda")
        rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, M, N, K, 1.0, S, ro,
                          co, A, N, 0.0, B, N)
        return B

    B, names = _kernels(rb, go)
    assert "saso_rows" in names and "saso_bucket" in names, names
    full = torch.zeros(D.n_rows, D.n_cols, dtype=torch.float64, device="cuda")
    full.index_put_((S.rows.long(), S.cols.long()), S.vals.double(), accumulate=True)
    Ssub = full[ro:ro + M, co:co + K]
    Am = A.view(K, N).double()
    ref = Ssub @ Am
    got = B.view(M, N).double()
    bound = (2 * K + 16) * 2.0**-23 * (Ssub.abs() @ Am.abs()) + 1e-300
    assert bool(((got - ref).abs() <= bound).all())
    rel = (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item()
    assert rel <= 1e-6, rel
    rb.set_deterministic(True)
    try:
        (B1, n1), (B2, _) = _kernels(rb, go), _kernels(rb, go)
    finally:
        rb.set_deterministic(False)
    assert "spmm_rows" in n1 and "saso_rows" not in n1, n1
    assert torch.equal(B1, B2)
    rel = (torch.linalg.norm(B1.view(M, N).double() - ref) / torch.linalg.norm(ref)).item()
    assert rel <= 1e-6, rel


def test_saso_prefilled_matches_sampled(rb):
    """A 1024 x 2^18 SASO sketch of a 2^18 x 256 matrix with the operator filled first: the
    row-bucketed kernels read the COO arrays and give the sampled path's result to FP32 rounding
    (<= 1e-6 relative)."""
    import torch
    m, d, n = 1 << 18, 1024, 256
    A = torch.randn(m * n, device="cuda", generator=torch.Generator(device="cuda").manual_seed(1))
    D = rb.SparseDist(d, m, 8)

    def sketch(S):
        B = torch.empty(d * n, device="cuda")
        rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 1.0, S, A,
                          n, 0.0, B, n)
        return B

    B_gen, n_gen = _kernels(rb, lambda: sketch(rb.SparseSkOp(D, rb.RNGState(9))))
    Sf = rb.SparseSkOp(D, rb.RNGState(9))
    rb.fill_sparse(Sf)
    B_fill, n_fill = _kernels(rb, lambda: sketch(Sf))
    assert "saso_rows" in n_gen and "saso_rows" in n_fill, (n_gen, n_fill)
    rel = (torch.linalg.norm(B_fill.double() - B_gen.double()) /
           torch.linalg.norm(B_gen.double())).item()
    assert rel <= 1e-6, rel


def test_sketch_sparse_generated_operator_fused(rb):
    """sketch_sparse with an unfilled dense operator and CSR data (left) or CSC data (right)
    generates the operator inside the SpMM (gen_spmm) instead of filling it first: the result
    matches the materialised operator's path (the operator filled explicitly) to FP32
    rounding, and repeats bit for bit.  The workload is the benchmark's: a Gaussian 1024 x 2^17
    operator and the 2^17 x 512 random_csr matrix with 5 nonzeros per row."""
    import torch
    d, m, n = 1024, 1 << 17, 512
    A, _ = rb.random_csr(m, n, 5 / n, rb.RNGState(11), dtype=torch.float32)
    D = rb.DenseDist(d, m, rb.ScalarDist.Gaussian)

    def left(S):
        B = torch.empty(d * n, device="cuda")
        rb.sketch_sparse(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 1.0, S, 0,
                         0, A, 0.0, B, n)
        return B

    S = rb.DenseSkOp(D, rb.RNGState(5))
    got, names = _kernels(rb, lambda: left(S))
    assert "gen_spmm" in names and "spmm_row_lists" not in names, names
    again = left(rb.DenseSkOp(D, rb.RNGState(5)))
    assert torch.equal(got, again)
    Sf = rb.DenseSkOp(D, rb.RNGState(5))
    rb.fill_dense(Sf)
    ref, names_f = _kernels(rb, lambda: left(Sf))
    assert "gen_spmm" not in names_f
    rel = float(torch.linalg.vector_norm(got - ref) / torch.linalg.vector_norm(ref))
    assert rel <= 1e-6, rel
    print("fused vs materialised operator: rel", rel)

    # right side: B (mr x dr) = A_csc (mr x nr) * S (nr x dr); the fused kernel's output
    # columns are B's rows, so the right side takes it for moderate mr
    mr, nr, dr = 300, 1 << 14, 256
    Ac, _ = rb.random_csc(mr, nr, 0.01, rb.RNGState(12), dtype=torch.float32)
    Dr = rb.DenseDist(nr, dr, rb.ScalarDist.Uniform)

    def right(S):
        B = torch.zeros(mr * dr, device="cuda")
        rb.sketch_sparse(rb.Layout.ColMajor, rb.Op.NoTrans, rb.Op.NoTrans, mr, dr, nr, 1.0, Ac,
                         S, 0, 0, 0.0, B, mr)
        return B

    got_r, names_r = _kernels(rb, lambda: right(rb.DenseSkOp(Dr, rb.RNGState(6))))
    assert "gen_spmm" in names_r, names_r
    Srf = rb.DenseSkOp(Dr, rb.RNGState(6))
    rb.fill_dense(Srf)
    ref_r = right(Srf)
    rel_r = float(torch.linalg.vector_norm(got_r - ref_r) / torch.linalg.vector_norm(ref_r))
    assert rel_r <= 1e-6, rel_r
