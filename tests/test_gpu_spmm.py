"""The public sparse x dense products on the GPU -- left_spmm, right_spmm and spmm
(RandBLAS/sparse_data/spmm_dispatch.hh:52-219, 298-302, 376-380) -- against the reference's
own outputs in tests/golden/spmm.npz: COO / CSR / CSC data, both ops on either operand, both
layouts, FP32 and FP64, COO submatrix offsets (coo_spmm_impl.hh:70-92) and repeated entries,
alpha = 0 (C = beta C, the sparse data unread), beta = 0 over a NaN-filled C, data without
nonzeros, and the reference's argument checks with their messages.

Criterion: the reference's componentwise bound (test/test_matmul_cores/linop_common.hh:
260-266), |C - C_ref| <= |alpha| (2K + 16) eps (|op(A)| |op(B)|) + 2 eps |beta| |C_in|; the
entries of C's buffer outside the d x n (or m x d) matrix stay as they were."""
import numpy as np
import pytest

from conftest import load_golden
from gpu_helpers import as_matrix, check_bound, to_dev, to_host

pytestmark = pytest.mark.gpu


def _spmat(rb, fmt, rows, cols, v, a, b):
    if fmt == 0:
        return rb.COOMatrix(rows, cols, to_dev(v), to_dev(a), to_dev(b))
    if fmt == 1:
        return rb.CSRMatrix(rows, cols, to_dev(v), to_dev(a), to_dev(b))
    return rb.CSCMatrix(rows, cols, to_dev(v), to_dev(b), to_dev(a))


def _dense_of(c, v, a, b):
    """The sparse operand as a dense FP64 array (repeated COO entries add up)."""
    M = np.zeros((c["S_rows"], c["S_cols"]))
    v = v.astype(np.float64)
    if c["fmt"] == 0:
        np.add.at(M, (a, b), v)
    elif c["fmt"] == 1:
        r = np.repeat(np.arange(c["S_rows"]), np.diff(a))
        np.add.at(M, (r, b), v)
    else:
        col = np.repeat(np.arange(c["S_cols"]), np.diff(a))
        np.add.at(M, (b, col), v)
    return M


def _run(rb, c, z, i, use_spmm=False, keep=None):
    v, a, b = z[f"v{i}"], z[f"a{i}"], z[f"b{i}"]
    A = _spmat(rb, c["fmt"], c["S_rows"], c["S_cols"], v, a, b)
    dense = to_dev(z[f"D{i}"])
    C = to_dev(z[f"C{i}"])
    if keep is not None:
        keep.append(C)
    lay, opA, opB = rb.Layout(c["layout"]), rb.Op(c["opA"]), rb.Op(c["opB"])
    if c["side"] == 0:
        if use_spmm:
            rb.spmm(lay, opA, opB, c["d"], c["n"], c["m"], c["alpha"], A, dense, c["ldd"],
                    c["beta"], C, c["ldc"])
        else:
            rb.left_spmm(lay, opA, opB, c["d"], c["n"], c["m"], c["alpha"], A, c["ro"], c["co"],
                         dense, c["ldd"], c["beta"], C, c["ldc"])
    else:
        if use_spmm:
            rb.spmm(lay, opA, opB, c["m"], c["d"], c["n"], c["alpha"], dense, c["ldd"], A,
                    c["beta"], C, c["ldc"])
        else:
            rb.right_spmm(lay, opA, opB, c["m"], c["d"], c["n"], c["alpha"], dense, c["ldd"], A,
                          c["ro"], c["co"], c["beta"], C, c["ldc"])
    return to_host(C)


def _check_case(c, z, i, got):
    lay = c["layout"]
    cr, cc = c["C_rows"], c["C_cols"]
    ref = as_matrix(z[f"O{i}"], cr, cc, lay, c["ldc"])
    out = as_matrix(got, cr, cc, lay, c["ldc"])
    cin = as_matrix(z[f"C{i}"], cr, cc, lay, c["ldc"])
    eps = np.finfo(np.float32 if c["dtype"] == 0 else np.float64).eps
    Sfull = _dense_of(c, z[f"v{i}"], z[f"a{i}"], z[f"b{i}"])
    dm = as_matrix(z[f"D{i}"], c["dense_rows"], c["dense_cols"], lay, c["ldd"]).astype(np.float64)
    if c["side"] == 0:
        sr, sc = (c["d"], c["m"]) if c["opA"] == 0 else (c["m"], c["d"])
        sub = Sfull[c["ro"]:c["ro"] + sr, c["co"]:c["co"] + sc]
        opS = sub if c["opA"] == 0 else sub.T
        opD = dm if c["opB"] == 0 else dm.T
        prod, K = np.abs(opS) @ np.abs(opD), c["m"]
    else:
        sr, sc = (c["n"], c["d"]) if c["opB"] == 0 else (c["d"], c["n"])
        sub = Sfull[c["ro"]:c["ro"] + sr, c["co"]:c["co"] + sc]
        opS = sub if c["opB"] == 0 else sub.T
        opD = dm if c["opA"] == 0 else dm.T
        prod, K = np.abs(opD) @ np.abs(opS), c["n"]
    cterm = 0.0 if c["beta"] == 0 else 2 * eps * abs(c["beta"]) * np.abs(cin)
    bound = abs(c["alpha"]) * (2 * K + 16) * eps * prod + cterm + 1e-300
    assert not np.isnan(out).any(), c
    check_bound(out, ref, bound, c)
    # entries outside the matrix (leading-dimension padding) are untouched, NaN included
    mask = np.ones(got.shape, bool)
    idx = np.arange(got.size).reshape(-1)
    ld = c["ldc"]
    inner = (idx % ld < (cr if lay == 0 else cc)) & (idx // ld < (cc if lay == 0 else cr))
    mask &= ~inner
    assert np.array_equal(got[mask], z[f"C{i}"][mask], equal_nan=True), c


def test_left_right_spmm_golden(rb):
    meta, z = load_golden("spmm")
    ran = 0
    for i, c in enumerate(meta):
        if c["rc"]:
            continue
        _check_case(c, z, i, _run(rb, c, z, i))
        ran += 1
    assert ran >= 130


def test_spmm_overloads_golden(rb):
    """spmm(...) picks the side from the sparse operand's position and takes no offsets: the
    golden cases without offsets give the same results through it."""
    meta, z = load_golden("spmm")
    ran = 0
    for i, c in enumerate(meta):
        if c["rc"] or c["ro"] or c["co"]:
            continue
        _check_case(c, z, i, _run(rb, c, z, i, use_spmm=True))
        ran += 1
    assert ran >= 50


def test_spmm_argument_checks_golden(rb):
    """CSR / CSC data must match the product's sizes and take no offsets, COO data must cover
    the submatrix, leading dimensions must cover the stored sizes: the same conditions fail as
    in the reference, with its messages, and C is left as it was."""
    meta, z = load_golden("spmm")
    checked = 0
    for i, c in enumerate(meta):
        if not c["rc"]:
            continue
        keep = []
        with pytest.raises(rb.RandBLASError) as e:
            _run(rb, c, z, i, keep=keep)
        assert e.value.code == c["rc"]
        assert str(e.value) == c["msg"], (str(e.value), c)
        checked += 1
        assert np.array_equal(to_host(keep[0]), z[f"C{i}"], equal_nan=True)
    assert checked == 30


def test_spmm_larger_random_csr(rb):
    """A 2000 x 3000 random_csr matrix (about 12 nonzeros per row) times a 3000 x 96 FP32
    matrix, both orders (left and right), against an FP64 product on the GPU."""
    import torch
    A, _ = rb.random_csr(2000, 3000, 0.004, rb.RNGState(17), dtype=torch.float32)
    g = torch.Generator(device="cuda").manual_seed(3)
    X = torch.randn(3000, 96, device="cuda", generator=g)
    Cl = torch.empty(2000, 96, device="cuda")
    rb.left_spmm(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, 2000, 96, 3000, 1.0, A, 0, 0,
                 X, 96, 0.0, Cl, 96)
    rows = torch.repeat_interleave(torch.arange(2000, device="cuda"),
                                   torch.diff(A.rowptr.long()))
    Ad = torch.zeros(2000, 3000, dtype=torch.float64, device="cuda")
    Ad.index_put_((rows, A.colidxs.long()), A.vals.double(), accumulate=True)
    ref = Ad @ X.double()
    assert ((Cl.double() - ref).norm() / ref.norm()).item() <= 1e-6
    # right: Y (96 x 2000) = X^T (96 x 3000) A^T (3000 x 2000), A^T as opB = Trans
    Y = torch.empty(96, 2000, device="cuda")
    rb.right_spmm(rb.Layout.RowMajor, rb.Op.Trans, rb.Op.Trans, 96, 2000, 3000, 1.0, X, 96, A,
                  0, 0, 0.0, Y, 2000)
    assert ((Y.double() - ref.T).norm() / ref.norm()).item() <= 1e-6
