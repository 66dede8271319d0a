"""GPU sparse-data conversions (sparse_data/base.hh:119-220, 278-302; conversions.hh:49-166)
against the reference's outputs (golden fixtures) and numpy: sort detection, sorting into CSR
or CSC order, compressed pointers to indices and back, format conversions and transposes, with
the reference's check messages."""
import numpy as np
import pytest

from conftest import load_golden
from gpu_helpers import to_dev, to_host

pytestmark = pytest.mark.gpu


def test_sparse_convert_golden(rb):
    meta, z = load_golden("sparse_convert")
    for i, c in enumerate(meta):
        rows, cols, vals = z[f"r{i}"], z[f"c{i}"], z[f"v{i}"]
        R, Cc = to_dev(rows), to_dev(cols)
        assert chr(int(rb.coo_arrays_determine_sort(R, Cc))) == c["determine"], c
        for s, flag in (("R", rb.NonzeroSort.CSR), ("C", rb.NonzeroSort.CSC)):
            A = rb.COOMatrix(c["m"], c["n"], to_dev(vals), to_dev(rows), to_dev(cols))
            A.sort_arrays(flag)
            assert A.sort == flag
            assert np.array_equal(to_host(A.vals), z[f"{s}v{i}"]), (c, s)
            assert np.array_equal(to_host(A.rows), z[f"{s}r{i}"]), (c, s)
            assert np.array_equal(to_host(A.cols), z[f"{s}c{i}"]), (c, s)
            major, comp = (A.rows, c["m"]) if s == "R" else (A.cols, c["n"])
            ptr = rb.sorted_idxs_to_compressed_ptr(major, comp)
            assert np.array_equal(to_host(ptr), z[f"{s}p{i}"]), (c, s)
            back = rb.compressed_ptr_to_sorted_idxs(ptr, c["nnz"])
            assert np.array_equal(to_host(back), to_host(major)), (c, s)


def test_conversion_round_trips(rb):
    import torch
    A, _ = rb.random_csr(3000, 700, 0.01, rb.RNGState(5), dtype=torch.float32)
    coo = rb.csr_to_coo(A)
    assert coo.sort == rb.NonzeroSort.CSR
    p = to_host(A.rowptr)
    assert np.array_equal(to_host(coo.rows), np.repeat(np.arange(3000), np.diff(p)))
    B = rb.coo_to_csr(coo)
    assert torch.equal(B.rowptr, A.rowptr) and torch.equal(B.colidxs, A.colidxs)
    assert torch.equal(B.vals, A.vals)
    # the same entries in a random order: coo_to_csr sorts a copy, the input is unchanged
    perm = torch.randperm(coo.vals.numel(), device="cuda",
                          generator=torch.Generator(device="cuda").manual_seed(2))
    shuffled = rb.COOMatrix(3000, 700, coo.vals[perm], coo.rows[perm], coo.cols[perm])
    assert rb.coo_arrays_determine_sort(shuffled.rows, shuffled.cols) == rb.NonzeroSort.NONE
    rows_before = shuffled.rows.clone()
    B2 = rb.coo_to_csr(shuffled)
    assert torch.equal(shuffled.rows, rows_before)
    assert torch.equal(B2.rowptr, A.rowptr) and torch.equal(B2.colidxs, A.colidxs)
    assert torch.equal(B2.vals, A.vals)
    # CSC of the same matrix, and back
    Ccsc = rb.coo_to_csc(shuffled)
    coo_c = rb.csc_to_coo(Ccsc)
    assert coo_c.sort == rb.NonzeroSort.CSC
    key = to_host(coo_c.cols).astype(np.int64) * 3000 + to_host(coo_c.rows)
    assert np.all(np.diff(key) > 0)
    dense = np.zeros((3000, 700))
    dense[to_host(coo_c.rows), to_host(coo_c.cols)] = to_host(coo_c.vals)
    dense_ref = np.zeros((3000, 700))
    dense_ref[np.repeat(np.arange(3000), np.diff(p)), to_host(A.colidxs)] = to_host(A.vals)
    assert np.array_equal(dense, dense_ref)
    # int32 indices and an empty matrix
    A32, _ = rb.random_csc(500, 400, 0.02, rb.RNGState(6), dtype=torch.float64,
                           itype=torch.int32)
    assert torch.equal(rb.coo_to_csc(rb.csc_to_coo(A32)).colptr, A32.colptr)
    E = rb.COOMatrix(5, 6, torch.empty(0, device="cuda"),
                     torch.empty(0, dtype=torch.int64, device="cuda"),
                     torch.empty(0, dtype=torch.int64, device="cuda"))
    assert not to_host(rb.coo_to_csr(E).rowptr).any()


def test_coo_sort_large_vs_numpy(rb):
    """2^22 duplicate-free entries in random order, int64 indices beyond 2^32 in the linear
    index: the stable two-pass radix sort equals numpy's lexsort."""
    import torch
    rng = np.random.default_rng(9)
    m, n, k = 1 << 20, 1 << 14, 1 << 22
    key = np.unique(rng.integers(0, m * n, size=k + k // 8))[:k]
    rng.shuffle(key)
    rows, cols = key // n, key % n
    vals = rng.standard_normal(key.size).astype(np.float32)
    A = rb.COOMatrix(m, n, to_dev(vals), to_dev(rows), to_dev(cols))
    A.sort_arrays(rb.NonzeroSort.CSC)
    o = np.lexsort((rows, cols))
    assert np.array_equal(to_host(A.rows), rows[o]) and np.array_equal(to_host(A.cols), cols[o])
    assert np.array_equal(to_host(A.vals), vals[o])
    A.sort_arrays(rb.NonzeroSort.CSR)
    o = np.lexsort((cols, rows))
    assert np.array_equal(to_host(A.rows), rows[o]) and np.array_equal(to_host(A.vals), vals[o])


def test_transposes_in_sketch_sparse(rb):
    """transpose_as_csc(A) shares A's arrays; sketching with op(A^T) = Trans gives the same
    product as sketching with A."""
    import torch
    A, _ = rb.random_csr(4096, 256, 0.02, rb.RNGState(7), dtype=torch.float32)
    At = rb.transpose_as_csc(A)
    assert At.vals.data_ptr() == A.vals.data_ptr() and (At.n_rows, At.n_cols) == (256, 4096)
    S = rb.DenseSkOp(rb.DenseDist(128, 4096, rb.ScalarDist.Uniform), rb.RNGState(8))
    B1 = torch.empty(128 * 256, device="cuda")
    B2 = torch.empty(128 * 256, device="cuda")
    rb.sketch_sparse(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, 128, 256, 4096, 1.0, S, 0,
                     0, A, 0.0, B1, 256)
    rb.sketch_sparse(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.Trans, 128, 256, 4096, 1.0, S, 0,
                     0, At, 0.0, B2, 256)
    assert torch.equal(B1, B2)
    Tc = rb.transpose_as_coo(rb.csr_to_coo(A), share_memory=False)
    assert Tc.sort == rb.NonzeroSort.CSC and (Tc.n_rows, Tc.n_cols) == (256, 4096)
    assert torch.equal(rb.transpose_as_csr(rb.coo_to_csc(Tc)).rowptr, A.rowptr)


def test_conversion_checks(rb):
    import torch
    with pytest.raises(rb.RandBLASError) as e:
        rb.sorted_idxs_to_compressed_ptr(torch.tensor([0, 2, 1], device="cuda"), 3)
    assert str(e.value) == ("(idxs[i - 1] <= idxs[i]) was required, but did not hold, in "
                            "function sorted_idxs_to_compressed_ptr")
    with pytest.raises(rb.RandBLASError) as e:
        rb.compressed_ptr_to_sorted_idxs(torch.tensor([0, 3, 2], device="cuda"), 5)
    assert "(col_nnz >= 0) was required" in str(e.value)
    with pytest.raises(rb.RandBLASError) as e:
        rb.compressed_ptr_to_sorted_idxs(torch.tensor([0, 3, 6], device="cuda"), 5)
    assert "(len_idxs >= ptr[num_comp]) was required" in str(e.value)
    # the reference's walk: a leading negative index leaves every pointer 0; indices past the
    # last compressed index are not counted
    p = rb.sorted_idxs_to_compressed_ptr(torch.tensor([-1, 0, 2], device="cuda"), 3)
    assert to_host(p).tolist() == [0, 0, 0, 0]
    p = rb.sorted_idxs_to_compressed_ptr(torch.tensor([0, 0, 1, 7], device="cuda"), 3)
    assert to_host(p).tolist() == [0, 2, 3, 3]
