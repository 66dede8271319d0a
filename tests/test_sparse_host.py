"""Host-side parts of the sparse-data API, CPU only: the transpose views of
sparse_data/conversions.hh:128-166 (shapes swapped, arrays shared unless copied, sort flags
swapped), NonzeroSort's values against the C header, and COOMatrix.deepcopy."""
import os
import re

import torch

import randblas_gb300 as rb

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "randblas_gb300.h")


def _coo():
    return rb.COOMatrix(3, 5, torch.tensor([1.0, 2.0, 3.0]), torch.tensor([0, 1, 2]),
                        torch.tensor([4, 0, 3]), rb.NonzeroSort.CSR)


def test_transpose_views():
    A = rb.CSRMatrix(3, 5, torch.tensor([1.0, 2.0]), torch.tensor([0, 1, 1, 2]),
                     torch.tensor([4, 0]))
    At = rb.transpose_as_csc(A)
    assert (At.n_rows, At.n_cols) == (5, 3)
    assert At.colptr is A.rowptr and At.rowidxs is A.colidxs and At.vals is A.vals
    Ac = rb.transpose_as_csc(A, share_memory=False)
    assert Ac.vals.data_ptr() != A.vals.data_ptr() and torch.equal(Ac.vals, A.vals)
    Att = rb.transpose_as_csr(At)
    assert (Att.n_rows, Att.n_cols) == (3, 5) and Att.rowptr is A.rowptr
    C = _coo()
    Ct = rb.transpose_as_coo(C)
    assert (Ct.n_rows, Ct.n_cols) == (5, 3) and Ct.sort == rb.NonzeroSort.CSC
    assert Ct.rows is C.cols and Ct.cols is C.rows
    C.sort = rb.NonzeroSort.NONE
    assert rb.transpose_as_coo(C).sort == rb.NonzeroSort.NONE


def test_nonzero_sort_matches_header():
    text = open(HEADER).read()
    m = re.search(r"RBG_SORT_CSC = '(.)', RBG_SORT_CSR = '(.)', RBG_SORT_NONE = '(.)'", text)
    assert m, "NonzeroSort values not found in the header"
    assert (rb.NonzeroSort.CSC, rb.NonzeroSort.CSR, rb.NonzeroSort.NONE) == tuple(
        ord(c) for c in m.groups())


def test_coo_deepcopy_is_independent():
    C = _coo()
    D = C.deepcopy()
    D.rows[0] = 7
    D.vals[1] = -1.0
    assert C.rows[0] == 0 and C.vals[1] == 2.0 and D.sort == C.sort
