"""Python mirror of RandBLAS's sketching API over the C ABI.

Names, argument order and meaning follow the reference (RandBLAS/base.hh, dense_skops.hh,
sparse_skops.hh, skge.hh, skve.hh, sparse_data/sksp.hh); matrices are CUDA ``torch``
tensors addressed through their data pointers with the BLAS-style layout / leading-dimension
arguments the reference takes.  Calls run on the current torch CUDA stream.  Failed
argument checks raise :class:`RandBLASError` carrying the reference's message
("(cond) was required, but did not hold, in function f").
"""
from __future__ import annotations

import ctypes as C
import warnings
from dataclasses import dataclass, field
from enum import IntEnum
from typing import Optional

import torch

from . import _lib
from ._lib import RandBLASError, call


class Layout(IntEnum):
    ColMajor = _lib.COL_MAJOR
    RowMajor = _lib.ROW_MAJOR


class Op(IntEnum):
    NoTrans = _lib.NO_TRANS
    Trans = _lib.TRANS


class ScalarDist(IntEnum):
    Gaussian = _lib.GAUSSIAN
    Uniform = _lib.UNIFORM


class Axis(IntEnum):
    Short = _lib.AXIS_SHORT
    Long = _lib.AXIS_LONG


_DT = {torch.float32: _lib.F32, torch.float64: _lib.F64}
_IT = {torch.int32: _lib.I32, torch.int64: _lib.I64}


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: Optional[torch.Tensor]):
    if t is None:
        return None
    if not t.is_cuda:
        raise RandBLASError(_lib.ERROR_INVALID_ARGUMENT, "buffers must be CUDA tensors")
    return C.c_void_p(t.data_ptr())


def _ptr_device_or_pinned(t: Optional[torch.Tensor]):
    """A CUDA tensor, or a CPU tensor in pinned memory (for calls that read and write host
    memory over the host link)."""
    if t is None:
        return None
    if not t.is_cuda and not t.is_pinned():
        raise RandBLASError(_lib.ERROR_INVALID_ARGUMENT,
                            "buffers must be CUDA tensors or pinned CPU tensors")
    return C.c_void_p(t.data_ptr())


def set_deterministic(on: bool) -> None:
    """Process-wide reproducibility switch (no reference counterpart): when on, every path
    adds in a fixed order; when off (default) the SASO shared-memory scatter (column-major data
    or d > 2048) and entries moved out of fill_sparse's layout in a pre-filled operator may vary
    in their last bits between runs."""
    call("rbg_set_deterministic", 1 if on else 0)


def deterministic() -> bool:
    return bool(_lib.lib().rbg_get_deterministic())


# ------------------------------------------------------------------------- RNGState
class RNGState:
    """RNGState<Philox4x32> (RandBLAS/base.hh:64-164): 128-bit counter, 64-bit key."""

    def __init__(self, key: int = 0, counter=(0, 0, 0, 0), key_words=None):
        self.counter = [int(c) & 0xFFFFFFFF for c in counter]
        if key_words is not None:
            self.key = [int(k) & 0xFFFFFFFF for k in key_words]
        else:
            s = _lib.rbg_state()
            call("rbg_state_from_key", C.c_uint64(int(key) & (2**64 - 1)), C.byref(s))
            self.key = list(s.key)

    @classmethod
    def _from_c(cls, s: "_lib.rbg_state") -> "RNGState":
        return cls(counter=list(s.counter), key_words=list(s.key))

    def _c(self) -> "_lib.rbg_state":
        s = _lib.rbg_state()
        for i in range(4):
            s.counter[i] = self.counter[i]
        for i in range(2):
            s.key[i] = self.key[i]
        return s

    def incr(self, n: int) -> "RNGState":
        out = _lib.rbg_state()
        call("rbg_state_incr", C.byref(self._c()), C.c_uint64(n), C.byref(out))
        return RNGState._from_c(out)

    def __eq__(self, other) -> bool:
        return isinstance(other, RNGState) and self.counter == other.counter and \
            self.key == other.key

    def __repr__(self) -> str:
        return f"RNGState(counter={self.counter}, key={self.key})"


# ------------------------------------------------------------------------- dense
class DenseDist:
    """DenseDist (RandBLAS/dense_skops.hh:231-350)."""

    def __init__(self, n_rows: int, n_cols: int, family: ScalarDist = ScalarDist.Gaussian,
                 major_axis: Axis = Axis.Long):
        self.n_rows, self.n_cols = int(n_rows), int(n_cols)
        self.family, self.major_axis = ScalarDist(family), Axis(major_axis)
        dm, dn, nl, sc = C.c_int64(), C.c_int64(), C.c_int32(), C.c_double()
        call("rbg_dense_dist_properties", C.byref(self._c()), C.byref(dm), C.byref(dn),
             C.byref(nl), C.byref(sc))
        self.dim_major, self.dim_minor = dm.value, dn.value
        self.natural_layout = Layout(nl.value)
        self.isometry_scale = sc.value

    def _c(self) -> "_lib.rbg_dense_dist":
        return _lib.rbg_dense_dist(self.n_rows, self.n_cols, int(self.family),
                                   int(self.major_axis))


class DenseSkOp:
    """DenseSkOp<T> (RandBLAS/dense_skops.hh:357-478).  ``buff`` stays None until
    fill_dense(S); sketching with an unfilled operator generates its entries in-kernel."""

    def __init__(self, dist: DenseDist, seed_state: RNGState, dtype=torch.float32):
        if dtype not in _DT:
            raise RandBLASError(_lib.ERROR_INVALID_ARGUMENT, "dtype must be float32 or float64")
        self.dist, self.seed_state, self.dtype = dist, seed_state, dtype
        nxt = _lib.rbg_state()
        call("rbg_dense_next_state", C.byref(dist._c()), C.byref(seed_state._c()), C.byref(nxt))
        self.next_state = RNGState._from_c(nxt)
        self.n_rows, self.n_cols = dist.n_rows, dist.n_cols
        self.layout = dist.natural_layout
        self.buff: Optional[torch.Tensor] = None
        self.own_memory = True

    def _c(self) -> "_lib.rbg_dense_skop":
        s = _lib.rbg_dense_skop()
        s.dist = self.dist._c()
        s.seed_state = self.seed_state._c()
        s.next_state = self.next_state._c()
        s.dtype = _DT[self.dtype]
        s.layout = int(self.layout)
        s.buff = self.buff.data_ptr() if self.buff is not None else None
        return s


def fill_dense_unpacked(layout: Layout, D: DenseDist, n_rows: int, n_cols: int, ro_s: int,
                        co_s: int, buff: torch.Tensor, seed: RNGState) -> RNGState:
    """fill_dense_unpacked (RandBLAS/dense_skops.hh:563-606)."""
    nxt = _lib.rbg_state()
    call("rbg_fill_dense_unpacked", _DT[buff.dtype], int(layout), C.byref(D._c()), n_rows,
         n_cols, ro_s, co_s, _ptr(buff), C.byref(seed._c()), C.byref(nxt), _stream())
    return RNGState._from_c(nxt)


def fill_dense(D_or_S, buff: Optional[torch.Tensor] = None, seed: Optional[RNGState] = None):
    """fill_dense(D, buff, seed) -> next state (dense_skops.hh:623-626), or fill_dense(S)
    (dense_skops.hh:649-658), which allocates S.buff when S owns its memory."""
    if isinstance(D_or_S, DenseSkOp):
        S = D_or_S
        if S.buff is None:
            if not S.own_memory:
                raise RandBLASError(_lib.ERROR_INVALID_ARGUMENT,
                                    "(S.buff != nullptr) was required, but did not hold, in "
                                    "function fill_dense")
            S.buff = torch.empty(S.n_rows * S.n_cols, dtype=S.dtype, device="cuda")
        call("rbg_fill_dense_skop", C.byref(S._c()), _stream())
        return None
    D = D_or_S
    nxt = _lib.rbg_state()
    call("rbg_fill_dense", _DT[buff.dtype], C.byref(D._c()), _ptr(buff), C.byref(seed._c()),
         C.byref(nxt), _stream())
    return RNGState._from_c(nxt)


# ------------------------------------------------------------------------- sparse
class SparseDist:
    """SparseDist (RandBLAS/sparse_skops.hh:131-246)."""

    def __init__(self, n_rows: int, n_cols: int, vec_nnz: int = 4,
                 major_axis: Axis = Axis.Short):
        self.n_rows, self.n_cols, self.vec_nnz = int(n_rows), int(n_cols), int(vec_nnz)
        self.major_axis = Axis(major_axis)
        dm, dn, fn, sc = C.c_int64(), C.c_int64(), C.c_int64(), C.c_double()
        call("rbg_sparse_dist_properties", C.byref(self._c()), C.byref(dm), C.byref(dn),
             C.byref(fn), C.byref(sc))
        self.dim_major, self.dim_minor, self.full_nnz = dm.value, dn.value, fn.value
        self.isometry_scale = sc.value

    def _c(self) -> "_lib.rbg_sparse_dist":
        return _lib.rbg_sparse_dist(self.n_rows, self.n_cols, self.vec_nnz,
                                    int(self.major_axis), 0)


class SparseSkOp:
    """SparseSkOp<T, RNG, sint_t> (RandBLAS/sparse_skops.hh:289-450); nnz = -1 until
    sampled."""

    def __init__(self, dist: SparseDist, seed_state: RNGState, dtype=torch.float32,
                 index_dtype=torch.int64):
        self.dist, self.seed_state = dist, seed_state
        self.dtype, self.index_dtype = dtype, index_dtype
        nxt = _lib.rbg_state()
        call("rbg_sparse_next_state", C.byref(dist._c()), C.byref(seed_state._c()),
             C.byref(nxt))
        self.next_state = RNGState._from_c(nxt)
        self.n_rows, self.n_cols = dist.n_rows, dist.n_cols
        self.nnz = -1
        self.vals = self.rows = self.cols = None
        self.own_memory = True

    def _c(self) -> "_lib.rbg_sparse_skop":
        s = _lib.rbg_sparse_skop()
        s.dist = self.dist._c()
        s.seed_state = self.seed_state._c()
        s.next_state = self.next_state._c()
        s.nnz = self.nnz
        s.dtype = _DT[self.dtype]
        s.itype = _IT[self.index_dtype]
        s.vals = self.vals.data_ptr() if self.vals is not None else None
        s.rows = self.rows.data_ptr() if self.rows is not None else None
        s.cols = self.cols.data_ptr() if self.cols is not None else None
        return s


def fill_sparse(S: SparseSkOp) -> None:
    """fill_sparse(S) (RandBLAS/sparse_skops.hh:587-603)."""
    n = S.dist.full_nnz
    if S.own_memory:
        if S.rows is None:
            S.rows = torch.empty(n, dtype=S.index_dtype, device="cuda")
        if S.cols is None:
            S.cols = torch.empty(n, dtype=S.index_dtype, device="cuda")
        if S.vals is None:
            S.vals = torch.empty(n, dtype=S.dtype, device="cuda")
    cs = S._c()
    call("rbg_fill_sparse", C.byref(cs), _stream())
    S.nnz = cs.nnz


def fill_sparse_unpacked_nosub(D: SparseDist, vals, rows, cols, seed: RNGState):
    """fill_sparse_unpacked_nosub (RandBLAS/sparse_skops.hh:515-565) -> (nnz, next state)."""
    nnz = C.c_int64()
    nxt = _lib.rbg_state()
    call("rbg_fill_sparse_unpacked_nosub", _DT[vals.dtype], _IT[rows.dtype], C.byref(D._c()),
         C.byref(nnz), _ptr(vals), _ptr(rows), _ptr(cols), C.byref(seed._c()), C.byref(nxt),
         _stream())
    return nnz.value, RNGState._from_c(nxt)


def repeated_fisher_yates(k: int, n: int, r: int, samples: torch.Tensor,
                          state: RNGState) -> RNGState:
    """repeated_fisher_yates(k, n, r, samples, state) (RandBLAS/sparse_skops.hh:259-264)."""
    nxt = _lib.rbg_state()
    call("rbg_repeated_fisher_yates", k, n, r, _ptr(samples), C.byref(state._c()),
         C.byref(nxt), _stream())
    return RNGState._from_c(nxt)


# ------------------------------------------------------------------------- sparse data
class NonzeroSort(IntEnum):
    """NonzeroSort (sparse_data/base.hh:108-117); NONE stands for the reference's None."""
    CSC = ord("C")
    CSR = ord("R")
    NONE = ord("N")


@dataclass
class COOMatrix:
    n_rows: int
    n_cols: int
    vals: torch.Tensor
    rows: torch.Tensor
    cols: torch.Tensor
    sort: NonzeroSort = NonzeroSort.NONE

    def _c(self):
        return _spmat(_lib.COO, self.n_rows, self.n_cols, self.vals, self.rows, self.cols)

    def sort_arrays(self, s: NonzeroSort) -> None:
        """COOMatrix::sort_arrays (sparse_data/coo_matrix.hh:222-226): sort the entries into
        CSR or CSC order in place (equal (row, col) entries keep their order)."""
        k = self.vals.numel()
        call("rbg_coo_apply_sort", int(s), _DT[self.vals.dtype], _IT[self.rows.dtype], k,
             _ptr(self.vals) if k else None, _ptr(self.rows) if k else None,
             _ptr(self.cols) if k else None, _stream())
        if s != NonzeroSort.NONE:
            self.sort = NonzeroSort(s)

    def deepcopy(self) -> "COOMatrix":
        return COOMatrix(self.n_rows, self.n_cols, self.vals.clone(), self.rows.clone(),
                         self.cols.clone(), self.sort)


@dataclass
class CSRMatrix:
    n_rows: int
    n_cols: int
    vals: torch.Tensor
    rowptr: torch.Tensor
    colidxs: torch.Tensor

    def _c(self):
        return _spmat(_lib.CSR, self.n_rows, self.n_cols, self.vals, self.rowptr, self.colidxs)


@dataclass
class CSCMatrix:
    n_rows: int
    n_cols: int
    vals: torch.Tensor
    rowidxs: torch.Tensor
    colptr: torch.Tensor

    def _c(self):
        return _spmat(_lib.CSC, self.n_rows, self.n_cols, self.vals, self.colptr, self.rowidxs)


def _spmat(fmt, n_rows, n_cols, vals, a, b):
    m = _lib.rbg_spmat()
    m.format = fmt
    m.dtype = _DT[vals.dtype]
    m.itype = _IT[b.dtype]
    m.n_rows, m.n_cols, m.nnz = n_rows, n_cols, vals.numel()
    m.vals = vals.data_ptr() if vals.numel() else None
    m.idx_a = a.data_ptr() if a.numel() else None
    m.idx_b = b.data_ptr() if b.numel() else None
    return m


# ------------------------------------------------------------------ sparse data conversions
def coo_arrays_determine_sort(rows: torch.Tensor, cols: torch.Tensor) -> NonzeroSort:
    """coo_arrays_determine_sort (sparse_data/base.hh:142-167)."""
    out = C.c_int32()
    k = rows.numel()
    call("rbg_coo_determine_sort", _IT[rows.dtype], k, _ptr(rows) if k else None,
         _ptr(cols) if k else None, C.byref(out), _stream())
    return NonzeroSort(out.value)


def compressed_ptr_to_sorted_idxs(ptr: torch.Tensor, len_idxs: int, dtype=None) -> torch.Tensor:
    """compressed_ptr_to_sorted_idxs (sparse_data/base.hh:292-302): a new index tensor of
    len_idxs entries (those past ptr[-1] - ptr[0] are zero)."""
    dtype = dtype or ptr.dtype
    idxs = torch.zeros(len_idxs, dtype=dtype, device=ptr.device)
    call("rbg_compressed_ptr_to_sorted_idxs", ptr.numel() - 1, _IT[ptr.dtype], _ptr(ptr),
         len_idxs, _IT[dtype], _ptr(idxs) if len_idxs else None, _stream())
    return idxs


def sorted_idxs_to_compressed_ptr(idxs: torch.Tensor, num_comp: int, dtype=None) -> torch.Tensor:
    """sorted_idxs_to_compressed_ptr (sparse_data/base.hh:278-290): a new pointer tensor of
    num_comp + 1 entries."""
    dtype = dtype or idxs.dtype
    ptr = torch.empty(num_comp + 1, dtype=dtype, device=idxs.device)
    k = idxs.numel()
    call("rbg_sorted_idxs_to_compressed_ptr", k, _IT[idxs.dtype], _ptr(idxs) if k else None,
         num_comp, _IT[dtype], _ptr(ptr), _stream())
    return ptr


def csr_to_coo(A: "CSRMatrix") -> COOMatrix:
    """csr_to_coo (sparse_data/conversions.hh:63-75): a new COOMatrix in CSR order."""
    k = A.vals.numel()
    rows = compressed_ptr_to_sorted_idxs(A.rowptr, k, A.colidxs.dtype)
    return COOMatrix(A.n_rows, A.n_cols, A.vals.clone(), rows, A.colidxs.clone(),
                     NonzeroSort.CSR)


def csc_to_coo(A: "CSCMatrix") -> COOMatrix:
    """csc_to_coo (sparse_data/conversions.hh:49-61): a new COOMatrix in CSC order."""
    k = A.vals.numel()
    cols = compressed_ptr_to_sorted_idxs(A.colptr, k, A.rowidxs.dtype)
    return COOMatrix(A.n_rows, A.n_cols, A.vals.clone(), A.rowidxs.clone(), cols,
                     NonzeroSort.CSC)


def coo_to_csr(A: COOMatrix) -> "CSRMatrix":
    """coo_to_csr (sparse_data/conversions.hh:101-121): a new CSRMatrix.  As in the reference,
    A.sort == CSR is trusted; otherwise a sorted copy of A is compressed."""
    B = A if A.sort == NonzeroSort.CSR else A.deepcopy()
    if B is not A:
        B.sort_arrays(NonzeroSort.CSR)
    rowptr = sorted_idxs_to_compressed_ptr(B.rows, A.n_rows)
    return CSRMatrix(A.n_rows, A.n_cols, B.vals if B is not A else A.vals.clone(), rowptr,
                     B.cols if B is not A else A.cols.clone())


def coo_to_csc(A: COOMatrix) -> "CSCMatrix":
    """coo_to_csc (sparse_data/conversions.hh:79-99): a new CSCMatrix."""
    B = A if A.sort == NonzeroSort.CSC else A.deepcopy()
    if B is not A:
        B.sort_arrays(NonzeroSort.CSC)
    colptr = sorted_idxs_to_compressed_ptr(B.cols, A.n_cols)
    return CSCMatrix(A.n_rows, A.n_cols, B.vals if B is not A else A.vals.clone(),
                     B.rows if B is not A else A.rows.clone(), colptr)


def transpose_as_csr(A: "CSCMatrix", share_memory: bool = True) -> "CSRMatrix":
    """transpose_as_csr (sparse_data/conversions.hh:128-136): A^T as CSR over A's arrays."""
    c = (lambda t: t) if share_memory else (lambda t: t.clone())
    return CSRMatrix(A.n_cols, A.n_rows, c(A.vals), c(A.colptr), c(A.rowidxs))


def transpose_as_csc(A: "CSRMatrix", share_memory: bool = True) -> "CSCMatrix":
    """transpose_as_csc (sparse_data/conversions.hh:138-146): A^T as CSC over A's arrays."""
    c = (lambda t: t) if share_memory else (lambda t: t.clone())
    return CSCMatrix(A.n_cols, A.n_rows, c(A.vals), c(A.colidxs), c(A.rowptr))


def transpose_as_coo(A: COOMatrix, share_memory: bool = True) -> COOMatrix:
    """transpose_as_coo (sparse_data/conversions.hh:148-166): rows and cols swapped, the sort
    flag swapped with them."""
    c = (lambda t: t) if share_memory else (lambda t: t.clone())
    flip = {NonzeroSort.CSC: NonzeroSort.CSR, NonzeroSort.CSR: NonzeroSort.CSC}
    return COOMatrix(A.n_cols, A.n_rows, c(A.vals), c(A.cols), c(A.rows),
                     flip.get(A.sort, NonzeroSort.NONE))


# ------------------------------------------------------------------ random sparse matrices
def _random_sparse(fmt, m: int, n: int, density: float, state: RNGState, dtype, itype):
    if dtype not in _DT or itype not in _IT:
        raise RandBLASError(_lib.ERROR_INVALID_ARGUMENT,
                            "dtype must be float32/float64 and itype int32/int64")
    h = C.c_void_p()
    nnz = C.c_int64()
    nxt = _lib.rbg_state()
    call("rbg_random_sparse_create", fmt, m, n, float(density), C.byref(state._c()),
         C.byref(h), C.byref(nnz), C.byref(nxt), _stream())
    try:
        dev = torch.device("cuda", torch.cuda.current_device())
        k = nnz.value
        nmaj = n if fmt == _lib.CSC else m
        vals = torch.empty(k, dtype=dtype, device=dev)
        a = torch.empty(k if fmt == _lib.COO else nmaj + 1, dtype=itype, device=dev)
        b = torch.empty(k, dtype=itype, device=dev)
        call("rbg_random_sparse_fill", h, _DT[dtype], _IT[itype], _ptr(vals) if k else None,
             _ptr(a) if a.numel() else None, _ptr(b) if k else None, _stream())
        ties = C.c_int64()
        call("rbg_random_sparse_info", h, C.byref(ties), None)
        if ties.value:
            warnings.warn(f"{ties.value} geometric skip(s) fell within 2^-48 of an integer; "
                          "the reference's host logarithm may round them differently")
    finally:
        call("rbg_random_sparse_destroy", h)
    return vals, a, b, RNGState._from_c(nxt)


def random_csr(m: int, n: int, density: float, state: RNGState, dtype=torch.float64,
               itype=torch.int64):
    """random_csr<T, sint_t>(m, n, density, state) (sparse_data/random_matrix.hh:135-207):
    returns (CSRMatrix, next_state); each entry is present with probability `density`,
    values standard Gaussian."""
    vals, rowptr, colidxs, nxt = _random_sparse(_lib.CSR, m, n, density, state, dtype, itype)
    return CSRMatrix(m, n, vals, rowptr, colidxs), nxt


def random_csc(m: int, n: int, density: float, state: RNGState, dtype=torch.float64,
               itype=torch.int64):
    """random_csc<T, sint_t>(m, n, density, state) (sparse_data/random_matrix.hh:217-285)."""
    vals, colptr, rowidxs, nxt = _random_sparse(_lib.CSC, m, n, density, state, dtype, itype)
    return CSCMatrix(m, n, vals, rowidxs, colptr), nxt


def random_coo(m: int, n: int, density: float, state: RNGState, dtype=torch.float64,
               itype=torch.int64):
    """random_coo<T, sint_t>(m, n, density, state) (sparse_data/random_matrix.hh:296-355):
    entries in CSR order."""
    vals, rows, cols, nxt = _random_sparse(_lib.COO, m, n, density, state, dtype, itype)
    return COOMatrix(m, n, vals, rows, cols, NonzeroSort.CSR), nxt


# ------------------------------------------------------------------------- sketching
def _is_skop(x) -> bool:
    return isinstance(x, (DenseSkOp, SparseSkOp))


def sketch_general(layout: Layout, op1: Op, op2: Op, a: int, b: int, c: int, alpha: float,
                   *args) -> None:
    """sketch_general (RandBLAS/skge.hh:756-1199).  The side follows the argument order, as in
    the reference:

    * left:  sketch_general(layout, opS, opA, d, n, m, alpha, S, [ro_s, co_s,] A, lda, beta, B,
      ldb) computes B = alpha * op(submat(S)) * op(A) + beta * B;
    * right: sketch_general(layout, opA, opS, m, d, n, alpha, A, lda, S, [ro_s, co_s,] beta, B,
      ldb) computes B = alpha * op(A) * op(submat(S)) + beta * B.
    """
    st = _stream()
    if _is_skop(args[0]):  # left
        S = args[0]
        if len(args) == 8:
            ro_s, co_s, A, lda, beta, B, ldb = args[1:]
        else:
            A, lda, beta, B, ldb = args[1:]
            ro_s = co_s = 0
            d, m = a, c
            rows, cols = (d, m) if Op(op1) == Op.NoTrans else (m, d)
            if S.n_rows != rows or S.n_cols != cols:
                raise RandBLASError(
                    _lib.ERROR_INVALID_ARGUMENT,
                    f"(S.n_rows == {rows} && S.n_cols == {cols}) was required, but did not "
                    "hold, in function sketch_general")
        fn = "rbg_lskge3" if isinstance(S, DenseSkOp) else "rbg_lskges"
        call(fn, int(layout), int(op1), int(op2), a, b, c, float(alpha), C.byref(S._c()), ro_s,
             co_s, _ptr(A), lda, float(beta), _ptr(B), ldb, st)
        return
    A, lda, S = args[0], args[1], args[2]
    if len(args) == 8:
        ro_s, co_s, beta, B, ldb = args[3:]
    else:
        beta, B, ldb = args[3:]
        ro_s = co_s = 0
        n, d = c, b
        rows, cols = (n, d) if Op(op2) == Op.NoTrans else (d, n)
        if S.n_rows != rows or S.n_cols != cols:
            raise RandBLASError(
                _lib.ERROR_INVALID_ARGUMENT,
                f"(S.n_rows == {rows} && S.n_cols == {cols}) was required, but did not hold, "
                "in function sketch_general")
    fn = "rbg_rskge3" if isinstance(S, DenseSkOp) else "rbg_rskges"
    call(fn, int(layout), int(op1), int(op2), a, b, c, float(alpha), _ptr(A), lda,
         C.byref(S._c()), ro_s, co_s, float(beta), _ptr(B), ldb, st)


def require_symmetric(layout: Layout, A: torch.Tensor, n: int, lda: int, tol: float) -> None:
    """require_symmetric (RandBLAS/util.hh:128-146); raises RandBLASError with the reference's
    message on the first failing pair; no check when tol < 0.  Synchronises."""
    call("rbg_require_symmetric", _DT[A.dtype], int(layout), _ptr(A), n, lda, float(tol),
         _stream())


def sketch_symmetric(layout: Layout, *args) -> None:
    """sketch_symmetric (RandBLAS/sksy.hh:158-529); the side follows the argument order, as in
    the reference, and A is n x n symmetric (checked with sym_check_tol, default 0):

    * sketch_symmetric(layout, d, n, alpha, S, ro_s, co_s, A, lda, beta, B, ldb[, tol])
      -> B = alpha * submat(S) * A + beta * B  (d x n)
    * sketch_symmetric(layout, n, d, alpha, A, lda, S, ro_s, co_s, beta, B, ldb[, tol])
      -> B = alpha * A * submat(S) + beta * B  (n x d)
    * sketch_symmetric(layout, alpha, S, A, lda, beta, B, ldb[, tol])  (whole operator, left)
    * sketch_symmetric(layout, alpha, A, lda, S, beta, B, ldb[, tol])  (whole operator, right)
    """
    if len(args) in (11, 12):
        tol = float(args[11]) if len(args) == 12 else 0.0
        if _is_skop(args[3]):
            d, n, alpha, S, ro_s, co_s, A, lda, beta, B, ldb = args[:11]
            side = 0
        else:
            n, d, alpha, A, lda, S, ro_s, co_s, beta, B, ldb = args[:11]
            side = 1
    elif len(args) in (7, 8):
        tol = float(args[7]) if len(args) == 8 else 0.0
        if _is_skop(args[1]):
            alpha, S, A, lda, beta, B, ldb = args[:7]
            side, ro_s, co_s = 0, 0, 0
            d, n = S.n_rows, S.n_cols
        else:
            alpha, A, lda, S, beta, B, ldb = args[:7]
            side, ro_s, co_s = 1, 0, 0
            n, d = S.n_rows, S.n_cols
    else:
        raise RandBLASError(_lib.ERROR_INVALID_ARGUMENT, "unrecognised sketch_symmetric arguments")
    fn = "rbg_sketch_symmetric" if isinstance(S, DenseSkOp) else "rbg_sketch_symmetric_sparse"
    call(fn, side, int(layout), d, n, float(alpha), C.byref(S._c()), ro_s, co_s, _ptr(A), lda,
         float(beta), _ptr(B), ldb, tol, _stream())


def sketch_vector(opS: Op, *args) -> None:
    """sketch_vector (RandBLAS/skve.hh:140-164, 232-246):
    sketch_vector(opS, d, m, alpha, S, ro_s, co_s, x, incx, beta, y, incy) or
    sketch_vector(opS, alpha, S, x, incx, beta, y, incy)."""
    if len(args) == 11:
        d, m, alpha, S, ro_s, co_s, x, incx, beta, y, incy = args
    else:
        alpha, S, x, incx, beta, y, incy = args
        d, m, ro_s, co_s = S.dist.n_rows, S.dist.n_cols, 0, 0
    fn = "rbg_sketch_vector" if isinstance(S, DenseSkOp) else "rbg_sketch_vector_sparse"
    call(fn, int(opS), d, m, float(alpha), C.byref(S._c()), ro_s, co_s, _ptr(x), incx,
         float(beta), _ptr(y), incy, _stream())


def sketch_sparse(layout: Layout, op1: Op, op2: Op, a: int, b: int, c: int, alpha: float,
                  *args) -> None:
    """sketch_sparse (RandBLAS/sparse_data/sksp.hh:418-539): dense operator, sparse data.

    * left:  sketch_sparse(layout, opS, opA, d, n, m, alpha, S, ro_s, co_s, A, beta, B, ldb)
    * right: sketch_sparse(layout, opA, opS, m, d, n, alpha, A, S, ro_s, co_s, beta, B, ldb)
    """
    st = _stream()
    if isinstance(args[0], DenseSkOp):
        S, ro_s, co_s, A, beta, B, ldb = args
        call("rbg_lsksp3", int(layout), int(op1), int(op2), a, b, c, float(alpha),
             C.byref(S._c()), ro_s, co_s, C.byref(A._c()), float(beta), _ptr(B), ldb, st)
    else:
        A, S, ro_s, co_s, beta, B, ldb = args
        call("rbg_rsksp3", int(layout), int(op1), int(op2), a, b, c, float(alpha),
             C.byref(A._c()), C.byref(S._c()), ro_s, co_s, float(beta), _ptr(B), ldb, st)


def left_spmm(layout, opA, opB, d, n, m, alpha, A, ro_a, co_a, B, ldb, beta, C_, ldc) -> None:
    """left_spmm (RandBLAS/sparse_data/spmm_dispatch.hh:52-179)."""
    call("rbg_left_spmm", int(layout), int(opA), int(opB), d, n, m, float(alpha),
         C.byref(A._c()), ro_a, co_a, _ptr(B), ldb, float(beta), _ptr(C_), ldc, _stream())


def right_spmm(layout, opA, opB, m, d, n, alpha, A, lda, B, ro_b, co_b, beta, C_, ldc) -> None:
    """right_spmm (RandBLAS/sparse_data/spmm_dispatch.hh:181-219)."""
    call("rbg_right_spmm", int(layout), int(opA), int(opB), m, d, n, float(alpha), _ptr(A), lda,
         C.byref(B._c()), ro_b, co_b, float(beta), _ptr(C_), ldc, _stream())


def spmm(layout, opA, opB, m, n, k, alpha, A, *rest) -> None:
    """spmm (RandBLAS/sparse_data/spmm_dispatch.hh:298-302, 376-380); the sparse operand's
    position picks the side:
    spmm(layout, opA, opB, m, n, k, alpha, A_sparse, B, ldb, beta, C, ldc) or
    spmm(layout, opA, opB, m, n, k, alpha, A, lda, B_sparse, beta, C, ldc)."""
    if isinstance(A, (COOMatrix, CSRMatrix, CSCMatrix)):
        B, ldb, beta, C_, ldc = rest
        left_spmm(layout, opA, opB, m, n, k, alpha, A, 0, 0, B, ldb, beta, C_, ldc)
    else:
        lda, B, beta, C_, ldc = rest
        right_spmm(layout, opA, opB, m, n, k, alpha, A, lda, B, 0, 0, beta, C_, ldc)
