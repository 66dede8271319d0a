"""ctypes/numpy front end of the CPU oracle (test infrastructure only).

``Oracle`` wraps ``oracle/liboracle.so`` (the plain-C restatement, oracle/oracle.c);
``RefLib`` wraps ``oracle/_ref/librbref.so`` (the reference's own headers compiled against
project shims, present only where the reference tree is).  Only tests/, the smoke check
and bench.py's CPU baseline import this module; the product never does.

Conventions shared with the product's C ABI: layout 0 = ColMajor, 1 = RowMajor; op 0 =
NoTrans, 1 = Trans; family 0 = Gaussian, 1 = Uniform; axis 0 = Short, 1 = Long; dtype 0 =
float32, 1 = float64; itype 0 = int32, 1 = int64.  A state is (counter[4], key[2]) uint32.
"""
from __future__ import annotations

import contextlib
import ctypes as C
import glob
import os

import numpy as np

from . import build as _build

U32x4 = C.c_uint32 * 4
U32x2 = C.c_uint32 * 2
P = C.c_void_p
I64 = C.c_int64
INT = C.c_int


class State(C.Structure):
    _fields_ = [("counter", C.c_uint32 * 4), ("key", C.c_uint32 * 2)]

    @classmethod
    def make(cls, counter=(0, 0, 0, 0), key=(0, 0)):
        s = cls()
        for i in range(4):
            s.counter[i] = int(counter[i]) & 0xFFFFFFFF
        for i in range(2):
            s.key[i] = int(key[i]) & 0xFFFFFFFF
        return s

    @classmethod
    def from_key(cls, k: int):
        return cls.make((0, 0, 0, 0), (k & 0xFFFFFFFF, (k >> 32) & 0xFFFFFFFF))

    def tuple(self):
        return tuple(self.counter), tuple(self.key)

    def ctr_int(self) -> int:
        return sum(int(self.counter[i]) << (32 * i) for i in range(4))


def _np_dtype(dtype: int):
    return np.float32 if dtype == 0 else np.float64


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _it(dtype) -> int:
    return 0 if np.dtype(dtype) == np.int32 else 1


class Oracle:
    """The C restatement (oracle/oracle.c)."""

    def __init__(self, path: str | None = None):
        path = path or _build.build_oracle()
        self.lib = C.CDLL(path)
        L = self.lib
        L.orc_set_math.argtypes = [INT]
        L.orc_get_math.restype = INT
        L.orc_philox4x32_10.argtypes = [P, P, P]
        L.orc_ctr_add.argtypes = [P, C.c_uint64]
        L.orc_uneg11.argtypes = [C.c_uint32]
        L.orc_uneg11.restype = C.c_float
        L.orc_u01.argtypes = [C.c_uint32]
        L.orc_u01.restype = C.c_float
        L.orc_boxmuller.argtypes = [C.c_uint32, C.c_uint32, P, P]
        L.orc_natural_layout.argtypes = [INT, I64, I64]
        L.orc_natural_layout.restype = INT
        L.orc_dim_major.argtypes = [INT, I64, I64]
        L.orc_dim_major.restype = I64
        L.orc_fill_dense_unpacked.argtypes = [INT, INT, I64, I64, INT, INT, I64, I64, I64, I64,
                                              P, P, P]
        L.orc_fill_dense_unpacked.restype = INT
        L.orc_fill_dense_submat.argtypes = [INT, INT, I64, P, I64, I64, I64, P, I64, P]
        L.orc_dense_next_state.argtypes = [INT, I64, I64, P, P]
        L.orc_repeated_fisher_yates.argtypes = [INT, INT, P, I64, I64, I64, P, P, P, P]
        L.orc_repeated_fisher_yates.restype = INT
        L.orc_fill_sparse.argtypes = [INT, INT, I64, I64, I64, INT, P, P, P, P, P, P]
        L.orc_fill_sparse.restype = INT
        L.orc_sparse_next_state.argtypes = [INT, I64, I64, I64, P, P]
        L.orc_random_sparse.argtypes = [INT, INT, INT, I64, I64, C.c_double, P, I64, P, P, P, P]
        L.orc_random_sparse.restype = I64
        L.orc_compressed_ptr_to_sorted_idxs.argtypes = [I64, INT, P, I64, INT, P]
        L.orc_compressed_ptr_to_sorted_idxs.restype = INT
        L.orc_sorted_idxs_to_compressed_ptr.argtypes = [I64, INT, P, I64, INT, P]
        L.orc_sorted_idxs_to_compressed_ptr.restype = INT
        L.orc_coo_determine_sort.argtypes = [INT, I64, P, P]
        L.orc_coo_determine_sort.restype = INT
        L.orc_coo_apply_sort.argtypes = [INT, INT, INT, I64, P, P, P]
        L.orc_coo_apply_sort.restype = INT

    # -- RNG ------------------------------------------------------------------------
    def set_math(self, mode: int) -> None:
        """Box-Muller's sin / cos / log: 0 = host libm (as the reference), 1 = the shared
        float-float specification the GPU evaluates (bit-for-bit comparisons)."""
        self.lib.orc_set_math(mode)

    @contextlib.contextmanager
    def shared_math(self):
        """Run a block with the shared math functions, then restore the previous mode."""
        prev = self.lib.orc_get_math()
        self.lib.orc_set_math(1)
        try:
            yield self
        finally:
            self.lib.orc_set_math(prev)

    def philox(self, counter, key) -> tuple:
        c, k, o = U32x4(*counter), U32x2(*key), U32x4()
        self.lib.orc_philox4x32_10(C.addressof(c), C.addressof(k), C.addressof(o))
        return tuple(o)

    def ctr_add(self, counter, n: int) -> tuple:
        c = U32x4(*counter)
        self.lib.orc_ctr_add(C.addressof(c), n)
        return tuple(c)

    def uneg11(self, u: int) -> float:
        return self.lib.orc_uneg11(u)

    def u01(self, u: int) -> float:
        return self.lib.orc_u01(u)

    def boxmuller(self, u0: int, u1: int):
        a, b = C.c_float(), C.c_float()
        self.lib.orc_boxmuller(u0, u1, C.addressof(a), C.addressof(b))
        return a.value, b.value

    # -- dense ----------------------------------------------------------------------
    def natural_layout(self, major_axis, n_rows, n_cols) -> int:
        return self.lib.orc_natural_layout(major_axis, n_rows, n_cols)

    def dim_major(self, major_axis, n_rows, n_cols) -> int:
        return self.lib.orc_dim_major(major_axis, n_rows, n_cols)

    def fill_dense_unpacked(self, dtype, layout, D_rows, D_cols, family, major_axis, n_rows,
                            n_cols, ro_s, co_s, seed: State):
        """Returns (buffer as a 1-D array in `layout`, next State)."""
        buf = np.zeros(n_rows * n_cols, dtype=_np_dtype(dtype))
        nxt = State()
        rc = self.lib.orc_fill_dense_unpacked(dtype, layout, D_rows, D_cols, family, major_axis,
                                              n_rows, n_cols, ro_s, co_s, _ptr(buf),
                                              C.addressof(seed), C.addressof(nxt))
        if rc:
            raise ValueError(f"orc_fill_dense_unpacked failed ({rc})")
        return buf, nxt

    def fill_dense_submat(self, dtype, family, n_cols, n_srows, n_scols, ptr, seed: State):
        """dense::fill_dense_submat_impl (dense_skops.hh:96-170): raw transform values (no
        uniform scaling), row-major n_srows x n_scols -> (array, next State)."""
        buf = np.zeros(n_srows * n_scols, dtype=_np_dtype(dtype))
        nxt = State()
        self.lib.orc_fill_dense_submat(dtype, family, n_cols, _ptr(buf), n_srows, n_scols, ptr,
                                       C.addressof(seed), 0, C.addressof(nxt))
        return buf, nxt

    def dense_matrix(self, dtype, D_rows, D_cols, family, major_axis, seed: State,
                     n_rows=None, n_cols=None, ro_s=0, co_s=0) -> np.ndarray:
        """The (sub)matrix as a 2-D numpy array (row-major view)."""
        n_rows = D_rows if n_rows is None else n_rows
        n_cols = D_cols if n_cols is None else n_cols
        buf, _ = self.fill_dense_unpacked(dtype, 1, D_rows, D_cols, family, major_axis, n_rows,
                                          n_cols, ro_s, co_s, seed)
        return buf.reshape(n_rows, n_cols)

    def dense_next_state(self, major_axis, D_rows, D_cols, seed: State) -> State:
        nxt = State()
        self.lib.orc_dense_next_state(major_axis, D_rows, D_cols, C.addressof(seed),
                                      C.addressof(nxt))
        return nxt

    # -- sparse ---------------------------------------------------------------------
    def fill_sparse(self, dtype, itype, D_rows, D_cols, vec_nnz, major_axis, seed: State):
        """Returns (vals, rows, cols, nnz, next State); arrays trimmed to nnz."""
        full = vec_nnz * max(D_rows, D_cols) if major_axis == 0 else vec_nnz * min(D_rows, D_cols)
        it = np.int32 if itype == 0 else np.int64
        vals = np.zeros(full, _np_dtype(dtype))
        rows = np.zeros(full, it)
        cols = np.zeros(full, it)
        nnz = C.c_int64()
        nxt = State()
        rc = self.lib.orc_fill_sparse(dtype, itype, D_rows, D_cols, vec_nnz, major_axis,
                                      _ptr(vals), _ptr(rows), _ptr(cols), C.addressof(nnz),
                                      C.addressof(seed), C.addressof(nxt))
        if rc:
            raise ValueError(f"orc_fill_sparse failed ({rc})")
        k = nnz.value
        return vals[:k], rows[:k], cols[:k], k, nxt

    def repeated_fisher_yates(self, k, n, r, seed: State):
        """r independent k-subsets of {0..n-1} (sparse_skops.hh:51-106) -> (samples, next)."""
        samples = np.zeros(max(k * r, 1), np.int64)
        nxt = State()
        rc = self.lib.orc_repeated_fisher_yates(0, 1, C.addressof(seed), k, n, r, _ptr(samples),
                                                None, None, C.addressof(nxt))
        if rc:
            raise ValueError(f"orc_repeated_fisher_yates failed ({rc})")
        return samples[:k * r], nxt

    def sparse_next_state(self, major_axis, D_rows, D_cols, vec_nnz, seed: State) -> State:
        nxt = State()
        self.lib.orc_sparse_next_state(major_axis, D_rows, D_cols, vec_nnz, C.addressof(seed),
                                       C.addressof(nxt))
        return nxt

    def random_sparse(self, fmt, dtype, itype, m, n, density, seed: State):
        """random_coo / random_csr / random_csc (fmt 0 / 1 / 2) -> (vals, a, b, next State).

        COO: a = rows, b = cols; CSR: a = rowptr, b = colidxs; CSC: a = colptr, b = rowidxs.
        """
        return _random_sparse(self.lib.orc_random_sparse, fmt, dtype, itype, m, n, density,
                              seed, lambda rc: ValueError(f"orc_random_sparse failed ({rc})"))

    # -- sparse conversions (sparse_data/base.hh:119-220, 278-302) -------------------
    def compressed_ptr_to_sorted_idxs(self, ptr: np.ndarray, len_idxs: int, idx_dtype):
        """-> idxs (len_idxs entries, those past ptr[-1] - ptr[0] zero); raises on a failed
        check (1: len_idxs < ptr[num_comp], 2: negative segment)."""
        idxs = np.zeros(max(len_idxs, 1), idx_dtype)
        rc = self.lib.orc_compressed_ptr_to_sorted_idxs(
            ptr.size - 1, _it(ptr.dtype), _ptr(ptr), len_idxs, _it(idx_dtype), _ptr(idxs))
        if rc:
            raise ValueError(f"compressed_ptr_to_sorted_idxs check {rc} failed")
        return idxs[:len_idxs]

    def sorted_idxs_to_compressed_ptr(self, idxs: np.ndarray, num_comp: int, ptr_dtype):
        ptr = np.zeros(num_comp + 1, ptr_dtype)
        rc = self.lib.orc_sorted_idxs_to_compressed_ptr(idxs.size, _it(idxs.dtype), _ptr(idxs),
                                                        num_comp, _it(ptr_dtype), _ptr(ptr))
        if rc:
            raise ValueError("sorted_idxs_to_compressed_ptr: indices not sorted")
        return ptr

    def coo_determine_sort(self, rows: np.ndarray, cols: np.ndarray) -> str:
        return chr(self.lib.orc_coo_determine_sort(_it(rows.dtype), rows.size, _ptr(rows),
                                                   _ptr(cols)))

    def coo_apply_sort(self, sort: str, vals, rows, cols):
        """Sorts copies; returns (vals, rows, cols)."""
        vals, rows, cols = vals.copy(), rows.copy(), cols.copy()
        rc = self.lib.orc_coo_apply_sort(ord(sort), 0 if vals.dtype == np.float32 else 1,
                                         _it(rows.dtype), vals.size, _ptr(vals), _ptr(rows),
                                         _ptr(cols))
        if rc:
            raise MemoryError("orc_coo_apply_sort")
        return vals, rows, cols

    def sparse_dense_matrix(self, dtype, D_rows, D_cols, vec_nnz, major_axis, seed: State):
        vals, rows, cols, _, _ = self.fill_sparse(dtype, 1, D_rows, D_cols, vec_nnz, major_axis,
                                                  seed)
        S = np.zeros((D_rows, D_cols), dtype=np.float64)
        np.add.at(S, (rows, cols), vals.astype(np.float64))
        return S


def _random_sparse(fn, fmt, dtype, itype, m, n, density, seed, err, ref=False):
    it = np.int32 if itype == 0 else np.int64
    nmaj = n if fmt == 2 else m
    cap = 0
    while True:
        vals = np.zeros(max(cap, 1), _np_dtype(dtype))
        a = np.zeros(max(nmaj + 1 if fmt else cap, 1), it)
        b = np.zeros(max(cap, 1), it)
        nxt = State()
        if ref:
            nnz = C.c_int64()
            rc = fn(fmt, dtype, itype, m, n, density, C.addressof(seed.counter),
                    C.addressof(seed.key), cap, _ptr(vals), _ptr(a), _ptr(b), C.addressof(nnz),
                    C.addressof(nxt.counter), C.addressof(nxt.key))
            if rc:
                raise err(rc)
            k = nnz.value
        else:
            k = fn(fmt, dtype, itype, m, n, density, C.addressof(seed), cap, _ptr(vals), _ptr(a),
                   _ptr(b), C.addressof(nxt))
            if k < 0:
                raise err(k)
        if k <= cap:
            if fmt == 0:
                return vals[:k], a[:k], b[:k], nxt
            return vals[:k], a[:nmaj + 1] if nmaj > 0 else a[:0], b[:k], nxt
        cap = k


def find_cblas():
    """Addresses of the 64-bit-integer CBLAS sgemm/dgemm bundled with numpy (or None)."""
    import numpy
    libs = glob.glob(os.path.join(os.path.dirname(numpy.__file__) + ".libs", "*openblas*"))
    for path in libs:
        try:
            lib = C.CDLL(path)
            s = lib.scipy_cblas_sgemm64_
            d = lib.scipy_cblas_dgemm64_
            try:
                lib.scipy_openblas_set_num_threads64_.argtypes = [C.c_int]
                lib.scipy_openblas_set_num_threads64_(os.cpu_count() or 1)
            except AttributeError:
                pass
            return lib, C.cast(s, C.c_void_p).value, C.cast(d, C.c_void_p).value
        except (OSError, AttributeError):
            continue
    return None, None, None


class RefLib:
    """The reference's own headers compiled against the shims (oracle/_ref)."""

    def __init__(self, path: str | None = None, use_cblas: bool = True):
        path = path or _build.build_ref()
        if path is None:
            raise FileNotFoundError("reference tree not present; oracle/_ref not built")
        self.lib = C.CDLL(path)
        L = self.lib
        L.rbref_last_error.restype = C.c_char_p
        L.rbref_set_math.argtypes = [INT]
        L.rbref_set_cblas.argtypes = [P, P]
        self._blas = None
        if use_cblas:
            self._blas, s, d = find_cblas()
            if s:
                L.rbref_set_cblas(s, d)
        L.rbref_philox.argtypes = [P, P, P]
        L.rbref_state_from_key.argtypes = [C.c_uint64, P, P]
        L.rbref_counter_incr.argtypes = [P, C.c_uint64]
        L.rbref_fill_dense_unpacked.argtypes = [INT, INT, I64, I64, INT, INT, I64, I64, I64, I64,
                                                P, P, P, P, P]
        L.rbref_dense_next_state.argtypes = [I64, I64, INT, INT, P, P, P, P, P, P]
        L.rbref_fill_sparse.argtypes = [INT, INT, I64, I64, I64, INT, P, P, P, P, P, P, P, P]
        L.rbref_sparse_next_state.argtypes = [I64, I64, I64, INT, P, P, P, P]
        L.rbref_repeated_fisher_yates.argtypes = [I64, I64, I64, P, P, P, P, P]
        L.rbref_sketch_dense.argtypes = [INT, INT, INT, INT, INT, I64, I64, I64, C.c_double, I64,
                                         I64, INT, INT, P, P, I64, I64, P, I64, C.c_double, P,
                                         I64, INT]
        L.rbref_sketch_saso.argtypes = [INT, INT, INT, INT, INT, I64, I64, I64, C.c_double, I64,
                                        I64, I64, INT, P, P, I64, I64, P, I64, C.c_double, P, I64]
        L.rbref_sketch_vector.argtypes = [INT, INT, I64, I64, C.c_double, I64, I64, INT, INT, P,
                                          P, I64, I64, P, I64, C.c_double, P, I64]
        L.rbref_compressed_ptr_to_sorted_idxs.argtypes = [I64, INT, P, I64, INT, P]
        L.rbref_sorted_idxs_to_compressed_ptr.argtypes = [I64, INT, P, I64, INT, P]
        L.rbref_coo_determine_sort.argtypes = [INT, I64, P, P, P]
        L.rbref_coo_apply_sort.argtypes = [INT, INT, INT, I64, P, P, P]
        L.rbref_random_sparse.argtypes = [INT, INT, INT, I64, I64, C.c_double, P, P, I64, P, P,
                                          P, P, P, P]
        L.rbref_sketch_sparse.argtypes = [INT, INT, INT, INT, INT, I64, I64, I64, C.c_double,
                                          I64, I64, INT, INT, P, P, I64, I64, INT, I64, I64, I64,
                                          P, P, P, C.c_double, P, I64]
        D = C.c_double
        L.rbref_left_spmm.argtypes = [INT, INT, INT, INT, I64, I64, I64, D, INT, I64, I64, I64,
                                      P, P, P, I64, I64, P, I64, D, P, I64]
        L.rbref_right_spmm.argtypes = [INT, INT, INT, INT, I64, I64, I64, D, P, I64, INT, I64,
                                       I64, I64, P, P, P, I64, I64, D, P, I64]

    def set_math(self, mode: int) -> None:
        """Box-Muller's sin / cos / log in the reference's own code: 0 = host libm, 1 = the
        shared float-float specification."""
        self.lib.rbref_set_math(mode)

    def _check(self, rc):
        if rc:
            raise RuntimeError(f"reference error {rc}: {self.lib.rbref_last_error().decode()}")

    def compressed_ptr_to_sorted_idxs(self, ptr: np.ndarray, len_idxs: int, idx_dtype):
        idxs = np.zeros(max(len_idxs, 1), idx_dtype)
        self._check(self.lib.rbref_compressed_ptr_to_sorted_idxs(
            ptr.size - 1, _it(ptr.dtype), _ptr(ptr), len_idxs, _it(idx_dtype), _ptr(idxs)))
        return idxs[:len_idxs]

    def sorted_idxs_to_compressed_ptr(self, idxs: np.ndarray, num_comp: int, ptr_dtype):
        ptr = np.zeros(num_comp + 1, ptr_dtype)
        self._check(self.lib.rbref_sorted_idxs_to_compressed_ptr(
            idxs.size, _it(idxs.dtype), _ptr(idxs), num_comp, _it(ptr_dtype), _ptr(ptr)))
        return ptr

    def coo_determine_sort(self, rows: np.ndarray, cols: np.ndarray) -> str:
        out = C.c_int()
        self._check(self.lib.rbref_coo_determine_sort(_it(rows.dtype), rows.size, _ptr(rows),
                                                      _ptr(cols), C.addressof(out)))
        return chr(out.value)

    def coo_apply_sort(self, sort: str, vals, rows, cols):
        vals, rows, cols = vals.copy(), rows.copy(), cols.copy()
        self._check(self.lib.rbref_coo_apply_sort(ord(sort), 0 if vals.dtype == np.float32 else 1,
                                                  _it(rows.dtype), vals.size, _ptr(vals),
                                                  _ptr(rows), _ptr(cols)))
        return vals, rows, cols

    def random_sparse(self, fmt, dtype, itype, m, n, density, seed: State):
        """The reference's random_coo / random_csr / random_csc; same returns as Oracle's."""
        return _random_sparse(
            self.lib.rbref_random_sparse, fmt, dtype, itype, m, n, density, seed,
            lambda rc: RuntimeError(
                f"reference error {rc}: {self.lib.rbref_last_error().decode()}"), ref=True)

    def philox(self, counter, key):
        c, k, o = U32x4(*counter), U32x2(*key), U32x4()
        self.lib.rbref_philox(C.addressof(c), C.addressof(k), C.addressof(o))
        return tuple(o)

    def state_from_key(self, k: int) -> State:
        s = State()
        self.lib.rbref_state_from_key(k, C.addressof(s.counter), C.addressof(s.key))
        return s

    def counter_incr(self, counter, n: int):
        c = U32x4(*counter)
        self.lib.rbref_counter_incr(C.addressof(c), n)
        return tuple(c)

    def fill_dense_unpacked(self, dtype, layout, D_rows, D_cols, family, major_axis, n_rows,
                            n_cols, ro_s, co_s, seed: State):
        buf = np.zeros(n_rows * n_cols, dtype=_np_dtype(dtype))
        nxt = State()
        rc = self.lib.rbref_fill_dense_unpacked(dtype, layout, D_rows, D_cols, family,
                                                major_axis, n_rows, n_cols, ro_s, co_s, _ptr(buf),
                                                C.addressof(seed.counter), C.addressof(seed.key),
                                                C.addressof(nxt.counter), C.addressof(nxt.key))
        self._check(rc)
        return buf, nxt

    def dense_next_state(self, D_rows, D_cols, family, major_axis, seed: State):
        nxt = State()
        nl = C.c_int()
        dm = C.c_int64()
        rc = self.lib.rbref_dense_next_state(D_rows, D_cols, family, major_axis,
                                             C.addressof(seed.counter), C.addressof(seed.key),
                                             C.addressof(nxt.counter), C.addressof(nxt.key),
                                             C.addressof(nl), C.addressof(dm))
        self._check(rc)
        return nxt, nl.value, dm.value

    def fill_sparse(self, dtype, itype, D_rows, D_cols, vec_nnz, major_axis, seed: State):
        full = vec_nnz * max(D_rows, D_cols) if major_axis == 0 else vec_nnz * min(D_rows, D_cols)
        it = np.int32 if itype == 0 else np.int64
        vals = np.zeros(full, _np_dtype(dtype))
        rows = np.zeros(full, it)
        cols = np.zeros(full, it)
        nnz = C.c_int64()
        nxt = State()
        rc = self.lib.rbref_fill_sparse(dtype, itype, D_rows, D_cols, vec_nnz, major_axis,
                                        _ptr(vals), _ptr(rows), _ptr(cols), C.addressof(nnz),
                                        C.addressof(seed.counter), C.addressof(seed.key),
                                        C.addressof(nxt.counter), C.addressof(nxt.key))
        self._check(rc)
        k = nnz.value
        return vals[:k], rows[:k], cols[:k], k, nxt

    def sparse_next_state(self, D_rows, D_cols, vec_nnz, major_axis, seed: State) -> State:
        nxt = State()
        rc = self.lib.rbref_sparse_next_state(D_rows, D_cols, vec_nnz, major_axis,
                                              C.addressof(seed.counter), C.addressof(seed.key),
                                              C.addressof(nxt.counter), C.addressof(nxt.key))
        self._check(rc)
        return nxt

    def sketch_dense(self, dtype, side, layout, opS, opA, d, n, m, alpha, D_rows, D_cols, family,
                     major_axis, seed: State, ro_s, co_s, A: np.ndarray, lda, beta,
                     B: np.ndarray, ldb, prefill=False):
        rc = self.lib.rbref_sketch_dense(dtype, side, layout, opS, opA, d, n, m, alpha, D_rows,
                                         D_cols, family, major_axis, C.addressof(seed.counter),
                                         C.addressof(seed.key), ro_s, co_s, _ptr(A), lda, beta,
                                         _ptr(B), ldb, int(prefill))
        self._check(rc)
        return B

    def sketch_saso(self, dtype, side, layout, opS, opA, d, n, m, alpha, D_rows, D_cols, vec_nnz,
                    major_axis, seed: State, ro_s, co_s, A, lda, beta, B, ldb):
        rc = self.lib.rbref_sketch_saso(dtype, side, layout, opS, opA, d, n, m, alpha, D_rows,
                                        D_cols, vec_nnz, major_axis, C.addressof(seed.counter),
                                        C.addressof(seed.key), ro_s, co_s, _ptr(A), lda, beta,
                                        _ptr(B), ldb)
        self._check(rc)
        return B

    def sketch_vector(self, dtype, opS, d, m, alpha, D_rows, D_cols, family, major_axis,
                      seed: State, ro_s, co_s, x, incx, beta, y, incy):
        rc = self.lib.rbref_sketch_vector(dtype, opS, d, m, alpha, D_rows, D_cols, family,
                                          major_axis, C.addressof(seed.counter),
                                          C.addressof(seed.key), ro_s, co_s, _ptr(x), incx, beta,
                                          _ptr(y), incy)
        self._check(rc)
        return y

    def left_spmm(self, dtype, layout, opA, opB, d, n, m, alpha, fmt, A_rows, A_cols, vals, a,
                  b, ro_a, co_a, B, ldb, beta, Cm, ldc):
        """RandBLAS::sparse_data::left_spmm (spmm_dispatch.hh:52-179) on host arrays; Cm is
        updated in place.  Returns (status, message)."""
        rc = self.lib.rbref_left_spmm(dtype, layout, opA, opB, d, n, m, alpha, fmt, A_rows,
                                      A_cols, len(vals), _ptr(vals), _ptr(a), _ptr(b), ro_a,
                                      co_a, _ptr(B), ldb, beta, _ptr(Cm), ldc)
        return rc, (self.lib.rbref_last_error().decode() if rc else "")

    def right_spmm(self, dtype, layout, opA, opB, m, d, n, alpha, A, lda, fmt, B_rows, B_cols,
                   vals, a, b, ro_b, co_b, beta, Cm, ldc):
        """RandBLAS::sparse_data::right_spmm (spmm_dispatch.hh:181-219) on host arrays."""
        rc = self.lib.rbref_right_spmm(dtype, layout, opA, opB, m, d, n, alpha, _ptr(A), lda,
                                       fmt, B_rows, B_cols, len(vals), _ptr(vals), _ptr(a),
                                       _ptr(b), ro_b, co_b, beta, _ptr(Cm), ldc)
        return rc, (self.lib.rbref_last_error().decode() if rc else "")

    def sketch_sparse(self, dtype, side, layout, opS, opA, d, n, m, alpha, D_rows, D_cols,
                      family, major_axis, seed: State, ro_s, co_s, fmt, A_rows, A_cols, nnz,
                      vals, a, b, beta, B, ldb):
        rc = self.lib.rbref_sketch_sparse(dtype, side, layout, opS, opA, d, n, m, alpha, D_rows,
                                          D_cols, family, major_axis, C.addressof(seed.counter),
                                          C.addressof(seed.key), ro_s, co_s, fmt, A_rows, A_cols,
                                          nnz, _ptr(vals), _ptr(a), _ptr(b), beta, _ptr(B), ldb)
        self._check(rc)
        return B
