"""ctypes binding of the C ABI in ``include/randblas_gb300.h``.

The shared library is loaded from the package directory (built in-tree by
``randblas_gb300/build.py``).  There is no fallback: if the library is missing the import
of :func:`lib` raises, so nothing can silently run on the CPU.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "librandblas_gb300.so")

# enums (values as in the header)
COL_MAJOR, ROW_MAJOR = 0, 1
NO_TRANS, TRANS = 0, 1
GAUSSIAN, UNIFORM = 0, 1
AXIS_SHORT, AXIS_LONG = 0, 1
F32, F64 = 0, 1
BF16 = 2  # storage type of A for rbg_lskge3_lowp_ex
I32, I64 = 0, 1
COO, CSR, CSC = 0, 1, 2
PREC_BF16, PREC_FP8_E4M3 = 0, 1

SUCCESS = 0
ERROR_INVALID_ARGUMENT = 1
ERROR_OVERFLOW = 2
ERROR_CUDA = 3
ERROR_TIMEOUT = 4
ERROR_UNSUPPORTED = 5
ERROR_ALLOC = 6


class rbg_state(C.Structure):
    _fields_ = [("counter", C.c_uint32 * 4), ("key", C.c_uint32 * 2)]


class rbg_dense_dist(C.Structure):
    _fields_ = [("n_rows", C.c_int64), ("n_cols", C.c_int64), ("family", C.c_int32),
                ("major_axis", C.c_int32)]


class rbg_dense_skop(C.Structure):
    _fields_ = [("dist", rbg_dense_dist), ("seed_state", rbg_state), ("next_state", rbg_state),
                ("dtype", C.c_int32), ("layout", C.c_int32), ("buff", C.c_void_p)]


class rbg_sparse_dist(C.Structure):
    _fields_ = [("n_rows", C.c_int64), ("n_cols", C.c_int64), ("vec_nnz", C.c_int64),
                ("major_axis", C.c_int32), ("reserved", C.c_int32)]


class rbg_sparse_skop(C.Structure):
    _fields_ = [("dist", rbg_sparse_dist), ("seed_state", rbg_state), ("next_state", rbg_state),
                ("nnz", C.c_int64), ("dtype", C.c_int32), ("itype", C.c_int32),
                ("vals", C.c_void_p), ("rows", C.c_void_p), ("cols", C.c_void_p)]


class rbg_spmat(C.Structure):
    _fields_ = [("format", C.c_int32), ("dtype", C.c_int32), ("itype", C.c_int32),
                ("reserved", C.c_int32), ("n_rows", C.c_int64), ("n_cols", C.c_int64),
                ("nnz", C.c_int64), ("vals", C.c_void_p), ("idx_a", C.c_void_p),
                ("idx_b", C.c_void_p)]


class rbg_batch_problem(C.Structure):
    _fields_ = [("d", C.c_int64), ("n", C.c_int64), ("m", C.c_int64), ("dist", rbg_dense_dist),
                ("seed", rbg_state), ("ro_s", C.c_int64), ("co_s", C.c_int64),
                ("A", C.c_void_p), ("lda", C.c_int64), ("B", C.c_void_p), ("ldb", C.c_int64),
                ("alpha", C.c_float), ("beta", C.c_float), ("tile_config", C.c_int32),
                ("reserved", C.c_int32)]


P = C.c_void_p
CI64 = C.c_int64
CI32 = C.c_int32
CD = C.c_double
PS = C.POINTER(rbg_state)

# name -> argtypes (restype int unless noted)
SIGNATURES = {
    "rbg_last_error": ([], C.c_char_p),
    "rbg_version": ([], C.c_int),
    "rbg_set_deterministic": ([C.c_int], C.c_int),
    "rbg_get_deterministic": ([], C.c_int),
    "rbg_kernel_launches": ([], C.c_uint64),
    "rbg_profile_enable": ([C.c_int], C.c_int),
    "rbg_profile_count": ([C.POINTER(CI32)], C.c_int),
    "rbg_profile_entry": ([CI32, C.c_char_p, CI32, C.POINTER(CD), C.POINTER(CI64)], C.c_int),
    "rbg_state_from_key": ([C.c_uint64, PS], C.c_int),
    "rbg_state_incr": ([PS, C.c_uint64, PS], C.c_int),
    "rbg_dense_dist_properties": ([C.POINTER(rbg_dense_dist), C.POINTER(CI64), C.POINTER(CI64),
                                   C.POINTER(CI32), C.POINTER(CD)], C.c_int),
    "rbg_dense_next_state": ([C.POINTER(rbg_dense_dist), PS, PS], C.c_int),
    "rbg_dense_skop_init": ([C.POINTER(rbg_dense_skop), C.POINTER(rbg_dense_dist), PS, CI32],
                            C.c_int),
    "rbg_sparse_dist_properties": ([C.POINTER(rbg_sparse_dist), C.POINTER(CI64), C.POINTER(CI64),
                                    C.POINTER(CI64), C.POINTER(CD)], C.c_int),
    "rbg_sparse_next_state": ([C.POINTER(rbg_sparse_dist), PS, PS], C.c_int),
    "rbg_sparse_skop_init": ([C.POINTER(rbg_sparse_skop), C.POINTER(rbg_sparse_dist), PS, CI32,
                              CI32], C.c_int),
    "rbg_fill_dense_unpacked": ([CI32, CI32, C.POINTER(rbg_dense_dist), CI64, CI64, CI64, CI64, P, PS,
                                 PS, P], C.c_int),
    "rbg_fill_dense": ([CI32, C.POINTER(rbg_dense_dist), P, PS, PS, P], C.c_int),
    "rbg_fill_dense_skop": ([C.POINTER(rbg_dense_skop), P], C.c_int),
    "rbg_fill_sparse_unpacked_nosub": ([CI32, CI32, C.POINTER(rbg_sparse_dist), C.POINTER(CI64), P,
                                        P, P, PS, PS, P], C.c_int),
    "rbg_fill_sparse": ([C.POINTER(rbg_sparse_skop), P], C.c_int),
    "rbg_repeated_fisher_yates": ([CI64, CI64, CI64, P, PS, PS, P], C.c_int),
    "rbg_lskge3": ([CI32, CI32, CI32, CI64, CI64, CI64, CD, C.POINTER(rbg_dense_skop), CI64, CI64, P, CI64,
                    CD, P, CI64, P], C.c_int),
    "rbg_rskge3": ([CI32, CI32, CI32, CI64, CI64, CI64, CD, P, CI64, C.POINTER(rbg_dense_skop), CI64, CI64,
                    CD, P, CI64, P], C.c_int),
    "rbg_lskge3_noalloc": ([CI32, CI32, CI32, CI64, CI64, CI64, CD, C.POINTER(rbg_dense_skop),
                            CI64, CI64, P, CI64, CD, P, CI64, P], C.c_int),
    "rbg_sketch_vector": ([CI32, CI64, CI64, CD, C.POINTER(rbg_dense_skop), CI64, CI64, P, CI64, CD, P,
                           CI64, P], C.c_int),
    "rbg_lskges": ([CI32, CI32, CI32, CI64, CI64, CI64, CD, C.POINTER(rbg_sparse_skop), CI64, CI64, P,
                    CI64, CD, P, CI64, P], C.c_int),
    "rbg_rskges": ([CI32, CI32, CI32, CI64, CI64, CI64, CD, P, CI64, C.POINTER(rbg_sparse_skop), CI64,
                    CI64, CD, P, CI64, P], C.c_int),
    "rbg_sketch_vector_sparse": ([CI32, CI64, CI64, CD, C.POINTER(rbg_sparse_skop), CI64, CI64, P, CI64,
                                  CD, P, CI64, P], C.c_int),
    "rbg_lsksp3": ([CI32, CI32, CI32, CI64, CI64, CI64, CD, C.POINTER(rbg_dense_skop), CI64, CI64,
                    C.POINTER(rbg_spmat), CD, P, CI64, P], C.c_int),
    "rbg_rsksp3": ([CI32, CI32, CI32, CI64, CI64, CI64, CD, C.POINTER(rbg_spmat),
                    C.POINTER(rbg_dense_skop), CI64, CI64, CD, P, CI64, P], C.c_int),
    "rbg_left_spmm": ([CI32, CI32, CI32, CI64, CI64, CI64, CD, C.POINTER(rbg_spmat), CI64, CI64, P, CI64, CD,
                       P, CI64, P], C.c_int),
    "rbg_right_spmm": ([CI32, CI32, CI32, CI64, CI64, CI64, CD, P, CI64, C.POINTER(rbg_spmat), CI64, CI64,
                        CD, P, CI64, P], C.c_int),
    "rbg_lskge3_lowp_workspace": ([CI32, CI64, CI64, CI64, C.POINTER(C.c_size_t)], C.c_int),
    "rbg_lskge3_lowp": ([CI32, CI32, CI32, CI32, CI64, CI64, CI64, C.c_float, C.POINTER(rbg_dense_skop),
                         CI64, CI64, P, CI64, C.c_float, P, CI64, P, C.c_size_t, P], C.c_int),
    "rbg_lskge3_lowp_ex": ([CI32, CI32, CI32, CI32, CI32, CI64, CI64, CI64, C.c_float,
                            C.POINTER(rbg_dense_skop), CI64, CI64, P, CI64, C.c_float, P, CI64, P,
                            C.c_size_t, P], C.c_int),
    "rbg_lowp_status": ([C.POINTER(CI32)], C.c_int),
    "rbg_require_symmetric": ([CI32, CI32, P, CI64, CI64, CD, P], C.c_int),
    "rbg_sketch_symmetric": ([CI32, CI32, CI64, CI64, CD, C.POINTER(rbg_dense_skop), CI64, CI64,
                              P, CI64, CD, P, CI64, CD, P], C.c_int),
    "rbg_sketch_symmetric_sparse": ([CI32, CI32, CI64, CI64, CD, C.POINTER(rbg_sparse_skop),
                                     CI64, CI64, P, CI64, CD, P, CI64, CD, P], C.c_int),
    "rbg_lskge3_batched": ([CI32, C.POINTER(rbg_batch_problem), CI64, CI32, P], C.c_int),
    "rbg_batched_tile_configs": ([C.POINTER(CI32)], C.c_int),
    "rbg_batched_tile_shape": ([CI32, C.POINTER(CI32), C.POINTER(CI32)], C.c_int),
    "rbg_batched_plan_create": ([CI32, C.POINTER(rbg_batch_problem), CI64, CI32,
                                 C.POINTER(P)], C.c_int),
    "rbg_batched_plan_execute": ([P, P], C.c_int),
    "rbg_batched_plan_info": ([P, C.POINTER(CI64), C.POINTER(CI64)], C.c_int),
    "rbg_batched_plan_destroy": ([P], C.c_int),
    "rbg_random_sparse_create": ([CI32, CI64, CI64, CD, PS, C.POINTER(P), C.POINTER(CI64), PS, P],
                                 C.c_int),
    "rbg_random_sparse_fill": ([P, CI32, CI32, P, P, P, P], C.c_int),
    "rbg_random_sparse_info": ([P, C.POINTER(CI64), C.POINTER(CI64)], C.c_int),
    "rbg_random_sparse_destroy": ([P], C.c_int),
    "rbg_compressed_ptr_to_sorted_idxs": ([CI64, CI32, P, CI64, CI32, P, P], C.c_int),
    "rbg_sorted_idxs_to_compressed_ptr": ([CI64, CI32, P, CI64, CI32, P, P], C.c_int),
    "rbg_coo_determine_sort": ([CI32, CI64, P, P, C.POINTER(CI32), P], C.c_int),
    "rbg_coo_apply_sort": ([CI32, CI32, CI32, CI64, P, P, P, P], C.c_int),
}

_lock = threading.Lock()
_lib = None


class RandBLASError(RuntimeError):
    """A failed call of the C ABI; ``code`` is the status, the message is rbg_last_error()."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def lib() -> C.CDLL:
    """The loaded library (raises if it was not built)."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not os.path.exists(LIB_PATH):
                    raise ImportError(
                        f"{LIB_PATH} is missing: build it with `python randblas_gb300/build.py` "
                        "(there is no CPU fallback)")
                handle = C.CDLL(LIB_PATH)
                for name, (args, res) in SIGNATURES.items():
                    fn = getattr(handle, name)
                    fn.argtypes = args
                    fn.restype = res
                _lib = handle
    return _lib


def check(rc: int) -> None:
    if rc != SUCCESS:
        msg = lib().rbg_last_error().decode(errors="replace")
        raise RandBLASError(rc, msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))
