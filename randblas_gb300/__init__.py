"""randblas_gb300 -- RandBLAS's sketching hot path on one GB300 (sm_103a).

The compute lives in ``librandblas_gb300.so`` (hand-written CUDA behind the C ABI of
``include/randblas_gb300.h``); this package is the host-side mirror of the reference's API
(:mod:`randblas_gb300.api`), the autograd front end (:mod:`randblas_gb300.autograd`) and the
batching front end (:mod:`randblas_gb300.batched`).
"""
from . import autograd, lowp, profile  # noqa: F401
from ._lib import RandBLASError, lib  # noqa: F401
from .api import (  # noqa: F401
    Axis, COOMatrix, CSCMatrix, CSRMatrix, DenseDist, DenseSkOp, Layout, NonzeroSort, Op, RNGState,
    compressed_ptr_to_sorted_idxs, coo_arrays_determine_sort, coo_to_csc, coo_to_csr, csc_to_coo,
    csr_to_coo, sorted_idxs_to_compressed_ptr, transpose_as_coo, transpose_as_csc, transpose_as_csr,
    ScalarDist, SparseDist, SparseSkOp, deterministic, fill_dense, fill_dense_unpacked, fill_sparse,
    fill_sparse_unpacked_nosub, left_spmm, random_coo, random_csc, random_csr,
    repeated_fisher_yates, right_spmm, sketch_general,
    require_symmetric, set_deterministic, sketch_sparse, sketch_symmetric, sketch_vector, spmm)

__version__ = "1.1.0"
