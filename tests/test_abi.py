"""The C ABI library: it loads, exports every function include/randblas_gb300.h declares,
and its host-only entry points (states, distributions, argument checks) behave like the
reference without touching a GPU.  CPU only."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT


def declared_functions():
    with open(os.path.join(ROOT, "include", "randblas_gb300.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^(?:int|uint64_t|const char \*)\s*(rbg_\w+)\s*\(", text,
                                 re.M)))


@pytest.fixture(scope="module")
def lib():
    from randblas_gb300 import build as rbuild
    rbuild.build()
    import randblas_gb300
    return randblas_gb300.lib()


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from randblas_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_state_and_distribution_logic(lib, oracle):
    import randblas_gb300 as rb
    from oracle.oracle import State
    s = rb.RNGState(42)
    assert s.key == [42, 0] and s.counter == [0, 0, 0, 0]
    assert rb.RNGState(2**40 + 5).key == [5, 256]
    assert s.incr(2**32 + 3).counter == [3, 1, 0, 0]
    for (r, c) in [(200, 10000), (10000, 200), (5, 5), (1, 7), (4096, 1 << 20)]:
        for fam in (rb.ScalarDist.Gaussian, rb.ScalarDist.Uniform):
            for ax in (rb.Axis.Long, rb.Axis.Short):
                D = rb.DenseDist(r, c, fam, ax)
                assert D.natural_layout == oracle.natural_layout(int(ax), r, c)
                assert D.dim_major == oracle.dim_major(int(ax), r, c)
                assert D.isometry_scale == pytest.approx(D.dim_minor ** -0.5)
                seed = rb.RNGState(7, counter=(1, 2, 3, 4))
                S = rb.DenseSkOp(D, seed)
                nx = oracle.dense_next_state(int(ax), r, c, State.make((1, 2, 3, 4), (7, 0)))
                assert S.next_state.counter == list(nx.counter)
    for (r, c, k) in [(1024, 1 << 20, 8), (50, 10, 4), (7, 7, 7)]:
        for ax in (rb.Axis.Short, rb.Axis.Long):
            D = rb.SparseDist(r, c, k, ax)
            S = rb.SparseSkOp(D, rb.RNGState(3))
            nx = oracle.sparse_next_state(int(ax), r, c, k, State.from_key(3))
            assert S.next_state.counter == list(nx.counter)
            assert D.full_nnz == k * D.dim_minor


def test_argument_checks_use_reference_messages(lib):
    import randblas_gb300 as rb
    with pytest.raises(rb.RandBLASError) as e:
        rb.DenseDist(0, 3)
    assert str(e.value) == "(D->n_rows > 0) was required, but did not hold, in function DenseDist"
    with pytest.raises(rb.RandBLASError) as e:
        rb.SparseDist(10, 20, 11)
    assert "in function SparseDist" in str(e.value) and e.value.code == 1
    # lskge3: submatrix out of range / leading dimensions (checked before any device work)
    S = rb.api.DenseSkOp(rb.DenseDist(10, 100), rb.RNGState(0))
    sc = S._c()
    rc = lib.rbg_lskge3(0, 0, 0, 10, 5, 100, 1.0, C.byref(sc), 1, 0, None, 100, 0.0, None, 10,
                        None)
    assert rc == 1
    assert "in function lskge3" in lib.rbg_last_error().decode()
    rc = lib.rbg_lskge3(0, 0, 0, 10, 5, 100, 1.0, C.byref(sc), 0, 0, None, 99, 0.0, None, 10,
                        None)
    assert rc == 1 and "(lda >= a.rows)" in lib.rbg_last_error().decode()
    # zero-sized problems are no-ops
    assert lib.rbg_lskge3(0, 0, 0, 0, 5, 100, 1.0, C.byref(sc), 0, 0, None, 100, 0.0, None, 1,
                          None) == 0
    # overflow of a size product
    big = rb._lib.rbg_dense_dist(2**62, 2**62, 0, 1)
    nxt = rb._lib.rbg_state()
    assert lib.rbg_dense_next_state(C.byref(big), C.byref(rb._lib.rbg_state()),
                                    C.byref(nxt)) == 2


def test_lowp_rejects_a_host_workspace(lib):
    """The tensor-core path's workspace must be device memory of the current GPU: host memory
    is refused before any device work (checked here without a GPU)."""
    import numpy as np

    import randblas_gb300 as rb
    S = rb.api.DenseSkOp(rb.DenseDist(256, 1024, rb.ScalarDist.Uniform), rb.RNGState(3))
    sc = S._c()
    ws = np.zeros(1 << 20, np.uint8)
    A = np.zeros((1024, 64), np.float32)
    B = np.zeros((256, 64), np.float32)
    rc = lib.rbg_lskge3_lowp(rb._lib.PREC_BF16, 1, 0, 0, 256, 64, 1024, 1.0, C.byref(sc), 0, 0,
                             A.ctypes.data, 64, 0.0, B.ctypes.data, 64, ws.ctypes.data,
                             ws.nbytes, None)
    assert rc == rb._lib.ERROR_INVALID_ARGUMENT
    assert "workspace must be device memory of the current GPU" in lib.rbg_last_error().decode()
