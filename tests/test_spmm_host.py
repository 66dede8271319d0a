"""left_spmm / right_spmm argument checks through the C ABI, on the CPU: every failing case of
tests/golden/spmm.npz (sizes of CSR / CSC data, offsets, COO covering the submatrix, leading
dimensions) fails here before any device work, with the reference's status and message
(RandBLAS/sparse_data/spmm_dispatch.hh:52-219)."""
import ctypes as C

import numpy as np

from conftest import load_golden


def _spmat(rb, c, v, a, b):
    m = rb._lib.rbg_spmat()
    m.format = (rb._lib.COO, rb._lib.CSR, rb._lib.CSC)[c["fmt"]]
    m.dtype = rb._lib.F32 if c["dtype"] == 0 else rb._lib.F64
    m.itype = rb._lib.I64
    m.n_rows, m.n_cols, m.nnz = c["S_rows"], c["S_cols"], len(v)
    m.vals = v.ctypes.data if len(v) else None
    m.idx_a = a.ctypes.data if len(a) else None
    m.idx_b = b.ctypes.data if len(b) else None
    return m


def test_spmm_checks_match_reference_messages(rb_host):
    rb = rb_host
    lib = rb.lib()
    meta, z = load_golden("spmm")
    n_checked = 0
    for i, c in enumerate(meta):
        if not c["rc"]:
            continue
        v, a, b = z[f"v{i}"], z[f"a{i}"], z[f"b{i}"]
        dense, Cm = z[f"D{i}"].copy(), z[f"C{i}"].copy()
        sp = _spmat(rb, c, v, a, b)
        if c["side"] == 0:
            rc = lib.rbg_left_spmm(c["layout"], c["opA"], c["opB"], c["d"], c["n"], c["m"],
                                   c["alpha"], C.byref(sp), c["ro"], c["co"], dense.ctypes.data,
                                   c["ldd"], c["beta"], Cm.ctypes.data, c["ldc"], None)
        else:
            rc = lib.rbg_right_spmm(c["layout"], c["opA"], c["opB"], c["m"], c["d"], c["n"],
                                    c["alpha"], dense.ctypes.data, c["ldd"], C.byref(sp),
                                    c["ro"], c["co"], c["beta"], Cm.ctypes.data, c["ldc"], None)
        assert rc == c["rc"], (c, lib.rbg_last_error())
        assert lib.rbg_last_error().decode() == c["msg"], c
        assert np.array_equal(Cm, z[f"C{i}"], equal_nan=True)
        n_checked += 1
    assert n_checked == 30
