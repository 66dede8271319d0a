"""The oracle against the golden fixtures produced by the reference's own headers
(tests/golden/make_golden.py), CPU only."""
import hashlib

import numpy as np

from conftest import golden_json, load_golden
from oracle.oracle import State


def test_fill_dense_matches_reference(oracle):
    meta, z = load_golden("fill_dense")
    for i, c in enumerate(meta):
        seed = State.make(c["ctr"], c["key"])
        buf, nxt = oracle.fill_dense_unpacked(c["dtype"], c["layout"], c["R"], c["C"],
                                              c["family"], c["axis"], c["nr"], c["nc"], c["ro"],
                                              c["co"], seed)
        assert np.array_equal(buf.view(np.uint8), z[f"c{i}"].view(np.uint8)), c
        assert [list(nxt.counter), list(nxt.key)] == c["next"], c


def test_fill_sparse_matches_reference(oracle):
    meta, z = load_golden("fill_sparse")
    for i, c in enumerate(meta):
        seed = State.make(c["ctr"], c["key"])
        vals, rows, cols, nnz, nxt = oracle.fill_sparse(c["dtype"], c["itype"], c["R"], c["C"],
                                                        c["vec_nnz"], c["axis"], seed)
        assert nnz == c["nnz"]
        assert [list(nxt.counter), list(nxt.key)] == c["next"]
        if c["axis"] == 1:
            order = np.lexsort((cols, rows))
            vals, rows, cols = vals[order], rows[order], cols[order]
        assert np.array_equal(rows, z[f"r{i}"]) and np.array_equal(cols, z[f"c{i}"])
        assert np.array_equal(vals, z[f"v{i}"])


def test_full_size_saso_digest(oracle):
    g = golden_json("full_size.json")["saso_1024x2^20_k8"]
    vals, rows, cols, nnz, nxt = oracle.fill_sparse(0, 1, 1024, 1 << 20, 8, 0,
                                                    State.make(*g["seed"]))
    assert nnz == g["nnz"]
    assert [list(nxt.counter), list(nxt.key)] == g["next"]
    assert hashlib.sha256(rows.tobytes()).hexdigest() == g["rows_sha256"]
    assert hashlib.sha256(cols.tobytes()).hexdigest() == g["cols_sha256"]
    assert hashlib.sha256(vals.tobytes()).hexdigest() == g["vals_sha256"]


def test_full_size_gaussian_sample(oracle):
    g = golden_json("full_size.json")["dense_200x10000_f64"]
    _, z = load_golden("dense_200x10000_sample")
    buf, nxt = oracle.fill_dense_unpacked(1, 1, 200, 10000, 0, 1, 200, 10000, 0, 0,
                                          State.make(*g["seed"]))
    assert [list(nxt.counter), list(nxt.key)] == g["next"]
    assert np.array_equal(buf[z["idx"]], z["vals"])


def test_random_sparse_matches_reference(oracle):
    """random_coo / random_csr / random_csc (sparse_data/random_matrix.hh:135-355): every
    array and the next state bit for bit, including densities 0 and 1 and empty shapes."""
    meta, z = load_golden("random_sparse")
    for i, c in enumerate(meta):
        vals, a, b, nxt = oracle.random_sparse(c["fmt"], c["dtype"], c["itype"], c["m"], c["n"],
                                               c["density"], State.make(c["ctr"], c["key"]))
        assert vals.size == c["nnz"], c
        assert [list(nxt.counter), list(nxt.key)] == c["next"], c
        assert np.array_equal(vals.view(np.uint8), z[f"v{i}"].view(np.uint8)), c
        assert np.array_equal(a, z[f"a{i}"]) and np.array_equal(b, z[f"b{i}"]), c


def test_random_sparse_structure_and_rate(oracle):
    """The reference's own checks (test/test_datastructures/test_spmats/test_random_matrix.cc):
    sorted in-range indices, pointers from 0 to nnz, nnz within 4 standard deviations of
    m * n * density, and a state that advances."""
    m = n = 1000
    density = 0.01
    sd = np.sqrt(m * n * density * (1 - density))
    for fmt in (0, 1, 2):
        seed = State.from_key(42)
        vals, a, b, nxt = oracle.random_sparse(fmt, 1, 1, m, n, density, seed)
        assert abs(vals.size - m * n * density) < 4 * sd
        assert nxt.tuple() != seed.tuple()
        if fmt == 0:
            key = a * n + b
            assert np.all(np.diff(key) > 0) and a.min() >= 0 and b.max() < n
        else:
            assert a[0] == 0 and a[-1] == vals.size and np.all(np.diff(a) >= 0)
            for i in range(len(a) - 1):
                seg = b[a[i]:a[i + 1]]
                assert np.all(np.diff(seg) > 0) and (seg.size == 0 or (seg[0] >= 0 and
                                                                       seg[-1] < 1000))
    with np.testing.assert_raises(ValueError):
        oracle.random_sparse(1, 1, 1, 4, 4, 1.5, State.from_key(1))


def test_full_size_random_csr_digest(oracle):
    g = golden_json("full_size.json")["random_csr_2^17x512"]
    vals, a, b, nxt = oracle.random_sparse(g["fmt"], 0, 1, g["m"], g["n"], g["density"],
                                           State.make(g["ctr"], g["key"]))
    assert vals.size == g["nnz"]
    assert [list(nxt.counter), list(nxt.key)] == g["next"]
    assert hashlib.sha256(a.tobytes()).hexdigest() == g["rowptr_sha256"]
    assert hashlib.sha256(b.tobytes()).hexdigest() == g["colidxs_sha256"]
    assert hashlib.sha256(vals.tobytes()).hexdigest() == g["vals_sha256"]


def test_sparse_conversions_match_reference(oracle):
    """coo_arrays_determine_sort, coo_arrays_apply_sort, sorted_idxs_to_compressed_ptr and
    compressed_ptr_to_sorted_idxs (sparse_data/base.hh:119-220, 278-302) on duplicate-free
    COO data, bit for bit."""
    meta, z = load_golden("sparse_convert")
    for i, c in enumerate(meta):
        rows, cols, vals = z[f"r{i}"], z[f"c{i}"], z[f"v{i}"]
        assert oracle.coo_determine_sort(rows, cols) == c["determine"], c
        for s in "RC":
            sv, sr, sc = oracle.coo_apply_sort(s, vals, rows, cols)
            assert np.array_equal(sv, z[f"{s}v{i}"]) and np.array_equal(sr, z[f"{s}r{i}"])
            assert np.array_equal(sc, z[f"{s}c{i}"]), (c, s)
            major, comp = (sr, c["m"]) if s == "R" else (sc, c["n"])
            ptr = oracle.sorted_idxs_to_compressed_ptr(major, comp, major.dtype)
            assert np.array_equal(ptr, z[f"{s}p{i}"]), (c, s)
            assert np.array_equal(oracle.compressed_ptr_to_sorted_idxs(ptr, c["nnz"],
                                                                       major.dtype), major)


def test_shared_math_oracle_digests(oracle):
    """The oracle in its shared-math mode reproduces the reference's own 200 x 10000 Gaussian
    operator computed with the same math functions (digests from tests/golden), FP64 and FP32,
    and its default mode is left untouched afterwards."""
    g = golden_json("full_size.json")["dense_200x10000_shared_math"]
    with oracle.shared_math():
        for name, dt in (("f64", 1), ("f32", 0)):
            buf, nxt = oracle.fill_dense_unpacked(dt, 1, 200, 10000, 0, 1, 200, 10000, 0, 0,
                                                  State.make(*g["seed"]))
            assert hashlib.sha256(buf.tobytes()).hexdigest() == g[name]["sha256"], name
            assert [list(nxt.counter), list(nxt.key)] == g[name]["next"]
    assert oracle.lib.orc_get_math() == 0
    buf, _ = oracle.fill_dense_unpacked(1, 1, 200, 10000, 0, 1, 200, 10000, 0, 0,
                                        State.make(*g["seed"]))
    assert hashlib.sha256(buf.tobytes()).hexdigest() != g["f64"]["sha256"]


def test_shared_math_oracle_matches_reference_code(oracle, reflib):
    """With the shared math functions in both, the restatement and the reference's own headers
    agree bit for bit on Gaussian fills (every layout, both types, submatrices) and on the
    values of random sparse matrices; run where the reference tree is present."""
    reflib.set_math(1)
    try:
        with oracle.shared_math():
            for dt, lay, (R, Cc, nr, nc, ro, co) in [
                    (0, 1, (300, 7000, 300, 7000, 0, 0)), (1, 0, (300, 7000, 120, 5001, 7, 11)),
                    (0, 0, (9000, 50, 8000, 33, 5, 3)), (1, 1, (9000, 50, 9000, 50, 0, 0))]:
                seed = State.make([17, 3, 0, 0], [9, 1])
                a, an = oracle.fill_dense_unpacked(dt, lay, R, Cc, 0, 1, nr, nc, ro, co, seed)
                b, bn = reflib.fill_dense_unpacked(dt, lay, R, Cc, 0, 1, nr, nc, ro, co, seed)
                assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
                assert list(an.counter) == list(bn.counter)
            for fmt in (0, 1, 2):
                ov, oa, ob, _ = oracle.random_sparse(fmt, 0, 1, 3000, 400, 0.01,
                                                     State.from_key(5))
                rv, ra, rb_, _ = reflib.random_sparse(fmt, 0, 1, 3000, 400, 0.01,
                                                      State.from_key(5))
                assert np.array_equal(ov.view(np.uint32), rv.view(np.uint32))
                assert np.array_equal(ob, rb_)
    finally:
        reflib.set_math(0)
