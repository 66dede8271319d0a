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
