"""GPU random_coo / random_csr / random_csc (sparse_data/random_matrix.hh:135-355) against the
reference's outputs (golden fixtures), its full-size digest and the oracle: nonzero counts,
index arrays, pointers and next states bit for bit; Gaussian values within the Box-Muller
bound of the dense fills against the reference's glibc build, and bit for bit against the
oracle evaluated with the shared math functions (the same transform on the same words)."""
import hashlib
import math
import warnings

import numpy as np
import pytest

from conftest import golden_json, load_golden
from gpu_helpers import st_list, state_of, to_host, ulp_distance
from oracle.oracle import State

pytestmark = pytest.mark.gpu

GAUSS_ULP_MAX_GLIBC = 3  # as for fill_dense's Gaussians: glibc's sincosf / logf vs the shared math


def _gen(rb, fmt, m, n, density, state, dtype, itype):
    fn = (rb.random_coo, rb.random_csr, rb.random_csc)[fmt]
    with warnings.catch_warnings():
        warnings.simplefilter("error")  # a near-tie skip would make the comparison moot
        A, nxt = fn(m, n, density, state, dtype=dtype, itype=itype)
    if fmt == 0:
        a, b = A.rows, A.cols
    elif fmt == 1:
        a, b = A.rowptr, A.colidxs
    else:
        a, b = A.colptr, A.rowidxs
    return to_host(A.vals), to_host(a), to_host(b), nxt


def _check_values(got, ref, what):
    assert got.shape == ref.shape, what
    if got.size == 0:
        return 1.0
    u = ulp_distance(got.astype(np.float32), ref.astype(np.float32))
    assert u.max() <= GAUSS_ULP_MAX_GLIBC, (what, int(u.max()))
    # FP64 matrices hold float Box-Muller values promoted to double, as in the reference
    assert np.array_equal(got.astype(np.float32).astype(got.dtype), got), what
    return float(np.mean(u == 0))


def test_random_sparse_golden(rb, oracle):
    import torch
    meta, z = load_golden("random_sparse")
    exact = []
    for i, c in enumerate(meta):
        dt = torch.float32 if c["dtype"] == 0 else torch.float64
        it = torch.int32 if c["itype"] == 0 else torch.int64
        vals, a, b, nxt = _gen(rb, c["fmt"], c["m"], c["n"], c["density"],
                               state_of([c["ctr"], c["key"]]), dt, it)
        assert vals.size == c["nnz"], c
        assert st_list(nxt) == c["next"], c
        ra = z[f"a{i}"]
        if c["fmt"] != 0 and c["m"] * c["n"] == 0 and ra.size == 0:
            ra = np.zeros(a.size, ra.dtype)  # the reference leaves an empty pointer array
        assert np.array_equal(a, ra), c
        assert np.array_equal(b, z[f"b{i}"]), c
        exact.append(_check_values(vals, z[f"v{i}"], c))
        with oracle.shared_math():
            ov, oa, ob, _ = oracle.random_sparse(c["fmt"], c["dtype"], c["itype"], c["m"],
                                                 c["n"], c["density"],
                                                 State.make(c["ctr"], c["key"]))
        assert np.array_equal(vals.view(np.uint8), ov.view(np.uint8)), c
    print("golden cases:", len(meta), "exact value fraction vs glibc (min):", min(exact))


def test_random_csr_full_size_digest(rb, oracle):
    """The sketch_sparse benchmark's data: 2^17 x 512 CSR with 5 expected nonzeros per row."""
    import torch
    g = golden_json("full_size.json")["random_csr_2^17x512"]
    seed = [g["ctr"], g["key"]]
    vals, rowptr, colidxs, nxt = _gen(rb, 1, g["m"], g["n"], g["density"], state_of(seed),
                                      torch.float32, torch.int64)
    assert vals.size == g["nnz"]
    assert st_list(nxt) == g["next"]
    assert hashlib.sha256(rowptr.tobytes()).hexdigest() == g["rowptr_sha256"]
    assert hashlib.sha256(colidxs.tobytes()).hexdigest() == g["colidxs_sha256"]
    ov, _, _, _ = oracle.random_sparse(1, 0, 1, g["m"], g["n"], g["density"], State.make(*seed))
    frac = _check_values(vals, ov, "full size")
    assert frac > 0.95
    with oracle.shared_math():
        ovs, _, _, _ = oracle.random_sparse(1, 0, 1, g["m"], g["n"], g["density"],
                                            State.make(*seed))
    assert np.array_equal(vals.view(np.uint32), ovs.view(np.uint32))
    print("2^17 x 512 CSR: nnz", vals.size, "exact values vs glibc", frac)


@pytest.mark.parametrize("fmt,m,n,density", [
    (1, 1 << 20, 4096, 1e-3),   # 4.2 M nonzeros, ~4 per row
    (2, 4096, 1 << 20, 1e-3),   # the same as CSC
    (0, 1 << 20, 4096, 1e-3),   # COO over a 2^32-entry index space
    (1, 200, 100000, 0.05),     # long rows: ~5000 nonzeros each
    (2, 3, 1 << 22, 0.5),       # 3-row columns, dense draws (2 pairs per 4 words)
    (1, 1 << 18, 3, 0.999),     # nearly full rows
])
def test_random_sparse_vs_oracle_large(rb, oracle, fmt, m, n, density):
    import torch
    seed = [[17, 0, 0, 0], [5, 9]]
    vals, a, b, nxt = _gen(rb, fmt, m, n, density, state_of(seed), torch.float64, torch.int64)
    ov, oa, ob, onx = oracle.random_sparse(fmt, 1, 1, m, n, density, State.make(*seed))
    assert vals.size == ov.size
    assert st_list(nxt) == [list(onx.counter), list(onx.key)]
    assert np.array_equal(a, oa) and np.array_equal(b, ob)
    frac = _check_values(vals, ov, (fmt, m, n, density))
    assert frac > 0.95
    print((fmt, m, n, density), "nnz", vals.size, "exact values", frac)


def test_random_sparse_reference_checks(rb):
    """The reference's own tests (test/test_datastructures/test_spmats/test_random_matrix.cc):
    structural validity, density 0 and 1, empty shapes, determinism, the nonzero count within
    4 standard deviations, and a state that advances."""
    import torch
    S = rb.RNGState(42)
    for fmt, fn in enumerate((rb.random_coo, rb.random_csr, rb.random_csc)):
        A, nxt = fn(1000, 1000, 0.01, S)
        sd = math.sqrt(1000 * 1000 * 0.01 * 0.99)
        assert abs(A.vals.numel() - 10000) < 4 * sd
        assert nxt != S
        A2, nxt2 = fn(1000, 1000, 0.01, S)
        assert torch.equal(A.vals, A2.vals) and nxt2 == nxt
        if fmt == 0:
            r, c = to_host(A.rows), to_host(A.cols)
            assert np.all(np.diff(r * 1000 + c) > 0)
        else:
            p = to_host(A.rowptr if fmt == 1 else A.colptr)
            idx = to_host(A.colidxs if fmt == 1 else A.rowidxs)
            assert p[0] == 0 and p[-1] == idx.size and np.all(np.diff(p) >= 0)
            starts = np.zeros(idx.size, bool)
            starts[p[:-1][p[:-1] < idx.size]] = True
            d = np.diff(idx)
            assert np.all((d > 0) | starts[1:]) and idx.min() >= 0 and idx.max() < 1000
        Z, zn = fn(10, 20, 0.0, S)
        assert Z.vals.numel() == 0 and zn == S
        if fmt:
            assert not to_host(Z.rowptr if fmt == 1 else Z.colptr).any()
        F, _ = fn(5, 8, 1.0, S)
        assert F.vals.numel() == 40
        E1, _ = fn(0, 10, 0.5, S)
        E2, _ = fn(10, 0, 0.5, S)
        assert E1.vals.numel() == 0 and E2.vals.numel() == 0


def test_random_sparse_errors(rb):
    S = rb.RNGState(1)
    with pytest.raises(rb.RandBLASError) as e:
        rb.random_csr(4, 4, 1.5, S)
    assert "density >= 0.0 && density <= 1.0" in str(e.value)
    assert "random_csr" in str(e.value)
    with pytest.raises(rb.RandBLASError):
        rb.random_coo(4, 4, float("nan"), S)
    with pytest.raises(rb.RandBLASError) as e:
        rb.random_csc(4, 4, 1e-20, S)
    assert e.value.code == rb._lib.ERROR_UNSUPPORTED


def test_random_csr_feeds_sketch_sparse(rb, oracle):
    """A generated CSR matrix used as the data of sketch_sparse equals the dense product."""
    import torch
    A, _ = rb.random_csr(3000, 64, 0.05, rb.RNGState(3), dtype=torch.float64)
    D = rb.DenseDist(40, 3000, rb.ScalarDist.Uniform)
    S = rb.DenseSkOp(D, rb.RNGState(8), dtype=torch.float64)
    B = torch.zeros(40, 64, dtype=torch.float64, device="cuda")
    rb.sketch_sparse(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, 40, 64, 3000, 1.0, S, 0, 0,
                     A, 0.0, B, 64)
    Ad = np.zeros((3000, 64))
    p, c, v = to_host(A.rowptr), to_host(A.colidxs), to_host(A.vals)
    for i in range(3000):
        Ad[i, c[p[i]:p[i + 1]]] = v[p[i]:p[i + 1]]
    Sd = oracle.dense_matrix(1, 40, 3000, 1, 1, State.make((0, 0, 0, 0), (8, 0)))
    ref = Sd @ Ad
    assert np.abs(to_host(B) - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max()) * 3000
