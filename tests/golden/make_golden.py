"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in a container that has the RandBLAS source tree (RANDBLAS_REF_DIR, else a directory
named "reference" beside this repository).  It builds oracle/_ref/librbref.so -- the
reference's own headers compiled against the project's Random123 / BLAS++ stand-ins -- and
records:

* philox_kat.json: the Philox4x32-10 known-answer rows of the reference's
  test/test_basic_rng/r123_kat_vectors.txt (parsed from that file);
* fill_dense.npz, fill_sparse.npz, sketch_*.npz: outputs of the reference's public functions on
  small seeded cases (every layout / op / side / submatrix combination the parity tests use);
* sparse_convert.npz: the reference's coo_arrays_determine_sort / coo_arrays_apply_sort /
  sorted_idxs_to_compressed_ptr / compressed_ptr_to_sorted_idxs on seeded duplicate-free COO
  data;
* random_sparse.npz: the reference's random_coo / random_csr / random_csc on small seeded
  cases (every format, value and index type, densities 0, 1 and in between, empty shapes);
* full_size.json: SHA-256 digests and next states of the full-size operators of the
  benchmark workloads (the 200 x 10000 Gaussian FP64 operator and its 10000 x 50 uniform data
  matrix; the 1024 x 2^20 SASO with 8 nonzeros per column), so the GPU tests can pin those
  bit for bit without shipping the arrays.

* spmm.npz: the reference's left_spmm / right_spmm over COO / CSR / CSC data, every op and
  layout, FP32 / FP64, COO offsets and duplicates, alpha = 0, beta = 0, empty data, and the
  argument checks with their messages.

* full_size.json also holds the digests of that 200 x 10000 operator (FP64 and FP32) from
  the reference's code with Box-Muller's sin / cos / log taken from the shared float-float
  specification (the "shared math" mode), which the GPU must match bit for bit.

Usage: python tests/golden/make_golden.py [random_sparse | sparse_convert | spmm | shared_math]
(an argument writes only that part)
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import RefLib, State  # noqa: E402
from oracle import build as obuild  # noqa: E402

import itertools  # noqa: E402

CASES = os.path.join(HERE)


def st(s: State):
    return [list(s.counter), list(s.key)]


def kat_rows():
    path = os.path.join(obuild.REF_DIR, "test", "test_basic_rng", "r123_kat_vectors.txt")
    rows = []
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) == 12 and parts[0] == "philox4x32" and parts[1] == "10":
                vals = [int(x, 16) for x in parts[2:]]
                rows.append({"ctr": vals[0:4], "key": vals[4:6], "out": vals[6:10]})
    return rows


def dense_fill_cases():
    cases = []
    dims = [(7, 13), (13, 7), (37, 90), (90, 37), (5, 5), (64, 65)]
    for (R, Cc), fam, ax, dt, lay in itertools.product(dims, (0, 1), (0, 1), (0, 1), (0, 1)):
        subs = [(R, Cc, 0, 0), (max(1, R - 3), max(1, Cc - 5), min(2, R - 1), min(3, Cc - 1)),
                (1, Cc, R - 1, 0), (R, 1, 0, Cc - 1)]
        for (nr, nc, ro, co) in subs:
            cases.append(dict(R=R, C=Cc, family=fam, axis=ax, dtype=dt, layout=lay, nr=nr, nc=nc,
                              ro=ro, co=co, ctr=[11, 0, 7, 0], key=[2024, 3]))
    return cases


RANDOM_SPARSE_SHAPES = [(100, 200, 0.05), (80, 150, 0.1), (5, 8, 1.0), (7, 9, 1.0),
                        (10, 20, 0.0), (0, 10, 0.5), (10, 0, 0.5), (1, 1, 0.5), (300, 7, 0.9),
                        (50, 3000, 1e-4), (2000, 2, 0.3), (13, 17, 0.999999), (64, 64, 0.02)]

# The sketch_sparse benchmark's data matrix: 2^17 x 512 CSR with 5 expected nonzeros per row.
RANDOM_CSR_FULL = dict(fmt=1, m=1 << 17, n=512, density=5 / 512, ctr=[0, 0, 0, 0], key=[11, 0])


def random_sparse_fixtures(ref):
    arrays, meta = {}, []
    for i, ((m, n, dens), fmt, dt, it) in enumerate(itertools.product(
            RANDOM_SPARSE_SHAPES, (0, 1, 2), (0, 1), (0, 1))):
        c = dict(fmt=fmt, dtype=dt, itype=it, m=m, n=n, density=dens, ctr=[5, 0, 0, 0],
                 key=[4242, i % 3])
        vals, a, b, nxt = ref.random_sparse(fmt, dt, it, m, n, dens,
                                            State.make(c["ctr"], c["key"]))
        arrays[f"v{i}"], arrays[f"a{i}"], arrays[f"b{i}"] = vals, a, b
        meta.append(dict(c, nnz=int(vals.size), next=st(nxt)))
    np.savez_compressed(os.path.join(HERE, "random_sparse.npz"), meta=json.dumps(meta), **arrays)
    f = RANDOM_CSR_FULL
    vals, a, b, nxt = ref.random_sparse(f["fmt"], 0, 1, f["m"], f["n"], f["density"],
                                        State.make(f["ctr"], f["key"]))
    return dict(f, nnz=int(vals.size), next=st(nxt),
                rowptr_sha256=hashlib.sha256(a.tobytes()).hexdigest(),
                colidxs_sha256=hashlib.sha256(b.tobytes()).hexdigest(),
                vals_sha256=hashlib.sha256(vals.tobytes()).hexdigest())


def sparse_convert_fixtures(ref):
    rng = np.random.default_rng(2024)
    arrays, meta = {}, []
    for i in range(16):
        m, n = int(rng.integers(1, 200)), int(rng.integers(1, 200))
        nnz = int(rng.integers(0, min(m * n, 800) + 1))
        it = np.int32 if i % 2 else np.int64
        key = rng.choice(m * n, size=nnz, replace=False)  # duplicate-free, random order
        if i % 6 == 1:
            key = np.sort(key)  # already in CSR order
        rows, cols = (key // n).astype(it), (key % n).astype(it)
        vals = rng.standard_normal(nnz).astype(np.float32 if i % 3 else np.float64)
        arrays[f"r{i}"], arrays[f"c{i}"], arrays[f"v{i}"] = rows, cols, vals
        rec = dict(m=m, n=n, nnz=nnz, determine=ref.coo_determine_sort(rows, cols))
        for s in "RC":
            sv, sr, sc = ref.coo_apply_sort(s, vals, rows, cols)
            arrays[f"{s}v{i}"], arrays[f"{s}r{i}"], arrays[f"{s}c{i}"] = sv, sr, sc
            major, comp = (sr, m) if s == "R" else (sc, n)
            ptr = ref.sorted_idxs_to_compressed_ptr(major, comp, it)
            arrays[f"{s}p{i}"] = ptr
            assert np.array_equal(ref.compressed_ptr_to_sorted_idxs(ptr, nnz, it), major)
        meta.append(rec)
    np.savez_compressed(os.path.join(HERE, "sparse_convert.npz"), meta=json.dumps(meta),
                        **arrays)


def _sparse_arrays(rng, rows, cols, density, fmt, npdt, dup=False):
    """Seeded sparse data in the reference's convention (fmt 0 COO (a = rows, b = cols) in
    random order, 1 CSR (a = rowptr, b = colidxs), 2 CSC (a = colptr, b = rowidxs)); int64
    indices.  dup: COO with some (row, col) pairs repeated."""
    dense = rng.standard_normal((rows, cols)) * (rng.random((rows, cols)) < density)
    r_, c_ = np.nonzero(dense)
    vals = dense[r_, c_]
    if fmt == 0:
        if dup and len(vals):
            k = max(1, len(vals) // 4)
            pick = rng.integers(0, len(vals), k)
            r_, c_ = np.concatenate([r_, r_[pick]]), np.concatenate([c_, c_[pick]])
            vals = np.concatenate([vals, rng.standard_normal(k)])
        perm = rng.permutation(len(vals))
        return vals[perm].astype(npdt), r_[perm].astype(np.int64), c_[perm].astype(np.int64)
    if fmt == 1:
        a = np.concatenate([[0], np.cumsum(np.bincount(r_, minlength=rows))]).astype(np.int64)
        return vals.astype(npdt), a, c_.astype(np.int64)
    order = np.lexsort((r_, c_))
    a = np.concatenate([[0], np.cumsum(np.bincount(c_, minlength=cols))]).astype(np.int64)
    return vals[order].astype(npdt), a, r_[order].astype(np.int64)


def spmm_fixtures(ref):
    """left_spmm / right_spmm (RandBLAS/sparse_data/spmm_dispatch.hh:52-219) over COO / CSR /
    CSC x opA x opB x layout x FP32/FP64, with COO submatrix offsets (coo_spmm_impl.hh:70-92),
    COO duplicates, alpha = 0, beta = 0 over NaN-filled C, an empty sparse matrix, and the
    argument checks the reference applies (nonzero offsets or mismatched sizes of CSR / CSC
    data) with their messages."""
    rng = np.random.default_rng(2024)
    arrays, meta = {}, []
    i = 0

    def record(rec, vals, a, b, dense_in, C0, Cout):
        nonlocal i
        arrays[f"v{i}"], arrays[f"a{i}"], arrays[f"b{i}"] = vals, a, b
        arrays[f"D{i}"], arrays[f"C{i}"], arrays[f"O{i}"] = dense_in, C0, Cout
        meta.append(rec)
        i += 1

    def one(side, fmt, lay, opA, opB, dt, d, n, m, alpha, beta, offs=(0, 0), extra=(0, 0),
            density=0.3, nan_c=False, dup=False, short_ld=None):
        npdt = np.float32 if dt == 0 else np.float64
        # the sparse operand, before its op: (sr x sc) = op^-1 of (d x m) on the left,
        # of (n x d) on the right (right: C (m x d) = op(A) (m x n) op(submat(B)) (n x d))
        if side == 0:
            sr, sc = (d, m) if opA == 0 else (m, d)
        else:
            sr, sc = (n, d) if opB == 0 else (d, n)
        ro, co = offs
        Sr, Sc = sr + ro + extra[0], sc + co + extra[1]
        vals, a, b = _sparse_arrays(rng, Sr, Sc, density, fmt, npdt, dup)
        if side == 0:
            br, bc = (m, n) if opB == 0 else (n, m)
            cr, cc = d, n
        else:
            br, bc = (m, n) if opA == 0 else (n, m)
            cr, cc = m, d
        ldd = (br if lay == 0 else bc) + (-1 if short_ld == "dense" else 2)
        ldc = (cr if lay == 0 else cc) + (-1 if short_ld == "C" else 1)
        dense_in = rng.standard_normal(ldd * (bc if lay == 0 else br)).astype(npdt)
        C0 = rng.standard_normal(ldc * (cc if lay == 0 else cr)).astype(npdt)
        if nan_c:
            C0[:] = np.nan
        Cout = C0.copy()
        if side == 0:
            rc, msg = ref.left_spmm(dt, lay, opA, opB, d, n, m, alpha, fmt, Sr, Sc, vals, a, b,
                                    ro, co, dense_in, ldd, beta, Cout, ldc)
        else:
            rc, msg = ref.right_spmm(dt, lay, opA, opB, m, d, n, alpha, dense_in, ldd, fmt, Sr,
                                     Sc, vals, a, b, ro, co, beta, Cout, ldc)
        record(dict(side=side, fmt=fmt, layout=lay, opA=opA, opB=opB, dtype=dt, d=d, n=n, m=m,
                    alpha=alpha, beta=beta, ro=ro, co=co, S_rows=Sr, S_cols=Sc, ldd=ldd,
                    ldc=ldc, dense_rows=br, dense_cols=bc, C_rows=cr, C_cols=cc, rc=rc, msg=msg),
               vals, a, b, dense_in, C0, Cout)

    for side, fmt, lay, opA, opB, dt in itertools.product((0, 1), (0, 1, 2), (0, 1), (0, 1),
                                                          (0, 1), (0, 1)):
        offs = (2, 3) if fmt == 0 else (0, 0)
        extra = (1, 2) if fmt == 0 else (0, 0)
        one(side, fmt, lay, opA, opB, dt, 9, 7, 40, 0.75 if i % 3 else -1.5,
            0.0 if i % 2 else 0.5, offs, extra, nan_c=(i % 4 == 1))
    # COO with repeated (row, col) pairs, with and without offsets
    for side, lay, opA, opB in itertools.product((0, 1), (0, 1), (0, 1), (0, 1)):
        one(side, 0, lay, opA, opB, 1, 11, 5, 33, 1.25, 0.25, (1, 1) if lay else (0, 0),
            (2, 1) if lay else (0, 0), density=0.4, dup=True)
    # alpha = 0: C = beta * C, the sparse data is not read
    for side, fmt in itertools.product((0, 1), (0, 1, 2)):
        one(side, fmt, 1, 0, 0, 1, 6, 4, 20, 0.0, -2.0)
        one(side, fmt, 0, 1, 0, 0, 6, 4, 20, 0.0, 0.0, nan_c=True)
    # no nonzeros at all
    for side, fmt in itertools.product((0, 1), (0, 1, 2)):
        one(side, fmt, 0, 0, 1, 1, 8, 3, 17, 1.0, 0.5, density=0.0)
    # a larger case (multi-block kernels): FP32, every format, both sides
    for side, fmt in itertools.product((0, 1), (0, 1, 2)):
        one(side, fmt, 1, 0, 0, 0, 64, 16, 300, 1.0, 0.0, density=0.05)
    # the reference's argument checks: CSR / CSC data must match the sizes exactly and take no
    # offsets; COO must be at least the submatrix
    for side, fmt in itertools.product((0, 1), (1, 2)):
        one(side, fmt, 0, 0, 0, 1, 6, 4, 20, 1.0, 0.0, offs=(1, 0), extra=(-1, 0))
        one(side, fmt, 1, 1, 0, 1, 6, 4, 20, 1.0, 0.0, offs=(0, 1), extra=(0, -1))
        one(side, fmt, 0, 0, 1, 1, 6, 4, 20, 1.0, 0.0, extra=(1, 0))
    for side in (0, 1):
        one(side, 0, 0, 0, 0, 1, 6, 4, 20, 1.0, 0.0, offs=(0, 0), extra=(-1, 0))
    # leading dimensions below the stored sizes
    for side, lay, opD, which in itertools.product((0, 1), (0, 1), (0, 1), ("dense", "C")):
        if side == 0:
            one(side, 1, lay, 0, opD, 0, 6, 4, 20, 1.0, 0.0, short_ld=which)
        else:
            one(side, 2, lay, opD, 0, 0, 6, 4, 20, 1.0, 0.0, short_ld=which)
    np.savez_compressed(os.path.join(HERE, "spmm.npz"), meta=json.dumps(meta), **arrays)
    return len(meta)


def shared_math_fixtures(ref, full):
    """Digests of the reference's own 200 x 10000 Gaussian FP64 operator (seeded after its data
    matrix, counter 125000) and of its FP32 form with Box-Muller's sin / cos / log taken from
    the shared float-float specification (RefLib.set_math(1)): with the same math functions
    the GPU must reproduce them bit for bit."""
    ref.set_math(1)
    try:
        out = {}
        for name, dt in (("f64", 1), ("f32", 0)):
            buf, nxt = ref.fill_dense_unpacked(dt, 1, 200, 10000, 0, 1, 200, 10000, 0, 0,
                                               State.make([125000, 0, 0, 0], [0, 0]))
            out[name] = dict(sha256=hashlib.sha256(buf.tobytes()).hexdigest(), next=st(nxt))
    finally:
        ref.set_math(0)
    full["dense_200x10000_shared_math"] = dict(dist=dict(n_rows=200, n_cols=10000, family=0,
                                                         axis=1),
                                               seed=[[125000, 0, 0, 0], [0, 0]], layout=1,
                                               **out)


def main():
    ref = RefLib()
    if sys.argv[1:] == ["shared_math"]:
        path = os.path.join(HERE, "full_size.json")
        with open(path) as f:
            full = json.load(f)
        shared_math_fixtures(ref, full)
        with open(path, "w") as f:
            json.dump(full, f, indent=1)
        print("shared-math digests written to", path)
        return
    if sys.argv[1:] == ["spmm"]:
        print(spmm_fixtures(ref), "spmm fixtures written to", HERE)
        return
    if sys.argv[1:] == ["sparse_convert"]:
        sparse_convert_fixtures(ref)
        print("sparse_convert fixtures written to", HERE)
        return
    if sys.argv[1:] == ["random_sparse"]:
        path = os.path.join(HERE, "full_size.json")
        with open(path) as f:
            full = json.load(f)
        full["random_csr_2^17x512"] = random_sparse_fixtures(ref)
        with open(path, "w") as f:
            json.dump(full, f, indent=1)
        print("random_sparse fixtures written to", HERE)
        return
    out = {}

    kat = kat_rows()
    assert len(kat) == 3, kat
    with open(os.path.join(HERE, "philox_kat.json"), "w") as f:
        json.dump(kat, f, indent=1)

    # ---- fill_dense_unpacked
    cases = dense_fill_cases()
    arrays = {}
    meta = []
    for i, c in enumerate(cases):
        seed = State.make(c["ctr"], c["key"])
        buf, nxt = ref.fill_dense_unpacked(c["dtype"], c["layout"], c["R"], c["C"], c["family"],
                                           c["axis"], c["nr"], c["nc"], c["ro"], c["co"], seed)
        arrays[f"c{i}"] = buf
        meta.append(dict(c, next=st(nxt)))
    np.savez_compressed(os.path.join(HERE, "fill_dense.npz"), meta=json.dumps(meta), **arrays)

    # ---- fill_sparse (SASO and LASO; LASO stored as per-vector sorted triplets)
    arrays, meta = {}, []
    sp_cases = []
    for (R, Cc, k), ax, dt, it in itertools.product(
            [(10, 50, 3), (50, 10, 4), (64, 3000, 8), (16, 16, 16), (3, 100, 3), (100, 3, 2),
             (7, 7, 1)], (0, 1), (0, 1), (0, 1)):
        sp_cases.append(dict(R=R, C=Cc, vec_nnz=k, axis=ax, dtype=dt, itype=it, ctr=[3, 1, 0, 0],
                             key=[77, 0]))
    for i, c in enumerate(sp_cases):
        seed = State.make(c["ctr"], c["key"])
        vals, rows, cols, nnz, nxt = ref.fill_sparse(c["dtype"], c["itype"], c["R"], c["C"],
                                                     c["vec_nnz"], c["axis"], seed)
        if c["axis"] == 1:
            order = np.lexsort((cols, rows))
            vals, rows, cols = vals[order], rows[order], cols[order]
        arrays[f"v{i}"], arrays[f"r{i}"], arrays[f"c{i}"] = vals, rows, cols
        meta.append(dict(c, nnz=int(nnz), next=st(nxt)))
    np.savez_compressed(os.path.join(HERE, "fill_sparse.npz"), meta=json.dumps(meta), **arrays)

    # ---- dense sketches (left / right, all layouts and ops, submatrices, alpha / beta)
    rng = np.random.default_rng(7)
    arrays, meta = {}, []
    i = 0
    for side, lay, opS, opA, dt, fam, prefill in itertools.product(
            (0, 1), (0, 1), (0, 1), (0, 1), (0, 1), (0, 1), (0, 1)):
        if prefill and (opA == 1 or fam == 1):
            continue
        d, n, m = 9, 5, 37
        # operator large enough to hold a shifted submatrix
        if side == 0:
            Sr, Sc = (d, m) if opS == 0 else (m, d)
        else:
            Sr, Sc = (n, d) if opS == 0 else (d, n)
        ro, co = 2, 3
        D_rows, D_cols = Sr + ro + 1, Sc + co + 2
        # A dims
        if side == 0:
            ar, ac = (m, n) if opA == 0 else (n, m)
            br, bc = d, n
        else:
            # right: op(A) is m x n in the reference's naming; here (d,n,m) passes (m,d,n)
            ar, ac = (m, n) if opA == 0 else (n, m)
            br, bc = m, d
        if side == 1:
            # reference right overload argument order: (m, d, n)
            ar, ac = (m, n) if opA == 0 else (n, m)
            Sr, Sc = (n, d) if opS == 0 else (d, n)
            D_rows, D_cols = Sr + ro + 1, Sc + co + 2
        lda = (ar if lay == 0 else ac) + 1
        ldb = (br if lay == 0 else bc) + 2
        npdt = np.float32 if dt == 0 else np.float64
        A = rng.standard_normal((lda * (ac if lay == 0 else ar),)).astype(npdt)
        B = rng.standard_normal((ldb * (bc if lay == 0 else br),)).astype(npdt)
        alpha, beta = 1.5, (0.0 if i % 3 == 0 else -0.5)
        seed = State.make([i, 0, 0, 0], [99, 1])
        Bout = B.copy()
        if prefill and (ro, co) != (0, 0):
            pass
        ref.sketch_dense(dt, side, lay, opS, opA, d if side == 0 else m, n if side == 0 else d,
                         m if side == 0 else n, alpha, D_rows, D_cols, fam, 1, seed, ro, co, A,
                         lda, beta, Bout, ldb, prefill=bool(prefill))
        arrays[f"A{i}"], arrays[f"B{i}"], arrays[f"O{i}"] = A, B, Bout
        meta.append(dict(side=side, layout=lay, opS=opS, opA=opA, dtype=dt, family=fam,
                         prefill=prefill, d=d, n=n, m=m, D_rows=D_rows, D_cols=D_cols, ro=ro,
                         co=co, lda=lda, ldb=ldb, alpha=alpha, beta=beta, ctr=[i, 0, 0, 0],
                         key=[99, 1]))
        i += 1
    np.savez_compressed(os.path.join(HERE, "sketch_dense.npz"), meta=json.dumps(meta), **arrays)

    # ---- sparse-operator sketches
    arrays, meta = {}, []
    i = 0
    for side, lay, opS, opA, dt, ax in itertools.product((0, 1), (0, 1), (0, 1), (0, 1), (0, 1),
                                                         (0, 1)):
        d, n, m = 11, 6, 200
        if side == 0:
            Sr, Sc = (d, m) if opS == 0 else (m, d)
            ar, ac = (m, n) if opA == 0 else (n, m)
            br, bc = d, n
        else:
            Sr, Sc = (m, d) if opS == 0 else (d, m)  # right: op(S) is n x d with n := m here
            ar, ac = (n, m) if opA == 0 else (m, n)
            br, bc = n, d
        ro, co = 1, 4
        D_rows, D_cols = Sr + ro + 2, Sc + co + 3
        vec_nnz = 3
        lda = (ar if lay == 0 else ac) + 1
        ldb = (br if lay == 0 else bc) + 1
        npdt = np.float32 if dt == 0 else np.float64
        A = rng.standard_normal((lda * (ac if lay == 0 else ar),)).astype(npdt)
        B = rng.standard_normal((ldb * (bc if lay == 0 else br),)).astype(npdt)
        alpha, beta = -0.75, (0.0 if i % 2 == 0 else 2.0)
        seed = State.make([5 * i, 0, 0, 1], [123, 0])
        Bout = B.copy()
        if side == 0:
            ref.sketch_saso(dt, 0, lay, opS, opA, d, n, m, alpha, D_rows, D_cols, vec_nnz, ax,
                            seed, ro, co, A, lda, beta, Bout, ldb)
        else:
            # reference right overload: (m_rows_of_B, d, n_inner) = (n, d, m)
            ref.sketch_saso(dt, 1, lay, opS, opA, n, d, m, alpha, D_rows, D_cols, vec_nnz, ax,
                            seed, ro, co, A, lda, beta, Bout, ldb)
        arrays[f"A{i}"], arrays[f"B{i}"], arrays[f"O{i}"] = A, B, Bout
        meta.append(dict(side=side, layout=lay, opS=opS, opA=opA, dtype=dt, axis=ax, d=d, n=n,
                         m=m, D_rows=D_rows, D_cols=D_cols, vec_nnz=vec_nnz, ro=ro, co=co,
                         lda=lda, ldb=ldb, alpha=alpha, beta=beta, ctr=[5 * i, 0, 0, 1],
                         key=[123, 0]))
        i += 1
    np.savez_compressed(os.path.join(HERE, "sketch_saso.npz"), meta=json.dumps(meta), **arrays)

    # ---- sketch_vector
    arrays, meta = {}, []
    for i, (opS, dt, fam, incx, incy) in enumerate(itertools.product((0, 1), (0, 1), (0, 1),
                                                                     (1, 3), (1, 2))):
        d, m = 8, 50
        ro, co = 1, 2
        D_rows, D_cols = d + ro + 1, m + co + 1
        xl = (m if opS == 0 else d)
        yl = (d if opS == 0 else m)
        npdt = np.float32 if dt == 0 else np.float64
        x = rng.standard_normal(xl * incx).astype(npdt)
        y = rng.standard_normal(yl * incy).astype(npdt)
        yout = y.copy()
        seed = State.make([i, 9, 0, 0], [5, 5])
        ref.sketch_vector(dt, opS, d, m, 0.5, D_rows, D_cols, fam, 1, seed, ro, co, x, incx,
                          (0.0 if i % 2 else 1.25), yout, incy)
        arrays[f"x{i}"], arrays[f"y{i}"], arrays[f"o{i}"] = x, y, yout
        meta.append(dict(opS=opS, dtype=dt, family=fam, incx=incx, incy=incy, d=d, m=m, ro=ro,
                         co=co, D_rows=D_rows, D_cols=D_cols, alpha=0.5,
                         beta=(0.0 if i % 2 else 1.25), ctr=[i, 9, 0, 0], key=[5, 5]))
    np.savez_compressed(os.path.join(HERE, "sketch_vector.npz"), meta=json.dumps(meta), **arrays)

    # ---- sketch_sparse (dense operator, sparse data in COO / CSR / CSC)
    arrays, meta = {}, []
    i = 0
    for side, lay, opS, opA, dt, fmt in itertools.product((0, 1), (0, 1), (0, 1), (0, 1), (0, 1),
                                                          (0, 1, 2)):
        d, n, m = 7, 9, 60
        if side == 0:
            Sr, Sc = (d, m) if opS == 0 else (m, d)
            Ar, Ac = (m, n) if opA == 0 else (n, m)
            br, bc = d, n
        else:
            # right: B (n x d) = op(A) (n x m) op(S) (m x d)
            Sr, Sc = (m, d) if opS == 0 else (d, m)
            Ar, Ac = (n, m) if opA == 0 else (m, n)
            br, bc = n, d
        ro, co = 2, 1
        D_rows, D_cols = Sr + ro + 1, Sc + co + 1
        dense = rng.standard_normal((Ar, Ac)) * (rng.random((Ar, Ac)) < 0.2)
        r_, c_ = np.nonzero(dense)
        npdt = np.float32 if dt == 0 else np.float64
        vals = dense[r_, c_].astype(npdt)
        if fmt == 0:
            perm = rng.permutation(len(vals))
            a, b, v = r_[perm].astype(np.int64), c_[perm].astype(np.int64), vals[perm]
        elif fmt == 1:
            a = np.concatenate([[0], np.cumsum(np.bincount(r_, minlength=Ar))]).astype(np.int64)
            b, v = c_.astype(np.int64), vals
        else:
            order = np.lexsort((r_, c_))
            a = np.concatenate([[0], np.cumsum(np.bincount(c_, minlength=Ac))]).astype(np.int64)
            b, v = r_[order].astype(np.int64), vals[order]
        ldb = (br if lay == 0 else bc) + 1
        B = rng.standard_normal((ldb * (bc if lay == 0 else br),)).astype(npdt)
        Bout = B.copy()
        alpha, beta = 0.625, (0.0 if i % 2 == 0 else 0.5)
        seed = State.make([i, 0, 3, 0], [31, 4])
        if side == 0:
            ref.sketch_sparse(dt, 0, lay, opS, opA, d, n, m, alpha, D_rows, D_cols, 0, 1, seed, ro,
                              co, fmt, Ar, Ac, len(v), v, a, b, beta, Bout, ldb)
        else:
            ref.sketch_sparse(dt, 1, lay, opS, opA, n, d, m, alpha, D_rows, D_cols, 0, 1, seed, ro,
                              co, fmt, Ar, Ac, len(v), v, a, b, beta, Bout, ldb)
        arrays[f"v{i}"], arrays[f"a{i}"], arrays[f"b{i}"] = v, a, b
        arrays[f"B{i}"], arrays[f"O{i}"] = B, Bout
        meta.append(dict(side=side, layout=lay, opS=opS, opA=opA, dtype=dt, fmt=fmt, d=d, n=n, m=m,
                         Ar=Ar, Ac=Ac, D_rows=D_rows, D_cols=D_cols, ro=ro, co=co, ldb=ldb,
                         alpha=alpha, beta=beta, ctr=[i, 0, 3, 0], key=[31, 4]))
        i += 1
    np.savez_compressed(os.path.join(HERE, "sketch_sparse.npz"), meta=json.dumps(meta), **arrays)

    # ---- full-size operators of the benchmark workloads
    full = {}
    # 200 x 10000 Gaussian FP64 operator seeded after its data matrix (counter 125000, key 0):
    # Gaussians are compared to within a few ulp, so keep every 97th entry, not a digest
    S_dist = dict(n_rows=200, n_cols=10000, family=0, axis=1)
    sbuf, snext = ref.fill_dense_unpacked(1, 1, 200, 10000, 0, 1, 200, 10000, 0, 0,
                                          State.make([125000, 0, 0, 0], [0, 0]))
    np.savez_compressed(os.path.join(HERE, "dense_200x10000_sample.npz"),
                        idx=np.arange(0, sbuf.size, 97), vals=sbuf[::97])
    full["dense_200x10000_f64"] = dict(dist=S_dist, seed=[[125000, 0, 0, 0], [0, 0]],
                                       next=st(snext), layout=1, sample_every=97)
    vals, rows, cols, nnz, nxt = ref.fill_sparse(0, 1, 1024, 1 << 20, 8, 0,
                                                 State.make([7, 0, 0, 0], [0, 0]))
    full["saso_1024x2^20_k8"] = dict(seed=[[7, 0, 0, 0], [0, 0]], nnz=int(nnz), next=st(nxt),
                                     rows_sha256=hashlib.sha256(rows.tobytes()).hexdigest(),
                                     cols_sha256=hashlib.sha256(cols.tobytes()).hexdigest(),
                                     vals_sha256=hashlib.sha256(vals.tobytes()).hexdigest())
    full["random_csr_2^17x512"] = random_sparse_fixtures(ref)
    shared_math_fixtures(ref, full)
    with open(os.path.join(HERE, "full_size.json"), "w") as f:
        json.dump(full, f, indent=1)
    sparse_convert_fixtures(ref)
    spmm_fixtures(ref)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
