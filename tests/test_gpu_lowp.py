"""The tensor-core precision path (rbg_lskge3_lowp): BF16 or FP8 e4m3 operands, FP32
accumulation.

1. Exactness of the tensor-core mapping: the result equals an FP64 product of the same
   rounded operands up to FP32 accumulation error (BF16: relative Frobenius <= 2e-5; 1e-4
   for Gaussian operators, whose entries this path computes with the hardware sine, cosine and
   logarithm, so that a small fraction of them round to the neighbouring BF16 value).  For
   e4m3 the reference rounds each column of A after dividing by one power-of-two scale over the
   whole column, the kernel per K slice; the two differ only for entries in e4m3's subnormal
   range, so the bound is 1e-3 there -- a wrong tile layout or descriptor gives O(1) errors.
2. Accuracy: relative Frobenius error against the FP64 product of the unrounded operator and
   data <= 1e-2 for BF16 (the target stated for this path), <= 6e-2 for e4m3 (3 mantissa
   bits).
Covers tails in every dimension, submatrix offsets (aligned and not), both operator
orientations, both layouts, alpha / beta, uniform and Gaussian operators."""
import numpy as np
import pytest

from gpu_helpers import to_dev, to_host

pytestmark = pytest.mark.gpu

CASES = [
    # d, n, m, ro_s, co_s, opS, layout, family, alpha, beta
    (128, 512, 256, 0, 0, 0, 1, 1, 1.0, 0.0),
    (300, 130, 5000, 3, 8, 0, 1, 1, 1.0, 0.0),
    (256, 1024, 6400, 0, 0, 0, 1, 0, 0.5, 0.0),
    (200, 77, 3001, 5, 6, 0, 0, 1, 1.0, 2.0),
    (140, 600, 1000, 7, 1, 1, 1, 1, -1.0, 0.0),
    (96, 40, 777, 0, 3, 1, 0, 0, 1.0, 0.5),
    # uniform operator over three 512-column tiles (cluster pairs sharing operator rows, the
    # 8-generator-warp form for BF16), column offset a multiple of 4, partial last tiles
    (200, 1030, 3000, 3, 4, 0, 1, 1, 1.0, 0.0),
    # several K slices written to the partial buffer by tensor stores: d = 300 leaves a
    # 32-row box reaching past the last row of each slice, n = 520 a 16-column box past n
    (300, 520, 6000, 0, 0, 0, 1, 1, 1.0, 0.0),
]


def _bf16(x):
    import torch
    return torch.as_tensor(x).to(torch.bfloat16).to(torch.float64)


def _e4m3(x):
    import torch
    return torch.as_tensor(x).to(torch.float8_e4m3fn).to(torch.float64)


def _e4m3_columns(A):
    """Each column of A (k x j) rounded to e4m3 after division by the smallest power of two
    that brings its largest magnitude to <= 448, then scaled back."""
    import torch
    amax = A.abs().amax(dim=0).clamp_min(1e-300)
    scale = torch.exp2(torch.ceil(torch.log2(amax / 448.0)))
    return _e4m3(A / scale) * scale


@pytest.mark.parametrize("prec", ["bf16", "fp8"])
@pytest.mark.parametrize("case", CASES)
def test_lowp(rb, oracle, case, prec):
    import torch
    from oracle.oracle import State
    from randblas_gb300 import lowp
    d, n, m, ro, co, opS, lay, fam, alpha, beta = case
    rows, cols = (d, m) if opS == 0 else (m, d)
    Dr, Dc = rows + ro + 2, cols + co + 3
    D = rb.DenseDist(Dr, Dc, rb.ScalarDist(fam))
    seed = rb.RNGState(17, counter=(9, 0, 0, 0))
    S = rb.DenseSkOp(D, seed)
    g = torch.Generator(device="cuda").manual_seed(3)
    Am = torch.randn(m, n, device="cuda", generator=g)        # op(A), m x n
    A = Am.contiguous() if lay == 1 else Am.T.contiguous()   # row-major / col-major storage
    lda = n if lay == 1 else m
    B0 = torch.randn(d, n, device="cuda", generator=g)
    B = B0.clone() if lay == 1 else B0.T.contiguous()
    ldb = n if lay == 1 else d
    precision = lowp.BF16 if prec == "bf16" else lowp.FP8_E4M3
    lowp.sketch_lowp(rb.Layout(lay), rb.Op(opS), rb.Op.NoTrans, d, n, m, alpha, S, ro, co, A,
                     lda, beta, B, ldb, precision=precision)
    assert lowp.status() == 0
    got = (B if lay == 1 else B.T).double().cpu()
    Ssub = torch.from_numpy(oracle.dense_matrix(0, Dr, Dc, fam, 1, State.make((9, 0, 0, 0),
                                                (17, 0)), rows, cols, ro, co))
    opSm = Ssub if opS == 0 else Ssub.T
    A64 = Am.double().cpu()
    if prec == "bf16":
        rounded = _bf16(opSm) @ _bf16(A64)
    else:
        rounded = _e4m3(opSm) @ _e4m3_columns(A64)
    exact_rounded = alpha * rounded + beta * B0.double().cpu()
    exact = alpha * (opSm.double() @ A64) + beta * B0.double().cpu()
    r1 = float((got - exact_rounded).norm() / exact_rounded.norm())
    r2 = float((got - exact).norm() / exact.norm())
    bound = 1e-3 if prec == "fp8" else (1e-4 if fam == 0 else 2e-5)
    assert r1 <= bound, (case, r1)
    assert r2 <= (1e-2 if prec == "bf16" else 6e-2), (case, r2)


@pytest.mark.parametrize("prec", ["bf16", "fp8"])
def test_lowp_tensor_store_padded_rows(rb, prec):
    """One K slice with beta = 0 and B's rows at a pitch of n + 4: the epilogue writes B by
    tensor stores whose boxes reach past row d and column n, which must be clipped there
    (the pitch padding keeps its value).  The same call with beta != 0 takes plain stores;
    both results agree to FP32 rounding."""
    import torch
    from randblas_gb300 import lowp
    d, n, m, ldb = 200, 100, 1000, 104
    S = rb.DenseSkOp(rb.DenseDist(d, m, rb.ScalarDist.Uniform), rb.RNGState(31))
    g = torch.Generator(device="cuda").manual_seed(9)
    A = torch.randn(m, n, device="cuda", generator=g)
    precision = lowp.BF16 if prec == "bf16" else lowp.FP8_E4M3
    B = torch.full((d + 3, ldb), 7.0, device="cuda")  # three rows past d as a guard
    lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 0.5, S, 0, 0,
                     A, n, 0.0, B.view(-1), ldb, precision=precision)
    Bp = torch.zeros((d, ldb), device="cuda")  # beta != 0 on zeros: the plain-store epilogue
    lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 0.5, S, 0, 0,
                     A, n, 1.0, Bp.view(-1), ldb, precision=precision)
    torch.cuda.synchronize()
    assert lowp.status() == 0
    assert bool((B[:d, n:] == 7.0).all()) and bool((B[d:] == 7.0).all())
    rel = float((B[:d, :n] - Bp[:, :n]).norm() / Bp[:, :n].norm())
    assert rel <= 1e-6, rel


@pytest.mark.parametrize("case", [
    # d, n, m, ro_s, co_s, family, precision: the operator enters transposed (tall, Short
    # axis: natural row-major, opS = Trans), so its natural rows follow k and, with co_s a
    # multiple of 4, each generator call covers 4 output rows (the transposed producer);
    # d = 202 leaves a partial quad, m = 3001 a partial last stage
    (202, 130, 3001, 5, 8, 1, "bf16"),
    (256, 520, 4096, 0, 0, 0, "bf16"),
    (202, 130, 3001, 5, 8, 1, "fp8"),
    (256, 64, 6000, 3, 4, 0, "fp8"),
])
def test_lowp_transposed_operator(rb, oracle, case):
    import torch
    from oracle.oracle import State
    from randblas_gb300 import lowp
    d, n, m, ro, co, fam, prec = case
    Dr, Dc = m + ro + 3, d + co + 4          # S is Dr x Dc, op(submat(S)) = submat(S)^T
    D = rb.DenseDist(Dr, Dc, rb.ScalarDist(fam), rb.Axis.Short)
    assert D.natural_layout == rb.Layout.RowMajor
    S = rb.DenseSkOp(D, rb.RNGState(23, counter=(4, 0, 0, 0)))
    g = torch.Generator(device="cuda").manual_seed(7)
    A = torch.randn(m, n, device="cuda", generator=g)
    B = torch.empty(d, n, device="cuda")
    precision = lowp.BF16 if prec == "bf16" else lowp.FP8_E4M3
    lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.Trans, rb.Op.NoTrans, d, n, m, 1.0, S, ro, co, A,
                     n, 0.0, B, n, precision=precision)
    assert lowp.status() == 0
    Ssub = torch.from_numpy(oracle.dense_matrix(0, Dr, Dc, fam, 0, State.make((4, 0, 0, 0),
                                                (23, 0)), m, d, ro, co))
    opSm = Ssub.T
    A64 = A.double().cpu()
    if prec == "bf16":
        rounded = _bf16(opSm) @ _bf16(A64)
    else:
        rounded = _e4m3(opSm) @ _e4m3_columns(A64)
    got = B.double().cpu()
    r1 = float((got - rounded).norm() / rounded.norm())
    bound = 1e-3 if prec == "fp8" else (1e-4 if fam == 0 else 2e-5)
    assert r1 <= bound, (case, r1)


@pytest.mark.parametrize("lay", [1, 0])
def test_lowp_host_a_and_b_streamed(rb, lay):
    """A and B both in pinned host memory, K streamed in seven chunks: the chunks accumulate into
    a device copy of B (read once for beta, written back once), in either layout and with
    leading-dimension padding, which stays untouched.  Same bound as against device buffers."""
    import torch
    from randblas_gb300 import lowp
    d, n, m = 200, 96, 300000
    S = rb.DenseSkOp(rb.DenseDist(d, m, rb.ScalarDist.Uniform), rb.RNGState(14))
    g = torch.Generator(device="cuda").manual_seed(8)
    Am = torch.randn(m, n, device="cuda", generator=g)
    Bm = torch.randn(d, n, device="cuda", generator=g)
    if lay == 1:
        A, lda = Am.contiguous(), n
        ldb = n + 5
        Bbuf = torch.full((d, ldb), 7.0, device="cuda")
        Bbuf[:, :n] = Bm
    else:
        A, lda = Am.T.contiguous(), m
        ldb = d + 3
        Bbuf = torch.full((n, ldb), 7.0, device="cuda")
        Bbuf[:, :d] = Bm.T
    B_dev = Bbuf.clone()
    lowp.sketch_lowp(rb.Layout(lay), rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 0.5, S, 0, 0, A,
                     lda, 0.25, B_dev.view(-1), ldb)
    A_host = A.cpu().pin_memory()
    B_host = Bbuf.cpu().pin_memory()
    lowp.sketch_lowp(rb.Layout(lay), rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 0.5, S, 0, 0,
                     A_host, lda, 0.25, B_host.view(-1), ldb)
    torch.cuda.synchronize()
    assert lowp.status() == 0
    got, want = B_host.double(), B_dev.cpu().double()
    inner = (slice(None), slice(0, n)) if lay == 1 else (slice(None), slice(0, d))
    pad = (slice(None), slice(n, ldb)) if lay == 1 else (slice(None), slice(d, ldb))
    rel = float((got[inner] - want[inner]).norm() / want[inner].norm())
    assert rel <= 2e-5, rel
    assert bool((got[pad] == 7.0).all())


def test_lowp_workspace_and_errors(rb):
    import torch
    from randblas_gb300 import lowp
    D = rb.DenseDist(256, 4096, rb.ScalarDist.Uniform)
    S = rb.DenseSkOp(D, rb.RNGState(1))
    A = torch.randn(4096, 64, device="cuda")
    need = lowp.workspace_bytes(lowp.BF16, 256, 64, 4096)
    ws = torch.empty(need + 1024, dtype=torch.uint8, device="cuda")
    off = (-ws.data_ptr()) % 1024
    ws_al = ws[off:off + need]
    B1 = torch.empty(256, 64, device="cuda")
    B2 = torch.empty(256, 64, device="cuda")
    lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, 256, 64, 4096, 1.0, S, 0,
                     0, A, 64, 0.0, B1, 64, workspace=ws_al)
    lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, 256, 64, 4096, 1.0, S, 0,
                     0, A, 64, 0.0, B2, 64)
    assert torch.equal(B1, B2)  # deterministic, caller workspace or not
    with pytest.raises(rb.RandBLASError):
        lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, 256, 64, 4096, 1.0, S,
                         0, 0, A, 63, 0.0, B1, 64)
    with pytest.raises(rb.RandBLASError):
        lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, 256, 64, 4096, 1.0, S,
                         0, 0, A, 64, 0.0, B1, 64, workspace=ws_al[:need - 1024])
    # the workspace must be memory of this GPU: pinned host memory is refused by the C ABI
    # (and by the Python front end before it), B is left as it was
    import ctypes as C
    host_ws = torch.empty(need + 1024, dtype=torch.uint8, pin_memory=True)
    hoff = (-host_ws.data_ptr()) % 1024
    B3 = torch.full((256, 64), 7.0, device="cuda")
    sc = S._c()
    rc = rb.lib().rbg_lskge3_lowp(lowp.BF16, 1, 0, 0, 256, 64, 4096, 1.0, C.byref(sc), 0, 0,
                                  C.c_void_p(A.data_ptr()), 64, 0.0, C.c_void_p(B3.data_ptr()),
                                  64, C.c_void_p(host_ws.data_ptr() + hoff), need,
                                  C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == rb._lib.ERROR_INVALID_ARGUMENT
    assert "workspace must be device memory of the current GPU" in \
        rb.lib().rbg_last_error().decode()
    with pytest.raises(rb.RandBLASError):
        lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, 256, 64, 4096, 1.0, S,
                         0, 0, A, 64, 0.0, B3, 64, workspace=host_ws[hoff:hoff + need])
    assert bool((B3 == 7.0).all())
    assert lowp.status() == 0


@pytest.mark.parametrize("prec", ["bf16", "fp8"])
@pytest.mark.parametrize("m,beta", [(9000, 0.25), (1500, 0.0)])
def test_lowp_host_buffers(rb, prec, m, beta):
    """A and B in pinned host memory, passed to the call itself (the A conversion pass reads A
    over the host link, B is written in place): the same bits as with device buffers.  With
    m = 1500 (one K slice) and beta = 0 the device call writes B by tensor stores and the host
    call by plain stores, so this also compares the two epilogues."""
    import torch
    from randblas_gb300 import lowp
    d, n = 256, 192
    S = rb.DenseSkOp(rb.DenseDist(d, m, rb.ScalarDist.Gaussian), rb.RNGState(12))
    g = torch.Generator(device="cuda").manual_seed(4)
    A = torch.randn(m, n, device="cuda", generator=g)
    B0 = torch.randn(d, n, device="cuda", generator=g)
    precision = lowp.BF16 if prec == "bf16" else lowp.FP8_E4M3
    B_dev = B0.clone()
    lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 0.5, S, 0, 0, A,
                     n, beta, B_dev, n, precision=precision)
    A_host = A.cpu().pin_memory()
    B_host = B0.cpu().pin_memory()
    lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 0.5, S, 0, 0,
                     A_host, n, beta, B_host, n, precision=precision)
    torch.cuda.synchronize()
    assert lowp.status() == 0
    assert torch.equal(B_host, B_dev.cpu())


@pytest.mark.parametrize("axis", ["Long", "Short"])
def test_lowp_host_a_streamed(rb, axis):
    """BF16 with A in pinned host memory, K = 300,000 rows in four 2^16-row chunks and then
    quarter chunks for the last 37,856 rows (16,384, 16,384 and 5,088): the copy engine brings
    chunk c + 1 in while the call converts and sketches chunk c, adding the chunks into B.
    The rounded operands are the same as with device buffers; only the K slices over which the
    tensor cores accumulate in FP32 differ, so the two results agree within the path's
    FP32-accumulation bound (2e-5 relative Frobenius, as against an FP64 product of the rounded
    operands).  Both operator orientations (the chunk offset moves the operator's columns or
    its rows)."""
    import torch
    from randblas_gb300 import lowp
    d, n, m = 200, 96, 300000
    S = rb.DenseSkOp(rb.DenseDist(d, m, rb.ScalarDist.Gaussian, getattr(rb.Axis, axis)),
                     rb.RNGState(13))
    g = torch.Generator(device="cuda").manual_seed(6)
    A = torch.randn(m, n, device="cuda", generator=g)
    B0 = torch.randn(d, n, device="cuda", generator=g)
    B_dev = B0.clone()
    lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 0.5, S, 0, 0, A,
                     n, 0.25, B_dev, n)
    A_host = A.cpu().pin_memory()
    B_str = B0.clone()
    rb.profile.enable(True)
    try:
        lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 0.5, S, 0, 0,
                         A_host, n, 0.25, B_str, n)
        torch.cuda.synchronize()
        launches = rb.profile.read()["lowp_sketch_bf16_tc"]["launches"]
    finally:
        rb.profile.enable(False)
    assert lowp.status() == 0
    assert launches == 7, launches
    rel = float((B_str.double() - B_dev.double()).norm() / B_dev.double().norm())
    assert rel <= 2e-5, rel


@pytest.mark.parametrize("prec", ["bf16", "fp8"])
@pytest.mark.parametrize("lay", [1, 0])
def test_lowp_transposed_data(rb, prec, lay):
    """op(A) = A^T: the data stored transposed and read with opA = Trans gives the same bits
    as the untransposed data with opA = NoTrans (the conversion pass builds the same k-blocked
    copy from either layout), in both layouts."""
    import torch
    from randblas_gb300 import lowp
    d, n, m = 200, 96, 3000
    S = rb.DenseSkOp(rb.DenseDist(d, m, rb.ScalarDist.Uniform), rb.RNGState(41))
    g = torch.Generator(device="cuda").manual_seed(41)
    Am = torch.randn(m, n, device="cuda", generator=g)          # op(A), m x n
    precision = lowp.BF16 if prec == "bf16" else lowp.FP8_E4M3
    row = lay == 1
    # NoTrans: A itself in the layout; Trans: A^T (n x m) in the layout
    A_nt, lda_nt = (Am.contiguous(), n) if row else (Am.T.contiguous(), m)
    A_t, lda_t = (Am.T.contiguous(), m) if row else (Am.contiguous(), n)
    shape_b = (d, n) if row else (n, d)
    ldb = n if row else d
    B1 = torch.zeros(shape_b, device="cuda")
    B2 = torch.zeros(shape_b, device="cuda")
    lowp.sketch_lowp(rb.Layout(lay), rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 1.0, S, 0, 0, A_nt,
                     lda_nt, 0.0, B1, ldb, precision=precision)
    lowp.sketch_lowp(rb.Layout(lay), rb.Op.NoTrans, rb.Op.Trans, d, n, m, 1.0, S, 0, 0, A_t,
                     lda_t, 0.0, B2, ldb, precision=precision)
    torch.cuda.synchronize()
    assert lowp.status() == 0
    assert torch.equal(B1, B2)
    assert float(B1.abs().sum()) > 0.0
