"""Scale granularity of the e4m3 precision form, on the CPU.

The tensor-core e4m3 sketch scales A by one power of two per (K slice, column) and feeds the
operator's entries unscaled (they lie in [-sqrt 3, sqrt 3], well inside e4m3's range).  A
finer scheme -- one power-of-two scale per 128 x 128 tile of A and of the operator, applied per
k tile as a block-scaled MMA would -- changes the error only where tiles differ in magnitude by
more than e4m3's exponent range covers.  On the precision workload's data (A = U diag(s) V^T,
singular values from 1 to 1e-6, random orthogonal factors; uniform operator) both schemes give
the same relative Frobenius error to three digits: e4m3's 3-bit mantissa sets it, not the
scales.  This test emulates both schemes in FP64 at a reduced size (d = 512, m = 2^15,
n = 256) and pins that, next to the BF16 error for scale."""
import math

import pytest

torch = pytest.importorskip("torch")


def _p2scale(amax):
    return torch.exp2(torch.ceil(torch.log2(torch.clamp(amax, min=1e-300) / 448.0)))


def _e4m3(x):
    return x.to(torch.float8_e4m3fn).to(torch.float64)


def test_tile_scales_match_slice_column_scales():
    m, n, d, tile = 1 << 15, 256, 512, 128
    g = torch.Generator().manual_seed(1)
    U, _ = torch.linalg.qr(torch.randn(m, n, dtype=torch.float64, generator=g))
    V, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, generator=g))
    A = (U * torch.logspace(0, -6, n, dtype=torch.float64)) @ V.T
    S = (torch.rand(d, m, dtype=torch.float64, generator=g) * 2 - 1) * math.sqrt(3)
    exact = S @ A

    def rel(B):
        return float((B - exact).norm() / exact.norm())

    # the kernel's scheme: K cut into slices, one scale per (slice, column) of A
    errs = {}
    for slices in (1, 8):
        ks = m // slices
        B = torch.zeros(d, n, dtype=torch.float64)
        for s0 in range(0, m, ks):
            Ab = A[s0:s0 + ks]
            sc = _p2scale(Ab.abs().amax(0))
            B += _e4m3(S[:, s0:s0 + ks]) @ (_e4m3(Ab / sc) * sc)
        errs[slices] = rel(B)
    # 128 x 128 tiles of A (k, j) and of the operator (i, k), scales applied per k tile
    B = torch.zeros(d, n, dtype=torch.float64)
    for k0 in range(0, m, tile):
        Ab = A[k0:k0 + tile].reshape(tile, n // tile, tile)
        sa = _p2scale(Ab.abs().amax(dim=(0, 2)))[None, :, None]
        Sb = S[:, k0:k0 + tile].reshape(d // tile, tile, tile)
        ss = _p2scale(Sb.abs().amax(dim=(1, 2)))[:, None, None]
        B += (_e4m3(Sb / ss) * ss).reshape(d, tile) @ (_e4m3(Ab / sa) * sa).reshape(tile, n)
    tiled = rel(B)
    bf16 = rel(S.to(torch.bfloat16).double() @ A.to(torch.bfloat16).double())
    print("e4m3 rel. Frobenius error: per (slice, column)", errs, "per 128-tile", tiled,
          "| BF16", bf16)
    assert 0.02 < errs[8] < 0.06
    assert abs(tiled - errs[8]) <= 0.01 * errs[8]
    assert abs(errs[1] - errs[8]) <= 0.01 * errs[8]
    assert bf16 < 0.1 * errs[8]
