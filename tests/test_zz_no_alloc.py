"""rbg_lskge3_noalloc, the allocation-free variant of the left dense sketch, called through the
C ABI: its output must match rbg_lskge3's on the same inputs, on consecutive calls that share
its fixed scratch array, and sizes beyond its limit must be rejected with a clear error.

Some callers cannot allocate device memory while they run -- a CUDA graph captured with a
fixed memory plan, or a host that forbids allocation after start-up -- which is why this entry
point keeps its split-K partial sums in a fixed device array instead."""
import ctypes as C
import ctypes.util
import glob
import os

import pytest

pytestmark = pytest.mark.gpu


def _skop(rb, dist, seed, dtype):
    import torch
    S = rb.DenseSkOp(dist, seed, dtype=dtype)
    return S._c()


def _run(rb, name, layout, d, n, m, alpha, sk, ro, co, A, lda, beta, B, ldb):
    import torch
    fn = getattr(rb.lib(), name)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = fn(layout, 0, 0, d, n, m, alpha, C.byref(sk), ro, co, C.c_void_p(A.data_ptr()), lda,
            beta, C.c_void_p(B.data_ptr()), ldb, stream)
    return rc


CASES = [
    # dtype, layout, family, d, n, m, ro_s, co_s, alpha, beta, rel tolerance
    ("f64", 0, 0, 200, 50, 10000, 0, 0, 1.0, 0.0, 1e-12),
    ("f32", 1, 1, 300, 130, 20000, 3, 5, 1.5, -0.5, 1e-6),
]


def _case(rb, case, seed_key):
    import torch
    dt, lay, fam, d, n, m, ro, co, alpha, beta, tol = case
    tdt = torch.float64 if dt == "f64" else torch.float32
    dist = rb.DenseDist(d + ro + 1, m + co + 2, rb.ScalarDist(fam))
    sk = _skop(rb, dist, rb.RNGState(seed_key), tdt)
    g = torch.Generator(device="cuda").manual_seed(seed_key)
    A = torch.randn(m * n, device="cuda", dtype=tdt, generator=g)
    lda = m if lay == 0 else n
    B0 = torch.randn(d * n, device="cuda", dtype=tdt, generator=g)
    ldb = d if lay == 0 else n
    B_ref, B_new = B0.clone(), B0.clone()
    assert _run(rb, "rbg_lskge3", lay, d, n, m, alpha, sk, ro, co, A, lda, beta, B_ref, ldb) == 0
    assert _run(rb, "rbg_lskge3_noalloc", lay, d, n, m, alpha, sk, ro, co, A, lda, beta, B_new,
                ldb) == 0, rb.lib().rbg_last_error()
    torch.cuda.synchronize()
    rel = float(torch.linalg.norm(B_new - B_ref) / torch.linalg.norm(B_ref))
    assert rel <= tol, (case, rel)
    return B_new


def test_noalloc_matches_allocating_entry_point(rb):
    import torch
    first = _case(rb, CASES[0], 11)    # call 1
    _case(rb, CASES[1], 12)            # call 2 reuses the same scratch array
    again = _case(rb, CASES[0], 11)    # call 3: same inputs as call 1
    assert torch.equal(first, again)


def test_noalloc_rejects_sizes_beyond_its_limit(rb):
    import torch
    d, n, m = 4096, 2048, 64  # 4096 * 2048 * 4 bytes = 32 MiB > 16 MiB
    sk = _skop(rb, rb.DenseDist(d, m), rb.RNGState(1), torch.float32)
    A = torch.zeros(m * n, device="cuda")
    B = torch.zeros(d * n, device="cuda")
    rc = _run(rb, "rbg_lskge3_noalloc", 1, d, n, m, 1.0, sk, 0, 0, A, n, 0.0, B, n)
    assert rc == 1
    msg = rb.lib().rbg_last_error().decode()
    assert "exceeds its limit" in msg and "rbg_lskge3" in msg


# cudaMemPoolAttr values (driver_types.h)
_RESERVED_CURRENT, _RESERVED_HIGH, _USED_CURRENT, _USED_HIGH = 5, 6, 7, 8


def _cudart():
    """The CUDA runtime, for device-wide memory queries (any copy in the process sees the same
    device memory pools)."""
    import torch
    cands = [ctypes.util.find_library("cudart"), "/usr/local/cuda/lib64/libcudart.so"]
    tdir = os.path.dirname(torch.__file__)
    cands += sorted(glob.glob(os.path.join(tdir, "lib", "libcudart*.so*")))
    cands += sorted(glob.glob(os.path.join(os.path.dirname(tdir), "nvidia", "*", "lib",
                                           "libcudart.so*")))
    cands += sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))
    for c in cands:
        if c and os.path.exists(c) or (c and "/" not in c):
            try:
                return C.CDLL(c)
            except OSError:
                continue
    pytest.fail("no CUDA runtime library found for the memory queries")


class _MemProbe:
    """The default memory pool's used/reserved bytes and high-water marks, plus cudaMemGetInfo."""

    def __init__(self):
        import torch
        self.rt = _cudart()
        self.pool = C.c_void_p()
        assert self.rt.cudaDeviceGetDefaultMemPool(C.byref(self.pool),
                                                   torch.cuda.current_device()) == 0

    def attr(self, a):
        v = C.c_uint64()
        assert self.rt.cudaMemPoolGetAttribute(self.pool, a, C.byref(v)) == 0
        return v.value

    def reset_highs(self):
        zero = C.c_uint64(0)
        for a in (_USED_HIGH, _RESERVED_HIGH):
            assert self.rt.cudaMemPoolSetAttribute(self.pool, a, C.byref(zero)) == 0

    def snapshot(self):
        free, total = C.c_size_t(), C.c_size_t()
        assert self.rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
        return {"used": self.attr(_USED_CURRENT), "used_high": self.attr(_USED_HIGH),
                "reserved": self.attr(_RESERVED_CURRENT),
                "reserved_high": self.attr(_RESERVED_HIGH), "free": free.value}


def test_noalloc_allocates_nothing(rb):
    """A warmed-up call changes neither the stream-ordered pool's used or reserved bytes (nor
    their high-water marks) nor the device's free memory.  The same probe around the
    allocating entry point shows that it does allocate split-K scratch on this case, so the
    case really uses the fixed array in the allocation-free variant."""
    import torch
    dt, lay, fam, d, n, m, ro, co, alpha, beta, tol = CASES[0]
    dist = rb.DenseDist(d + ro + 1, m + co + 2, rb.ScalarDist(fam))
    sk = _skop(rb, dist, rb.RNGState(21), torch.float64)
    g = torch.Generator(device="cuda").manual_seed(21)
    A = torch.randn(m * n, device="cuda", dtype=torch.float64, generator=g)
    B = torch.zeros(d * n, device="cuda", dtype=torch.float64)
    probe = _MemProbe()

    def call(name):
        assert _run(rb, name, lay, d, n, m, alpha, sk, ro, co, A, m, beta, B, d) == 0, \
            rb.lib().rbg_last_error()
        torch.cuda.synchronize()

    call("rbg_lskge3_noalloc")  # warm-up: first call on the device, module loading
    call("rbg_lskge3")
    probe.reset_highs()
    before = probe.snapshot()
    call("rbg_lskge3_noalloc")
    call("rbg_lskge3_noalloc")
    after = probe.snapshot()
    assert after["used_high"] <= before["used"], (before, after)
    assert after["reserved_high"] <= before["reserved"], (before, after)
    assert after["used"] == before["used"] and after["reserved"] == before["reserved"]
    assert after["free"] == before["free"], (before, after)
    # positive control: the allocating entry point takes stream-ordered scratch here
    probe.reset_highs()
    base = probe.snapshot()
    call("rbg_lskge3")
    assert probe.snapshot()["used_high"] > base["used"], "control case needs no scratch"
