"""The random sparse generators' host-side bookkeeping through the C ABI, CPU only: for
densities 0 and 1 no device work is needed, so the handle's nnz and next state can be checked
against the oracle (random_matrix.hh:141-160, 219-238, 298-313), together with the reference's
density check and this library's limits."""
import ctypes as C

import pytest

from oracle.oracle import State


def _create(rb, fmt, m, n, density, key):
    lib = rb._lib
    h = C.c_void_p()
    nnz = C.c_int64()
    nxt = lib.rbg_state()
    seed = rb.RNGState(key)._c()
    lib.call("rbg_random_sparse_create", fmt, m, n, float(density), C.byref(seed), C.byref(h),
             C.byref(nnz), C.byref(nxt), None)
    lib.call("rbg_random_sparse_destroy", h)
    return nnz.value, (tuple(nxt.counter), tuple(nxt.key))


@pytest.mark.parametrize("fmt", [0, 1, 2])
def test_density_zero_and_one_bookkeeping(rb_host, oracle, fmt):
    for (m, n) in [(5, 8), (7, 9), (1, 1), (0, 10), (10, 0), (300, 7)]:
        for density in (0.0, 1.0):
            key = 1000 + m + 7 * n
            nnz, nxt = _create(rb_host, fmt, m, n, density, key)
            vals, _, _, onx = oracle.random_sparse(fmt, 0, 1, m, n, density, State.from_key(key))
            assert nnz == vals.size, (fmt, m, n, density)
            assert nxt == onx.tuple(), (fmt, m, n, density)


def test_density_checks(rb_host):
    for fmt, name in ((0, "random_coo"), (1, "random_csr"), (2, "random_csc")):
        with pytest.raises(rb_host.RandBLASError) as e:
            _create(rb_host, fmt, 4, 4, 1.5, 1)
        assert str(e.value) == ("(density >= 0.0 && density <= 1.0) was required, but did not "
                                f"hold, in function {name}")
    with pytest.raises(rb_host.RandBLASError):
        _create(rb_host, 1, 4, 4, float("nan"), 1)
    with pytest.raises(rb_host.RandBLASError) as e:
        _create(rb_host, 1, 4, 4, 1e-20, 1)  # log(1 - density) rounds to 0
    assert e.value.code == rb_host._lib.ERROR_UNSUPPORTED
    with pytest.raises(rb_host.RandBLASError):
        _create(rb_host, 3, 4, 4, 0.5, 1)  # not a format
