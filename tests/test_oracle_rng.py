"""The oracle's Philox, counter arithmetic and transforms against the reference's own
known-answer vectors and asserts (CPU only)."""
import math
import struct

import numpy as np
import pytest

from conftest import golden_json


def test_philox_kat(oracle):
    # test/test_basic_rng/r123_kat_vectors.txt:19-21, parsed into tests/golden/philox_kat.json
    rows = golden_json("philox_kat.json")
    assert len(rows) == 3
    for r in rows:
        assert list(oracle.philox(r["ctr"], r["key"])) == r["out"]


def test_state_from_key(oracle):
    # test/test_basic_rng/test_r123.cc:675-703: RNGState(42) -> key {42, 0}, counter 0
    from oracle.oracle import State
    s = State.from_key(42)
    assert list(s.key) == [42, 0] and list(s.counter) == [0, 0, 0, 0]


def test_counter_increment(oracle):
    # the 128-bit carry semantics asserted at test/test_basic_rng/test_r123.cc:705-797
    i32max = 2**32 - 1
    c = (0, 0, 0, 0)
    c = oracle.ctr_add(c, i32max)
    assert c == (i32max, 0, 0, 0)
    c = oracle.ctr_add(c, 1)
    assert c == (0, 1, 0, 0)
    c = oracle.ctr_add(c, 3)
    assert c == (3, 1, 0, 0)
    assert oracle.ctr_add((0, 0, 0, 0), 2**32 - 1) == (i32max, 0, 0, 0)
    assert oracle.ctr_add((0, 0, 0, 0), 2**32) == (0, 1, 0, 0)
    c = oracle.ctr_add((0, 0, 0, 0), 2**63)
    c = oracle.ctr_add(c, 2**63 - 2**32)
    assert c == (0, i32max, 0, 0)
    assert oracle.ctr_add(c, 2**32) == (0, 0, 1, 0)
    assert oracle.ctr_add((i32max, i32max, i32max, 0), 1) == (0, 0, 0, 1)


def _f32(x):
    return struct.unpack("f", struct.pack("f", x))[0]


def test_transforms_ranges(oracle):
    # one rounding after an exact scaling; in float the extremes round onto the interval's
    # ends, so uneg11 is in [-1, 1] and never 0, and u01 is in (0, 1]
    for u in (0, 1, 2**31 - 1, 2**31, 2**32 - 1, 12345, 3**20):
        v = oracle.uneg11(u)
        s = u - 2**32 if u >= 2**31 else u
        assert v == _f32(_f32(float(s)) * 2.0**-31 + 2.0**-32)
        assert -1.0 <= v <= 1.0 and v != 0.0
        w = oracle.u01(u)
        assert w == _f32(_f32(float(u)) * 2.0**-32 + 2.0**-33)
        assert 0.0 < w <= 1.0


def test_boxmuller_definition(oracle):
    # boxmuller(u0, u1) = (sin(pi*uneg11(u0)) * r, cos(pi*uneg11(u0)) * r), r = sqrt(-2 ln u01(u1))
    rng = np.random.default_rng(0)
    for u0, u1 in rng.integers(0, 2**32, size=(200, 2)):
        a, b = oracle.boxmuller(int(u0), int(u1))
        th = math.pi * oracle.uneg11(int(u0))
        r = math.sqrt(-2.0 * math.log(oracle.u01(int(u1))))
        assert a == pytest.approx(math.sin(th) * r, rel=1e-5, abs=1e-6)
        assert b == pytest.approx(math.cos(th) * r, rel=1e-5, abs=1e-6)
