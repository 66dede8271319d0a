"""Per-kernel CUDA-event timing exposed by the library (rbg_profile_*)."""
from __future__ import annotations

import ctypes as C

from ._lib import call


def enable(on: bool = True) -> None:
    """Start (and clear) or stop recording events around the library's main kernels."""
    call("rbg_profile_enable", 1 if on else 0)


def read() -> dict:
    """{kernel name: {"ms": total milliseconds, "launches": count}} recorded so far."""
    n = C.c_int32()
    call("rbg_profile_count", C.byref(n))
    out = {}
    for i in range(n.value):
        name = C.create_string_buffer(128)
        ms = C.c_double()
        k = C.c_int64()
        call("rbg_profile_entry", i, name, 128, C.byref(ms), C.byref(k))
        out[name.value.decode()] = {"ms": ms.value, "launches": k.value}
    return out
