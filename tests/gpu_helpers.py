"""Helpers shared by the GPU parity tests."""
import numpy as np


def to_dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def to_host(t):
    return t.detach().cpu().numpy()


def ulp_distance(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Distance in units in the last place between float32 arrays (same sign assumed for
    nonzero pairs; distinct signs count as the sum of both distances to zero)."""
    ai = a.astype(np.float32).view(np.int32).astype(np.int64)
    bi = b.astype(np.float32).view(np.int32).astype(np.int64)
    ai = np.where(ai < 0, -(ai & 0x7FFFFFFF), ai)
    bi = np.where(bi < 0, -(bi & 0x7FFFFFFF), bi)
    return np.abs(ai - bi)


def state_of(st_list):
    import randblas_gb300 as rb
    return rb.RNGState(counter=st_list[0], key_words=st_list[1])


def st_list(s):
    return [list(s.counter), list(s.key)]


def as_matrix(flat, rows, cols, layout, ld):
    """The rows x cols matrix stored in `flat` with `layout` (0 col-major, 1 row-major)."""
    flat = np.asarray(flat)
    if layout == 0:
        return flat[:ld * cols].reshape(cols, ld)[:, :rows].T
    return flat[:ld * rows].reshape(rows, ld)[:, :cols]


def check_bound(got, ref, bound, what=""):
    """|got - ref| <= bound elementwise (the componentwise criterion of the reference's
    test/test_matmul_cores/linop_common.hh:260-266, with the slack stated by the caller)."""
    err = np.abs(got.astype(np.float64) - ref.astype(np.float64))
    bad = err > bound
    assert not bad.any(), (what, float(err.max()), float(bound[bad].min()) if bad.any() else 0.0,
                           int(bad.sum()))
