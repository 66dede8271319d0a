"""Batching path: many independent left dense sketches of uneven shapes,

    B_i = alpha_i * submat(S_i) * A_i + beta_i * B_i      (LSKGE3 semantics, T = float),

in one persistent launch of the library's batched kernel (rbg_lskge3_batched /
rbg_batched_plan_*).  No reference counterpart: the reference sketches one problem per call
(RandBLAS/skge.hh:154-202).  Each problem has its own generated operator S_i (its own
RNGState), data A_i and output B_i, all row-major or all column-major CUDA tensors.

* :func:`sketch_batched` -- one stream-ordered call.
* :class:`BatchedPlan` -- validate and upload once, then :meth:`BatchedPlan.execute` (a memset
  and one kernel launch, capturable) or :meth:`BatchedPlan.capture` into a CUDA graph.
* :class:`Autotuner` -- picks each problem's output tile (128 x 128, 128 x 64, 128 x 32,
  64 x 256, or 128-row blocks over all columns) per shape class by timing every candidate on
  the same synthetic batch on the device, and caches the choices as JSON.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
import threading
from dataclasses import dataclass
from typing import Callable, Dict, List, Optional, Sequence

import torch

from . import _lib
from ._lib import ERROR_INVALID_ARGUMENT, RandBLASError, call
from .api import DenseSkOp, Layout, _stream


@dataclass
class BatchProblem:
    """One left sketch of a batch; lda / ldb default to the tight leading dimensions."""
    S: DenseSkOp
    A: torch.Tensor
    B: torch.Tensor
    d: int
    n: int
    m: int
    alpha: float = 1.0
    beta: float = 0.0
    ro_s: int = 0
    co_s: int = 0
    lda: Optional[int] = None
    ldb: Optional[int] = None
    tile_config: int = 0


def tile_configs() -> List[int]:
    n = C.c_int32()
    call("rbg_batched_tile_configs", C.byref(n))
    return list(range(1, n.value + 1))


def tile_shape(config: int):
    """(rows, columns) of the output tile of a configuration; columns 0 is a row block over
    every column of the problem (operator rows generated once, used by every 128-column
    pass)."""
    r, c = C.c_int32(), C.c_int32()
    call("rbg_batched_tile_shape", int(config), C.byref(r), C.byref(c))
    return r.value, c.value


def _c_problems(problems: Sequence[BatchProblem], layout: Layout):
    arr = (_lib.rbg_batch_problem * max(len(problems), 1))()
    for i, p in enumerate(problems):
        for t, what in ((p.A, "A"), (p.B, "B")):
            if not t.is_cuda or t.dtype != torch.float32:
                raise RandBLASError(ERROR_INVALID_ARGUMENT, f"{what} must be an FP32 CUDA tensor")
        if p.S.dtype != torch.float32 or p.S.buff is not None:
            raise RandBLASError(ERROR_INVALID_ARGUMENT,
                                "batched operators are FP32 and generated (unfilled)")
        row = Layout(layout) == Layout.RowMajor
        lda = p.lda if p.lda is not None else (p.n if row else p.m)
        ldb = p.ldb if p.ldb is not None else (p.n if row else p.d)
        q = arr[i]
        q.d, q.n, q.m = p.d, p.n, p.m
        q.dist = p.S.dist._c()
        q.seed = p.S.seed_state._c()
        q.ro_s, q.co_s = p.ro_s, p.co_s
        q.A, q.lda = p.A.data_ptr(), lda
        q.B, q.ldb = p.B.data_ptr(), ldb
        q.alpha, q.beta = float(p.alpha), float(p.beta)
        q.tile_config = int(p.tile_config)
    return arr


def sketch_batched(problems: Sequence[BatchProblem], layout: Layout = Layout.RowMajor,
                   tile_config: int = 0, tuner: Optional["Autotuner"] = None) -> None:
    """All problems in one persistent launch on the current stream (stream-ordered)."""
    if tuner is not None:
        tuner.assign(problems)
    arr = _c_problems(problems, layout)
    call("rbg_lskge3_batched", int(layout), arr, len(problems), int(tile_config), _stream())


class BatchedPlan:
    """A batch validated and uploaded once; execute() is a memset plus one kernel launch on
    the current stream.  The plan keeps references to the problems' tensors."""

    def __init__(self, problems: Sequence[BatchProblem], layout: Layout = Layout.RowMajor,
                 tile_config: int = 0, tuner: Optional["Autotuner"] = None):
        if tuner is not None:
            tuner.assign(problems)
        self._keep = [(p.A, p.B) for p in problems]
        arr = _c_problems(problems, layout)
        h = C.c_void_p()
        call("rbg_batched_plan_create", int(layout), arr, len(problems), int(tile_config),
             C.byref(h))
        self._h = h
        self.flops = sum(2.0 * p.d * p.n * p.m for p in problems)

    def execute(self) -> None:
        if self._h is None:
            raise RandBLASError(ERROR_INVALID_ARGUMENT, "plan is closed")
        call("rbg_batched_plan_execute", self._h, _stream())

    def info(self):
        items, nbytes = C.c_int64(), C.c_int64()
        call("rbg_batched_plan_info", self._h, C.byref(items), C.byref(nbytes))
        return {"work_items": items.value, "device_bytes": nbytes.value}

    def capture(self) -> torch.cuda.CUDAGraph:
        """A CUDA graph holding one execute(); replay() reruns the whole batch."""
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self.execute()  # warm-up outside the capture
        torch.cuda.current_stream().wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.execute()
        return g

    def close(self) -> None:
        if self._h is not None:
            torch.cuda.synchronize()
            call("rbg_batched_plan_destroy", self._h)
            self._h = None

    def __del__(self):
        try:
            if self._h is not None and _lib is not None:
                _lib.lib().rbg_batched_plan_destroy(self._h)
        except Exception:
            pass


def _default_cache_path() -> str:
    env = os.environ.get("RBG_AUTOTUNE_CACHE")
    if env:
        return env
    return os.path.join(os.path.expanduser("~"), ".cache", "randblas_gb300", "batched_tiles.json")


class Autotuner:
    """Per-shape-class choice of the batched kernel's output tile.

    A problem's class is (operator family, d, n rounded up to powers of two, round(log2 m)).
    The first time a class is seen on a device, one synthetic batch of that class (problems
    enough to fill the device, N(0,1) data, m capped at ``m_cap``) runs once per tile
    configuration and once with the library's own choice (configuration 0).  A configuration
    replaces the library's choice only when it is faster by more than ``margin`` (the
    synthetic batch stands in for the real one, so small differences are not trusted).
    Choices are stored in a JSON file keyed by device name, so later processes reuse them.
    ``measure(config, d, n, m, family) -> seconds`` can replace the device timing (tests)."""

    def __init__(self, cache_path: Optional[str] = None,
                 measure: Optional[Callable[[int, int, int, int, int], float]] = None,
                 m_cap: int = 1 << 15, margin: float = 0.03):
        self.cache_path = cache_path or _default_cache_path()
        self._external = measure
        self.m_cap = m_cap
        self.margin = margin
        self._lock = threading.Lock()
        self.cache: Dict[str, Dict[str, int]] = {}
        if os.path.exists(self.cache_path):
            try:
                with open(self.cache_path) as f:
                    self.cache = json.load(f)
            except (OSError, ValueError):
                self.cache = {}

    @staticmethod
    def _pow2(x: int, lo: int) -> int:
        b = lo
        while b < x:
            b *= 2
        return b

    @classmethod
    def shape_class(cls, d: int, n: int, m: int, family: int = 0) -> str:
        mb = int(round(math.log2(max(m, 1))))
        return f"f{int(family)}_d{cls._pow2(d, 16)}_n{cls._pow2(n, 16)}_m{mb}"

    def _device_key(self) -> str:
        if self._external is not None:
            return "external"
        p = torch.cuda.get_device_properties(torch.cuda.current_device())
        return f"{p.name}/{p.multi_processor_count}sm"

    def choose(self, d: int, n: int, m: int, family: int = 0) -> int:
        key = self.shape_class(d, n, m, family)
        dev = self._device_key()
        with self._lock:
            hit = self.cache.get(dev, {}).get(key)
        if hit is not None:
            return int(hit)
        if self._external is not None:
            times = {c: self._external(c, d, n, m, family) for c in [0] + tile_configs()}
        else:
            times = self._time_all(d, n, m, family)
        best = min(times, key=lambda c: (times[c], c))
        if times[best] > (1.0 - self.margin) * times[0]:
            best = 0
        with self._lock:
            self.cache.setdefault(dev, {})[key] = best
            self._save()
        return best

    def assign(self, problems: Sequence[BatchProblem]) -> None:
        for p in problems:
            if p.tile_config == 0:
                p.tile_config = self.choose(p.d, p.n, p.m, int(p.S.dist.family))

    def tune_batch(self, problems: Sequence[BatchProblem], layout: Layout = Layout.RowMajor,
                   runs: int = 2) -> "BatchedPlan":
        """A plan for this batch: the per-class choices (``assign``) checked against the
        library's own choices on the batch itself.  Both plans run ``runs`` times after one
        warm-up, and the faster is returned (the other is closed).  The problems'
        tile_config fields are left as the returned plan uses them."""
        requested = [p.tile_config for p in problems]
        self.assign(problems)
        tuned_cfg = [p.tile_config for p in problems]
        if all(c == r for c, r in zip(tuned_cfg, requested)):
            return BatchedPlan(problems, layout)

        def timed(plan: "BatchedPlan") -> float:
            plan.execute()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(runs):
                plan.execute()
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1)

        tuned = BatchedPlan(problems, layout)
        t_tuned = timed(tuned)
        for p, r in zip(problems, requested):
            p.tile_config = r
        library = BatchedPlan(problems, layout)
        t_library = timed(library)
        if t_tuned < t_library:
            library.close()
            for p, c in zip(problems, tuned_cfg):
                p.tile_config = c
            return tuned
        tuned.close()
        return library

    def _save(self) -> None:
        try:
            os.makedirs(os.path.dirname(self.cache_path) or ".", exist_ok=True)
            tmp = self.cache_path + ".tmp"
            with open(tmp, "w") as f:
                json.dump(self.cache, f, indent=1, sort_keys=True)
            os.replace(tmp, self.cache_path)
        except OSError:
            pass

    def _time_all(self, d: int, n: int, m: int, family: int) -> Dict[int, float]:
        """Seconds per run of one synthetic batch of the class, for every configuration and
        for the library's choice (0)."""
        from .api import DenseDist, RNGState, ScalarDist
        m = min(m, self.m_cap)
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        # enough problems that every configuration's items fill the device several times over,
        # counting the coarsest (a row block over all columns is one item)
        row_blocks = math.ceil(d / 128)
        count = max(2, min(64, math.ceil(4 * sms / max(row_blocks, 1))))
        g = torch.Generator(device="cuda").manual_seed(0)
        probs = []
        for i in range(count):
            S = DenseSkOp(DenseDist(d, m, ScalarDist(family)), RNGState(i))
            A = torch.randn(m, n, device="cuda", generator=g)
            probs.append(BatchProblem(S, A, torch.empty(d, n, device="cuda"), d, n, m))
        times = {}
        for c in [0] + tile_configs():
            for p in probs:
                p.tile_config = c
            plan = BatchedPlan(probs)
            plan.execute()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(3):
                plan.execute()
            e1.record()
            torch.cuda.synchronize()
            plan.close()
            times[c] = e0.elapsed_time(e1) / 3e3
        return times
