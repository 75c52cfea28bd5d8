"""Autotuner of the persistent schedule's launch shape.

The persistent kernel has three shape parameters: the paths of one work item
(`tile_paths`), the CTAs resident per SM (`ctas_per_sm`, which trades occupancy against
registers) and the path units run between lane refills (`refill`).  None of them
changes a price -- every path's payoff is reduced in a fixed order whatever the
schedule -- so they can be tuned freely: `tune` times a set of candidates on the book
itself (device time of the whole pricing call -- plan compilation, path kernel and
reductions -- from CUDA events) and returns the fastest.  Results
are cached per book signature (model, sampling, precision, number of contracts and
the orders of magnitude of samples and grid steps), so an engine tunes once per kind
of book.
"""
import ctypes as C
import json
import math
import os
import statistics
import threading
from dataclasses import dataclass
from typing import Dict, Iterable, Optional, Tuple

from . import abi

TILES = (32, 64, 128, 256)
CTAS_PER_SM = (2, 3, 4)
REFILLS = (4, 8, 16)


@dataclass(frozen=True)
class Shape:
    tile_paths: int
    ctas_per_sm: int
    refill: int


def candidates(coarse: bool = False) -> Iterable[Shape]:
    tiles = (64, 128) if coarse else TILES
    ctas = (2, 4) if coarse else CTAS_PER_SM
    refills = (8, 16) if coarse else REFILLS
    for t in tiles:
        for c in ctas:
            for r in refills:
                yield Shape(t, c, r)


def signature(model_kind: int, packed, settings) -> Tuple:
    """What a good shape depends on: the model, sampling and precision, the number of
    contracts and the orders of magnitude of their samples and grid steps."""
    counts = packed.contracts["path_count"]
    paths = [int(p) if p > 0 else int(settings.path_count) for p in counts]
    steps = [int(s) for s in packed.contracts["step_count"]]
    return (int(model_kind), int(settings.sampling), int(settings.precision), len(paths),
            int(math.log2(max(1, sum(paths)))), int(math.log2(max(1, max(steps)))))


class Cache:
    """Tuned shapes by signature, optionally persisted as JSON."""

    def __init__(self, path: Optional[str] = None):
        self.path = path
        self._lock = threading.Lock()
        self._shapes: Dict[Tuple, Shape] = {}
        if path and os.path.exists(path):
            with open(path) as f:
                for key, value in json.load(f).items():
                    self._shapes[tuple(json.loads(key))] = Shape(**value)

    def get(self, key: Tuple) -> Optional[Shape]:
        with self._lock:
            return self._shapes.get(key)

    def put(self, key: Tuple, shape: Shape) -> None:
        with self._lock:
            self._shapes[key] = shape
            if self.path:
                data = {json.dumps(list(k)): vars(v) for k, v in self._shapes.items()}
                with open(self.path, "w") as f:
                    json.dump(data, f, indent=1)


DEFAULT_CACHE = Cache()


def _time_shape(native, model, book, settings, shape: Shape, repeats: int, n: int) -> float:
    s = abi.Settings.from_buffer_copy(settings)
    s.tile_paths, s.ctas_per_sm, s.refill = shape.tile_paths, shape.ctas_per_sm, shape.refill
    out = (abi.Estimate * n)()
    times = []
    for _ in range(repeats + 1):
        native.check(native.lib.kgpu_price_book(native.handle, C.byref(model), C.byref(book),
                                                C.byref(s), out, None))
        times.append(native.last_kernel_ms)
    return statistics.median(times[1:])


def tune(native, ctx, packed, settings, cache: Cache = DEFAULT_CACHE,
         repeats: int = 5) -> Tuple[Shape, Dict[Shape, float]]:
    """The fastest shape of the persistent schedule for this book (cached by signature),
    with the measured device time of every candidate timed."""
    if settings.schedule != abi.SCHEDULE_PERSISTENT:
        raise ValueError("only the persistent schedule has a launch shape to tune")
    model = ctx.kgpu_model()
    key = signature(model.kind, packed, settings)
    cached = cache.get(key)
    if cached is not None:
        return cached, {}
    book = packed.struct()
    n = len(packed.contracts)
    first = Shape(0, 0, 0)  # the kernel's defaults
    base = _time_shape(native, model, book, settings, first, repeats, n)
    # Long pricings get a coarse grid and single repeats, so tuning stays a few seconds.
    coarse = base > 50.0
    reps = 1 if coarse else repeats
    timings = {first: base}
    for shape in candidates(coarse):
        timings[shape] = _time_shape(native, model, book, settings, shape, reps, n)
    best = min(timings, key=timings.get)
    cache.put(key, best)
    return best, timings


def apply(settings, shape: Shape):
    """A copy of `settings` with the shape applied."""
    s = abi.Settings.from_buffer_copy(settings)
    s.tile_paths, s.ctas_per_sm, s.refill = shape.tile_paths, shape.ctas_per_sm, shape.refill
    return s
