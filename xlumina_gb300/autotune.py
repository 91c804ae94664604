"""Batch packing chosen by measurement.

For a class of requests (kind and grid side), the tuner times batched
launches of 1, 2, 4, ... requests and keeps the smallest batch whose
throughput (requests per second) is within ``tolerance`` of the best one:
packing more requests into one launch past that point adds latency to the
first of them and no throughput.  With a latency bound (seconds per
launch), only batches whose launch fits in it are candidates.  A small field leaves most SMs idle, so its
class packs many requests per launch; a 2048^2 field fills the GPU alone.

Choices are cached on disk as JSON, per GPU model and class, so the
measurement runs once per machine type.  The cache file is
``$XL_AUTOTUNE_CACHE`` if set, else ``~/.cache/xlumina_gb300/autotune.json``.
"""
from __future__ import annotations

import json
import os
import statistics
import threading
import time

DEFAULT_CANDIDATES = (1, 2, 4, 8, 16, 32)


def default_cache_path() -> str:
    p = os.environ.get("XL_AUTOTUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "xlumina_gb300", "autotune.json")


class BatchTuner:
    """``best_batch(cls, measure)``: the batch size for request class ``cls``
    (a tuple of str / int / float), measuring with ``measure(b)`` (seconds for
    one launch of ``b`` requests, device work included) when the class is not
    in the cache yet."""

    def __init__(self, path: str | None = None, device_name: str | None = None, tolerance: float = 0.05,
                 candidates=DEFAULT_CANDIDATES, repeats: int = 3):
        self.path = path or default_cache_path()
        self.device_name = device_name or self._device_name()
        self.tolerance = float(tolerance)
        self.candidates = tuple(sorted(set(int(c) for c in candidates)))
        self.repeats = int(repeats)
        self._lock = threading.Lock()
        self._cache = self._load()

    @staticmethod
    def _device_name() -> str:
        try:
            import torch
            if torch.cuda.is_available():
                return torch.cuda.get_device_name()
        except Exception:   # no torch or no device: a host-only name
            pass
        return "cpu"

    @staticmethod
    def class_key(cls) -> str:
        return "|".join(str(v) for v in cls)

    def _load(self) -> dict:
        try:
            with open(self.path) as f:
                data = json.load(f)
            return data if isinstance(data, dict) else {}
        except (OSError, ValueError):
            return {}

    def save(self) -> None:
        d = os.path.dirname(self.path)
        if d:
            os.makedirs(d, exist_ok=True)
        tmp = f"{self.path}.{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(self._cache, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)

    def cached(self, cls):
        return self._cache.get(self.device_name, {}).get(self.class_key(cls))

    def choose(self, rates: dict, launch_s: dict | None = None, max_launch_s: float | None = None) -> int:
        """Smallest candidate within the tolerance of the best requests/s,
        among those whose launch takes at most ``max_launch_s`` (a request
        waits for its whole batch, so this bounds the latency batching adds);
        the smallest candidate if none is that fast."""
        if max_launch_s is not None and launch_s is not None:
            ok = {b: r for b, r in rates.items() if launch_s[b] <= max_launch_s}
            if not ok:
                return int(min(rates))
            rates = ok
        best = max(rates.values())
        for b in sorted(rates):
            if rates[b] >= (1.0 - self.tolerance) * best:
                return int(b)
        return int(max(rates, key=rates.get))

    def best_batch(self, cls, measure, max_batch: int | None = None, max_launch_s: float | None = None) -> int:
        """``max_launch_s``: a latency bound, seconds per batched launch (None: throughput alone)."""
        key = tuple(cls) + (("launch<=", float(max_launch_s)),) if max_launch_s is not None else tuple(cls)
        with self._lock:
            hit = self.cached(key)
        if hit is not None:
            b = int(hit["batch"])
            return min(b, max_batch) if max_batch else b
        cands = [c for c in self.candidates if not max_batch or c <= max_batch] or [1]
        rates, launch = {}, {}
        for b in cands:
            measure(b)                                     # warm-up (spectra, caches)
            ts = [measure(b) for _ in range(self.repeats)]
            launch[b] = statistics.median(ts)
            rates[b] = b / max(launch[b], 1e-9)
        b = self.choose(rates, launch, max_launch_s)
        with self._lock:
            self._cache.setdefault(self.device_name, {})[self.class_key(key)] = {
                "batch": b, "rates": {str(k): v for k, v in rates.items()},
                "launch_ms": {str(k): 1e3 * v for k, v in launch.items()}, "when": time.time()}
            try:
                self.save()
            except OSError:
                pass   # a read-only cache location still tunes, for this process
        return b


class VariantTuner:
    """Kernel variant of a pass chosen by measurement, per GPU model.

    The library has several kernels for some passes at one transform length
    (the one-line column pass and the packed two-line ones, interleaved in
    the warps or in barrier groups); they agree to float32 rounding and differ
    in speed by GPU and workload shape.  ``best_variant(pass_id, log2_len,
    measure)`` times every variant with ``measure()`` (seconds of one launch,
    device work included) and selects the fastest in the library
    (``xl_set_kernel_variant``); the choice is cached with the batch packings,
    keyed by device model, pass and length, so later processes select it
    without measuring.  ``count`` / ``select`` default to the library's entry
    points and can be replaced (tests without a GPU)."""

    def __init__(self, path: str | None = None, device_name: str | None = None, repeats: int = 5,
                 count=None, select=None):
        self._tuner = BatchTuner(path=path, device_name=device_name)
        self.repeats = int(repeats)
        self._count = count
        self._select = select

    def _lib_count(self, pass_id, log2_len):
        from . import engine
        return int(engine.lib().xl_kernel_variant_count(int(pass_id), int(log2_len)))

    def _lib_select(self, pass_id, log2_len, v):
        from . import _lib, engine
        _lib.check(engine.lib().xl_set_kernel_variant(int(pass_id), int(log2_len), int(v)), "xl_set_kernel_variant")

    def count(self, pass_id, log2_len) -> int:
        return (self._count or self._lib_count)(pass_id, log2_len)

    def select(self, pass_id, log2_len, v) -> None:
        (self._select or self._lib_select)(pass_id, log2_len, v)

    def best_variant(self, pass_id: int, log2_len: int, measure, force: bool = False) -> dict:
        """{"variant": v, "ms": {v: median ms}} (``ms`` empty on a cache hit);
        ``force`` measures even when the choice is cached."""
        cls = ("variant", int(pass_id), int(log2_len))
        n = self.count(pass_id, log2_len)
        with self._tuner._lock:
            hit = self._tuner.cached(cls)
        if hit is not None and not force and int(hit["variant"]) < n:
            self.select(pass_id, log2_len, int(hit["variant"]))
            return {"variant": int(hit["variant"]), "ms": {}, "cached": True}
        ms = {}
        for v in range(n):
            self.select(pass_id, log2_len, v)
            measure()                                   # warm-up (smem carve-out, caches)
            ms[v] = 1e3 * statistics.median(measure() for _ in range(self.repeats))
        best = min(ms, key=ms.get)
        self.select(pass_id, log2_len, best)
        with self._tuner._lock:
            self._tuner._cache.setdefault(self._tuner.device_name, {})[self._tuner.class_key(cls)] = {
                "variant": best, "ms": {str(k): v for k, v in ms.items()}, "when": time.time()}
            try:
                self._tuner.save()
            except OSError:
                pass
        return {"variant": best, "ms": ms, "cached": False}


def cuda_event_timer(fn):
    """measure() for VariantTuner: seconds of one call of ``fn`` on the
    current stream, from CUDA events around it."""
    import torch

    def measure():
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        fn()
        e.record()
        e.synchronize()
        return s.elapsed_time(e) / 1e3
    return measure
