"""Continuous-batching propagation server on one GPU.

Requests (scalar RS, VRS, CZT, or one fwd+bwd gradient of an SLM phase
through RS) arrive at any time.  A scheduler thread keeps them in a queue,
groups compatible ones (same kind, grid, wavelength and output grid) into one
batched launch (the kernels take a different distance per batch entry), and
admits a batch only while the bytes of all batches in flight stay inside an
HBM budget and a stream slot is free.  Batches run on a small pool of CUDA
streams, so work admitted while others are on the GPU overlaps with them;
finished batches are detected with CUDA events and their requests completed.

Every request's fields and masks stay on the device; results are returned as
device tensors.  Latency (arrival to completion) is recorded per request.
"""
from __future__ import annotations

import collections
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from . import autograd, engine


@dataclass
class Request:
    kind: str                       # "rs" | "vrs" | "czt" | "grad"
    fields: list                    # complex64 device tensors (ny, nx): [U] or [Ex, Ey]
    x: np.ndarray
    y: np.ndarray
    wavelength: float
    z: float
    xout: np.ndarray = None         # czt output grid
    yout: np.ndarray = None
    phase: torch.Tensor = None      # grad: SLM phase (ny, nx) float32
    target: torch.Tensor = None     # grad: target intensity (ny, nx) float32
    t_arrival: float = 0.0
    future: Future = field(default_factory=Future)

    def key(self):
        k = (self.kind, len(self.y), len(self.x), float(self.x[0]), float(self.x[-1]), float(self.y[0]),
             float(self.y[-1]), float(self.wavelength))
        if self.kind == "czt":   # distances differ freely within a batch (per-entry chirps)
            k += (len(self.yout), len(self.xout), float(self.xout[0]), float(self.xout[-1]),
                  float(self.yout[0]), float(self.yout[-1]))
        return k

    def nbytes(self):
        """Device bytes a request holds while in flight (fields, workspace, outputs)."""
        n = len(self.y) * len(self.x)
        q = 2 ** int(np.ceil(np.log2(max(len(self.y), len(self.x), 16))))
        if self.kind == "rs":
            return 8 * n * 2 + 8 * len(self.y) * 2 * q
        if self.kind == "vrs":
            return 8 * n * 5 + 3 * 8 * len(self.y) * 2 * q
        if self.kind == "czt":
            return 8 * n + 8 * len(self.y) * len(self.xout) + 8 * len(self.yout) * len(self.xout)
        return 3 * (8 * n * 2 + 8 * len(self.y) * 2 * q) + 12 * n


def run_batch(reqs):
    """Execute a group of compatible requests as one batched launch; returns per-request results."""
    r0 = reqs[0]
    zs = [r.z for r in reqs]
    if r0.kind == "rs":
        f = torch.stack([r.fields[0] for r in reqs])
        out = engine.rs_propagate([f], r0.x, r0.y, r0.wavelength, zs, vector=False)[0]
        return [out[i] for i in range(len(reqs))]
    if r0.kind == "vrs":
        ex = torch.stack([r.fields[0] for r in reqs])
        ey = torch.stack([r.fields[1] for r in reqs])
        o = engine.rs_propagate([ex, ey], r0.x, r0.y, r0.wavelength, zs, vector=True)
        return [(o[0][i], o[1][i], o[2][i]) for i in range(len(reqs))]
    if r0.kind == "czt":
        f = torch.stack([r.fields[0] for r in reqs])
        zc = zs if len(set(zs)) > 1 else r0.z   # one distance: the cached host chirps
        out = engine.czt_propagate([f], r0.x, r0.y, r0.wavelength, zc, r0.xout, r0.yout, "scalar")[0]
        return [out[i] for i in range(len(reqs))]
    if r0.kind == "grad":
        with torch.enable_grad():
            f = torch.stack([r.fields[0] for r in reqs])
            ph = torch.stack([r.phase for r in reqs]).detach().requires_grad_(True)
            tgt = torch.stack([r.target for r in reqs])
            plan = autograd.RsPlan(r0.x, r0.y, r0.wavelength, zs, False, [engine.op_phase(ph)])
            out = autograd.fused_propagate(plan, [f], 1)[0]
            I = torch.abs(out) ** 2
            loss = torch.sum((I - tgt) ** 2, dim=(-2, -1)) / (I.shape[-1] * I.shape[-2])
            loss.sum().backward()
        return [(loss[i].detach(), ph.grad[i]) for i in range(len(reqs))]
    raise ValueError(f"unknown request kind {r0.kind!r}")


def request_class(r: Request):
    """The batch-packing class of a request: its kind and grid."""
    return (r.kind, len(r.y), len(r.x))


class Server:
    """``tuner`` (an ``autotune.BatchTuner``): the batch size per request class
    comes from it once the class is tuned (``tune``), else ``max_batch``.
    ``max_launch_ms``: the tuner keeps only batch sizes whose launch takes at
    most this long, which bounds the latency that batching adds to a request
    (None: throughput alone)."""

    def __init__(self, hbm_budget_bytes=150e9, max_batch=16, streams=2, device=None, tuner=None,
                 max_launch_ms=None):
        self.budget = float(hbm_budget_bytes)
        self.max_batch = int(max_batch)
        self.tuner = tuner
        self.max_launch_s = None if max_launch_ms is None else float(max_launch_ms) / 1e3
        self._caps = {}
        self.device = device or engine.device()
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(streams)]
        self._q = collections.deque()
        self._cv = threading.Condition()
        self._inflight = []      # (event, reqs, results, bytes, stream index)
        self._bytes = 0.0
        self._stop = False
        self.latencies = []
        self.batches = 0
        self.completed = 0
        self._thread = threading.Thread(target=self._loop, daemon=True)
        self._thread.start()

    def tune(self, examples) -> dict:
        """Measure the batch packing of each example request's class (before
        serving); returns {class: batch size}."""
        if self.tuner is None:
            return {}
        out = {}
        for r in examples:
            cls = request_class(r)

            def measure(b, r=r):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                run_batch([r] * b)
                torch.cuda.synchronize()
                return time.perf_counter() - t0

            out[cls] = self._caps[cls] = self.tuner.best_batch(cls, measure, self.max_batch, self.max_launch_s)
        return out

    def batch_cap(self, r: Request) -> int:
        return self._caps.get(request_class(r), self.max_batch)

    # -- client side
    def submit(self, req: Request) -> Future:
        if req.future.done():
            raise ValueError("this request was served already (its future is done): submit a copy "
                             "(dataclasses.replace(req, future=Future()))")
        if req.nbytes() > self.budget:
            req.future.set_exception(MemoryError("request larger than the HBM budget"))
            return req.future
        req.t_arrival = time.perf_counter()
        with self._cv:
            self._q.append(req)
            self._cv.notify()
        return req.future

    def close(self):
        with self._cv:
            self._stop = True
            self._cv.notify()
        self._thread.join()

    def reset_stats(self):
        """Forget the latencies and counts recorded so far (e.g. after a warm-up)."""
        with self._cv:
            self.latencies = []
            self.batches = 0
            self.completed = 0

    def stats(self):
        lat = np.asarray(self.latencies) * 1e3
        if lat.size == 0:
            return {"completed": 0}
        return {"completed": int(self.completed), "batches": int(self.batches),
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "mean_batch": float(self.completed / max(1, self.batches))}

    # -- scheduler
    def _free_slot(self):
        used = {s for (_, _, _, _, s) in self._inflight}
        for i in range(len(self.streams)):
            if i not in used:
                return i
        return None

    def _reap(self, block=False):
        done = []
        for item in self._inflight:
            ev = item[0]
            if block and item is self._inflight[0]:
                ev.synchronize()
            if ev.query():
                done.append(item)
        for item in done:
            self._inflight.remove(item)
            ev, reqs, results, nb, _ = item
            self._bytes -= nb
            now = time.perf_counter()
            try:   # a kernel wait that ran out: the batch's results are not valid
                _lib.check_device_status()
                err = None
            except _lib.XlError as e:
                err = e
            for r, res in zip(reqs, results):
                self.latencies.append(now - r.t_arrival)
                self.completed += 1
                if err is None:
                    r.future.set_result(res)
                else:
                    r.future.set_exception(err)
        return bool(done)

    def _take_batch(self):
        """First queued request, plus every queued request compatible with it, inside the budget."""
        head = self._q[0]
        key = head.key()
        cap = self.batch_cap(head)
        picked, rest = [], collections.deque()
        nb = 0.0
        while self._q:
            r = self._q.popleft()
            if r.key() == key and len(picked) < cap and self._bytes + nb + r.nbytes() <= self.budget:
                picked.append(r)
                nb += r.nbytes()
            else:
                rest.append(r)
        self._q = rest
        return picked, nb

    def _loop(self):
        torch.cuda.set_device(self.device)
        while True:
            with self._cv:
                while not self._q and not self._inflight and not self._stop:
                    self._cv.wait(timeout=0.05)
                if self._stop and not self._q and not self._inflight:
                    return
                can_admit = bool(self._q) and self._free_slot() is not None and \
                    self._bytes + self._q[0].nbytes() <= self.budget
                if can_admit:
                    reqs, nb = self._take_batch()
                else:
                    reqs = None
            if reqs:
                si = self._free_slot()
                s = self.streams[si]
                s.wait_stream(torch.cuda.default_stream(self.device))   # inputs made by clients
                with torch.cuda.stream(s):
                    try:
                        results = run_batch(reqs)
                    except Exception as e:  # report the failure to every request of the batch
                        for r in reqs:
                            r.future.set_exception(e)
                        continue
                    ev = torch.cuda.Event()
                    ev.record(s)
                self._bytes += nb
                self._inflight.append((ev, reqs, results, nb, si))
                self.batches += 1
            else:
                if not self._reap(block=False):
                    if self._inflight and (self._free_slot() is None or not self._q):
                        self._reap(block=True)
                    else:
                        time.sleep(0.0002)
                continue
            self._reap(block=False)
