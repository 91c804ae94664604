"""Captured plans: a fixed-shape propagation, or one optimisation step of a
table, recorded once into a CUDA graph and replayed.

Replaying a graph costs one launch from the host, whatever the number of
kernels, torch operations and ctypes calls the eager call makes; small
fields and deep tables, whose eager cost is mostly host work, run several
times faster.  The recipe is torch's: warm-up runs on a side stream (they
build the transfer spectra, chirps and lens coefficients the call needs and
fill the host caches), then one capture.  Every device buffer the captured
kernels read is either a static input, allocated in the graph's own memory
pool during capture, or a host-cache buffer that the plan keeps alive.

Inputs are copied into the plan's static tensors before each replay; the
returned outputs are the plan's static tensors, overwritten by the next
replay (clone them to keep a result).
"""
from __future__ import annotations

import torch

from . import engine


class CapturedPlan:
    """``fn(*static_inputs)`` (device tensors in, a tensor or a sequence of
    tensors out) recorded into a CUDA graph."""

    def __init__(self, fn, *static_inputs, warmup: int = 2):
        if not torch.cuda.is_available():
            raise RuntimeError("captured plans need a CUDA device")
        engine.lib().xl_init()
        self.fn = fn
        self.static_inputs = tuple(static_inputs)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(max(1, warmup)):
                fn(*self.static_inputs)
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        self._keep = []
        engine._capture_keep.items = self._keep
        try:
            with torch.cuda.graph(self.graph):
                self.static_outputs = fn(*self.static_inputs)
        finally:
            engine._capture_keep.items = None

    def replay(self):
        self.graph.replay()
        return self.static_outputs

    def __call__(self, *inputs):
        """Copy ``inputs`` (None: keep the static value) into the static inputs and replay."""
        if len(inputs) > len(self.static_inputs):
            raise ValueError(f"the plan takes {len(self.static_inputs)} inputs, got {len(inputs)}")
        for dst, src in zip(self.static_inputs, inputs):
            if src is not None and src is not dst:
                dst.copy_(src, non_blocking=True)
        return self.replay()


class CapturedStep:
    """One optimisation step of a table (forward, hand-written adjoints
    backward, optimiser update) recorded into a CUDA graph.

    ``table`` is a ``tables.FourFTable`` or ``tables.HighNATable`` (anything
    with ``loss()``, ``opt`` and ``params()``); its optimiser must have been
    made with ``capturable=True`` so the step count lives on the device.
    """

    def __init__(self, table, warmup: int = 3):
        if not torch.cuda.is_available():
            raise RuntimeError("captured plans need a CUDA device")
        engine.lib().xl_init()
        self.table = table
        opt = table.opt
        for g in opt.param_groups:
            if not g.get("capturable", False):
                raise ValueError("build the table's optimiser with capturable=True to capture its step")
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(max(1, warmup)):
                opt.zero_grad(set_to_none=True)
                table.loss().backward()
                opt.step()
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        self._keep = []
        opt.zero_grad(set_to_none=True)
        engine._capture_keep.items = self._keep
        try:
            with torch.cuda.graph(self.graph):
                self.loss = table.loss()
                self.loss.backward()
                opt.step()
        finally:
            engine._capture_keep.items = None

    def __call__(self):
        """Run one step; returns the device tensor holding this step's loss."""
        self.graph.replay()
        return self.loss
