"""Activation checkpointing of deep optical tables.

A table's backward needs the fields its forward produced.  A deep table
(optical_elements.py:964-2120 builds grids of splitters with up to ~70
propagations per step) keeps many of them, and a batch of noisy copies
multiplies that.  ``CheckpointPolicy`` decides which wavefronts of a splitter
grid (the splitters with i + j = k and the edges leaving them) keep their
fields and which are recomputed in the backward:

* ``every = K``: the inputs of every K-th wavefront are stored; the K
  wavefronts of a segment run again in the backward from them (peak memory
  ~ stored boundaries + one segment's fields; one extra forward overall);
* ``budget_bytes``: the leading wavefronts keep their fields (no
  recomputation) while their estimated activation bytes stay within the
  budget; only the rest are checkpointed, in segments of K.

``run_grid(..., checkpoint=...)`` takes ``False`` (keep everything),
``True`` (K = 1), an int K, or a policy.
"""
from __future__ import annotations

from dataclasses import dataclass


@dataclass(frozen=True)
class CheckpointPolicy:
    every: int = 1
    budget_bytes: float | None = None
    # activation bytes a wavefront keeps per output light, in units of that
    # light's field bytes (the splitter outputs and the propagators' inputs)
    kept_per_light: float = 3.0

    def __post_init__(self):
        if int(self.every) < 1:
            raise ValueError(f"checkpoint every K wavefronts needs K >= 1, got {self.every}")

    @staticmethod
    def coerce(spec):
        """None for no checkpointing, else a policy."""
        if spec is None or spec is False:
            return None
        if spec is True:
            return CheckpointPolicy(1)
        if isinstance(spec, CheckpointPolicy):
            return spec
        if isinstance(spec, int):
            return CheckpointPolicy(spec)
        raise TypeError(f"checkpoint must be a bool, an int or a CheckpointPolicy, got {type(spec).__name__}")

    def segments(self, wavefront_lights, light_bytes):
        """[(k0, k1, checkpointed)] covering wavefronts 0 .. n-1, for
        ``wavefront_lights[k]`` output lights of ``light_bytes`` each."""
        n = len(wavefront_lights)
        out, k = [], 0
        if self.budget_bytes is not None:
            used = 0.0
            while k < n:
                cost = self.kept_per_light * wavefront_lights[k] * light_bytes
                if used + cost > self.budget_bytes:
                    break
                used += cost
                k += 1
            if k:
                out.append((0, k, False))
        while k < n:
            k1 = min(n, k + int(self.every))
            out.append((k, k1, True))
            k = k1
        return out
