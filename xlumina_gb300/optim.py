"""AdamW for the optimisation tables.

The float32 CUDA parameters of a step are updated by one libxlgb launch
(``xl_adamw_step``: one pass over p, g, m, v), with the step count on the
device, so the update can be recorded in a CUDA graph; other parameters
(e.g. float64 distances and angles, a handful of values) go through torch's
AdamW.  The update is torch.optim.AdamW's (decoupled weight decay), which is
what optax.adamw computes in the reference's experiments
(experiments/hybrid_optimizer.py:33, four_f_optimizer.py).
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib, engine


class AdamW(torch.optim.Optimizer):
    def __init__(self, params, lr=1e-3, betas=(0.9, 0.999), eps=1e-8, weight_decay=1e-2, capturable=True):
        defaults = dict(lr=lr, betas=betas, eps=eps, weight_decay=weight_decay, capturable=True)
        super().__init__(params, defaults)
        self._fallback = {}
        self._steps = {}

    def _split(self, group):
        fast = [p for p in group["params"] if p.is_cuda and p.dtype == torch.float32 and p.is_contiguous()]
        rest = [p for p in group["params"] if not (p.is_cuda and p.dtype == torch.float32 and p.is_contiguous())]
        return fast, rest

    @torch.no_grad()
    def step(self, closure=None):
        loss = None
        if closure is not None:
            with torch.enable_grad():
                loss = closure()
        L = engine.lib()
        for group in self.param_groups:
            fast, rest = self._split(group)
            fast = [p for p in fast if p.grad is not None]
            if fast:
                dev = fast[0].device
                key = (id(group), dev)
                step = self._steps.get(key)
                if step is None:
                    step = self._steps[key] = torch.zeros((), dtype=torch.float32, device=dev)
                step.add_(1.0)
                for chunk in range(0, len(fast), _lib.XL_ADAMW_MAX_TENSORS):
                    a = _lib.XlAdamWArgs()
                    ps = fast[chunk:chunk + _lib.XL_ADAMW_MAX_TENSORS]
                    a.count = len(ps)
                    keep = []
                    for i, p in enumerate(ps):
                        st = self.state[p]
                        if "exp_avg" not in st:
                            st["exp_avg"] = torch.zeros_like(p)
                            st["exp_avg_sq"] = torch.zeros_like(p)
                        g = p.grad if p.grad.is_contiguous() else p.grad.contiguous()
                        keep.append(g)
                        a.t[i].p, a.t[i].g = p.data_ptr(), g.data_ptr()
                        a.t[i].m, a.t[i].v = st["exp_avg"].data_ptr(), st["exp_avg_sq"].data_ptr()
                        a.t[i].n = p.numel()
                    b1, b2 = group["betas"]
                    a.lr, a.beta1, a.beta2 = float(group["lr"]), float(b1), float(b2)
                    a.eps, a.weight_decay = float(group["eps"]), float(group["weight_decay"])
                    a.step = step.data_ptr()
                    _lib.check(L.xl_adamw_step(engine.stream_handle(), ctypes.byref(a)), "xl_adamw_step")
            rest = [p for p in rest if p.grad is not None]
            if rest:
                self._torch_step(group, rest)
        return loss

    def _torch_step(self, group, params):
        """Parameters the kernel does not take, through torch's AdamW (kept per group)."""
        key = (id(group), tuple(id(p) for p in params))
        opt = self._fallback.get(key)
        if opt is None:
            opt = torch.optim.AdamW(params, lr=group["lr"], betas=group["betas"], eps=group["eps"],
                                    weight_decay=group["weight_decay"],
                                    capturable=all(p.is_cuda for p in params))
            self._fallback[key] = opt
        opt.param_groups[0]["lr"] = group["lr"]
        opt.step()
