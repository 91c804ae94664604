"""Differentiation of the propagation path through hand-written adjoints.

Each propagator call becomes one ``torch.autograd.Function`` that runs the
fused forward kernels (Jones program + propagator), and whose backward runs:

* the adjoint propagator on the output gradients: conjugate transfer spectrum
  for RS / VRS, conjugate-transpose chirp-z for CZT / VCZT / the high-NA
  focus, with the Ez derivation folded back in;
* then ``xl_ops_backward`` for the Jones program, which gives the gradient of
  the input field and of every trainable mask parameter.

This replaces ``jax.grad`` through RS_propagation_jit / CZT_jit and the masks
(e.g. experiments/four_f_optimizer.py:43, experiments/hybrid_optimizer.py:60).
Gradients follow torch's convention for complex tensors.

An RS / VRS distance given as a tensor that requires grad is differentiable
too (jax traces z through RS_propagation_jit, wave_optics.py:281-297):
dL/dz = sum Re(conj(g) dout/dz), with dout/dz one more propagation of the
Jones program's output through the spectrum of dH/dz, plus, for VRS, the
term of the input-plane Ez's own z-dependence (vectorized_optics.py:258-261)
reduced against the adjoint's unfolded Ez gradient.  Wavelengths, chirp-z
distances and lens geometry are not differentiable here.
"""
from __future__ import annotations

import torch

from . import engine


def _trainable(ops):
    """(op index, slot, tensor) for every parameter tensor that requires grad."""
    out = []
    for k, o in enumerate(ops):
        for q, p in enumerate(o.params):
            if isinstance(p, torch.Tensor) and p.requires_grad:
                out.append((k, q, p))
    return out


def needs_grad(base, ops, z=None) -> bool:
    if not torch.is_grad_enabled():
        return False
    if any(isinstance(b, torch.Tensor) and b.requires_grad for b in base):
        return True
    if isinstance(z, torch.Tensor) and z.requires_grad:
        return True
    return bool(_trainable(ops))


class RsPlan:
    """RS (one component) or VRS ((Ex, Ey) -> (Ex, Ey, Ez)) with a fused Jones prologue."""

    def __init__(self, x, y, wavelength, z, vector, ops):
        self.z, self.z_tensor = engine.z_values(z)
        self.x, self.y, self.wavelength, self.vector = x, y, wavelength, vector
        self.ops = list(ops or ())
        self.ny, self.nx = len(y), len(x)

    def forward(self, base):
        call = engine.RsCall(list(base), self.x, self.y, self.wavelength, self.z, self.vector, pre=self.ops)
        self._spectra = call.device_spectra   # a device distance's spectra, reused by the adjoint
        return call.run()

    def adjoint(self, grads, want_ez=False):
        return engine.RsCall(list(grads), self.x, self.y, self.wavelength, self.z, self.vector,
                             adjoint=True, want_ez=want_ez, spectra=getattr(self, "_spectra", None)).run()

    def z_grad(self, base, gouts, gez):
        """dL/dz for output gradients ``gouts``; ``gez``: the adjoint's unfolded
        Ez gradient (VRS).  Shaped like the distance tensor (summed over the
        batch for one distance)."""
        douts = engine.RsCall(list(base), self.x, self.y, self.wavelength, self.z, self.vector, pre=self.ops,
                              dz=True).run()
        if self.vector:
            e = engine.apply_ops(list(base), self.ops, self.ny, self.nx) if self.ops else list(base)
            acc = engine.rs_z_gradient(gouts, douts, self.x, self.y, self.z, e[0], e[1], gez)
        else:
            acc = engine.rs_z_gradient(gouts, douts, self.x, self.y, self.z)
        zt = self.z_tensor
        if zt.numel() == 1:
            return acc.sum().reshape(zt.shape).to(device=zt.device, dtype=zt.dtype)
        if acc.numel() != zt.numel():
            raise ValueError(f"{zt.numel()} distances for a batch of {acc.numel()} fields")
        return acc.reshape(zt.shape).to(device=zt.device, dtype=zt.dtype)


class CztPlan:
    """CZT (one component), VCZT, or the high-NA focus (lens op inside ``ops``).
    ``z`` is one distance or one per batch entry; it is a constant here (the
    distances that the reference's experiments optimise go through RS / VRS
    propagation, which differentiates them)."""

    def __init__(self, x, y, wavelength, z, xout, yout, mode, ops, lens=None):
        if isinstance(z, torch.Tensor) and z.requires_grad:
            raise NotImplementedError("chirp-z propagation does not differentiate the distance; "
                                      "pass z detached, or propagate with RS / VRS to optimise it")
        self.x, self.y, self.wavelength, self.z = x, y, wavelength, z
        self.xout, self.yout, self.mode, self.lens = xout, yout, mode, lens
        self.ops = list(ops or ())
        self.ny, self.nx = len(y), len(x)

    @property
    def vector(self):
        return self.mode != "scalar"

    def forward(self, base):
        return engine.CztCall(list(base), self.x, self.y, self.wavelength, self.z, self.xout, self.yout,
                              self.mode, pre=self.ops, lens=self.lens).run()

    def adjoint(self, grads):
        g = engine.CztCall(list(grads), self.x, self.y, self.wavelength, self.z, self.xout, self.yout,
                           self.mode, lens=self.lens, adjoint=True).run()
        if self.mode == "high_na_ez":   # the program's outputs (e0, e1): e1's gradient is zero
            g = [g[0], None]
        return g


def _z_tensor(plan):
    zt = getattr(plan, "z_tensor", None)
    return zt if (zt is not None and zt.requires_grad) else None


class _Fused(torch.autograd.Function):
    @staticmethod
    def forward(ctx, plan, n_base, n_out, *tensors):
        base = tensors[:n_base]
        ctx.plan = plan
        ctx.n_base = n_base
        ctx.save_for_backward(*base)
        outs = plan.forward(base)
        return tuple(outs[:n_out])

    @staticmethod
    def backward(ctx, *gouts):
        plan = ctx.plan
        base = ctx.saved_tensors
        ref = next((g for g in gouts if g is not None), None)
        gouts = [g if g is not None else torch.zeros_like(ref) for g in gouts]
        gouts = [g.to(torch.complex64).contiguous() for g in gouts]
        want_z = _z_tensor(plan) is not None and ctx.needs_input_grad[-1]
        gez = None
        if want_z and plan.vector:
            gprog = plan.adjoint(gouts, want_ez=True)
            gprog, gez = gprog[:2], gprog[2]
        else:
            gprog = plan.adjoint(gouts)           # gradient of the Jones program's output
        trainable = _trainable(plan.ops)
        if plan.ops:
            nb = len(gprog)
            b = list(base) + [None] * (nb - len(base))
            gin, pgrads = engine.ops_backward(b[:nb], gprog, plan.ops, plan.ny, plan.nx,
                                              want_input=any(t.requires_grad for t in base))
        else:
            gin, pgrads = gprog, {}
        gbase = []
        for i, t in enumerate(base):
            gbase.append(gin[i] if (t.requires_grad and i < len(gin)) else None)
        gparams = [pgrads.get((k, q)) for (k, q, _) in trainable]
        if _z_tensor(plan) is None:
            return (None, None, None, *gbase, *gparams)
        gz = plan.z_grad(base, gouts, gez) if want_z else None
        return (None, None, None, *gbase, *gparams, gz)


def fused_propagate(plan, base, n_out):
    """Run ``plan`` through autograd; ``base`` are the input planes."""
    params = [p for (_, _, p) in _trainable(plan.ops)]
    zt = _z_tensor(plan)
    extra = [zt] if zt is not None else []
    return list(_Fused.apply(plan, len(base), n_out, *base, *params, *extra))


class _Ops(torch.autograd.Function):
    """A Jones program materialised on its own (a light's component is read)."""

    @staticmethod
    def forward(ctx, ops, ny, nx, n_base, *tensors):
        base = tensors[:n_base]
        ctx.ops, ctx.ny, ctx.nx = ops, ny, nx
        ctx.save_for_backward(*base)
        return tuple(engine.apply_ops(list(base), ops, ny, nx))

    @staticmethod
    def backward(ctx, *gouts):
        base = ctx.saved_tensors
        ref = next((g for g in gouts if g is not None), None)
        gouts = [(g if g is not None else torch.zeros_like(ref)).to(torch.complex64).contiguous() for g in gouts]
        want = any(t.requires_grad for t in base)
        gin, pgrads = engine.ops_backward(list(base), gouts, ctx.ops, ctx.ny, ctx.nx, want_input=want)
        trainable = _trainable(ctx.ops)
        gbase = [gin[i] if (base[i].requires_grad and gin[i] is not None) else None for i in range(len(base))]
        return (None, None, None, None, *gbase, *[pgrads.get((k, q)) for (k, q, _) in trainable])


def apply_ops(base, ops, ny, nx):
    if needs_grad(base, ops):
        params = [p for (_, _, p) in _trainable(ops)]
        return list(_Ops.apply(list(ops), ny, nx, len(base), *base, *params))
    return engine.apply_ops(base, ops, ny, nx)


class _MseIntensity(torch.autograd.Function):
    """Intensity (amplitude, phase) MSE per plane with the hand-written gradient of libxlgb."""

    @staticmethod
    def forward(ctx, a, b, kind="intensity"):
        ctx.save_for_backward(a, b)
        ctx.kind = kind
        return engine.mse_intensity(a, b, kind)

    @staticmethod
    def backward(ctx, g):
        a, b = ctx.saved_tensors
        want_a, want_b = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        ga, gb = engine.mse_intensity_grad(a, b, g, want_a, want_b, ctx.kind)
        if gb is not None and tuple(b.shape) != tuple(gb.shape):   # a broadcast target
            gb = gb.reshape((-1,) + tuple(b.shape[-2:])).sum(0).reshape(b.shape)
        return ga, gb, None


def mse_intensity(a, b, kind="intensity"):
    return _MseIntensity.apply(a, b, kind)


class _AreaLoss(torch.autograd.Function):
    """small_area_hybrid per plane (fused passes of libxlgb) with the
    hand-written gradient seeded per plane."""

    @staticmethod
    def forward(ctx, x):
        out, work = engine.area_loss(x)
        ctx.save_for_backward(x, work)
        return out

    @staticmethod
    def backward(ctx, g):
        x, work = ctx.saved_tensors
        return engine.area_loss_grad(x, work, g).reshape(x.shape)


def area_loss(x):
    """Per-plane small_area_hybrid of intensities, or of |x|^2 for a complex field."""
    return _AreaLoss.apply(x)


class _NormIntensityMse(torch.autograd.Function):
    """The 4f normalised intensity MSE per plane with the hand-written gradient."""

    @staticmethod
    def forward(ctx, x, target):
        out, work = engine.norm_intensity_mse(x, target)
        ctx.save_for_backward(x, target, work)
        return out

    @staticmethod
    def backward(ctx, g):
        x, target, work = ctx.saved_tensors
        return engine.norm_intensity_mse_grad(x, target, work, g).reshape(x.shape), None


def norm_intensity_mse(x, target):
    """Per-plane normalised intensity MSE of intensities, or of |x|^2 for a complex field."""
    return _NormIntensityMse.apply(x, target)


def _sum_to(g, shape):
    """Sum a per-batch gradient down to a broadcast input's shape."""
    if g is None or tuple(g.shape) == tuple(shape):
        return g
    return g.reshape((-1,) + tuple(g.shape[-2:])).sum(0).reshape(shape)


class _BeamSplitter(torch.autograd.Function):
    """Two-port mixing c, d = M [a; b] with the hand-written backward of
    libxlgb; ``m`` is the matrix (kind 0) or the splitting angle (the lossy
    kinds, M built inside the kernels)."""

    @staticmethod
    def forward(ctx, kind, m, a_ex, a_ey, b_ex, b_ey):
        b = None if b_ex is None else [b_ex, b_ey]
        ctx.has_b = b is not None
        ctx.kind = kind
        ctx.save_for_backward(m, a_ex, a_ey, b_ex, b_ey)
        return tuple(engine.beam_splitter([a_ex, a_ey], b, m, kind))

    @staticmethod
    def backward(ctx, *gouts):
        m, a_ex, a_ey, b_ex, b_ey = ctx.saved_tensors
        need = ctx.needs_input_grad
        want_m, want_a = need[1], need[2] or need[3]
        want_b = ctx.has_b and (need[4] or need[5])
        b = [b_ex, b_ey] if ctx.has_b else None
        ga, gb, s = engine.beam_splitter_backward([a_ex, a_ey], b, m, list(gouts), want_a, want_b, want_m,
                                                  ctx.kind)
        gm = None
        if want_m:
            gm = torch.conj(s) if ctx.kind == 0 else s
            if gm.numel() != m.numel():     # one matrix / angle for the batch
                gm = gm.sum(0)
            gm = gm.reshape(m.shape).to(device=m.device, dtype=m.dtype)
        out = [None, gm, None, None, None, None]
        if ga is not None:
            out[2], out[3] = _sum_to(ga[0], a_ex.shape), _sum_to(ga[1], a_ey.shape)
        if gb is not None:
            out[4], out[5] = _sum_to(gb[0], b_ex.shape), _sum_to(gb[1], b_ey.shape)
        return tuple(out)


def beam_splitter(a, b, m, kind=0):
    """[c.Ex, c.Ey, d.Ex, d.Ey] = M [a; b]; differentiable in a, b and M (or the angle)."""
    tensors = [m] + list(a) + (list(b) if b is not None else [])
    if torch.is_grad_enabled() and any(isinstance(t, torch.Tensor) and t.requires_grad for t in tensors):
        bx, by = (b[0], b[1]) if b is not None else (None, None)
        return list(_BeamSplitter.apply(kind, m, a[0], a[1], bx, by))
    return engine.beam_splitter(a, b, m, kind)
