"""Prebuilt optimisation tables on the propagation path (one fwd+bwd step each).

* ``FourFTable``: SLM1 -> RS(f) -> thin lens(f) -> CZT to an ROI -> SLM2 -> CZT,
  matched to target intensities with the normalised intensity MSE; a batch of
  input masks shares the SLM parameters (the structure of
  experiments/four_f_optical_table.py:36-127, with the table's propagators).
* ``HighNATable``: LCD + sSLM -> VCZT through a high-NA objective lens, with an
  Ez-weighted focal-spot loss (small_area_hybrid, loss_functions.py:24-40);
  one set of sSLM phases per batch entry (the sharp-focus table of
  experiments/hybrid_sharp_optical_table.py).

Both are built only from the public API (``wave_optics``, ``vectorized_optics``,
``optical_elements``), so a step runs the fused kernels forward and the
hand-written adjoints backward.
"""
from __future__ import annotations

import numpy as np
import torch

from . import loss_functions as lf
from .optim import AdamW
from . import optical_elements as oe
from . import toolbox
from .vectorized_optics import VectorizedLight
from .wave_optics import LightSource


class FourFTable:
    """A batch of B 4f tables.  ``independent`` (the default): every table has
    its own seed, hence its own input mask, binary target and pair of SLM
    phase planes (phase1 (B, n, n), phase2 (B, m, m)), so the step optimises B
    independent parameter sets at once.  ``independent=False``: the B input
    masks share one pair of SLM planes, the structure of
    experiments/four_f_optical_table.py:36-127 (a batch of inputs through one
    setup)."""

    def __init__(self, n=1024, roi_n=512, batch=16, wavelength=0.532, half_width=1500.0, f=2.5e5,
                 roi_half_width=1000.0, waist=1200.0, seed=2000, device="cuda", capturable=False,
                 independent=True):
        self.n, self.m, self.B, self.f = n, roi_n, batch, f
        self.independent = independent
        self.x, self.y = toolbox.space(half_width, n)
        self.xo, self.yo = toolbox.space(roi_half_width, roi_n)
        self.wavelength = wavelength
        self.lens_r = (half_width, half_width)
        src = LightSource(self.x, self.y, wavelength)
        src.gaussian_beam(w0=(waist, waist), E0=1)
        if independent:
            seeds = [np.random.default_rng(seed + b) for b in range(batch)]
            masks = np.stack([(r.uniform(0, 1, (n, n)) > 0.5).astype(np.float32) for r in seeds])
            tgt = np.stack([(r.uniform(0, 1, (roi_n, roi_n)) < 0.1).astype(np.float32) for r in seeds])
            p1 = np.stack([r.uniform(-np.pi, np.pi, (n, n)).astype(np.float32) for r in seeds])
            p2 = np.stack([r.uniform(-np.pi, np.pi, (roi_n, roi_n)).astype(np.float32) for r in seeds])
        else:
            rng = np.random.default_rng(seed)
            masks = (rng.uniform(0, 1, (batch, n, n)) > 0.5).astype(np.float32)
            tgt = (rng.uniform(0, 1, (batch, roi_n, roi_n)) < 0.1).astype(np.float32)
            p1 = rng.uniform(-np.pi, np.pi, (n, n)).astype(np.float32)
            p2 = rng.uniform(-np.pi, np.pi, (roi_n, roi_n)).astype(np.float32)
        self.inputs = src.field[None] * torch.as_tensor(masks, device=device)
        tgt /= tgt.sum(axis=(-2, -1), keepdims=True)
        self.target = torch.as_tensor(tgt, device=device)
        self.phase1 = torch.as_tensor(p1, device=device).requires_grad_(True)
        self.phase2 = torch.as_tensor(p2, device=device).requires_grad_(True)
        # capturable: the step count lives on the device, so plans.CapturedStep can record a step
        self.opt = AdamW([self.phase1, self.phase2], lr=0.05, capturable=capturable)

    def entry(self, b):
        """The inputs, target and SLM planes of table b (float64 / complex128
        host arrays), for checking one table against the oracle."""
        def host(t):
            return t.detach().cpu().numpy().astype(np.float64)
        p1 = self.phase1[b] if self.independent else self.phase1
        p2 = self.phase2[b] if self.independent else self.phase2
        return (self.inputs[b].detach().cpu().numpy().astype(np.complex128), host(self.target[b]),
                host(p1), host(p2))

    def intensities(self, inputs=None, tables=None):
        """The output intensities of the tables, each normalised to sum 1
        (B, m, m).  ``tables``: a slice of the batch."""
        I = torch.abs(self.output_field(inputs, tables)) ** 2
        return I / torch.sum(I, dim=(-2, -1), keepdim=True)

    def output_field(self, inputs=None, tables=None):
        """The tables' output fields (B, m, m) (a slice of the batch with ``tables``)."""
        sl = slice(None) if tables is None else tables
        inputs = self.inputs[sl] if inputs is None else inputs
        p1 = self.phase1[sl] if self.independent else self.phase1
        p2 = self.phase2[sl] if self.independent else self.phase2
        light = LightSource(self.x, self.y, self.wavelength)
        light.field = inputs
        l1, _ = oe.SLM(light, p1, self.n)
        l2, _ = l1.RS_propagation(self.f)
        l3, _ = oe.lens(l2, self.lens_r, (self.f, self.f))
        l4 = l3.CZT(self.f, self.xo, self.yo)
        l5, _ = oe.SLM(l4, p2, self.m)
        return l5.CZT(self.f).field

    def loss(self, inputs=None, target=None, tables=None):
        """Mean over the tables of the normalised intensity MSE
        (experiments/four_f_optical_table.py:129-141), fused into two
        reduction passes over the output fields with a hand-written gradient."""
        sl = slice(None) if tables is None else tables
        target = self.target[sl] if target is None else target
        return torch.mean(lf.normalized_intensity_mse(self.output_field(inputs, tables), target))

    def step(self, inputs=None, target=None, tables=None):
        self.opt.zero_grad(set_to_none=True)
        L = self.loss(inputs, target, tables)
        L.backward()
        self.opt.step()
        return L


def small_area_hybrid_batched(I):
    """loss_functions.py:24-40 for each leading-batch entry, then the mean."""
    In = I / (torch.sum(I, dim=(-2, -1), keepdim=True) + 1e-08)
    mx = torch.amax(In, dim=(-2, -1), keepdim=True)
    mask = (In > 0.7 * mx).to(In.dtype)
    return torch.mean(torch.sum(mask, dim=(-2, -1)) / (torch.sum(mask * In, dim=(-2, -1)) + 1e-08))


class HighNATable:
    """B high-NA focusing tables, each with its own parameter set: an LCD
    (eta, theta) and an sSLM (alpha, phi), per-pixel float32 planes drawn
    U[0, 2 pi) (B, n, n each), in front of a VCZT objective lens; the loss is
    the Ez spot-size loss (small_area_hybrid) averaged over the tables.
    ``shared_lcd``: one LCD setting for the whole batch instead (the sharp-
    focus table's structure).  ``checkpoint``: the focal fields are not kept
    for the backward; it recomputes them from the parameters (the
    intermediate fields of a table are then never stored).  ``ez_only``
    (default): the focus computes the Ez component alone, the only one the
    loss reads (VCZT_objective_lens_ez); False runs the full three-component
    focus and takes its Ez."""

    def __init__(self, n=2048, roi_n=1024, batch=32, wavelength=0.650, half_width=2700.0, na=0.9,
                 f=3000.0, roi_half_width=1.0, waist=1500.0, seed=3000, device="cuda", capturable=False,
                 checkpoint=False, shared_lcd=False, ez_only=True):
        self.n, self.m, self.B = n, roi_n, batch
        self.checkpoint = checkpoint
        self.ez_only = ez_only
        self.x, self.y = toolbox.space(half_width, n)
        self.xo, self.yo = toolbox.space(roi_half_width, roi_n)
        self.wavelength, self.f, self.r = wavelength, f, na * f
        rng = np.random.default_rng(seed)
        src = LightSource(self.x, self.y, wavelength)
        src.gaussian_beam(w0=(waist, waist), E0=1)
        self.Ex = src.field
        self.Ey = torch.zeros_like(src.field)

        def planes(lead):
            return torch.as_tensor(rng.uniform(0, 2 * np.pi, lead + (n, n)).astype(np.float32),
                                   device=device).requires_grad_(True)
        lcd_lead = () if shared_lcd else (batch,)
        self.eta, self.theta = planes(lcd_lead), planes(lcd_lead)
        self.alpha, self.phi = planes((batch,)), planes((batch,))
        self.opt = AdamW([self.eta, self.theta, self.alpha, self.phi], lr=0.05, capturable=capturable)

    def entry(self, b):
        """Table b's parameter planes (float64 host arrays), for checking one
        table against the oracle."""
        def host(t):
            return t.detach().cpu().numpy().astype(np.float64)
        e, t = (self.eta, self.theta) if self.eta.dim() == 2 else (self.eta[b], self.theta[b])
        return host(e), host(t), host(self.alpha[b]), host(self.phi[b])

    def _focal_ez(self):
        light = VectorizedLight(self.x, self.y, self.wavelength)
        light.Ex = self.Ex.expand(self.B, self.n, self.n)
        light.Ey = self.Ey.expand(self.B, self.n, self.n)
        masked = oe.sSLM(oe.LCD(light, self.eta, self.theta), self.alpha, self.phi)
        if self.ez_only:
            return oe.VCZT_objective_lens_ez(masked, self.r, self.f, self.xo, self.yo)
        return oe.VCZT_objective_lens(masked, self.r, self.f, self.xo, self.yo).Ez

    def _spot_intensity(self):
        return torch.abs(self._focal_ez()) ** 2

    def _table_losses(self):
        # the area loss of |Ez|^2 in two fused passes, gradient to Ez
        return lf.small_area_hybrid_field(self._focal_ez())

    def loss(self):
        if self.checkpoint and torch.is_grad_enabled():
            # the focal fields are recomputed in the backward instead of kept
            from torch.utils.checkpoint import checkpoint
            losses = checkpoint(self._table_losses, use_reentrant=False)
        else:
            losses = self._table_losses()
        return torch.mean(losses)

    def step(self):
        self.opt.zero_grad(set_to_none=True)
        L = self.loss()
        L.backward()
        self.opt.step()
        return L


class VrsLcdTable:
    """2048^2 VRS optimisation: per-field LCD retarder maps (eta, theta) in
    front of a linear polarizer shape a radially polarised source, which is
    propagated by VRS to z; the loss is the reference's vectorial intensity
    MSE (vMSE_Intensity, loss_functions.py:93-107: Ex, Ey and Ez each against
    a target field), averaged.  One step is a forward through the fused
    kernels, the hand-written adjoints backward (the fused loss gradient
    first), and AdamW.  ``fields`` selects a subset of the batch (the plain
    form: one field per call)."""

    def __init__(self, n=2048, batch=8, wavelength=0.633, half_width=2000.0, waist=1000.0, z=5e4,
                 seed=5000, device="cuda", capturable=False):
        self.n, self.B, self.z, self.wavelength = n, batch, z, wavelength
        self.x, self.y = toolbox.space(half_width, n)
        X, Y = np.meshgrid(self.x, self.y)
        g = np.exp(-(X ** 2 + Y ** 2) / waist ** 2)
        self.Ex = torch.as_tensor(((X / waist) * g).astype(np.complex64), device=device)
        self.Ey = torch.as_tensor(((Y / waist) * g).astype(np.complex64), device=device)
        rng = np.random.default_rng(seed)
        self.eta = torch.as_tensor(rng.uniform(0, 2 * np.pi, (batch, n, n)).astype(np.float32),
                                   device=device).requires_grad_(True)
        self.theta = torch.as_tensor(rng.uniform(0, 2 * np.pi, (batch, n, n)).astype(np.float32),
                                     device=device).requires_grad_(True)
        g = torch.Generator(device=device).manual_seed(seed)
        self.target = [0.01 * torch.randn((batch, n, n), dtype=torch.complex64, device=device, generator=g)
                       for _ in range(3)]
        self.alpha = float(rng.uniform(0, np.pi))
        self.opt = AdamW([self.eta, self.theta], lr=0.05, capturable=capturable)

    def loss(self, fields=None):
        sl = slice(None) if fields is None else fields
        eta, theta = self.eta[sl], self.theta[sl]
        b = eta.shape[0]
        light = VectorizedLight(self.x, self.y, self.wavelength)
        light.Ex = self.Ex.expand(b, self.n, self.n)
        light.Ey = self.Ey.expand(b, self.n, self.n)
        out, _ = oe.linear_polarizer(oe.LCD(light, eta, theta), self.alpha).VRS_propagation(self.z)
        target = VectorizedLight(self.x, self.y, self.wavelength)
        target.Ex, target.Ey, target.Ez = (t[sl] for t in self.target)
        return torch.mean(lf.vMSE_Intensity(out, target))

    def step(self, fields=None):
        self.opt.zero_grad(set_to_none=True)
        L = self.loss(fields)
        L.backward()
        self.opt.step()
        return L


class SharpFocusTable:
    """The hybrid sharp-focus discovery step of
    experiments/hybrid_sharp_optical_table.py and hybrid_optimizer.py:
    hybrid_setup_sharp_focus on a 1024^2 grid (2.5 mm, 635 nm, every source
    the same polarised Gaussian), six objective-lens detectors onto 400^2
    (10 um, NA 0.9), loss softmin(vectorized_loss_hybrid(|Ez|^2)), AdamW over
    all 29 parameters (six phase masks, three LCDs, nine splitter angles,
    eight distances)."""

    def __init__(self, n=1024, roi_n=400, wavelength=0.635, half_width=2500.0, waist=1200.0, seed=2100,
                 device="cuda", capturable=False, checkpoint=False):
        self.checkpoint = checkpoint
        from .vectorized_optics import PolarizedLightSource
        self.x, self.y = toolbox.space(half_width, n)
        self.xo, self.yo = toolbox.space(10.0, roi_n)
        r_lens = 3.6e3 / 2
        self.fixed = [r_lens, r_lens / 0.9, self.xo, self.yo]
        self.src = PolarizedLightSource(self.x, self.y, wavelength)
        self.src.gaussian_beam(w0=(waist, waist), jones_vector=(1, 1))
        rng = np.random.default_rng(seed)
        self.params = []
        for k in range(29):
            # phase masks in float32 (the kernels' precision); the settings in
            # float64, as distances need it
            plane = k < 18 and k % 6 in (0, 1)
            self.params.append(torch.as_tensor(rng.uniform(0, 1, (n, n) if plane else (1,)),
                                               dtype=torch.float32 if plane else torch.float64,
                                               device=device).requires_grad_(True))
        # capturable: the step count lives on the device, so plans.CapturedStep can record a step
        self.opt = AdamW(self.params, lr=0.05, weight_decay=1e-4, capturable=capturable)

    def loss(self):
        s = self.src
        I, _ = oe.hybrid_setup_sharp_focus(s, s, s, s, s, s, self.params, self.fixed, checkpoint=self.checkpoint)
        return toolbox.softmin(lf.vectorized_loss_hybrid(I))

    def step(self):
        self.opt.zero_grad(set_to_none=True)
        L = self.loss()
        L.backward()
        self.opt.step()
        return L
