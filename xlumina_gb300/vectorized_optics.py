"""Vectorial optical fields: ``VectorizedLight``, ``PolarizedLightSource`` and
the VRS / VCZT propagators (reference: xlumina/vectorized_optics.py).

Ex, Ey, Ez are complex64 CUDA tensors.  Jones devices applied to a light are
kept as a pending per-pixel program and fused into the first pass of the next
propagation; reading a component materialises them.
"""
from __future__ import annotations

import time

import numpy as np
import torch

from . import autograd, engine
from .wave_optics import _Grid, _report


class VectorizedLight(_Grid):
    """Vector field (Ex, Ey, Ez) (vectorized_optics.py:36-49)."""

    def __init__(self, x=None, y=None, wavelength=None):
        self._init_grid(x, y, wavelength)
        self._E = [None, None, None]   # None means zeros of shape (len(x), len(y))
        self._ops = []
        self.info = 'Vectorized light'

    @classmethod
    def _wrap(cls, x, y, wavelength, comps, ops=(), info=None):
        obj = VectorizedLight.__new__(VectorizedLight)
        obj.x, obj.y = x, y
        obj.wavelength = wavelength
        obj.k = 2 * np.pi / wavelength
        obj.n = 1
        obj._XY = None
        obj._E = list(comps)
        obj._ops = list(ops)
        obj.info = info or 'Vectorized light'
        return obj

    def _zeros(self):
        shape = next((c.shape for c in self._E if c is not None), (len(self.x), len(self.y)))
        return torch.zeros(shape, dtype=torch.complex64, device=engine.device())

    def _base(self, n=3):
        return [c if c is not None else self._zeros() for c in self._E[:n]]

    def _materialize(self):
        if self._ops:
            E = self._base()
            ny, nx = E[0].shape[-2:]
            self._E = autograd.apply_ops(E, self._ops, ny, nx)
            self._ops = []
        for i in range(3):
            if self._E[i] is None:
                self._E[i] = self._zeros()

    def _get(self, i):
        self._materialize()
        return self._E[i]

    def _set(self, i, v):
        if self._ops:
            self._materialize()
        self._E[i] = engine.as_field(v)

    Ex = property(lambda s: s._get(0), lambda s, v: s._set(0, v))
    Ey = property(lambda s: s._get(1), lambda s, v: s._set(1, v))
    Ez = property(lambda s: s._get(2), lambda s, v: s._set(2, v))

    def _with_op(self, op):
        return VectorizedLight._wrap(self.x, self.y, self.wavelength, self._E, self._ops + [op])

    def draw(self, *args, **kwargs):
        raise NotImplementedError("plotting is not part of xlumina_gb300 (read Ex/Ey/Ez and plot them)")

    draw_intensity_profile = draw

    def VRS_propagation(self, z, out=None):
        """vectorized_optics.py:244-284: Ez derived from Ex, Ey; returns (light, quality_factor).

        ``out``: optional (Ex, Ey, Ez) planes to write the result into, CUDA
        tensors or pinned host tensors; a result wanted on the host is then
        stored there by the last pass, with no device-to-host copy (not for a
        propagation that needs gradients)."""
        tic = time.perf_counter()
        zv, _ = engine.z_values(z)
        qf = engine.quality_factor(self.x, self.y, self.wavelength, zv)
        E = self._base(2)
        if autograd.needs_grad(E, self._ops, z):
            if out is not None:
                raise ValueError("out= is for propagations without gradients")
            plan = autograd.RsPlan(self.x, self.y, self.wavelength, z, True, self._ops)
            Ex, Ey, Ez = autograd.fused_propagate(plan, E, 3)
        else:
            Ex, Ey, Ez = engine.rs_propagate(E, self.x, self.y, self.wavelength, zv, vector=True, pre=self._ops,
                                             outs=None if out is None else list(out))
        _report("VRS", tic)
        return VectorizedLight._wrap(self.x, self.y, self.wavelength, [Ex, Ey, Ez]), qf

    def get_VRS_minimum_z(self, n=1, quality_factor=1):
        """vectorized_optics.py:286-319: prints the minimum distance and returns None."""
        range_x = self.x[-1] - self.x[0]
        range_y = self.y[-1] - self.y[0]
        dx = range_x / np.size(self.x)
        dy = range_y / np.size(self.y)
        dr_real = np.sqrt(dx ** 2 + dy ** 2)
        rmax = np.sqrt(range_x ** 2 + range_y ** 2)
        factor = (((quality_factor * dr_real + rmax) ** 2 - (self.wavelength / n) ** 2 - rmax ** 2) /
                  (2 * self.wavelength / n)) ** 2 - rmax ** 2
        z_min = np.sqrt(factor) if factor > 0 else 0
        return print("Minimum distance to propagate (in um):", z_min)

    def VCZT(self, z, xout, yout):
        """vectorized_optics.py:321-361: Ez = (Ex X/r + Ey Y/r) z/r, chirp-z onto (xout, yout)."""
        tic = time.perf_counter()
        xout = self.x if xout is None else engine.as_grid(xout)
        yout = self.y if yout is None else engine.as_grid(yout)
        E = self._base(2)
        if autograd.needs_grad(E, self._ops):
            plan = autograd.CztPlan(self.x, self.y, self.wavelength, z, xout, yout, "vczt", self._ops)
            outs = autograd.fused_propagate(plan, E, 3)
        else:
            outs = engine.czt_propagate(E, self.x, self.y, self.wavelength, z, xout, yout, mode="vczt",
                                        pre=self._ops)
        _report("VCZT", tic)
        return VectorizedLight._wrap(xout, yout, self.wavelength, outs)


class PolarizedLightSource(VectorizedLight):
    """Polarised sources (vectorized_optics.py:396-490)."""

    def __init__(self, x, y, wavelength):
        super().__init__(x, y, wavelength)
        self.info = 'Vectorized light source'

    def gaussian_beam(self, w0, jones_vector, center=(0, 0), z_w0=(0, 0), alpha=0):
        """vectorized_optics.py:402-465: normalised Jones vector times the scalar beam; Ez = 0."""
        jv = np.asarray(jones_vector)
        jv = jv / np.linalg.norm(jv)
        g = engine.gaussian_field(self.x, self.y, self.wavelength, w0, 1.0, center, z_w0, alpha)
        self._ops = []
        self._E = [g * complex(jv[0]), g * complex(jv[1]), self._zeros()]

    def plane_wave(self, jones_vector, theta=0, phi=0, z0=0):
        """vectorized_optics.py:467-490."""
        jv = np.asarray(jones_vector)
        jv = jv / np.linalg.norm(jv)
        pw = engine.plane_wave_field(self.x, self.y, self.wavelength, 1.0, theta, phi, z0)
        self._ops = []
        self._E = [pw * complex(jv[0]), pw * complex(jv[1]), self._zeros()]


# The array-level entry points the reference's classes call inside.
from .functional import VRS_propagation_jit, VCZT_jit, vectorized_CZT_for_high_NA  # noqa: E402,F401
