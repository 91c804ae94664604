"""Scalar optical fields: ``ScalarLight``, ``LightSource`` and the RS / CZT
propagators (reference: xlumina/wave_optics.py).

A ``ScalarLight`` holds its field as a complex64 CUDA tensor.  Masks applied
to a light (SLM phase, thin lens) are kept as a pending per-pixel program and
fused into the first pass of the next propagation; reading ``.field``
materialises them with one elementwise kernel.
"""
from __future__ import annotations

import os
import time

import numpy as np
import torch

from . import autograd, engine

_PRINT_TIMES = os.environ.get("XL_PRINT_TIMES", "0") not in ("", "0")


def _report(what, tic):
    if _PRINT_TIMES:
        torch.cuda.synchronize()
        print(f"Time taken to perform one {what} propagation (in seconds): {time.perf_counter() - tic:.4f}")


class _Grid:
    """Grid metadata shared by scalar and vector lights (x, y as float64 host arrays)."""

    def _init_grid(self, x, y, wavelength):
        self.x = engine.as_grid(x)
        self.y = engine.as_grid(y)
        self.wavelength = wavelength
        self.k = 2 * np.pi / wavelength
        self.n = 1
        self._XY = None

    def _meshgrid(self):
        if self._XY is None:
            dev = engine.device()
            xt = torch.tensor(self.x, device=dev)
            yt = torch.tensor(self.y, device=dev)
            self._XY = torch.meshgrid(xt, yt, indexing="xy")
        return self._XY

    @property
    def X(self):
        return self._meshgrid()[0]

    @property
    def Y(self):
        return self._meshgrid()[1]


class ScalarLight(_Grid):
    """Scalar field U(x, y) (wave_optics.py:43-53).  ``field`` is (ny, nx) complex64."""

    def __init__(self, x, y, wavelength):
        self._init_grid(x, y, wavelength)
        self._field = None   # None means zeros of shape (len(x), len(y)), as the reference
        self._ops = []       # pending per-pixel program
        self.info = 'Wave optics light'

    @classmethod
    def _wrap(cls, x, y, wavelength, field, ops=(), info=None):
        obj = ScalarLight.__new__(ScalarLight)
        obj.x, obj.y = x, y
        obj.wavelength = wavelength
        obj.k = 2 * np.pi / wavelength
        obj.n = 1
        obj._XY = None
        obj._field = field
        obj._ops = list(ops)
        obj.info = info or 'Wave optics light'
        return obj

    @property
    def field(self):
        if self._field is None:
            self._field = torch.zeros((len(self.x), len(self.y)), dtype=torch.complex64, device=engine.device())
        if self._ops:
            ny, nx = self._field.shape[-2:]
            self._field = autograd.apply_ops([self._field], self._ops, ny, nx)[0]
            self._ops = []
        return self._field

    @field.setter
    def field(self, value):
        self._field = engine.as_field(value)
        self._ops = []

    def _base(self):
        if self._field is None:
            return self.field
        return self._field

    def _with_op(self, op):
        return ScalarLight._wrap(self.x, self.y, self.wavelength, self._base(), self._ops + [op])

    def draw(self, *args, **kwargs):
        raise NotImplementedError("plotting is not part of xlumina_gb300 (read .field and plot it)")

    # -- masks (wave_optics.py:96-171): plain geometric stops, applied on the device with torch.
    def _apply_mask(self, mask):
        out = ScalarLight(self.x, self.y, self.wavelength)
        out.field = self.field * mask.to(torch.complex64)
        return out

    def apply_circular_mask(self, r):
        rx, ry = r
        return self._apply_mask((self.X ** 2 / rx ** 2 + self.Y ** 2 / ry ** 2) < 1)

    def apply_triangular_mask(self, r, angle, m, height):
        from .toolbox import rotate_mask
        x0, y0 = r
        Xrot, Yrot = rotate_mask(self.X, self.Y, angle, origin=(x0, y0))
        Yl = -m * torch.abs(Xrot - x0) + y0
        return self._apply_mask((Yrot < Yl) & (Yrot > (y0 - height)))

    def apply_rectangular_mask(self, center, width, height, angle):
        from .toolbox import rotate_mask
        angle = angle * (np.pi / 180)
        Xrot, Yrot = rotate_mask(self.X, self.Y, angle, center)
        return self._apply_mask((Xrot < (width / 2)) & (Xrot > (-width / 2)) & (Yrot < (height / 2)) &
                                (Yrot > (-height / 2)))

    def apply_annular_aperture(self, di, do):
        di = di / 2
        do = do / 2
        r2 = self.X ** 2 + self.Y ** 2
        return self._apply_mask(~((r2 / di ** 2) < 1) & ((r2 / do ** 2) < 1))

    # -- propagators
    def RS_propagation(self, z):
        """wave_optics.py:173-196: returns (ScalarLight, quality_factor)."""
        tic = time.perf_counter()
        zv, _ = engine.z_values(z)
        qf = engine.quality_factor(self.x, self.y, self.wavelength, zv)
        base = [self._base()]
        if autograd.needs_grad(base, self._ops, z):
            plan = autograd.RsPlan(self.x, self.y, self.wavelength, z, False, self._ops)
            out = autograd.fused_propagate(plan, base, 1)[0]
        else:
            out = engine.rs_propagate(base, self.x, self.y, self.wavelength, zv, vector=False, pre=self._ops)[0]
        _report("RS", tic)
        return ScalarLight._wrap(self.x, self.y, self.wavelength, out), qf

    def get_RS_minimum_z(self, n=1, quality_factor=1):
        """wave_optics.py:198-231: prints the minimum distance and returns None, as the reference."""
        range_x = self.x[-1] - self.x[0]
        range_y = self.y[-1] - self.y[0]
        dx = range_x / np.size(self.x)
        dy = range_y / np.size(self.y)
        dr_real = np.sqrt(dx ** 2 + dy ** 2)
        rmax = np.sqrt(range_x ** 2 + range_y ** 2)
        factor = (((quality_factor * dr_real + rmax) ** 2 - (self.wavelength / n) ** 2 - rmax ** 2) /
                  (2 * self.wavelength / n)) ** 2 - rmax ** 2
        z_min = np.sqrt(factor) if factor > 0 else 0
        return print("Minimum distance to propagate (in microns):", z_min)

    def CZT(self, z, xout=None, yout=None):
        """wave_optics.py:233-263: chirp-z propagation onto (xout, yout)."""
        tic = time.perf_counter()
        xout = self.x if xout is None else engine.as_grid(xout)
        yout = self.y if yout is None else engine.as_grid(yout)
        base = [self._base()]
        if autograd.needs_grad(base, self._ops):
            plan = autograd.CztPlan(self.x, self.y, self.wavelength, z, xout, yout, "scalar", self._ops)
            out = autograd.fused_propagate(plan, base, 1)[0]
        else:
            out = engine.czt_propagate(base, self.x, self.y, self.wavelength, z, xout, yout,
                                       mode="scalar", pre=self._ops)[0]
        _report("CZT", tic)
        return ScalarLight._wrap(xout, yout, self.wavelength, out)


class LightSource(ScalarLight):
    """Scalar light sources (wave_optics.py:462-542)."""

    def __init__(self, x, y, wavelength):
        super().__init__(x, y, wavelength)
        self.info = 'Wave optics light source'

    def gaussian_beam(self, w0, E0, center=(0, 0), z_w0=(0, 0), alpha=0):
        """wave_optics.py:468-523 (the R_y test of z_w0x at :507 is kept)."""
        self.field = engine.gaussian_field(self.x, self.y, self.wavelength, w0, E0, center, z_w0, alpha)

    def plane_wave(self, A=1, theta=0, phi=0, z0=0):
        """wave_optics.py:525-542."""
        self.field = engine.plane_wave_field(self.x, self.y, self.wavelength, A, theta, phi, z0)


def build_grid(x, y):
    """wave_optics.py:265-279: (nx, ny, dx, dy, Xext, Yext) on the 2N-1 offset grid (host float64)."""
    x = engine.as_grid(x)
    y = engine.as_grid(y)
    Xext, Yext = np.meshgrid(engine.rs_offset_axis(x), engine.rs_offset_axis(y))
    return len(x), len(y), x[1] - x[0], y[1] - y[0], Xext, Yext


def compute_np2(x):
    """wave_optics.py:373-383."""
    return 2 ** (np.ceil(np.log2(x))).astype(int)


def build_CZT_grid(z, wavelength, xin, yin, xout, yout):
    """wave_optics.py:299-331 (host float64)."""
    g = engine.czt_grid(z, wavelength, engine.as_grid(xin), engine.as_grid(yin), engine.as_grid(xout),
                        engine.as_grid(yout))
    Xout, Yout = np.meshgrid(xout, yout)
    return g["nx"], g["ny"], g["dx"], g["dy"], Xout, Yout, g["Dm"], g["fy1"], g["fy2"], g["fx1"], g["fx2"]


# The array-level entry points the reference's classes call inside.
from .functional import transfer_function_RS, RS_propagation_jit, CZT_jit, CZT_for_high_NA_jit, compute_fft, Bluestein_method  # noqa: E402,F401
