"""Helpers of the propagation path (reference: xlumina/toolbox.py)."""
from __future__ import annotations

import numpy as np
import torch


def space(x_total, num_pix):
    """toolbox.py:49-61: ``linspace(-x_total, x_total, num_pix)`` (half-width argument), float64."""
    x = np.linspace(-x_total, x_total, num_pix, dtype=np.float64)
    y = np.linspace(-x_total, x_total, num_pix, dtype=np.float64)
    return x, y


def wrap_phase(phase):
    """toolbox.py:63-72."""
    if isinstance(phase, torch.Tensor):
        return torch.atan2(torch.sin(phase), torch.cos(phase))
    return np.arctan2(np.sin(phase), np.cos(phase))


def is_conserving_energy(light_source, propagated_light):
    """toolbox.py:74-96: total propagated intensity over source intensity."""
    def tot(light):
        if light.info in ('Wave optics light', 'Wave optics light source'):
            return torch.sum(torch.abs(light.field) ** 2, dtype=torch.float64)
        return sum(torch.sum(torch.abs(c) ** 2, dtype=torch.float64) for c in (light.Ex, light.Ey, light.Ez))
    return tot(propagated_light) / tot(light_source)


def softmin(args, beta=90):
    """toolbox.py:98-103."""
    args = torch.as_tensor(args)
    return -torch.logsumexp(-beta * args, dim=-1) / beta


def delta_kronecker(a, b):
    """toolbox.py:106-118."""
    return 1 if a == b else 0


def build_LCD_cell(eta, theta, shape):
    """toolbox.py:121-135: constant (eta, theta) cell.  The propagation path keeps
    scalars unexpanded; this returns the explicit arrays for callers that want them."""
    return eta * np.ones((shape, shape)), theta * np.ones((shape, shape))


def rotate_mask(X, Y, angle, origin=None):
    """toolbox.py:269-289."""
    if origin is None:
        x0 = (X[-1] + X[0]) / 2
        y0 = (Y[-1] + Y[0]) / 2
    else:
        x0, y0 = origin
    lib = torch if isinstance(X, torch.Tensor) else np
    Xrot = (X - x0) * lib.cos(torch.as_tensor(angle) if lib is torch else angle) + \
        (Y - y0) * lib.sin(torch.as_tensor(angle) if lib is torch else angle)
    Yrot = -(X - x0) * lib.sin(torch.as_tensor(angle) if lib is torch else angle) + \
        (Y - y0) * lib.cos(torch.as_tensor(angle) if lib is torch else angle)
    return Xrot, Yrot


# toolbox.py:698-739: the 4f training-data loader (device batches, prefetched).
from .datasets import MultiHDF5DataLoader  # noqa: E402,F401
