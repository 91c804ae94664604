"""Loss functions of the optimisation tables (reference: xlumina/loss_functions.py)."""
from __future__ import annotations

import torch

from . import autograd


def _t(a):
    return a if isinstance(a, torch.Tensor) else torch.as_tensor(a)


def small_area_hybrid(detected_intensity):
    """loss_functions.py:24-40: area above 0.7*max over the enclosed normalised
    intensity, in two fused libxlgb passes with a hand-written gradient (a
    CUDA tensor; other inputs go through torch)."""
    I = _t(detected_intensity)
    if I.is_cuda:
        return autograd.area_loss(I)
    In = I / (torch.sum(I) + 1e-08)
    mask = (In > 0.7 * torch.max(In)).to(In.dtype)
    return torch.sum(mask) / (torch.sum(mask * In) + 1e-08)


def vectorized_loss_hybrid(detected_intensities):
    """loss_functions.py:42-50: small_area_hybrid of every plane (one fused launch on the GPU)."""
    I = _t(detected_intensities)
    if I.is_cuda:
        return autograd.area_loss(I)
    return torch.stack([small_area_hybrid(i) for i in I])


def small_area_hybrid_field(field):
    """small_area_hybrid of |field|^2 per plane, the intensity formed inside
    the fused kernels (no intensity tensor; the gradient goes to the field)."""
    return autograd.area_loss(field)


def normalized_intensity_mse(field, target):
    """The 4f tables' loss per plane (experiments/four_f_optical_table.py:129-141):
    In = |field|^2 / sum |field|^2, sum((In - target)^2) / npix, fused, with
    the gradient to the field."""
    return autograd.norm_intensity_mse(field, target)


def MSE_Intensity(input_light, target_light):
    """loss_functions.py:137-149: sum((|a|^2 - |b|^2)^2) / num_pix over the last
    two dims, one fused libxlgb reduction (and a fused gradient kernel)."""
    return autograd.mse_intensity(input_light, target_light)


def _on_device(a, b):
    return (isinstance(a, torch.Tensor) and a.is_cuda) or (isinstance(b, torch.Tensor) and b.is_cuda)


def MSE_Amplitude(input_light, target_light):
    """loss_functions.py:109-121, per plane; one fused libxlgb reduction with a
    hand-written gradient for device fields (host arrays go through torch)."""
    if _on_device(input_light, target_light):
        return autograd.mse_intensity(input_light, target_light, "amplitude")
    a, b = _t(input_light), _t(target_light)
    n = a.shape[-1] * a.shape[-2]
    return torch.sum((torch.abs(a) - torch.abs(b)) ** 2, dim=(-2, -1)) / n


def MSE_Phase(input_light, target_light):
    """loss_functions.py:123-135, per plane; fused like MSE_Amplitude."""
    if _on_device(input_light, target_light):
        return autograd.mse_intensity(input_light, target_light, "phase")
    a, b = _t(input_light), _t(target_light)
    n = a.shape[-1] * a.shape[-2]
    return torch.sum((torch.angle(a) - torch.angle(b)) ** 2, dim=(-2, -1)) / n


def mean_batch_MSE_Intensity(optimized, target):
    """loss_functions.py:52-59."""
    mse = MSE_Intensity(optimized, target)
    return torch.mean(mse), mse


def _stack(light):
    return torch.stack([light.Ex, light.Ey, light.Ez])


def vMSE_Amplitude(input_light, target_light):
    """loss_functions.py:61-75."""
    return MSE_Amplitude(_stack(input_light), _stack(target_light))


def vMSE_Phase(input_light, target_light):
    """loss_functions.py:77-91."""
    return MSE_Phase(_stack(input_light), _stack(target_light))


def vMSE_Intensity(input_light, target_light):
    """loss_functions.py:93-107: MSE_Intensity of each of Ex, Ey, Ez (stacked
    results, leading dimension 3), without stacking the fields themselves."""
    return torch.stack([MSE_Intensity(getattr(input_light, c), getattr(target_light, c))
                        for c in ("Ex", "Ey", "Ez")])
