"""Optical elements (reference: xlumina/optical_elements.py).

Jones devices (SLM, sSLM, LCD, polarizer, thin lens) return a new light that
carries the device as a pending per-pixel op; it is fused into the first pass
of the next propagation, or materialised by one elementwise kernel when a
component is read.  The high-NA objective lens fuses into the chirp-z pass of
``VCZT_objective_lens``.
"""
from __future__ import annotations

import time

import numpy as np
import torch

from . import autograd, cm, engine, um  # noqa: F401  (units re-exported as in the reference)
from .toolbox import build_LCD_cell, rotate_mask  # noqa: F401
from .vectorized_optics import VectorizedLight
from .wave_optics import ScalarLight, _report

_SCALAR = ('Wave optics light', 'Wave optics light source')
_VECTOR = ('Vectorized light', 'Vectorized light source')


def _phase_mask(phase, ny, nx):
    """exp(i phase) materialised on the device (the mask an SLM returns)."""
    ones = torch.ones((ny, nx), dtype=torch.complex64, device=engine.device())
    return engine.apply_ops([ones], [engine.op_phase(phase)], ny, nx)[0]


# ---------------------------------------------------------------- scalar --

def phase_scalar_SLM(phase):
    """optical_elements.py:76-85."""
    if isinstance(phase, torch.Tensor):
        return torch.polar(torch.ones_like(phase, dtype=torch.float32), phase.to(torch.float32))
    return np.exp(1j * np.asarray(phase))


def SLM(input_field, phase_array, shape):
    """optical_elements.py:87-103: returns (light * exp(i phase), exp(i phase))."""
    op = engine.op_phase(phase_array)
    out = input_field._with_op(op)
    p = op.params[0]
    if not isinstance(p, torch.Tensor):
        p = torch.full((shape, shape), p, dtype=torch.float32, device=engine.device())
    return out, _phase_mask(p, *p.shape[-2:])


# ---------------------------------------------------------- Jones matrices --

def _jm(entries):
    return torch.tensor(entries, dtype=torch.complex64)


def jones_LP(alpha):
    """optical_elements.py:109-120."""
    c, s = np.cos(alpha), np.sin(alpha)
    return _jm([[c ** 2, c * s], [c * s, s ** 2]])


def jones_general_retarder(eta, theta, delta):
    """optical_elements.py:122-139."""
    em, ep = np.exp(-0.5j * eta), np.exp(0.5j * eta)
    c, s = np.cos(theta), np.sin(theta)
    return _jm([[em * c ** 2 + ep * s ** 2, (em - ep) * np.exp(-1j * delta) * s * c],
                [(em - ep) * np.exp(1j * delta) * s * c, em * s ** 2 + ep * c ** 2]])


def jones_sSLM(alpha, phi):
    """optical_elements.py:141-152."""
    return _jm([[np.exp(1j * alpha), 0], [0, np.exp(1j * phi)]])


def jones_sSLM_with_amplitude(alpha, phi, a1, a2):
    """optical_elements.py:154-167."""
    return _jm([[a1 * np.exp(1j * alpha), 0], [0, a2 * np.exp(1j * phi)]])


def jones_LCD(eta, theta):
    """optical_elements.py:169-180."""
    return jones_general_retarder(eta, theta, 0.0)


# ---------------------------------------------------- polarization devices --

def sSLM(input_field, alpha_array=None, phi_array=None):
    """optical_elements.py:186-222: diag(e^{i alpha}, e^{i phi}); Ez passes unchanged."""
    return input_field._with_op(engine.op_sslm(alpha_array, phi_array))


def sSLM_with_amplitude(input_field, alpha_array=None, phi_array=None, A1_array=None, A2_array=None):
    """optical_elements.py:224-264."""
    return input_field._with_op(engine.op_sslm_amp(alpha_array, phi_array, A1_array, A2_array))


def LCD(input_field, eta, theta):
    """optical_elements.py:266-305: retarder with scalar or per-pixel (eta, theta); Ez kept."""
    return input_field._with_op(engine.op_lcd(eta, theta))


def linear_polarizer(input_field, alpha):
    """optical_elements.py:307-332: per-pixel polarizer; the output Ez is zero."""
    return input_field._with_op(engine.op_lp(alpha))


def BS_symmetric(a, b, theta):
    """optical_elements.py:334-391: lossy symmetric beam splitter (1% loss of T), on the device."""
    T = abs(np.cos(theta))
    R = abs(np.sin(theta))
    noise = T * 0.01
    T, R = T - noise, R - noise
    c = VectorizedLight(a.x, a.y, a.wavelength)
    d = VectorizedLight(a.x, a.y, a.wavelength)
    c.Ex = R * a.Ex + 1j * T * b.Ex
    c.Ey = R * a.Ey + 1j * T * b.Ey
    d.Ex = 1j * T * a.Ex + R * b.Ex
    d.Ey = 1j * T * a.Ey + R * b.Ey
    return c, d


def high_NA_objective_lens(input_field, radius, f):
    """optical_elements.py:515-553: returns ((3, N, N) field, sin(theta_max))."""
    op, s_max = engine.op_high_na(input_field.x, input_field.y, radius, f)
    E = input_field._base()
    ny, nx = len(input_field.y), len(input_field.x)
    out = autograd.apply_ops(E, input_field._ops + [op], ny, nx)
    return torch.stack(out), s_max


def build_high_NA_VCZT_grid(f, r, wavelength, xin, xout, yout):
    """optical_elements.py:640-672."""
    Dm = f * wavelength * (len(xin) - 1) / (2 * r)
    xout = engine.as_grid(xout)
    yout = engine.as_grid(yout)
    return len(xout), len(yout), Dm, yout[0] + Dm / 2, yout[-1] + Dm / 2, xout[0] + Dm / 2, xout[-1] + Dm / 2


def VCZT_objective_lens(input_field, r, f, xout, yout):
    """optical_elements.py:600-638: high-NA lens fused into the first chirp-z pass."""
    tic = time.perf_counter()
    xout = engine.as_grid(xout)
    yout = engine.as_grid(yout)
    op, s_max = engine.op_high_na(input_field.x, input_field.y, r, f)
    E = input_field._base(2)
    ops = input_field._ops + [op]
    if autograd.needs_grad(E, ops):
        plan = autograd.CztPlan(input_field.x, input_field.y, input_field.wavelength, None, xout, yout,
                                "high_na", ops, lens=(r, f, s_max))
        outs = autograd.fused_propagate(plan, E, 3)
    else:
        outs = engine.czt_propagate(E, input_field.x, input_field.y, input_field.wavelength, None, xout, yout,
                                    mode="high_na", pre=ops, lens=(r, f, s_max))
    _report("VCZT through objective lens", tic)
    return VectorizedLight._wrap(xout, yout, input_field.wavelength, outs)


# ------------------------------------------------------- general elements --

def circular_mask(X, Y, r):
    """optical_elements.py:781-795."""
    rx, ry = r
    return torch.where((X ** 2 / rx ** 2 + Y ** 2 / ry ** 2) < 1, 1, 0)


def lens(input_field, radius, focal):
    """optical_elements.py:678-703: returns (light, lens mask); the vector lens drops Ez."""
    if input_field.info in _SCALAR:
        vector = False
    elif input_field.info in _VECTOR:
        vector = True
    else:
        raise ValueError("Invalid input. Please use ScalarLight or VectorizedLight object.")
    op = engine.op_lens(input_field.x, input_field.y, input_field.wavelength, radius, focal, vector)
    ny, nx = len(input_field.y), len(input_field.x)
    ones = torch.ones((ny, nx), dtype=torch.complex64, device=engine.device())
    mask = engine.apply_ops([ones], [engine.op_lens(input_field.x, input_field.y, input_field.wavelength,
                                                    radius, focal, False)], ny, nx)[0]
    if vector:
        out = input_field._with_op(op)
        out.info = 'Vectorized light'
    else:
        out = input_field._with_op(op)
        out.info = 'Wave optics light'
    return out, mask


# --------------------------------------------------------- prebuilt blocks --

def bb_amplitude_and_phase_mod(input_light, alpha, phi, amp1, amp2, z, eta, theta):
    """optical_elements.py:894-917: sSLM (amplitude+phase) -> VRS(z) -> LCD."""
    l_mod = sSLM_with_amplitude(input_light, alpha, phi, amp1, amp2)
    l_prop, _ = l_mod.VRS_propagation(z)
    return LCD(l_prop, eta, theta)


def building_block(input_light, alpha, phi, z, eta, theta):
    """optical_elements.py:919-939: sSLM -> VRS(z) -> LCD."""
    l_mod = sSLM(input_light, alpha, phi)
    l_prop, _ = l_mod.VRS_propagation(z)
    return LCD(l_prop, eta, theta)
