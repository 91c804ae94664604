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

from . import _lib, autograd, cm, engine, um  # noqa: F401  (units re-exported as in the reference)
from .toolbox import build_LCD_cell, rotate_mask  # noqa: F401
from .vectorized_optics import VectorizedLight
from .wave_optics import ScalarLight, _report

_SCALAR = ('Wave optics light', 'Wave optics light source')
_VECTOR = ('Vectorized light', 'Vectorized light source')


def _phase_mask(phase, ny, nx):
    """exp(i phase) materialised on the device (the mask an SLM returns), one
    elementwise kernel."""
    p = phase.detach() if isinstance(phase, torch.Tensor) else torch.as_tensor(phase, device=engine.device())
    p = p.to(torch.float32)
    return torch.polar(torch.ones((), dtype=torch.float32, device=p.device).expand_as(p), p)


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


def _is_t(v):
    return isinstance(v, torch.Tensor)


def _bs_matrix(entries, like):
    """Complex 2x2 splitter matrix (row-major entries), on the device: a
    differentiable torch tensor when any entry is one, else a cached copy."""
    if any(_is_t(e) for e in entries):
        dev = engine.device()
        shape = torch.broadcast_shapes(*[e.shape for e in entries if _is_t(e)])
        ents = [e.to(device=dev, dtype=torch.complex128) if _is_t(e) else
                torch.full(shape, complex(e), dtype=torch.complex128, device=dev) for e in entries]
        m = torch.stack([e.expand(shape) for e in ents], -1).reshape(tuple(shape) + (2, 2))
        return m.to(torch.complex64)
    m = np.stack([np.broadcast_to(np.asarray(e, dtype=np.complex128), np.shape(like)) for e in entries], -1)
    return engine.device_array(m.reshape(np.shape(like) + (2, 2)), torch.complex64)


def _bs_apply(a, b, m, kind=0):
    """Mix the (Ex, Ey) of lights a, b (b may be None); outputs (c, d) with Ez zero."""
    pa = [a.Ex, a.Ey]
    pb = [b.Ex, b.Ey] if b is not None else None
    cx, cy, dx, dy = autograd.beam_splitter(pa, pb, m, kind)
    c = VectorizedLight._wrap(a.x, a.y, a.wavelength, [cx, cy, None])
    d = VectorizedLight._wrap(a.x, a.y, a.wavelength, [dx, dy, None])
    return c, d


def _bs_angle(theta):
    """The splitting angle on the device (float64): a tensor as it is (its
    gradient flows), a number from the constant cache."""
    if _is_t(theta):
        return theta
    return engine.device_array(np.asarray(theta, dtype=np.float64).reshape(-1), torch.float64)


def BS_symmetric(a, b, theta):
    """optical_elements.py:334-391: lossy symmetric beam splitter, c = R a + iT b,
    d = iT a + R b (R = |sin theta|, T = |cos theta|, both less 1% of T), as one
    kernel that builds the matrix from the angle; differentiable in the fields
    and in a tensor theta."""
    return _bs_apply(a, b, _bs_angle(theta), _lib.XL_BS_SYMMETRIC)


def bs_port0(a_Ex, a_Ey, c_Ex, c_Ey, d_Ex, d_Ey, T, R):
    """optical_elements.py:393-400: single input at port 0."""
    return R * a_Ex, R * a_Ey, 1j * T * a_Ex, 1j * T * a_Ey


def bs_port1(a_Ex, a_Ey, c_Ex, c_Ey, d_Ex, d_Ey, T, R):
    """optical_elements.py:402-409: single input at port 1."""
    return 1j * T * a_Ex, 1j * T * a_Ey, R * a_Ex, R * a_Ey


def BS_symmetric_SI(a, theta, port=0):
    """optical_elements.py:411-460: single-input lossy splitter; port 0 gives
    c = R a, d = iT a, port 1 gives c = iT a, d = R a."""
    kind = _lib.XL_BS_SINGLE_PORT0 if int(port) == 0 else _lib.XL_BS_SINGLE_PORT1
    return _bs_apply(a, None, _bs_angle(theta), kind)


def BS(a1, a2, R, T, phase):
    """optical_elements.py:462-512: lossless splitter, b1 = sqrt(T) a1 + sqrt(R)
    e^{i phase} a2, b2 = -sqrt(R) e^{-i phase} a1 + sqrt(T) a2."""
    if any(_is_t(v) for v in (R, T, phase)):
        dev = engine.device()
        R, T, phase = (v.to(device=dev, dtype=torch.float64) if _is_t(v) else
                       torch.tensor(float(v), dtype=torch.float64, device=dev) for v in (R, T, phase))
        sT, sR = torch.sqrt(T).to(torch.complex128), torch.sqrt(R)
        m = _bs_matrix([sT, torch.polar(sR, phase), -torch.polar(sR, -phase), sT], None)
    else:
        sT, sR = np.sqrt(T), np.sqrt(R)
        m = _bs_matrix([sT, sR * np.exp(1j * phase), -sR * np.exp(-1j * phase), sT], np.asarray(0.0))
    return _bs_apply(a1, a2, m)


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


def VCZT_objective_lens_ez(input_field, r, f, xout, yout):
    """The Ez component of VCZT_objective_lens (optical_elements.py:600-638)
    alone, as a tensor: the lens's Ez row fused into the first chirp-z pass
    and one transformed component instead of three.  A loss that reads only
    the focal Ez (the Ez spot size of hybrid_sharp_optical_table.py) needs no
    more; jax's jit drops the unread Ex and Ey of the reference's focus the
    same way."""
    xout = engine.as_grid(xout)
    yout = engine.as_grid(yout)
    op, s_max = engine.op_high_na(input_field.x, input_field.y, r, f, ez_only=True)
    E = input_field._base(2)
    ops = input_field._ops + [op]
    if autograd.needs_grad(E, ops):
        plan = autograd.CztPlan(input_field.x, input_field.y, input_field.wavelength, None, xout, yout,
                                "high_na_ez", ops, lens=(r, f, s_max))
        return autograd.fused_propagate(plan, E, 1)[0]
    return engine.czt_propagate(E, input_field.x, input_field.y, input_field.wavelength, None, xout, yout,
                                mode="high_na_ez", pre=ops, lens=(r, f, s_max))[0]


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


def _apply_phase_mask(input_field, mask):
    """Multiply a light by a complex mask as a pending op; a vector light's Ez
    becomes zero (the reference builds a new light from Ex, Ey only)."""
    op = engine.op_cmul(mask)
    if input_field.info in _SCALAR:
        return input_field._with_op(op)
    if input_field.info in _VECTOR:
        E = input_field._E
        return VectorizedLight._wrap(input_field.x, input_field.y, input_field.wavelength, [E[0], E[1], None],
                                     input_field._ops + [op])
    raise ValueError("Invalid input. Please use ScalarLight or VectorizedLight object.")


def cylindrical_lens(input_field, focal_length, refractive_index=1.5, angle=0):
    """optical_elements.py:705-744: plano-convex cylindrical lens (phase along
    the rotated x axis); returns (light, lens mask)."""
    X, Y = input_field.X, input_field.Y
    c, s = np.cos(angle), np.sin(angle)
    Xrot = X * c + Y * s
    R = focal_length * (refractive_index - 1)
    thickness = R - torch.sqrt(R ** 2 - Xrot ** 2)
    phase = input_field.k * (refractive_index - 1) * (Xrot ** 2 / (2 * focal_length) + thickness)
    mask = torch.polar(torch.ones_like(phase), -phase).to(torch.complex64)
    return _apply_phase_mask(input_field, mask), mask


def axicon_lens(input_field, alpha, n=1.5):
    """optical_elements.py:746-779: axicon phase k r (n-1) sin(alpha) tan(alpha);
    returns (light, axicon mask)."""
    r = torch.sqrt(input_field.X ** 2 + input_field.Y ** 2)
    phase = input_field.k * r * (n - 1) * np.sin(alpha) * np.tan(alpha)
    mask = torch.polar(torch.ones_like(phase), -phase).to(torch.complex64)
    return _apply_phase_mask(input_field, mask), mask


def triangular_mask(X, Y, r, angle, m, height):
    """optical_elements.py:797-817 (angle in degrees)."""
    x0, y0 = r
    Xrot, Yrot = rotate_mask(X, Y, angle * (np.pi / 180), r)
    Yl = -m * torch.abs(Xrot - x0) + y0
    return torch.where((Yrot < Yl) & (Yrot > y0 - height), 1, 0)


def rectangular_mask(X, Y, center, width, height, angle):
    """optical_elements.py:819-836 (angle in degrees)."""
    Xrot, Yrot = rotate_mask(X, Y, angle * (np.pi / 180), center)
    return torch.where((Xrot < width / 2) & (Xrot > -width / 2) & (Yrot < height / 2) & (Yrot > -height / 2), 1, 0)


def annular_aperture(di, do, X, Y):
    """optical_elements.py:838-854: ring between diameters di and do."""
    di, do = di / 2, do / 2
    r2 = X ** 2 + Y ** 2
    stop = torch.where(r2 / di ** 2 < 1, 0, 1)
    ring = torch.where(r2 / do ** 2 < 1, 1, 0)
    return stop * ring


def forked_grating(X, Y, center, angle, period, l, kind=''):
    """optical_elements.py:856-889: 'Amplitude' gives the binary mask, 'Phase'
    exp(i pi mask); any other kind returns None, as the reference."""
    Xrot, Yrot = rotate_mask(X, Y, angle * (np.pi / 180), center)
    theta = torch.atan2(Xrot, Yrot)
    g = torch.angle(torch.exp(1j * torch.cos(l * theta - 2 * np.pi / period * Xrot)))
    amp = torch.where(g < 0, 0, 1)
    if kind == 'Amplitude':
        return amp
    if kind == 'Phase':
        return torch.exp(1j * np.pi * amp.to(torch.float64))
    return None


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


def fluorescence(i_ex, i_dep, beta=1):
    """optical_elements.py:941-954: STED effective intensity
    i_ex (1 - beta (1 - exp(-i_dep / (i_ex + 1e-8)))), elementwise on the device."""
    i_ex = engine.as_real_param(i_ex) if not _is_t(i_ex) else i_ex
    i_dep = engine.as_real_param(i_dep) if not _is_t(i_dep) else i_dep
    return i_ex * (1 - beta * (1 - torch.exp(-(i_dep / (i_ex + 1e-8)))))


def vectorized_fluorophores(i_ex, i_dep):
    """optical_elements.py:956-962: fluorescence over a stack of detectors
    (the vmap over the leading axis is the elementwise expression itself)."""
    return fluorescence(i_ex, i_dep)


# The prebuilt large-scale tables (optical_elements.py:964-2120) live in
# hybrid_setups.py; exported here under the reference's names.
from .hybrid_setups import (batch_robust_discovery, hybrid_setup_fixed_slms,  # noqa: E402,F401
                            hybrid_setup_fixed_slms_fluorophores, hybrid_setup_fluorophores,
                            hybrid_setup_sharp_focus, robust_discovery, six_times_six_ansatz)
# Table noise (optical_elements.py:2127-2301; shake_setup_jit reads noise.NS).
from .noise import batch_shake_setup, keychain_optical_tables, shake_setup, shake_setup_jit  # noqa: E402,F401


# The array-level entry points the reference's classes call inside.
from .functional import _high_NA_objective_lens_  # noqa: E402,F401
