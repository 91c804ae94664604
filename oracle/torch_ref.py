"""Differentiable FP64 restatement of the propagation path in torch (CPU, complex128).

TEST INFRASTRUCTURE ONLY: the gradient oracle.  It restates the same
reference functions as ``oracle/xlumina_ref.py`` (same layouts: the 2N-1 RS
pad, the transposed Bluestein, the Ez formulas) with torch operations so that
torch autograd gives the gradients jax.grad would give through the reference
(e.g. experiments/four_f_optimizer.py:43).  ``tests/test_oracle_golden.py``
pins its forward values to the numpy oracle.
"""
from __future__ import annotations

import numpy as np
import torch

from . import xlumina_ref as ref

C128 = torch.complex128


def _t(a):
    return a if isinstance(a, torch.Tensor) else torch.as_tensor(np.asarray(a))


def rs_propagate(field, x, y, wavelength, z):
    """wave_optics.py:281-289."""
    ny, nx = len(y), len(x)
    k = 2 * np.pi / wavelength
    Xe, Ye = np.meshgrid(ref.rs_offset_axis(x), ref.rs_offset_axis(y))
    H = torch.as_tensor(ref.rs_transfer(z, Xe, Ye, k))
    U = torch.zeros((2 * ny - 1, 2 * nx - 1), dtype=C128)
    U = U.index_put((torch.arange(ny)[:, None], torch.arange(nx)[None, :]), _t(field).to(C128))
    out = torch.fft.ifft2(torch.fft.fft2(U) * torch.fft.fft2(H)) * (x[1] - x[0]) * (y[1] - y[0])
    return out[ny - 1:, nx - 1:]


def vrs_propagate(Ex, Ey, x, y, wavelength, z):
    """vectorized_optics.py:244-284."""
    X, Y = np.meshgrid(x, y)
    r = np.sqrt(X ** 2 + Y ** 2 + z ** 2)
    Ez = Ex * torch.as_tensor(X / r) + Ey * torch.as_tensor(Y / r)
    return tuple(rs_propagate(c, x, y, wavelength, z) for c in (Ex, Ey, Ez))


def bluestein(xmat, f1, f2, Dm, M):
    """wave_optics.py:412-460 (transposed output)."""
    m, n = xmat.shape
    L, pre, g, post = ref.bluestein_vectors(m, f1, f2, Dm, M)
    b = torch.fft.fft(xmat * torch.as_tensor(pre)[:, None], L, dim=0)
    b = torch.fft.ifft(b * torch.as_tensor(g)[:, None], dim=0)
    return b[m:m + M, :n].T * torch.as_tensor(post)[None, :]


def czt(field, x, y, wavelength, z, xout, yout):
    """wave_optics.py:233-263, 333-357."""
    k = 2 * np.pi / wavelength
    g = ref.czt_grid(z, wavelength, x, y, xout, yout)
    X, Y = np.meshgrid(x, y)
    Xo, Yo = np.meshgrid(xout, yout)
    F0 = torch.as_tensor(ref.rs_transfer(z, Xo, Yo, k))
    F = torch.as_tensor(ref.rs_transfer(z, X, Y, k))
    U = bluestein(_t(field).to(C128) * F, g["fy1"], g["fy2"], g["Dm"], g["ny"])
    U = bluestein(U, g["fx1"], g["fx2"], g["Dm"], g["nx"])
    return F0 * U * z * g["dx"] * g["dy"] * wavelength


def vczt(Ex, Ey, x, y, wavelength, z, xout, yout):
    """vectorized_optics.py:321-361."""
    X, Y = np.meshgrid(x, y)
    r = np.sqrt(X ** 2 + Y ** 2 + z ** 2)
    Ez = (Ex * torch.as_tensor(X / r) + Ey * torch.as_tensor(Y / r)) * torch.as_tensor(z / r)
    return tuple(czt(c, x, y, wavelength, z, xout, yout) for c in (Ex, Ey, Ez))


def high_na_lens(Ex, Ey, x, y, radius, f):
    """optical_elements.py:515-594 (the per-pixel weights are geometry: float64 constants)."""
    X, Y = np.meshgrid(x, y)
    s_max = radius / np.sqrt(radius ** 2 + f ** 2)
    with np.errstate(invalid="ignore", divide="ignore"):
        rho = np.sqrt(X ** 2 + Y ** 2)
        th = rho / f
        ph = np.arctan2(Y, X)
        ux, uy = X / rho, Y / rho
        G = np.real(np.where((X ** 2 + Y ** 2) / radius ** 2 < 1, 1, 0) /
                    np.sqrt(np.abs(1 - ((X / radius) ** 2 + (Y / radius) ** 2) * s_max ** 2)))
    ct, st, cp, sp = np.cos(th), np.sin(th), np.cos(ph), np.sin(ph)
    w = np.sqrt(np.abs(ct)) * G
    T = lambda a: torch.as_tensor(a)  # noqa: E731
    Ez = Ex * T(ux) + Ey * T(uy)
    ox = Ex * T(ct * cp ** 2 + sp ** 2) + Ey * T(ct * cp * sp - sp * cp) + Ez * T(-cp * st)
    oy = Ex * T(sp * ct * cp - cp * sp) + Ey * T(ct * sp ** 2 + cp ** 2) + Ez * T(-sp * st)
    oz = Ex * T(st * cp) + Ey * T(st * sp) + Ez * T(ct)
    return (ox * T(w), oy * T(w), oz * T(w)), s_max


def vczt_objective_lens(Ex, Ey, x, y, wavelength, r, f, xout, yout):
    """optical_elements.py:600-638."""
    E, s_max = high_na_lens(Ex, Ey, x, y, r, f)
    g = ref.high_na_grid(f, r, wavelength, x, xout, yout)
    cte = -(1j * s_max ** 2 / (f * wavelength))
    out = []
    for c in E:
        U = bluestein(c, g["fy1"], g["fy2"], g["Dm"], g["ny"])
        U = bluestein(U, g["fx1"], g["fx2"], g["Dm"], g["nx"])
        out.append(cte * U)
    return tuple(out)


def slm(field, phase):
    """optical_elements.py:87-103."""
    return field * torch.exp(1j * _t(phase).to(torch.float64))


def sslm(Ex, Ey, alpha, phi):
    """optical_elements.py:186-222."""
    return Ex * torch.exp(1j * _t(alpha).to(torch.float64)), Ey * torch.exp(1j * _t(phi).to(torch.float64))


def lcd(Ex, Ey, eta, theta):
    """optical_elements.py:266-305 via the retarder of :122-139 (delta = 0)."""
    eta = _t(eta).to(torch.float64)
    theta = _t(theta).to(torch.float64)
    em, ep = torch.exp(-0.5j * eta), torch.exp(0.5j * eta)
    c, s = torch.cos(theta), torch.sin(theta)
    a = em * c ** 2 + ep * s ** 2
    b = (em - ep) * s * c
    d = em * s ** 2 + ep * c ** 2
    return a * Ex + b * Ey, b * Ex + d * Ey


def linear_polarizer(Ex, Ey, alpha):
    """optical_elements.py:307-332."""
    alpha = _t(alpha).to(torch.float64)
    c, s = torch.cos(alpha), torch.sin(alpha)
    return c * c * Ex + c * s * Ey, c * s * Ex + s * s * Ey


def lens(field, x, y, wavelength, radius, focal):
    """optical_elements.py:678-703."""
    return field * torch.as_tensor(ref.lens_mask(x, y, wavelength, radius, focal))


def bs_symmetric(aEx, aEy, bEx, bEy, theta):
    """optical_elements.py:334-391."""
    theta = _t(theta).to(torch.float64)
    T, R = torch.abs(torch.cos(theta)), torch.abs(torch.sin(theta))
    noise = T * 0.01
    T, R = T - noise, R - noise
    return R * aEx + 1j * T * bEx, R * aEy + 1j * T * bEy, 1j * T * aEx + R * bEx, 1j * T * aEy + R * bEy


def bs_symmetric_si(aEx, aEy, theta, port=0):
    """optical_elements.py:393-460."""
    theta = _t(theta).to(torch.float64)
    T, R = torch.abs(torch.cos(theta)), torch.abs(torch.sin(theta))
    noise = T * 0.01
    T, R = T - noise, R - noise
    if port == 0:
        return R * aEx, R * aEy, 1j * T * aEx, 1j * T * aEy
    return 1j * T * aEx, 1j * T * aEy, R * aEx, R * aEy


def fluorescence(i_ex, i_dep, beta=1):
    """optical_elements.py:941-954."""
    return i_ex * (1 - beta * (1 - torch.exp(-(i_dep / (i_ex + 1e-8)))))


def mse_intensity(a, b):
    """loss_functions.py:137-149."""
    return torch.sum((torch.abs(a) ** 2 - torch.abs(b) ** 2) ** 2) / (a.shape[0] * a.shape[1])


def small_area_hybrid(I):
    """loss_functions.py:24-40."""
    In = I / (torch.sum(I) + 1e-08)
    mask = (In > 0.7 * torch.max(In)).to(In.dtype)
    return torch.sum(mask) / (torch.sum(mask * In) + 1e-08)
