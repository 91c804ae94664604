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


def rs_transfer(z, Xe, Ye, k):
    """wave_optics.py:291-297 with a distance that may be a tensor (differentiable in z)."""
    if not isinstance(z, torch.Tensor):
        return torch.as_tensor(ref.rs_transfer(z, Xe, Ye, k))
    z = z.to(torch.float64).reshape(())
    r = torch.sqrt(torch.as_tensor(Xe) ** 2 + torch.as_tensor(Ye) ** 2 + z ** 2)
    amp = z / (2.0 * np.pi * r ** 2) * (1.0 / r - 1j * k)
    sgn = 1.0 if float(z.detach()) > 0 else -1.0
    return torch.exp(sgn * 1j * k * r) * amp


def rs_propagate(field, x, y, wavelength, z):
    """wave_optics.py:281-289."""
    ny, nx = len(y), len(x)
    k = 2 * np.pi / wavelength
    Xe, Ye = np.meshgrid(ref.rs_offset_axis(x), ref.rs_offset_axis(y))
    H = rs_transfer(z, Xe, Ye, k)
    U = torch.zeros((2 * ny - 1, 2 * nx - 1), dtype=C128)
    U = U.index_put((torch.arange(ny)[:, None], torch.arange(nx)[None, :]), _t(field).to(C128))
    out = torch.fft.ifft2(torch.fft.fft2(U) * torch.fft.fft2(H)) * (x[1] - x[0]) * (y[1] - y[0])
    return out[ny - 1:, nx - 1:]


def vrs_propagate(Ex, Ey, x, y, wavelength, z):
    """vectorized_optics.py:244-284."""
    X, Y = (torch.as_tensor(a) for a in np.meshgrid(x, y))
    zz = z.to(torch.float64).reshape(()) if isinstance(z, torch.Tensor) else z
    r = torch.sqrt(X ** 2 + Y ** 2 + zz ** 2)
    Ez = Ex * (X / r) + Ey * (Y / r)
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


def building_block(Ex, Ey, x, y, wavelength, alpha, phi, z, eta, theta):
    """optical_elements.py:919-939: sSLM -> VRS(z) -> LCD (Ez of the output is the VRS's)."""
    ax, ay = sslm(Ex, Ey, alpha, phi)
    px, py, pz = vrs_propagate(ax, ay, x, y, wavelength, z)
    lx, ly = lcd(px, py, eta, theta)
    return lx, ly, pz


def hybrid_setup_sharp_focus(src, x, y, wavelength, parameters, r, f, xout, yout, distance_offset=8.9):
    """optical_elements.py:1503-1649 restated step by step (every source is
    ``src`` = (Ex, Ey)); returns the six detectors' |Ez|^2 stacked."""
    cm = 1e4

    def ang(p):
        return _t(p).to(torch.float64) * 2 * np.pi - np.pi

    def dist(p):
        return (torch.abs(_t(p).to(torch.float64)) * 100 + distance_offset) * cm

    P = parameters
    ph = [(ang(P[6 * b]), ang(P[6 * b + 1])) for b in range(3)]
    eta = [ang(P[6 * b + 2]) for b in range(3)]
    th = [ang(P[6 * b + 3]) for b in range(3)]
    z = [(dist(P[6 * b + 4]), dist(P[6 * b + 5])) for b in range(3)]
    bs = [ang(P[18 + k]) for k in range(9)]
    z4, z5 = dist(P[27]), dist(P[28])

    def V(E, zz):
        return vrs_propagate(E[0], E[1], x, y, wavelength, zz)

    def BB(E, b, z1, z2):
        lx, ly, _ = building_block(E[0], E[1], x, y, wavelength, ph[b][0], ph[b][1], z1, eta[b], th[b])
        return V((lx, ly), z2)

    def BS(a, b, t):
        cx, cy, dx, dy = bs_symmetric(a[0], a[1], b[0], b[1], t)
        return (cx, cy), (dx, dy)

    def det(E):
        return vczt_objective_lens(E[0], E[1], x, y, wavelength, r, f, xout, yout)

    c1, d1 = BS(src, src, bs[0])
    b2 = BB(c1, 0, z[0][0], z[0][1])
    c2, d2 = BS(src, b2, bs[1])
    b3 = V(c2, z[1][0] + z[1][1])
    c3, d3 = BS(src, b3, bs[2])
    det1 = det(V(c3, z[2][0] + z[2][1]))
    a5, a6 = V(d2, z4), V(d3, z4)
    c4, d4 = BS(d1, src, bs[3])
    b5 = V(c4, z[0][0] + z[0][1])
    c5, d5 = BS(a5, b5, bs[4])
    b6 = BB(c5, 1, z[1][0], z[1][1])
    c6, d6 = BS(a6, b6, bs[5])
    det2 = det(V(c6, z[2][0] + z[2][1]))
    a8, a9 = V(d5, z5), V(d6, z5)
    c7, d7 = BS(d4, src, bs[6])
    b8 = V(c7, z[0][0] + z[0][1])
    c8, d8 = BS(a8, b8, bs[7])
    b9 = V(c8, z[1][0] + z[1][1])
    c9, d9 = BS(a9, b9, bs[8])
    det3 = det(BB(c9, 2, z[2][0], z[2][1]))
    dets = [det1, det2, det3, det(d7), det(d8), det(d9)]
    return torch.stack([torch.abs(d[2]) ** 2 for d in dets])
