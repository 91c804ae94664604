"""The reference's array-level entry points (the functions its light classes
call inside): RS_propagation_jit, transfer_function_RS, CZT_jit,
CZT_for_high_NA_jit, Bluestein_method, compute_fft (wave_optics.py:281-460),
VRS_propagation_jit, VCZT_jit, vectorized_CZT_for_high_NA
(vectorized_optics.py:362-394) and _high_NA_objective_lens_
(optical_elements.py:555-594), with the same arguments and results.

The propagators run on the library's kernels: a grid is rebuilt from the
spacings and output grids passed in (the transfer function depends on
coordinate differences only), and the stacked (3, N, N) forms run as a
batch of three fields.  ``Bluestein_method`` and ``compute_fft``, the
one-axis building blocks, keep the reference's float64 chirps and run their
transforms on the library's complex64 line FFTs (xl_fft_lines); the
propagators do not use them.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib, engine


def _axis(n, d):
    return np.arange(int(n), dtype=np.float64) * float(d)


def _c64(a):
    return engine.as_field(a)


# ------------------------------------------------------------------- RS --

def transfer_function_RS(z, Xext, Yext, k):
    """wave_optics.py:291-297: the RS impulse response on the grids given (float64 on the device)."""
    dev = engine.device()
    X = torch.as_tensor(np.asarray(Xext, dtype=np.float64) if not isinstance(Xext, torch.Tensor) else Xext,
                        device=dev, dtype=torch.float64)
    Y = torch.as_tensor(np.asarray(Yext, dtype=np.float64) if not isinstance(Yext, torch.Tensor) else Yext,
                        device=dev, dtype=torch.float64)
    zt = z.to(device=dev, dtype=torch.float64) if isinstance(z, torch.Tensor) else torch.tensor(float(z), device=dev,
                                                                                               dtype=torch.float64)
    r = torch.sqrt(X ** 2 + Y ** 2 + zt ** 2)
    factor = zt / (2 * np.pi * r ** 2) * (1 / r - 1j * k)
    one = torch.ones((), dtype=torch.float64, device=dev)
    sgn = torch.where(zt > 0, one, -one)            # float64: k r is ~1e4 rad and more
    return torch.polar(torch.ones_like(r), sgn * k * r) * factor


def RS_propagation_jit(input_field, z, nx, ny, dx, dy, Xext, Yext, k):
    """wave_optics.py:281-289: one (ny, nx) field propagated over z."""
    wl = 2 * np.pi / k
    return engine.rs_propagate([_c64(input_field)], _axis(nx, dx), _axis(ny, dy), wl, z, vector=False)[0]


def VRS_propagation_jit(input_field, z, nx, ny, dx, dy, Xext, Yext, k):
    """vectorized_optics.py:362-373: the three components of a (3, N, N) field
    propagated with the same transfer function (one batched call)."""
    return RS_propagation_jit(input_field, z, nx, ny, dx, dy, Xext, Yext, k)


# ------------------------------------------------------------------ CZT --

def CZT_jit(field, z, wavelength, k, nx, ny, dx, dy, Xout, Yout, X, Y, Dm, fy_1, fy_2, fx_1, fx_2):
    """wave_optics.py:333-357 (grids from build_CZT_grid); a leading batch axis is allowed."""
    x, y = np.asarray(X)[0, :], np.asarray(Y)[:, 0]
    xo, yo = np.asarray(Xout)[0, :], np.asarray(Yout)[:, 0]
    return engine.czt_propagate([_c64(field)], x, y, wavelength, z, xo, yo, mode="scalar")[0]


def VCZT_jit(field, z, wavelength, k, nx, ny, dx, dy, Xout, Yout, X, Y, Dm, fy_1, fy_2, fx_1, fx_2):
    """vectorized_optics.py:375-384: CZT_jit of each component of a (3, N, N) field (one batched call)."""
    return CZT_jit(field, z, wavelength, k, nx, ny, dx, dy, Xout, Yout, X, Y, Dm, fy_1, fy_2, fx_1, fx_2)


def CZT_for_high_NA_jit(field, nx, ny, Dm, fy_1, fy_2, fx_1, fx_2):
    """wave_optics.py:359-371: the two Bluestein transforms alone onto ny x nx
    outputs (no transfer functions); a leading batch axis is allowed."""
    return engine.czt_plain([_c64(field)], int(nx), int(ny), Dm, fy_1, fy_2, fx_1, fx_2)[0]


def vectorized_CZT_for_high_NA(field, nx, ny, Dm, fy_1, fy_2, fx_1, fx_2):
    """vectorized_optics.py:386-394: CZT_for_high_NA_jit of each component (one batched call)."""
    return CZT_for_high_NA_jit(field, nx, ny, Dm, fy_1, fy_2, fx_1, fx_2)


def compute_np2(x):
    """wave_optics.py:373-383: the next power of two >= x."""
    return 2 ** (np.ceil(np.log2(x))).astype(int)


def fft_lines(a: torch.Tensor, n: int, dim: int, inverse: bool = False) -> torch.Tensor:
    """The n-point FFT (n a power of two, up to 8192) of ``a`` along ``dim``,
    zero-padded or cropped to n as jnp.fft.fft(a, n, axis) does; unnormalised
    forward, or inverse with the 1/n of jnp.fft.ifft.  Runs in complex64 on the
    library's line transforms (xl_fft_lines) and returns complex128."""
    n = int(n)
    logn = int(np.log2(n))
    if 1 << logn != n or logn > 13:
        raise ValueError(f"FFT length must be a power of two up to 8192, got {n}")
    a = torch.movedim(a, dim, -1)
    m = a.shape[-1]
    lines = a.reshape(-1, m)
    buf = torch.zeros((lines.shape[0], n), dtype=torch.complex64, device=a.device)
    buf[:, :min(m, n)] = lines[:, :min(m, n)].to(torch.complex64)
    out = buf if logn >= 5 else torch.empty_like(buf)
    _lib.check(engine.lib().xl_fft_lines(engine.stream_handle(), logn, buf.shape[0], 1 if inverse else -1,
                                         buf.data_ptr(), out.data_ptr()), "xl_fft_lines")
    res = out.to(torch.complex128)
    if inverse:
        res = res / n
    return torch.movedim(res.reshape(a.shape[:-1] + (n,)), -1, dim)


def compute_fft(x, D1, D2, Dm, m, n, mp, M_out, np2):
    """wave_optics.py:385-410: Bluestein's convolution along axis 0 of an (m, n)
    array (length-np2 transforms on the library's line FFTs); returns (b, h)."""
    dev = engine.device()
    x = torch.as_tensor(np.asarray(x) if not isinstance(x, torch.Tensor) else x, device=dev).to(torch.complex128)
    A = np.exp(1j * 2 * np.pi * D1 / Dm)
    W = np.exp(-1j * 2 * np.pi * (D2 - D1) / (M_out * Dm))
    kk = np.arange(-m + 1, max(M_out - 1, m - 1) + 1, dtype=np.float64)
    h = torch.as_tensor(W ** (kk ** 2 / 2), device=dev)
    ft = fft_lines(1 / h[:mp + 1], np2, 0)
    b = torch.as_tensor(A ** (-np.arange(m, dtype=np.float64)), device=dev) * h[m - 1:2 * m - 1]
    B = fft_lines(x * b[:, None], np2, 0)
    return fft_lines(B * ft[:, None], np2, 0, inverse=True), h


def Bluestein_method(x, f1, f2, Dm, M_out):
    """wave_optics.py:412-460: chirp-z along axis 0 of an (m, n) array onto
    M_out points of [f1, f2]; the result is transposed, (n, M_out)."""
    m, n = x.shape
    D1 = f1 + (M_out * Dm + f2 - f1) / (2 * M_out)
    D2 = f2 + (M_out * Dm + f2 - f1) / (2 * M_out)
    mp = m + M_out - 1
    b, h = compute_fft(x, D1, D2, Dm, m, n, mp, M_out, compute_np2(mp))
    if M_out > 1:
        b = b[m:mp + 1, 0:n].T * h[m - 1:mp][None, :]
    else:
        b = b[0] * h[0]
    dev = b.device
    l = torch.linspace(0, M_out - 1, M_out, dtype=torch.float64, device=dev) / M_out * (D2 - D1) + D1
    shift = torch.exp(-1j * 2 * np.pi * l * (-m / 2 + 1 / 2) / Dm)
    return b * shift[None, :]


# ----------------------------------------------------------- high-NA lens --

def _high_NA_objective_lens_(incoming_light, theta, phi, G):
    """optical_elements.py:555-594: E' = sqrt|cos theta| G RL(theta, phi) E for
    incoming_light (N, N, 3) (Ex, Ey, Ez last); returns (3, N, N)."""
    dev = engine.device()

    def t(a):
        return torch.as_tensor(np.asarray(a) if not isinstance(a, torch.Tensor) else a, device=dev)
    E = t(incoming_light)
    th, ph, G = (t(a).to(torch.float64) for a in (theta, phi, G))
    Ex, Ey, Ez = E[..., 0], E[..., 1], E[..., 2]
    ct, st, cp, sp = torch.cos(th), torch.sin(th), torch.cos(ph), torch.sin(ph)
    w = torch.sqrt(torch.abs(ct)) * G
    ox = (ct * cp ** 2 + sp ** 2) * Ex + (ct * cp * sp - sp * cp) * Ey - cp * st * Ez
    oy = (sp * ct * cp - cp * sp) * Ex + (ct * sp ** 2 + cp ** 2) * Ey - sp * st * Ez
    oz = st * cp * Ex + st * sp * Ey + ct * Ez
    return torch.stack([w * ox, w * oy, w * oz])
