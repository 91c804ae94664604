"""FP64 CPU restatement of XLuminA's light-propagation path.

TEST INFRASTRUCTURE ONLY: this module is the oracle.  Only the tests, the
package smoke check and the benchmark's CPU-baseline / reference arms may
import it, and only to check or to time the CPU algorithm.  The product path
(``xlumina_gb300``) never calls it.

Every function restates one reference function in numpy float64 / complex128
(the reference forces ``jax_enable_x64`` at import, ``wave_optics.py:10-13``),
keeping the reference's layout choices and quirks so that results agree to
rounding: the (2N-1)-point RS pad, the reflect-built offset grid, the
transposed Bluestein output, the VRS / VCZT / high-NA ``Ez`` formulas, and the
polarizer / lens dropping ``Ez``.  Citations are ``file:line`` inside the
XLuminA repository.

Pinning: ``tests/golden/make_golden.py`` runs the reference's own source
(numpy-backed stand-in for jax) and stores its outputs as fixtures; the CPU
test-suite checks this module against them to ~1e-12.
"""
from __future__ import annotations

import os

import numpy as np
import scipy.fft as sfft

WORKERS = os.cpu_count() or 1

# units, xlumina/__init__.py:14-20
um = 1.0
nm = 1e-3
mm = 1e3
cm = 1e4


def _fft2(a):
    return sfft.fft2(a, workers=WORKERS)


def _ifft2(a):
    return sfft.ifft2(a, workers=WORKERS)


# ---------------------------------------------------------------- grids --

def space(x_total, num_pix):
    """toolbox.py:49-61 -- ``linspace(-x_total, x_total, num_pix)`` twice (half-width argument)."""
    x = np.linspace(-x_total, x_total, num_pix, dtype=np.float64)
    return x, x.copy()


def rs_offset_axis(x):
    """wave_optics.py:265-279 -- the 2N-1 offsets [-(N-1)dx .. 0 .. (N-1)dx].

    The reference reflect-pads ``x[0] - x[::-1]`` and flips the sign of the
    right half; the values are ``x[0]-x[N-1-j]`` then ``x[m]-x[0]``.
    """
    x = np.asarray(x, dtype=np.float64)
    left = x[0] - x[::-1]                       # -(N-1)dx ... 0
    right = x[1:] - x[0]                        # dx ... (N-1)dx
    return np.concatenate([left, right])


def rs_transfer(z, Xe, Ye, k):
    """wave_optics.py:291-297 -- RS impulse response on an offset grid.

    ``r = sqrt(X^2+Y^2+z^2)``; ``H = exp(+-ikr) * z/(2 pi r^2) * (1/r - ik)``,
    the sign of the exponent following the sign of z.
    """
    r = np.sqrt(Xe ** 2 + Ye ** 2 + z ** 2)
    amp = z / (2.0 * np.pi * r ** 2) * (1.0 / r - 1j * k)
    sgn = 1.0 if z > 0 else -1.0
    return np.exp(sgn * 1j * k * r) * amp


def rs_quality_factor(x, y, wavelength, z):
    """wave_optics.py:187-191 (and vectorized_optics.py:264-270)."""
    dx = x[1] - x[0]
    dy = y[1] - y[0]
    dr_real = np.sqrt(dx ** 2 + dy ** 2)
    rmax = np.sqrt((x ** 2).max() + (y ** 2).max())
    dr_ideal = np.sqrt(wavelength ** 2 + rmax ** 2 + 2 * wavelength * np.sqrt(rmax ** 2 + z ** 2)) - rmax
    return dr_ideal / dr_real


# ------------------------------------------------------------------ RS --

def rs_propagate(field, x, y, wavelength, z):
    """wave_optics.py:281-289 -- zero-pad to (2ny-1, 2nx-1), multiply spectra, crop.

    ``out = ifft2(fft2(U) * fft2(H)) * dx * dy`` cropped to ``[ny-1:, nx-1:]``.
    """
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    ny, nx = len(y), len(x)
    k = 2 * np.pi / wavelength
    dx = x[1] - x[0]
    dy = y[1] - y[0]
    Xe, Ye = np.meshgrid(rs_offset_axis(x), rs_offset_axis(y))
    H = rs_transfer(z, Xe, Ye, k)
    U = np.zeros((2 * ny - 1, 2 * nx - 1), dtype=np.complex128)
    U[:ny, :nx] = field
    out = _ifft2(_fft2(U) * _fft2(H)) * dx * dy
    return out[ny - 1:, nx - 1:]


def vrs_ez(Ex, Ey, x, y, z):
    """vectorized_optics.py:258-261 -- ``Ez = Ex*X/r + Ey*Y/r`` with r = sqrt(X^2+Y^2+z^2)."""
    X, Y = np.meshgrid(x, y)
    r = np.sqrt(X ** 2 + Y ** 2 + z ** 2)
    return Ex * X / r + Ey * Y / r


def vrs_propagate(Ex, Ey, x, y, wavelength, z):
    """vectorized_optics.py:244-284, 364-373 -- RS on (Ex, Ey, Ez), Ez derived, H shared.

    The incoming Ez is discarded.  Returns (Ex', Ey', Ez').
    """
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    ny, nx = len(y), len(x)
    k = 2 * np.pi / wavelength
    dx = x[1] - x[0]
    dy = y[1] - y[0]
    Ez = vrs_ez(Ex, Ey, x, y, z)
    Xe, Ye = np.meshgrid(rs_offset_axis(x), rs_offset_axis(y))
    Hhat = _fft2(rs_transfer(z, Xe, Ye, k))
    outs = []
    for comp in (Ex, Ey, Ez):
        U = np.zeros((2 * ny - 1, 2 * nx - 1), dtype=np.complex128)
        U[:ny, :nx] = comp
        outs.append((_ifft2(_fft2(U) * Hhat) * dx * dy)[ny - 1:, nx - 1:])
    return tuple(outs)


# ----------------------------------------------------------------- CZT --

def czt_grid(z, wavelength, xin, yin, xout, yout):
    """wave_optics.py:299-331 -- ``Dm = lambda z / dx`` and the frequency limits."""
    dx = xin[1] - xin[0]
    dy = yin[1] - yin[0]
    Dm = wavelength * z / dx
    return dict(nx=len(xout), ny=len(yout), dx=dx, dy=dy, Dm=Dm,
                fy1=yout[0] + Dm / 2, fy2=yout[-1] + Dm / 2,
                fx1=xout[0] + Dm / 2, fx2=xout[-1] + Dm / 2)


def next_pow2(v):
    """wave_optics.py:373-383 -- smallest power of two >= v."""
    return int(2 ** int(np.ceil(np.log2(v))))


def bluestein_vectors(m, f1, f2, Dm, M):
    """The 1-D chirp data of wave_optics.py:385-460 for an m-point input and M outputs.

    Returns ``(L, pre, g, post)``: Bluestein length L = next_pow2(m+M-1); the
    input weights ``pre[n] = A^-n h[m-1+n]``; the kernel spectrum
    ``g = fft(1/h[:mp+1], L)``; and the output weights
    ``post[l] = h[m-1+l] * exp(-i 2 pi l_f (1/2 - m/2) / Dm)``, where
    ``h[q] = W^((q-m+1)^2/2)`` (complex power, principal branch).
    """
    if M < 2:
        raise ValueError("Bluestein with a single output sample is not supported")
    D1 = f1 + (M * Dm + f2 - f1) / (2 * M)
    D2 = f2 + (M * Dm + f2 - f1) / (2 * M)
    mp = m + M - 1
    L = next_pow2(mp)
    A = np.exp(1j * 2 * np.pi * D1 / Dm)
    W = np.exp(-1j * 2 * np.pi * (D2 - D1) / (M * Dm))
    q = np.arange(-m + 1, max(M - 1, m - 1) + 1)
    h = W ** (q ** 2 / 2)
    g = np.fft.fft(1 / h[:mp + 1], L)
    pre = A ** (-np.arange(m)) * h[m - 1:2 * m - 1]
    lf = np.linspace(0, M - 1, M) / M * (D2 - D1) + D1
    post = h[m - 1:mp] * np.exp(-1j * 2 * np.pi * lf * (-m / 2 + 0.5) / Dm)
    return L, pre, g, post


def bluestein(xmat, f1, f2, Dm, M):
    """wave_optics.py:412-460 -- chirp-z along axis 0; the result is TRANSPOSED, shape (n, M)."""
    m, n = xmat.shape
    L, pre, g, post = bluestein_vectors(m, f1, f2, Dm, M)
    b = sfft.fft(xmat * pre[:, None], L, axis=0, workers=WORKERS)
    b = sfft.ifft(b * g[:, None], axis=0, workers=WORKERS)
    return b[m:m + M, :n].T * post[None, :]


def czt(field, x, y, wavelength, z, xout=None, yout=None):
    """wave_optics.py:233-263, 333-357 -- ``F0 * B_x(B_y(field*F)) * z*dx*dy*lambda``."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    xout = x if xout is None else np.asarray(xout, np.float64)
    yout = y if yout is None else np.asarray(yout, np.float64)
    k = 2 * np.pi / wavelength
    g = czt_grid(z, wavelength, x, y, xout, yout)
    X, Y = np.meshgrid(x, y)
    Xo, Yo = np.meshgrid(xout, yout)
    F0 = rs_transfer(z, Xo, Yo, k)
    F = rs_transfer(z, X, Y, k)
    U = bluestein(field * F, g["fy1"], g["fy2"], g["Dm"], g["ny"])
    U = bluestein(U, g["fx1"], g["fx2"], g["Dm"], g["nx"])
    return F0 * U * z * g["dx"] * g["dy"] * wavelength


def vczt_ez(Ex, Ey, x, y, z):
    """vectorized_optics.py:340-344 -- ``Ez = (Ex*X/r + Ey*Y/r) * z/r``."""
    X, Y = np.meshgrid(x, y)
    r = np.sqrt(X ** 2 + Y ** 2 + z ** 2)
    return (Ex * X / r + Ey * Y / r) * z / r


def vczt(Ex, Ey, x, y, wavelength, z, xout=None, yout=None):
    """vectorized_optics.py:321-361, 375-384 -- CZT of (Ex, Ey, Ez) with Ez derived."""
    Ez = vczt_ez(Ex, Ey, x, y, z)
    return tuple(czt(c, x, y, wavelength, z, xout, yout) for c in (Ex, Ey, Ez))


# ------------------------------------------------------- high-NA lens --

def high_na_lens(Ex, Ey, x, y, radius, f):
    """optical_elements.py:515-594 -- returns ((3,N,N) field, sin(theta_max)).

    theta = rho/f (not arcsin); Ez = Ex*X/rho + Ey*Y/rho (NaN at rho = 0);
    pupil-weighted G; E' = sqrt|cos theta| * G * RL(theta, phi) E.
    """
    X, Y = np.meshgrid(x, y)
    s_max = radius / np.sqrt(radius ** 2 + f ** 2)
    with np.errstate(invalid="ignore", divide="ignore"):
        rho = np.sqrt(X ** 2 + Y ** 2)
        phi = np.arctan2(Y, X)
        theta = rho / f
        Ez = Ex * X / rho + Ey * Y / rho
        u = X / radius
        v = Y / radius
        pupil = np.where((X ** 2 + Y ** 2) / radius ** 2 < 1, 1, 0)
        G = np.real(pupil * (1 / np.sqrt(np.abs(1 - (u ** 2 + v ** 2) * s_max ** 2))))
    ct, st, cp, sp = np.cos(theta), np.sin(theta), np.cos(phi), np.sin(phi)
    w = np.sqrt(np.abs(ct)) * G
    ox = (ct * cp ** 2 + sp ** 2) * Ex + (ct * cp * sp - sp * cp) * Ey - cp * st * Ez
    oy = (sp * ct * cp - cp * sp) * Ex + (ct * sp ** 2 + cp ** 2) * Ey - sp * st * Ez
    oz = st * cp * Ex + st * sp * Ey + ct * Ez
    return np.stack([w * ox, w * oy, w * oz]), s_max


def high_na_grid(f, r, wavelength, xin, xout, yout):
    """optical_elements.py:640-672 -- ``Dm = f*lambda*(Din-1)/(2r)`` and the limits."""
    Dm = f * wavelength * (len(xin) - 1) / (2 * r)
    return dict(nx=len(xout), ny=len(yout), Dm=Dm,
                fy1=yout[0] + Dm / 2, fy2=yout[-1] + Dm / 2,
                fx1=xout[0] + Dm / 2, fx2=xout[-1] + Dm / 2)


def vczt_objective_lens(Ex, Ey, x, y, wavelength, r, f, xout, yout):
    """optical_elements.py:600-638 with vectorized_optics.py:386-394 and wave_optics.py:359-371."""
    E, s_max = high_na_lens(Ex, Ey, x, y, r, f)
    g = high_na_grid(f, r, wavelength, x, xout, yout)
    cte = -(1j * s_max ** 2 / (f * wavelength))
    out = []
    for c in E:
        U = bluestein(c, g["fy1"], g["fy2"], g["Dm"], g["ny"])
        U = bluestein(U, g["fx1"], g["fx2"], g["Dm"], g["nx"])
        out.append(cte * U)
    return tuple(out)


# --------------------------------------------------------------- masks --

def slm(field, phase):
    """optical_elements.py:76-103 -- ``field * exp(i phase)``; returns (field, mask)."""
    mask = np.exp(1j * np.asarray(phase))
    return field * mask, mask


def jones_retarder(eta, theta, delta=0.0):
    """optical_elements.py:122-139 -- general retarder (LCD is delta = 0, :169-180)."""
    em, ep = np.exp(-0.5j * eta), np.exp(0.5j * eta)
    c, s = np.cos(theta), np.sin(theta)
    return (em * c ** 2 + ep * s ** 2, (em - ep) * np.exp(-1j * delta) * s * c,
            (em - ep) * np.exp(1j * delta) * s * c, em * s ** 2 + ep * c ** 2)


def lcd(Ex, Ey, eta, theta):
    """optical_elements.py:266-305 -- per-pixel (or scalar) retarder; Ez passes unchanged."""
    a, b, c, d = jones_retarder(eta, theta)
    return a * Ex + b * Ey, c * Ex + d * Ey


def linear_polarizer(Ex, Ey, alpha):
    """optical_elements.py:307-332 -- per-pixel LP; the output Ez is zero."""
    c, s = np.cos(alpha), np.sin(alpha)
    return c * c * Ex + c * s * Ey, c * s * Ex + s * s * Ey


def sslm(Ex, Ey, alpha, phi, a1=None, a2=None):
    """optical_elements.py:186-264 -- diag(A1 e^{i alpha}, A2 e^{i phi}); Ez passes unchanged."""
    ox = Ex * np.exp(1j * alpha)
    oy = Ey * np.exp(1j * phi)
    if a1 is not None:
        ox = a1 * ox
        oy = a2 * oy
    return ox, oy


def circular_mask(X, Y, r):
    """optical_elements.py:781-795."""
    rx, ry = r
    return np.where((X ** 2 / rx ** 2 + Y ** 2 / ry ** 2) < 1, 1, 0)


def lens_mask(x, y, wavelength, radius, focal):
    """optical_elements.py:678-703 -- ``pupil * exp(-ik(X^2/2fx + Y^2/2fy))``."""
    X, Y = np.meshgrid(x, y)
    k = 2 * np.pi / wavelength
    fx, fy = focal
    return circular_mask(X, Y, radius) * np.exp(-1j * k * (X ** 2 / (2 * fx) + Y ** 2 / (2 * fy)))


# ------------------------------------------------------------- sources --

def gaussian_beam(x, y, wavelength, w0, E0=1.0, center=(0, 0), z_w0=(0, 0), alpha=0.0):
    """wave_optics.py:468-523 -- scalar Gaussian (the R_y test of z_w0x at :507 is kept)."""
    k = 2 * np.pi / wavelength
    w0x, w0y = w0
    x0, y0 = center
    zx, zy = z_w0
    Rx_l = k * w0x ** 2 / 2
    Ry_l = k * w0y ** 2 / 2
    gx = np.arctan2(zx, Rx_l)
    gy = np.arctan2(zy, Ry_l)
    wx = w0x * np.sqrt(1 + (zx / Rx_l) ** 2)
    wy = w0y * np.sqrt(1 + (zy / Ry_l) ** 2)
    Rx = 1e12 if zx == 0 else zx * (1 + (Rx_l / zx) ** 2)
    Ry = 1e12 if zx == 0 else zy * (1 + (Ry_l / zy) ** 2)
    X, Y = np.meshgrid(x, y)
    xr = X * np.cos(alpha) + Y * np.sin(alpha)
    yr = -X * np.sin(alpha) + Y * np.cos(alpha)
    phase = np.exp(-1j * ((k * zx + k * X ** 2 / (2 * Rx) - gx) + (k * zy + k * Y ** 2 / (2 * Ry) - gy)))
    amp = (w0x / wx) * (w0y / wy) * np.exp(-(xr - x0) ** 2 / wx ** 2 - (yr - y0) ** 2 / wy ** 2)
    return E0 * amp * phase


def polarized_gaussian_beam(x, y, wavelength, w0, jones_vector, center=(0, 0), z_w0=(0, 0), alpha=0.0):
    """vectorized_optics.py:402-465 -- normalised Jones vector times the scalar beam; Ez = 0."""
    jv = np.asarray(jones_vector)
    jv = jv / np.linalg.norm(jv)
    g = gaussian_beam(x, y, wavelength, w0, 1.0, center, z_w0, alpha)
    return jv[0] * g, jv[1] * g


def plane_wave(x, y, wavelength, A=1.0, theta=0.0, phi=0.0, z0=0.0):
    """wave_optics.py:525-542."""
    k = 2 * np.pi / wavelength
    X, Y = np.meshgrid(x, y)
    return A * np.exp(1j * k * (X * np.sin(theta) * np.cos(phi) + Y * np.sin(theta) * np.sin(phi)
                                + z0 * np.cos(theta)))


# ------------------------------------------------------- beam splitters --

def bs_loss_rt(theta):
    """optical_elements.py:376-383 -- R = |sin|, T = |cos|, both less 1% of |cos|."""
    T = np.abs(np.cos(theta))
    R = np.abs(np.sin(theta))
    noise = T * 0.01
    return R - noise, T - noise


def bs_symmetric(aEx, aEy, bEx, bEy, theta):
    """optical_elements.py:334-391 -- returns (cEx, cEy, dEx, dEy); Ez of c, d is zero."""
    R, T = bs_loss_rt(theta)
    return R * aEx + 1j * T * bEx, R * aEy + 1j * T * bEy, 1j * T * aEx + R * bEx, 1j * T * aEy + R * bEy


def bs_symmetric_si(aEx, aEy, theta, port=0):
    """optical_elements.py:393-460 -- single input; port 0: c = R a, d = iT a; port 1 swaps."""
    R, T = bs_loss_rt(theta)
    if port == 0:
        return R * aEx, R * aEy, 1j * T * aEx, 1j * T * aEy
    return 1j * T * aEx, 1j * T * aEy, R * aEx, R * aEy


def bs_lossless(a1Ex, a1Ey, a2Ex, a2Ey, R, T, phase):
    """optical_elements.py:462-512 -- returns (b1Ex, b1Ey, b2Ex, b2Ey)."""
    sT, sR = np.sqrt(T), np.sqrt(R)
    e, ec = np.exp(1j * phase), np.exp(-1j * phase)
    return (sT * a1Ex + sR * e * a2Ex, sT * a1Ey + sR * e * a2Ey,
            -sR * ec * a1Ex + sT * a2Ex, -sR * ec * a1Ey + sT * a2Ey)


def fluorescence(i_ex, i_dep, beta=1):
    """optical_elements.py:941-954 -- i_ex (1 - beta (1 - exp(-i_dep / (i_ex + 1e-8))))."""
    return i_ex * (1 - beta * (1 - np.exp(-(i_dep / (i_ex + 1e-8)))))


# -------------------------------------------------------------- losses --

def mse_intensity(a, b):
    """loss_functions.py:137-149 -- ``sum((|a|^2 - |b|^2)^2) / num_pix``."""
    return np.sum((np.abs(a) ** 2 - np.abs(b) ** 2) ** 2) / (a.shape[0] * a.shape[1])


def small_area_hybrid(I):
    """loss_functions.py:24-40 -- area over the 0.7*max threshold / enclosed intensity."""
    In = I / (np.sum(I) + 1e-08)
    mask = np.where(In > 0.7 * np.max(In), 1, 0)
    return np.sum(mask) / (np.sum(mask * In) + 1e-08)


# ---------------------------------------------------------------- noise --
# The table noise is drawn with Philox4x32-10 (Salmon et al., SC 2011), not
# with jax's streams; this restatement pins the device generator bit for bit.

def philox4x32_10(counter, key):
    """Philox4x32 with 10 rounds on python ints: 4-word counter, 2-word key."""
    c = [int(v) & 0xFFFFFFFF for v in counter]
    k0, k1 = int(key[0]) & 0xFFFFFFFF, int(key[1]) & 0xFFFFFFFF
    for r in range(10):
        p0 = 0xD2511F53 * c[0]
        p1 = 0xCD9E8D57 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k0) & 0xFFFFFFFF, p1 & 0xFFFFFFFF,
             ((p0 >> 32) ^ c[3] ^ k1) & 0xFFFFFFFF, p0 & 0xFFFFFFFF]
        if r < 9:
            k0 = (k0 + 0x9E3779B9) & 0xFFFFFFFF
            k1 = (k1 + 0xBB67AE85) & 0xFFFFFFFF
    return c


def table_noise_element(key, plane_index, min_phase, max_phase, discretize=False):
    """(slm, amp) noise value of flat plane element ``plane_index`` of a table
    keyed ``key``: one magnitude (stream 2), two signs (streams 3 and 4)."""
    e = int(plane_index)
    cm = philox4x32_10((e & 0xFFFFFFFF, e >> 32, 2, 0), key)
    cs = philox4x32_10((e & 0xFFFFFFFF, e >> 32, 3, 0), key)
    ca = philox4x32_10((e & 0xFFFFFFFF, e >> 32, 4, 0), key)
    lo = np.float32(min_phase)
    span = np.float32(float(max_phase) - float(min_phase))
    u = np.float32((cm[0] >> 8) * (1.0 / 16777216.0))
    mag = np.float32(lo + np.float32(span * u))        # float32 product, then float32 sum
    neg = np.float32(255.0 if discretize else -1.0)
    return (np.float32((1.0 if cs[0] & 1 else neg) * mag), np.float32((1.0 if ca[0] & 1 else neg) * mag))


def table_noise_scalars(key, n_distances, n_wps, min_d, max_d, min_phase, max_phase):
    """(distances, waveplate noise) of a table keyed ``key`` (streams 1, 5, 6)."""
    def u53(a, b):
        return ((a >> 5) * 67108864.0 + (b >> 6)) * (1.0 / 9007199254740992.0)
    d = []
    for i in range(n_distances):
        c = philox4x32_10((i, 0, 1, 0), key)
        d.append(min_d + (max_d - min_d) * u53(c[0], c[1]))
    w = []
    for i in range(n_wps):
        cs = philox4x32_10((i, 0, 5, 0), key)
        cm = philox4x32_10((i, 0, 6, 0), key)
        w.append((1.0 if cs[0] & 1 else -1.0) * (min_phase + (max_phase - min_phase) * u53(cm[0], cm[1])))
    return np.array(d), np.array(w)
