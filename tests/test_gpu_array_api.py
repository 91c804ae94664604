"""The reference's array-level entry points (RS_propagation_jit,
VRS_propagation_jit, transfer_function_RS, CZT_jit, CZT_for_high_NA_jit,
vectorized forms, Bluestein_method, _high_NA_objective_lens_) against the
outputs of the reference's own source (tests/golden/array_api.npz).
Bars: propagators rel-L2 1e-5 (complex64 kernels); Bluestein_method 1e-5
(float64 chirps, complex64 line transforms); the other float64 helpers 1e-10."""
import numpy as np
import pytest

from tests.conftest import golden, rel_l2

pytestmark = pytest.mark.gpu


def test_array_level_entry_points():
    import xlumina_gb300.optical_elements as oe
    import xlumina_gb300.vectorized_optics as vo
    import xlumina_gb300.wave_optics as wo
    g = golden("array_api")
    x, y, wl = g["x"], g["y"], float(g["wavelength"])
    k = 2 * np.pi / wl
    nx, ny, dx, dy, Xe, Ye = wo.build_grid(x, y)
    out = wo.RS_propagation_jit(g["field"], 2100.0, nx, ny, dx, dy, Xe, Ye, k)
    assert rel_l2(out.cpu().numpy(), g["rs_jit"]) < 1e-5
    out3 = vo.VRS_propagation_jit(g["E3"], 2100.0, nx, ny, dx, dy, Xe, Ye, k)
    assert out3.shape == (3, 36, 36) and rel_l2(out3.cpu().numpy(), g["vrs_jit"]) < 1e-5
    H = wo.transfer_function_RS(2100.0, Xe, Ye, k)
    assert rel_l2(H.cpu().numpy(), g["H"]) < 1e-10
    xo, yo = g["xout"], g["yout"]
    Dm, fy1, fy2, fx1, fx2 = g["czt_grid"]
    Xg, Yg = np.meshgrid(x, y)
    Xo, Yo = np.meshgrid(xo, yo)
    c = wo.CZT_jit(g["field"], 2500.0, wl, k, len(xo), len(yo), dx, dy, Xo, Yo, Xg, Yg, Dm, fy1, fy2, fx1, fx2)
    assert rel_l2(c.cpu().numpy(), g["czt_jit"]) < 1e-5
    hnx, hny, hDm, hfy1, hfy2, hfx1, hfx2 = g["hna_grid"]
    p = wo.CZT_for_high_NA_jit(g["field"], int(hnx), int(hny), hDm, hfy1, hfy2, hfx1, hfx2)
    assert rel_l2(p.cpu().numpy(), g["plain"]) < 1e-5
    p3 = vo.vectorized_CZT_for_high_NA(np.stack([g["field"]] * 3), int(hnx), int(hny), hDm, hfy1, hfy2, hfx1, hfx2)
    assert p3.shape == (3, int(hny), int(hnx)) and rel_l2(p3[1].cpu().numpy(), g["plain"]) < 1e-5
    b = wo.Bluestein_method(g["field"], -12.0, 15.0, 60.0, 20)
    assert rel_l2(b.cpu().numpy(), g["bluestein"]) < 1e-5
    lh = oe._high_NA_objective_lens_(np.moveaxis(g["E3"], 0, -1), g["theta"], g["phi"], g["G"])
    assert rel_l2(lh.cpu().numpy(), g["lens_helper"]) < 1e-10


@pytest.mark.parametrize("logn", [0, 2, 4, 5, 9, 12, 13])
@pytest.mark.parametrize("inverse", [False, True])
def test_fft_lines_match_numpy(logn, inverse):
    """The bare line transforms behind compute_fft / Bluestein_method (no
    cuFFT): along either axis, with zero padding and cropping, against numpy."""
    import torch

    from xlumina_gb300 import functional as fn
    n = 1 << logn
    rng = np.random.default_rng(logn + 50 * inverse)
    for m, axis in ((max(1, n - 3), 0), (n + 5, 1)):
        a = rng.standard_normal((m, 7)) + 1j * rng.standard_normal((m, 7))
        if axis == 1:
            a = a.T.copy()
        got = fn.fft_lines(torch.as_tensor(a, device="cuda"), n, axis, inverse=inverse).cpu().numpy()
        exp = np.fft.ifft(a, n, axis=axis) if inverse else np.fft.fft(a, n, axis=axis)
        assert rel_l2(got, exp) < 1e-6 * max(1, logn)
