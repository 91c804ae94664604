"""Chirp-z propagation on the GPU (CZT, VCZT, high-NA lens and focus, a 4f
chain) against the golden fixtures from the reference's own source and the
FP64 oracle.  Tolerance: complex64 rel-L2 <= 1e-5."""
import numpy as np
import pytest

from oracle import xlumina_ref as ref
from tests.conftest import golden, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _np(t):
    return t.detach().cpu().numpy().astype(np.complex128)


@pytest.fixture(scope="module")
def xl():
    import xlumina_gb300.optical_elements as oe
    import xlumina_gb300.vectorized_optics as vo
    import xlumina_gb300.wave_optics as wo
    return wo, vo, oe


def test_czt_default_and_roi_golden(xl):
    wo, vo, oe = xl
    g = golden("czt")
    light = wo.ScalarLight(g["x"], g["y"], float(g["wavelength"]))
    light.field = g["field_in"]
    out = light.CZT(float(g["z"]))
    assert out.field.shape == (64, 64)
    assert rel_l2(_np(out.field), g["out_default"]) < TOL
    out = light.CZT(float(g["z"]), g["xout"], g["yout"])
    assert out.field.shape == (40, 48)
    assert rel_l2(_np(out.field), g["out_roi"]) < TOL


def test_vczt_golden(xl):
    wo, vo, oe = xl
    g = golden("vczt")
    light = vo.VectorizedLight(g["x"], g["y"], float(g["wavelength"]))
    light.Ex, light.Ey = g["Ex_in"], g["Ey_in"]
    out = light.VCZT(float(g["z"]), g["xout"], g["yout"])
    for key in ("Ex", "Ey", "Ez"):
        assert rel_l2(_np(getattr(out, key)), g[key]) < TOL, key


def test_high_na_lens_and_focus_golden(xl):
    wo, vo, oe = xl
    g = golden("high_na")
    light = vo.VectorizedLight(g["x"], g["y"], float(g["wavelength"]))
    light.Ex, light.Ey = g["Ex_in"], g["Ey_in"]
    E, smax = oe.high_NA_objective_lens(light, float(g["radius"]), float(g["f"]))
    assert smax == pytest.approx(float(g["sin_theta_max"]), rel=1e-14)
    assert rel_l2(_np(E), g["lens_out"]) < 1e-6
    out = oe.VCZT_objective_lens(light, float(g["radius"]), float(g["f"]), g["xout"], g["yout"])
    for key in ("Ex", "Ey", "Ez"):
        assert rel_l2(_np(getattr(out, key)), g[key]) < TOL, key


def test_four_f_chain_golden(xl):
    wo, vo, oe = xl
    g = golden("four_f")
    f = float(g["f"])
    src = wo.LightSource(g["x"], g["y"], float(g["wavelength"]))
    src.field = g["source"]
    l1, _ = oe.SLM(src, g["phase1"], 64)
    l2, _ = l1.RS_propagation(f)
    assert rel_l2(_np(l2.field), g["after_rs"]) < TOL
    l3, _ = oe.lens(l2, (200.0, 200.0), (f, f))
    l4 = l3.CZT(f, g["xout"], g["yout"])
    assert rel_l2(_np(l4.field), g["after_czt1"]) < TOL
    l5, _ = oe.SLM(l4, g["phase2"], 32)
    l6 = l5.CZT(f)
    assert rel_l2(_np(l6.field), g["out"]) < TOL
    assert rel_l2(np.abs(_np(l6.field)) ** 2, g["intensity"]) < TOL


@pytest.mark.parametrize("n,m", [(256, 128), (512, 300), (1000, 500)])
def test_czt_against_oracle(xl, n, m):
    wo, vo, oe = xl
    x, y = ref.space(1500.0, n)
    rng = np.random.default_rng(n + m)
    field = ref.gaussian_beam(x, y, 0.532, (600.0, 600.0)) * np.exp(1j * rng.uniform(-np.pi, np.pi, (n, n)))
    xo = np.linspace(-200.0, 200.0, m)
    yo = np.linspace(-150.0, 150.0, m + 3)
    light = wo.ScalarLight(x, y, 0.532)
    light.field = field
    out = light.CZT(2.5e5, xo, yo)
    exp = ref.czt(field, x, y, 0.532, 2.5e5, xo, yo)
    assert rel_l2(_np(out.field), exp) < TOL


def test_high_na_focus_full_size(xl):
    """2048^2 input at 650 nm, NA 0.9, f = 3 mm, focal ROI 1024^2 over 2 um."""
    wo, vo, oe = xl
    n = 2048
    x, y = ref.space(2700.0, n)
    f = 3000.0
    r = 0.9 * f
    rng = np.random.default_rng(3)
    Ex, Ey = ref.polarized_gaussian_beam(x, y, 0.650, (1500.0, 1500.0), (1, 0))
    eta, theta = 1.1, 0.4
    a, p = rng.uniform(0, 2 * np.pi, (n, n)), rng.uniform(0, 2 * np.pi, (n, n))
    src = vo.VectorizedLight(x, y, 0.650)
    src.Ex, src.Ey = Ex, Ey
    light = oe.sSLM(oe.LCD(src, eta, theta), a, p)
    xo, yo = ref.space(1.0, 1024)
    out = oe.VCZT_objective_lens(light, r, f, xo, yo)
    Ex1, Ey1 = ref.sslm(*ref.lcd(Ex, Ey, eta, theta), a, p)
    exp = ref.vczt_objective_lens(Ex1, Ey1, x, y, 0.650, r, f, xo, yo)
    for o, e in zip((out.Ex, out.Ey, out.Ez), exp):
        assert rel_l2(_np(o), e) < TOL


def test_high_na_lens_odd_grid_keeps_the_reference_nan(xl):
    """optical_elements.py:538 divides by rho: on an odd grid the centre pixel
    (rho = 0) is NaN in every component, in the reference and here; every
    other pixel matches the oracle."""
    wo, vo, oe = xl
    n = 33
    x, y = ref.space(500.0, n)
    rng = np.random.default_rng(33)
    Ex = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    Ey = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    light = vo.VectorizedLight(x, y, 0.65)
    light.Ex, light.Ey = Ex.astype(np.complex64), Ey.astype(np.complex64)
    E, _ = oe.high_NA_objective_lens(light, 400.0, 400.0 / 0.9)
    got = _np(E)
    want = np.asarray(ref.high_na_lens(Ex.astype(np.complex64).astype(np.complex128),
                                       Ey.astype(np.complex64).astype(np.complex128), x, y, 400.0, 400.0 / 0.9)[0])
    assert np.array_equal(np.isnan(got), np.isnan(want))
    assert np.isnan(got[:, n // 2, n // 2]).all() and np.isnan(got).sum() == 3
    ok = ~np.isnan(want)
    assert rel_l2(got[ok], want[ok]) < 1e-6


def test_ez_only_focus_matches_the_full_focus_and_its_gradients():
    """VCZT_objective_lens_ez (the lens's Ez row, one transformed component)
    gives the full focus's Ez, and the same gradients of an Ez loss with
    respect to the fields and the mask parameters in front of the lens."""
    import torch

    import xlumina_gb300.optical_elements as oe
    import xlumina_gb300.vectorized_optics as vo
    n, m = 192, 64
    x, y = ref.space(1500.0, n)
    xo, yo = ref.space(2.0, m)
    rng = np.random.default_rng(88)
    Ex0 = (ref.gaussian_beam(x, y, 0.65, (800.0, 800.0)) * np.exp(1j * rng.uniform(0, 1, (n, n))))
    res = []
    for ez_only in (False, True):
        light = vo.VectorizedLight(x, y, 0.65)
        ex = torch.as_tensor(Ex0.astype(np.complex64), device="cuda").requires_grad_(True)
        light.Ex, light.Ey = ex, 0.3 * ex.detach()
        a = torch.as_tensor(rng.uniform(0, 2 * np.pi, (n, n)).astype(np.float32), device="cuda")
        a = a if not res else res[0][3].detach().clone()
        a.requires_grad_(True)
        eta = torch.full((n, n), 0.7, device="cuda", requires_grad=True)
        lit = oe.sSLM(oe.LCD(light, eta, 0.4), a, a)
        ez = (oe.VCZT_objective_lens_ez(lit, 1800.0, 2000.0, xo, yo) if ez_only
              else oe.VCZT_objective_lens(lit, 1800.0, 2000.0, xo, yo).Ez)
        w = torch.as_tensor(rng.uniform(0, 1, (m, m)).astype(np.float32), device="cuda") if not res else res[0][4]
        (w * torch.abs(ez) ** 2).sum().backward()
        res.append((ez.detach(), ex.grad, eta.grad, a, w, a.grad))
    (e0, gx0, ge0, _, _, ga0), (e1, gx1, ge1, _, _, ga1) = res
    assert rel_l2(_np(e1), _np(e0)) < 1e-6
    for g1, g0 in ((gx1, gx0), (ge1, ge0), (ga1, ga0)):
        assert rel_l2(g1.cpu().numpy(), g0.cpu().numpy()) < 1e-5
