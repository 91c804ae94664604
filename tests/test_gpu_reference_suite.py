"""The reference's own test cases (tests/test_optical_elements.py,
tests/test_wave_optics.py, tests/test_vectorized_optics.py,
tests/test_toolbox.py), restated against this package: shapes, the mask
identities (SLM with zero phase, sSLM with 0 and pi, LCD(0, 0), a polarizer
aligned with and crossed to the input), the splitter formula at theta = 0,
and the toolbox helpers on the propagation path.  Same inputs as the
reference's setUp (512 or 1024 pixels over +-1500 um, 633 nm)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    import torch

    import xlumina_gb300.optical_elements as oe
    import xlumina_gb300.toolbox as tb
    import xlumina_gb300.vectorized_optics as vo
    import xlumina_gb300.wave_optics as wo
    return torch, oe, tb, vo, wo


N_OE, N_PROP = 512, 1024
WL = 0.633


def _grid(n):
    return np.linspace(-1500, 1500, n), np.linspace(-1500, 1500, n)


def _close(torch, a, b, tol=1e-6):
    a, b = torch.as_tensor(a).cpu(), torch.as_tensor(b).cpu()
    return torch.allclose(a.to(torch.complex128), b.to(torch.complex128), atol=tol, rtol=tol)


def test_slm_zero_phase_and_jones_shapes(mods):
    torch, oe, tb, vo, wo = mods
    x, y = _grid(N_OE)
    light = wo.LightSource(x, y, WL)
    light.gaussian_beam(w0=(1200, 1200), E0=1)
    out, _ = oe.SLM(light, np.zeros((N_OE, N_OE)), N_OE)
    assert out.field.shape == (N_OE, N_OE) and _close(torch, out.field, light.field)
    for m in (oe.jones_LP(np.pi / 4), oe.jones_general_retarder(np.pi / 2, np.pi / 4, 0),
              oe.jones_sSLM(np.pi / 2, np.pi / 4), oe.jones_LCD(np.pi / 2, np.pi / 4)):
        assert tuple(m.shape) == (2, 2)


def test_polarization_device_identities(mods):
    torch, oe, tb, vo, wo = mods
    x, y = _grid(N_OE)
    light = vo.PolarizedLightSource(x, y, WL)
    light.gaussian_beam(w0=(1200, 1200), jones_vector=(1, 1))
    zeros = np.zeros((N_OE, N_OE))
    s0 = oe.sSLM(light, zeros, zeros)
    assert s0.Ex.shape == s0.Ey.shape == s0.Ez.shape == (N_OE, N_OE)
    assert _close(torch, s0.Ex, light.Ex) and _close(torch, s0.Ey, light.Ey) and _close(torch, s0.Ez, light.Ez)
    pi = np.pi * np.ones((N_OE, N_OE))
    sp = oe.sSLM(light, pi, pi)
    assert _close(torch, sp.Ex, -light.Ex) and _close(torch, sp.Ey, -light.Ey) and _close(torch, sp.Ez, light.Ez)

    light = vo.PolarizedLightSource(x, y, WL)
    light.gaussian_beam(w0=(1200, 1200), jones_vector=(1, 0))
    lcd = oe.LCD(light, 0, 0)
    assert _close(torch, lcd.Ex, light.Ex) and _close(torch, lcd.Ey, light.Ey) and _close(torch, lcd.Ez, light.Ez)
    aligned = oe.linear_polarizer(light, zeros)
    assert _close(torch, aligned.Ex, light.Ex) and _close(torch, aligned.Ey, light.Ey)
    assert _close(torch, aligned.Ez, light.Ez)
    crossed = oe.linear_polarizer(light, np.pi / 2 * np.ones((N_OE, N_OE)))
    assert _close(torch, crossed.Ex, zeros) and _close(torch, crossed.Ey, zeros)


def test_beam_splitter_fully_transmissive(mods):
    torch, oe, tb, vo, wo = mods
    x, y = _grid(N_OE)
    l1 = vo.PolarizedLightSource(x, y, WL)
    l1.gaussian_beam(w0=(1200, 1200), jones_vector=(1, 0))
    l2 = vo.PolarizedLightSource(x, y, WL)
    l2.gaussian_beam(w0=(1200, 1200), jones_vector=(1, 0))
    c, d = oe.BS_symmetric(l1, l2, 0)
    T, R, noise = 1.0, 0.0, 0.01
    assert _close(torch, c.Ex, (T - noise) * 1j * l2.Ex + (R - noise) * l1.Ex)
    assert _close(torch, c.Ey, (T - noise) * 1j * l2.Ey + (R - noise) * l1.Ey)
    assert _close(torch, d.Ex, (T - noise) * 1j * l1.Ex + (R - noise) * l2.Ex)
    assert _close(torch, d.Ey, (T - noise) * 1j * l1.Ey + (R - noise) * l2.Ey)


def test_objective_lens_lenses_and_building_block_shapes(mods):
    torch, oe, tb, vo, wo = mods
    x, y = _grid(N_OE)
    r = 3.6e3 / 2
    light = vo.PolarizedLightSource(x, y, WL)
    light.gaussian_beam(w0=(1200, 1200), jones_vector=(1, 0))
    out, _ = oe.high_NA_objective_lens(light, r, r / 0.9)
    assert tuple(out.shape) == (3, N_OE, N_OE)
    foc = oe.VCZT_objective_lens(light, r, r / 0.9, x, y)
    assert foc.Ex.shape == foc.Ey.shape == foc.Ez.shape == (N_OE, N_OE)
    s = wo.LightSource(x, y, WL)
    s.gaussian_beam(w0=(1200, 1200), E0=1)
    for lo in (oe.lens(s, (50, 50), (1000, 1000))[0], oe.cylindrical_lens(s, 1000)[0], oe.axicon_lens(s, 0.1)[0]):
        assert lo.field.shape == (N_OE, N_OE)
    v = vo.VectorizedLight(x, y, WL)
    v.Ex, v.Ey, v.Ez = light.Ex, light.Ey, light.Ez
    for lo in (oe.lens(v, (50, 50), (1000, 1000))[0], oe.cylindrical_lens(v, 1000)[0], oe.axicon_lens(v, 0.1)[0]):
        assert lo.Ex.shape == lo.Ey.shape == (N_OE, N_OE)
    bb = oe.building_block(light, np.zeros((N_OE, N_OE)), np.zeros((N_OE, N_OE)), 1000, np.pi / 2, np.pi / 4)
    assert bb.Ex.shape == bb.Ey.shape == bb.Ez.shape == (N_OE, N_OE)


def test_lights_sources_and_propagators(mods):
    torch, oe, tb, vo, wo = mods
    x, y = _grid(N_PROP)
    sl = wo.ScalarLight(x, y, WL)
    assert sl.wavelength == WL and sl.k == 2 * np.pi / WL and sl.field.shape == (N_PROP, N_PROP)
    src = wo.LightSource(x, y, WL)
    src.gaussian_beam(w0=(1200, 1200), E0=1)
    assert torch.sum(torch.abs(src.field) ** 2) > 0
    pw = wo.LightSource(x, y, WL)
    pw.plane_wave(A=1, theta=0, phi=0, z0=0)
    assert torch.sum(torch.abs(pw.field) ** 2) > 0
    assert src.RS_propagation(z=1000)[0].field.shape == (N_PROP, N_PROP)
    assert src.CZT(z=1000).field.shape == (N_PROP, N_PROP)

    vl = vo.VectorizedLight(x, y, WL)
    assert vl.Ex.shape == vl.Ey.shape == vl.Ez.shape == (N_PROP, N_PROP)
    for jv, ex_on, ey_on in (((1, 0), True, False), ((0, 1), False, True), ((1, 1), True, True)):
        s = vo.PolarizedLightSource(x, y, WL)
        s.gaussian_beam(w0=(1200, 1200), jones_vector=jv)
        assert (torch.sum(torch.abs(s.Ex) ** 2) > 0) == ex_on
        assert (torch.sum(torch.abs(s.Ey) ** 2) > 0) == ey_on
    s = vo.PolarizedLightSource(x, y, WL)
    s.gaussian_beam(w0=(1200, 1200), jones_vector=(1, 1))
    p, _ = s.VRS_propagation(z=1000)
    assert p.Ex.shape == p.Ey.shape == p.Ez.shape == (N_PROP, N_PROP)
    c = s.VCZT(1000, x, y)
    assert c.Ex.shape == c.Ey.shape == c.Ez.shape == (N_PROP, N_PROP)


def test_toolbox_helpers(mods):
    torch, oe, tb, vo, wo = mods
    x, y = _grid(N_OE)
    xs, ys = tb.space(1500, N_OE)
    assert np.allclose(xs, x) and np.allclose(ys, y)
    w = tb.wrap_phase(np.array([0, np.pi, 2 * np.pi, 3 * np.pi, -3 * np.pi]))
    assert np.allclose(w, [0, np.pi, 0, np.pi, -np.pi])
    l1 = vo.VectorizedLight(x, y, WL)
    l2 = vo.VectorizedLight(x, y, WL)
    l1.Ex = np.ones((N_OE, N_OE))
    l2.Ex = np.ones((N_OE, N_OE))
    assert abs(float(tb.is_conserving_energy(l1, l2)) - 1.0) < 1e-6
    l2.Ex = 0 * l2.Ex
    assert float(tb.is_conserving_energy(l1, l2)) == 0
    assert float(tb.softmin(np.array([1.0, 2.0, 3.0]))) == 1.0
    assert tb.delta_kronecker(1, 1) == 1 and tb.delta_kronecker(1, 2) == 0
    eta, theta = tb.build_LCD_cell(np.pi / 2, np.pi / 4, N_OE)
    assert np.allclose(eta, np.pi / 2) and np.allclose(theta, np.pi / 4)
    X, Y = np.meshgrid(x, y)
    Xr, Yr = tb.rotate_mask(X, Y, np.pi / 4)
    assert Xr.shape == Yr.shape == (N_OE, N_OE)
