"""Pin the FP64 oracle to the golden fixtures produced by the reference's own source.

These run on CPU only.  The bar is rounding-level agreement (rel-L2 <= 1e-10):
both sides compute in float64 / complex128 with the same formulas and layouts.
"""
import numpy as np
import pytest

from oracle import xlumina_ref as ref
from tests.conftest import golden, rel_l2

TOL = 1e-10


def test_rs_square_both_signs_of_z():
    g = golden("rs_square")
    field = ref.slm(ref.gaussian_beam(g["x"], g["y"], g["wavelength"], (40.0, 40.0)), g["phase"])[0]
    assert rel_l2(field, g["field_in"]) < 1e-13
    for tag in ("pos", "neg"):
        out = ref.rs_propagate(g["field_in"], g["x"], g["y"], g["wavelength"], float(g[f"z_{tag}"]))
        assert rel_l2(out, g[f"out_{tag}"]) < TOL
        qf = ref.rs_quality_factor(g["x"], g["y"], g["wavelength"], float(g[f"z_{tag}"]))
        assert qf == pytest.approx(float(g[f"qf_{tag}"]), rel=1e-12)


@pytest.mark.parametrize("case", ["rs_complex", "rs_odd"])
def test_rs_random_fields(case):
    g = golden(case)
    out = ref.rs_propagate(g["field_in"], g["x"], g["y"], g["wavelength"], float(g["z"]))
    assert rel_l2(out, g["out"]) < TOL


def test_vrs_behind_lcd_and_polarizer():
    g = golden("vrs")
    Ex0, Ey0 = ref.polarized_gaussian_beam(g["x"], g["y"], g["wavelength"], (50.0, 50.0), (1, 0.5))
    assert rel_l2(Ex0, g["Ex0"]) < 1e-13 and rel_l2(Ey0, g["Ey0"]) < 1e-13
    Ex1, Ey1 = ref.lcd(g["Ex0"], g["Ey0"], g["eta"], g["theta"])
    assert rel_l2(Ex1, g["lcd_Ex"]) < 1e-13 and rel_l2(Ey1, g["lcd_Ey"]) < 1e-13
    Ex2, Ey2 = ref.linear_polarizer(Ex1, Ey1, g["alpha"])
    assert rel_l2(Ex2, g["lp_Ex"]) < 1e-13 and rel_l2(Ey2, g["lp_Ey"]) < 1e-13
    assert np.all(g["lp_Ez"] == 0)
    out = ref.vrs_propagate(g["lp_Ex"], g["lp_Ey"], g["x"], g["y"], g["wavelength"], float(g["z"]))
    for o, key in zip(out, ("Ex", "Ey", "Ez")):
        assert rel_l2(o, g[key]) < TOL


def test_czt_default_and_roi():
    g = golden("czt")
    out = ref.czt(g["field_in"], g["x"], g["y"], g["wavelength"], float(g["z"]))
    assert rel_l2(out, g["out_default"]) < TOL
    out = ref.czt(g["field_in"], g["x"], g["y"], g["wavelength"], float(g["z"]), g["xout"], g["yout"])
    assert out.shape == (len(g["yout"]), len(g["xout"]))
    assert rel_l2(out, g["out_roi"]) < TOL


def test_vczt():
    g = golden("vczt")
    out = ref.vczt(g["Ex_in"], g["Ey_in"], g["x"], g["y"], g["wavelength"], float(g["z"]), g["xout"], g["yout"])
    for o, key in zip(out, ("Ex", "Ey", "Ez")):
        assert rel_l2(o, g[key]) < TOL


def test_high_na_lens_and_focus():
    g = golden("high_na")
    E, s = ref.high_na_lens(g["Ex_in"], g["Ey_in"], g["x"], g["y"], float(g["radius"]), float(g["f"]))
    assert s == pytest.approx(float(g["sin_theta_max"]), rel=1e-14)
    assert rel_l2(E, g["lens_out"]) < 1e-13
    out = ref.vczt_objective_lens(g["Ex_in"], g["Ey_in"], g["x"], g["y"], g["wavelength"],
                                  float(g["radius"]), float(g["f"]), g["xout"], g["yout"])
    for o, key in zip(out, ("Ex", "Ey", "Ez")):
        assert rel_l2(o, g[key]) < TOL


def test_masks_and_sources():
    g = golden("masks")
    x, y, wl = g["x"], g["y"], g["wavelength"]
    gb = ref.gaussian_beam(x, y, wl, (40.0, 55.0), 1.5, (10.0, -5.0), (300.0, 200.0), 0.3)
    assert rel_l2(gb, g["gauss"]) < 1e-13
    assert rel_l2(ref.plane_wave(x, y, wl, 2.0, 0.01, 0.7, 3.0), g["plane"]) < 1e-13
    Ex, Ey = ref.polarized_gaussian_beam(x, y, wl, (40.0, 40.0), (1, 1j), (3.0, 4.0))
    assert rel_l2(Ex, g["pol_Ex"]) < 1e-13 and rel_l2(Ey, g["pol_Ey"]) < 1e-13
    ox, oy = ref.sslm(g["pol_Ex"], g["pol_Ey"], g["alpha"], g["phi"])
    assert rel_l2(ox, g["sslm_Ex"]) < 1e-13 and rel_l2(oy, g["sslm_Ey"]) < 1e-13
    ox, oy = ref.sslm(g["pol_Ex"], g["pol_Ey"], g["alpha"], g["phi"], g["A1"], g["A2"])
    assert rel_l2(ox, g["sslma_Ex"]) < 1e-13 and rel_l2(oy, g["sslma_Ey"]) < 1e-13
    m = ref.lens_mask(x, y, wl, (120.0, 100.0), (2000.0, 2500.0))
    assert rel_l2(m, g["lens_mask"]) < 1e-13
    assert rel_l2(g["gauss"] * m, g["lens_scalar"]) < 1e-13
    mv = ref.lens_mask(x, y, wl, (120.0, 120.0), (3000.0, 3000.0))
    assert rel_l2(g["pol_Ex"] * mv, g["lens_vec_Ex"]) < 1e-13
    assert np.all(g["lens_vec_Ez"] == 0)
    lx, ly = ref.lcd(g["pol_Ex"], g["pol_Ey"], 1.1, 0.4)
    assert rel_l2(lx, g["lcd_scalar_Ex"]) < 1e-13 and rel_l2(ly, g["lcd_scalar_Ey"]) < 1e-13
    assert np.array_equal(g["lcd_scalar_Ez"], g["vin_Ez"])


def test_losses():
    g = golden("losses")
    assert ref.mse_intensity(g["a"], g["b"]) == pytest.approx(float(g["mse_intensity"]), rel=1e-13)
    assert ref.small_area_hybrid(g["I"]) == pytest.approx(float(g["small_area"]), rel=1e-13)


def test_building_block_chain():
    g = golden("building_block")
    Ex, Ey = ref.sslm(g["Ex_in"], g["Ey_in"], g["alpha"], g["phi"])
    Ex, Ey, Ez = ref.vrs_propagate(Ex, Ey, g["x"], g["y"], g["wavelength"], float(g["z"]))
    Ex, Ey = ref.lcd(Ex, Ey, float(g["eta"]), float(g["theta"]))
    for o, key in zip((Ex, Ey, Ez), ("Ex", "Ey", "Ez")):
        assert rel_l2(o, g[key]) < TOL


def test_four_f_chain():
    g = golden("four_f")
    x, y, wl, f = g["x"], g["y"], g["wavelength"], float(g["f"])
    u = ref.slm(g["source"], g["phase1"])[0]
    u = ref.rs_propagate(u, x, y, wl, f)
    assert rel_l2(u, g["after_rs"]) < TOL
    u = u * ref.lens_mask(x, y, wl, (200.0, 200.0), (f, f))
    assert rel_l2(u, g["after_lens"]) < TOL
    u = ref.czt(u, x, y, wl, f, g["xout"], g["yout"])
    assert rel_l2(u, g["after_czt1"]) < TOL
    u = ref.slm(u, g["phase2"])[0]
    u = ref.czt(u, g["xout"], g["yout"], wl, f)
    assert rel_l2(u, g["out"]) < TOL


# ---- the torch restatement (gradient oracle) is pinned to the numpy oracle ----

def test_torch_restatement_matches_numpy_oracle():
    import torch
    from oracle import torch_ref as tr
    g = golden("four_f")
    x, y, wl, f = g["x"], g["y"], g["wavelength"], float(g["f"])
    u = tr.slm(torch.as_tensor(g["source"]), torch.as_tensor(g["phase1"]))
    u = tr.rs_propagate(u, x, y, wl, f)
    assert rel_l2(u.numpy(), g["after_rs"]) < TOL
    u = tr.lens(u, x, y, wl, (200.0, 200.0), (f, f))
    u = tr.czt(u, x, y, wl, f, g["xout"], g["yout"])
    assert rel_l2(u.numpy(), g["after_czt1"]) < TOL
    h = golden("high_na")
    out = tr.vczt_objective_lens(torch.as_tensor(h["Ex_in"]), torch.as_tensor(h["Ey_in"]), h["x"], h["y"],
                                 h["wavelength"], float(h["radius"]), float(h["f"]), h["xout"], h["yout"])
    for o, key in zip(out, ("Ex", "Ey", "Ez")):
        assert rel_l2(o.numpy(), h[key]) < TOL
    v = golden("vrs")
    Ex, Ey = tr.lcd(torch.as_tensor(v["Ex0"]), torch.as_tensor(v["Ey0"]), v["eta"], v["theta"])
    Ex, Ey = tr.linear_polarizer(Ex, Ey, v["alpha"])
    out = tr.vrs_propagate(Ex, Ey, v["x"], v["y"], v["wavelength"], float(v["z"]))
    for o, key in zip(out, ("Ex", "Ey", "Ez")):
        assert rel_l2(o.numpy(), v[key]) < TOL


def test_torch_restatement_gradients_match_finite_differences():
    """Central differences in float64 on a few mask parameters of a 4f-style chain."""
    import torch
    from oracle import torch_ref as tr
    n = 24
    x, y = ref.space(120.0, n)
    rng = np.random.default_rng(11)
    src = torch.as_tensor(ref.gaussian_beam(x, y, 0.6, (50.0, 50.0)))
    w = torch.as_tensor(rng.uniform(0, 1, (16, 16)))
    xo, yo = ref.space(40.0, 16)

    def loss(ph, eta):
        u = tr.slm(src, ph)
        u = tr.rs_propagate(u, x, y, 0.6, 3000.0)
        ex, ey = tr.lcd(u, 0.3 * u, eta, 0.7)
        u = tr.czt(ex + ey, x, y, 0.6, 3000.0, xo, yo)
        return torch.sum(w * torch.abs(u) ** 2)

    ph = torch.as_tensor(rng.uniform(-np.pi, np.pi, (n, n)), dtype=torch.float64).requires_grad_(True)
    eta = torch.as_tensor(rng.uniform(0, 2 * np.pi, (n, n)), dtype=torch.float64).requires_grad_(True)
    L = loss(ph, eta)
    L.backward()
    h = 1e-6
    for (i, j) in [(3, 4), (12, 12), (20, 7)]:
        for t, gt in ((ph, ph.grad), (eta, eta.grad)):
            with torch.no_grad():
                t[i, j] += h
                lp = loss(ph, eta).item()
                t[i, j] -= 2 * h
                lm = loss(ph, eta).item()
                t[i, j] += h
            fd = (lp - lm) / (2 * h)
            assert abs(fd - gt[i, j].item()) <= 1e-6 * max(1.0, abs(fd)) + 1e-9 * abs(L.item())


def test_beam_splitters_and_fluorescence():
    g = golden("beam_splitters")
    a, b = (g["aEx"], g["aEy"]), (g["bEx"], g["bEy"])
    out = ref.bs_symmetric(*a, *b, float(g["theta"]))
    for got, key in zip(out, ("cEx", "cEy", "dEx", "dEy")):
        assert rel_l2(got, g[key]) < 1e-14
    assert not np.any(g["cEz"]) and not np.any(g["dEz"])
    for port, th in ((0, float(g["theta"])), (1, float(g["theta_si1"]))):
        out = ref.bs_symmetric_si(*a, th, port)
        for got, key in zip(out, ("cEx", "cEy", "dEx", "dEy")):
            assert rel_l2(got, g[f"si{port}_{key}"]) < 1e-14
    out = ref.bs_lossless(*a, *b, float(g["R"]), float(g["T"]), float(g["phase"]))
    for got, key in zip(out, ("b1Ex", "b1Ey", "b2Ex", "b2Ey")):
        assert rel_l2(got, g[key]) < 1e-14
    fl = ref.fluorescence(g["i_ex"][0], g["i_dep"][0], float(g["beta"]))
    assert rel_l2(fl, g["fluorescence"]) < 1e-14
    assert rel_l2(ref.fluorescence(g["i_ex"], g["i_dep"]), g["vfluorophores"]) < 1e-14


def test_torch_restatement_of_the_sharp_focus_table():
    """The step-by-step complex128 restatement of hybrid_setup_sharp_focus (the
    table's gradient oracle) against the reference's own output."""
    import torch

    from oracle import torch_ref as tr
    g = golden("hybrid_tables")
    src = (torch.as_tensor(g["red_Ex"]), torch.as_tensor(g["red_Ey"]))
    params = [g[f"p_sharp_{k}"] for k in range(29)]
    I = tr.hybrid_setup_sharp_focus(src, g["x"], g["y"], 0.65, params, float(g["r"]), float(g["f"]), g["xout"],
                                    g["yout"])
    assert rel_l2(I.numpy(), g["i_sharp"]) < 1e-9   # 16 chained propagations of rounding
