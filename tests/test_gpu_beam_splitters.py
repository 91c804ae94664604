"""Beam splitters (optical_elements.py:334-512) on the GPU: forward against the
golden fixtures made by the reference's own source, gradients against torch
autograd through the complex128 oracle.  Bars: fields rel-L2 1e-6 (complex64
storage of float64 values); gradients rel 1e-4."""
import numpy as np
import pytest

from oracle import xlumina_ref as ref
from tests.conftest import golden, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    import torch

    import xlumina_gb300.optical_elements as oe
    import xlumina_gb300.vectorized_optics as vo
    return torch, oe, vo


def _light(vo, torch, x, y, wl, ex, ey):
    light = vo.VectorizedLight(x, y, wl)
    light.Ex = torch.as_tensor(np.asarray(ex).astype(np.complex64), device="cuda")
    light.Ey = torch.as_tensor(np.asarray(ey).astype(np.complex64), device="cuda")
    return light


def test_beam_splitters_match_golden(mods):
    torch, oe, vo = mods
    g = golden("beam_splitters")
    x, y, wl = g["x"], g["y"], float(g["wavelength"])
    la = _light(vo, torch, x, y, wl, g["aEx"], g["aEy"])
    lb = _light(vo, torch, x, y, wl, g["bEx"], g["bEy"])

    def check(c, d, keys):
        for comp, key in zip((c.Ex, c.Ey, d.Ex, d.Ey), keys):
            assert rel_l2(comp.cpu().numpy(), g[key]) < 1e-6, key
        assert not torch.any(c.Ez) and not torch.any(d.Ez)

    check(*oe.BS_symmetric(la, lb, float(g["theta"])), ("cEx", "cEy", "dEx", "dEy"))
    check(*oe.BS_symmetric_SI(la, float(g["theta"]), port=0), ("si0_cEx", "si0_cEy", "si0_dEx", "si0_dEy"))
    check(*oe.BS_symmetric_SI(la, float(g["theta_si1"]), port=1), ("si1_cEx", "si1_cEy", "si1_dEx", "si1_dEy"))
    check(*oe.BS(la, lb, float(g["R"]), float(g["T"]), float(g["phase"])), ("b1Ex", "b1Ey", "b2Ex", "b2Ey"))
    # a tensor angle gives the same fields
    th = torch.tensor(float(g["theta"]), device="cuda")
    check(*oe.BS_symmetric(la, lb, th), ("cEx", "cEy", "dEx", "dEy"))
    fl = oe.vectorized_fluorophores(torch.as_tensor(g["i_ex"], device="cuda"),
                                    torch.as_tensor(g["i_dep"], device="cuda"))
    assert rel_l2(fl.cpu().numpy(), g["vfluorophores"]) < 1e-12


def test_splitter_angle_and_field_gradients(mods):
    """LCD(a) and b mixed by BS_symmetric(theta), then VRS of both outputs; the
    gradients of theta, the LCD retardance and b's Ex against the oracle."""
    torch, oe, vo = mods
    from oracle import torch_ref as tr
    n, wl = 48, 0.65
    x, y = ref.space(150.0, n)
    rng = np.random.default_rng(21)

    def rnd():
        return ((rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * 0.2).astype(np.complex64)

    aEx, aEy, bEx, bEy = rnd(), rnd(), rnd(), rnd()
    eta = rng.uniform(0, 2 * np.pi, (n, n)).astype(np.float32)
    w = [rng.uniform(0, 1, (n, n)) for _ in range(6)]
    th0 = 0.9
    la = _light(vo, torch, x, y, wl, aEx, aEy)
    lb = vo.VectorizedLight(x, y, wl)
    bx = torch.as_tensor(bEx, device="cuda").requires_grad_(True)
    lb.Ex, lb.Ey = bx, torch.as_tensor(bEy, device="cuda")
    pe = torch.as_tensor(eta, device="cuda").requires_grad_(True)
    th = torch.tensor(th0, dtype=torch.float32, device="cuda", requires_grad=True)
    c, d = oe.BS_symmetric(oe.LCD(la, pe, 0.4), lb, th)
    oc, _ = c.VRS_propagation(2000.0)
    od, _ = d.VRS_propagation(2600.0)
    comps = (oc.Ex, oc.Ey, oc.Ez, od.Ex, od.Ey, od.Ez)
    L = sum(torch.sum(torch.as_tensor(wi, device="cuda") * torch.abs(ci) ** 2) for wi, ci in zip(w, comps))
    L.backward()

    c128 = lambda a: torch.as_tensor(a.astype(np.complex128))
    per = torch.as_tensor(eta.astype(np.float64)).requires_grad_(True)
    bxr = c128(bEx).requires_grad_(True)
    thr = torch.tensor(float(np.float32(th0)), dtype=torch.float64, requires_grad=True)
    ax, ay = tr.lcd(c128(aEx), c128(aEy), per, 0.4)
    cx, cy, dx, dy = tr.bs_symmetric(ax, ay, bxr, c128(bEy), thr)
    outs = tr.vrs_propagate(cx, cy, x, y, wl, 2000.0) + tr.vrs_propagate(dx, dy, x, y, wl, 2600.0)
    Lr = sum(torch.sum(torch.as_tensor(wi) * torch.abs(ci) ** 2) for wi, ci in zip(w, outs))
    Lr.backward()
    assert L.item() == pytest.approx(Lr.item(), rel=1e-5)
    assert th.grad.item() == pytest.approx(thr.grad.item(), rel=1e-4)
    assert rel_l2(pe.grad.cpu().numpy(), per.grad.numpy()) < 1e-4
    assert rel_l2(bx.grad.cpu().numpy(), bxr.grad.numpy()) < 1e-4


def test_single_input_and_batched_angles(mods):
    """BS_symmetric_SI on both ports with a tensor angle, and a batch of fields
    mixed with one shared input plane at one angle per batch entry."""
    torch, oe, vo = mods
    from oracle import torch_ref as tr
    n, wl, B = 40, 0.6, 3
    x, y = ref.space(100.0, n)
    rng = np.random.default_rng(22)

    def rnd(*s):
        return ((rng.standard_normal(s) + 1j * rng.standard_normal(s)) * 0.3).astype(np.complex64)

    aEx, aEy = rnd(n, n), rnd(n, n)
    w = rng.uniform(0, 1, (n, n))
    for port in (0, 1):
        th = torch.tensor(-1.3, dtype=torch.float32, device="cuda", requires_grad=True)
        c, d = oe.BS_symmetric_SI(_light(vo, torch, x, y, wl, aEx, aEy), th, port=port)
        L = torch.sum(torch.as_tensor(w, device="cuda") * (torch.abs(c.Ex) ** 2 + 2 * torch.abs(d.Ey) ** 2))
        L.backward()
        thr = torch.tensor(float(np.float32(-1.3)), dtype=torch.float64, requires_grad=True)
        cx, cy, dx, dy = tr.bs_symmetric_si(torch.as_tensor(aEx.astype(np.complex128)),
                                            torch.as_tensor(aEy.astype(np.complex128)), thr, port)
        Lr = torch.sum(torch.as_tensor(w) * (torch.abs(cx) ** 2 + 2 * torch.abs(dy) ** 2))
        Lr.backward()
        assert th.grad.item() == pytest.approx(thr.grad.item(), rel=1e-5)

    bEx, bEy = rnd(B, n, n), rnd(B, n, n)
    ths = np.array([0.2, 1.0, 2.5], dtype=np.float32)
    th = torch.tensor(ths, device="cuda", requires_grad=True)
    la = _light(vo, torch, x, y, wl, aEx, aEy)
    lb = _light(vo, torch, x, y, wl, bEx, bEy)
    c, d = oe.BS_symmetric(la, lb, th)
    assert c.Ex.shape == (B, n, n)
    L = torch.sum(torch.as_tensor(w, device="cuda") * (torch.abs(c.Ey) ** 2 + torch.abs(d.Ex) ** 2))
    L.backward()
    for b in range(B):
        want = ref.bs_symmetric(aEx, aEy, bEx[b], bEy[b], float(ths[b]))
        for got, wv in zip((c.Ex[b], c.Ey[b], d.Ex[b], d.Ey[b]), want):
            assert rel_l2(got.detach().cpu().numpy(), wv) < 1e-6
        thr = torch.tensor(float(ths[b]), dtype=torch.float64, requires_grad=True)
        cx, cy, dx, dy = tr.bs_symmetric(*(torch.as_tensor(a.astype(np.complex128)) for a in (aEx, aEy, bEx[b], bEy[b])),
                                         thr)
        Lr = torch.sum(torch.as_tensor(w) * (torch.abs(cy) ** 2 + torch.abs(dx) ** 2))
        Lr.backward()
        assert th.grad[b].item() == pytest.approx(thr.grad.item(), rel=1e-4)
