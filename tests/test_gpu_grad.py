"""Hand-written adjoints on the GPU against autograd through the complex128
torch restatement of the reference (the gradient oracle, itself checked against
finite differences).  Bar: gradients agree within rel-L2 1e-4; loss values
within 1e-5."""
import numpy as np
import pytest

from oracle import xlumina_ref as ref
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu
GTOL = 1e-4


@pytest.fixture(scope="module")
def mods():
    import torch
    from oracle import torch_ref as tr

    import xlumina_gb300.loss_functions as lf
    import xlumina_gb300.optical_elements as oe
    import xlumina_gb300.vectorized_optics as vo
    import xlumina_gb300.wave_optics as wo
    return torch, tr, wo, vo, oe, lf


def _param(torch, a, dev):
    return torch.as_tensor(np.asarray(a, dtype=np.float32), device=dev).requires_grad_(True)


def _ref_param(torch, a):
    return torch.as_tensor(np.asarray(a, dtype=np.float32).astype(np.float64)).requires_grad_(True)


def test_rs_slm_phase_gradient(mods):
    torch, tr, wo, vo, oe, lf = mods
    n = 96
    x, y = ref.space(300.0, n)
    rng = np.random.default_rng(1)
    ph = rng.uniform(-np.pi, np.pi, (n, n))
    w = rng.uniform(0, 1, (n, n))
    src = wo.LightSource(x, y, 0.633)
    src.gaussian_beam(w0=(120.0, 120.0), E0=1)
    p = _param(torch, ph, "cuda")
    out, _ = oe.SLM(src, p, n)[0].RS_propagation(4000.0)
    L = torch.sum(torch.as_tensor(w, device="cuda") * torch.abs(out.field) ** 2)
    L.backward()
    pr = _ref_param(torch, ph)
    s = torch.as_tensor(ref.gaussian_beam(x, y, 0.633, (120.0, 120.0)))
    Lr = torch.sum(torch.as_tensor(w) * torch.abs(tr.rs_propagate(tr.slm(s, pr), x, y, 0.633, 4000.0)) ** 2)
    Lr.backward()
    assert L.item() == pytest.approx(Lr.item(), rel=1e-5)
    assert rel_l2(p.grad.cpu().numpy(), pr.grad.numpy()) < GTOL


def test_vrs_lcd_polarizer_gradients(mods):
    torch, tr, wo, vo, oe, lf = mods
    n = 64
    x, y = ref.space(200.0, n)
    rng = np.random.default_rng(2)
    eta, theta = rng.uniform(0, 2 * np.pi, (n, n)), rng.uniform(0, 2 * np.pi, (n, n))
    alpha = np.full((n, n), 0.6)
    Ex0, Ey0 = ref.polarized_gaussian_beam(x, y, 0.633, (70.0, 70.0), (1, 0.4))
    Ex0 = Ex0 * np.exp(1j * rng.uniform(0, 1, (n, n)))
    wts = [rng.uniform(0, 1, (n, n)) for _ in range(3)]
    light = vo.VectorizedLight(x, y, 0.633)
    ex = torch.as_tensor(Ex0.astype(np.complex64), device="cuda").requires_grad_(True)
    light.Ex, light.Ey = ex, Ey0
    pe, pt, pa = _param(torch, eta, "cuda"), _param(torch, theta, "cuda"), _param(torch, alpha, "cuda")
    out, _ = oe.linear_polarizer(oe.LCD(light, pe, pt), pa).VRS_propagation(3000.0)
    L = sum(torch.sum(torch.as_tensor(w, device="cuda") * torch.abs(c) ** 2) for w, c in zip(wts, (out.Ex, out.Ey, out.Ez)))
    L.backward()
    exr = torch.as_tensor(Ex0.astype(np.complex64).astype(np.complex128)).requires_grad_(True)
    per, ptr_, par = _ref_param(torch, eta), _ref_param(torch, theta), _ref_param(torch, alpha)
    a, b = tr.lcd(exr, torch.as_tensor(Ey0), per, ptr_)
    a, b = tr.linear_polarizer(a, b, par)
    outr = tr.vrs_propagate(a, b, x, y, 0.633, 3000.0)
    Lr = sum(torch.sum(torch.as_tensor(w) * torch.abs(c) ** 2) for w, c in zip(wts, outr))
    Lr.backward()
    assert L.item() == pytest.approx(Lr.item(), rel=1e-5)
    for got, exp in ((pe, per), (pt, ptr_), (pa, par)):
        assert rel_l2(got.grad.cpu().numpy(), exp.grad.numpy()) < GTOL
    assert rel_l2(ex.grad.cpu().numpy(), exr.grad.numpy()) < GTOL


def test_four_f_batched_step_gradients(mods):
    """SLM1 -> RS(f) -> lens(f) -> CZT(ROI) -> SLM2 -> CZT, normalised-intensity MSE,
    two input masks sharing the SLM parameters."""
    torch, tr, wo, vo, oe, lf = mods
    n, m = 64, 32
    f = 6000.0
    x, y = ref.space(200.0, n)
    xo, yo = ref.space(60.0, m)
    rng = np.random.default_rng(3)
    p1, p2 = rng.uniform(-np.pi, np.pi, (n, n)), rng.uniform(-np.pi, np.pi, (m, m))
    masks = (rng.uniform(0, 1, (2, n, n)) > 0.3).astype(np.float64)
    target = (rng.uniform(0, 1, (2, m, m)) < 0.1).astype(np.float64)
    g = ref.gaussian_beam(x, y, 0.532, (80.0, 80.0))

    src = wo.ScalarLight(x, y, 0.532)
    src.field = torch.as_tensor((g[None] * masks).astype(np.complex64), device="cuda")
    q1, q2 = _param(torch, p1, "cuda"), _param(torch, p2, "cuda")
    l1, _ = oe.SLM(src, q1, n)
    l2, _ = l1.RS_propagation(f)
    l3, _ = oe.lens(l2, (200.0, 200.0), (f, f))
    l4 = l3.CZT(f, xo, yo)
    l5, _ = oe.SLM(l4, q2, m)
    I = torch.abs(l5.CZT(f).field) ** 2
    I = I / torch.sum(I, dim=(-2, -1), keepdim=True)
    T = torch.as_tensor(target / target.sum(axis=(-2, -1), keepdims=True), device="cuda", dtype=torch.float32)
    L = torch.mean(torch.sum((I - T) ** 2, dim=(-2, -1)) / (m * m))
    L.backward()

    r1, r2 = _ref_param(torch, p1), _ref_param(torch, p2)
    losses = []
    for bi in range(2):
        u = tr.slm(torch.as_tensor(g * masks[bi]), r1)
        u = tr.rs_propagate(u, x, y, 0.532, f)
        u = tr.lens(u, x, y, 0.532, (200.0, 200.0), (f, f))
        u = tr.czt(u, x, y, 0.532, f, xo, yo)
        u = tr.czt(tr.slm(u, r2), xo, yo, 0.532, f, xo, yo)
        Ir = torch.abs(u) ** 2
        Ir = Ir / torch.sum(Ir)
        Tr = torch.as_tensor(target[bi] / target[bi].sum())
        losses.append(torch.sum((Ir - Tr) ** 2) / (m * m))
    Lr = sum(losses) / 2
    Lr.backward()
    assert L.item() == pytest.approx(Lr.item(), rel=1e-4)
    assert rel_l2(q1.grad.cpu().numpy(), r1.grad.numpy()) < GTOL
    assert rel_l2(q2.grad.cpu().numpy(), r2.grad.numpy()) < GTOL


def test_high_na_focus_gradients(mods):
    """LCD + sSLM (per-pixel phases) -> VCZT objective lens -> Ez-weighted spot loss."""
    torch, tr, wo, vo, oe, lf = mods
    n, m = 64, 32
    x, y = ref.space(1500.0, n)
    f = 2000.0
    r = 0.9 * f
    xo, yo = ref.space(1.0, m)
    rng = np.random.default_rng(4)
    a, ph = rng.uniform(0, 2 * np.pi, (n, n)), rng.uniform(0, 2 * np.pi, (n, n))
    Ex0, Ey0 = ref.polarized_gaussian_beam(x, y, 0.65, (1200.0, 1200.0), (1, 0.2))
    light = vo.VectorizedLight(x, y, 0.65)
    light.Ex, light.Ey = Ex0, Ey0
    qa, qp = _param(torch, a, "cuda"), _param(torch, ph, "cuda")
    out = oe.VCZT_objective_lens(oe.sSLM(oe.LCD(light, 0.8, 0.3), qa, qp), r, f, xo, yo)
    I = torch.abs(out.Ez) ** 2 + 0.1 * torch.abs(out.Ex) ** 2
    L = lf.small_area_hybrid(I)
    L.backward()
    ra, rp = _ref_param(torch, a), _ref_param(torch, ph)
    ex, ey = tr.lcd(torch.as_tensor(Ex0), torch.as_tensor(Ey0), 0.8, 0.3)
    ex, ey = tr.sslm(ex, ey, ra, rp)
    o = tr.vczt_objective_lens(ex, ey, x, y, 0.65, r, f, xo, yo)
    Lr = tr.small_area_hybrid(torch.abs(o[2]) ** 2 + 0.1 * torch.abs(o[0]) ** 2)
    Lr.backward()
    assert L.item() == pytest.approx(Lr.item(), rel=1e-4)
    assert rel_l2(qa.grad.cpu().numpy(), ra.grad.numpy()) < GTOL
    assert rel_l2(qp.grad.cpu().numpy(), rp.grad.numpy()) < GTOL


def test_adjoint_dot_product_identity(mods):
    """<A u, v> = <u, A^H v> for RS, VRS and CZT adjoints (complex64, rel 1e-5)."""
    torch, tr, wo, vo, oe, lf = mods
    from xlumina_gb300 import engine
    n = 96
    x, y = ref.space(250.0, n)
    xo, yo = np.linspace(-80.0, 80.0, 40), np.linspace(-60.0, 60.0, 36)
    rng = np.random.default_rng(5)

    def rnd(*s):
        return torch.as_tensor((rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(np.complex64),
                               device="cuda")

    def dot(a, b):
        return complex(torch.sum(a.to(torch.complex128) * torch.conj(b.to(torch.complex128))).item())

    u, v = rnd(n, n), rnd(n, n)
    Au = engine.RsCall([u], x, y, 0.6, 3500.0, False).run()[0]
    Ahv = engine.RsCall([v], x, y, 0.6, 3500.0, False, adjoint=True).run()[0]
    assert abs(dot(Au, v) - dot(u, Ahv)) <= 1e-5 * abs(dot(Au, v))
    ux, uy = rnd(n, n), rnd(n, n)
    vs = [rnd(n, n) for _ in range(3)]
    Au = engine.RsCall([ux, uy], x, y, 0.6, 3500.0, True).run()
    Ahv = engine.RsCall(vs, x, y, 0.6, 3500.0, True, adjoint=True).run()
    lhs = sum(dot(a, b) for a, b in zip(Au, vs))
    rhs = dot(ux, Ahv[0]) + dot(uy, Ahv[1])
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)
    w = rnd(36, 40)
    Au = engine.CztCall([u], x, y, 0.6, 3500.0, xo, yo, "scalar").run()[0]
    Ahw = engine.CztCall([w], x, y, 0.6, 3500.0, xo, yo, "scalar", adjoint=True).run()[0]
    assert abs(dot(Au, w) - dot(u, Ahw)) <= 1e-5 * abs(dot(Au, w))
    ws = [rnd(36, 40) for _ in range(3)]
    Au = engine.CztCall([ux, uy], x, y, 0.6, 3500.0, xo, yo, "vczt").run()
    Ahw = engine.CztCall(ws, x, y, 0.6, 3500.0, xo, yo, "vczt", adjoint=True).run()
    lhs = sum(dot(a, b) for a, b in zip(Au, ws))
    rhs = dot(ux, Ahw[0]) + dot(uy, Ahw[1])
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_prebuilt_tables_step(mods):
    torch, tr, wo, vo, oe, lf = mods
    from xlumina_gb300.tables import FourFTable, HighNATable
    t4 = FourFTable(n=128, roi_n=64, batch=4, half_width=400.0, f=2.0e4, roi_half_width=150.0, waist=300.0)
    p0 = t4.phase1.detach().clone()
    l0 = t4.step().item()
    l1 = t4.step().item()
    assert np.isfinite(l0) and np.isfinite(l1)
    assert not torch.equal(p0, t4.phase1.detach())
    th = HighNATable(n=128, roi_n=64, batch=3, half_width=1500.0, f=2000.0, waist=1200.0)
    a0 = th.alpha.detach().clone()
    assert np.isfinite(th.step().item())
    assert not torch.equal(a0, th.alpha.detach())


def test_broadcast_batch_inputs_match_materialised(mods):
    torch, tr, wo, vo, oe, lf = mods
    from xlumina_gb300 import engine
    n = 128
    x, y = ref.space(300.0, n)
    rng = np.random.default_rng(8)
    e = torch.as_tensor((rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64),
                        device="cuda")
    a = torch.as_tensor(rng.uniform(0, 6, (3, n, n)).astype(np.float32), device="cuda")
    ops = [engine.op_sslm(a, a)]
    xo, yo = ref.space(100.0, 64)
    b1 = engine.rs_propagate([e.expand(3, n, n), e.expand(3, n, n)], x, y, 0.6, [1e4, 2e4, 3e4], True, pre=ops)
    b2 = engine.rs_propagate([e.expand(3, n, n).contiguous(), e.expand(3, n, n).contiguous()], x, y, 0.6,
                             [1e4, 2e4, 3e4], True, pre=ops)
    for u, v in zip(b1, b2):
        assert torch.equal(u, v)
    c1 = engine.czt_propagate([e.expand(3, n, n), e.expand(3, n, n)], x, y, 0.6, 2e4, xo, yo, "vczt", pre=ops)
    c2 = engine.czt_propagate([e.expand(3, n, n).contiguous()] * 2, x, y, 0.6, 2e4, xo, yo, "vczt", pre=ops)
    for u, v in zip(c1, c2):
        assert torch.equal(u, v)
