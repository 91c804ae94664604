"""Fused intensity MSE (loss_functions.MSE_Intensity / vMSE_Intensity) against
the golden value from the reference and against torch autograd of the formula."""
import numpy as np
import pytest

from tests.conftest import golden, rel_l2

pytestmark = pytest.mark.gpu


def test_mse_intensity_golden():
    import xlumina_gb300.loss_functions as lf
    g = golden("losses")
    v = float(lf.MSE_Intensity(g["a"], g["b"]))
    assert abs(v - float(g["mse_intensity"])) <= 1e-5 * abs(float(g["mse_intensity"]))


def test_mse_intensity_values_and_gradients_batched():
    import torch

    import xlumina_gb300.loss_functions as lf
    rng = np.random.default_rng(12)
    B, n = 3, 96
    a0 = torch.as_tensor((rng.standard_normal((B, n, n)) + 1j * rng.standard_normal((B, n, n))).astype(np.complex64),
                         device="cuda")
    b0 = torch.as_tensor((rng.standard_normal((B, n, n)) + 1j * rng.standard_normal((B, n, n))).astype(np.complex64),
                         device="cuda")
    w = torch.as_tensor(rng.uniform(0.5, 2.0, B).astype(np.float32), device="cuda")
    a = a0.clone().requires_grad_(True)
    b = b0.clone().requires_grad_(True)
    L = lf.MSE_Intensity(a, b)
    assert L.shape == (B,)
    (L * w).sum().backward()
    # reference: the formula in complex128 torch autograd
    ar = a0.to(torch.complex128).requires_grad_(True)
    br = b0.to(torch.complex128).requires_grad_(True)
    Lr = torch.sum((torch.abs(ar) ** 2 - torch.abs(br) ** 2) ** 2, dim=(-2, -1)) / (n * n)
    (Lr * w.double()).sum().backward()
    assert rel_l2(L.detach().cpu().numpy(), Lr.detach().cpu().numpy()) < 1e-5
    assert rel_l2(a.grad.cpu().numpy(), ar.grad.cpu().numpy()) < 1e-5
    assert rel_l2(b.grad.cpu().numpy(), br.grad.cpu().numpy()) < 1e-5
    # same inputs, same result (fixed-order sums)
    assert torch.equal(lf.MSE_Intensity(a0, b0), lf.MSE_Intensity(a0, b0))


def test_vmse_intensity_and_broadcast_target():
    import torch

    import xlumina_gb300.loss_functions as lf
    from xlumina_gb300.vectorized_optics import VectorizedLight
    rng = np.random.default_rng(13)
    n = 64
    x = np.linspace(-50, 50, n)
    mk = lambda *s: torch.as_tensor((rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(np.complex64),  # noqa: E731
                                    device="cuda")
    u = VectorizedLight(x, x, 0.5)
    v = VectorizedLight(x, x, 0.5)
    u.Ex, u.Ey, u.Ez = mk(2, n, n), mk(2, n, n), mk(2, n, n)
    v.Ex, v.Ey, v.Ez = mk(2, n, n), mk(2, n, n), mk(2, n, n)
    got = lf.vMSE_Intensity(u, v)
    assert got.shape == (3, 2)
    exp = torch.stack([torch.sum((torch.abs(getattr(u, c)) ** 2 - torch.abs(getattr(v, c)) ** 2) ** 2, dim=(-2, -1))
                       / (n * n) for c in ("Ex", "Ey", "Ez")])
    assert rel_l2(got.cpu().numpy(), exp.cpu().numpy()) < 1e-5
    t = mk(n, n)
    got_b = lf.MSE_Intensity(u.Ex, t)
    exp_b = torch.sum((torch.abs(u.Ex) ** 2 - torch.abs(t) ** 2) ** 2, dim=(-2, -1)) / (n * n)
    assert rel_l2(got_b.cpu().numpy(), exp_b.cpu().numpy()) < 1e-5


def test_area_loss_golden():
    """The fused small_area_hybrid and vectorized_loss_hybrid against the
    reference's own values (losses.npz, losses_more.npz)."""
    import torch

    import xlumina_gb300.loss_functions as lf
    g = golden("losses")
    v = lf.small_area_hybrid(torch.as_tensor(g["I"].astype(np.float32), device="cuda"))
    assert v.shape == () and abs(float(v) - float(g["small_area"])) <= 1e-5 * abs(float(g["small_area"]))
    g2 = golden("losses_more")
    got = lf.vectorized_loss_hybrid(torch.as_tensor(g2["I6"].astype(np.float32), device="cuda"))
    assert rel_l2(got.cpu().numpy(), g2["loss_hybrid"]) < 1e-5


def _spots(rng, B, n):
    """Smooth focal spots with noise: a clear maximum and a mask of a few hundred pixels."""
    X, Y = np.meshgrid(np.linspace(-1, 1, n), np.linspace(-1, 1, n))
    f = np.stack([np.exp(-((X - 0.1 * b) ** 2 + Y ** 2) / 0.02) * (1 + 0.3 * rng.standard_normal((n, n)))
                  for b in range(B)])
    return (f * np.exp(1j * rng.uniform(-np.pi, np.pi, (B, n, n)))).astype(np.complex64)


def test_area_loss_fused_from_fields_values_and_gradients():
    """Area loss of |Ez|^2 formed in the kernel, per plane, against torch
    autograd of the reference formula in complex128 (same masks)."""
    import torch

    import xlumina_gb300.loss_functions as lf
    from xlumina_gb300.tables import small_area_hybrid_batched
    rng = np.random.default_rng(21)
    B, n = 4, 128
    e0 = torch.as_tensor(_spots(rng, B, n), device="cuda")
    w = torch.as_tensor(rng.uniform(0.5, 2.0, B).astype(np.float32), device="cuda")
    e = e0.clone().requires_grad_(True)
    L = lf.small_area_hybrid_field(e)
    assert L.shape == (B,)
    (L * w).sum().backward()
    er = e0.to(torch.complex128).requires_grad_(True)
    Ir = torch.abs(er) ** 2
    In = Ir / (torch.sum(Ir, dim=(-2, -1), keepdim=True) + 1e-8)
    mask = (In > 0.7 * torch.amax(In, dim=(-2, -1), keepdim=True)).double()
    Lr = torch.sum(mask, dim=(-2, -1)) / (torch.sum(mask * In, dim=(-2, -1)) + 1e-8)
    (Lr * w.double()).sum().backward()
    assert rel_l2(L.detach().cpu().numpy(), Lr.detach().cpu().numpy()) < 1e-5
    assert rel_l2(e.grad.cpu().numpy(), er.grad.cpu().numpy()) < 1e-4
    # the mean over planes equals the torch batched form, and repeats exactly
    I = torch.abs(e0) ** 2
    assert float(torch.mean(lf.small_area_hybrid_field(e0))) == pytest.approx(
        float(small_area_hybrid_batched(I)), rel=1e-5)
    assert torch.equal(lf.small_area_hybrid_field(e0), lf.small_area_hybrid_field(e0))


def test_area_loss_on_intensities_gradient():
    import torch

    import xlumina_gb300.loss_functions as lf
    rng = np.random.default_rng(22)
    I0 = torch.as_tensor(np.abs(_spots(rng, 3, 96)) ** 2, device="cuda")
    I = I0.clone().requires_grad_(True)
    lf.vectorized_loss_hybrid(I).sum().backward()
    Ir = I0.double().requires_grad_(True)
    In = Ir / (torch.sum(Ir, dim=(-2, -1), keepdim=True) + 1e-8)
    mask = (In > 0.7 * torch.amax(In, dim=(-2, -1), keepdim=True)).double()
    (torch.sum(mask, dim=(-2, -1)) / (torch.sum(mask * In, dim=(-2, -1)) + 1e-8)).sum().backward()
    assert rel_l2(I.grad.cpu().numpy(), Ir.grad.cpu().numpy()) < 1e-4


@pytest.mark.parametrize("shared_target", [False, True])
def test_normalised_intensity_mse_values_and_gradients(shared_target):
    """The 4f loss (experiments/four_f_optical_table.py:129-141) fused, against
    torch autograd of the formula in complex128."""
    import torch

    import xlumina_gb300.loss_functions as lf
    rng = np.random.default_rng(23 + shared_target)
    B, m = 3, 80
    u0 = torch.as_tensor((rng.standard_normal((B, m, m)) + 1j * rng.standard_normal((B, m, m))).astype(np.complex64),
                         device="cuda")
    t = (rng.uniform(0, 1, (m, m) if shared_target else (B, m, m)) < 0.1).astype(np.float32)
    t /= t.sum(axis=(-2, -1), keepdims=True)
    tg = torch.as_tensor(t, device="cuda")
    w = torch.as_tensor(rng.uniform(0.5, 2.0, B).astype(np.float32), device="cuda")
    u = u0.clone().requires_grad_(True)
    L = lf.normalized_intensity_mse(u, tg)
    (L * w).sum().backward()
    ur = u0.to(torch.complex128).requires_grad_(True)
    Ir = torch.abs(ur) ** 2
    Ir = Ir / torch.sum(Ir, dim=(-2, -1), keepdim=True)
    Lr = torch.sum((Ir - tg.double()) ** 2, dim=(-2, -1)) / (m * m)
    (Lr * w.double()).sum().backward()
    assert rel_l2(L.detach().cpu().numpy(), Lr.detach().cpu().numpy()) < 1e-5
    assert rel_l2(u.grad.cpu().numpy(), ur.grad.cpu().numpy()) < 1e-4


def test_amplitude_and_phase_mse_golden_and_gradients():
    """MSE_Amplitude / MSE_Phase and their per-component forms fused on the
    device: against the reference's values (losses_more.npz) and torch
    autograd of the formulas in complex128."""
    import torch

    import xlumina_gb300.loss_functions as lf
    from xlumina_gb300.vectorized_optics import VectorizedLight
    g = golden("losses_more")
    a3 = torch.as_tensor(g["a3"].astype(np.complex64), device="cuda")
    b3 = torch.as_tensor(g["b3"].astype(np.complex64), device="cuda")
    assert float(lf.MSE_Amplitude(a3[0], b3[0])) == pytest.approx(float(g["mse_amplitude"]), rel=1e-5)
    assert float(lf.MSE_Phase(a3[0], b3[0])) == pytest.approx(float(g["mse_phase"]), rel=1e-5)
    x = np.linspace(-10, 10, 20)
    la, lb = VectorizedLight(x, x, 0.5), VectorizedLight(x, x, 0.5)
    la.Ex, la.Ey, la.Ez = a3[0], a3[1], a3[2]
    lb.Ex, lb.Ey, lb.Ez = b3[0], b3[1], b3[2]
    assert rel_l2(lf.vMSE_Amplitude(la, lb).cpu().numpy(), g["vmse_amplitude"]) < 1e-5
    assert rel_l2(lf.vMSE_Phase(la, lb).cpu().numpy(), g["vmse_phase"]) < 1e-5
    rng = np.random.default_rng(31)
    w = torch.as_tensor(rng.uniform(0.5, 2.0, 3).astype(np.float32), device="cuda")
    for fn, ref_fn in ((lf.MSE_Amplitude, lambda u, v: (torch.abs(u) - torch.abs(v)) ** 2),
                       (lf.MSE_Phase, lambda u, v: (torch.angle(u) - torch.angle(v)) ** 2)):
        a = a3.clone().requires_grad_(True)
        b = b3.clone().requires_grad_(True)
        (fn(a, b) * w).sum().backward()
        ar = a3.to(torch.complex128).requires_grad_(True)
        br = b3.to(torch.complex128).requires_grad_(True)
        (torch.sum(ref_fn(ar, br), dim=(-2, -1)) / 400 * w.double()).sum().backward()
        assert rel_l2(a.grad.cpu().numpy(), ar.grad.cpu().numpy()) < 1e-4
        assert rel_l2(b.grad.cpu().numpy(), br.grad.cpu().numpy()) < 1e-4
