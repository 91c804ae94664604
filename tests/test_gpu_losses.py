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
