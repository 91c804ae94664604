"""The two optimisation steps the benchmark times, at their configured sizes,
against the complex128 torch restatement of the reference (the gradient
oracle; jax.grad is not installable on these machines):

* the 4f step: 16 independent tables (own input mask, target and SLM planes),
  1024^2 -> RS 25 cm -> lens 25 cm -> CZT onto a 512^2 ROI -> SLM2 -> CZT,
  532 nm, normalised-intensity MSE (experiments/four_f_optical_table.py:129-141,
  experiments/four_f_optimizer.py:43);
* the high-NA step: 32 tables of 2048^2 with per-pixel LCD and sSLM planes
  U[0, 2 pi) -> VCZT objective lens (NA 0.9, f = 3 mm) onto a 1024^2 ROI of
  2 um, Ez spot-size loss (loss_functions.py:24-40), with and without
  activation checkpointing.

The GPU runs the whole batch through the fused kernels and the hand-written
adjoints; the oracle checks two tables of it (the batch loss is the mean of
the tables' losses, and a table's loss depends on its own parameters only).
Bars: the normalised output intensities within rel-L2 1e-5, each table's
loss within 1e-5 relative, the parameter gradients within rel-L2 1e-4.
"""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu
ITOL = 1e-5
GTOL = 1e-4


def _f64(a):
    import torch
    return torch.as_tensor(np.asarray(a, dtype=np.float64)).requires_grad_(True)


def test_four_f_step_full_size():
    import torch

    from oracle import torch_ref as tr
    from xlumina_gb300.tables import FourFTable
    t = FourFTable()
    assert (t.n, t.m, t.B) == (1024, 512, 16) and t.phase1.shape == (16, 1024, 1024)
    I = t.intensities()
    L = torch.mean(torch.sum((I - t.target) ** 2, dim=(-2, -1)) / (t.m * t.m))
    L.backward()
    assert L.item() == pytest.approx(t.loss().item(), rel=1e-6)
    for b in (0, 11):
        inp, tgt, p1, p2 = t.entry(b)
        P1, P2 = _f64(p1), _f64(p2)
        l1 = tr.slm(torch.as_tensor(inp), P1)
        l2 = tr.rs_propagate(l1, t.x, t.y, t.wavelength, t.f)
        l3 = tr.lens(l2, t.x, t.y, t.wavelength, t.lens_r, (t.f, t.f))
        l4 = tr.czt(l3, t.x, t.y, t.wavelength, t.f, t.xo, t.yo)
        l5 = tr.slm(l4, P2)
        Ir = torch.abs(tr.czt(l5, t.xo, t.yo, t.wavelength, t.f, t.xo, t.yo)) ** 2
        Ir = Ir / torch.sum(Ir)
        Lb = torch.sum((Ir - torch.as_tensor(tgt)) ** 2) / (t.m * t.m)
        Lb.backward()
        assert rel_l2(I[b].detach().cpu().numpy(), Ir.detach().numpy()) < ITOL, b
        Lg = torch.sum((I[b].detach().double() - t.target[b].double()) ** 2).item() / (t.m * t.m)
        assert Lg == pytest.approx(Lb.item(), rel=ITOL)
        # d mean / d table b's parameters = (1 / B) d L_b / d parameters
        assert rel_l2(t.phase1.grad[b].cpu().numpy(), P1.grad.numpy() / t.B) < GTOL, b
        assert rel_l2(t.phase2.grad[b].cpu().numpy(), P2.grad.numpy() / t.B) < GTOL, b


@pytest.mark.parametrize("checkpoint", [False, True])
def test_high_na_step_full_size(checkpoint):
    import torch

    from oracle import torch_ref as tr
    from xlumina_gb300.tables import HighNATable, small_area_hybrid_batched
    t = HighNATable(checkpoint=checkpoint)
    assert (t.n, t.m, t.B) == (2048, 1024, 32) and t.eta.shape == (32, 2048, 2048)
    with torch.no_grad():
        I = t._spot_intensity()
    L = t.loss()
    L.backward()
    assert L.item() == pytest.approx(small_area_hybrid_batched(I).item(), rel=1e-6)
    Ex = t.Ex.cpu().numpy().astype(np.complex128)
    for b in ((0, 17) if not checkpoint else (5,)):
        eta, theta, alpha, phi = (_f64(a) for a in t.entry(b))
        ax, ay = tr.lcd(torch.as_tensor(Ex), torch.zeros_like(torch.as_tensor(Ex)), eta, theta)
        ax, ay = tr.sslm(ax, ay, alpha, phi)
        foc = tr.vczt_objective_lens(ax, ay, t.x, t.y, t.wavelength, t.r, t.f, t.xo, t.yo)
        Ir = torch.abs(foc[2]) ** 2
        Lb = tr.small_area_hybrid(Ir)
        Lb.backward()
        assert rel_l2(I[b].cpu().numpy(), Ir.detach().numpy()) < ITOL, b
        assert float(small_area_hybrid_batched(I[b:b + 1]).item()) == pytest.approx(Lb.item(), rel=ITOL)
        for got, exp in ((t.eta, eta), (t.theta, theta), (t.alpha, alpha), (t.phi, phi)):
            assert rel_l2(got.grad[b].cpu().numpy(), exp.grad.numpy() / t.B) < GTOL, b
