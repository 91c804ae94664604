"""Captured CUDA-graph plans replay exactly what the eager calls compute."""
import numpy as np
import pytest

from oracle import xlumina_ref as ref
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_captured_vrs_plan_matches_eager():
    import torch

    from xlumina_gb300 import engine, plans
    n, B = 256, 3
    x, y = ref.space(500.0, n)
    rng = np.random.default_rng(31)
    E = torch.as_tensor((rng.standard_normal((2, B, n, n)) + 1j * rng.standard_normal((2, B, n, n)))
                        .astype(np.complex64), device="cuda")
    eta = torch.as_tensor(rng.uniform(0, 6, (B, n, n)).astype(np.float32), device="cuda")
    theta = torch.as_tensor(rng.uniform(0, 6, (B, n, n)).astype(np.float32), device="cuda")
    zs = [1e4, 3e4, 1e4]
    ex, ey = E[0].clone(), E[1].clone()

    def fn(ex, ey, eta, theta):
        return engine.rs_propagate([ex, ey], x, y, 0.6, zs, True, pre=[engine.op_lcd(eta, theta), engine.op_lp(0.3)])

    plan = plans.CapturedPlan(fn, ex, ey, eta, theta)
    got = [o.clone() for o in plan.replay()]
    exp = fn(ex, ey, eta, theta)
    for g, e in zip(got, exp):
        assert torch.equal(g, e)
    # new inputs through the same graph
    ex2 = torch.roll(E[0], 7, dims=-1)
    got2 = [o.clone() for o in plan(ex2)]
    exp2 = fn(ex2, ey, eta, theta)
    for g, e in zip(got2, exp2):
        assert torch.equal(g, e)
    # and against the oracle for one entry
    ax, ay = ref.linear_polarizer(*ref.lcd(ex2[1].cpu().numpy().astype(np.complex128),
                                           ey[1].cpu().numpy().astype(np.complex128),
                                           eta[1].cpu().numpy().astype(np.float64),
                                           theta[1].cpu().numpy().astype(np.float64)), 0.3 * np.ones((n, n)))
    o = ref.vrs_propagate(ax, ay, x, y, 0.6, zs[1])
    for g, e in zip(got2, o):
        assert rel_l2(g[1].cpu().numpy(), e) < 1e-5


def test_captured_czt_plan_matches_eager():
    import torch

    from xlumina_gb300 import engine, plans
    n = 256
    x, y = ref.space(400.0, n)
    xo, yo = ref.space(100.0, 128)
    rng = np.random.default_rng(32)
    f = torch.as_tensor((rng.standard_normal((2, n, n)) + 1j * rng.standard_normal((2, n, n)))
                        .astype(np.complex64), device="cuda")

    def fn(u):
        return engine.czt_propagate([u], x, y, 0.55, 2e4, xo, yo, "scalar")

    plan = plans.CapturedPlan(fn, f.clone())
    got = plan(f)[0].clone()
    assert torch.equal(got, fn(f)[0])


def test_captured_table_step_matches_eager_steps():
    import torch

    from xlumina_gb300 import plans
    from xlumina_gb300.tables import FourFTable
    kw = dict(n=128, roi_n=64, batch=4, half_width=800.0, f=5e4, roi_half_width=300.0, waist=500.0, seed=7)
    eager = FourFTable(**kw, capturable=True)
    capt = FourFTable(**kw, capturable=True)
    step = plans.CapturedStep(capt, warmup=3)
    for _ in range(3):     # the capture's warm-up steps
        eager.step()
    for _ in range(4):
        le = float(eager.step().detach())
        lc = float(step())
        assert abs(le - lc) <= 1e-5 * abs(le) + 1e-12, (le, lc)
    assert torch.allclose(eager.phase1, capt.phase1, rtol=1e-5, atol=1e-6)


def test_vrs_lcd_table_captured_matches_eager():
    import torch

    from xlumina_gb300 import plans
    from xlumina_gb300.tables import VrsLcdTable
    kw = dict(n=128, batch=2, half_width=400.0, waist=150.0, z=2e4, seed=9)
    eager = VrsLcdTable(**kw, capturable=True)
    capt = VrsLcdTable(**kw, capturable=True)
    step = plans.CapturedStep(capt, warmup=3)
    for _ in range(3):
        eager.step()
    l0 = None
    for _ in range(4):
        le = float(eager.step().detach())
        lc = float(step())
        l0 = le if l0 is None else l0
        assert abs(le - lc) <= 1e-5 * abs(le) + 1e-12, (le, lc)
    assert le < l0
    assert torch.allclose(eager.eta, capt.eta, rtol=1e-5, atol=1e-6)


def test_captured_hybrid_table_step_matches_eager():
    """The sharp-focus discovery step (trainable distances, splitter angles,
    LCD settings and masks) records into one CUDA graph: distances stay on the
    device, so nothing in the step reads back to the host."""
    import torch

    from xlumina_gb300.plans import CapturedStep
    from xlumina_gb300.tables import SharpFocusTable
    kw = dict(n=128, roi_n=48, seed=7)
    eager = SharpFocusTable(**kw, capturable=True)
    cap = SharpFocusTable(**kw, capturable=True)
    for a, b in zip(eager.params, cap.params):
        b.data.copy_(a.data)
    cs = CapturedStep(cap, warmup=3)
    for _ in range(3):          # the warm-up steps the plan took
        eager.step()
    le = [float(eager.step().detach()) for _ in range(3)]
    lc = [float(cs().detach()) for _ in range(3)]
    assert all(abs(a - b) <= 1e-4 * abs(a) for a, b in zip(le, lc)), (le, lc)
    for a, b in zip(eager.params, cap.params):
        assert torch.allclose(a, b, rtol=1e-4, atol=1e-5)
