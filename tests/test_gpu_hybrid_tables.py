"""The prebuilt hybrid tables (optical_elements.py:964-2120) on the GPU.

Forward: every table against the outputs of the reference's own source on a
32 x 32 grid (``tests/golden/hybrid_tables.npz``); rel-L2 2e-4 over 16 to 60
chained complex64 propagations.  Gradients of the sharp-focus table (splitter
angles, distances, LCD settings and phase masks, all tensors that require
grad) against torch autograd through its complex128 restatement; rel 1e-3.
"""
import numpy as np
import pytest

from tests.conftest import golden, rel_l2

pytestmark = pytest.mark.gpu
FWD = 2e-4


@pytest.fixture(scope="module")
def setup():
    import torch

    import xlumina_gb300.optical_elements as oe
    import xlumina_gb300.vectorized_optics as vo
    g = golden("hybrid_tables")

    def source(color):
        wl = 0.65 if color == "red" else 0.532
        s = vo.VectorizedLight(g["x"], g["y"], wl)
        s.Ex = torch.as_tensor(g[f"{color}_Ex"].astype(np.complex64), device="cuda")
        s.Ey = torch.as_tensor(g[f"{color}_Ey"].astype(np.complex64), device="cuda")
        return s
    return torch, oe, g, source("red"), source("green")


def _params(torch, g, name, n, grad=False):
    """The table's raw parameters as float64 device tensors (as the reference's
    x64 arrays; distances need float64)."""
    return [torch.as_tensor(np.asarray(g[f"{name}_{k}"], dtype=np.float64), device="cuda").requires_grad_(grad)
            for k in range(n)]


def test_sharp_focus_and_fluorophore_tables(setup):
    torch, oe, g, red, green = setup
    fixed = [float(g["r"]), float(g["f"]), g["xout"], g["yout"]]
    p = _params(torch, g, "p_sharp", 29)
    I, dets = oe.hybrid_setup_sharp_focus(red, red, red, red, red, red, p, fixed)
    assert len(dets) == 6
    assert rel_l2(I.cpu().numpy(), g["i_sharp"]) < FWD
    i_sted = oe.hybrid_setup_fluorophores(red, green, red, green, red, green, p, fixed, distance_offset=10)
    assert rel_l2(i_sted.cpu().numpy(), g["i_sted"]) < FWD


def test_fixed_mask_tables(setup):
    torch, oe, g, red, green = setup
    pms = [torch.as_tensor(g[f"pm_{k}"].astype(np.float32), device="cuda") for k in range(6)]
    fixed = [float(g["r"]), float(g["f"]), g["xout"], g["yout"]] + pms
    p = _params(torch, g, "p_fixed", 25)
    I, _ = oe.hybrid_setup_fixed_slms(red, red, red, red, red, red, p, fixed)
    assert rel_l2(I.cpu().numpy(), g["i_fixed"]) < FWD
    i_sted = oe.hybrid_setup_fixed_slms_fluorophores(red, green, red, green, red, green, p, fixed)
    assert rel_l2(i_sted.cpu().numpy(), g["i_fixed_sted"]) < FWD


def test_robust_and_six_by_six_tables(setup):
    torch, oe, g, red, green = setup
    fixed = [float(g["r"]), float(g["f"]), g["xout"], g["yout"]]
    p = _params(torch, g, "p_robust", 35)
    noise = {k: [torch.as_tensor(np.asarray(g[f"noise_{k}_{i}"], dtype=np.float64), device="cuda")
                 for i in range(8 if k == "d" else 6)] for k in "dswa"}
    I = oe.robust_discovery(red, red, red, red, red, red, p, fixed, noise["d"], noise["s"], noise["w"], noise["a"])
    assert rel_l2(I.cpu().numpy(), g["i_robust"]) < FWD
    pms = [torch.as_tensor(g[f"pm_{k}"].astype(np.float32), device="cuda") for k in range(4)]
    p6 = _params(torch, g, "p_six", 52)
    I6 = oe.six_times_six_ansatz(*([red] * 12), p6, fixed + pms, distance_offset=9.5)
    assert I6.shape[0] == 12
    assert rel_l2(I6.cpu().numpy(), g["i_six"]) < FWD


def test_sharp_focus_table_gradients(setup):
    torch, oe, g, red, green = setup
    from oracle import torch_ref as tr
    fixed = [float(g["r"]), float(g["f"]), g["xout"], g["yout"]]
    rng = np.random.default_rng(31)
    w = rng.uniform(0, 1, (6, 16, 16))
    p = _params(torch, g, "p_sharp", 29, grad=True)
    I, _ = oe.hybrid_setup_sharp_focus(red, red, red, red, red, red, p, fixed)
    L = torch.sum(torch.as_tensor(w, device="cuda") * I) / torch.sum(I.detach())
    L.backward()
    pr = [torch.as_tensor(np.asarray(g[f"p_sharp_{k}"], dtype=np.float64)).requires_grad_(True) for k in range(29)]
    src = (torch.as_tensor(g["red_Ex"].astype(np.complex64).astype(np.complex128)),
           torch.as_tensor(g["red_Ey"].astype(np.complex64).astype(np.complex128)))
    Ir = tr.hybrid_setup_sharp_focus(src, g["x"], g["y"], 0.65, pr, *fixed)
    Lr = torch.sum(torch.as_tensor(w) * Ir) / torch.sum(Ir.detach())
    Lr.backward()
    assert L.item() == pytest.approx(Lr.item(), rel=1e-4)
    # Scalar gradients are inner products of FP32 fields whose terms cancel:
    # the bar is 1e-3 of the gradient plus 2e-5 of the largest gradient of the
    # same kind (distances: indices 4, 5, 10, 11, 16, 17, 27, 28; the others
    # are angles), which bounds the sum of the terms' magnitudes from below.
    dist = {4, 5, 10, 11, 16, 17, 27, 28}
    scalar = [k for k in range(29) if pr[k].grad.numel() == 1]
    top = {kind: max(abs(pr[k].grad.item()) for k in scalar if (k in dist) == kind) for kind in (True, False)}
    bad = []
    for k in range(29):
        got, want = p[k].grad.cpu().numpy(), pr[k].grad.numpy()
        if want.size > 1:       # a phase mask
            if rel_l2(got, want) >= 1e-3:
                bad.append((k, rel_l2(got, want)))
        elif abs(got.item() - want.item()) > 1e-3 * abs(want.item()) + 2e-5 * top[k in dist]:
            bad.append((k, got.item(), want.item()))
    assert not bad, bad


def test_checkpointed_tables_give_the_same_step():
    """Activation checkpointing (wavefronts of the sharp-focus table: every
    one, every second, every second within a memory budget; the focus of the
    high-NA table) gives the same gradients.  The deep table
    keeps less at its peak; the one-focus table does not (its peak is the
    chirp-z workspace, which the recomputation needs again)."""
    import torch

    from xlumina_gb300.tables import HighNATable, SharpFocusTable
    for cls, kw in ((SharpFocusTable, dict(n=128, roi_n=48, seed=9)),
                    (HighNATable, dict(n=256, roi_n=64, batch=4, seed=9))):
        from xlumina_gb300.checkpointing import CheckpointPolicy
        grads = []
        peaks = []
        specs = (False, True, 2, CheckpointPolicy(every=2, budget_bytes=64 << 20)) if cls is SharpFocusTable \
            else (False, True)
        for ck in specs:
            t = cls(**kw, checkpoint=ck)
            # one unmeasured step first: the caches (transfer spectra and planes,
            # chirps) then hold everything, and the measured peak is the step's own
            t.loss().backward()
            for q in (t.params if hasattr(t, "params") else [t.eta, t.theta, t.alpha, t.phi]):
                q.grad = None
            torch.cuda.synchronize()
            torch.cuda.reset_peak_memory_stats()
            base = torch.cuda.memory_allocated()
            L = t.loss()
            L.backward()
            torch.cuda.synchronize()
            peaks.append(torch.cuda.max_memory_allocated() - base)
            params = t.params if hasattr(t, "params") else [t.eta, t.theta, t.alpha, t.phi]
            grads.append([p.grad.detach().clone() for p in params])
        for other in grads[1:]:
            for a, b in zip(grads[0], other):
                assert torch.allclose(a, b, rtol=1e-5, atol=1e-7)
        if cls is SharpFocusTable:
            # every policy keeps less than the unchecked step.  Segments of two
            # wavefronts store half the boundaries of one per wavefront, but at
            # 128^2 a boundary is small against the step's transient buffers,
            # so the two peaks agree within 1 % (the boundary counts are
            # checked on the CPU, tests/test_checkpointing_cpu.py)
            assert all(pk < peaks[0] for pk in peaks[1:]), peaks
            assert peaks[2] < 1.01 * peaks[1], peaks
