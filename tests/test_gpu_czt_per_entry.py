"""Chirp-z at one distance per batch entry (CZT_jit over a stack of z,
wave_optics.py:233-357): the device-built chirps against the host float64
plan of the same formulas (wave_optics.py:385-460), per-entry batches against
one call per distance, the oracle at small sizes, and the serving path that
packs requests at different distances into one launch.

Tolerances: chirp vectors complex64 rel-L2 <= 1e-6 (both round float64
values to complex64; the phases agree to ~1e-8 rad); propagated fields
rel-L2 <= 1e-6 against single-distance calls and <= 1e-5 against the
oracle, as for the single-distance chirp-z."""
import numpy as np
import pytest

from oracle import xlumina_ref as ref
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy().astype(np.complex128)


@pytest.fixture(scope="module")
def torch_engine():
    import torch

    from xlumina_gb300 import engine
    return torch, engine


def _field(rng, ny, nx, B=None):
    shape = (ny, nx) if B is None else (B, ny, nx)
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


@pytest.mark.parametrize("n,m,adjoint", [(96, 48, False), (96, 48, True), (200, 120, False),
                                         (3000, 1500, False), (3000, 1500, True)])
def test_device_chirps_match_host_plan(torch_engine, n, m, adjoint):
    torch, engine = torch_engine
    x, _ = ref.space(1500.0, n)
    y = x.copy()
    xo, _ = ref.space(400.0, m)
    yo, _ = ref.space(300.0, m)
    wl = 0.633
    zs = np.array([2.0e4, 7.5e4, 1.9e5])
    zt = torch.tensor(zs, device="cuda", dtype=torch.float64)
    Lx, Ly, prex, gx, postx, prey, gy, posty, cte = engine.entry_chirps(zt, wl, x, y, xo, yo, adjoint)
    ix, ox = (m, n) if adjoint else (n, m)
    for b, z in enumerate(zs):
        Dm = wl * z / (x[1] - x[0])
        for (L_, pre, g, post, o0, o1, i_len, o_len) in (
                (Lx, prex, gx, postx, xo[0], xo[-1], ix, ox), (Ly, prey, gy, posty, yo[0], yo[-1], ix, ox)):
            Lh, ph, gh, qh = engine.device_chirps(n, o0 + Dm / 2, o1 + Dm / 2, Dm, m, adjoint)
            assert Lh == L_
            got = [_np(v) for v in (pre[b * i_len:(b + 1) * i_len], g[b * L_:(b + 1) * L_],
                                    post[b * o_len:(b + 1) * o_len])]
            for a, w in zip(got, (ph, gh, qh)):
                assert rel_l2(a, _np(w)) < 1e-6
        want = z * (x[1] - x[0]) * (y[1] - y[0]) * wl
        assert abs(complex(_np(cte[b:b + 1])[0]) - want) <= 1e-6 * abs(want)


def test_per_entry_czt_matches_single_calls_and_oracle(torch_engine):
    torch, engine = torch_engine
    rng = np.random.default_rng(11)
    n, m = 72, 40
    x, _ = ref.space(600.0, n)
    xo, _ = ref.space(150.0, m)
    yo, _ = ref.space(120.0, m + 2)
    wl = 0.532
    zs = [1.5e4, 4.0e4, 1.1e5, 2.0e5]
    f = _field(rng, n, n, B=len(zs))
    dev = torch.tensor(f, device="cuda")
    out = engine.czt_propagate([dev], x, x, wl, zs, xo, yo, "scalar")[0]
    assert tuple(out.shape) == (len(zs), m + 2, m)
    for b, z in enumerate(zs):
        one = engine.czt_propagate([dev[b]], x, x, wl, z, xo, yo, "scalar")[0]
        assert rel_l2(_np(out[b]), _np(one)) < 1e-6
        assert rel_l2(_np(out[b]), ref.czt(f[b].astype(np.complex128), x, x, wl, z, xo, yo)) < 1e-5
    # distances as a device tensor: same result, no host copy of z
    zt = torch.tensor(zs, device="cuda", dtype=torch.float64)
    out_t = engine.czt_propagate([dev], x, x, wl, zt, xo, yo, "scalar")[0]
    assert rel_l2(_np(out_t), _np(out)) < 1e-7


def test_per_entry_vczt_forward_and_adjoint(torch_engine):
    torch, engine = torch_engine
    rng = np.random.default_rng(12)
    n, m = 64, 36
    x, _ = ref.space(500.0, n)
    xo, _ = ref.space(100.0, m)
    wl = 0.633
    zs = [3.0e4, 9.0e4, 1.6e5]
    B = len(zs)
    ex, ey = _field(rng, n, n, B), _field(rng, n, n, B)
    dex, dey = torch.tensor(ex, device="cuda"), torch.tensor(ey, device="cuda")
    outs = engine.czt_propagate([dex, dey], x, x, wl, zs, xo, xo, "vczt")
    for b, z in enumerate(zs):
        want = ref.vczt(ex[b].astype(np.complex128), ey[b].astype(np.complex128), x, x, wl, z, xo, xo)
        one = engine.czt_propagate([dex[b], dey[b]], x, x, wl, z, xo, xo, "vczt")
        for c in range(3):
            assert rel_l2(_np(outs[c][b]), _np(one[c])) < 1e-6
            assert rel_l2(_np(outs[c][b]), want[c]) < 1e-5
    # adjoint: per entry against one adjoint call per distance
    gs = [torch.tensor(_field(rng, m, m, B), device="cuda") for _ in range(3)]
    adj = engine.CztCall(gs, x, x, wl, zs, xo, xo, "vczt", adjoint=True).run()
    for b, z in enumerate(zs):
        one = engine.CztCall([g[b] for g in gs], x, x, wl, z, xo, xo, "vczt", adjoint=True).run()
        for c in range(2):
            assert rel_l2(_np(adj[c][b]), _np(one[c])) < 1e-6


def test_per_entry_scalar_adjoint_dot_product(torch_engine):
    """<A u, v> = <u, A^H v> entry by entry for the per-entry scalar transform."""
    torch, engine = torch_engine
    rng = np.random.default_rng(13)
    n, m = 80, 44
    x, _ = ref.space(700.0, n)
    xo, _ = ref.space(180.0, m)
    zs = [2.5e4, 1.2e5]
    u = torch.tensor(_field(rng, n, n, 2), device="cuda")
    v = torch.tensor(_field(rng, m, m, 2), device="cuda")
    Au = engine.czt_propagate([u], x, x, 0.65, zs, xo, xo, "scalar")[0]
    AHv = engine.CztCall([v], x, x, 0.65, zs, xo, xo, "scalar", adjoint=True).run()[0]
    for b in range(2):
        lhs = np.vdot(_np(v[b]), _np(Au[b]))
        rhs = np.vdot(_np(AHv[b]), _np(u[b]))
        assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_per_entry_rejects_wrong_count(torch_engine):
    torch, engine = torch_engine
    x, _ = ref.space(500.0, 64)
    f = torch.zeros((3, 64, 64), dtype=torch.complex64, device="cuda")
    with pytest.raises(ValueError, match="distances for a batch"):
        engine.czt_propagate([f], x, x, 0.6, [1e4, 2e4], x, x, "scalar")


def test_light_czt_over_a_stack_of_distances():
    """ScalarLight.CZT with a batched field and one z per entry (an axial scan)."""
    import torch

    import xlumina_gb300.wave_optics as wo
    x, y = ref.space(800.0, 96)
    xo, _ = ref.space(60.0, 50)
    src = wo.LightSource(x, y, 0.633)
    src.gaussian_beam(w0=(300, 300), E0=1)
    zs = np.linspace(2e4, 8e4, 5)
    stack = wo.ScalarLight(x, y, 0.633)
    stack.field = src.field.expand(len(zs), -1, -1).contiguous()
    out = stack.CZT(torch.tensor(zs, device="cuda"), xo, xo)
    f0 = _np(src.field)
    for b, z in enumerate(zs):
        assert rel_l2(_np(out.field[b]), ref.czt(f0, x, y, 0.633, z, xo, xo)) < 1e-5


def test_serving_batches_czt_requests_across_distances():
    import torch

    from xlumina_gb300.serving import Request, run_batch
    rng = np.random.default_rng(14)
    x, y = ref.space(900.0, 128)
    xo, yo = ref.space(90.0, 64)
    f = torch.tensor(_field(rng, 128, 128), device="cuda")
    reqs = [Request("czt", [f], x, y, 0.633, float(z), xout=xo, yout=yo) for z in (1.2e4, 5e4, 1.9e5)]
    assert len({r.key() for r in reqs}) == 1
    outs = run_batch(reqs)
    for r, o in zip(reqs, outs):
        assert rel_l2(_np(o), _np(run_batch([r])[0])) < 1e-6


def test_phase_gradient_through_per_entry_czt():
    """d loss / d SLM phase through a chirp-z with one z per entry equals the
    single-distance gradients entry by entry (the adjoint reads the same
    per-entry chirps)."""
    import torch

    from xlumina_gb300 import autograd, engine
    rng = np.random.default_rng(15)
    n, m = 64, 30
    x, _ = ref.space(450.0, n)
    xo, _ = ref.space(90.0, m)
    zs = [2.0e4, 6.0e4, 1.5e5]
    f = torch.tensor(_field(rng, n, n, len(zs)), device="cuda")
    ph0 = torch.tensor(rng.uniform(-np.pi, np.pi, (len(zs), n, n)), device="cuda", dtype=torch.float32)
    tgt = torch.tensor(rng.uniform(0, 1, (len(zs), m, m)), device="cuda", dtype=torch.float32)

    def grad(field, phase, z, target):
        ph = phase.detach().clone().requires_grad_(True)
        plan = autograd.CztPlan(x, x, 0.633, z, xo, xo, "scalar", [engine.op_phase(ph)])
        out = autograd.fused_propagate(plan, [field], 1)[0]
        ((torch.abs(out) ** 2 - target) ** 2).sum().backward()
        return ph.grad

    g_all = grad(f, ph0, zs, tgt)
    for b, z in enumerate(zs):
        g_one = grad(f[b], ph0[b], z, tgt[b])
        assert rel_l2(_np(g_all[b]), _np(g_one)) < 1e-5
    with pytest.raises(NotImplementedError):
        autograd.CztPlan(x, x, 0.633, torch.tensor(zs, device="cuda", requires_grad=True), xo, xo, "scalar", [])


def test_transfer_planes_give_identical_results(torch_engine):
    """The second call with a geometry reads F and F0 from cached planes
    (xl_czt_transfer_plane); they hold the values the kernels compute per
    pixel, so the result is bit-identical, forward and adjoint."""
    torch, engine = torch_engine
    rng = np.random.default_rng(16)
    n, m = 96, 40
    x, _ = ref.space(700.0, n)
    xo, _ = ref.space(120.0, m)
    f = torch.tensor(_field(rng, n, n, 3), device="cuda")
    ey = torch.tensor(_field(rng, n, n, 3), device="cuda")
    gs = [torch.tensor(_field(rng, m, m, 3), device="cuda") for _ in range(3)]
    for z in (3.3e4, -2.1e4):
        engine.TRANSFER_PLANES.clear()
        b0 = engine.TRANSFER_PLANES.builds
        first = engine.czt_propagate([f], x, x, 0.633, z, xo, xo, "scalar")[0]
        assert engine.TRANSFER_PLANES.builds == b0            # first sight: evaluated in the kernels
        second = engine.czt_propagate([f], x, x, 0.633, z, xo, xo, "scalar")[0]
        assert engine.TRANSFER_PLANES.builds == b0 + 2        # F and F0 planes
        assert torch.equal(first, second)
        v1 = engine.czt_propagate([f, ey], x, x, 0.633, z, xo, xo, "vczt")
        v2 = engine.czt_propagate([f, ey], x, x, 0.633, z, xo, xo, "vczt")
        for a, b in zip(v1, v2):
            assert torch.equal(a, b)
        a1 = engine.CztCall(gs, x, x, 0.633, z, xo, xo, "vczt", adjoint=True).run()
        a2 = engine.CztCall(gs, x, x, 0.633, z, xo, xo, "vczt", adjoint=True).run()
        for a, b in zip(a1, a2):
            assert torch.equal(a, b)
        assert rel_l2(_np(second[1]), ref.czt(f[1].cpu().numpy().astype(np.complex128), x, x, 0.633, z, xo, xo)) < 1e-5
