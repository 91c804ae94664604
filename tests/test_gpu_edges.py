"""Edge cases of the propagators against the FP64 oracle: the smallest
grids, odd and non-square grids (the oracle restates the (2ny-1) x (2nx-1)
pad for any shape; the reference's own build_grid assumes nx == ny),
negative distances for VRS, and one batch mixing distances of both signs.
Bar: rel-L2 1e-5 (complex64)."""
import numpy as np
import pytest

from oracle import xlumina_ref as ref
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _rnd(rng, *s):
    return rng.standard_normal(s) + 1j * rng.standard_normal(s)


@pytest.mark.parametrize("ny,nx", [(2, 2), (3, 3), (5, 7), (17, 16), (33, 64), (100, 37)])
def test_rs_small_odd_and_non_square(ny, nx):
    from xlumina_gb300 import engine
    rng = np.random.default_rng(ny * 100 + nx)
    x = np.linspace(-40.0, 40.0, nx)
    y = np.linspace(-30.0, 30.0, ny) if ny > 1 else np.array([0.0])
    f = _rnd(rng, ny, nx)
    out = engine.rs_propagate([engine.as_field(f)], x, y, 0.6, 900.0, vector=False)[0].cpu().numpy()
    assert rel_l2(out, ref.rs_propagate(f, x, y, 0.6, 900.0)) < TOL


def test_vrs_negative_distance_and_mixed_batch():
    import torch

    from xlumina_gb300 import engine
    rng = np.random.default_rng(77)
    n = 96
    x, y = ref.space(240.0, n)
    Ex, Ey = _rnd(rng, 3, n, n), _rnd(rng, 3, n, n)
    zs = [-2200.0, 1500.0, -900.0]
    outs = engine.rs_propagate([torch.as_tensor(Ex.astype(np.complex64), device="cuda"),
                                torch.as_tensor(Ey.astype(np.complex64), device="cuda")], x, y, 0.55, zs, vector=True)
    for b, z in enumerate(zs):
        exp = ref.vrs_propagate(Ex[b], Ey[b], x, y, 0.55, z)
        for o, e in zip(outs, exp):
            assert rel_l2(o[b].cpu().numpy(), e) < TOL
    # the same batch with the distances on the device (spectra built there)
    zt = torch.tensor(zs, dtype=torch.float64, device="cuda")
    outs_d = engine.rs_propagate([torch.as_tensor(Ex.astype(np.complex64), device="cuda"),
                                  torch.as_tensor(Ey.astype(np.complex64), device="cuda")], x, y, 0.55, zt, vector=True)
    for o, od in zip(outs, outs_d):
        assert torch.equal(o, od)


def test_czt_non_square_roi_and_negative_distance():
    from xlumina_gb300 import engine
    rng = np.random.default_rng(78)
    x, y = ref.space(300.0, 80)
    f = _rnd(rng, 80, 80)
    xo = np.linspace(-50.0, 40.0, 33)
    yo = np.linspace(-20.0, 60.0, 18)
    for z in (3000.0, -3000.0):
        out = engine.czt_propagate([engine.as_field(f)], x, y, 0.6, z, xo, yo, "scalar")[0].cpu().numpy()
        assert rel_l2(out, ref.czt(f, x, y, 0.6, z, xo, yo)) < TOL


@pytest.mark.parametrize("n,mx,my", [(5, 3, 5), (9, 6, 2), (31, 7, 11)])
def test_czt_small_grids(n, mx, my):
    from xlumina_gb300 import engine
    rng = np.random.default_rng(n * 7 + mx)
    x = np.linspace(-20.0, 20.0, n)
    f = _rnd(rng, n, n)
    xo = np.linspace(-5.0, 6.0, mx)
    yo = np.linspace(-4.0, 3.0, my)
    out = engine.czt_propagate([engine.as_field(f)], x, x, 0.5, 800.0, xo, yo, "scalar")[0].cpu().numpy()
    assert rel_l2(out, ref.czt(f, x, x, 0.5, 800.0, xo, yo)) < TOL


def test_full_size_energy_and_adjoint_identity():
    """Size-independent properties at the benchmark's 2048² size: RS conserves
    the power of a beam well inside the window (the reference's
    is_conserving_energy, toolbox.py:74-96; the FP64 oracle gives 1 - 1e-11
    here), and <A u, v> = <u, A^H v> for a batch of VRS fields at two
    distances."""
    import torch

    from xlumina_gb300 import engine, toolbox
    from xlumina_gb300 import wave_optics as wo
    n = 2048
    x, y = ref.space(2000.0, n)
    src = wo.LightSource(x, y, 0.65)
    src.gaussian_beam(w0=(300.0, 300.0), E0=1)
    out, _ = src.RS_propagation(5e4)
    assert abs(toolbox.is_conserving_energy(src, out).item() - 1.0) < 1e-5

    rng = np.random.default_rng(79)

    def rnd(*s):
        return torch.as_tensor((rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(np.complex64),
                               device="cuda")

    def dot(a, b):
        return complex(torch.sum(a.to(torch.complex128) * torch.conj(b.to(torch.complex128))).item())

    zs = [1e4, 1e5]
    ux, uy = rnd(2, n, n), rnd(2, n, n)
    vs = [rnd(2, n, n) for _ in range(3)]
    Au = engine.RsCall([ux, uy], x, y, 0.633, zs, True).run()
    Ahv = engine.RsCall(vs, x, y, 0.633, zs, True, adjoint=True).run()
    lhs = sum(dot(a, b) for a, b in zip(Au, vs))
    rhs = dot(ux, Ahv[0]) + dot(uy, Ahv[1])
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)
