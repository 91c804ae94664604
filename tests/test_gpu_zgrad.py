"""Distance gradients of RS / VRS (a z tensor that requires grad, as jax.grad
traces z through RS_propagation_jit, wave_optics.py:281-297) against central
finite differences of the FP64 numpy oracle.

Bar: |dL/dz - fd| <= 1e-4 * ||dL/dout|| * ||dout/dz|| (the Cauchy-Schwarz
scale of the inner product the gradient is; the FP32 propagation's error is a
relative 1e-6 of each factor), per distance.  The finite difference step is
1e-4 um, so k h ~ 1e-3 and its truncation error is far below the bar."""
import numpy as np
import pytest

from oracle import xlumina_ref as ref

pytestmark = pytest.mark.gpu
H = 1e-4
BAR = 1e-4


@pytest.fixture(scope="module")
def mods():
    import torch

    import xlumina_gb300.optical_elements as oe
    import xlumina_gb300.vectorized_optics as vo
    import xlumina_gb300.wave_optics as wo
    return torch, wo, vo, oe


def _check(g, loss_of_z, outs_of_z, dloss_dout, z):
    """g: the GPU gradient; loss_of_z / outs_of_z: the oracle at a distance;
    dloss_dout(outs): the loss gradient (torch's convention) at the oracle's outputs."""
    fd = (loss_of_z(z + H) - loss_of_z(z - H)) / (2 * H)
    dout = [(a - b) / (2 * H) for a, b in zip(outs_of_z(z + H), outs_of_z(z - H))]
    gl = dloss_dout(outs_of_z(z))
    scale = np.sqrt(sum(np.sum(np.abs(a) ** 2) for a in gl)) * np.sqrt(sum(np.sum(np.abs(d) ** 2) for d in dout))
    assert abs(g - fd) <= BAR * scale, (g, fd, scale)
    return fd


def test_rs_distance_gradient_with_slm(mods):
    """SLM phase -> RS(z): z.grad and the phase gradient together."""
    torch, wo, vo, oe = mods
    n, lam = 96, 0.633
    x, y = ref.space(300.0, n)
    rng = np.random.default_rng(11)
    ph = rng.uniform(-np.pi, np.pi, (n, n)).astype(np.float32)
    w = rng.uniform(0, 1, (n, n))
    v = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    src = wo.LightSource(x, y, lam)
    src.gaussian_beam(w0=(120.0, 120.0), E0=1)
    p = torch.as_tensor(ph, device="cuda").requires_grad_(True)
    z = torch.tensor(4000.0, dtype=torch.float64, requires_grad=True)
    out, _ = oe.SLM(src, p, n)[0].RS_propagation(z)
    f = out.field
    L = torch.sum(torch.as_tensor(w, device="cuda") * torch.abs(f) ** 2) + \
        torch.sum(torch.real(torch.conj(torch.as_tensor(v.astype(np.complex64), device="cuda")) * f))
    L.backward()
    assert p.grad is not None and z.grad is not None

    u = ref.slm(ref.gaussian_beam(x, y, lam, (120.0, 120.0)), ph.astype(np.float64))[0]

    def outs(zz):
        return [ref.rs_propagate(u, x, y, lam, zz)]

    def loss(zz):
        o = outs(zz)[0]
        return float(np.sum(w * np.abs(o) ** 2) + np.sum(np.real(np.conj(v) * o)))

    _check(z.grad.item(), loss, outs, lambda o: [2 * w * o[0] + v], 4000.0)


def test_vrs_per_entry_distance_gradients(mods):
    """A batch of three VRS fields, one distance each, behind a shared LCD;
    the Ez derivation's own z-dependence enters every entry's gradient."""
    torch, wo, vo, oe = mods
    n, lam, B = 64, 0.633, 3
    x, y = ref.space(200.0, n)
    rng = np.random.default_rng(12)
    eta, theta = rng.uniform(0, 2 * np.pi, (n, n)), rng.uniform(0, 2 * np.pi, (n, n))
    zs = np.array([2500.0, 3000.0, 4200.0])
    Ex0 = np.stack([ref.polarized_gaussian_beam(x, y, lam, (60.0 + 10 * b, 70.0), (1, 0.3 + 0.2 * b))[0]
                    for b in range(B)]) * np.exp(1j * rng.uniform(0, 1, (B, n, n)))
    Ey0 = np.stack([ref.polarized_gaussian_beam(x, y, lam, (60.0 + 10 * b, 70.0), (1, 0.3 + 0.2 * b))[1]
                    for b in range(B)])
    wts = [rng.uniform(0, 1, (n, n)) for _ in range(3)]
    light = vo.VectorizedLight(x, y, lam)
    light.Ex = torch.as_tensor(Ex0.astype(np.complex64), device="cuda")
    light.Ey = torch.as_tensor(Ey0.astype(np.complex64), device="cuda")
    pe = torch.as_tensor(eta.astype(np.float32), device="cuda").requires_grad_(True)
    z = torch.tensor(zs, dtype=torch.float64, requires_grad=True)
    out, _ = oe.LCD(light, pe, theta.astype(np.float32)).VRS_propagation(z)
    L = sum(torch.sum(torch.as_tensor(w, device="cuda") * torch.abs(c) ** 2) for w, c in zip(wts, (out.Ex, out.Ey, out.Ez)))
    L.backward()
    assert z.grad.shape == (B,)
    eta32, th32 = eta.astype(np.float32).astype(np.float64), theta.astype(np.float32).astype(np.float64)
    for b in range(B):
        ex, ey = ref.lcd(Ex0[b].astype(np.complex64).astype(np.complex128),
                         Ey0[b].astype(np.complex64).astype(np.complex128), eta32, th32)

        def outs(zz):
            return list(ref.vrs_propagate(ex, ey, x, y, lam, zz))

        def loss(zz):
            return float(sum(np.sum(w * np.abs(c) ** 2) for w, c in zip(wts, outs(zz))))

        _check(z.grad[b].item(), loss, outs, lambda o: [2 * w * c for w, c in zip(wts, o)], zs[b])


def test_vrs_shared_distance_gradient_sums_the_batch(mods):
    """One distance tensor for a batch: its gradient is the batch's sum."""
    torch, wo, vo, oe = mods
    n, lam, B = 64, 0.532, 2
    x, y = ref.space(150.0, n)
    rng = np.random.default_rng(13)
    Ex0 = (rng.standard_normal((B, n, n)) + 1j * rng.standard_normal((B, n, n))) * 0.1
    Ey0 = (rng.standard_normal((B, n, n)) + 1j * rng.standard_normal((B, n, n))) * 0.1
    w = rng.uniform(0, 1, (n, n))
    light = vo.VectorizedLight(x, y, lam)
    light.Ex = torch.as_tensor(Ex0.astype(np.complex64), device="cuda")
    light.Ey = torch.as_tensor(Ey0.astype(np.complex64), device="cuda")
    z = torch.tensor(1800.0, dtype=torch.float64, requires_grad=True)
    out, _ = light.VRS_propagation(z)
    L = torch.sum(torch.as_tensor(w, device="cuda") * torch.abs(out.Ez) ** 2)
    L.backward()
    e64 = [Ex0.astype(np.complex64).astype(np.complex128), Ey0.astype(np.complex64).astype(np.complex128)]

    def outs(zz):
        return [c for b in range(B) for c in ref.vrs_propagate(e64[0][b], e64[1][b], x, y, lam, zz)]

    def loss(zz):
        o = outs(zz)
        return float(sum(np.sum(w * np.abs(o[3 * b + 2]) ** 2) for b in range(B)))

    def dl(o):
        return [2 * w * c if i % 3 == 2 else np.zeros_like(c) for i, c in enumerate(o)]

    _check(z.grad.item(), loss, outs, dl, 1800.0)


def test_derivative_spectrum_propagation(mods):
    """Propagating through the spectrum of dH/dz gives dout/dz (RS and VRS,
    rel-L2 1e-4 against the oracle's central difference)."""
    torch, wo, vo, oe = mods
    from tests.conftest import rel_l2
    from xlumina_gb300 import engine
    n, lam, z = 80, 0.6, 2200.0
    x, y = ref.space(220.0, n)
    rng = np.random.default_rng(14)
    u = ((rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * 0.1).astype(np.complex64)
    v = ((rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * 0.1).astype(np.complex64)
    tu, tv = torch.as_tensor(u, device="cuda"), torch.as_tensor(v, device="cuda")
    d = engine.RsCall([tu], x, y, lam, z, False, dz=True).run()[0].cpu().numpy()
    fd = (ref.rs_propagate(u.astype(np.complex128), x, y, lam, z + H) -
          ref.rs_propagate(u.astype(np.complex128), x, y, lam, z - H)) / (2 * H)
    assert rel_l2(d, fd) < 1e-4
    # VRS with the derivative spectrum: the Ez derived at z, then propagated through dH/dz
    dv = [t.cpu().numpy() for t in engine.RsCall([tu, tv], x, y, lam, z, True, dz=True).run()]
    u64, v64 = u.astype(np.complex128), v.astype(np.complex128)
    ez = ref.vrs_ez(u64, v64, x, y, z)
    for got, comp in zip(dv, (u64, v64, ez)):
        want = (ref.rs_propagate(comp, x, y, lam, z + H) - ref.rs_propagate(comp, x, y, lam, z - H)) / (2 * H)
        assert rel_l2(got, want) < 1e-4


def test_ez_distance_term_and_inner_products(mods):
    """The two reductions of the distance gradient against numpy in float64:
    sum Re(conj(g) dEz/dz) per batch entry and sum Re(conj(a) b) per plane."""
    torch, wo, vo, oe = mods
    from xlumina_gb300 import engine
    n, B = 72, 3
    x, y = ref.space(180.0, n)
    zs = [900.0, 1500.0, -1200.0]
    rng = np.random.default_rng(15)

    def rnd(*s):
        return ((rng.standard_normal(s) + 1j * rng.standard_normal(s)) * 0.1).astype(np.complex64)

    ex, ey, g = rnd(B, n, n), rnd(B, n, n), rnd(B, n, n)
    got = engine.vrs_dz_ez(*(torch.as_tensor(a, device="cuda") for a in (ex, ey, g)), x, y, zs).cpu().numpy()
    X, Y = np.meshgrid(x, y)
    for b in range(B):
        r = np.sqrt(X ** 2 + Y ** 2 + zs[b] ** 2)
        dez = -(ex[b].astype(np.complex128) * X + ey[b].astype(np.complex128) * Y) * zs[b] / r ** 3
        want = np.sum(np.real(np.conj(g[b].astype(np.complex128)) * dez))
        scale = np.sqrt(np.sum(np.abs(g[b]) ** 2) * np.sum(np.abs(dez) ** 2))
        assert abs(got[b] - want) <= 1e-5 * scale
    a, c = rnd(B, n, n), rnd(B, n, n)
    got = engine.re_inner(torch.as_tensor(a, device="cuda"), torch.as_tensor(c, device="cuda")).cpu().numpy()
    want = np.sum(np.real(np.conj(a.astype(np.complex128)) * c.astype(np.complex128)), axis=(-2, -1))
    scale = np.sqrt(np.sum(np.abs(a) ** 2, axis=(-2, -1)) * np.sum(np.abs(c) ** 2, axis=(-2, -1)))
    assert np.all(np.abs(got - want) <= 1e-5 * scale)
