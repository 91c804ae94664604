"""Every kernel variant of a pass gives the oracle's result: the packed
two-line column pass (interleaved, in barrier groups, with prefetching), the
prefetching and the persistent one-line kernels and, at 4096 points, the
radix-64 kernel and the persistent kernel that keeps each unit's spectrum
values in Tensor Memory (variant 10), against the one-line kernel and the FP64 oracle, for the
transform lengths that have them (1024, 2048 and 4096 points: fields of
257..2048 per side).

Tolerance: relative L2 <= 1e-5 against the oracle (the path's bar); the
variants agree with each other to float32 rounding (<= 1e-6).
"""
import numpy as np
import pytest

from oracle import xlumina_ref as ref
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _np(t):
    return t.detach().cpu().numpy().astype(np.complex128)


@pytest.fixture
def variants():
    """(set, count) for the RS column pass; restores the selection afterwards."""
    from xlumina_gb300 import _lib, engine
    lib = engine.lib()
    saved = {l: lib.xl_get_kernel_variant(_lib.XL_PASS_RS_COLS, l) for l in range(10, 13)}

    def select(log2_len, v):
        _lib.check(lib.xl_set_kernel_variant(_lib.XL_PASS_RS_COLS, log2_len, v), "xl_set_kernel_variant")

    yield select, lambda l: lib.xl_kernel_variant_count(_lib.XL_PASS_RS_COLS, l)
    for l, v in saved.items():
        select(l, v)


def test_variant_table_bounds():
    from xlumina_gb300 import _lib, engine
    lib = engine.lib()
    assert lib.xl_kernel_variant_count(_lib.XL_PASS_RS_COLS, 12) == 11
    assert lib.xl_kernel_variant_count(_lib.XL_PASS_RS_COLS, 11) == 9
    assert lib.xl_kernel_variant_count(_lib.XL_PASS_RS_COLS, 6) == 1
    assert lib.xl_kernel_variant_count(_lib.XL_PASS_CZT_ROWS, 12) == 5
    assert lib.xl_kernel_variant_count(_lib.XL_PASS_CZT_ROWS, 11) == 4
    assert lib.xl_kernel_variant_count(_lib.XL_PASS_CZT_COLS, 12) == 2
    assert lib.xl_get_kernel_variant(_lib.XL_PASS_CZT_COLS, 12) == 1   # the default at 4096 points
    assert lib.xl_kernel_variant_count(99, 12) == 0
    assert lib.xl_set_kernel_variant(_lib.XL_PASS_RS_COLS, 12, 11) == _lib.XL_EINVAL
    assert lib.xl_set_kernel_variant(_lib.XL_PASS_RS_COLS, 11, 9) == _lib.XL_EINVAL
    assert lib.xl_get_kernel_variant(_lib.XL_PASS_RS_COLS, 12) == 8   # the default at 4096 points
    assert lib.xl_set_kernel_variant(_lib.XL_PASS_RS_COLS, 6, 1) == _lib.XL_EINVAL
    assert lib.xl_get_kernel_variant(-1, 12) == _lib.XL_EINVAL


@pytest.mark.parametrize("n,vector", [(300, True), (1000, False), (1024, True), (2048, False)])
def test_rs_column_variants_match_oracle(variants, n, vector):
    import torch

    from xlumina_gb300 import engine
    select, count = variants
    logp = engine.rs_logq(n, n) + 1
    nv = count(logp)
    assert nv == (11 if logp == 12 else 9)
    x, y = ref.space(1000.0, n)
    rng = np.random.default_rng(n + vector)
    Ex = ref.gaussian_beam(x, y, 0.633, (300.0, 300.0)) * np.exp(1j * rng.uniform(-np.pi, np.pi, (n, n)))
    Ey = 0.5 * ref.gaussian_beam(x, y, 0.633, (250.0, 250.0)) * np.exp(1j * rng.uniform(-1, 1, (n, n)))
    z = 3.0e4
    comps = [torch.as_tensor(Ex.astype(np.complex64), device="cuda")]
    if vector:
        comps.append(torch.as_tensor(Ey.astype(np.complex64), device="cuda"))
        exp = ref.vrs_propagate(Ex.astype(np.complex64), Ey.astype(np.complex64), x, y, 0.633, z)
    else:
        exp = [ref.rs_propagate(Ex.astype(np.complex64), x, y, 0.633, z)]
    outs = []
    for v in range(nv):
        select(logp, v)
        got = engine.rs_propagate(comps, x, y, 0.633, z, vector=vector)
        torch.cuda.synchronize()
        outs.append([_np(g) for g in got])
        for g, e in zip(outs[-1], exp):
            assert rel_l2(g, e) < TOL, (v, rel_l2(g, e))
    for v in range(1, nv):
        for g, g0 in zip(outs[v], outs[0]):
            assert rel_l2(g, g0) < 1e-6, v


@pytest.mark.parametrize("v,n", [(1, 700), (2, 700), (3, 700), (4, 700), (5, 700), (6, 700), (7, 700), (8, 700),
                                 (8, 1100), (9, 1100), (10, 1100)])
def test_rs_column_variants_adjoint_and_batch(variants, v, n):
    """The adjoint (conjugate spectrum) and a batch with a distance per entry
    through a variant equal the one-line kernel's results (the radix-64
    variant 9 and the Tensor Memory variant 10 exist for 4096-point
    transforms only: fields of 1025..2048)."""
    import torch

    from xlumina_gb300 import engine
    select, _ = variants
    x, y = ref.space(600.0, n)
    rng = np.random.default_rng(77)
    E = torch.as_tensor((rng.standard_normal((3, 2, n, n)) + 1j * rng.standard_normal((3, 2, n, n)))
                        .astype(np.complex64), device="cuda")
    zs = [1e4, 2e4, 5e4]
    logp = engine.rs_logq(n, n) + 1
    res = {}
    for var in (0, v):
        select(logp, var)
        fwd = engine.rs_propagate([E[:, 0], E[:, 1]], x, y, 0.6, zs, vector=True)
        adj = engine.RsCall([E[:, 0], E[:, 1], E[:, 0]], x, y, 0.6, zs, vector=True, adjoint=True).run()
        res[var] = [_np(t) for t in fwd] + [_np(t) for t in adj]
    for a, b in zip(res[v], res[0]):
        assert rel_l2(a, b) < 1e-6


@pytest.mark.parametrize("v", [1, 2, 3])
def test_czt_row_variants_match(v):
    """The chirp-z x transform with every plane staged for one CTA per SM
    (1), unstaged (2) or with registers for two CTAs per SM (3) gives the
    default kernel's result (the stage capped for two CTAs per SM): a VCZT
    behind an LCD and the Ez-only high-NA focus behind an sSLM."""
    import torch

    import xlumina_gb300.optical_elements as oe
    import xlumina_gb300.vectorized_optics as vo
    from xlumina_gb300 import _lib, engine
    lib = engine.lib()
    n, m = 512, 128
    x, y = ref.space(1500.0, n)
    xo, yo = ref.space(300.0, m)
    rng = np.random.default_rng(99)
    E = torch.as_tensor((rng.standard_normal((2, n, n)) + 1j * rng.standard_normal((2, n, n))).astype(np.complex64),
                        device="cuda")
    eta = torch.as_tensor(rng.uniform(0, 6, (n, n)).astype(np.float32), device="cuda")
    logl = [lg for lg in range(5, 14)]
    saved = {lg: lib.xl_get_kernel_variant(_lib.XL_PASS_CZT_ROWS, lg) for lg in logl}
    res = {}
    try:
        for var in (0, v):
            for lg in logl:
                _lib.check(lib.xl_set_kernel_variant(_lib.XL_PASS_CZT_ROWS, lg, var))
            light = vo.VectorizedLight(x, y, 0.6)
            light.Ex, light.Ey = E[0], E[1]
            a = oe.VCZT_objective_lens_ez(oe.sSLM(light, eta, eta), 1800.0, 2000.0, xo, yo)
            b = oe.LCD(light, eta, 0.3).VCZT(2.0e4, xo, yo)
            res[var] = [_np(a), _np(b.Ex), _np(b.Ey), _np(b.Ez)]
    finally:
        for lg, s in saved.items():
            lib.xl_set_kernel_variant(_lib.XL_PASS_CZT_ROWS, lg, s)
    for got, exp in zip(res[v], res[0]):
        assert rel_l2(got, exp) < 1e-6


@pytest.mark.parametrize("v", [0, 1, 2])
def test_czt_row_variants_with_the_fixed_high_na_program(v):
    """The high-NA table's program (LCD, sSLM, the lens's Ez row) at 4096-point
    lines runs a kernel with its op kinds fixed; every stage / register
    variant of it gives the default variant's (3) focal Ez."""
    import torch

    import xlumina_gb300.optical_elements as oe
    import xlumina_gb300.vectorized_optics as vo
    from xlumina_gb300 import _lib, engine
    lib = engine.lib()
    n, m = 1500, 600           # Bluestein length 4096 on both axes
    x, y = ref.space(1800.0, n)
    xo, yo = ref.space(3.0, m)
    rng = np.random.default_rng(7 + v)
    E = torch.as_tensor((rng.standard_normal((2, 2, n, n)) + 1j * rng.standard_normal((2, 2, n, n)))
                        .astype(np.complex64), device="cuda")
    P = [torch.as_tensor(rng.uniform(0, 2 * np.pi, (2, n, n)).astype(np.float32), device="cuda") for _ in range(4)]
    saved = lib.xl_get_kernel_variant(_lib.XL_PASS_CZT_ROWS, 12)
    assert saved == 3
    res = {}
    try:
        for var in (3, v):
            _lib.check(lib.xl_set_kernel_variant(_lib.XL_PASS_CZT_ROWS, 12, var))
            light = vo.VectorizedLight(x, y, 0.65)
            light.Ex, light.Ey = E[0], E[1]
            lit = oe.sSLM(oe.LCD(light, P[0], P[1]), P[2], P[3])
            res[var] = _np(oe.VCZT_objective_lens_ez(lit, 900.0, 1000.0, xo, yo))
    finally:
        lib.xl_set_kernel_variant(_lib.XL_PASS_CZT_ROWS, 12, saved)
    assert np.all(np.isfinite(res[3]))
    assert rel_l2(res[v], res[3]) < 1e-6


def test_czt_column_variants_match():
    """The persistent chirp-z y transform (variant 1) gives the per-tile
    kernel's (0) results: a VCZT behind an LCD, forward and adjoint (the Ez
    fold), and a batch with a distance per entry."""
    import torch

    import xlumina_gb300.optical_elements as oe
    import xlumina_gb300.vectorized_optics as vo
    from xlumina_gb300 import _lib, engine
    lib = engine.lib()
    n, m = 400, 160
    x, y = ref.space(1200.0, n)
    xo, yo = ref.space(300.0, m)
    rng = np.random.default_rng(123)
    E = torch.as_tensor((rng.standard_normal((2, 3, n, n)) + 1j * rng.standard_normal((2, 3, n, n)))
                        .astype(np.complex64), device="cuda")
    G = torch.as_tensor((rng.standard_normal((3, 3, m, m)) + 1j * rng.standard_normal((3, 3, m, m)))
                        .astype(np.complex64), device="cuda")
    eta = torch.as_tensor(rng.uniform(0, 6, (3, n, n)).astype(np.float32), device="cuda")
    logl = list(range(5, 14))
    saved = {lg: lib.xl_get_kernel_variant(_lib.XL_PASS_CZT_COLS, lg) for lg in logl}
    res = {}
    try:
        for var in (0, 1):
            for lg in logl:
                _lib.check(lib.xl_set_kernel_variant(_lib.XL_PASS_CZT_COLS, lg, var))
            light = vo.VectorizedLight(x, y, 0.6)
            light.Ex, light.Ey = E[0], E[1]
            fwd = oe.LCD(light, eta, 0.3).VCZT([1.5e4, 2.0e4, 3.0e4], xo, yo)
            adj = engine.CztCall([G[0], G[1], G[2]], x, y, 0.6, 2.0e4, xo, yo, "vczt", adjoint=True).run()
            torch.cuda.synchronize()
            res[var] = [_np(fwd.Ex), _np(fwd.Ey), _np(fwd.Ez)] + [_np(a) for a in adj]
    finally:
        for lg, s in saved.items():
            lib.xl_set_kernel_variant(_lib.XL_PASS_CZT_COLS, lg, s)
    for got, exp in zip(res[1], res[0]):
        assert np.all(np.isfinite(exp))
        assert rel_l2(got, exp) < 1e-6


def test_czt_row_one_group_variant_matches():
    """Variant 4 of the 4096-point chirp-z x transform (one component group
    transforming Ex, Ey, Ez one after the other, two CTAs per SM) gives the
    default kernel's VCZT behind an LCD, and the full high-NA focus."""
    import torch

    import xlumina_gb300.optical_elements as oe
    import xlumina_gb300.vectorized_optics as vo
    from xlumina_gb300 import _lib, engine
    lib = engine.lib()
    n, m = 1500, 600           # Bluestein length 4096 on both axes
    x, y = ref.space(1800.0, n)
    xo, yo = ref.space(300.0, m)
    rng = np.random.default_rng(44)
    E = torch.as_tensor((rng.standard_normal((2, 2, n, n)) + 1j * rng.standard_normal((2, 2, n, n)))
                        .astype(np.complex64), device="cuda")
    eta = torch.as_tensor(rng.uniform(0, 6, (2, n, n)).astype(np.float32), device="cuda")
    saved = lib.xl_get_kernel_variant(_lib.XL_PASS_CZT_ROWS, 12)
    res = {}
    try:
        for var in (saved, 4):
            _lib.check(lib.xl_set_kernel_variant(_lib.XL_PASS_CZT_ROWS, 12, var))
            light = vo.VectorizedLight(x, y, 0.65)
            light.Ex, light.Ey = E[0], E[1]
            a = oe.LCD(light, eta, 0.3).VCZT(2.0e4, xo, yo)
            xf, yf = ref.space(3.0, m)
            b = oe.VCZT_objective_lens(oe.sSLM(light, eta, eta), 900.0, 1000.0, xf, yf)
            torch.cuda.synchronize()
            res[var] = [_np(a.Ex), _np(a.Ey), _np(a.Ez), _np(b.Ex), _np(b.Ey), _np(b.Ez)]
    finally:
        lib.xl_set_kernel_variant(_lib.XL_PASS_CZT_ROWS, 12, saved)
    for got, exp in zip(res[4], res[saved]):
        assert np.all(np.isfinite(exp))
        assert rel_l2(got, exp) < 1e-6
