"""The Jones-program backward specialised for the programs the tables run
(LCD-sSLM-lens, LCD-polarizer, phase SLM, thin lens: kernels with the op
kinds fixed at compile time) gives the generic kernel's gradients.  The generic kernel is
reached by adding an exact identity op (a complex multiply by 1 + 0i) after
the first op, which changes the program's signature and not its values."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(n=96, batch=3, seed=21):
    import torch
    rng = np.random.default_rng(seed)
    d = lambda a: torch.as_tensor(a, device="cuda")  # noqa: E731
    E = d((rng.standard_normal((2, batch, n, n)) + 1j * rng.standard_normal((2, batch, n, n))).astype(np.complex64))
    G = d((rng.standard_normal((3, batch, n, n)) + 1j * rng.standard_normal((3, batch, n, n))).astype(np.complex64))
    P = [d(rng.uniform(0, 2 * np.pi, (batch, n, n)).astype(np.float32)).requires_grad_(True) for _ in range(4)]
    one = d(np.ones((n, n), dtype=np.complex64))
    return E, G, P, one


def _rel(a, b):
    a, b = a.double().cpu().numpy(), b.double().cpu().numpy()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def _compare(ops, ops_generic, base, gout, n):
    from xlumina_gb300 import engine
    gin_f, pg_f = engine.ops_backward(base, gout, ops, n, n)
    gin_g, pg_g = engine.ops_backward(base, gout, ops_generic, n, n)
    for a, b in zip(gin_f, gin_g):
        if a is not None:
            assert _rel(a, b) < 1e-6
    # the generic program has the identity op at index 1: later ops shift by one
    for (k, q), t in pg_f.items():
        kg = k if k == 0 else k + 1
        assert _rel(t, pg_g[(kg, q)]) < 1e-6, (k, q)


@pytest.mark.parametrize("ez_only", [True, False])
def test_lcd_sslm_lens(ez_only):
    from oracle import xlumina_ref as ref
    from xlumina_gb300 import engine
    n = 96
    E, G, P, one = _setup(n)
    x, y = ref.space(900.0, n)
    lens, _ = engine.op_high_na(x, y, 400.0, 1000.0, ez_only=ez_only)
    ops = [engine.op_lcd(P[0], P[1]), engine.op_sslm(P[2], P[3]), lens]
    gen = [ops[0], engine.op_cmul(one), ops[1], ops[2]]
    gout = [G[0]] + ([None, None] if ez_only else [G[1], G[2]])
    _compare(ops, gen, [E[0], E[1], None], gout, n)


def test_lcd_polarizer():
    from xlumina_gb300 import engine
    n = 96
    E, G, P, one = _setup(n)
    ops = [engine.op_lcd(P[0], P[1]), engine.op_lp(P[2])]
    gen = [ops[0], engine.op_cmul(one), ops[1]]
    _compare(ops, gen, [E[0], E[1], None], [G[0], G[1], G[2]], n)


def test_phase_slm():
    from xlumina_gb300 import engine
    n = 96
    E, G, P, one = _setup(n)
    ops = [engine.op_phase(P[0])]
    gen = [ops[0], engine.op_cmul(one)]
    _compare(ops, gen, [E[0]], [G[0]], n)


def test_thin_lens():
    """The 4f table's lens (a separable mask with a float64 pupil test, no
    parameters): only the input gradient."""
    from oracle import xlumina_ref as ref
    from xlumina_gb300 import engine
    n = 96
    E, G, P, one = _setup(n)
    x, y = ref.space(900.0, n)
    lens = engine.op_lens(x, y, 0.532, (300.0, 300.0), (2.0e4, 2.0e4), False)
    gen = [lens, engine.op_cmul(one)]
    _compare([lens], gen, [E[0]], [G[0]], n)
