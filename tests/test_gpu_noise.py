"""Table noise (shake_setup, optical_elements.py:2127-2301) on the GPU: the
reference's shapes, ranges and sign conventions, the device generator bit for
bit against the oracle's Philox4x32-10, one launch for many tables equal to
the tables one by one, and noisy tables batched through robust_discovery."""
import numpy as np
import pytest

from oracle import xlumina_ref as ref

pytestmark = pytest.mark.gpu

NS = {"n_tables": 3, "number of distances": 8, "number of sSLM": 3, "number of wps": 3,
      "noise_level": "tunable", "misalignment": (10, 100), "phase_noise": (0.01, 0.1), "discretize": False}


def test_shake_setup_shapes_ranges_and_bits():
    from xlumina_gb300 import noise
    key = noise.PRNGKey(1234)
    d, s, w, a, key0, k = noise.shake_setup(key, 64, NS)
    assert d.shape == (8,) and s.shape == (6, 64, 64) and w.shape == (6,) and a.shape == (6, 64, 64)
    d, s, w, a = (t.cpu().numpy() for t in (d, s, w, a))
    assert ((d >= 10) & (d < 100)).all()
    for t in (s, a, w):
        m = np.abs(t)
        assert ((m >= 0.01 - 1e-7) & (m < 0.1 + 1e-7)).all()
        assert 0.3 < (t > 0).mean() < 0.7
    assert np.array_equal(np.abs(s), np.abs(a))          # shared magnitudes, as the reference's draws
    assert not np.array_equal(s, a)
    assert (k == key).all() and not (key0 == key).all()
    # bit for bit against the oracle's generator
    kn = noise.split(key, 2)[1]
    flat_s, flat_a = s.ravel(), a.ravel()
    for e in [0, 1, 2, 4095, 4096, 12345, flat_s.size - 1]:
        vs, va = ref.table_noise_element(kn, e, 0.01, 0.1)
        assert flat_s[e] == vs and flat_a[e] == va
    rd, rw = ref.table_noise_scalars(kn, 8, 6, 10.0, 100.0, 0.01, 0.1)
    assert np.array_equal(d, rd) and np.array_equal(w, rw)


def test_discretize_and_levels():
    from xlumina_gb300 import noise
    ns = dict(NS, discretize=True, noise_level="mild")
    _, s, w, a, _, _ = noise.shake_setup(noise.PRNGKey(5), 32, ns)
    s = s.cpu().numpy()
    neg = s[s > 0.5 + 1e-6]          # a negative sign cast to uint8 is 255
    assert neg.size > 0 and ((neg >= 255 * 0.05 - 1e-4) & (neg < 255 * 0.5 + 1e-3)).all()
    assert (np.abs(w.cpu().numpy()) < 0.5 + 1e-9).all()


def test_batch_shake_setup_matches_tables_one_by_one():
    import torch

    from xlumina_gb300 import noise
    keys = noise.keychain_optical_tables(99, 3)
    x = np.zeros(48)
    d, s, w, a, key0, old = noise.batch_shake_setup(keys, x, NS)
    assert d.shape == (3, 8) and s.shape == (3, 6, 48, 48)
    for t in range(3):
        dt, st, wt, at, k0, _ = noise.shake_setup(keys[t], 48, NS)
        assert torch.equal(d[t], dt) and torch.equal(s[t], st) and torch.equal(w[t], wt) and torch.equal(a[t], at)
        assert (key0[t] == k0).all()


def test_batched_noisy_tables_match_one_by_one():
    """batch_robust_discovery (every table in the same launches) against
    robust_discovery run per table with that table's noise."""
    import torch

    from tests.conftest import golden, rel_l2
    import xlumina_gb300.optical_elements as oe
    import xlumina_gb300.vectorized_optics as vo
    from xlumina_gb300 import noise
    g = golden("hybrid_tables")
    red = vo.VectorizedLight(g["x"], g["y"], 0.65)
    red.Ex = torch.as_tensor(g["red_Ex"].astype(np.complex64), device="cuda")
    red.Ey = torch.as_tensor(g["red_Ey"].astype(np.complex64), device="cuda")
    fixed = [float(g["r"]), float(g["f"]), g["xout"], g["yout"]]
    p = [torch.as_tensor(np.asarray(g[f"p_robust_{k}"], dtype=np.float64), device="cuda") for k in range(35)]
    ns = dict(NS, **{"number of distances": 8, "number of sSLM": 3, "number of wps": 3})
    d, s, w, a, _, _ = noise.batch_shake_setup(noise.keychain_optical_tables(3, 3), np.zeros(32), ns)
    I = oe.batch_robust_discovery(red, red, red, red, red, red, p, fixed, d, s, w, a)
    assert I.shape == (3, 6, 16, 16)
    for t in range(3):
        It = oe.robust_discovery(red, red, red, red, red, red, p, fixed, list(d[t]), list(s[t]), list(w[t]),
                                 list(a[t]))
        assert rel_l2(I[t].cpu().numpy(), It.cpu().numpy()) < 1e-5
