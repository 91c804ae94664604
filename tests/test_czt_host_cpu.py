"""Host-side planning of the chirp-z calls (no kernel runs): the Bluestein
length rule of wave_optics.py:373-383, 438 and its rejected sizes, which
distances count as one per batch entry, and the transfer-plane cache's
policy (evaluate in the kernels on first sight of a geometry, read planes
from the second use on, never build during graph capture)."""
import numpy as np
import pytest

from oracle import xlumina_ref as ref


def test_bluestein_length_follows_the_reference():
    from xlumina_gb300 import engine
    for m, M in ((1024, 512), (2048, 1024), (96, 48), (10, 7), (3000, 1500)):
        mp = m + M - 1
        L = ref.next_pow2(mp)
        if L == mp:
            continue
        assert engine.bluestein_length(m, M) == max(L, 32)
    with pytest.raises(ValueError, match="power of two"):
        engine.bluestein_length(5, 4)      # m + M - 1 = 8
    with pytest.raises(ValueError, match="2 output samples"):
        engine.bluestein_length(64, 1)


def test_per_entry_distances_are_sequences_and_1d_tensors():
    import torch

    from xlumina_gb300 import engine
    assert engine._per_entry([1e4, 2e4]) and engine._per_entry((1e4,)) and engine._per_entry(np.array([1e4]))
    assert engine._per_entry(torch.tensor([1e4, 2e4]))
    assert not engine._per_entry(1e4) and not engine._per_entry(np.float64(1e4))
    assert not engine._per_entry(torch.tensor(1e4))


def test_transfer_plane_policy(monkeypatch):
    import torch

    from xlumina_gb300 import engine
    cache = engine.TransferPlaneCache()
    built = []

    def fake_plane(k, x, y, z, wavelength):
        built.append(k)
        with engine._LOCK:
            cache._d.setdefault(k, object())
        return f"plane{len(built)}"

    monkeypatch.setattr(cache, "_plane", fake_plane)
    monkeypatch.setattr(torch.cuda, "current_device", lambda: 0)
    monkeypatch.setattr(torch.cuda, "is_current_stream_capturing", lambda: False)
    x, _ = ref.space(500.0, 64)
    xo, _ = ref.space(50.0, 32)
    assert cache.pair(x, x, xo, xo, 1e4, 0.633) == (None, None)        # first sight: in the kernels
    fin, fout = cache.pair(x, x, xo, xo, 1e4, 0.633)                   # second use: both planes
    assert fin is not None and fout is not None and len(built) == 2
    assert cache.pair(x, x, xo, xo, 2e4, 0.633) == (None, None)        # another distance starts over
    monkeypatch.setattr(torch.cuda, "is_current_stream_capturing", lambda: True)
    assert cache.pair(x, x, xo, xo, 2e4, 0.633) == (None, None)        # never built under capture
    assert len(built) == 2
