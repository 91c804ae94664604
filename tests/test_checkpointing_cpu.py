"""The wavefront checkpoint policy of the deep tables (no GPU needed)."""
import pytest

from xlumina_gb300.checkpointing import CheckpointPolicy


def test_segments_of_k_wavefronts():
    assert CheckpointPolicy(1).segments([2, 4, 6, 4, 2], 100) == [(k, k + 1, True) for k in range(5)]
    assert CheckpointPolicy(2).segments([2, 4, 6, 4, 2], 100) == [(0, 2, True), (2, 4, True), (4, 5, True)]
    assert CheckpointPolicy(9).segments([2, 4, 6], 100) == [(0, 3, True)]


def test_budget_keeps_leading_wavefronts_unchecked():
    # kept bytes per wavefront: 3 * lights * 100 -> 600, 1200, 1800, ...
    p = CheckpointPolicy(every=2, budget_bytes=2000)
    assert p.segments([2, 4, 6, 4, 2], 100) == [(0, 2, False), (2, 4, True), (4, 5, True)]
    assert CheckpointPolicy(every=3, budget_bytes=10 ** 9).segments([2, 4], 100) == [(0, 2, False)]
    assert CheckpointPolicy(every=1, budget_bytes=0).segments([2, 4], 100) == [(0, 1, True), (1, 2, True)]


def test_coerce_and_validation():
    assert CheckpointPolicy.coerce(False) is None and CheckpointPolicy.coerce(None) is None
    assert CheckpointPolicy.coerce(True) == CheckpointPolicy(1)
    assert CheckpointPolicy.coerce(3) == CheckpointPolicy(3)
    p = CheckpointPolicy(2, 1e6)
    assert CheckpointPolicy.coerce(p) is p
    with pytest.raises(ValueError):
        CheckpointPolicy(0)
    with pytest.raises(TypeError):
        CheckpointPolicy.coerce("yes")
