"""Host helpers of the reference's API against values the reference's own
source produced (tests/golden/host_helpers.npz): build_CZT_grid
(wave_optics.py:299-331) and the minimum trustworthy RS / VRS distances
(wave_optics.py:198-231, vectorized_optics.py:286-319), which print the
distance and return None."""
import contextlib
import io

import numpy as np
import pytest

from tests.conftest import golden


def _printed(fn):
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        ret = fn()
    return ret, buf.getvalue()


@pytest.mark.parametrize("case", [0, 1])
def test_build_czt_grid_matches_reference(case):
    from xlumina_gb300 import wave_optics as wo
    g = golden("host_helpers")
    k = f"g{case}_"
    out = wo.build_CZT_grid(float(g[k + "z"]), float(g[k + "wl"]), g[k + "xin"], g[k + "yin"], g[k + "xo"],
                            g[k + "yo"])
    nx, ny, dx, dy, Xo, Yo, Dm, fy1, fy2, fx1, fx2 = out
    np.testing.assert_allclose([nx, ny, dx, dy, Dm, fy1, fy2, fx1, fx2], g[k + "scal"], rtol=1e-14, atol=0)
    np.testing.assert_array_equal(Xo, g[k + "Xo"])
    np.testing.assert_array_equal(Yo, g[k + "Yo"])


def test_minimum_distances_match_reference():
    from xlumina_gb300.vectorized_optics import VectorizedLight
    from xlumina_gb300.wave_optics import ScalarLight
    from xlumina_gb300 import toolbox as tb
    g = golden("host_helpers")
    for h, n, wl, nidx, qf, zs, zv in g["minz"]:
        x, y = tb.space(h, int(n))
        ret, text = _printed(lambda: ScalarLight(x, y, wl).get_RS_minimum_z(n=nidx, quality_factor=qf))
        assert ret is None and text.startswith("Minimum distance to propagate (in microns):")
        assert float(text.split(":")[-1]) == pytest.approx(zs, rel=1e-12, abs=0)
        ret, text = _printed(lambda: VectorizedLight(x, y, wl).get_VRS_minimum_z(n=nidx, quality_factor=qf))
        assert ret is None and text.startswith("Minimum distance to propagate (in um):")
        assert float(text.split(":")[-1]) == pytest.approx(zv, rel=1e-12, abs=0)
    assert any(row[5] == 0 for row in g["minz"])   # the factor <= 0 branch is covered
