"""Host logic of the serving loop (no kernel runs): which requests may share
a batched launch.  Requests of one kind and grid share one whatever their
distances (RS / VRS through stacked transfer spectra, chirp-z through
per-entry chirps); a different grid, output window or wavelength starts a new
batch."""
import numpy as np

from oracle import xlumina_ref as ref


def _req(kind, z, n=64, wl=0.633, m=32, roi=50.0):
    from xlumina_gb300.serving import Request
    x, y = ref.space(500.0, n)
    xo, yo = ref.space(roi, m)
    if kind == "czt":
        return Request(kind, [None], x, y, wl, z, xout=xo, yout=yo)
    return Request(kind, [None], x, y, wl, z)


def test_distances_do_not_split_batches():
    for kind in ("rs", "vrs", "czt", "grad"):
        keys = {_req(kind, z).key() for z in (1e4, 5e4, 1.9e5)}
        assert len(keys) == 1, kind


def test_grid_window_and_wavelength_split_batches():
    base = _req("czt", 1e4).key()
    assert _req("czt", 1e4, n=96).key() != base
    assert _req("czt", 1e4, m=40).key() != base
    assert _req("czt", 1e4, roi=60.0).key() != base
    assert _req("czt", 1e4, wl=0.532).key() != base
    assert _req("rs", 1e4).key() != _req("vrs", 1e4).key()


def test_request_class_is_kind_and_size():
    from xlumina_gb300.serving import request_class
    assert request_class(_req("czt", 1e4)) == ("czt", 64, 64)
    assert request_class(_req("rs", 2e4, n=128)) == ("rs", 128, 128)
    assert np.isfinite(_req("vrs", 1e4).nbytes())


def test_a_served_request_cannot_be_resubmitted():
    """A request's future completes once; submitting it again is refused on
    the client side (the scheduler thread never sees it)."""
    import numpy as np
    import pytest

    from xlumina_gb300.serving import Request, Server
    r = Request("rs", [], np.zeros(4), np.zeros(4), 0.5, 1.0)
    r.future.set_result(None)
    srv = Server.__new__(Server)     # the client-side check needs no device
    with pytest.raises(ValueError):
        Server.submit(srv, r)
