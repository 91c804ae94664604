"""The Jones matrix constructors (optical_elements.py:109-180), the scalar
SLM phase (:76-85) and the single-input splitter ports (:393-409) against
the golden fixture made from the reference's own source.  These build 2x2
matrices and small arrays on the host, so they run without a GPU.
Bars: complex64 matrices 1e-6, float64 arrays 1e-12."""
import numpy as np

from oracle import xlumina_ref as ref
from tests.conftest import golden


def _np(t):
    return np.asarray(t.numpy() if hasattr(t, "numpy") else t).astype(np.complex128)


def test_jones_matrices_match_the_reference():
    import xlumina_gb300.optical_elements as oe
    g = golden("jones")
    al, ph, et, th, de = (float(g[k]) for k in ("alpha", "phi", "eta", "theta", "delta"))
    a1, a2 = float(g["a1"]), float(g["a2"])
    got = {"lp": oe.jones_LP(al), "retarder": oe.jones_general_retarder(et, th, de),
           "sslm": oe.jones_sSLM(al, ph), "sslm_amp": oe.jones_sSLM_with_amplitude(al, ph, a1, a2),
           "lcd": oe.jones_LCD(et, th)}
    for k, v in got.items():
        assert tuple(v.shape) == (2, 2), k
        assert np.abs(_np(v) - g[k]).max() < 1e-6, k


def test_oracle_retarder_matches_the_reference():
    g = golden("jones")
    want = g["retarder"]
    # the oracle returns the entries (J00, J01, J10, J11)
    got = np.asarray(ref.jones_retarder(float(g["eta"]), float(g["theta"]), float(g["delta"]))).reshape(2, 2)
    assert np.abs(got - want).max() < 1e-12
    got = np.asarray(ref.jones_retarder(float(g["eta"]), float(g["theta"]))).reshape(2, 2)
    assert np.abs(got - g["lcd"]).max() < 1e-12


def test_scalar_slm_phase_and_splitter_ports():
    import xlumina_gb300.optical_elements as oe
    g = golden("jones")
    assert np.abs(oe.phase_scalar_SLM(g["phase_plane"]) - g["slm_phase"]).max() < 1e-12
    z = np.zeros_like(g["aEx"])
    T, R = float(g["T"]), float(g["R"])
    for fn, key in ((oe.bs_port0, "port0"), (oe.bs_port1, "port1")):
        out = np.stack(fn(g["aEx"], g["aEy"], z, z, z, z, T, R))
        assert np.abs(out - g[key]).max() < 1e-12, key
