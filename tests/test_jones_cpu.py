"""The host-side pieces of the API against golden fixtures made from the
reference's own source: the Jones matrix constructors
(optical_elements.py:109-180), the scalar SLM phase (:76-85), the
single-input splitter ports (:393-409), and the amplitude, phase and area
losses (loss_functions.py:42-135).  They build 2x2 matrices and reduce small
arrays on the host, so they run without a GPU.
Bars: complex64 matrices 1e-6, float64 values 1e-12 (the area loss 1e-9
relative)."""
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


def test_amplitude_phase_and_area_losses_match_the_reference():
    """MSE_Amplitude, MSE_Phase (loss_functions.py:109-135), their per-component
    forms vMSE_Amplitude, vMSE_Phase (:61-91) and vectorized_loss_hybrid
    (:42-50) on host tensors against the reference's outputs (float64)."""
    import types

    import torch

    import xlumina_gb300.loss_functions as lf
    g = golden("losses_more")
    a3, b3 = torch.as_tensor(g["a3"]), torch.as_tensor(g["b3"])
    assert abs(float(lf.MSE_Amplitude(a3[0], b3[0])) - float(g["mse_amplitude"])) < 1e-12
    assert abs(float(lf.MSE_Phase(a3[0], b3[0])) - float(g["mse_phase"])) < 1e-12
    la = types.SimpleNamespace(Ex=a3[0], Ey=a3[1], Ez=a3[2])
    lb = types.SimpleNamespace(Ex=b3[0], Ey=b3[1], Ez=b3[2])
    assert np.abs(lf.vMSE_Amplitude(la, lb).numpy() - g["vmse_amplitude"]).max() < 1e-12
    assert np.abs(lf.vMSE_Phase(la, lb).numpy() - g["vmse_phase"]).max() < 1e-12
    got = lf.vectorized_loss_hybrid(torch.as_tensor(g["I6"])).numpy()
    assert np.abs(got - g["loss_hybrid"]).max() < 1e-9 * np.abs(g["loss_hybrid"]).max()
