"""CPU checks of the C ABI library and of the host-side planning code.

No kernel runs here: the library must load and export every entry point that
include/xlgb.h declares, the ctypes mirrors must have the C layout, and the
host geometry must match the reference's formulas.
"""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import xlumina_ref as ref
from tests.conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "xlgb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(xl_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from xlumina_gb300 import _build, _lib
    _build.build()
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    from xlumina_gb300 import _lib
    names = _declared()
    assert "xl_rs_propagate" in names and "xl_last_error" in names
    for name in names:
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} declared in xlgb.h but not bound in _lib"


def test_ctypes_layouts():
    from xlumina_gb300 import _lib
    assert ctypes.sizeof(_lib.XlOp) == 96
    assert _lib.XlOp.dval.offset == 64
    assert ctypes.sizeof(_lib.XlProg) == 8 + 8 * 96
    assert _lib.XlRsArgs.inp.offset == 24
    assert _lib.XlRsArgs.pre.offset % 8 == 0


def test_size_helpers(lib):
    assert lib.xl_rs_spectrum_bytes(2048, 2048) == 4096 * 4096 * 8
    assert lib.xl_rs_spectrum_bytes(1000, 1000) == 2048 * 2048 * 8
    assert lib.xl_rs_work_bytes(8, 3, 2048, 2048) == 8 * 3 * 2048 * 4096 * 8
    assert lib.xl_rs_spectrum_bytes(10, 10) == 64 * 64 * 8     # the smallest transform, P = 64
    assert lib.xl_rs_spectrum_bytes(1, 10) == 0
    assert lib.xl_rs_spectrum_bytes(8192, 8192) == 0


def test_argument_errors_without_gpu(lib):
    from xlumina_gb300 import _lib
    a = _lib.XlRsArgs()
    a.batch, a.comps_in, a.comps_out, a.ny, a.nx = 1, 2, 2, 64, 64
    assert lib.xl_rs_propagate(None, ctypes.byref(a)) == _lib.XL_EINVAL
    assert b"comps_in/comps_out" in lib.xl_last_error()
    assert lib.xl_rs_stage(None, ctypes.byref(a), 7) == _lib.XL_EINVAL
    rc = lib.xl_rs_transfer_spectrum(None, 64, 64, None, None, 1.0, 0.5, 1.0, None, None)
    assert rc == _lib.XL_EINVAL


def test_wrapped_offsets_match_reference_grid():
    from xlumina_gb300 import engine
    for n in (5, 8, 63, 64):
        x, _ = ref.space(100.0, n)
        ext = ref.rs_offset_axis(x)
        P = 2 << engine.rs_logq(n, n)
        w = engine.rs_wrapped_offsets(x, P)
        for d in range(-(n - 1), n):
            assert w[d % P] == ext[d + n - 1]
        assert np.isnan(w).sum() == P - (2 * n - 1)


def test_quality_factor_and_lens_factors():
    from xlumina_gb300 import engine
    x, y = ref.space(150.0, 48)
    assert engine.quality_factor(x, y, 0.633, 2e3) == ref.rs_quality_factor(x, y, 0.633, 2e3)
    cf, rf, tc, tr = engine.lens_factors(x, y, 0.633, (120.0, 100.0), (2000.0, 2500.0))
    m = np.where((tc[None, :] + tr[:, None]) < 1, 1, 0) * (rf[:, None] * cf[None, :])
    assert np.max(np.abs(m - ref.lens_mask(x, y, 0.633, (120.0, 100.0), (2000.0, 2500.0)))) < 1e-12


def test_cuda_required_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from xlumina_gb300 import wave_optics
    with pytest.raises(RuntimeError, match="CUDA"):
        wave_optics.ScalarLight(np.linspace(-1, 1, 8), np.linspace(-1, 1, 8), 0.5).field


def test_bluestein_plan_matches_oracle_chirps():
    from xlumina_gb300 import engine
    for m, M, f1, f2, Dm in [(64, 48, -40.0, 40.0, 800.0), (2048, 1024, -1.0, 1.0, 3.4), (63, 3, 5.0, 6.0, 90.0)]:
        L, pre, g, post = engine.bluestein_plan(m, f1, f2, Dm, M)
        Lr, pre_r, g_r, post_r = ref.bluestein_vectors(m, f1, f2, Dm, M)
        assert L == max(Lr, 32)
        assert np.allclose(pre, pre_r, rtol=0, atol=1e-12)
        assert np.allclose(post * L, post_r, rtol=0, atol=1e-12)
        if L == Lr:
            assert np.allclose(g_r, g, rtol=0, atol=1e-9)


def test_bluestein_rejects_power_of_two_window():
    from xlumina_gb300 import engine
    with pytest.raises(ValueError, match="power of two"):
        engine.bluestein_plan(1024, -1.0, 1.0, 10.0, 1025)


def test_czt_argument_errors(lib):
    from xlumina_gb300 import _lib
    a = _lib.XlCztArgs()
    a.batch, a.comps_in, a.comps_out, a.mode, a.ny, a.nx, a.my, a.mx = 1, 2, 2, _lib.XL_CZT_VECTOR, 64, 64, 32, 32
    assert lib.xl_czt(None, ctypes.byref(a)) == _lib.XL_EINVAL
    a.comps_out = 3
    a.log2_lx, a.log2_ly = 6, 7   # 64 < 64 + 32
    assert lib.xl_czt(None, ctypes.byref(a)) == _lib.XL_EINVAL
    assert b"Bluestein" in lib.xl_last_error()


def test_philox_known_answers():
    """The table-noise generator against the Random123 known-answer vectors of
    Philox4x32-10, through the library (host code) and the oracle."""
    import ctypes

    from oracle import xlumina_ref as ref
    from xlumina_gb300 import _lib
    L = _lib.load()
    kat = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
           ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
           ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
            (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for ctr, key, want in kat:
        out = (ctypes.c_uint32 * 4)()
        assert L.xl_philox4x32_10((ctypes.c_uint32 * 4)(*ctr), (ctypes.c_uint32 * 2)(*key), out) == 0
        assert tuple(out) == want
        assert tuple(ref.philox4x32_10(ctr, key)) == want


def test_noise_keys():
    from xlumina_gb300 import noise
    k = noise.PRNGKey(42)
    assert k.tolist() == [0, 42]
    a, b = noise.split(k, 2), noise.split(k, 2)
    assert (a == b).all() and not (a[0] == a[1]).all()
    chain = noise.keychain_optical_tables(7, 3)
    assert chain.shape == (3, 2) and chain[:, 1].tolist() == [7, 8, 9]


def test_ctypes_mirrors_match_the_c_structs(lib):
    """Every argument struct the binding mirrors has the size the library was built with."""
    from xlumina_gb300 import _lib
    names = ("XlOp", "XlProg", "XlRsArgs", "XlCztArgs", "XlCztChirpArgs", "XlBsArgs", "XlNoiseArgs",
             "XlAdamWTensor", "XlAdamWArgs")
    for name in names:
        assert lib.xl_struct_size(name.encode()) == ctypes.sizeof(getattr(_lib, name)), name
    assert lib.xl_struct_size(b"NoSuchStruct") == 0
    src = open(os.path.join(ROOT, "include", "xlgb.h")).read()
    assert set(re.findall(r"}\s*(Xl[A-Za-z]+)\s*;", src)) == set(names)


def test_chirp_builder_argument_errors_without_gpu(lib):
    from xlumina_gb300 import _lib
    a = _lib.XlCztChirpArgs()
    a.batch, a.ny, a.nx, a.my, a.mx, a.log2_lx, a.log2_ly = 2, 64, 64, 32, 32, 7, 7
    assert lib.xl_czt_chirps(None, ctypes.byref(a)) == _lib.XL_EINVAL
    assert b"null pointer" in lib.xl_last_error()
    a.log2_lx = 6   # 64 < 64 + 32
    assert lib.xl_czt_chirps(None, ctypes.byref(a)) == _lib.XL_EINVAL
    assert b"Bluestein lengths" in lib.xl_last_error()
    c = _lib.XlCztArgs()
    c.batch, c.comps_in, c.comps_out, c.mode = 1, 1, 1, _lib.XL_CZT_PLAIN
    c.ny, c.nx, c.my, c.mx, c.log2_lx, c.log2_ly = 64, 64, 32, 32, 7, 7
    for f in ("pre_x", "g_x", "post_x", "pre_y", "g_y", "post_y", "work"):
        setattr(c, f, 16)
    c.z_batch = 16
    assert lib.xl_czt(None, ctypes.byref(c)) == _lib.XL_EINVAL
    assert b"per-entry distances" in lib.xl_last_error()
