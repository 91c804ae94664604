"""The device FFT engine's pass code, run on the CPU, against numpy's FFT."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def fftlib(tmp_path_factory):
    out = tmp_path_factory.mktemp("fftcore") / "libfftcore.so"
    src = os.path.join(HERE, "native", "fft_core_check.cpp")
    subprocess.check_call(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", src, "-o", str(out)])
    lib = ctypes.CDLL(str(out))
    lib.fft_core_check.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.fft_core_check_stw.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.fft_core_check_zu.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.fft_pair_check.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 4
    lib.fft64_check.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    return lib


@pytest.mark.parametrize("logn", range(4, 14))
@pytest.mark.parametrize("direction", [-1, 1])
@pytest.mark.parametrize("tables", ["global", "shared"])
@pytest.mark.parametrize("elems", [16, 8])
def test_block_fft_matches_numpy(fftlib, logn, direction, tables, elems):
    n = 1 << logn
    rng = np.random.default_rng(logn * 7 + (direction > 0))
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    out = np.empty_like(x)
    fftlib.fft_core_set_e(elems)
    fn = fftlib.fft_core_check if tables == "global" else fftlib.fft_core_check_stw
    assert fn(logn, direction, x.ctypes.data, out.ctypes.data) == 0
    ref = np.fft.fft(x.astype(np.complex128)) if direction < 0 else np.fft.ifft(x.astype(np.complex128)) * n
    err = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert err < 2e-7 * logn, err


@pytest.mark.parametrize("logn", range(5, 14))
@pytest.mark.parametrize("direction", [-1, 1])
def test_zero_padded_fft_matches_numpy(fftlib, logn, direction):
    """The pruned first pass of a line whose upper half is zero (the propagators'
    zero padding): only the lower half is read, the result is the full FFT."""
    n = 1 << logn
    rng = np.random.default_rng(100 + logn)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    garbage = x.copy()
    garbage[n // 2:] = 1e30   # never read
    x[n // 2:] = 0
    out = np.empty_like(x)
    assert fftlib.fft_core_check_zu(logn, direction, garbage.ctypes.data, out.ctypes.data) == 0
    ref = np.fft.fft(x.astype(np.complex128)) if direction < 0 else np.fft.ifft(x.astype(np.complex128)) * n
    err = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert err < 2e-7 * logn, err


@pytest.mark.parametrize("logn", range(5, 14))
@pytest.mark.parametrize("direction", [-1, 1])
@pytest.mark.parametrize("pruned", [False, True])
def test_pair_fft_matches_numpy(fftlib, logn, direction, pruned):
    """The packed two-line engine (fft_pair.cuh): two independent lines per
    thread, each against numpy, with and without the pruned first pass."""
    n = 1 << logn
    rng = np.random.default_rng(300 + logn + 20 * pruned)
    a = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    b = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    ga, gb = a.copy(), b.copy()
    if pruned:
        a[n // 2:] = 0
        b[n // 2:] = 0
        ga[n // 2:] = 1e30   # never read
        gb[n // 2:] = -1e30
    oa, ob = np.empty_like(a), np.empty_like(b)
    assert fftlib.fft_pair_check(logn, direction, int(pruned), ga.ctypes.data, gb.ctypes.data,
                                 oa.ctypes.data, ob.ctypes.data) == 0
    for x, out in ((a, oa), (b, ob)):
        ref = np.fft.fft(x.astype(np.complex128)) if direction < 0 else np.fft.ifft(x.astype(np.complex128)) * n
        err = np.linalg.norm(out - ref) / np.linalg.norm(ref)
        assert err < 2e-7 * logn, err


@pytest.mark.parametrize("direction", [-1, 1])
@pytest.mark.parametrize("zin,zout", [(False, False), (True, False), (False, True), (True, True)])
def test_radix64_fft_matches_numpy(fftlib, direction, zin, zout):
    """The radix-64 4096-point engine (fft64.cuh): 64 threads of 64 elements,
    one exchange; pruned input (upper half zero, never read) and pruned output
    (only the lower half produced)."""
    n = 4096
    rng = np.random.default_rng(500 + direction + 3 * zin + 7 * zout)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    g = x.copy()
    if zin:
        x[n // 2:] = 0
        g[n // 2:] = 1e30   # never read
    out = np.full_like(x, 7.0)
    assert fftlib.fft64_check(direction, int(zin), int(zout), g.ctypes.data, out.ctypes.data) == 0
    ref = np.fft.fft(x.astype(np.complex128)) if direction < 0 else np.fft.ifft(x.astype(np.complex128)) * n
    keep = n // 2 if zout else n
    err = np.linalg.norm(out[:keep] - ref[:keep]) / np.linalg.norm(ref[:keep])
    assert err < 2e-7 * 12, err
    if zout:
        assert np.all(out[keep:] == 7.0)


def test_radix64_exchange_is_conflict_free(fftlib):
    """Every half-warp write and gather of the radix-64 exchange (four lines
    interleaved in the lanes) touches 16 distinct 8-byte bank pairs."""
    assert fftlib.fft64_min_banks() == 16
