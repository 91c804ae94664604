"""Noisy optical tables: shake_setup and its batched form
(optical_elements.py:2127-2301, examples/noisy_optimization.ipynb).

Keys are pairs of uint32 words, like jax's ``PRNGKey`` (``PRNGKey(seed)`` is
``[0, seed]``); ``split`` derives new keys with the same counter-based
generator the noise kernel uses (Philox4x32-10, ``xl_philox4x32_10``).  The
noise itself is drawn on the device for every table at once
(``xl_table_noise``), with the reference's shapes, ranges and sign
conventions; the values are not jax's streams.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib, engine, um

_SPLIT_TAG = 0x53504C54   # counter word 3 of a key split

# (misalignment min, max) in um, (phase / amplitude noise min, max): optical_elements.py:2160-2190
NOISE_LEVELS = {
    "low": ((10 * um, 50 * um), (0.01, 0.05)),
    "mild": ((50 * um, 500 * um), (0.05, 0.5)),
    "high": ((500 * um, 1000 * um), (0.5, 1.0)),
    "all": ((10 * um, 1000 * um), (0.01, 1.0)),
}


def PRNGKey(seed: int) -> np.ndarray:
    """A key from an integer seed: [high word, low word], as jax.random.PRNGKey."""
    seed = int(seed)
    return np.array([(seed >> 32) & 0xFFFFFFFF, seed & 0xFFFFFFFF], dtype=np.uint32)


def philox(counter, key) -> np.ndarray:
    """Philox4x32-10 of a 4-word counter and a 2-word key (libxlgb, on the host)."""
    c = (ctypes.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in counter])
    k = (ctypes.c_uint32 * 2)(*[int(v) & 0xFFFFFFFF for v in np.asarray(key).ravel()[:2]])
    out = (ctypes.c_uint32 * 4)()
    _lib.check(engine.lib().xl_philox4x32_10(c, k, out), "xl_philox4x32_10")
    return np.array(list(out), dtype=np.uint32)


def split(key, num: int = 2) -> np.ndarray:
    """``num`` new keys from ``key`` (shape (num, 2))."""
    return np.stack([philox((i, 0, 0, _SPLIT_TAG), key)[:2] for i in range(num)])


def keychain_optical_tables(seed: int, number_of_tables: int) -> np.ndarray:
    """One key per optical table, PRNGKey(seed + table) (examples/noisy_optimization.ipynb)."""
    return np.stack([PRNGKey(seed + t) for t in range(number_of_tables)])


def _ranges(NS):
    level = NS["noise_level"]
    if level == "tunable":
        return tuple(NS["misalignment"]), tuple(NS["phase_noise"])
    if level not in NOISE_LEVELS:
        raise ValueError(f"unknown noise level {level!r}")
    return NOISE_LEVELS[level]


def table_noise(keys, resolution: int, NS: dict):
    """Noise for every key in ``keys`` (shape (T, 2)) in one launch: (distances
    (T, n_d) float64, slms (T, 2 n_sslm, R, R) float32, wps (T, 2 n_wps)
    float64, amps (T, 2 n_sslm, R, R) float32), device tensors."""
    keys = np.ascontiguousarray(np.asarray(keys, dtype=np.uint32).reshape(-1, 2))
    T = keys.shape[0]
    if T > _lib.XL_NOISE_MAX_TABLES:
        raise ValueError(f"at most {_lib.XL_NOISE_MAX_TABLES} tables per call")
    (dmin, dmax), (pmin, pmax) = _ranges(NS)
    nd, ns, nw = int(NS["number of distances"]), int(NS["number of sSLM"]), int(NS["number of wps"])
    dev = engine.device()
    dist = torch.empty((T, nd), dtype=torch.float64, device=dev)
    slms = torch.empty((T, 2 * ns, resolution, resolution), dtype=torch.float32, device=dev)
    amps = torch.empty_like(slms)
    wps = torch.empty((T, 2 * nw), dtype=torch.float64, device=dev)
    a = _lib.XlNoiseArgs()
    a.tables, a.resolution, a.planes = T, int(resolution), 2 * ns
    a.n_distances, a.n_wps = nd, 2 * nw
    a.min_d, a.max_d, a.min_phase, a.max_phase = float(dmin), float(dmax), float(pmin), float(pmax)
    a.discretize = 1 if NS.get("discretize", False) else 0
    a.distances, a.slms, a.amps, a.wps = dist.data_ptr(), slms.data_ptr(), amps.data_ptr(), wps.data_ptr()
    kp = keys.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    _lib.check(engine.lib().xl_table_noise(engine.stream_handle(), ctypes.byref(a), kp), "xl_table_noise")
    return dist, slms, wps, amps


def _noise_key(key):
    """shake_setup's split (optical_elements.py:2153): key0 (the next key) and
    the key the noise is drawn from."""
    ks = split(key, 2)
    return ks[0], ks[1]


def shake_setup(key, resolution: int, NS: dict):
    """optical_elements.py:2127-2217: noise for one table; returns
    (distances, slms, wps, amps, key0, key)."""
    key = np.asarray(key, dtype=np.uint32).reshape(2)
    key0, kn = _noise_key(key)
    d, s, w, a = table_noise(kn[None], resolution, NS)
    return d[0], s[0], w[0], a[0], key0, key


# the noise settings shake_setup_jit reads, as the reference's global
NS: dict = {}


def shake_setup_jit(key, resolution: int):
    """optical_elements.py:2219-2301: shake_setup with the module's ``NS``."""
    return shake_setup(key, resolution, NS)


def batch_shake_setup(key_array, array_for_shape, settings: dict = None):
    """Noise for every table of ``key_array`` (examples/noisy_optimization.ipynb),
    drawn in one launch: (distances (T, n_d), slms (T, 2 n_sslm, R, R),
    wps (T, 2 n_wps), amps (T, 2 n_sslm, R, R), next keys (T, 2), keys)."""
    keys = np.asarray(key_array, dtype=np.uint32).reshape(-1, 2)
    R = int(np.shape(array_for_shape)[0])
    pairs = [_noise_key(k) for k in keys]
    key0 = np.stack([p[0] for p in pairs])
    kn = np.stack([p[1] for p in pairs])
    d, s, w, a = table_noise(kn, R, NS if settings is None else settings)
    return d, s, w, a, key0, keys
