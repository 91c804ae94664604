"""A numpy-backed stand-in for the parts of ``jax`` (0.4.33) that XLuminA imports.

Test infrastructure only.  It lets ``make_golden.py`` import and run the
reference package's own Python source in a container that has no jax: every
``jax.numpy`` call goes to numpy in float64/complex128 (the reference forces
``jax_enable_x64`` at import, so this is the precision it computes in), ``jit``
is the identity, ``vmap`` is a Python loop over the mapped axis, and
``jnp.fromfunction`` evaluates its function once per index pair, as jax's
vmap-based implementation does (numpy's own ``fromfunction`` passes whole index
arrays instead, which is not what the reference's Jones-matrix code expects).
FFTs run in numpy's pocketfft instead of XLA's DUCC; both are float64-accurate.

Nothing in the product imports this module.
"""
from __future__ import annotations

import sys
import types

import numpy as np
import scipy.special


class AtArray(np.ndarray):
    """ndarray with jax's functional ``x.at[idx].set(v)`` update syntax."""

    @property
    def at(self):
        arr = self

        class _Idx:
            def __getitem__(self, idx):
                class _Upd:
                    def set(self, value):
                        out = np.array(arr, copy=True).view(AtArray)
                        out[idx] = value
                        return out

                    def add(self, value):
                        out = np.array(arr, copy=True).view(AtArray)
                        out[idx] += value
                        return out

                return _Upd()

        return _Idx()


def _zeros(shape, dtype=float):
    return np.zeros(shape, dtype=dtype).view(AtArray)


def _fromfunction(function, shape, dtype=int, **kwargs):
    """Per-element evaluation, stacking each result's own shape after ``shape``."""
    shape = tuple(int(s) for s in shape)
    first = None
    out = None
    for idx in np.ndindex(*shape):
        val = np.asarray(function(*[dtype(i) for i in idx], **kwargs))
        if first is None:
            first = val
            out = np.empty(shape + val.shape, dtype=np.result_type(val.dtype, np.complex128)
                           if np.iscomplexobj(val) else val.dtype)
        out[idx] = val
    return out


def _array(obj, dtype=None, **kw):
    """``jnp.array`` on nested lists of scalars/arrays (the Jones matrices)."""
    if isinstance(obj, (list, tuple)):
        flat = []

        def _walk(o):
            if isinstance(o, (list, tuple)):
                for e in o:
                    _walk(e)
            else:
                flat.append(np.asarray(o))

        _walk(obj)
        bshape = np.broadcast_shapes(*[f.shape for f in flat]) if flat else ()
        if bshape != ():
            def _bcast(o):
                if isinstance(o, (list, tuple)):
                    return [_bcast(e) for e in o]
                return np.broadcast_to(np.asarray(o), bshape)

            obj = _bcast(obj)
    return np.array(obj, dtype=dtype)


def _vmap(fun, in_axes=0, out_axes=0):
    def mapped(*args):
        axes = in_axes if isinstance(in_axes, (list, tuple)) else (in_axes,) * len(args)
        size = None
        for a, ax in zip(args, axes):
            if ax is not None:
                size = np.shape(a)[ax]
                break
        results = []
        for b in range(size):
            call = [np.take(a, b, axis=ax) if ax is not None else a for a, ax in zip(args, axes)]
            results.append(fun(*call))
        if isinstance(results[0], tuple):
            return tuple(np.stack([r[i] for r in results], axis=0) for i in range(len(results[0])))
        return np.stack(results, axis=0)

    return mapped


def _jit(fun=None, **kwargs):
    if fun is None:
        return lambda f: f
    return fun


def install() -> None:
    """Register the stand-in modules in ``sys.modules`` (jax, matplotlib, h5py, PIL)."""
    jnp = types.ModuleType("jax.numpy")

    def _getattr(name):
        return getattr(np, name)

    jnp.__getattr__ = _getattr  # type: ignore[attr-defined]
    jnp.zeros = _zeros
    jnp.fromfunction = _fromfunction
    jnp.array = _array
    jnp.fft = np.fft
    jnp.linalg = np.linalg
    jnp.pi = np.pi

    jax = types.ModuleType("jax")
    jax.numpy = jnp
    jax.jit = _jit
    jax.vmap = _vmap

    class _Config:
        def update(self, *a, **k):
            pass

    jax.config = _Config()
    lax = types.ModuleType("jax.lax")
    lax.cond = lambda pred, t, f, *ops: t(*ops) if pred else f(*ops)
    jax.lax = lax
    nn = types.ModuleType("jax.nn")
    nn.logsumexp = scipy.special.logsumexp
    jax.nn = nn
    jax.random = types.ModuleType("jax.random")

    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    h5py = types.ModuleType("h5py")
    pil = types.ModuleType("PIL")
    pil.Image = types.ModuleType("PIL.Image")

    sys.modules.update({
        "jax": jax, "jax.numpy": jnp, "jax.lax": lax, "jax.nn": nn,
        "jax.random": jax.random, "matplotlib": mpl, "matplotlib.pyplot": plt,
        "h5py": h5py, "PIL": pil, "PIL.Image": pil.Image,
    })
