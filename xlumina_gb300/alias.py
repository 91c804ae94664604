"""Import the package under the reference's name.

``import xlumina_gb300.alias`` registers ``xlumina`` and its submodules
(``xlumina.wave_optics``, ``xlumina.vectorized_optics``,
``xlumina.optical_elements``, ``xlumina.toolbox``, ``xlumina.loss_functions``)
as names of this package's modules, with the reference's unit constants on
``xlumina`` itself (xlumina/__init__.py:14-20).  An optical table written
against the reference's modules (experiments/*.py) then imports unchanged.

What does not carry over is jax itself: a table's own array code uses torch
in place of ``jax.numpy`` (``torch.abs`` for ``jnp.abs``), a leading batch
dimension in place of ``vmap``, nothing in place of ``jit``, and torch
autograd in place of ``jax.grad``.
"""
from __future__ import annotations

import sys
import types

from . import loss_functions, optical_elements, toolbox, vectorized_optics, wave_optics
from . import cm, degrees, mm, nm, radians, um

_MODULES = {"wave_optics": wave_optics, "vectorized_optics": vectorized_optics,
            "optical_elements": optical_elements, "toolbox": toolbox, "loss_functions": loss_functions}


def install() -> types.ModuleType:
    """Register the alias (idempotent); returns the ``xlumina`` module."""
    pkg = sys.modules.get("xlumina")
    if pkg is None or not getattr(pkg, "_is_xlumina_gb300_alias", False):
        pkg = types.ModuleType("xlumina", "xlumina_gb300 under the reference package's name")
        pkg.__path__ = []
        pkg._is_xlumina_gb300_alias = True
        for k, v in dict(um=um, nm=nm, mm=mm, cm=cm, radians=radians, degrees=degrees).items():
            setattr(pkg, k, v)
        sys.modules["xlumina"] = pkg
    for name, mod in _MODULES.items():
        sys.modules[f"xlumina.{name}"] = mod
        setattr(pkg, name, mod)
    # the reference's experiments import the units from xlumina.__init__
    sys.modules["xlumina.__init__"] = pkg
    return pkg


install()
