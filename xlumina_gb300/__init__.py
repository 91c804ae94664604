"""xlumina_gb300 -- XLuminA's light-propagation path on GB300 (sm_103a).

Same module and class names as the reference package (``wave_optics``,
``vectorized_optics``, ``optical_elements``, ``toolbox``, ``loss_functions``)
and the same units (xlumina/__init__.py:14-20): lengths in microns, angles in
radians.  Fields are complex64 torch tensors on the CUDA device; every
propagator and mask runs in libxlgb.so (hand-written sm_103a kernels).
"""
import math

um = 1
nm = 1e-3
mm = 1e3
cm = 1e4

radians = 1
degrees = 180 / math.pi

__version__ = "0.1.0"
