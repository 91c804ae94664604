"""A reference-style optical table through the ``xlumina`` import alias.

The table below is written the way experiments/four_f_optical_table.py:36-127
writes its 4f batch table: star-imports from ``xlumina.wave_optics``,
``SLM`` from ``xlumina.optical_elements``, ``space`` from
``xlumina.toolbox``, the units from ``xlumina.__init__``.  Its array code
uses torch where the reference uses jax.numpy, and a leading batch
dimension where it uses vmap.  It runs on the package's kernels and agrees
with the FP64 oracle (rel-L2 1e-5)."""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_reference_style_table_runs_through_the_alias():
    import torch

    import xlumina_gb300.alias  # noqa: F401  (registers xlumina.*)
    from xlumina.__init__ import cm, nm, um
    from xlumina.optical_elements import SLM
    from xlumina.toolbox import space
    from xlumina.wave_optics import LightSource

    from oracle import xlumina_ref as ref

    wavelength = 632.8 * nm
    x, y = space(300 * um, 128)
    shape = 128
    input_light = LightSource(x, y, wavelength)
    input_light.gaussian_beam(w0=(120 * um, 120 * um), E0=1)

    def batch_dual_slm_4f(input_masks, parameters):
        offset = 1.2
        light = LightSource(x, y, wavelength)
        light.field = input_light.field * input_masks
        stage0, _ = light.RS_propagation(z=(torch.abs(parameters[0]) * 100 + offset).item() * cm)
        mod1, _ = SLM(stage0, parameters[3] * (2 * np.pi) - np.pi, shape)
        stage1, _ = mod1.RS_propagation(z=(torch.abs(parameters[1]) * 100 + offset).item() * cm)
        mod2, _ = SLM(stage1, parameters[4] * (2 * np.pi) - np.pi, shape)
        out, _ = mod2.RS_propagation(z=(torch.abs(parameters[2]) * 100 + offset).item() * cm)
        return torch.abs(out.field) ** 2

    rng = np.random.default_rng(9)
    masks = (rng.uniform(0, 1, (2, shape, shape)) > 0.5).astype(np.float32)
    zs = rng.uniform(0, 0.01, 3)
    p3, p4 = rng.uniform(0, 1, (shape, shape)), rng.uniform(0, 1, (shape, shape))
    params = [torch.tensor(v) for v in zs] + [torch.as_tensor(p3, dtype=torch.float32, device="cuda"),
                                               torch.as_tensor(p4, dtype=torch.float32, device="cuda")]
    got = batch_dual_slm_4f(torch.as_tensor(masks, device="cuda"), params).cpu().numpy()
    assert got.shape == (2, shape, shape)
    src = ref.gaussian_beam(x, y, wavelength, (120.0, 120.0))
    ph3 = p3.astype(np.float32).astype(np.float64) * 2 * np.pi - np.pi
    ph4 = p4.astype(np.float32).astype(np.float64) * 2 * np.pi - np.pi
    for b in range(2):
        u = src.astype(np.complex64).astype(np.complex128) * masks[b]
        u = ref.rs_propagate(u, x, y, wavelength, (abs(zs[0]) * 100 + 1.2) * 1e4)
        u = ref.rs_propagate(ref.slm(u, ph3)[0], x, y, wavelength, (abs(zs[1]) * 100 + 1.2) * 1e4)
        u = ref.rs_propagate(ref.slm(u, ph4)[0], x, y, wavelength, (abs(zs[2]) * 100 + 1.2) * 1e4)
        assert rel_l2(got[b], np.abs(u) ** 2) < 1e-5
