"""Cylindrical and axicon lenses and the geometric masks
(optical_elements.py:705-889) on the device against the reference's own
outputs (tests/golden/lenses_masks.npz).  Masks exact; fields rel-L2 1e-6."""
import numpy as np
import pytest

from tests.conftest import golden, rel_l2

pytestmark = pytest.mark.gpu


def test_lenses_and_masks_match_golden():
    import torch

    import xlumina_gb300.optical_elements as oe
    import xlumina_gb300.vectorized_optics as vo
    import xlumina_gb300.wave_optics as wo
    g = golden("lenses_masks")
    x, y = g["x"], g["y"]
    sl = wo.ScalarLight(x, y, 0.6)
    sl.field = torch.as_tensor(g["source"].astype(np.complex64), device="cuda")
    vl = vo.VectorizedLight(x, y, 0.6)
    vl.Ex, vl.Ey, vl.Ez = (torch.as_tensor(g[k].astype(np.complex64), device="cuda") for k in ("vEx", "vEy", "vEz"))

    cyl_s, cyl_mask = oe.cylindrical_lens(sl, 5000.0, 1.5, angle=0.4)
    assert rel_l2(cyl_mask.cpu().numpy(), g["cyl_mask"]) < 1e-6
    assert rel_l2(cyl_s.field.cpu().numpy(), g["cyl_scalar"]) < 1e-6
    cyl_v, _ = oe.cylindrical_lens(vl, 5000.0, 1.5, angle=0.4)
    for c in ("Ex", "Ey"):
        assert rel_l2(getattr(cyl_v, c).cpu().numpy(), g[f"cyl_{c}"]) < 1e-6
    assert not torch.any(cyl_v.Ez) and not np.any(g["cyl_Ez"])
    ax_s, ax_mask = oe.axicon_lens(sl, 0.02, 1.45)
    assert rel_l2(ax_mask.cpu().numpy(), g["ax_mask"]) < 1e-6
    assert rel_l2(ax_s.field.cpu().numpy(), g["ax_scalar"]) < 1e-6
    ax_v, _ = oe.axicon_lens(vl, 0.02, 1.45)
    for c in ("Ex", "Ey"):
        assert rel_l2(getattr(ax_v, c).cpu().numpy(), g[f"ax_{c}"]) < 1e-6
    assert not torch.any(ax_v.Ez)

    X, Y = sl.X, sl.Y
    assert np.array_equal(oe.triangular_mask(X, Y, (10.0, 60.0), 20.0, 1.2, 150.0).cpu().numpy(), g["triangle"])
    assert np.array_equal(oe.rectangular_mask(X, Y, (15.0, -10.0), 180.0, 90.0, 30.0).cpu().numpy(), g["rectangle"])
    assert np.array_equal(oe.annular_aperture(100.0, 300.0, X, Y).cpu().numpy(), g["annulus"])
    fa = oe.forked_grating(X, Y, (5.0, 5.0), 10.0, 60.0, 2, kind='Amplitude')
    assert np.array_equal(fa.cpu().numpy(), g["forked_amplitude"])
    fp = oe.forked_grating(X, Y, (5.0, 5.0), 10.0, 60.0, 2, kind='Phase')
    assert np.abs(fp.cpu().numpy() - g["forked_phase"]).max() < 1e-12


def test_synthetic_data_and_device_loader(tmp_path):
    """The synthetic 4f data (experiments/generate_synthetic_data.py): a target
    is 0.25 x the input mask at twice the size; the loader hands out CUDA
    tensors prefetched on a side stream."""
    import torch

    import xlumina_gb300.optical_elements as oe
    from xlumina_gb300 import datasets
    X, Y = datasets._grid(128)
    rng = np.random.default_rng(3)
    ins, outs = datasets.generate_synthetic_circles(X, Y, 2, rng)
    rng = np.random.default_rng(3)
    r1, r2 = rng.uniform(100, 1000), rng.uniform(100, 1000)
    assert torch.equal(ins[0], oe.circular_mask(X, Y, (r1, r2)))
    assert torch.equal(outs[0], 0.25 * oe.circular_mask(X, Y, (2 * r1, 2 * r2)))
    paths = datasets.generate_synthetic_files(str(tmp_path), n_files=2, num_samples=4, n=128, seed=1)
    assert len(paths) == 2
    loader = datasets.MultiHDF5DataLoader(str(tmp_path), batch_size=5, seed=2)
    a, b = next(loader)
    assert a.is_cuda and b.is_cuda and a.shape == (5, 128, 128)
    assert torch.all((b == 0) | (b == 0.25))
    loader.close()
