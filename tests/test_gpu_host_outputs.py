"""Output planes in pinned host memory: the last pass of a propagation stores
the result straight into page-locked host memory (xl_host_mapped gives the
address kernels use), so a result wanted on the host needs no separate
device-to-host copy.  The values are the ones the device path writes, bit for
bit; anything but pinned host or device memory is refused before a launch."""
import ctypes

import numpy as np
import pytest

from oracle import xlumina_ref as ref

pytestmark = pytest.mark.gpu


def _light(n=384, batch=2, seed=5):
    import torch

    import xlumina_gb300.vectorized_optics as vo
    x, y = ref.space(500.0, n)
    rng = np.random.default_rng(seed)
    E = (rng.standard_normal((2, n, n)) + 1j * rng.standard_normal((2, n, n))).astype(np.complex64)
    light = vo.VectorizedLight(x, y, 0.633)
    light.Ex = torch.as_tensor(E[0], device="cuda").expand(batch, n, n)
    light.Ey = torch.as_tensor(E[1], device="cuda").expand(batch, n, n)
    eta = torch.as_tensor(rng.uniform(0, 6, (batch, n, n)).astype(np.float32), device="cuda")
    return light, eta


@pytest.mark.parametrize("on_host", [(0, 1, 2), (2,), (1, 2)])
def test_host_outputs_equal_device_outputs(on_host):
    import torch

    import xlumina_gb300.optical_elements as oe
    light, eta = _light()
    zs = np.array([2.0e4, 5.0e4])
    exp, _ = oe.LCD(light, eta, 0.3).VRS_propagation(zs)
    torch.cuda.synchronize()
    outs = []
    for c in range(3):
        shape = tuple(exp.Ex.shape)
        if c in on_host:
            outs.append(torch.full(shape, 7.0 + 0j, dtype=torch.complex64).pin_memory())
        else:
            outs.append(torch.empty(shape, dtype=torch.complex64, device="cuda"))
    got, _ = oe.LCD(light, eta, 0.3).VRS_propagation(zs, out=outs)
    torch.cuda.synchronize()
    for g, o, e in zip((got.Ex, got.Ey, got.Ez), outs, (exp.Ex, exp.Ey, exp.Ez)):
        assert g.data_ptr() == o.data_ptr()
        assert torch.equal(g.cpu(), e.cpu())


def test_outputs_that_kernels_cannot_reach_are_refused():
    import torch

    import xlumina_gb300.optical_elements as oe
    from xlumina_gb300 import _lib, engine
    light, eta = _light(n=128, batch=1)
    shape = (1, 128, 128)
    pageable = [torch.empty(shape, dtype=torch.complex64) for _ in range(3)]
    with pytest.raises(ValueError):
        oe.LCD(light, eta, 0.3).VRS_propagation(2e4, out=pageable)
    wrong = [torch.empty((1, 128, 64), dtype=torch.complex64, device="cuda") for _ in range(3)]
    with pytest.raises(ValueError):
        oe.LCD(light, eta, 0.3).VRS_propagation(2e4, out=wrong)
    lib = engine.lib()
    d = ctypes.c_void_p()
    dev_t = torch.empty(16, device="cuda")
    host_t = torch.empty(16)
    assert lib.xl_host_mapped(ctypes.c_void_p(dev_t.data_ptr()), ctypes.byref(d)) == _lib.XL_EINVAL
    assert lib.xl_host_mapped(ctypes.c_void_p(host_t.data_ptr()), ctypes.byref(d)) == _lib.XL_EINVAL
    pinned = torch.empty(16).pin_memory()
    assert lib.xl_host_mapped(ctypes.c_void_p(pinned.data_ptr()), ctypes.byref(d)) == _lib.XL_OK
    assert d.value


def test_gradients_with_out_are_refused():
    import torch

    import xlumina_gb300.optical_elements as oe
    light, eta = _light(n=128, batch=1)
    eta.requires_grad_(True)
    outs = [torch.empty((1, 128, 128), dtype=torch.complex64, device="cuda") for _ in range(3)]
    with pytest.raises(ValueError):
        oe.LCD(light, eta, 0.3).VRS_propagation(2e4, out=outs)
