"""xl_rs_propagate_noalloc: RS / VRS without any device allocation.

This entry point is for callers of the library that cannot call cudaMalloc,
for example a host that hands all device memory to its own pool at start-up,
or a loop driving optical hardware that cannot absorb cudaMalloc's implicit
synchronisation.  Its workspace is a fixed array inside the library.  The
test calls it through the C ABI twice in a row, with different inputs and
distances, so the second call runs on scratch the first call left behind.
It checks each result against the workspace-taking entry point
xl_rs_propagate, at the tolerance the other GPU tests use (rel-L2 1e-5), for
a 512^2 vectorial field and for a 2048^2 scalar field, whose scratch fills the
fixed array exactly.  Around the second call it checks that no device memory
was allocated: torch's allocated bytes and the driver's free bytes
(cudaMemGetInfo) are unchanged.

The file is named to be collected last: if it fails, a run stopped at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from oracle import xlumina_ref as ref
from tests.conftest import rel_l2

TOL = 1e-5


def test_noalloc_rejects_work_beyond_the_fixed_scratch():
    from xlumina_gb300 import _build, _lib
    _build.build()
    lib = _lib.load()
    a = _lib.XlRsArgs()
    a.batch, a.comps_in, a.comps_out, a.ny, a.nx = 1, 2, 3, 2048, 2048   # 192 MiB of scratch
    assert lib.xl_rs_work_bytes(1, 3, 2048, 2048) > _lib.XL_RS_NOALLOC_MAX_WORK_BYTES
    assert lib.xl_rs_propagate_noalloc(None, ctypes.byref(a)) == _lib.XL_EINVAL
    assert b"fixed limit" in lib.xl_last_error()


def _noalloc(lib, args):
    import torch
    return lib.xl_rs_propagate_noalloc(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream),
                                       ctypes.byref(args))


@pytest.mark.gpu
@pytest.mark.parametrize("n,vector", [(512, True), (2048, False)])
def test_noalloc_matches_workspace_entry_point_two_calls(n, vector):
    import torch

    from xlumina_gb300 import _lib, engine
    lib = _lib.load()
    comps = 2 if vector else 1
    if not vector:   # the largest call the fixed scratch takes
        assert lib.xl_rs_work_bytes(1, 1, n, n) == _lib.XL_RS_NOALLOC_MAX_WORK_BYTES
    x, y = ref.space(800.0 * n / 512, n)
    rng = np.random.default_rng(2024 + n)
    for call_no, z in enumerate((1.5e4, 4.0e4)):
        E = rng.standard_normal((comps, n, n)) + 1j * rng.standard_normal((comps, n, n))
        fields = [torch.as_tensor(E[c].astype(np.complex64), device="cuda") for c in range(comps)]
        if vector:
            eta = torch.as_tensor(rng.uniform(0, 2 * np.pi, (n, n)).astype(np.float32), device="cuda")
            theta = torch.as_tensor(rng.uniform(0, 2 * np.pi, (n, n)).astype(np.float32), device="cuda")
            pre = [engine.op_lcd(eta, theta)]
        else:
            pre = [engine.op_phase(torch.as_tensor(rng.uniform(-np.pi, np.pi, (n, n)).astype(np.float32),
                                                   device="cuda"))]
        call = engine.RsCall(fields, x, y, 0.633, z, vector=vector, pre=pre)
        expected = [o.clone() for o in call.run()]

        outs = [torch.full((n, n), complex(np.nan, np.nan), dtype=torch.complex64, device="cuda")
                for _ in range(3 if vector else 1)]
        args = _lib.XlRsArgs.from_buffer_copy(call.args)
        for i, o in enumerate(outs):
            args.out[i] = o.data_ptr()
        args.work = None
        torch.cuda.synchronize()
        before = (torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0])
        rc = _noalloc(lib, args)
        assert rc == _lib.XL_OK, lib.xl_last_error()
        torch.cuda.synchronize()
        after = (torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0])
        if call_no == 1:   # the first call may load kernels; the second allocates nothing
            assert after == before, (before, after)
        for got, exp in zip(outs, expected):
            assert rel_l2(got.cpu().numpy(), exp.cpu().numpy()) < TOL


@pytest.mark.gpu
def test_noalloc_rejects_a_stream_of_another_device():
    """The scratch address is the current device's: a stream that belongs to
    another device is refused (only runs where there are two devices)."""
    import torch

    from xlumina_gb300 import _lib
    if torch.cuda.device_count() < 2:
        pytest.skip("one device")
    lib = _lib.load()
    s1 = torch.cuda.Stream(device=1)
    a = _lib.XlRsArgs()
    a.batch, a.comps_in, a.comps_out, a.ny, a.nx = 1, 1, 1, 64, 64
    with torch.cuda.device(0):
        rc = lib.xl_rs_propagate_noalloc(ctypes.c_void_p(s1.cuda_stream), ctypes.byref(a))
    assert rc == _lib.XL_EINVAL and b"belongs to device" in lib.xl_last_error()
