"""xl_rs_propagate_noalloc: RS / VRS without any device allocation.

This entry point is for callers of the library that cannot call cudaMalloc,
for example a host that hands all device memory to its own pool at start-up,
or a loop driving optical hardware that cannot absorb cudaMalloc's implicit
synchronisation.  Its workspace is a fixed array inside the library.  The
test calls it through the C ABI twice in a row, with different inputs and
distances, so the second call runs on scratch the first call left behind.
It checks each result against the workspace-taking entry point
xl_rs_propagate, at the tolerance the other GPU tests use (rel-L2 1e-5).

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


@pytest.mark.gpu
def test_noalloc_matches_workspace_entry_point_two_calls():
    import torch

    from xlumina_gb300 import _lib, engine
    lib = _lib.load()
    n = 512
    x, y = ref.space(800.0, n)
    rng = np.random.default_rng(2024)
    for z in (1.5e4, 4.0e4):
        E = rng.standard_normal((2, n, n)) + 1j * rng.standard_normal((2, n, n))
        Ex = torch.as_tensor(E[0].astype(np.complex64), device="cuda")
        Ey = torch.as_tensor(E[1].astype(np.complex64), device="cuda")
        eta = torch.as_tensor(rng.uniform(0, 2 * np.pi, (n, n)).astype(np.float32), device="cuda")
        theta = torch.as_tensor(rng.uniform(0, 2 * np.pi, (n, n)).astype(np.float32), device="cuda")
        call = engine.RsCall([Ex, Ey], x, y, 0.633, z, vector=True, pre=[engine.op_lcd(eta, theta)])
        expected = [o.clone() for o in call.run()]

        outs = [torch.full((n, n), complex(np.nan, np.nan), dtype=torch.complex64, device="cuda")
                for _ in range(3)]
        args = _lib.XlRsArgs.from_buffer_copy(call.args)
        for i, o in enumerate(outs):
            args.out[i] = o.data_ptr()
        args.work = None
        rc = lib.xl_rs_propagate_noalloc(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream),
                                         ctypes.byref(args))
        assert rc == _lib.XL_OK, lib.xl_last_error()
        torch.cuda.synchronize()
        for got, exp in zip(outs, expected):
            assert rel_l2(got.cpu().numpy(), exp.cpu().numpy()) < TOL
