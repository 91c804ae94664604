"""Bounded waits that run out reach the caller as an error.

The row kernels stage their input rows into shared memory with TMA bulk
copies and wait for them on an mbarrier with a time limit (one second by
default).  xl_set_wait_limit(0) is the test setting that makes every such
wait give up at once: the kernel lets its copy in flight land, raises the
status word in mapped host memory and returns, without a fault or a hang.
The package must then raise XlError (XL_ETIMEOUT) instead of handing the
output on: at the next propagation call, at an explicit check, and in the
serving loop.  Afterwards, with the default limit restored, results are
correct again."""
import ctypes

import numpy as np
import pytest

from oracle import xlumina_ref as ref
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture
def zero_wait():
    """Every bounded wait gives up at once; the chirp-z row pass stages every
    plane that fits (kernel variant 1), so that its rows are waited for at
    every transform length."""
    from xlumina_gb300 import _lib, engine
    lib = engine.lib()
    flag, n = ctypes.c_uint(0), ctypes.c_uint(0)
    lib.xl_device_status(ctypes.byref(flag), 1)
    lib.xl_device_timeouts(ctypes.byref(n), 1)
    saved = {lg: lib.xl_get_kernel_variant(_lib.XL_PASS_CZT_ROWS, lg) for lg in range(5, 14)}
    for lg in saved:
        _lib.check(lib.xl_set_kernel_variant(_lib.XL_PASS_CZT_ROWS, lg, 1), "xl_set_kernel_variant")
    _lib.check(lib.xl_set_wait_limit(0), "xl_set_wait_limit")
    yield lib
    _lib.check(lib.xl_set_wait_limit(10 ** 9), "xl_set_wait_limit")
    for lg, v in saved.items():
        _lib.check(lib.xl_set_kernel_variant(_lib.XL_PASS_CZT_ROWS, lg, v), "xl_set_kernel_variant")
    lib.xl_device_status(ctypes.byref(flag), 1)
    lib.xl_device_timeouts(ctypes.byref(n), 1)


def _inputs(n=256):
    import torch
    x, y = ref.space(400.0, n)
    rng = np.random.default_rng(31)
    E = (rng.standard_normal((2, n, n)) + 1j * rng.standard_normal((2, n, n))).astype(np.complex64)
    eta = rng.uniform(0, 2 * np.pi, (n, n)).astype(np.float32)
    d = lambda a: torch.as_tensor(a, device="cuda")  # noqa: E731
    return x, y, E, eta, [d(E[0]), d(E[1])], d(eta)


def test_timed_out_wait_raises_at_the_next_call_and_at_a_check(zero_wait):
    import torch

    from xlumina_gb300 import _lib, engine
    lib = zero_wait
    x, y, E, eta, (ex, ey), eta_d = _inputs()
    pre = [engine.op_lcd(eta_d, 0.4)]
    engine.rs_propagate([ex, ey], x, y, 0.633, 2e4, True, pre=pre)   # staged rows: the waits give up
    torch.cuda.synchronize()
    n = ctypes.c_uint(0)
    _lib.check(lib.xl_device_timeouts(ctypes.byref(n), 0))
    assert n.value > 0
    with pytest.raises(_lib.XlError) as ei:
        engine.rs_propagate([ex, ey], x, y, 0.633, 2e4, True, pre=pre)   # reported before launching
    assert ei.value.code == _lib.XL_ETIMEOUT
    # the chirp-z row pass takes the same path
    xo, yo = ref.space(100.0, 128)
    engine.czt_propagate([ex, ey], x, y, 0.633, 2e4, xo, yo, "vczt", pre=pre)
    torch.cuda.synchronize()
    with pytest.raises(_lib.XlError) as ei:
        _lib.check_device_status()
    assert ei.value.code == _lib.XL_ETIMEOUT
    _lib.check_device_status()   # cleared by the raise


def test_serving_fails_the_requests_of_a_timed_out_batch(zero_wait):
    from xlumina_gb300 import _lib
    from xlumina_gb300.serving import Request, Server
    x, y, E, eta, (ex, ey), eta_d = _inputs()
    srv = Server(hbm_budget_bytes=4e9, max_batch=4, streams=1)
    try:
        fut = srv.submit(Request("vrs", [ex, ey], x, y, 0.633, 2e4))
        with pytest.raises(_lib.XlError):
            fut.result(timeout=60)
    finally:
        srv.close()


def test_results_are_valid_again_after_the_limit_is_restored():
    import torch

    from xlumina_gb300 import _lib, engine
    lib = engine.lib()
    _lib.check(lib.xl_set_wait_limit(10 ** 9))
    flag = ctypes.c_uint(0)
    lib.xl_device_status(ctypes.byref(flag), 1)
    x, y, E, eta, (ex, ey), eta_d = _inputs()
    out = engine.rs_propagate([ex, ey], x, y, 0.633, 2e4, True, pre=[engine.op_lcd(eta_d, 0.4)])
    torch.cuda.synchronize()
    _lib.check_device_status()
    ax, ay = ref.lcd(E[0].astype(np.complex128), E[1].astype(np.complex128), eta.astype(np.float64), 0.4)
    exp = ref.vrs_propagate(ax, ay, x, y, 0.633, 2e4)
    for o, e in zip(out, exp):
        assert rel_l2(o.cpu().numpy(), e) < 1e-5
