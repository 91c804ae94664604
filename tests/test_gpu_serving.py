"""The continuous-batching server: every result is the same alone and in the mix
(rel-L2 <= 1e-6; batching changes no arithmetic), admission respects the HBM
budget, and oversize requests are refused without touching the GPU."""
import numpy as np
import pytest

from oracle import xlumina_ref as ref
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _mk(kind, n, z, seed):
    import torch

    from xlumina_gb300.serving import Request
    rng = np.random.default_rng(seed)
    x, y = ref.space(400.0 * n / 256, n)

    def f():
        return torch.as_tensor((rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64),
                               device="cuda")
    if kind == "rs":
        return Request("rs", [f()], x, y, 0.633, z)
    if kind == "vrs":
        return Request("vrs", [f(), f()], x, y, 0.633, z)
    if kind == "czt":
        xo, yo = ref.space(100.0, n // 2)
        return Request("czt", [f()], x, y, 0.633, z, xout=xo, yout=yo)
    ph = torch.as_tensor(rng.uniform(-np.pi, np.pi, (n, n)).astype(np.float32), device="cuda")
    tgt = torch.as_tensor(rng.uniform(0, 1, (n, n)).astype(np.float32), device="cuda")
    return Request("grad", [f()], x, y, 0.633, z, phase=ph, target=tgt)


def _np(r):
    if isinstance(r, tuple):
        return [t.detach().cpu().numpy() for t in r]
    return [r.detach().cpu().numpy()]


def test_results_same_alone_and_in_the_mix():
    from xlumina_gb300.serving import Server
    specs = [(k, n, z) for k in ("rs", "vrs", "czt", "grad") for n in (64, 128) for z in (1e4, 3e4)]
    alone = []
    srv = Server(max_batch=8, streams=2)
    for i, (k, n, z) in enumerate(specs):
        alone.append(_np(srv.submit(_mk(k, n, z, i)).result(timeout=120)))
    futs = [srv.submit(_mk(k, n, z, i)) for i, (k, n, z) in enumerate(specs)]
    futs += [srv.submit(_mk(k, n, z, 100 + i)) for i, (k, n, z) in enumerate(specs)]   # extra traffic
    mixed = [_np(f.result(timeout=120)) for f in futs[:len(specs)]]
    srv.close()
    st = srv.stats()
    assert st["completed"] == 3 * len(specs)
    assert st["batches"] < 3 * len(specs)            # requests were batched
    for a, b in zip(alone, mixed):
        for u, v in zip(a, b):
            assert rel_l2(v, u) <= 1e-6


def test_admission_budget_and_oversize_refusal():
    from xlumina_gb300.serving import Server
    r = _mk("vrs", 128, 2e4, 1)
    budget = 2.5 * r.nbytes()
    srv = Server(hbm_budget_bytes=budget, max_batch=16, streams=2)
    futs = [srv.submit(_mk("vrs", 128, 2e4 + i, i)) for i in range(6)]
    for f in futs:
        f.result(timeout=120)
    big = _mk("vrs", 512, 2e4, 9)
    with pytest.raises(MemoryError):
        srv.submit(big).result(timeout=10)
    srv.close()
    assert srv.stats()["mean_batch"] <= 2.0 + 1e-9    # the budget admits at most two at a time


def test_tuned_batch_packing(tmp_path):
    import torch

    from xlumina_gb300 import toolbox
    from xlumina_gb300.autotune import BatchTuner
    from xlumina_gb300.serving import Request, Server
    n = 64
    x, y = toolbox.space(100.0, n)
    f = torch.randn((n, n), dtype=torch.complex64, device="cuda")
    tuner = BatchTuner(path=str(tmp_path / "tune.json"), candidates=(1, 2, 4), repeats=1)
    srv = Server(max_batch=4, tuner=tuner)
    try:
        packing = srv.tune([Request("rs", [f], x, y, 0.5, 1e3)])
        b = packing[("rs", n, n)]
        assert b in (1, 2, 4)
        assert srv.batch_cap(Request("rs", [f], x, y, 0.5, 2e3)) == b
        futs = [srv.submit(Request("rs", [f], x, y, 0.5, 1e3 * (i + 1))) for i in range(6)]
        outs = [fu.result(timeout=120) for fu in futs]
        assert all(o.shape == (n, n) for o in outs)
    finally:
        srv.close()
    assert (tmp_path / "tune.json").exists()
