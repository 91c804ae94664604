"""The tables' AdamW (one libxlgb launch for the float32 parameters) against
torch.optim.AdamW, and recorded in a CUDA graph."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _params(torch, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    shapes = [(256, 256), (3, 64, 64), (1000,), (1003,), (1,)]   # 1003: four-wide body and a tail
    ps = [torch.randn(s, generator=g, device="cuda") for s in shapes]
    # a view one element into its storage, not 16-byte aligned: the element-wise path
    ps.append(torch.randn((1002,), generator=g, device="cuda")[1:].detach())
    ps.append(torch.randn((1,), generator=g, device="cuda", dtype=torch.float64))   # through torch's AdamW
    return [p.requires_grad_(True) for p in ps]


def test_adamw_matches_torch():
    import torch

    from xlumina_gb300.optim import AdamW
    a, b = _params(torch, 1), _params(torch, 1)
    oa = AdamW(a, lr=0.05, weight_decay=1e-3)
    ob = torch.optim.AdamW(b, lr=0.05, weight_decay=1e-3)
    g = torch.Generator(device="cuda").manual_seed(2)
    for _ in range(6):
        for pa, pb in zip(a, b):
            grad = torch.randn(pa.shape, generator=g, device="cuda", dtype=pa.dtype)
            pa.grad, pb.grad = grad.clone(), grad.clone()
        oa.step()
        ob.step()
    for pa, pb in zip(a, b):
        assert torch.allclose(pa, pb, rtol=2e-6, atol=2e-6), (pa - pb).abs().max()


def test_adamw_step_records_in_a_graph():
    import torch

    from xlumina_gb300.optim import AdamW
    p = torch.randn(4096, device="cuda").requires_grad_(True)
    ref = p.detach().clone().requires_grad_(True)
    opt, oref = AdamW([p], lr=0.01), torch.optim.AdamW([ref], lr=0.01)
    grad = torch.randn(4096, device="cuda")
    p.grad, ref.grad = grad.clone(), grad.clone()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        opt.step()
    torch.cuda.current_stream().wait_stream(s)
    oref.step()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        opt.step()
    for _ in range(3):
        graph.replay()
        oref.step()
    torch.cuda.synchronize()
    assert torch.allclose(p, ref, rtol=2e-6, atol=2e-6)
