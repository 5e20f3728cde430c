"""The native AdamW step (angelo_gb.optim.AdamW, angelo_adamw_step) against
torch.optim.AdamW's single-tensor reference implementation on the same
parameters, gradients and hyper-parameters (the reference's optimizer is
torch.optim.AdamW, systems/utils.py:314-325)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from angelo_gb import build
    build.build()
    return torch.device("cuda:0")


@pytest.mark.parametrize("n", [1, 7, 4096, (1 << 20) + 3])
def test_adamw_matches_torch(dev, n):
    from angelo_gb.optim import AdamW
    g = torch.Generator(device="cpu").manual_seed(n)
    p0 = torch.randn(n, generator=g) * 0.1
    ours = torch.nn.Parameter(p0.clone().to(dev))
    ref = torch.nn.Parameter(p0.clone().to(dev))
    # hyper-parameters of the reference's config (lr 0.01, betas 0.9/0.99,
    # eps 1e-15, default weight decay 0.01)
    kw = dict(lr=0.01, betas=(0.9, 0.99), eps=1e-15, weight_decay=0.01)
    o1 = AdamW([ours], **kw)
    o2 = torch.optim.AdamW([ref], foreach=False, fused=False, **kw)
    for step in range(6):
        gr = torch.randn(n, generator=g)
        gr[torch.rand(n, generator=g) < 0.5] = 0.0      # untouched table rows get zero gradient
        ours.grad = gr.to(dev)
        ref.grad = gr.to(dev)
        o1.step()
        o2.step()
    a, b = ours.detach().cpu().numpy(), ref.detach().cpu().numpy()
    np.testing.assert_allclose(a, b, rtol=2e-5, atol=1e-7)
    # moments: fp32 rounding of values of order 0.1-1 (the first moment
    # nearly cancels where gradients change sign)
    for k in ("exp_avg", "exp_avg_sq"):
        np.testing.assert_allclose(o1.state[ours][k].cpu().numpy(), o2.state[ref][k].cpu().numpy(),
                                   rtol=1e-5, atol=2e-7)
    assert float(o1.state[ours]["step"]) == 6.0


def test_adamw_param_groups_and_unaligned(dev):
    from angelo_gb.optim import AdamW
    base = torch.randn(1 + 4096, device=dev)
    w = torch.nn.Parameter(base[1:].clone())      # contiguous
    b = torch.nn.Parameter(torch.randn(5, device=dev))
    w2 = torch.nn.Parameter(w.detach().clone())
    b2 = torch.nn.Parameter(b.detach().clone())
    o1 = AdamW([{"params": [w], "lr": 0.01}, {"params": [b], "lr": 0.001}], betas=(0.9, 0.99),
               eps=1e-15)
    o2 = torch.optim.AdamW([{"params": [w2], "lr": 0.01}, {"params": [b2], "lr": 0.001}],
                           betas=(0.9, 0.99), eps=1e-15, foreach=False)
    for _ in range(3):
        gw, gb = torch.randn_like(w), torch.randn_like(b)
        w.grad, w2.grad, b.grad, b2.grad = gw, gw.clone(), gb, gb.clone()
        o1.step()
        o2.step()
    np.testing.assert_allclose(w.detach().cpu().numpy(), w2.detach().cpu().numpy(), rtol=2e-5, atol=1e-7)
    np.testing.assert_allclose(b.detach().cpu().numpy(), b2.detach().cpu().numpy(), rtol=2e-5, atol=1e-7)
    # an unaligned contiguous parameter takes the scalar pass
    u = torch.nn.Parameter(torch.zeros(4099, device=dev)[3:])
    assert u.data_ptr() % 16 != 0
    u2 = torch.nn.Parameter(u.detach().clone())
    o3, o4 = AdamW([u], lr=0.01), torch.optim.AdamW([u2], lr=0.01, foreach=False)
    gu = torch.randn_like(u)
    u.grad, u2.grad = gu, gu.clone()
    o3.step()
    o4.step()
    np.testing.assert_allclose(u.detach().cpu().numpy(), u2.detach().cpu().numpy(), rtol=2e-5, atol=1e-7)


def test_multi_tensor_launch_is_bit_identical(dev):
    """Small tensors go through one angelo_adamw_step_multi launch; the update
    equals angelo_adamw_step on each tensor bit for bit."""
    import ctypes
    from angelo_gb._lib import call
    from angelo_gb.ops import _p, _s
    g = torch.Generator(device="cpu").manual_seed(5)
    sizes = [1, 3, 64 * 35, 4096, 2049, 65]
    ps = [torch.randn(n, generator=g).to(dev) for n in sizes]
    gs = [torch.randn(n, generator=g).to(dev) for n in sizes]
    ms = [torch.rand(n, generator=g).to(dev) * 0.1 for n in sizes]
    vs = [torch.rand(n, generator=g).to(dev) * 0.01 for n in sizes]
    single = [[t.clone() for t in ts] for ts in (ps, ms, vs)]
    hp = [(0.01 * (i + 1), 0.9, 0.99, 1e-15, 0.01, 1 - 0.9 ** 3, 1 - 0.99 ** 3) for i in range(len(sizes))]
    for i in range(len(sizes)):
        call("angelo_adamw_step", _p(single[0][i]), _p(gs[i]), _p(single[1][i]), _p(single[2][i]),
             sizes[i], *hp[i], _s(dev))
    n = len(sizes)
    ptr = lambda ts: (ctypes.c_void_p * n)(*[t.data_ptr() for t in ts])
    f32 = lambda j: (ctypes.c_float * n)(*[h[j] for h in hp])
    call("angelo_adamw_step_multi", n, ptr(ps), ptr(gs), ptr(ms), ptr(vs), (ctypes.c_int64 * n)(*sizes),
         *[f32(j) for j in range(7)], _s(dev))
    for a, b in zip(ps + ms + vs, single[0] + single[1] + single[2]):
        assert torch.equal(a, b)
