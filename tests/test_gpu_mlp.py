"""The fused ReLU VanillaMLP (angelo_mlp_fused_fwd / _bwd: the learned
background's density network, models/network_utils.py:96-140) against float64
autograd of the same weights: outputs, dL/dx and every weight gradient, for
one and two hidden layers, ragged row counts (empty, one row, partial tiles,
many tiles per CTA) and strided inputs."""
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


def _mlp(in_dim, n_hidden, out_dim, seed):
    from angelo_gb.network_utils import VanillaMLP
    torch.manual_seed(seed)
    m = VanillaMLP(in_dim, out_dim, dict(n_neurons=64, n_hidden_layers=n_hidden, activation="ReLU",
                                         output_activation="none"))
    with torch.no_grad():
        for lin in m.linears():
            lin.bias.uniform_(-0.2, 0.2)
    return m


# bf16x3 operands: every product carries ~2^-16 of its operands' magnitude
FWD_TOL = 2e-5
BWD_TOL = 5e-5
# rows whose float64 pre-activations come within this of zero are left out of
# the exact comparison: ReLU's derivative jumps at 0, and a pre-activation
# that close may fall on the other side in any arithmetic that is not float64
# (bf16x3 is ~3e-5 off on pre-activations of order 1)
MASK_MARGIN = 2e-3


def _pre_acts(m, x64):
    h, pre = x64, []
    lins = m.linears()
    for i, lin in enumerate(lins[:-1]):
        z = h @ lin.weight.detach().double().t() + lin.bias.detach().double()
        pre.append(z)
        h = torch.relu(z)
    return pre


def _clear_rows(m, n, in_dim, g, dev):
    """n rows uniform in [-1, 1]^in_dim whose pre-activations all stay
    MASK_MARGIN away from zero."""
    rows = []
    have = 0
    while have < n:
        x = torch.rand(max(2 * (n - have), 64), in_dim, generator=g) * 2 - 1
        ok = torch.ones(x.shape[0], dtype=torch.bool)
        for z in _pre_acts(m.cpu(), x.double()):
            ok &= (z.abs() > MASK_MARGIN).all(dim=1)
        rows.append(x[ok])
        have += int(ok.sum())
    m.to(dev)
    return torch.cat(rows)[:n]


def _fp64(m, x, gout):
    x64 = x.detach().double().requires_grad_(True)
    ws = [(lin.weight.detach().double().requires_grad_(True), lin.bias.detach().double().requires_grad_(True))
          for lin in m.linears()]
    h = x64
    for i, (W, b) in enumerate(ws):
        h = h @ W.t() + b
        if i + 1 < len(ws):
            h = torch.relu(h)
    (h * gout.double()).sum().backward()
    return h.detach(), x64.grad, ws


@pytest.mark.parametrize("shape", [(35, 1, 8), (19, 1, 8), (24, 2, 3), (64, 2, 16), (5, 1, 1)])
@pytest.mark.parametrize("n", [0, 1, 127, 129, 70001])
def test_fused_mlp_matches_fp64(dev, shape, n):
    from angelo_gb import fused
    in_dim, nh, od = shape
    m = _mlp(in_dim, nh, od, seed=in_dim * 7 + nh)
    m.fused = True
    assert fused.mlp_supported(m)
    g = torch.Generator(device="cpu").manual_seed(n + in_dim)
    xs = _clear_rows(m, n, in_dim, g, dev) if n else torch.zeros(0, in_dim)
    m.to(dev)
    # strided input: rows of a wider buffer (the encodings' layout)
    buf = torch.zeros(n, in_dim + 5)
    buf[:, 2:2 + in_dim] = xs
    x = buf.to(dev)[:, 2:2 + in_dim].requires_grad_(True)
    out = m(x)
    assert out.shape == (n, od)
    gout = torch.randn(n, od, generator=g).to(dev)
    (out * gout).sum().backward()
    h, gx, ws = _fp64(m, x, gout)
    if n == 0:
        return
    scale = float(h.abs().max()) + 1e-12
    assert float((out.detach().double() - h).abs().max()) <= FWD_TOL * scale
    gs = float(gx.abs().max()) + 1e-12
    assert float((x.grad.double() - gx).abs().max()) <= BWD_TOL * gs
    for lin, (W, b) in zip(m.linears(), ws):
        for a, r in ((lin.weight.grad, W.grad), (lin.bias.grad, b.grad)):
            sc = float(r.abs().max()) + 1e-12
            assert float((a.double() - r).abs().max()) <= BWD_TOL * sc


def test_fused_mlp_mask_flips_stay_local(dev):
    """Unfiltered rows: a hidden unit whose pre-activation sits within the
    products' rounding of zero may take the other side of the ReLU than
    float64.  Every difference from float64 must then be made of such units'
    terms: per element it stays within the sum of |term| over the (row, unit)
    pairs whose float64 pre-activation is within DELTA of zero, plus a
    rounding tolerance."""
    DELTA = 2e-4   # ~10x the bf16x3 error of these pre-activations
    m = _mlp(35, 1, 8, seed=11)
    m.fused = True
    m.to(dev)
    g = torch.Generator(device="cpu").manual_seed(12)
    x = (torch.rand(100000, 35, generator=g) * 2 - 1).to(dev).requires_grad_(True)
    gout = torch.randn(100000, 8, generator=g).to(dev)
    out = m(x)
    (out * gout).sum().backward()
    h, gx, ws = _fp64(m, x, gout)
    assert float((out.detach().double() - h).abs().max()) <= FWD_TOL * float(h.abs().max())
    (W1, b1), (W3, _) = ws
    x64 = x.detach().double()
    z = x64 @ W1.detach().t() + b1.detach()
    amb = (z.abs() < DELTA).double()                       # (rows, units)
    dh = gout.double() @ W3.detach()                       # dL/dH before the mask
    term = amb * dh.abs()
    assert float(amb.sum()) > 0                            # the case is exercised
    tol = lambda r: 1e-4 * float(r.abs().max())            # noqa: E731
    bound_dx = term @ W1.detach().abs()                    # per row of dL/dx
    assert bool(((x.grad.double() - gx).abs() <= bound_dx + tol(gx)).all())
    lin1 = m.linears()[0]
    bound_w = term.t() @ x64.abs()                         # per element of dW1
    assert bool(((lin1.weight.grad.double() - W1.grad).abs() <= bound_w + tol(W1.grad)).all())
    assert bool(((lin1.bias.grad.double() - b1.grad).abs() <= term.sum(0) + tol(b1.grad)).all())
    lin3 = m.linears()[1]
    # dW3 = H^T dY: a flipped unit's activation is within DELTA of zero
    for a, r in ((lin3.weight.grad, ws[1][0].grad), (lin3.bias.grad, ws[1][1].grad)):
        assert float((a.double() - r).abs().max()) <= 1e-3 * float(r.abs().max())


def test_fused_mlp_no_input_gradient(dev):
    """dL/dx is not written when x needs no gradient (d_x = NULL); the weight
    gradients are the same as with it."""
    m = _mlp(35, 1, 8, seed=3).to(dev)
    m.fused = True
    x = torch.rand(3000, 35, device=dev) * 2 - 1
    gout = torch.randn(3000, 8, device=dev)
    (m(x) * gout).sum().backward()
    g1 = [p.grad.clone() for p in m.parameters()]
    m.zero_grad()
    xr = x.clone().requires_grad_(True)
    (m(xr) * gout).sum().backward()
    # the CTAs add their weight gradients with atomics in any order: equal up
    # to the rounding of that order, relative to the tensor's largest entry
    for a, b in zip(g1, [p.grad for p in m.parameters()]):
        assert float((a - b).abs().max()) <= 1e-5 * float(b.abs().max())


def test_fused_mlp_deterministic_rows(dev):
    """A row's output does not depend on the batch it is in (the background
    reuses the visibility pass's outputs on the kept samples)."""
    m = _mlp(35, 1, 8, seed=5).to(dev)
    m.fused = True
    x = torch.rand(5000, 35, device=dev)
    with torch.no_grad():
        a = m(x)
        idx = torch.randperm(5000, device=dev)[:1234]
        b = m(x[idx])
    assert torch.equal(a[idx], b)


def test_fused_mlp_backward_reads_rows_by_index(dev):
    """angelo_mlp_fused_bwd with x_rows (the background's kept samples read
    in place from the visibility pass's encodings) equals the backward on the
    gathered rows: dL/dx bit for bit, dL/dW up to the CTAs' atomic order."""
    from angelo_gb import _lib, fused
    from angelo_gb.ops import _p, _s
    m = _mlp(35, 1, 8, seed=21).to(dev)
    g = torch.Generator(device="cpu").manual_seed(22)
    X = (torch.rand(20000, 35, generator=g) * 2 - 1).to(dev)
    rows = torch.randperm(20000, generator=g)[:7777].sort().values.to(dev)
    gout = torch.randn(7777, 8, generator=g).to(dev)
    net = fused.MlpNet(35, 1, 8, dev)
    net.prepare(m.effective_weights())
    outs = []
    for x, r in ((X.index_select(0, rows).contiguous(), None), (X, rows.to(torch.int32))):
        dx = torch.empty(7777, 35, device=dev)
        dn = torch.zeros(net.grad_size, device=dev)
        _lib.call("angelo_mlp_fused_bwd", 35, 1, 8, _p(net.buf), _p(x), x.stride(0), _p(r), 7777,
                  _p(gout), gout.stride(0), _p(dx), dx.stride(0), _p(dn), _s(dev))
        outs.append((dx, dn))
    torch.cuda.synchronize()
    assert torch.equal(outs[0][0], outs[1][0])
    assert float((outs[0][1] - outs[1][1]).abs().max()) <= 1e-5 * float(outs[0][1].abs().max())
