"""The tcgen05 building block of the fused MLP kernels (angelo_tc_gemm_x3 of
the test-only probe library, tests/native/tc_probe.cu, built from the
product's tensor-core helpers):
D = A B^T with both operands split into bf16 hi/lo in shared memory, the
three products accumulated in fp32 in tensor memory, against float64.
K-major operands feed the per-row layer products, MN-major operands the
weight-gradient products over samples; the layout convention the library
uses is variant 0 (descriptor LBO = core-matrix stride along K, SBO = along
M or N, for either major)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from angelo_gb import build
    from native import build as probe
    build.build()
    probe.build()
    return torch.device("cuda:0")


def _run(dev, M, N, K, a_mn, b_mn, variant, seed=0):
    from angelo_gb.ops import _p, _s
    from native.build import call
    g = torch.Generator(device="cpu").manual_seed(seed)
    A = torch.randn(M, K, generator=g).to(dev)
    B = torch.randn(N, K, generator=g).to(dev)
    D = torch.full((128, 2 * N if M == 64 else N), float("nan"), device=dev)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    call("angelo_tc_gemm_x3", _p(A), _p(B), _p(D), M, N, K, a_mn, b_mn, variant, _p(st), _s(dev))
    torch.cuda.synchronize()
    return int(st.item()), A.double() @ B.double().T, D.double()


def _gemm(dev, N, K, a_mn, b_mn, variant, seed=0):
    st, ref, D = _run(dev, 128, N, K, a_mn, b_mn, variant, seed)
    err = ((D - ref).abs().max() / ref.abs().max()).item()
    return st, err


@pytest.mark.parametrize("N,K", [(16, 16), (64, 48), (80, 64), (128, 32), (256, 64)])
def test_tc_gemm_x3_kmajor(dev, N, K):
    st, err = _gemm(dev, N, K, 0, 0, 0)
    assert st == 0, "tensor-core completion wait timed out"
    # bf16x3 keeps ~2^-16 of each operand; K <= 64 terms
    assert err < 2e-5, err


@pytest.mark.parametrize("N,K", [(16, 16), (64, 32), (112, 16)])
@pytest.mark.parametrize("a_mn,b_mn", [(1, 1), (1, 0), (0, 1)])
def test_tc_gemm_x3_mnmajor(dev, N, K, a_mn, b_mn):
    st, err = _gemm(dev, N, K, a_mn, b_mn, 0)
    assert st == 0, "tensor-core completion wait timed out"
    assert err < 2e-5, err


def test_tc_layout_variant_is_pinned(dev):
    """Variant 1 exchanges the descriptor's two core-matrix strides: it must
    not agree with float64 where variant 0 does, so the stride convention the
    kernels use is the only one that reproduces the product."""
    for a_mn, b_mn in [(0, 0), (1, 1)]:
        st0, err0 = _gemm(dev, 64, 16, a_mn, b_mn, 0, seed=1)
        st1, err1 = _gemm(dev, 64, 16, a_mn, b_mn, 1, seed=1)
        assert st0 == 0 and st1 == 0
        assert err0 < 2e-5, (a_mn, b_mn, err0)
        assert err1 > 1e-2, (a_mn, b_mn, err1)


def test_tc_m64_accumulator_layout(dev):
    """M = 64: every row of the product is found in exactly one tensor-memory
    (lane, column block); the mapping is printed (the layout an M = 64
    kernel would read)."""
    st, ref, D = _run(dev, 64, 32, 32, 0, 0, 0, seed=3)
    assert st == 0
    found = []
    for i in range(64):
        hits = []
        for b in range(2):                        # the row's two 16-column blocks
            hits.append([(lane, c0) for lane in range(128) for c0 in range(0, 64 - 15)
                         if torch.allclose(D[lane, c0:c0 + 16], ref[i, 16 * b:16 * b + 16],
                                           rtol=1e-4, atol=1e-4)])
        found.append(hits)
    print("\nM=64 row -> [(lane, first column) of its column blocks]:")
    for i, h in enumerate(found):
        print(i, h)
    assert all(len(h[0]) >= 1 and len(h[1]) >= 1 for h in found)


@pytest.mark.parametrize("N,K", [(48, 64), (64, 64), (80, 32), (16, 64)])
def test_tc_m64_mn_major_weight_gradient(dev, N, K):
    """The weight-gradient products of the backward MLP: M = 64 units, both
    operands MN-major (transposed [sample][column] stagings), read back with
    row i in tensor-memory lane 32 (i / 16) + i % 16."""
    st, ref, D = _run(dev, 64, N, K, 1, 1, 0, seed=5)
    assert st == 0
    lanes = torch.tensor([32 * (i // 16) + i % 16 for i in range(64)])
    got = D[lanes, :N]
    err = ((got - ref).abs().max() / ref.abs().max()).item()
    assert err < 2e-5, err


def test_tc_mma_issue_rate(dev):
    """Cycles per back-to-back tcgen05.mma (bf16, K = 16) by shape: the cost
    model behind the fused MLP kernels' round structure.  128 x 256 runs at
    the dense rate (128 x 256 x 16 MACs in >= 128 cycles); a small product
    (N <= 64) completes in fewer cycles than the largest one but in more than
    its share of the dense rate (a per-instruction floor)."""
    from angelo_gb.ops import _p, _s
    from native.build import call
    rows = []
    for M, N in [(128, 256), (128, 128), (128, 64), (128, 16), (64, 64), (64, 16)]:
        cyc = torch.zeros(2, dtype=torch.int64, device=dev)
        st = torch.zeros(1, dtype=torch.int32, device=dev)
        call("angelo_tc_mma_rate", M, N, 1024, _p(cyc), _p(st), _s(dev))
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        c = cyc.cpu().tolist()
        rows.append((M, N, round(c[0] / 1024, 1), round(c[1] / 1024, 1)))
    print("\n(M, N, issue cycles / mma, complete cycles / mma):", rows)
    assert rows[0][3] >= 100
    small = {(M, N): c for M, N, _, c in rows}
    for shape in ((128, 16), (64, 16), (64, 64)):
        assert small[shape] < rows[0][3], (shape, rows)
        # dense rate would be N / 2 cycles for M = 128 (N / 4 for M = 64)
        assert small[shape] > shape[1] / 2, (shape, rows)
