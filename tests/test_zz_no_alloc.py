"""The allocation-free scan (angelo_scan_noalloc) against the regular scan
(angelo_scan), called through the C ABI.

Some callers cannot allocate device memory -- a host that gives this library
only fixed, pre-sized buffers from its own pool, or code running where
cudaMalloc is not allowed -- so they cannot pass the workspace angelo_scan
needs.  angelo_scan_noalloc keeps that workspace in a fixed array inside the
library.  The offsets are integers, so the two must agree exactly; two calls
in a row check that what the first call leaves in the shared array does not
leak into the second.  Collected last (tests/test_zz_*) and self-contained:
it builds and loads the library itself."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from angelo_gb import _lib, build
    build.build()
    return _lib.load()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _scan_both(lib, counts):
    dev = counts.device
    n = counts.numel()
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    ref = torch.empty(n + 1, dtype=torch.int64, device=dev)
    ws = torch.empty(lib.angelo_scan_workspace_size(n), dtype=torch.uint8, device=dev)
    assert lib.angelo_scan(_ptr(counts), n, _ptr(ref), _ptr(ws), stream) == 0
    got = torch.empty(n + 1, dtype=torch.int64, device=dev)
    rc = lib.angelo_scan_noalloc(_ptr(counts), n, _ptr(got), stream)
    assert rc == 0, lib.angelo_last_error_string()
    torch.cuda.synchronize(dev)
    return ref.cpu().numpy(), got.cpu().numpy()


def test_noalloc_scan_matches_regular_scan_twice(lib):
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(0)
    # first call: many tiles; second call: fewer tiles, so stale tile sums of
    # the first call sit in the shared array beyond what the second one uses
    for n in (3_000_001, 4099):
        counts = torch.from_numpy(rng.integers(0, 600, n).astype(np.int32)).to(dev)
        ref, got = _scan_both(lib, counts)
        np.testing.assert_array_equal(got, ref)
        assert got[-1] == int(counts.long().sum().item())


def test_noalloc_scan_rejects_sizes_beyond_its_limit(lib):
    dev = torch.device("cuda:0")
    out = torch.empty(1, dtype=torch.int64, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    # the limit is checked on the host before anything is read or launched
    rc = lib.angelo_scan_noalloc(_ptr(out), (1 << 24) + 1, _ptr(out), stream)
    assert rc != 0
    assert b"limit" in lib.angelo_last_error_string()
