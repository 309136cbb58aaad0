"""The no-allocation scan (hx_exclusive_scan_u32_noalloc) against the
allocating one (hx_exclusive_scan_u32), called through the C ABI.

The no-allocation entry point exists for callers that may not allocate device
memory when they scan; its scratch is one static device array shared by all
calls, so this test makes two calls in a row with different inputs and sizes
to show that each call resets what the previous one left behind. Integer
results: the tolerance is zero.

Named to be collected last, so that a run stopping at its first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

from gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu

MAX_N = 1 << 28  # HX_NOALLOC_SCAN_MAX_N in include/hx.h


def _entry(hx):
    lib = hx.lib()
    f = lib.hx_exclusive_scan_u32_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return lib, f


def _both(hx, x: np.ndarray, stream: int):
    lib, noalloc = _entry(hx)
    import torch
    d_in = to_dev(x)
    want = torch.zeros_like(d_in)
    got = torch.full_like(d_in, 0x5A5A5A5A)
    n = len(x)
    assert lib.hx_exclusive_scan_u32(d_in.data_ptr(), want.data_ptr(), n, None, 0, stream) == 0
    assert noalloc(d_in.data_ptr(), got.data_ptr(), n, stream) == 0
    torch.cuda.synchronize()
    return from_dev(got, np.uint32), from_dev(want, np.uint32)


def test_noalloc_scan_matches_allocating_scan_twice(hx):
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(2718)
    # first call: a large input that uses many tiles of the shared scratch
    x1 = rng.integers(0, 2**32, size=3_000_017, dtype=np.uint64).astype(np.uint32)
    got1, want1 = _both(hx, x1, stream)
    np.testing.assert_array_equal(got1, want1)
    # second call, right after: a different, smaller input over the same scratch
    x2 = rng.integers(0, 16, size=70_001, dtype=np.uint32)
    got2, want2 = _both(hx, x2, stream)
    np.testing.assert_array_equal(got2, want2)


def test_noalloc_scan_rejects_sizes_beyond_its_scratch(hx):
    import torch
    _, noalloc = _entry(hx)
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    # nothing is launched for an oversize request, so the small buffers are never touched
    assert noalloc(buf.data_ptr(), buf.data_ptr(), MAX_N + 1, None) == hx.HX_ERR_INVALID_ARG
    assert noalloc(buf.data_ptr(), buf.data_ptr(), 0, None) == hx.HX_OK
