"""The no-allocation scan (hx_exclusive_scan_u32_noalloc) against the
allocating one (hx_exclusive_scan_u32), called through the C ABI.

The no-allocation entry point exists for callers that may not allocate device
memory when they scan; its scratch is one static device array shared by all
calls, so this test makes two calls in a row with different inputs and sizes
to show that each call resets what the previous one left behind. Integer
results: the tolerance is zero. The outputs are also compared with the exact
exclusive sum computed on the host (numpy, wrapping modulo 2^32), on the
TMA-staged path (16-byte-aligned buffers), the register path (buffers that
are not), in place, and at the largest size the static scratch holds.

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
    st = lib.hx_exclusive_scan_u32(d_in.data_ptr(), want.data_ptr(), n, None, 0, stream)
    assert st == 0, f"status {st}, cudaError {lib.hx_last_cuda_error()}"
    st = noalloc(d_in.data_ptr(), got.data_ptr(), n, stream)
    assert st == 0, f"status {st}, cudaError {lib.hx_last_cuda_error()}"
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


def _host_scan(x: np.ndarray) -> np.ndarray:
    out = np.zeros_like(x)
    if len(x) > 1:
        np.cumsum(x[:-1], dtype=np.uint32, out=out[1:])
    return out


def test_noalloc_scan_unaligned_and_in_place(hx):
    """A 4-byte offset from a 16-byte-aligned allocation takes the register
    kernel; d_out == d_in scans in place. Each call follows a larger one."""
    import torch
    lib, noalloc = _entry(hx)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(31415)
    x = rng.integers(0, 2**32, size=2_500_003, dtype=np.uint64).astype(np.uint32)
    # a larger call first, so the unaligned call runs over scratch left dirty
    big = rng.integers(0, 1 << 20, size=4_000_037, dtype=np.uint32)
    d_big, o_big = to_dev(big), torch.empty(len(big), dtype=torch.int32, device="cuda")
    assert noalloc(d_big.data_ptr(), o_big.data_ptr(), len(big), stream) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(from_dev(o_big, np.uint32), _host_scan(big))
    # unaligned input and output: element 1 onwards of aligned buffers
    d_in = to_dev(np.concatenate([np.zeros(1, np.uint32), x]))
    d_out = torch.full((len(x) + 1,), 0x5A5A5A5A, dtype=torch.int32, device="cuda")
    assert d_in.data_ptr() % 16 == 0 and d_out.data_ptr() % 16 == 0
    assert noalloc(d_in.data_ptr() + 4, d_out.data_ptr() + 4, len(x), stream) == 0
    want = torch.zeros(len(x), dtype=torch.int32, device="cuda")
    assert lib.hx_exclusive_scan_u32(d_in.data_ptr() + 4, want.data_ptr(), len(x), None, 0, stream) == 0
    torch.cuda.synchronize()
    got = from_dev(d_out, np.uint32)
    assert got[0] == 0x5A5A5A5A  # nothing written before the output
    np.testing.assert_array_equal(got[1:], _host_scan(x))
    np.testing.assert_array_equal(got[1:], from_dev(want, np.uint32))
    # in place, after the larger calls above
    y = rng.integers(0, 16, size=1_000_001, dtype=np.uint32)
    d_y = to_dev(y)
    assert noalloc(d_y.data_ptr(), d_y.data_ptr(), len(y), stream) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(from_dev(d_y, np.uint32), _host_scan(y))


def test_noalloc_scan_at_its_largest_size(hx):
    """n = 2^28, every tile status of the static scratch in use, twice in a row."""
    import torch
    lib, noalloc = _entry(hx)
    stream = torch.cuda.current_stream().cuda_stream
    g = torch.Generator(device="cuda").manual_seed(99)
    d_in = torch.randint(0, 16, (MAX_N,), dtype=torch.int32, device="cuda", generator=g)
    got = torch.empty_like(d_in)
    want = torch.empty_like(d_in)
    assert lib.hx_exclusive_scan_u32(d_in.data_ptr(), want.data_ptr(), MAX_N, None, 0, stream) == 0
    for _ in range(2):
        got.fill_(-1)
        assert noalloc(d_in.data_ptr(), got.data_ptr(), MAX_N, stream) == 0
        torch.cuda.synchronize()
        assert torch.equal(got, want)
    x = from_dev(d_in, np.uint32)
    np.testing.assert_array_equal(from_dev(got, np.uint32), _host_scan(x))


def test_noalloc_scan_rejects_sizes_beyond_its_scratch(hx):
    import torch
    _, noalloc = _entry(hx)
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    # nothing is launched for an oversize request, so the small buffers are never touched
    assert noalloc(buf.data_ptr(), buf.data_ptr(), MAX_N + 1, None) == hx.HX_ERR_INVALID_ARG
    assert noalloc(buf.data_ptr(), buf.data_ptr(), 0, None) == hx.HX_OK
