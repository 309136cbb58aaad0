"""The streaming configuration at its full size, element for element: copy_if
on 2^28 uniform u32 with (x % 100) < s for s = 1, 50, 99; the exclusive scan
of 2^28 u32 in [0, 16); extractPattern (value even) and extractAllKeys on the
u32 map of 2^26 keys in 2^27 buckets. The expected outputs come from the host:
numpy's mask and filter (order-preserving), numpy's cumsum wrapping modulo
2^32, and an order-preserving filter of the map's own bucket array (the
bucket order of a concurrently built table is the device's, so the filter
runs over the device's buckets). At this size the multi-tile paths run with
their full tile counts and their persistent grids wrap many times, which the
oracle-sized cases in test_tools_gpu.py do not reach. Tolerance: zero."""
import numpy as np
import pytest

from gpu_util import bucket_array

pytestmark = pytest.mark.gpu

N = 1 << 28


@pytest.fixture(scope="module")
def stream_input():
    import torch
    g = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randint(0, 2**31 - 1, (N,), dtype=torch.int64, device="cuda", generator=g)
    x = (x * 2 + (x >> 17 & 1)).to(torch.int32)  # uniform over the 32-bit range
    return x, x.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("s", [1, 50, 99])
def test_copy_if_full_size(hx, stream_input, s):
    import torch
    x, xh = stream_input
    out = torch.full_like(x, -1)
    dc = torch.zeros(1, dtype=torch.int64, device="cuda")
    for _ in range(2):  # twice: the second call runs over the scratch the first left behind
        c = hx.tools.copy_if(x, out, hx.Pred.mod_lt(100, s))
    want = xh[(xh % np.uint32(100)) < s]
    assert c == len(want)
    np.testing.assert_array_equal(out[:c].cpu().numpy().view(np.uint32), want)
    assert (out[c:c + 1024].cpu().numpy() == -1).all()  # nothing written past the count
    # count on the device, no host synchronisation in the call
    hx.tools.copy_if(x, out, hx.Pred.mod_lt(100, s), d_count=dc)
    torch.cuda.synchronize()
    assert int(dc.item()) == len(want)


def test_exclusive_scan_full_size(hx, stream_input):
    import torch
    x, xh = stream_input
    y = (x & 15).contiguous()
    out = torch.full_like(y, -1)
    hx.tools.split_prefix_scan(y, out)
    yh = xh & np.uint32(15)
    want = np.zeros(N, np.uint32)
    np.cumsum(yh[:-1], dtype=np.uint32, out=want[1:])
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), want)
    # in place
    hx.tools.split_prefix_scan(y, y)
    np.testing.assert_array_equal(y.cpu().numpy().view(np.uint32), want)


def test_extract_full_size(hx):
    import torch
    from hashinator_gb300 import workloads
    keys, vals, _, _ = workloads.map_workload(1 << 26, 4, 2026, erase_frac=0.0)
    m = hx.Hashmap(27, 4)
    m.insert(torch.from_numpy(keys.view(np.int32)).cuda(), torch.from_numpy(vals.view(np.int32)).cuda(),
             target_lf=0.0)
    b = bucket_array(m, 4)
    valid = b[:, 0] < np.uint32(0xFFFFFFFE)
    assert int(valid.sum()) == 1 << 26
    sel = valid & (b[:, 1] % np.uint32(2) == 0)
    ex = torch.full((2 * (1 << 26),), -1, dtype=torch.int32, device="cuda")
    c = m.extract_pattern(hx.Pred.value_even(), ex, capacity=1 << 26)
    assert c == int(sel.sum()) == int((vals % 2 == 0).sum())
    np.testing.assert_array_equal(ex[:2 * c].cpu().numpy().view(np.uint32), b[sel].reshape(-1))
    ek = torch.full((1 << 26,), -1, dtype=torch.int32, device="cuda")
    ck = m.extract_all_keys(ek)
    assert ck == 1 << 26
    np.testing.assert_array_equal(ek.cpu().numpy().view(np.uint32), b[valid, 0])
    m.close()
