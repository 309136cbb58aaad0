"""GPU parity of split::tools replacements (copy_if, split_prefix_scan)
against the oracle, plus the reference's own known answers (race.cu,
unit.cu)."""
import numpy as np
import pytest

from gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 3, 31, 32, 33, 100, 1023, 1024, 1025, 2999, 4095, 4096, 4097, 65535, 65536, 1 << 20,
         (1 << 20) + 17, 3_000_001]


@pytest.mark.parametrize("n", SIZES)
def test_scan_matches_oracle(hx, oracle_mod, n):
    x = np.random.default_rng(n).integers(0, 16, size=n, dtype=np.uint32)
    out = to_dev(np.zeros(n, np.uint32))
    hx.tools.split_prefix_scan(to_dev(x), out)
    np.testing.assert_array_equal(from_dev(out, np.uint32), oracle_mod.exclusive_scan_u32(x))


@pytest.mark.parametrize("power", range(2, 18))
def test_scan_iota_known_answer(hx, power):
    # race.cu: input[i] = i, exclusive scan == thrust::exclusive_scan (wraps mod 2^32)
    n = 1 << power
    out = to_dev(np.zeros(n, np.uint32))
    hx.tools.split_prefix_scan(to_dev(np.arange(n, dtype=np.uint32)), out)
    i = np.arange(n, dtype=np.uint64)
    np.testing.assert_array_equal(from_dev(out, np.uint32), ((i * (i - 1)) // 2 % (1 << 32)).astype(np.uint32))


def test_scan_wraps_and_in_place(hx, oracle_mod):
    x = np.full(1 << 20, 0xFFFFFFF0, np.uint32)
    d = to_dev(x)
    hx.tools.split_prefix_scan(d, d)  # in place
    np.testing.assert_array_equal(from_dev(d, np.uint32), oracle_mod.exclusive_scan_u32(x))


def test_scan_caller_scratch(hx, oracle_mod):
    import torch
    n = 1_000_003
    x = np.random.default_rng(1).integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    nb = hx.tools.scratch_bytes(hx.SCRATCH_SCAN, n)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    out = to_dev(np.zeros(n, np.uint32))
    for _ in range(2):
        hx.tools.split_prefix_scan(to_dev(x), out, scratch=scratch, scratch_bytes=nb)
        np.testing.assert_array_equal(from_dev(out, np.uint32), oracle_mod.exclusive_scan_u32(x))
    with pytest.raises(hx.HXError):
        hx.tools.split_prefix_scan(to_dev(x), out, scratch=scratch, scratch_bytes=16)


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("s", [1, 50, 99])
def test_copy_if_u32_mod_lt(hx, oracle_mod, n, s):
    x = np.random.default_rng(n + s).integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    out = to_dev(np.zeros(n, np.uint32))
    c = hx.tools.copy_if(to_dev(x), out, hx.Pred.mod_lt(100, s))
    want = oracle_mod.copy_if(x, 4, oracle_mod.pred(1, 0, 100, s))
    assert c == len(want)
    np.testing.assert_array_equal(from_dev(out, np.uint32)[:c], want)


@pytest.mark.parametrize("power", range(5, 25, 3))
def test_copy_if_iota_evens(hx, power):
    n = 1 << power
    out = to_dev(np.zeros(n, np.uint32))
    c = hx.tools.copy_if(to_dev(np.arange(n, dtype=np.uint32)), out, hx.Pred.even())
    assert c == n // 2
    np.testing.assert_array_equal(from_dev(out, np.uint32)[:c], np.arange(0, n, 2, dtype=np.uint32))


@pytest.mark.parametrize("size", list(range(32, 3000, 97)) + [2999])
def test_copy_if_flag_split(hx, size):
    # unit.cu Compaction_Tests_Linear: 8-byte {num, flag} elements, both splits
    num = np.arange(1, size + 1, dtype=np.uint32)
    arr = np.stack([num, (num % 2 == 0).astype(np.uint32)], axis=1).reshape(-1)
    d = to_dev(arr)
    on, off = to_dev(np.zeros_like(arr)), to_dev(np.zeros_like(arr))
    c1 = hx.tools.copy_if(d, on, hx.Pred(hx.PRED_EQ, hx.FIELD_VALUE, 1), elem_bytes=8)
    c0 = hx.tools.copy_if(d, off, hx.Pred(hx.PRED_EQ, hx.FIELD_VALUE, 0), elem_bytes=8)
    assert c1 + c0 == size and c1 == size // 2
    a1 = from_dev(on, np.uint32).reshape(-1, 2)[:c1]
    a0 = from_dev(off, np.uint32).reshape(-1, 2)[:c0]
    assert (a1[:, 1] == 1).all() and (a0[:, 1] == 0).all()
    np.testing.assert_array_equal(a1[:, 0], num[num % 2 == 0])


@pytest.mark.parametrize("eb", [8, 16])
@pytest.mark.parametrize("n", [5, 1000, 123457])
def test_copy_if_pairs_matches_oracle(hx, oracle_mod, eb, n):
    dt = np.uint32 if eb == 8 else np.uint64
    rng = np.random.default_rng(eb * n)
    arr = rng.integers(0, np.iinfo(dt).max, size=2 * n, dtype=dt, endpoint=True)
    arr[::7] = np.iinfo(dt).max  # EMPTY keys in the mix
    out = to_dev(np.zeros_like(arr))
    for hp, op in [(hx.Pred.value_even(), oracle_mod.pred(6, 2, 1, 0, 1)),
                   (hx.Pred.valid_key(), oracle_mod.pred(8)),
                   (hx.Pred(hx.PRED_MOD_LT, hx.FIELD_KEY, 7, 3, hx.PRED_NEGATE), oracle_mod.pred(1, 1, 7, 3, 2))]:
        c = hx.tools.copy_if(to_dev(arr), out, hp, elem_bytes=eb)
        want = oracle_mod.copy_if(arr, eb, op)
        assert 2 * c == len(want)
        np.testing.assert_array_equal(from_dev(out, dt)[: 2 * c], want)


def test_copy_if_capacity_and_device_count(hx, oracle_mod):
    import torch
    x = np.arange(10000, dtype=np.uint32)
    out = to_dev(np.zeros(100, np.uint32))
    c = hx.tools.copy_if(to_dev(x), out, hx.Pred.even(), capacity=100)
    assert c == 5000  # the full count is reported; only 100 written
    np.testing.assert_array_equal(from_dev(out, np.uint32), np.arange(0, 200, 2, dtype=np.uint32))
    dc = torch.zeros(1, dtype=torch.int64, device="cuda")
    big = to_dev(np.zeros(10000, np.uint32))
    assert hx.tools.copy_if(to_dev(x), big, hx.Pred.even(), d_count=dc) == -1
    torch.cuda.synchronize()
    assert int(dc.item()) == 5000


@pytest.mark.parametrize("eb", [4, 8, 16])
@pytest.mark.parametrize("off", [0, 4, 8, 12])
def test_copy_if_output_offsets_and_capacity_cuts(hx, eb, off):
    """Outputs that start 4, 8 or 12 bytes past a 16-byte boundary, and
    capacities that cut a CTA's run of output anywhere (each CTA writes its
    selections at an offset that no alignment constrains). The bytes before
    the output and after the last stored element stay as they were. An output
    that is not a multiple of the element size from 16-byte alignment (8-byte
    pairs at 4 bytes, 16-byte pairs at 4, 8, 12) is rejected before any
    device work."""
    import torch
    n = (1 << 20) + 12345
    dt = np.uint32 if eb in (4, 8) else np.uint64
    words = n * eb // np.dtype(dt).itemsize
    x = np.random.default_rng(eb * 100 + off).integers(0, np.iinfo(dt).max, size=words, dtype=dt, endpoint=True)
    rows = x.reshape(n, -1)
    key = rows[:, 0]
    sel = (key % dt(3)) < dt(2)  # about two thirds selected: long runs per CTA
    want = rows[sel].reshape(-1)
    pred = hx.Pred(hx.PRED_MOD_LT, hx.FIELD_ELEM if eb == 4 else hx.FIELD_KEY, 3, 2)
    d_in = to_dev(x)
    total = len(want) * np.dtype(dt).itemsize
    buf = torch.full((total + 64,), 0x5A, dtype=torch.uint8, device="cuda")
    base = buf.data_ptr() + off
    if off % eb:
        with pytest.raises(hx.HXError):
            hx.tools.copy_if(d_in, base, pred, elem_bytes=eb, n=n, capacity=len(want))
        assert (buf.cpu().numpy() == 0x5A).all()
        return
    for cap in (int(sel.sum()), int(sel.sum()) // 3 + 1, 1, 0, 16384 * 5 + 3):
        buf.fill_(0x5A)
        c = hx.tools.copy_if(d_in, base, pred, elem_bytes=eb, n=n, capacity=cap)
        assert c == int(sel.sum())
        got = buf.cpu().numpy()
        kept = min(cap, c) * eb
        assert (got[:off] == 0x5A).all()
        np.testing.assert_array_equal(got[off:off + kept], want.view(np.uint8)[:kept])
        assert (got[off + kept:] == 0x5A).all()


def test_copy_if_empty_input(hx):
    import torch
    e = torch.zeros(0, dtype=torch.int32, device="cuda")
    assert hx.tools.copy_if(e, e, hx.Pred.even()) == 0


# (x % a) < b is evaluated with a multiply-high remainder in the compaction
# kernel: check divisors at the edges of the 32-bit range, on u32 elements and
# on the key / value fields of u32 pairs, against the oracle's plain `%`.
DIVISORS = [1, 2, 3, 7, 100, 641, 65535, 65536, 65537, 2**31 - 1, 2**31, 2**31 + 11, 2**32 - 2, 2**32 - 1]


@pytest.mark.parametrize("a", DIVISORS)
def test_copy_if_mod_lt_divisors(hx, oracle_mod, a):
    rng = np.random.default_rng(a)
    x = rng.integers(0, 2**32, size=200_003, dtype=np.uint64).astype(np.uint32)
    x[:6] = [0, 1, a - 1 if a > 1 else 0, (a * 3) % 2**32, 2**32 - 1, 2**32 - 2]
    for b in sorted({1, max(1, a // 2), a - 1 if a > 1 else 1}):
        out = to_dev(np.zeros(len(x), np.uint32))
        c = hx.tools.copy_if(to_dev(x), out, hx.Pred.mod_lt(a, b))
        want = oracle_mod.copy_if(x, 4, oracle_mod.pred(1, 0, a, b))
        assert c == len(want) == int(((x.astype(np.uint64) % a) < b).sum())
        np.testing.assert_array_equal(from_dev(out, np.uint32)[:c], want)
    pairs = rng.integers(0, 2**32, size=2 * 50_001, dtype=np.uint64).astype(np.uint32)
    pairs[::11] = 2**32 - 1  # EMPTY keys
    for field, flags in [(hx.FIELD_KEY, 0), (hx.FIELD_VALUE, hx.PRED_SKIP_SENTINELS), (hx.FIELD_VALUE, hx.PRED_NEGATE)]:
        b = max(1, a // 3)
        out = to_dev(np.zeros_like(pairs))
        c = hx.tools.copy_if(to_dev(pairs), out, hx.Pred(hx.PRED_MOD_LT, field, a, b, flags), elem_bytes=8)
        want = oracle_mod.copy_if(pairs, 8, oracle_mod.pred(1, field, a, b, flags))
        assert 2 * c == len(want)
        np.testing.assert_array_equal(from_dev(out, np.uint32)[: 2 * c], want)


def test_copy_if_concurrent_host_threads_and_streams(hx, oracle_mod):
    """Arena-backed copy_if from 8 host threads at once, each on its own
    stream with its own caller scratch and device count (the reference's
    preallocated.cu: 8 OpenMP threads x 512 vectors): every result equals the
    oracle's."""
    import threading
    import torch
    rng = np.random.default_rng(8)
    sizes = [int(s) for s in rng.integers(1, 150_000, size=8 * 24)]
    data = [rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32) for n in sizes]
    results = [None] * len(sizes)
    errors = []

    def worker(t):
        try:
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                for i in range(t, len(sizes), 8):
                    n = sizes[i]
                    x = to_dev(data[i])
                    out = torch.zeros(n, dtype=torch.int32, device="cuda")
                    nb = hx.tools.scratch_bytes(hx.SCRATCH_COPY_IF, n)
                    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
                    dc = torch.zeros(1, dtype=torch.int64, device="cuda")
                    hx.tools.copy_if(x, out, hx.Pred.mod_lt(100, 37), scratch=scratch, scratch_bytes=nb, stream=s,
                                     d_count=dc)
                    s.synchronize()
                    c = int(dc.item())
                    results[i] = out.cpu().numpy().view(np.uint32)[:c]
        except Exception as e:  # reported below, in the main thread
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(8)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for i, x in enumerate(data):
        want = oracle_mod.copy_if(x, 4, oracle_mod.pred(1, 0, 100, 37))
        np.testing.assert_array_equal(results[i], want)
