"""Known-answer and property checks of the oracle's split::tools restatement,
taken from the reference's own tests: race.cu (scan and compaction of
input[i] = i against thrust, unit_tests/stream_compaction/race.cu:100-113)
and unit.cu (flag counts over sizes 32..2999 and powers of two,
unit_tests/stream_compaction/unit.cu:36-107)."""
import numpy as np
import pytest

from hashinator_gb300 import workloads


@pytest.mark.parametrize("power", range(2, 18))
def test_scan_of_iota_known_answer(oracle_mod, power):
    n = 1 << power
    x = np.arange(n, dtype=np.uint64)
    want = ((x * (x - 1)) // 2 % (1 << 32)).astype(np.uint32)  # sum_{j<i} j mod 2^32
    got = oracle_mod.exclusive_scan_u32(np.arange(n, dtype=np.uint32))
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("power", range(2, 18))
def test_compaction_of_iota_evens(oracle_mod, power):
    n = 1 << power
    p = oracle_mod.pred(6, 0, 1, 0)  # (x & 1) == 0
    got = oracle_mod.copy_if(np.arange(n, dtype=np.uint32), 4, p)
    np.testing.assert_array_equal(got, np.arange(0, n, 2, dtype=np.uint32))


@pytest.mark.parametrize("size", [32, 33, 100, 1023, 1024, 1025, 2047, 2999])
def test_flag_split_counts(oracle_mod, size):
    # test_t{num, flag}: 8-byte elements, flag = (num % 2 == 0), num = 1..size
    num = np.arange(1, size + 1, dtype=np.uint32)
    arr = np.stack([num, (num % 2 == 0).astype(np.uint32)], axis=1).reshape(-1)
    on = oracle_mod.copy_if(arr, 8, oracle_mod.pred(4, 2, 1))   # value == 1
    off = oracle_mod.copy_if(arr, 8, oracle_mod.pred(4, 2, 0))  # value == 0
    assert (on.reshape(-1, 2)[:, 1] == 1).all() and (off.reshape(-1, 2)[:, 1] == 0).all()
    assert len(on) // 2 + len(off) // 2 == size
    assert len(on) // 2 == size // 2


def test_mod_lt_matches_numpy(oracle_mod):
    x = np.random.default_rng(3).integers(0, 2**32, size=100_000, dtype=np.uint64).astype(np.uint32)
    for s in (1, 50, 99):
        got = oracle_mod.copy_if(x, 4, oracle_mod.pred(1, 0, 100, s))
        np.testing.assert_array_equal(got, x[(x % 100) < s])


def test_fib_hash_restatement(oracle_mod):
    # HashFunctions::Fibonacci (hashinator/hashfunctions.h:39-56) restated in Python
    rng = np.random.default_rng(5)
    for sp in (1, 5, 13, 21, 27, 31):
        for k in rng.integers(0, 2**32, size=50, dtype=np.uint64):
            k = int(k)
            kk = k ^ (k >> (32 - sp))
            want = ((kk * 2654435769) >> (32 - sp)) & 0xFFFFFFFF
            assert oracle_mod.fib_hash(k, sp, 4) == want
        for k in rng.integers(0, 2**63, size=50, dtype=np.uint64):
            k = int(k) * 2 + 1
            kk = k ^ (k >> (64 - sp))
            want = ((kk * 11400714819323198485) & (2**64 - 1)) >> (64 - sp)
            assert oracle_mod.fib_hash(k, sp, 8) == want


def test_workload_keys_distinct_and_sentinel_free():
    for w in (4, 8):
        k = workloads.distinct_keys(100_000, w, 7)
        assert len(np.unique(k)) == len(k)
        e = (1 << (8 * w)) - 1
        assert not np.isin(k, np.array([e, e - 1], dtype=k.dtype)).any()
        keys, vals, q, er = workloads.map_workload(50_000, w, 9, hit_frac=0.5)
        assert np.isin(q, keys).sum() == 25_000


def test_oracle_overflow_reports_fail(oracle_mod):
    m = oracle_mod.OracleMap(4, 4)  # 16 buckets
    keys = workloads.distinct_keys(20, 4, 1)
    assert m.insert(keys, keys, target_lf=0.0) == 1
    assert m.info()["fill"] == 16


def test_oracle_extract_value_even(oracle_mod):
    keys, vals, _, _ = workloads.map_workload(3000, 4, 4)
    m = oracle_mod.OracleMap(13, 4)
    m.insert(keys, vals, 0.0)
    c, out = m.extract(oracle_mod.pred(6, 2, 1, 0, 1))  # value even, sentinels skipped
    assert c == int((vals % 2 == 0).sum())
    b = m.buckets()
    sel = (b[:, 0] < 0xFFFFFFFE) & (b[:, 1] % 2 == 0)
    np.testing.assert_array_equal(out, b[sel])
