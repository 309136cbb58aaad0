"""GPU parity of the libhx map against the reference's CPU-build golden
fixtures and against the oracle on the same seeded inputs (bit-exact:
mapping, every query output buffer, fill and tombstone counts)."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
from gpu_util import bucket_array, device_mapping, from_dev, full_dev, to_dev
from hashinator_gb300 import workloads

pytestmark = pytest.mark.gpu

GROUPS = [1, 2, 4, 8, 16, 32]
# (group width, keys per thread, blind insert CAS, window bytes); group 0 = automatic policy
TUNINGS = [(0, 0, True, 32), (1, 1, True, 32), (1, 2, False, 32), (1, 4, True, 32), (1, 8, False, 32),
           (1, 1, True, 64), (1, 2, False, 64), (1, 4, True, 64), (2, 1, True, 32), (4, 1, False, 32),
           (8, 1, True, 32), (16, 1, True, 32), (32, 1, True, 32)]


def _tune(m, t):
    m.set_tuning(group_width=t[0], keys_per_thread=t[1])
    m.set_insert_mode(t[2])
    m.set_window_bytes(t[3])
FILL = {4: 0xA5A5A5A5, 8: 0xA5A5A5A5A5A5A5A5}


def _dt(w):
    return np.uint32 if w == 4 else np.uint64


@pytest.mark.parametrize("tuning", TUNINGS)
@pytest.mark.parametrize("name", golden_cases())
def test_golden_parity(hx, name, tuning):
    g = load_golden(name)
    w, sp = int(g["key_bytes"]), int(g["size_power"])
    dt = _dt(w)
    m = hx.Hashmap(sp, w)
    _tune(m, tuning)
    m.insert(to_dev(g["keys"]), to_dev(g["vals"]), target_lf=0.0)
    inf = m.info()
    assert inf.fill == int(g["size_after_insert"])
    assert m.peek_status() == hx.STATUS_SUCCESS
    assert m.peek_status() == hx.STATUS_INVALID  # peek resets (hashinator.h:434-438)
    q = to_dev(g["queries"])
    out = full_dev(len(g["queries"]), int(g["fill_pattern"]), w)
    m.retrieve(q, out)
    np.testing.assert_array_equal(from_dev(out, dt), g["q1_vals"])
    m.erase(to_dev(g["erase"]))
    inf = m.info()
    assert inf.fill == int(g["size_after_erase"])
    assert inf.tombstone_counter == int(g["n_erased"])
    out2 = full_dev(len(g["queries"]), int(g["fill_pattern"]), w)
    m.retrieve(q, out2)
    np.testing.assert_array_equal(from_dev(out2, dt), g["q2_vals"])
    k, v, _ = device_mapping(m, w)
    np.testing.assert_array_equal(k, g["map_keys"])
    np.testing.assert_array_equal(v, g["map_vals"])
    m.close()


def _run_cycle(hx, oracle_mod, w, sp, n, tuning, seed, erase_frac=0.3, hit=0.5, target_lf=0.0):
    dt = _dt(w)
    keys, vals, q, e = workloads.map_workload(n, w, seed, hit_frac=hit, erase_frac=erase_frac)
    m = hx.Hashmap(sp, w)
    _tune(m, tuning)
    om = oracle_mod.OracleMap(sp, w)
    m.insert(to_dev(keys), to_dev(vals), target_lf=target_lf)
    assert om.insert(keys, vals, target_lf) == 0
    assert m.peek_status() == hx.STATUS_SUCCESS
    inf, oi = m.info(), om.info()
    assert (inf.fill, inf.size_power) == (oi["fill"], oi["size_power"])

    def check_queries():
        out = full_dev(len(q), FILL[w], w)
        m.retrieve(to_dev(q), out)
        want = np.full(len(q), FILL[w], dt)
        om.retrieve(q, want)
        np.testing.assert_array_equal(from_dev(out, dt), want)

    def check_mapping():
        k, v, _ = device_mapping(m, w)
        ok, ov = om.mapping()
        np.testing.assert_array_equal(k, ok)
        np.testing.assert_array_equal(v, ov)

    check_queries()
    check_mapping()
    m.erase(to_dev(e))
    om.erase(e)
    inf, oi = m.info(), om.info()
    assert (inf.fill, inf.tombstone_counter) == (oi["fill"], oi["tombstones"])
    check_queries()
    check_mapping()
    m.clean_tombstones()
    om.clean_tombstones()
    inf, oi = m.info(), om.info()
    assert (inf.fill, inf.tombstone_counter) == (oi["fill"], oi["tombstones"]) and inf.tombstone_counter == 0
    check_queries()
    check_mapping()
    # after a clean every key sits in its home bucket or is reachable; re-insert all
    m.insert(to_dev(keys), to_dev(vals), target_lf=target_lf)
    om.insert(keys, vals, target_lf)
    inf, oi = m.info(), om.info()
    assert inf.fill == oi["fill"] == n
    check_queries()
    check_mapping()
    return m, om


@pytest.mark.parametrize("w", [4, 8])
@pytest.mark.parametrize("tuning", TUNINGS)
@pytest.mark.parametrize("lf", [0.5, 0.75, 0.9])
def test_oracle_parity_cycle(hx, oracle_mod, w, tuning, lf):
    sp = 16
    n = int(lf * (1 << sp))
    _run_cycle(hx, oracle_mod, w, sp, n, tuning, seed=100 + tuning[0] + 7 * tuning[1] + tuning[3])


@pytest.mark.parametrize("w", [4, 8])
def test_oracle_parity_cycle_large(hx, oracle_mod, w):
    """cfg1 shape in full: 2^20 keys, size power 21, 2^21 queries 50/50, erase 25%."""
    sp, n = 21, 1 << 20
    _run_cycle(hx, oracle_mod, w, sp, n, (0, 0, True, 32), seed=7, erase_frac=0.25)


@pytest.mark.parametrize("w", [4, 8])
def test_growth_rule_matches_reference(hx, oracle_mod, w):
    # insert() grows to ceil(log2((fill + len) / targetLF)) first (hashinator.h:1329-1332)
    keys, vals, q, _ = workloads.map_workload(3000, w, 31)
    m = hx.Hashmap(10, w)
    om = oracle_mod.OracleMap(10, w)
    for part in np.array_split(np.arange(3000), 3):
        m.insert(to_dev(keys[part]), to_dev(vals[part]), target_lf=0.5)
        om.insert(keys[part], vals[part], 0.5)
        assert m.info().size_power == om.info()["size_power"]
    assert m.info().size_power == 13
    k, v, _ = device_mapping(m, w)
    ok, ov = om.mapping()
    np.testing.assert_array_equal(k, ok)
    np.testing.assert_array_equal(v, ov)


@pytest.mark.parametrize("w", [4, 8])
@pytest.mark.parametrize("tuning", TUNINGS)
def test_overflow_sets_fail(hx, w, tuning):
    keys = workloads.distinct_keys(20, w, 3)
    m = hx.Hashmap(4, w)
    _tune(m, tuning)
    m.insert(to_dev(keys), to_dev(keys), target_lf=0.0)
    assert m.peek_status() == hx.STATUS_FAIL
    assert m.info().fill == 16


def test_duplicate_insertion(hx):
    g = load_golden("u32_duplicates")
    m = hx.Hashmap(12, 4)
    m.insert(to_dev(g["keys"]), to_dev(g["vals"]), target_lf=1.0)
    assert m.peek_status() == hx.STATUS_SUCCESS
    assert m.info().fill == int(g["size_after_insert"]) == 1024
    k, v, _ = device_mapping(m, 4)
    np.testing.assert_array_equal(k, g["map_keys"])
    np.testing.assert_array_equal(v, g["map_vals"])


@pytest.mark.parametrize("w", [4, 8])
def test_duplicate_erase_counts_once(hx, w):
    keys = workloads.distinct_keys(100, w, 8)
    m = hx.Hashmap(10, w)
    m.insert(to_dev(keys), to_dev(keys), 0.0)
    m.erase(to_dev(np.concatenate([keys[:10]] * 4)))
    inf = m.info()
    assert inf.fill == 90 and inf.tombstone_counter == 10


@pytest.mark.parametrize("w", [4, 8])
def test_sentinel_keys_are_skipped(hx, w):
    dt = _dt(w)
    e = np.iinfo(dt).max
    keys = np.concatenate([workloads.distinct_keys(10, w, 2), np.array([e, e - 1], dt)])
    m = hx.Hashmap(8, w)
    m.insert(to_dev(keys), to_dev(keys), 0.0)
    assert m.info().fill == 10
    out = full_dev(len(keys), 7, w)
    m.retrieve(to_dev(keys), out)
    got = from_dev(out, dt)
    np.testing.assert_array_equal(got[:10], keys[:10])
    assert (got[10:] == 7).all()


@pytest.mark.parametrize("w", [4, 8])
@pytest.mark.parametrize("sp", [1, 2, 3, 4, 5])
def test_tiny_tables(hx, oracle_mod, w, sp):
    n = (1 << sp) - 1 if sp > 1 else 1
    keys = workloads.distinct_keys(n, w, 40 + sp)
    vals = workloads.values(n, w, 40 + sp)
    for tuning in TUNINGS:
        m = hx.Hashmap(sp, w)
        _tune(m, tuning)
        m.insert(to_dev(keys), to_dev(vals), 0.0)
        assert m.peek_status() == hx.STATUS_SUCCESS
        out = full_dev(n, 0, w)
        m.retrieve(to_dev(keys), out)
        np.testing.assert_array_equal(from_dev(out, _dt(w)), vals)
        m.erase(to_dev(keys[: n // 2]))
        m.clean_tombstones()
        assert m.info().fill == n - n // 2


@pytest.mark.parametrize("w", [4, 8])
def test_zero_length_calls(hx, w):
    m = hx.Hashmap(6, w)
    empty = to_dev(np.zeros(0, _dt(w)))
    m.insert(empty, empty)
    assert m.peek_status() == hx.STATUS_SUCCESS  # insert(len 0) sets success (hashinator.h:1322-1325)
    m.retrieve(empty, empty)
    m.erase(empty)
    m.clean_tombstones()
    assert m.info().fill == 0


@pytest.mark.parametrize("w", [4, 8])
def test_ragged_lengths_and_unaligned_views(hx, oracle_mod, w):
    dt = _dt(w)
    keys, vals, q, _ = workloads.map_workload(5000, w, 55)
    m = hx.Hashmap(14, w)
    om = oracle_mod.OracleMap(14, w)
    m.insert(to_dev(keys), to_dev(vals), 0.0)
    om.insert(keys, vals, 0.0)
    qd = to_dev(q)
    for start, stop in [(0, 1), (1, 33), (3, 4999), (7, len(q))]:
        out = full_dev(len(q), FILL[w], w)
        m.retrieve(qd[start:stop], out[start:stop])
        want = np.full(len(q), FILL[w], dt)
        om.retrieve(q[start:stop], want[start:stop])
        np.testing.assert_array_equal(from_dev(out, dt), want)


@pytest.mark.parametrize("w", [4, 8])
def test_pairs_api(hx, oracle_mod, w):
    dt = _dt(w)
    keys, vals, q, _ = workloads.map_workload(20000, w, 66)
    pairs = np.stack([keys, vals], axis=1).reshape(-1)
    m = hx.Hashmap(16, w)
    m.insert_pairs(to_dev(pairs), n=len(keys), target_lf=0.0)
    qp = np.stack([q, np.full(len(q), FILL[w], dt)], axis=1).reshape(-1)
    qpd = to_dev(qp)
    m.retrieve_pairs(qpd, n=len(q))
    om = oracle_mod.OracleMap(16, w)
    om.insert(keys, vals, 0.0)
    want = np.full(len(q), FILL[w], dt)
    om.retrieve(q, want)
    got = from_dev(qpd, dt).reshape(-1, 2)
    np.testing.assert_array_equal(got[:, 0], q)
    np.testing.assert_array_equal(got[:, 1], want)


@pytest.mark.parametrize("w", [4, 8])
def test_upsert_overwrites(hx, w):
    dt = _dt(w)
    keys = workloads.distinct_keys(1000, w, 77)
    m = hx.Hashmap(12, w)
    m.insert(to_dev(keys), to_dev(keys), 0.0)
    m.insert(to_dev(keys), to_dev(keys + dt(1)), 0.0)
    assert m.info().fill == 1000
    out = full_dev(1000, 0, w)
    m.retrieve(to_dev(keys), out)
    np.testing.assert_array_equal(from_dev(out, dt), keys + dt(1))


@pytest.mark.parametrize("w", [4, 8])
def test_resize_and_clear(hx, oracle_mod, w):
    keys, vals, q, e = workloads.map_workload(30000, w, 88)
    m = hx.Hashmap(16, w)
    m.insert(to_dev(keys), to_dev(vals), 0.0)
    m.erase(to_dev(e))
    om = oracle_mod.OracleMap(16, w)
    om.insert(keys, vals, 0.0)
    om.erase(e)
    for sp in (17, 19, 16):
        m.resize(sp)
        om.resize(sp)
        inf = m.info()
        assert inf.size_power == sp and inf.tombstone_counter == 0 and inf.fill == om.info()["fill"]
        assert m.peek_status() == hx.STATUS_SUCCESS
        k, v, _ = device_mapping(m, w)
        ok, ov = om.mapping()
        np.testing.assert_array_equal(k, ok)
        np.testing.assert_array_equal(v, ov)
    m.clear()
    inf = m.info()
    assert inf.fill == 0 and inf.tombstone_counter == 0
    b = bucket_array(m, w)
    assert (b[:, 0] == np.iinfo(_dt(w)).max).all() and (b[:, 1] == 0).all()


@pytest.mark.parametrize("w", [4, 8])
def test_extract_pattern(hx, oracle_mod, w):
    dt = _dt(w)
    keys, vals, _, e = workloads.map_workload(40000, w, 99)
    m = hx.Hashmap(17, w)
    m.insert(to_dev(keys), to_dev(vals), 0.0)
    m.erase(to_dev(e))
    om = oracle_mod.OracleMap(17, w)
    om.insert(keys, vals, 0.0)
    om.erase(e)
    # (rule on device, rule in the oracle, result independent of bucket layout)
    rules = [(hx.Pred.value_even(), oracle_mod.pred(6, 2, 1, 0, 1), True),
             (hx.Pred.value_even(skip_sentinels=False), oracle_mod.pred(6, 2, 1, 0, 0), True),
             (hx.Pred.key_lt(1 << (8 * w - 3)), oracle_mod.pred(2, 1, 1 << (8 * w - 3)), True),
             (hx.Pred.valid_key(), oracle_mod.pred(8), True),
             # which key sits in its home bucket depends on insertion order
             (hx.Pred.not_home(), oracle_mod.pred(9), False)]
    b = bucket_array(m, w)
    for hp, op, layout_free in rules:
        out = to_dev(np.zeros(2 * (1 << 17), dt))
        c = m.extract_pattern(hp, out)
        got = from_dev(out, dt).reshape(-1, 2)[:c]
        # (ii) order = the device's own bucket order: the oracle filter over the device buckets
        np.testing.assert_array_equal(got, _filter_buckets(oracle_mod, b, w, op))
        if layout_free:
            # (i) count and (iii) sorted-by-key content equal the oracle's
            oc, oout = om.extract(op)
            assert c == oc
            np.testing.assert_array_equal(np.sort(got[:, 0]), np.sort(oout[:, 0]))
    # capacity smaller than the count: count still reported, HX_ERR_CAPACITY swallowed by wrapper
    small = to_dev(np.zeros(2 * 10, dt))
    assert m.extract_pattern(hx.Pred.valid_key(), small, capacity=10) == om.info()["fill"]


@pytest.mark.parametrize("w", [4, 8])
def test_extract_keys(hx, oracle_mod, w):
    """extractKeysByPattern / extractAllKeys: the keys of the pairs that
    extractPattern selects, in the same bucket order."""
    dt = _dt(w)
    keys, vals, _, e = workloads.map_workload(30000, w, 123)
    m = hx.Hashmap(16, w)
    m.insert(to_dev(keys), to_dev(vals), 0.0)
    m.erase(to_dev(e))
    om = oracle_mod.OracleMap(16, w)
    om.insert(keys, vals, 0.0)
    om.erase(e)
    b = bucket_array(m, w)
    for hp, op in [(hx.Pred.value_even(), oracle_mod.pred(6, 2, 1, 0, 1)), (hx.Pred.valid_key(), oracle_mod.pred(8)),
                   (hx.Pred.not_home(), oracle_mod.pred(9))]:
        out = to_dev(np.full(1 << 16, 7, dt))
        c = m.extract_keys_by_pattern(hp, out)
        got = from_dev(out, dt)
        want = _filter_buckets(oracle_mod, b, w, op)[:, 0]
        assert c == len(want)
        np.testing.assert_array_equal(got[:c], want)
        assert (got[c:] == 7).all()  # nothing written past the count
    out = to_dev(np.zeros(1 << 16, dt))
    c = m.extract_all_keys(out)
    ok, _ = om.mapping()
    assert c == len(ok)
    np.testing.assert_array_equal(np.sort(from_dev(out, dt)[:c]), ok)
    # capacity below the count: exact count, only `capacity` keys written
    small = to_dev(np.full(11, 7, dt))
    assert m.extract_all_keys(small, capacity=10) == len(ok)
    assert from_dev(small, dt)[10] == 7


def _filter_buckets(oracle_mod, b, w, op):
    """Order-preserving CPU filter of an arbitrary bucket array (the device's)."""
    flat = np.ascontiguousarray(b.reshape(-1))
    # not-home needs the table: evaluate in Python
    dt = b.dtype
    e = np.iinfo(dt).max
    k, v = b[:, 0], b[:, 1]
    sent = (k == e) | (k == e - 1)
    if op.op == 9:
        sp = int(np.log2(len(b)))
        homes = np.array([oracle_mod.fib_hash(int(x), sp, w) & ((1 << sp) - 1) if not s else 0
                          for x, s in zip(k, sent)], dtype=np.int64)
        sel = ~sent & (b[homes, 0] != k)
        return b[sel]
    return oracle_mod.copy_if(flat, 2 * w, op).reshape(-1, 2)


@pytest.mark.parametrize("w", [4, 8])
def test_insert_index(hx, oracle_mod, w):
    """insertIndex: keys[i] -> i, with the reference's growth rule."""
    dt = _dt(w)
    keys, _, q, _ = workloads.map_workload(50000, w, 31)
    m = hx.Hashmap(10, w)  # grows: ceil(log2(50000 / 0.5)) = 17
    m.insert_index(to_dev(keys))
    om = oracle_mod.OracleMap(10, w)
    om.insert(keys, np.arange(len(keys), dtype=dt))
    inf = m.info()
    assert inf.size_power == om.info()["size_power"] == 17 and inf.fill == len(keys)
    k, v, _ = device_mapping(m, w)
    ok, ov = om.mapping()
    np.testing.assert_array_equal(k, ok)
    np.testing.assert_array_equal(v, ov)
    out = to_dev(np.full(len(q), 0xA5, dt))
    m.retrieve(to_dev(q), out)
    want = np.full(len(q), 0xA5, dt)
    om.retrieve(q, want)
    np.testing.assert_array_equal(from_dev(out, dt), want)


@pytest.mark.parametrize("w", [4, 8])
def test_resize_to_lf_and_cleanup_tasks(hx, oracle_mod, w):
    keys, vals, _, e = workloads.map_workload(int(0.9 * (1 << 16)), w, 41, erase_frac=0.1)
    m = hx.Hashmap(16, w)
    m.insert(to_dev(keys), to_dev(vals), 0.0)
    om = oracle_mod.OracleMap(16, w)
    om.insert(keys, vals, 0.0)
    m.resize_to_lf(0.95)  # already below: nothing happens
    assert m.info().size_power == 16
    # performCleanupTasks: tombstone ratio 0.09 > 0.025 -> clean; probe bound > 32 at LF 0.9 -> grow
    m.erase(to_dev(e))
    om.erase(e)
    assert m.info().max_probe > 32
    m.perform_cleanup_tasks()
    inf = m.info()
    assert inf.tombstone_counter == 0 and inf.max_probe <= 32 and inf.size_power > 16
    assert inf.current_max_bucket_overflow == 32
    k, v, _ = device_mapping(m, w)
    ok, ov = om.mapping()
    np.testing.assert_array_equal(k, ok)
    np.testing.assert_array_equal(v, ov)
    m.resize_to_lf(0.1)
    sp = 16
    while inf.fill / (1 << sp) > 0.1:
        sp += 1
    inf = m.info()
    assert inf.size_power == sp and inf.fill == len(ok)
    k, v, _ = device_mapping(m, w)
    np.testing.assert_array_equal(k, ok)
    np.testing.assert_array_equal(v, ov)
