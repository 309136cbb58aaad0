"""Inserts reordered by table region (hx_map_set_insert_partition) give the
same maps as plain inserts: the same key-sorted mapping and fill for keys
with values, for hash_pair input, for insertIndex (value = position in the
batch, carried through the reordering), with duplicate keys in the batch, and
after inserts into a map that already holds keys (upserts). Queries then
return exactly the known answers. Tolerance: zero (integers)."""
import numpy as np
import pytest

from gpu_util import device_mapping, from_dev, to_dev
from hashinator_gb300 import workloads

pytestmark = pytest.mark.gpu


def _sp(w):
    return 22 if w == 4 else 21  # tables of 32 MiB: 32 and 16 regions of about 1 MiB


@pytest.mark.parametrize("w", [4, 8])
def test_reordered_insert_equals_plain_insert(hx, w):
    sp = _sp(w)
    n = 1 << (sp - 1)
    keys, vals, q, _ = workloads.map_workload(n, w, 606 + w, erase_frac=0.0)
    maps = []
    for mode in (0, 1, -1):
        m = hx.Hashmap(sp, w)
        m.set_insert_partition(mode)
        m.insert(to_dev(keys[: n // 2]), to_dev(vals[: n // 2]), target_lf=0.0)
        # upserts of present keys with new values, and the rest of the keys
        v2 = vals.copy()
        v2[: n // 4] ^= v2.dtype.type(0x5A5A)
        m.insert(to_dev(keys[: n // 4]), to_dev(v2[: n // 4]), target_lf=0.0)
        m.insert(to_dev(keys[n // 2:]), to_dev(vals[n // 2:]), target_lf=0.0)
        assert m.peek_status() == hx.STATUS_SUCCESS
        assert m.info().fill == n
        maps.append(m)
    k0, v0, _ = device_mapping(maps[0], w)
    for m in maps[1:]:
        k, v, _ = device_mapping(m, w)
        np.testing.assert_array_equal(k, k0)
        np.testing.assert_array_equal(v, v0)
    want, _ = workloads.query_expectation(keys, np.concatenate([v2[: n // 4], vals[n // 4:]]), q,
                                          np.iinfo(keys.dtype).max - 5)
    out = to_dev(np.full(len(q), np.iinfo(keys.dtype).max - 5, keys.dtype))
    maps[1].retrieve(to_dev(q), out)
    np.testing.assert_array_equal(from_dev(out, keys.dtype), want)
    for m in maps:
        m.close()


@pytest.mark.parametrize("w", [4, 8])
def test_reordered_pairs_index_and_duplicates(hx, w):
    sp = _sp(w)
    n = 1 << (sp - 2)
    dt = np.uint32 if w == 4 else np.uint64
    keys = workloads.distinct_keys(n, w, 707 + w)
    vals = workloads.values(n, w, 707 + w)
    pairs = np.stack([keys, vals], axis=1).reshape(-1)
    # hash_pair input
    a, b = hx.Hashmap(sp, w), hx.Hashmap(sp, w)
    a.set_insert_partition(1)
    b.set_insert_partition(0)
    for m in (a, b):
        m.insert_pairs(to_dev(pairs), target_lf=0.0)
    ka, va, _ = device_mapping(a, w)
    kb, vb, _ = device_mapping(b, w)
    np.testing.assert_array_equal(ka, kb)
    np.testing.assert_array_equal(va, vb)
    o = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(ka, keys[o])
    np.testing.assert_array_equal(va, vals[o])
    a.close()
    b.close()
    # insertIndex: each key's value is its position in the batch
    c = hx.Hashmap(sp, w)
    c.set_insert_partition(1)
    c.insert_index(to_dev(keys), target_lf=0.0)
    kc, vc, _ = device_mapping(c, w)
    np.testing.assert_array_equal(kc, keys[o])
    np.testing.assert_array_equal(vc, o.astype(dt))
    c.close()
    # duplicate keys (equal values) counted once
    dup = np.concatenate([keys, keys[: n // 3], np.full(1000, keys[7], dt)])
    dv = np.concatenate([vals, vals[: n // 3], np.full(1000, vals[7], dt)])
    perm = np.random.default_rng(5).permutation(len(dup))
    d = hx.Hashmap(sp, w)
    d.set_insert_partition(1)
    d.insert(to_dev(dup[perm]), to_dev(dv[perm]), target_lf=0.0)
    assert d.info().fill == n
    kd, vd, _ = device_mapping(d, w)
    np.testing.assert_array_equal(kd, keys[o])
    np.testing.assert_array_equal(vd, vals[o])
    d.close()
