"""The large single map at its full size (2^27 buckets; 2^26 .. 0.9 * 2^27
keys, u32 and u64), checked through properties that do not need the serial
oracle: keys are distinct, so the expected result of every query is known
exactly. Checked whole, on the device: every query output after insert,
after erasing 30% and after clean_tombstones; fill and tombstone counts; and
the set of keys that extractAllKeys returns. Tolerance: zero (integers)."""
import numpy as np
import pytest

import hashinator_gb300 as hxm
from hashinator_gb300 import workloads

pytestmark = pytest.mark.gpu

SP = 27


def _dev(a, torch):
    sig = np.int32 if a.dtype == np.uint32 else np.int64
    return torch.from_numpy(np.ascontiguousarray(a).view(sig)).cuda()


@pytest.mark.parametrize("lf", [0.5, 0.75, 0.9])
@pytest.mark.parametrize("w", [4, 8])
def test_large_map_full_size(hx, w, lf):
    import torch
    n = int(lf * (1 << SP))
    keys = workloads.distinct_keys(n, w, 901 + w)
    vals = workloads.values(n, w, 901 + w)
    dt = keys.dtype
    rng = np.random.default_rng(w * 100 + int(lf * 100))
    hsel = workloads.affine_sample(n, n // 2, rng)  # indices of the keys queried as hits
    miss = workloads.distinct_keys(n - n // 2, w, 901 + w, offset=n + 4096)
    perm = workloads.affine_sample(n, n, rng)
    q = np.concatenate([keys[hsel], miss])[perm]
    src = np.concatenate([hsel, np.full(len(miss), -1, np.int64)])[perm]  # inserted index, or -1 for a miss
    fill = np.iinfo(dt).max - 7  # output pre-fill; a hit whose value equals it still compares equal
    esel = workloads.affine_sample(n, int(0.3 * n), rng)
    erased = np.zeros(n, bool)
    erased[esel] = True

    def expect(after_erase):
        e = np.full(n, fill, dt)
        hit = src >= 0
        if after_erase:
            hit &= ~erased[np.where(src >= 0, src, 0)]
        e[hit] = vals[src[hit]]
        return _dev(e, torch)

    dk, dv, dq = _dev(keys, torch), _dev(vals, torch), _dev(q, torch)
    m = hx.Hashmap(SP, w)
    m.insert(dk, dv, target_lf=0.0)
    assert m.peek_status() == hx.STATUS_SUCCESS
    inf = m.info()
    assert inf.size_power == SP and inf.fill == n and inf.tombstone_counter == 0

    def query_equals(after_erase):
        out = _dev(np.full(n, fill, dt), torch)
        m.retrieve(dq, out)
        return bool(torch.equal(out, expect(after_erase)))

    assert query_equals(False)
    m.erase(_dev(keys[esel], torch))
    inf = m.info()
    assert inf.fill == n - len(esel) and inf.tombstone_counter == len(esel)
    assert query_equals(True)
    m.clean_tombstones()
    inf = m.info()
    assert inf.fill == n - len(esel) and inf.tombstone_counter == 0
    assert query_equals(True)
    # the live key set, through extractAllKeys, equals the inserted minus the erased keys
    live = _dev(keys[~erased], torch)
    ek = torch.empty(n, dtype=live.dtype, device="cuda")
    c = m.extract_all_keys(ek)
    assert c == n - len(esel)
    assert torch.equal(torch.sort(ek[:c]).values, torch.sort(live).values)
    # no TOMBSTONE left after clean: a rule that selects the tombstone key finds nothing
    tomb = int(np.iinfo(dt).max) - 1
    small = torch.empty(64, dtype=live.dtype, device="cuda")
    assert m.extract_keys_by_pattern(hxm.Pred(hxm.PRED_EQ, hxm.FIELD_KEY, tomb), small) == 0
    m.close()
