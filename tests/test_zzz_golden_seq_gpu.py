"""GPU parity of libhx against the reference's CPU build on operation
sequences (insert after erase, upserts of present keys, clean followed by
inserts; tests/golden/seq/) under several probe tunings, and on the plain
single-map workload at its full size (2^20 u32 keys into 2^21 buckets,
2^21 queries, 25% erased) through the digests of the reference's outputs.
Exact: tolerance zero. Collected late, so a failure here comes after every
other GPU result."""
import numpy as np
import pytest

import golden_replay
from gpu_util import device_mapping, from_dev, to_dev

pytestmark = pytest.mark.gpu


class _LibhxAdapter:
    def __init__(self, hx, sp, kb, tuning):
        self.hx, self.kb, self.sp = hx, kb, sp
        self.m = hx.Hashmap(sp, kb)
        if tuning:
            self.m.set_tuning(group_width=tuning)
        self.dt = np.uint32 if kb == 4 else np.uint64

    def insert(self, k, v):
        self.m.insert(to_dev(k), to_dev(v), target_lf=0.0)
        assert self.m.peek_status() == self.hx.STATUS_SUCCESS

    def retrieve(self, q, out):
        d = to_dev(out)
        self.m.retrieve(to_dev(q), d)
        out[:] = from_dev(d, self.dt)

    def erase(self, k):
        self.m.erase(to_dev(k))

    def clean(self, sp):
        if sp == self.sp:
            self.m.clean_tombstones()
            assert self.m.info().tombstone_counter == 0
        else:
            self.m.resize(sp)
            self.sp = sp

    def fill(self):
        return int(self.m.info().fill)

    def mapping(self):
        k, v, _ = device_mapping(self.m, self.kb)
        return k, v


@pytest.mark.parametrize("tuning", [0, 1, 4, 32])
@pytest.mark.parametrize("name", golden_replay.seq_cases())
def test_sequences_match_reference(hx, name, tuning):
    g = golden_replay.load_seq(name)
    a = _LibhxAdapter(hx, int(g["size_power"]), int(g["key_bytes"]), tuning)
    golden_replay.replay(g, a)
    a.m.close()


@pytest.mark.parametrize("tuning", [0, 1])
def test_full_size_plain_map_matches_reference(hx, tuning):
    d = golden_replay.cfg1_expected()
    a = _LibhxAdapter(hx, d["size_power"], 4, tuning)
    golden_replay.check_cfg1(a, d)
    a.m.close()
