"""Randomised operation sequences (tests/fuzz_ops.py) on libhx under several
probe tunings, against the dict model that the oracle is checked against on
CPU: after every insert, query, erase, clean_tombstones and resize, the
device map's fill, tombstone count, size power and sorted (key, value)
mapping, and every query output buffer, equal the model's."""
import numpy as np
import pytest

from fuzz_ops import Sequence
from gpu_util import device_mapping, from_dev, full_dev, to_dev
from test_map_gpu import _tune

pytestmark = pytest.mark.gpu

# (group width, keys per thread, blind insert CAS, window bytes); group 0 = automatic policy
FUZZ_TUNINGS = [(0, 0, True, 32), (1, 4, True, 32), (1, 2, False, 64), (4, 1, False, 32), (32, 1, True, 32)]


@pytest.mark.parametrize("tuning", FUZZ_TUNINGS)
@pytest.mark.parametrize("width", [4, 8])
@pytest.mark.parametrize("seed", range(4))
def test_random_sequences_match_the_model(hx, seed, width, tuning):
    seq = Sequence(width, seed)
    m = hx.Hashmap(seq.sp0, width)
    _tune(m, tuning)
    for op in seq.ops():
        if op[0] == "insert":
            if len(op[1]):
                m.insert(to_dev(op[1]), to_dev(op[2]), target_lf=0.0)
                assert m.peek_status() == hx.STATUS_SUCCESS
        elif op[0] == "query":
            out = full_dev(len(op[1]), int(seq.fill), width)
            m.retrieve(to_dev(op[1]), out)
            np.testing.assert_array_equal(from_dev(out, seq.dt), op[2])
        elif op[0] == "erase":
            m.erase(to_dev(op[1]))
        elif op[0] == "clean":
            m.clean_tombstones()
        else:
            m.resize(op[1])
        inf = m.info()
        assert (inf.fill, inf.tombstone_counter, inf.size_power) == (len(seq.model), seq.tomb, seq.sp), op[0]
        k, v, _ = device_mapping(m, width)
        ek, ev = seq.expected_mapping()
        np.testing.assert_array_equal(k, ek)
        np.testing.assert_array_equal(v, ev)
    m.close()
