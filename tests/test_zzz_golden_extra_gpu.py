"""GPU parity with the reference's CPU-build golden fixtures on edge cases
(tests/golden/extra/): the u64 / load factor 0.75 pair, queries that all hit
or all miss, erasing every key, tiny tables and a ragged key count. The same
checks as the main golden parity test, under every probe tuning: fill after
insert, every query output buffer before and after the erase, fill and
tombstone counts, and the sorted (key, value) mapping."""
import numpy as np
import pytest

from conftest import golden_extra_cases, load_golden
from gpu_util import device_mapping, from_dev, full_dev, to_dev
from test_map_gpu import TUNINGS, _dt, _tune

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tuning", TUNINGS)
@pytest.mark.parametrize("name", golden_extra_cases())
def test_golden_extra_parity(hx, name, tuning):
    g = load_golden(name)
    w, sp = int(g["key_bytes"]), int(g["size_power"])
    dt = _dt(w)
    m = hx.Hashmap(sp, w)
    _tune(m, tuning)
    m.insert(to_dev(g["keys"]), to_dev(g["vals"]), target_lf=0.0)
    assert m.info().fill == int(g["size_after_insert"])
    assert m.peek_status() == hx.STATUS_SUCCESS
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
