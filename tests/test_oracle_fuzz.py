"""Randomised operation sequences on the oracle against a plain dict model
(CPU only; the sequences are tests/fuzz_ops.py's): after every step the
oracle's sorted mapping, fill and tombstone count, and every query output,
equal the model's."""
import numpy as np
import pytest

from fuzz_ops import Sequence


@pytest.mark.parametrize("width", [4, 8])
@pytest.mark.parametrize("seed", range(6))
def test_random_sequences_match_a_dict_model(oracle_mod, width, seed):
    seq = Sequence(width, seed)
    om = oracle_mod.OracleMap(seq.sp0, width)
    for op in seq.ops():
        if op[0] == "insert":
            assert om.insert(op[1], op[2], target_lf=0.0) == 0
        elif op[0] == "query":
            out = np.full(len(op[1]), seq.fill, seq.dt)
            om.retrieve(op[1], out)
            np.testing.assert_array_equal(out, op[2])
        elif op[0] == "erase":
            om.erase(op[1])
        elif op[0] == "clean":
            om.clean_tombstones()
        else:
            om.resize(op[1])
        inf = om.info()
        assert (inf["fill"], inf["tombstones"], inf["size_power"]) == (len(seq.model), seq.tomb, seq.sp)
        k, v = om.mapping()
        ek, ev = seq.expected_mapping()
        np.testing.assert_array_equal(k, ek)
        np.testing.assert_array_equal(v, ev)
