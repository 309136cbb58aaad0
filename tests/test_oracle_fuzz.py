"""Randomised operation sequences on the oracle against a plain dict model
(CPU only): insert batches (fresh keys and upserts of present ones), query
batches (misses keep the pre-fill), erase batches with repeated keys (each
present key counts once), clean_tombstones and resize. After every step the
oracle's sorted mapping, fill and tombstone count equal the model's."""
import numpy as np
import pytest

from hashinator_gb300 import workloads


def _check(om, model, tomb, dt):
    inf = om.info()
    assert inf["fill"] == len(model)
    assert inf["tombstones"] == tomb
    k, v = om.mapping()
    ks = np.array(sorted(model), dtype=dt)
    np.testing.assert_array_equal(k, ks)
    np.testing.assert_array_equal(v, np.array([model[int(x)] for x in ks], dtype=dt))


@pytest.mark.parametrize("width", [4, 8])
@pytest.mark.parametrize("seed", range(6))
def test_random_sequences_match_a_dict_model(oracle_mod, width, seed):
    rng = np.random.default_rng(1000 * width + seed)
    dt = np.uint32 if width == 4 else np.uint64
    sp = int(rng.integers(4, 9))
    universe = workloads.distinct_keys(1 << sp, width, 500 + seed)  # never more keys than buckets
    om = oracle_mod.OracleMap(sp, width)
    model: dict[int, int] = {}
    tomb = 0
    fill_pat = dt(np.iinfo(dt).max - 3)
    for _ in range(60):
        op = rng.choice(["insert", "query", "erase", "clean", "resize"], p=[0.35, 0.3, 0.2, 0.1, 0.05])
        cap = 1 << om.info()["size_power"]
        if op == "insert":
            # at most 85% of the table occupied by keys plus tombstones (insert never reuses a tombstone)
            room = int(0.85 * cap) - len(model) - tomb
            present = np.array(sorted(model), dtype=dt)
            fresh_pool = np.setdiff1d(universe, present)
            n_fresh = int(rng.integers(0, max(0, min(room, len(fresh_pool))) + 1))
            n_up = int(rng.integers(0, len(present) + 1)) if len(present) else 0
            keys = np.concatenate([rng.choice(fresh_pool, n_fresh, replace=False) if n_fresh else fresh_pool[:0],
                                   rng.choice(present, n_up, replace=False) if n_up else present[:0]]).astype(dt)
            rng.shuffle(keys)
            vals = rng.integers(0, np.iinfo(dt).max, size=len(keys), dtype=dt, endpoint=True)
            assert om.insert(keys, vals, target_lf=0.0) == 0
            for k, v in zip(keys.tolist(), vals.tolist()):
                model[k] = v
        elif op == "query":
            q = rng.choice(universe, int(rng.integers(1, 64)), replace=True).astype(dt)
            out = np.full(len(q), fill_pat, dt)
            om.retrieve(q, out)
            want = np.array([model.get(int(k), int(fill_pat)) for k in q], dtype=dt)
            np.testing.assert_array_equal(out, want)
        elif op == "erase":
            e = rng.choice(universe, int(rng.integers(1, 32)), replace=True).astype(dt)  # repeats on purpose
            om.erase(e)
            for k in set(e.tolist()):
                if k in model:
                    del model[k]
                    tomb += 1
        elif op == "clean":
            om.clean_tombstones()
            tomb = 0
        else:
            new_sp = int(np.clip(om.info()["size_power"] + rng.integers(0, 2), sp, 12))
            om.resize(new_sp)
            tomb = 0
        _check(om, model, tomb, dt)
