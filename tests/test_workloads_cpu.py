"""The seeded synthetic workloads have the shapes and distributions the
benchmarks and GPU tests rely on: distinct sentinel-free keys, exact hit and
erase fractions, load factor 0.5 tables, velocity-block ids from a 30-60 cell
shell of a 200^3 grid, Poisson arrivals and the request mix of the serving
trace. CPU only."""
import numpy as np
import pytest

from hashinator_gb300 import workloads as wl


@pytest.mark.parametrize("width", [4, 8])
def test_distinct_keys_and_disjoint_offsets(width):
    n = 1 << 16
    k = wl.distinct_keys(n, width, 3)
    assert len(k) == n and len(np.unique(k)) == n
    empty = np.iinfo(k.dtype).max
    assert not np.any((k == empty) | (k == empty - 1))
    assert np.array_equal(k, wl.distinct_keys(n, width, 3))  # a pure function of (n, width, seed)
    far = wl.distinct_keys(n, width, 3, offset=n + 64)
    assert len(np.intersect1d(k, far)) == 0
    assert not np.array_equal(k, wl.distinct_keys(n, width, 4))


@pytest.mark.parametrize("width", [4, 8])
@pytest.mark.parametrize("hit_frac", [0.0, 0.5, 1.0])
def test_map_workload_fractions(width, hit_frac):
    n = 5000
    keys, vals, q, er = wl.map_workload(n, width, 11, hit_frac=hit_frac, erase_frac=0.25)
    assert len(vals) == n and vals.dtype == keys.dtype
    assert len(q) == n
    assert int(np.isin(q, keys).sum()) == round(n * hit_frac)
    assert len(er) == round(n * 0.25) and len(np.unique(er)) == len(er) and np.isin(er, keys).all()


@pytest.mark.parametrize("n,k", [(1, 1), (10, 10), (97, 40), (1 << 12, 1 << 12), (1000, 0)])
def test_affine_sample_distinct(n, k):
    s = wl.affine_sample(n, k, np.random.default_rng(n + k))
    assert len(s) == k and len(np.unique(s)) == k
    if k:
        assert s.min() >= 0 and s.max() < n


def test_large_map_workload_fractions():
    n = 1 << 15
    keys, _, q, er = wl.large_map_workload(n, 4, 5)
    assert len(np.unique(keys)) == n
    assert len(np.unique(q)) == n and int(np.isin(q, keys).sum()) == n // 2
    assert len(er) == round(0.3 * n) and len(np.unique(er)) == len(er) and np.isin(er, keys).all()


def test_batched_workload_shapes():
    n_maps, grid = 96, 200
    w = wl.batched_workload(n_maps, 4096)
    n = w["n"]
    assert len(n) == n_maps and n.min() >= 64 and n.max() <= 1 << 16
    lg = np.log2(n)
    assert 9.5 < lg.mean() < 12.5  # log-uniform on [6, 16]: mean 11
    sp = w["size_powers"]
    assert np.array_equal(sp, np.ceil(np.log2(n / 0.5)).astype(np.int32))
    lf = n / (2.0 ** sp)
    assert (lf <= 0.5).all() and (lf > 0.25).all()
    io, qo, eo = (w[k].astype(np.int64) for k in ("ins_offsets", "query_offsets", "erase_offsets"))
    assert io[-1] == len(w["keys"]) == len(w["vals"]) and qo[-1] == len(w["queries"]) and eo[-1] == len(w["erase"])
    for i in range(n_maps):
        k = w["keys"][io[i]:io[i + 1]]
        q = w["queries"][qo[i]:qo[i + 1]]
        e = w["erase"][eo[i]:eo[i + 1]]
        assert len(k) == n[i] and len(np.unique(k)) == n[i]
        assert len(q) == n[i] and len(np.unique(q)) == n[i]
        assert int(np.isin(q, k).sum()) == int(np.rint(n[i] * 0.7))
        assert len(e) == int(np.rint(n[i] * 0.1)) and len(np.unique(e)) == len(e) and np.isin(e, k).all()
        # velocity-block ids of a 200^3 grid, inside one 30-60 cell shell (extent at most 121 cells per axis)
        allids = np.concatenate([k, q]).astype(np.int64)
        x, y, z = allids % grid, (allids // grid) % grid, allids // (grid * grid)
        assert z.max() < grid
        for c in (x, y, z):
            assert c.max() - c.min() <= 120
        c = np.array([x.mean(), y.mean(), z.mean()])
        d = np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2)
        assert d.max() <= 60 + 10 and (n[i] < 4096 or d.min() >= 30 - 10)


def test_shell_offsets_radii():
    s = wl.shell_offsets().astype(np.int64)
    r2 = (s * s).sum(axis=1)
    assert r2.min() >= 900 and r2.max() <= 3600 and len(np.unique(s, axis=0)) == len(s)


@pytest.mark.parametrize("width", [4, 8])
def test_serving_trace_properties(width):
    n_maps, n_req, rate = 16, 4000, 2e5
    t = wl.serving_trace(n_maps, n_req, 13, init_log=(4.0, 8.0), size_log=(0.0, 8.0), rate_req_s=rate, width=width)
    arr = t["arrival_ns"].astype(np.int64)
    assert (np.diff(arr) >= 0).all()
    assert abs(arr[-1] / n_req - 1e9 / rate) < 0.1 * 1e9 / rate  # mean gap of a Poisson process
    ops = t["req_op"]
    for op, p in enumerate((0.2, 0.7, 0.1)):
        assert abs((ops == op).mean() - p) < 0.03
    rn = t["req_n"]
    assert rn.min() >= 1 and rn.max() <= 256
    assert t["req_offsets"][-1] == len(t["req_keys"]) == len(t["req_vals"]) == rn.sum()
    n0 = t["n0"]
    assert np.array_equal(t["size_powers"], np.maximum(np.ceil(np.log2(n0 / 0.5)), 2).astype(np.int32))
    # replay per map: inserts bring keys never inserted before; erases name keys inserted before
    io, ro = t["init_offsets"], t["req_offsets"]
    inserted = [set(t["init_keys"][io[m]:io[m + 1]].tolist()) for m in range(n_maps)]
    for m in range(n_maps):
        assert len(inserted[m]) == n0[m]
    present = total_q = 0
    for i in range(n_req):
        m, op = int(t["req_map"][i]), int(t["req_op"][i])
        k = t["req_keys"][ro[i]:ro[i + 1]].tolist()
        if op == 0:
            assert not (set(k) & inserted[m]) and len(set(k)) == len(k)
            inserted[m].update(k)
        elif op == 1:
            present += sum(x in inserted[m] for x in k)
            total_q += len(k)
        else:
            assert all(x in inserted[m] for x in k)
    assert abs(present / total_q - 0.8) < 0.03
    if width == 8:
        allk = [x for s in inserted for x in s]
        assert len(allk) == len(set(allk))  # maps never share keys
