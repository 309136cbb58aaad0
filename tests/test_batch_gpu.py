"""Batched maps: one persistent fused launch over a table directory must give,
per map, exactly the results of the plain path (the per-map launches) and of
the oracle: query outputs, mapping, fill and tombstone counts."""
import numpy as np
import pytest

from gpu_util import device_bytes, from_dev, to_dev
from hashinator_gb300 import workloads

pytestmark = pytest.mark.gpu

FILL = 0xA5A5A5A5


def _work(n_maps=40, seed=3, lo=6.0, hi=12.0):
    return workloads.batched_workload(n_maps, seed, log_lo=lo, log_hi=hi)


def _plan(hx, batch, w, dev, clean=True, erase=True):
    d = {k: to_dev(w[k]) for k in ("keys", "vals", "queries", "erase")}
    out = to_dev(np.full(len(w["queries"]), FILL, np.uint32))
    plan = batch.plan(d["keys"], d["vals"], w["ins_offsets"], d["queries"], out, w["query_offsets"],
                      d["erase"] if erase else None, w["erase_offsets"] if erase else None, clean=clean)
    return plan, out, d


def _map_buckets(batch, i):
    import torch
    ptr, n = batch.bucket_data(i)
    torch.cuda.synchronize()
    return device_bytes(ptr, n * 8).cpu().numpy().view(np.uint32).reshape(n, 2)


def _mapping(b):
    sel = b[:, 0] < 0xFFFFFFFE
    k, v = b[sel, 0], b[sel, 1]
    o = np.argsort(k)
    return k[o], v[o]


def _oracle(oracle_mod, w, clean=True, erase=True):
    res = []
    io, qo, eo = w["ins_offsets"], w["query_offsets"], w["erase_offsets"]
    for i, sp in enumerate(w["size_powers"]):
        om = oracle_mod.OracleMap(int(sp), 4)
        om.insert(w["keys"][io[i]:io[i + 1]], w["vals"][io[i]:io[i + 1]], 0.0)
        q = w["queries"][qo[i]:qo[i + 1]]
        out = np.full(len(q), FILL, np.uint32)
        om.retrieve(q, out)
        if erase:
            om.erase(w["erase"][eo[i]:eo[i + 1]])
        if clean:
            om.clean_tombstones()
        res.append((out, om.mapping(), om.info()))
    return res


def _check_against(batch, out, w, ref):
    got = from_dev(out, np.uint32)
    qo = w["query_offsets"]
    for i, (o_out, (ok, ov), oinf) in enumerate(ref):
        np.testing.assert_array_equal(got[qo[i]:qo[i + 1]], o_out, err_msg=f"map {i} queries")
        k, v = _mapping(_map_buckets(batch, i))
        np.testing.assert_array_equal(k, ok, err_msg=f"map {i} keys")
        np.testing.assert_array_equal(v, ov, err_msg=f"map {i} values")
        inf = batch.map_info(i)
        assert (inf.fill, inf.tombstone_counter) == (oinf["fill"], oinf["tombstones"]), i


@pytest.fixture(scope="module")
def small_work():
    return _work()


def test_fused_matches_oracle_and_per_map(hx, oracle_mod, small_work):
    import torch
    w = small_work
    ref = _oracle(oracle_mod, w)
    b1 = hx.Batch(w["size_powers"])
    p1, out1, _ = _plan(hx, b1, w, "cuda")
    p1.run()
    torch.cuda.synchronize()
    assert p1.check() == 0
    _check_against(b1, out1, w, ref)
    b2 = hx.Batch(w["size_powers"])
    p2, out2, _ = _plan(hx, b2, w, "cuda")
    p2.run_per_map()
    torch.cuda.synchronize()
    _check_against(b2, out2, w, ref)


@pytest.mark.parametrize("group", [1, 4, 8, 16, 32])
@pytest.mark.parametrize("block,tile", [(128, 64), (256, 512), (512, 4096)])
def test_every_tuning_is_exact(hx, oracle_mod, small_work, group, block, tile):
    import torch
    w = small_work
    ref = _oracle(oracle_mod, w)
    b = hx.Batch(w["size_powers"])
    p, out, _ = _plan(hx, b, w, "cuda")
    p.set_tuning(group, block, tile)
    p.run()
    torch.cuda.synchronize()
    assert p.check() == 0
    _check_against(b, out, w, ref)


def test_graph_replay_and_reset(hx, oracle_mod, small_work):
    import torch
    w = small_work
    ref = _oracle(oracle_mod, w)
    b = hx.Batch(w["size_powers"])
    p, out, _ = _plan(hx, b, w, "cuda")
    for _ in range(3):
        b.clear()
        out.fill_(int(np.int32(np.uint32(FILL).view(np.int32))))
        p.run_graph()
        torch.cuda.synchronize()
        assert p.check() == 0
        _check_against(b, out, w, ref)


def test_sections_optional(hx, oracle_mod):
    import torch
    w = _work(n_maps=12, seed=9)
    ref = _oracle(oracle_mod, w, clean=False, erase=False)
    b = hx.Batch(w["size_powers"])
    p, out, _ = _plan(hx, b, w, "cuda", clean=False, erase=False)
    p.run()
    torch.cuda.synchronize()
    _check_against(b, out, w, ref)


def test_autotune_keeps_results_exact(hx, oracle_mod):
    import torch
    from hashinator_gb300.autotune import autotune_batch
    w = _work(n_maps=24, seed=5)
    ref = _oracle(oracle_mod, w)
    b = hx.Batch(w["size_powers"])
    p, out, _ = _plan(hx, b, w, "cuda")
    res = autotune_batch(p, b.clear, groups=(1, 8), blocks=(128, 256), tiles=(256, 2048), reps=1)
    assert res["best"] in {(g, bl, t) for g in (1, 8) for bl in (128, 256) for t in (256, 2048)}
    out.fill_(int(np.int32(np.uint32(FILL).view(np.int32))))
    p.run()
    torch.cuda.synchronize()
    _check_against(b, out, w, ref)


def test_bounded_wait_reports_timeout_and_context_survives(hx, oracle_mod):
    """Failure detection without a GPU fault: one map's insert phase is never
    counted off (a flag nothing sets), its later tiles' bounded waits run out,
    the launch returns, the error word says timeout, and the next clean run on
    the same context is exact."""
    import time
    import torch
    w = _work(n_maps=6, seed=21, lo=6.0, hi=7.0)  # one tile per phase per map
    ref = _oracle(oracle_mod, w)
    b = hx.Batch(w["size_powers"])
    p, out, _ = _plan(hx, b, w, "cuda")
    p.inject_stall(0, 0)  # phase 0 (insert) of map 0
    t0 = time.time()
    p.run()
    torch.cuda.synchronize()
    assert p.check() == 1  # a bounded wait ran out
    assert time.time() - t0 < 30
    p.inject_stall(0, 0, enable=False)
    b.clear()
    out.fill_(int(np.int32(np.uint32(FILL).view(np.int32))))
    p.run()
    torch.cuda.synchronize()
    assert p.check() == 0
    _check_against(b, out, w, ref)
