"""Serving loop: requests batched into rounds (continuous batching, several
rounds in flight, growth by on-device rehash) must give every request the same
result it gets when the requests of its map are replayed one by one, in
admission order, through the plain per-map path. Tolerance: zero (integers)."""
import numpy as np
import pytest

from gpu_util import device_bytes, from_dev, to_dev
import hashinator_gb300 as hxm
from hashinator_gb300 import workloads

pytestmark = pytest.mark.gpu

FILL = 0xA5A5A5A5A5A5A5A5


def _mapping_from(ptr, n, width):
    import torch
    dt = np.uint32 if width == 4 else np.uint64
    torch.cuda.synchronize()
    b = device_bytes(ptr, n * 2 * width).cpu().numpy().view(dt).reshape(n, 2)
    e = np.iinfo(dt).max
    sel = (b[:, 0] != e) & (b[:, 0] != e - 1)
    k, v = b[sel, 0], b[sel, 1]
    o = np.argsort(k)
    return k[o], v[o]


def _setup(hx, t, width=8, **kw):
    srv = hx.Server(key_bytes=width, **kw)
    ids = [srv.add_map(int(sp)) for sp in t["size_powers"]]
    d = {"ik": to_dev(t["init_keys"]), "iv": to_dev(t["init_vals"]), "rk": to_dev(t["req_keys"]),
         "rv": to_dev(t["req_vals"])}
    fill = FILL if width == 8 else 0xA5A5A5A5
    d["out"] = to_dev(np.full(len(t["req_keys"]), fill, np.uint64 if width == 8 else np.uint32))
    io = t["init_offsets"]
    init = [(ids[m], hxm.OP_INSERT, d["ik"].data_ptr() + int(io[m]) * width,
             d["iv"].data_ptr() + int(io[m]) * width, 0, int(io[m + 1] - io[m]), m) for m in range(len(ids))]
    ro = t["req_offsets"]
    reqs = []
    for i in range(len(t["req_map"])):
        a = int(ro[i]) * width
        reqs.append((int(t["req_map"][i]), int(t["req_op"][i]), d["rk"].data_ptr() + a, d["rv"].data_ptr() + a,
                     d["out"].data_ptr() + a, int(t["req_n"][i]), 1_000_000 + i))
    return srv, ids, d, init, reqs


def _make_room(hm, n, lim=0.8):
    """The serving maintenance rule with exact counts: rehash (dropping
    tombstones, growing only if the live keys need it) when fill + tombstones
    + n would pass the load-factor limit."""
    inf = hm.info()
    if inf.fill + inf.tombstone_counter + n > lim * inf.bucket_count:
        sp = inf.size_power
        while inf.fill + n > lim * (1 << sp):
            sp += 1
        hm.resize(sp)


def _replay(hx, t, width, statuses):
    """The requests of each map, one by one in admission order, through hx.Hashmap."""
    dt = np.uint32 if width == 4 else np.uint64
    fill = FILL if width == 8 else 0xA5A5A5A5
    ro, io = t["req_offsets"], t["init_offsets"]
    out = np.full(len(t["req_keys"]), fill, dt)
    maps = []
    for m, sp in enumerate(t["size_powers"]):
        hm = hx.Hashmap(int(sp), width)
        _make_room(hm, int(io[m + 1] - io[m]))
        hm.insert(to_dev(t["init_keys"][io[m]:io[m + 1]]), to_dev(t["init_vals"][io[m]:io[m + 1]]), target_lf=0.0)
        maps.append(hm)
    for i in range(len(t["req_map"])):
        if statuses is not None and statuses[i] != 0:
            continue  # not admitted by the server: not applied
        m, op = int(t["req_map"][i]), int(t["req_op"][i])
        k = to_dev(t["req_keys"][ro[i]:ro[i + 1]])
        if op == 0:
            _make_room(maps[m], int(ro[i + 1] - ro[i]))
            maps[m].insert(k, to_dev(t["req_vals"][ro[i]:ro[i + 1]]), target_lf=0.0)
            assert maps[m].peek_status() == hx.STATUS_SUCCESS
        elif op == 1:
            o = to_dev(out[ro[i]:ro[i + 1]])
            maps[m].retrieve(k, o)
            out[ro[i]:ro[i + 1]] = from_dev(o, dt)
        else:
            maps[m].erase(k)
    return out, maps


@pytest.mark.parametrize("width", [8, 4])
def test_each_result_same_alone_and_in_the_mix(hx, width):
    import torch
    t = workloads.serving_trace(16, 1500, 77 + width, init_log=(4.0, 10.0), size_log=(0.0, 10.0), width=width)
    srv, ids, d, init, reqs = _setup(hx, t, width, memory_budget=1 << 32, max_round_requests=64,
                                     max_round_keys=1 << 14, rounds_in_flight=3)
    srv.submit(init)
    srv.drain()
    srv.poll()
    srv.submit(reqs)
    srv.drain()
    comps = {tag: st for tag, _, st in srv.poll()}
    assert len(comps) == len(reqs) and all(st == 0 for st in comps.values())
    torch.cuda.synchronize()
    dt = np.uint32 if width == 4 else np.uint64
    got = from_dev(d["out"], dt)
    want, maps = _replay(hx, t, width, None)
    np.testing.assert_array_equal(got, want)
    grew = 0
    for m in range(len(ids)):
        ptr, n = srv.bucket_data(ids[m])
        grew += n > (1 << int(t["size_powers"][m]))
        k, v = _mapping_from(ptr, n, width)
        p2, n2 = maps[m].bucket_data()
        k2, v2 = _mapping_from(p2, n2, width)
        np.testing.assert_array_equal(k, k2)
        np.testing.assert_array_equal(v, v2)
        inf, inf2 = srv.map_info(ids[m]), maps[m].info()
        assert inf.fill == inf2.fill and (inf.fill + inf.tombstone_counter) / n <= 0.8 + 1e-9
        assert inf.err != hx.STATUS_FAIL  # no insert ever ran out of buckets
    assert grew > 0  # the trace grew some tables on the device


def test_budget_rejects_growth_and_new_maps(hx):
    import torch
    width = 8
    t = workloads.serving_trace(4, 200, 5, init_log=(6.0, 8.0), size_log=(6.0, 9.0), mix=(1.0, 0.0, 0.0),
                                width=width)
    table_bytes = sum((1 << int(sp)) * 16 for sp in t["size_powers"])
    srv, ids, d, init, reqs = _setup(hx, t, width, memory_budget=table_bytes + 4096, max_round_requests=16,
                                     max_round_keys=1 << 12)
    assert srv.try_add_map(12) is None  # over the budget: not admitted
    srv.submit(init)
    srv.drain()
    srv.poll()
    srv.submit(reqs)
    srv.drain()
    st = {tag - 1_000_000: s for tag, _, s in srv.poll()}
    statuses = np.array([st[i] for i in range(len(reqs))])
    assert (statuses == hx.HX_ERR_OOM).any() and (statuses == 0).any()
    used, budget = srv.memory()
    assert used <= budget
    torch.cuda.synchronize()
    _, maps = _replay(hx, t, width, statuses)
    for m in range(len(ids)):
        ptr, n = srv.bucket_data(ids[m])
        k, v = _mapping_from(ptr, n, width)
        p2, n2 = maps[m].bucket_data()
        k2, v2 = _mapping_from(p2, n2, width)
        np.testing.assert_array_equal(k, k2)
        np.testing.assert_array_equal(v, v2)


def test_real_time_trace(hx):
    import torch
    width = 8
    t = workloads.serving_trace(32, 3000, 9, init_log=(6.0, 12.0), size_log=(0.0, 12.0), rate_req_s=2e5,
                                width=width)
    srv, ids, d, init, reqs = _setup(hx, t, width, memory_budget=1 << 33, max_round_requests=256,
                                     max_round_keys=1 << 18)
    srv.submit(init)
    srv.drain()
    srv.poll()
    comp, st = srv.run_trace(reqs, t["arrival_ns"])
    assert (st == 0).all()
    assert (comp >= t["arrival_ns"]).all()
    torch.cuda.synchronize()
    dt = np.uint64
    want, _ = _replay(hx, t, width, None)
    np.testing.assert_array_equal(from_dev(d["out"], dt), want)
