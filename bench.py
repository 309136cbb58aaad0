"""Benchmark of the Hashinator hot path on GB300.

Workload (one step): the large single-map configuration with 32-bit keys and
values — clear a table of 2^27 buckets, insert 2^26 distinct keys (load
factor 0.5), then retrieve 2^26 queries of which half are present and half
absent. Metric: insert + query throughput in Mkeys/s (2 x 2^26 keys per step).
The table (1 GiB) and key arrays (256 MiB each) are larger than L2 (129 MB),
so no L2 flush is needed between steps.

value: device-resident inputs, CUDA events around the K timed steps.
e2e:   the same step through the C ABI with pinned HOST buffers: the H2D copy
       of keys, values and queries and the D2H copy of the query results are
       inside the timed region.
roofline: the dominant kernel's algorithmic bytes (insert 72 B/key, query
       40 B/key: key+value in, one 32 B bucket sector read, written back for
       insert) over its event-timed duration, against the measured HBM copy
       bandwidth (MEASURED_PEAKS.json).
cpu_baseline: the oracle's serial C restatement of the reference's CPU path on
       a bounded sample (2^24 keys into 2^25 buckets, same load factor), as
       one serial map per host thread (keys sharded by home bucket) and on one
       core; beside it, the streaming primitives on 2^24 u32 (one core and all
       host threads).

--impl reference times the reference's CPU implementation of the path (the
oracle port of it on this machine) on the same metric.
Multi-GPU: replicas only (each rank runs the same single-map workload on its
own GPU; value is the sum over ranks).
"""
from __future__ import annotations

import argparse
import functools
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

INSERT_BYTES_PER_KEY = {4: 72, 8: 80}
QUERY_BYTES_PER_KEY = {4: 40, 8: 48}
HEADLINE_FILL = 0xA5A5A5A5  # query-output pre-fill of the headline step
METRIC = "insert+query Mkeys/s (u32 keys/values, 2^26 keys, 2^27 buckets, LF 0.5, 50% hit queries)"
DATA = "synthetic (seeded bijective keys, PCG64 values)"


def headline_metric(log_keys: int) -> str:
    """The headline metric string for 2^log_keys keys in 2^(log_keys+1) buckets."""
    return METRIC if log_keys == 26 else METRIC.replace("2^26 keys, 2^27", f"2^{log_keys} keys, 2^{log_keys + 1}")


def headline_config(log_keys: int, group: int) -> dict:
    """The headline workload's config; both arms report it."""
    return {"workload": f"single map u32/u32: clear + insert 2^{log_keys} + retrieve 2^{log_keys} (50% hit)",
            "size_power": log_keys + 1, "keys": 1 << log_keys, "load_factor": 0.5, "parallelism": "replicas",
            "l2": "inputs larger than L2 (1 GiB table, 256 MiB arrays); no flush",
            "group_width": group or "default"}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def traffic_from_profiles(kernel_tag: str):
    """Per-launch DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one kernel at the headline size,
    from the ncu capture recorded in profiles/roofline_traffic.json (each entry carries the command that
    produced it), or None when no capture of that kernel exists."""
    p = ROOT / "profiles" / "roofline_traffic.json"
    try:
        d = json.loads(p.read_text())
        e = d["kernels"].get(kernel_tag)
        return None if e is None else float(e["dram_bytes_per_launch"])
    except Exception:  # noqa: BLE001
        return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    from hashinator_gb300.dist import env_ranks
    return env_ranks()


def _shard_of(keys, sp, shard_bits):
    """Top shard_bits of each key's home bucket in a table of 2^sp buckets (the Fibonacci hash)."""
    k = keys.astype(np.uint64)
    if keys.dtype == np.uint32:
        k = k ^ (k >> np.uint64(32 - sp))
        h = (k * np.uint64(2654435769)) >> np.uint64(32 - sp)
        h &= np.uint64((1 << sp) - 1)
    else:
        k = k ^ (k >> np.uint64(64 - sp))
        h = (k * np.uint64(11400714819323198485)) >> np.uint64(64 - sp)
    return (h >> np.uint64(sp - shard_bits)).astype(np.int64)


@functools.lru_cache(maxsize=4)
def _cpu_parts(width: int, log_n: int, tb: int):
    """The CPU sample (keys, values, queries), split into 2^tb shards; generated once per process."""
    from hashinator_gb300 import workloads
    keys, vals, q, _ = workloads.map_workload(1 << log_n, width, 1234, erase_frac=0.0)
    if not tb:
        return [(keys, vals, q)]
    ks, qs = _shard_of(keys, log_n + 1, tb), _shard_of(q, log_n + 1, tb)
    return [(np.ascontiguousarray(keys[ks == i]), np.ascontiguousarray(vals[ks == i]),
             np.ascontiguousarray(q[qs == i])) for i in range(1 << tb)]


def cpu_insert_query(width: int = 4, log_n: int = 24, threads: int = 1, reps: int = 1):
    """The reference's CPU path (the oracle port: serial insert + find) on a bounded sample: 2^log_n keys into
    2^(log_n+1) buckets, then 2^log_n queries (50% hit). With threads > 1 (a power of two) the host runs one
    serial map per thread, keys sharded by the top bits of their home bucket, each map a slice of the table at the
    same load factor; the oracle's calls release the GIL. Returns (Mkeys/s, insert Mkeys/s, query Mkeys/s, s)."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor
    n = 1 << log_n
    tb = max(0, threads.bit_length() - 1)
    sp = log_n + 1
    parts = _cpu_parts(width, log_n, tb)
    outs = [np.zeros(len(p[2]), p[0].dtype) for p in parts]
    best = None
    with ThreadPoolExecutor(max_workers=len(parts)) as ex:
        for _ in range(reps):
            maps = [oracle.OracleMap(sp - tb, width) for _ in parts]
            t0 = time.perf_counter()
            list(ex.map(lambda i: maps[i].insert(parts[i][0], parts[i][1], 0.0), range(len(parts))))
            t1 = time.perf_counter()
            list(ex.map(lambda i: maps[i].retrieve(parts[i][2], outs[i]), range(len(parts))))
            t2 = time.perf_counter()
            del maps
            if best is None or t2 - t0 < best[2] - best[0]:
                best = (t0, t1, t2)
    t0, t1, t2 = best
    return 2 * n / (t2 - t0) / 1e6, n / (t1 - t0) / 1e6, n / (t2 - t1) / 1e6, t2 - t0


def host_cpu() -> dict:
    """The host the CPU baseline ran on: logical CPUs and the CPU model (lscpu, else /proc/cpuinfo)."""
    import platform
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().lower().startswith("model name"):
                model = ln.split(":", 1)[1].strip()
                break
    except Exception:  # noqa: BLE001
        pass
    if not model:
        try:
            for ln in Path("/proc/cpuinfo").read_text().splitlines():
                if ln.lower().startswith("model name"):
                    model = ln.split(":", 1)[1].strip()
                    break
        except Exception:  # noqa: BLE001
            pass
    return {"nproc": os.cpu_count(), "cpu_model": model or platform.processor() or "unknown",
            "arch": platform.machine()}


def host_threads() -> int:
    """Host threads for the CPU baseline: the largest power of two not above the core count."""
    c = os.cpu_count() or 1
    return 1 << (c.bit_length() - 1)


def cpu_baseline(width: int = 4, log_n: int = 24):
    """The CPU baseline reported beside the GPU number: all host threads (sharded serial maps) and one core."""
    t = host_threads()
    v, vi, vq, secs = cpu_insert_query(width, log_n, t)
    v1, vi1, vq1, secs1 = cpu_insert_query(width, log_n, 1)
    return {"value": round(v, 3), "unit": "Mkeys/s", "cores": t, "kind": "port",
            "sample": f"2^{log_n} u32 keys into 2^{log_n + 1} buckets (LF 0.5) + 2^{log_n} queries 50% hit; "
                      f"{t} serial maps (the reference's CPU path restated), keys sharded by the top bits of their "
                      f"home bucket; insert {vi:.1f} Mkeys/s, query {vq:.1f} Mkeys/s",
            "single_core": {"value": round(v1, 3), "insert_Mkeys_s": round(vi1, 1), "query_Mkeys_s": round(vq1, 1)},
            "seconds": round(secs + secs1, 3), "host": _guarded(host_cpu), "streaming": _guarded(cpu_streaming)}


def _guarded(fn):
    """fn() or, if it raises, a record of the error (an optional section never ends the run)."""
    try:
        return fn()
    except Exception as e:  # noqa: BLE001
        return {"error": f"{type(e).__name__}: {e}"}


def cpu_batched(w: dict, gpu_out=None, threads: int | None = None, reps: int = 2) -> dict:
    """CPU baseline of one batched round: for every map, the oracle's serial map (the reference's CPU path
    restated) is created empty at its size power, then insert all (no growth), query, erase, clean_tombstones
    — the same round as the fused GPU launch, maps dealt round-robin to host threads (the oracle's calls release
    the GIL). If gpu_out (the fused launch's query outputs, pre-filled with all ones) is given, the CPU query
    outputs are compared with it element for element."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor
    t = threads or host_threads()
    io, qo, eo = (w[k].astype(np.int64) for k in ("ins_offsets", "query_offsets", "erase_offsets"))
    sp = w["size_powers"]
    keys, vals, qs, er = (np.ascontiguousarray(w[k]).view(np.uint32) for k in ("keys", "vals", "queries", "erase"))
    out = np.full(len(qs), 0xFFFFFFFF, np.uint32)

    def work(tid):
        for i in range(tid, len(sp), t):
            m = oracle.OracleMap(int(sp[i]), 4)
            m.insert(keys[io[i]:io[i + 1]], vals[io[i]:io[i + 1]], 0.0)
            m.retrieve(qs[qo[i]:qo[i + 1]], out[qo[i]:qo[i + 1]])
            m.erase(er[eo[i]:eo[i + 1]])
            m.clean_tombstones()
            del m

    best = None
    with ThreadPoolExecutor(max_workers=t) as ex:
        for _ in range(reps):
            out.fill(0xFFFFFFFF)
            t0 = time.perf_counter()
            list(ex.map(work, range(t)))
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
    n_ops = len(keys) + len(qs) + len(er)
    r = {"ms": round(best * 1e3, 1), "Mops_s": round(n_ops / best / 1e6, 1), "threads": t, "kind": "port",
         "sample": "the whole round (every map), one serial map per map, maps dealt round-robin to host threads"}
    if gpu_out is not None:
        r["query_outputs_equal_gpu"] = bool(np.array_equal(out, np.asarray(gpu_out).view(np.uint32)))
    return r


SERVE_FILL = 0xA5A5A5A5A5A5A5A5  # query-output pre-fill of the CPU replay (misses leave it)


def cpu_serving(tr: dict, gpu_out=None, threads: int | None = None, max_lf: float = 0.8) -> dict:
    """CPU baseline of the serving workload: every map an oracle serial map (the reference's CPU path restated),
    maps dealt round-robin to host threads, each thread replaying its maps' requests in admission order (the
    trace's order) with the server's maintenance rule: before an insert that would take keys plus tombstones past
    max_lf, rehash (dropping tombstones, growing while the live keys need it). The initial inserts are not timed,
    as on the GPU. If gpu_out (the serving run's query outputs, 64-bit) is given, it is compared with the CPU's
    at every query position where the CPU found the key (the GPU buffer is not pre-filled, so misses are not
    compared)."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor
    t = threads or host_threads()
    sps = tr["size_powers"]
    nm = len(sps)
    io, ro = tr["init_offsets"].astype(np.int64), tr["req_offsets"].astype(np.int64)
    rmap, rop = tr["req_map"], tr["req_op"]
    ik, iv, rk, rv = (np.ascontiguousarray(tr[k]).view(np.uint64)
                      for k in ("init_keys", "init_vals", "req_keys", "req_vals"))
    out = np.full(len(rk), SERVE_FILL, np.uint64)
    order = np.argsort(rmap, kind="stable")
    starts = np.searchsorted(rmap[order], np.arange(nm + 1))
    maps = [None] * nm
    growths = [0] * t

    def init(tid):
        for m in range(tid, nm, t):
            om = oracle.OracleMap(int(sps[m]), 8)
            om.insert(ik[io[m]:io[m + 1]], iv[io[m]:io[m + 1]], 0.0)
            maps[m] = om

    def replay(tid):
        for m in range(tid, nm, t):
            om = maps[m]
            for i in order[starts[m]:starts[m + 1]].tolist():
                a, b = int(ro[i]), int(ro[i + 1])
                op = int(rop[i])
                if op == 0:
                    inf = om.info()
                    sp = inf["size_power"]
                    if inf["fill"] + inf["tombstones"] + (b - a) > max_lf * (1 << sp):
                        while inf["fill"] + (b - a) > max_lf * (1 << sp):
                            sp += 1
                        om.resize(sp)
                        growths[tid] += 1
                    om.insert(rk[a:b], rv[a:b], 0.0)
                elif op == 1:
                    om.retrieve(rk[a:b], out[a:b])
                else:
                    om.erase(rk[a:b])

    with ThreadPoolExecutor(max_workers=t) as ex:
        list(ex.map(init, range(t)))
        t0 = time.perf_counter()
        list(ex.map(replay, range(t)))
        dt = time.perf_counter() - t0
    keys = int(ro[-1])
    r = {"ms": round(dt * 1e3, 1), "Mkeys_s": round(keys / dt / 1e6, 1), "threads": t, "kind": "port",
         "rehashes": int(sum(growths)),
         "sample": "the whole trace (every request), no arrival times: one serial map per map, maps dealt "
                   "round-robin to host threads"}
    if gpu_out is not None:
        q = np.zeros(len(rk), bool)
        for i in np.flatnonzero(rop == 1).tolist():
            q[int(ro[i]):int(ro[i + 1])] = True
        hit = q & (out != np.uint64(SERVE_FILL))
        g = np.asarray(gpu_out).view(np.uint64)
        r["query_hits_compared"] = int(hit.sum())
        r["query_hits_equal_gpu"] = bool(np.array_equal(out[hit], g[hit]))
    del maps
    return r


def cpu_streaming(log_n: int = 24, threads: int | None = None, reps: int = 3) -> dict:
    """CPU baseline of the streaming primitives on a bounded sample of 2^log_n u32 (uniform; scan input in
    [0, 16)): the oracle's serial copy_if with (x % 100) < s, s = 1/50/99, and its serial exclusive scan, on one
    core and as two-pass chunked versions on `threads` host threads (chunk results, then chunk offsets, then a
    parallel placement; the oracle's calls and numpy's copies release the GIL). The reference has no CPU code for
    these (split::tools is device-only), so this restates them. Rates in G elements/s and GB/s of the same
    algorithmic bytes as the GPU figures (copy_if 4 B per element + 4 B per selected; scan 8 B per element)."""
    import ctypes
    import oracle
    from concurrent.futures import ThreadPoolExecutor
    t = threads or host_threads()
    n = 1 << log_n
    rng = np.random.default_rng(28)
    x = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    xs = rng.integers(0, 16, size=n, dtype=np.uint32)
    bounds = [(i * n // t, (i + 1) * n // t) for i in range(t)]
    lib = oracle.lib()

    def best_of(fn):
        best = None
        for _ in range(reps):
            t0 = time.perf_counter()
            r = fn()
            dt = time.perf_counter() - t0
            if best is None or dt < best[0]:
                best = (dt, r)
        return best

    def rates(dt, nbytes):
        return {"ms": round(dt * 1e3, 3), "Gelem_s": round(n / dt / 1e9, 3), "GB_s": round(nbytes / dt / 1e9, 1)}

    out = {"sample": f"2^{log_n} u32", "threads": t, "kind": "port"}
    with ThreadPoolExecutor(max_workers=t) as ex:
        for s in (1, 50, 99):
            p = oracle.pred(1, 0, 100, s)
            dt1, c1 = best_of(lambda: len(oracle.copy_if(x, 4, p)))

            def par_copy_if():
                tmp = [np.empty(hi - lo, np.uint32) for lo, hi in bounds]
                cnt = list(ex.map(lambda i: lib.ox_copy_if(oracle._p(x[bounds[i][0]:]), oracle._p(tmp[i]),
                                                             bounds[i][1] - bounds[i][0], 4, ctypes.byref(p)),
                                  range(t)))
                off = np.concatenate([[0], np.cumsum(cnt)])
                res = np.empty(int(off[-1]), np.uint32)
                list(ex.map(lambda i: res.__setitem__(slice(int(off[i]), int(off[i + 1])), tmp[i][:cnt[i]]),
                            range(t)))
                return len(res)

            dtt, ct = best_of(par_copy_if)
            assert c1 == ct
            nbytes = 4 * n + 4 * c1
            out[f"copy_if_s{s}"] = {"selected": c1, "one_core": rates(dt1, nbytes), "all_threads": rates(dtt, nbytes)}
        dt1, r1 = best_of(lambda: oracle.exclusive_scan_u32(xs))

        def par_scan():
            res = np.empty(n, np.uint32)
            list(ex.map(lambda i: lib.ox_exclusive_scan_u32(oracle._p(xs[bounds[i][0]:]), oracle._p(res[bounds[i][0]:]),
                                                            bounds[i][1] - bounds[i][0]), range(t)))
            tot = [int(res[hi - 1]) + int(xs[hi - 1]) for lo, hi in bounds]
            off = np.concatenate([[0], np.cumsum(tot)]).astype(np.uint64) & np.uint64(0xFFFFFFFF)
            list(ex.map(lambda i: np.add(res[bounds[i][0]:bounds[i][1]], np.uint32(off[i]),
                                         out=res[bounds[i][0]:bounds[i][1]]), range(t)))
            return res

        dtt, rt = best_of(par_scan)
        assert np.array_equal(r1, rt)
        out["exclusive_scan"] = {"one_core": rates(dt1, 8 * n), "all_threads": rates(dtt, 8 * n)}
    return out


def run_batched(args, stream, dev):
    """4096 velocity-block maps (key counts log-uniform in [2^6, 2^16], LF 0.5): insert all, query (70% hit),
    erase 10%, clean_tombstones. Fused: one persistent launch, autotuned, replayed from a CUDA graph. Plain:
    the per-map launches of the single-map API on the same data. Both start from empty maps every step."""
    import torch
    import hashinator_gb300 as hx
    from hashinator_gb300 import workloads
    from hashinator_gb300.autotune import autotune_batch
    t0 = time.perf_counter()
    w = workloads.batched_workload(args.batched_maps, 4096)
    gen_s = time.perf_counter() - t0

    def dev_u32(a):
        return torch.from_numpy(a.view(np.int32)).to(dev)

    d = {k: dev_u32(w[k]) for k in ("keys", "vals", "queries", "erase")}
    outs, batches, plans = [], [], []
    for _ in range(2):
        b = hx.Batch(w["size_powers"], stream=stream)
        o = torch.full((len(w["queries"]),), -1, dtype=torch.int32, device=dev)
        pl = b.plan(d["keys"], d["vals"], w["ins_offsets"], d["queries"], o, w["query_offsets"], d["erase"],
                    w["erase_offsets"], clean=True, stream=stream)
        batches.append(b)
        plans.append(pl)
        outs.append(o)
    bf, bp = batches
    pf, pp = plans
    if args.batched_tuning:
        g, b_, t_ = args.batched_tuning
        pf.set_tuning(g, b_, t_, stream=stream)
        tune = {"best": (g, b_, t_)}
    else:
        tune = autotune_batch(pf, None, stream=stream)  # the round starts from empty maps: libhx clears them

    def timed(fn, reps):
        ts = []
        for r in range(reps + 1):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            if r:
                ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    fused_ms = timed(lambda: (bf.clear(stream=stream), pf.run_graph(stream=stream)), max(3, args.steps // 5))
    plain_ms = timed(lambda: (bp.clear(stream=stream), pp.run_per_map(stream=stream)), 3)
    err = pf.check(stream=stream)
    same_q = bool(torch.equal(outs[0], outs[1]))
    fills_equal = all(bf.map_info(i).fill == bp.map_info(i).fill and
                      bf.map_info(i).tombstone_counter == bp.map_info(i).tombstone_counter
                      for i in range(0, bf.n_maps, max(1, bf.n_maps // 256)))
    n_ops = len(w["keys"]) + len(w["queries"]) + len(w["erase"])
    return {"workload": f"{args.batched_maps} u32 maps, keys log-uniform in [2^6, 2^16] (velocity-block ids in a "
                        f"30-60 cell shell of a 200^3 grid), LF 0.5: insert all, query n_i (70% hit), erase 10%, "
                        f"clean_tombstones",
            "keys_inserted": int(len(w["keys"])), "queries": int(len(w["queries"])), "erased": int(len(w["erase"])),
            "buckets": int((2 ** w["size_powers"].astype(np.int64)).sum()),
            "fused_ms": round(fused_ms, 3), "plain_ms": round(plain_ms, 3),
            "speedup_vs_per_map": round(plain_ms / fused_ms, 2),
            "fused_Mops_s": round(n_ops / fused_ms / 1e3, 1), "plain_Mops_s": round(n_ops / plain_ms / 1e3, 1),
            "autotuned": {"group_width": tune["best"][0], "block": tune["best"][1], "tile_keys": tune["best"][2]},
            "bit_exact_vs_per_map": same_q and fills_equal and err == 0, "generate_s": round(gen_s, 1),
            "timing": "CUDA events around clear + run, median; fused replays a captured CUDA graph",
            "cpu_baseline": _guarded(lambda: cpu_batched(w, outs[0].cpu().numpy()))}


def run_serving(args, dev):
    """1024 resident u64 maps (initial key counts log-uniform in [2^8, 2^20], tables at LF <= 0.5), a 40 GB
    device-memory budget, on-device growth past LF 0.8; Poisson arrivals at swept rates, requests of
    log-uniform 1..2^16 keys, insert/query/erase 20/70/10, queries 80% present. Each rate starts from the
    same initial maps; the native loop submits each request at its arrival time."""
    import torch
    import hashinator_gb300 as hx
    from hashinator_gb300 import workloads
    t0 = time.perf_counter()
    base_rate = 1e6
    tr = workloads.serving_trace(args.serving_maps, args.serving_requests, 5, init_log=(8.0, 20.0),
                                 size_log=(0.0, 16.0), rate_req_s=base_rate, width=8)
    gen_s = time.perf_counter() - t0

    def dev64(a):
        return torch.from_numpy(a.view(np.int64)).to(dev)

    ik, iv, rk, rv = dev64(tr["init_keys"]), dev64(tr["init_vals"]), dev64(tr["req_keys"]), dev64(tr["req_vals"])
    out = torch.empty(len(tr["req_keys"]), dtype=torch.int64, device=dev)
    io, ro = tr["init_offsets"], tr["req_offsets"]
    n_req = len(tr["req_map"])
    total_keys = int(ro[-1])
    results = []
    for rate in args.serving_rates:
        srv = hx.Server(key_bytes=8, memory_budget=40 << 30, max_load_factor=0.8, max_maps=args.serving_maps,
                        max_round_requests=4096, max_round_keys=1 << 23, rounds_in_flight=3)
        ids = [srv.add_map(int(sp)) for sp in tr["size_powers"]]
        srv.submit([(ids[m], hx.OP_INSERT, ik.data_ptr() + int(io[m]) * 8, iv.data_ptr() + int(io[m]) * 8, 0,
                     int(io[m + 1] - io[m]), m) for m in range(len(ids))])
        srv.drain()
        srv.poll()
        torch.cuda.synchronize()
        reqs = srv.requests([(ids[int(tr["req_map"][i])], int(tr["req_op"][i]), rk.data_ptr() + int(ro[i]) * 8,
                              rv.data_ptr() + int(ro[i]) * 8, out.data_ptr() + int(ro[i]) * 8, int(tr["req_n"][i]), i)
                             for i in range(n_req)])
        arrival = (tr["arrival_ns"].astype(np.float64) * (base_rate / rate)).astype(np.uint64)
        comp, st = srv.run_trace(reqs, arrival)
        lat = (comp.astype(np.float64) - arrival.astype(np.float64)) / 1e3
        span = (comp.max() - arrival.min()) / 1e9
        used, _ = srv.memory()
        sst = srv.stats()
        results.append({"rounds": sst["rounds"], "growths": sst["growths"], "max_stage_depth": sst["max_stage_depth"],
                        "host_ms_forming_rounds": round(sst["host_ns_step"] / 1e6, 1), "offered_req_s": rate,
                        "offered_Mkeys_s": round(total_keys / (arrival.max() / 1e9) / 1e6, 1),
                        "p50_us": round(float(np.percentile(lat, 50)), 1),
                        "p99_us": round(float(np.percentile(lat, 99)), 1),
                        "sustained_Mkeys_s": round(total_keys / span / 1e6, 1),
                        "ok": int((st == 0).sum()), "rejected": int((st != 0).sum()),
                        "device_GB": round(used / 1e9, 2)})
        srv.close()
    return {"workload": f"{args.serving_maps} u64 maps, initial keys log-uniform [2^8, 2^20], 40 GB budget, grow "
                        f"past LF 0.8; {n_req} Poisson requests of log-uniform 1..2^16 keys, insert/query/erase "
                        f"20/70/10, queries 80% present",
            "keys_per_run": total_keys, "initial_keys": int(io[-1]), "rates": results, "generate_s": round(gen_s, 1),
            "latency": "arrival (host clock) to the end of the request's round (CUDA event on the serving stream)",
            "cpu_baseline": _guarded(lambda: cpu_serving(tr, out.cpu().numpy()))}


class _DevWords:
    """A raw device range of 32-bit words as a __cuda_array_interface__ object."""

    def __init__(self, ptr: int, count: int):
        self.__cuda_array_interface__ = {"shape": (count,), "typestr": "<i4", "data": (ptr, False),
                                         "version": 3, "strides": None}


def _device_words(ptr: int, count: int, dev):
    """A torch view of `count` 32-bit words of device memory at `ptr` (a map's bucket array)."""
    import torch
    return torch.as_tensor(_DevWords(ptr, count), device=dev)


def _ev_time(stream, fn, reps=3):
    import torch
    ts = []
    for r in range(reps + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        if r:
            ts.append(e0.elapsed_time(e1) / 1e3)
    return float(np.median(ts))


def run_lf_sweep(args, stream, dev, peak):
    """The large single map: u32 and u64 keys, 2^27 buckets, LF 0.5/0.75/0.9 (key count adjusted):
    insert, 50/50 query, erase 30%, clean_tombstones, re-query. Each op timed alone with CUDA events
    on a fresh table (insert) or the state the sequence reaches."""
    import torch
    import hashinator_gb300 as hx
    from hashinator_gb300 import workloads
    sp = 27
    out = []
    for width in (4, 8):
        sig = np.int32 if width == 4 else np.int64
        nmax = int(0.9 * (1 << sp))
        keys, vals, q, er = workloads.large_map_workload(nmax, width, 31 + width)

        def dev_t(a):
            return torch.from_numpy(np.ascontiguousarray(a).view(sig)).to(dev)

        dk, dv = dev_t(keys), dev_t(vals)
        ib, qb, eb = {4: 72, 8: 80}[width], {4: 40, 8: 48}[width], {4: 68, 8: 72}[width]
        for lf in (0.5, 0.75, 0.9):
            n = int(lf * (1 << sp))
            rng = np.random.default_rng(int(lf * 100) + width)
            # queries: half hits among the first n keys, half absent keys, shuffled
            hsel = workloads.affine_sample(n, n // 2, rng)
            miss = workloads.distinct_keys(n - n // 2, width, 31 + width, offset=nmax + 4096)
            fill = np.iinfo(keys.dtype).max - 7
            perm = workloads.affine_sample(n, n, rng)
            qq = np.concatenate([keys[hsel], miss])[perm]
            expect = np.concatenate([vals[hsel], np.full(len(miss), fill, keys.dtype)])[perm]
            eidx = workloads.affine_sample(n, int(0.3 * n), rng)
            ee = keys[eidx]
            er_flag = np.zeros(n, bool)
            er_flag[eidx] = True
            erased_q = np.concatenate([er_flag[hsel], np.zeros(len(miss), bool)])[perm]
            del er_flag
            dq, de = dev_t(qq), dev_t(ee)
            o = dev_t(np.full(n, fill, keys.dtype))
            m = hx.Hashmap(sp, width, stream=stream)
            t_ins = _ev_time(stream, lambda: (m.clear(stream=stream), m.insert(dk[:n], dv[:n], target_lf=0.0,
                                                                                 stream=stream)))
            t_clear = _ev_time(stream, lambda: m.clear(stream=stream))
            t_ins -= t_clear
            m.clear(stream=stream)
            m.insert(dk[:n], dv[:n], target_lf=0.0, stream=stream)
            t_q = _ev_time(stream, lambda: m.retrieve(dq, o, stream=stream))
            # a clean with no tombstones skips its pass but sizes the map's scratch, so the timed clean
            # below measures the pass, not a first-time stream-ordered allocation
            m.clean_tombstones(stream=stream)
            exact = bool(np.array_equal(o.cpu().numpy().view(keys.dtype), expect))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            m.erase(de, stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            t_e = e0.elapsed_time(e1) / 1e3
            e0.record(stream)
            m.clean_tombstones(stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            t_c = e0.elapsed_time(e1) / 1e3
            inf = m.info(stream=stream)
            o.copy_(dev_t(np.full(n, fill, keys.dtype)))
            t_q2 = _ev_time(stream, lambda: m.retrieve(dq, o, stream=stream))
            # after erasing ee and clean_tombstones: erased keys now miss
            expect2 = expect.copy()
            expect2[erased_q] = fill
            exact2 = bool(np.array_equal(o.cpu().numpy().view(keys.dtype), expect2))
            pb = 8 if width == 4 else 16
            moved = int(inf.last_clean_moved)
            clean_bytes = (1 << sp) * pb + ib * moved  # scan of every bucket + one insert per moved key
            out.append({"key_bytes": width, "load_factor": lf, "keys": n,
                        "insert_Mkeys_s": round(n / t_ins / 1e6, 1), "insert_frac": round(n * ib / t_ins / 1e9 / peak, 4),
                        "query_Mkeys_s": round(n / t_q / 1e6, 1), "query_frac": round(n * qb / t_q / 1e9 / peak, 4),
                        "erase_Mkeys_s": round(len(ee) / t_e / 1e6, 1),
                        "erase_frac": round(len(ee) * eb / t_e / 1e9 / peak, 4),
                        "clean_ms": round(t_c * 1e3, 3), "clean_moved": moved,
                        "clean_GB_s": round(clean_bytes / t_c / 1e9, 1),
                        "clean_frac": round(clean_bytes / t_c / 1e9 / peak, 4),
                        "requery_Mkeys_s": round(n / t_q2 / 1e6, 1),
                        "fill_after": int(inf.fill), "tombstones_after_clean": int(inf.tombstone_counter),
                        "fill_ok": int(inf.fill) == n - len(ee), "query_exact": exact, "requery_exact": exact2})
            m.close()
            del dq, de, o
        del dk, dv
        torch.cuda.empty_cache()
    return {"note": "fraction of the measured HBM copy bandwidth for algorithmic bytes (insert 72/80, query 40/48, "
                    "erase 68/72 B per key; clean_tombstones 8/16 B per bucket scanned + 72/80 B per moved key); "
                    "query_exact/requery_exact compare every query output with the known answer",
            "runs": out}


def run_streaming(args, stream, dev, peak):
    """copy_if on 2^28 u32 with (x % 100) < s, s = 1/50/99; exclusive scan of 2^28 u32 in [0, 16);
    extractPattern (value even, valid keys) and extractAllKeys on the 2^26-key u32 map of 2^27 buckets.
    Every output of the timed calls is compared, element for element, with a host computation: numpy's
    mask-and-filter for copy_if, numpy's cumsum (wrapping modulo 2^32) for the scan, and an order-preserving
    filter of the map's own bucket array for the extractions."""
    import torch
    import hashinator_gb300 as hx
    from hashinator_gb300 import workloads
    n = 1 << args.stream_log_n
    x = torch.randint(0, 2**31 - 1, (n,), dtype=torch.int64, device=dev, generator=torch.Generator(device=dev).manual_seed(7))
    x = (x * 2 + (x >> 17 & 1)).to(torch.int32)  # uniform over the 32-bit range, as int32 bits
    out = torch.empty_like(x)
    x_h = x.cpu().numpy().view(np.uint32)
    r_h = (x_h % np.uint32(100)).astype(np.uint8)
    res = {}
    for s_ in (1, 50, 99):
        c = hx.tools.copy_if(x, out, hx.Pred.mod_lt(100, s_))
        nb = hx.tools.scratch_bytes(hx.SCRATCH_COPY_IF, n)
        scratch = torch.empty(max(nb, 1), dtype=torch.uint8, device=dev)
        dc = torch.zeros(1, dtype=torch.int64, device=dev)
        out.fill_(-1)
        t = _ev_time(stream, lambda: hx.tools.copy_if(x, out, hx.Pred.mod_lt(100, s_), scratch=scratch,
                                                      scratch_bytes=nb, stream=stream, d_count=dc))
        want = x_h[r_h < s_]
        got = out[:c].cpu().numpy().view(np.uint32)
        res[f"copy_if_s{s_}"] = {"selected": int(c), "ms": round(t * 1e3, 3),
                                 "GB_s": round((4 * n + 4 * c) / t / 1e9, 1),
                                 "frac": round((4 * n + 4 * c) / t / 1e9 / peak, 4),
                                 "exact": bool(int(dc.item()) == len(want) and np.array_equal(got, want))}
        del want, got
    res["copy_if_functor"] = _guarded(lambda: functor_leg(args.stream_log_n))
    y = (x & 15).contiguous()
    y_h = (x_h & np.uint32(15))
    del r_h
    nb = hx.tools.scratch_bytes(hx.SCRATCH_SCAN, n)
    scratch = torch.empty(max(nb, 1), dtype=torch.uint8, device=dev)
    out.fill_(-1)
    t = _ev_time(stream, lambda: hx.tools.split_prefix_scan(y, out, scratch=scratch, scratch_bytes=nb, stream=stream))
    want = np.zeros(n, np.uint32)
    np.cumsum(y_h[:-1], dtype=np.uint32, out=want[1:])
    res["exclusive_scan"] = {"ms": round(t * 1e3, 3), "GB_s": round(8 * n / t / 1e9, 1),
                             "frac": round(8 * n / t / 1e9 / peak, 4),
                             "exact": bool(np.array_equal(out.cpu().numpy().view(np.uint32), want))}
    del x, y, out, scratch, x_h, y_h, want
    keys, vals, _, _ = workloads.map_workload(1 << 26, 4, 2026, erase_frac=0.0)
    m = hx.Hashmap(27, 4, stream=stream)
    m.insert(torch.from_numpy(keys.view(np.int32)).to(dev), torch.from_numpy(vals.view(np.int32)).to(dev),
             target_lf=0.0, stream=stream)
    ex = torch.empty(2 * (1 << 26), dtype=torch.int32, device=dev)
    c = m.extract_pattern(hx.Pred.value_even(), ex, capacity=1 << 26, stream=stream)
    dc = torch.zeros(1, dtype=torch.int64, device=dev)
    ex.fill_(-1)
    t = _ev_time(stream, lambda: m.extract_pattern(hx.Pred.value_even(), ex, capacity=1 << 26, stream=stream,
                                                   d_count=dc))
    ptr, nbk = m.bucket_data()
    torch.cuda.synchronize()
    b = _device_words(ptr, 2 * nbk, dev).cpu().numpy().view(np.uint32).reshape(nbk, 2)
    valid = b[:, 0] < np.uint32(0xFFFFFFFE)
    sel = valid & (b[:, 1] % np.uint32(2) == 0)
    want = b[sel].reshape(-1)
    byts = 8 * (1 << 27) + 8 * c
    res["extract_pattern_value_even"] = {
        "selected": int(c), "expected": int((vals % 2 == 0).sum()), "ms": round(t * 1e3, 3),
        "GB_s": round(byts / t / 1e9, 1), "frac": round(byts / t / 1e9 / peak, 4),
        "exact": bool(int(dc.item()) == int(sel.sum()) and
                      np.array_equal(ex[:2 * int(c)].cpu().numpy().view(np.uint32), want))}
    ek = torch.empty(1 << 26, dtype=torch.int32, device=dev)
    ck = m.extract_all_keys(ek, stream=stream)
    ek.fill_(-1)
    t = _ev_time(stream, lambda: m.extract_keys_by_pattern(hx.Pred.valid_key(), ek, capacity=1 << 26,
                                                           stream=stream, d_count=dc))
    byts = 8 * (1 << 27) + 4 * ck
    res["extract_all_keys"] = {"selected": int(ck), "expected": 1 << 26, "ms": round(t * 1e3, 3),
                               "GB_s": round(byts / t / 1e9, 1), "frac": round(byts / t / 1e9 / peak, 4),
                               "exact": bool(int(dc.item()) == int(valid.sum()) and
                                             np.array_equal(ek[:int(ck)].cpu().numpy().view(np.uint32),
                                                            b[valid, 0]))}
    del b, valid, sel, want
    m.close()
    return res


FUNCTOR_LEG_SRC = r"""
// copy_if with a caller's functor through the drop-in header (the rule compiled
// into the single-pass kernel in this translation unit) against libhx's
// descriptor copy_if, on the same 2^k uniform u32 elements.
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "hashinator_compat.h"
struct ModLt {  // x % 100 < b, the divisor a constant as in the reference's own test rules
  uint32_t b;
  __host__ __device__ bool operator()(const uint32_t& x) const { return x % 100u < b; }
};
__global__ void k_gen(uint32_t* x, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    unsigned long long z = (i + 0x9E3779B97F4A7C15ull) * 0xBF58476D1CE4E5B9ull;
    z ^= z >> 31; z *= 0x94D049BB133111EBull; z ^= z >> 29;
    x[i] = (uint32_t)z;
  }
}
int main(int argc, char** argv) {
  const size_t n = (size_t)1 << atoi(argv[1]);
  uint32_t *x, *o1, *o2; size_t* c1; void* sc;
  cudaMalloc(&x, n * 4); cudaMalloc(&o1, n * 4); cudaMalloc(&o2, n * 4); cudaMalloc(&c1, 8);
  const size_t need = split::tools::detail::compaction_scratch_bytes<uint32_t>(n);
  cudaMalloc(&sc, need);
  k_gen<<<4096, 256>>>(x, n);
  cudaStream_t s; cudaStreamCreate(&s);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  std::printf("{");
  for (uint32_t sel : {1u, 50u, 99u}) {
    float best = 1e9f;
    for (int rep = 0; rep < 6; ++rep) {
      cudaEventRecord(e0, s);
      split::tools::detail::compact(x, o1, n, n, ModLt{sel}, split::tools::detail::Identity{}, c1, ~(size_t)0, sc, s);
      cudaEventRecord(e1, s); cudaEventSynchronize(e1);
      float ms; cudaEventElapsedTime(&ms, e0, e1);
      if (rep && ms < best) best = ms;
    }
    size_t fc = 0; uint64_t dc = 0;
    cudaMemcpy(&fc, c1, 8, cudaMemcpyDeviceToHost);
    hx_pred p{HX_PRED_MOD_LT, HX_FIELD_ELEM, 0, 0, 100, sel};
    hx_copy_if(x, o2, n, 4, &p, n, nullptr, &dc, nullptr, 0, s);
    std::vector<uint32_t> a(fc), b(dc);
    cudaMemcpy(a.data(), o1, fc * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(b.data(), o2, dc * 4, cudaMemcpyDeviceToHost);
    std::printf("%s\"s%u\": {\"ms\": %.4f, \"selected\": %zu, \"equal_to_descriptor\": %s}", sel == 1 ? "" : ", ", sel,
                best, fc, (fc == dc && a == b) ? "true" : "false");
  }
  std::printf("}\n");
  return cudaDeviceSynchronize() != cudaSuccess;
}
"""


def functor_leg(log_n: int) -> dict:
    """The drop-in header's functor copy_if (a caller's rule compiled into the single-pass kernel) timed with CUDA
    events on 2^log_n uniform u32, and compared element for element with libhx's descriptor copy_if. The program is
    built with nvcc into hashinator_gb300/_build/ once."""
    from hashinator_gb300 import build
    bdir = ROOT / "hashinator_gb300" / "_build"
    bdir.mkdir(exist_ok=True)
    src, exe = bdir / "functor_copy_if.cu", bdir / "functor_copy_if"
    if not exe.exists() or not src.exists() or src.read_text() != FUNCTOR_LEG_SRC:
        src.write_text(FUNCTOR_LEG_SRC)
        lib_dir = str(ROOT / "hashinator_gb300")
        subprocess.run([build._nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                        "-I", str(ROOT / "include"), str(src), "-o", str(exe), "-L", lib_dir, "-lhx",
                        f"-Xlinker=-rpath,{lib_dir}"], check=True, capture_output=True, timeout=600)
    r = subprocess.run([str(exe), str(log_n)], capture_output=True, text=True, timeout=600, check=True)
    out = json.loads(r.stdout.strip().splitlines()[-1])
    out["rule"] = "struct ModLt { x % 100u < s } (constant divisor) through split::tools (hashinator_compat.h), CUDA events"
    return out


def run_reference(args):
    """The reference's CPU path (the oracle's restatement of its serial insert + find) on the headline
    workload itself: 2^log_keys u32 keys into 2^(log_keys+1) buckets, 2^log_keys queries (50% hit), one
    serial map per host thread with keys sharded by the top bits of their home bucket (each map a slice of
    the table at the same load factor). The one-core figure beside it runs a 2^24-key sample."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    log_n = args.log_keys
    n = 1 << log_n
    t = host_threads()
    times = []
    for i in range(args.warmup + args.steps):
        _, _, _, dt = cpu_insert_query(4, log_n, t)
        if i >= args.warmup:
            times.append(dt)
    v1, _, _, _ = cpu_insert_query(4, min(log_n, 24), 1)
    ms = float(np.mean(times))
    v = 2 * n / ms / 1e6
    sample = (f"the headline workload: 2^{log_n} u32 keys into 2^{log_n + 1} buckets (LF 0.5) + 2^{log_n} queries "
              f"50% hit per step; {t} serial maps (the reference's CPU path, restated in the oracle), keys sharded "
              f"by the top bits of their home bucket; one core on 2^{min(log_n, 24)} keys: {v1:.1f} Mkeys/s")
    config = headline_config(args.log_keys, args.group)
    config.update({"reference_sample": f"2^{log_n} keys into 2^{log_n + 1} buckets per step (the full workload)",
                   "reference_host_threads": t})
    line = {"impl": "reference", "metric": headline_metric(args.log_keys), "value": round(v, 3), "unit": "Mkeys/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": DATA,
            "config": config,
            "cpu_baseline": {"value": round(v, 3), "unit": "Mkeys/s", "cores": t, "kind": "port", "sample": sample,
                             "host": _guarded(host_cpu)},
            "e2e": {"value": round(v, 3), "unit": "Mkeys/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _summary(line: dict) -> dict:
    """The figures a reader of the end of the JSON line needs: headline, e2e, roofline, exactness checks,
    streaming times, the batched speed-up over per-map launches and the serving latencies."""
    def g(d, *ks):
        for k in ks:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return d

    out = {"value_Mkeys_s": line.get("value"), "e2e_Mkeys_s": g(line, "e2e", "value"),
           "roofline_frac": g(line, "roofline", "frac"), "roofline_kernel": g(line, "roofline", "kernel"),
           "checks_exact": all(v for k, v in (line.get("checks") or {}).items() if isinstance(v, bool))}
    st = line.get("streaming")
    if isinstance(st, dict):
        out["streaming_ms"] = {k: v.get("ms") for k, v in st.items() if isinstance(v, dict) and "ms" in v}
        out["streaming_exact"] = all(v.get("exact", True) for v in st.values() if isinstance(v, dict))
        fl = st.get("copy_if_functor")
        if isinstance(fl, dict) and "s1" in fl:
            out["copy_if_functor_ms"] = {k: v["ms"] for k, v in fl.items() if isinstance(v, dict)}
            out["copy_if_functor_equal"] = all(v["equal_to_descriptor"] for v in fl.values() if isinstance(v, dict))
    sw = g(line, "large_map_lf_sweep", "runs")
    if isinstance(sw, list):
        out["lf_sweep_exact"] = all(r.get("query_exact") and r.get("requery_exact") for r in sw)
    b = line.get("batched")
    if isinstance(b, dict) and "fused_ms" in b:
        out["batched"] = {"fused_ms": b["fused_ms"], "per_map_ms": b["plain_ms"],
                          "speedup_vs_per_map": b["speedup_vs_per_map"], "bit_exact": b["bit_exact_vs_per_map"]}
    sv = g(line, "serving", "rates")
    if isinstance(sv, list):
        out["serving"] = [{"offered_req_s": r["offered_req_s"], "p50_us": r["p50_us"], "p99_us": r["p99_us"],
                           "sustained_Mkeys_s": r["sustained_Mkeys_s"]} for r in sv]
    return out


def run_ours(args):
    import torch
    import hashinator_gb300 as hx
    from hashinator_gb300 import workloads

    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    hx.lib()
    width = 4
    n = 1 << args.log_keys
    sp = args.log_keys + 1
    from hashinator_gb300.dist import max_over_ranks, replica_seed
    keys, vals, q, _ = workloads.map_workload(n, width, replica_seed(2026, rank), erase_frac=0.0)

    def to_dev(a):
        return torch.from_numpy(a.view(np.int32)).to(dev)

    d_keys, d_vals, d_q = to_dev(keys), to_dev(vals), to_dev(q)
    # Query outputs start as FILL; a miss leaves its element as it was, so after
    # any number of steps the whole buffer must equal `expect` (keys are
    # distinct, so every query's answer is known exactly).
    expect, found = workloads.query_expectation(keys, vals, q, HEADLINE_FILL)
    d_out = to_dev(np.full(n, HEADLINE_FILL, np.uint32))
    stream = torch.cuda.Stream(device=dev)
    m = hx.Hashmap(sp, width, stream=stream)
    if args.group:
        m.set_tuning(group_width=args.group)

    def step(ev=None):
        if ev:
            ev[0].record(stream)
        m.clear(stream=stream)
        if ev:
            ev[1].record(stream)
        m.insert(d_keys, d_vals, target_lf=0.5, stream=stream)
        if ev:
            ev[2].record(stream)
        m.retrieve(d_q, d_out, stream=stream)
        if ev:
            ev[3].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # every retrieve output of the warm-up steps, element for element (not timed)
    host_out = d_out.cpu().numpy().view(np.uint32)
    checks = {"expected_hits": int(found.sum()), "queries": n,
              "retrieve_exact_after_warmup": bool(np.array_equal(host_out, expect))}

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    l0 = hx.kernel_launch_count()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for i in range(args.steps):
        step(evs[i])
    stop.record(stream)
    torch.cuda.synchronize()
    launches = hx.kernel_launch_count() - l0
    elapsed = max_over_ranks(start.elapsed_time(stop) / 1e3, dev)
    checks["retrieve_exact_after_timed"] = bool(np.array_equal(d_out.cpu().numpy().view(np.uint32), expect))
    info = m.info(stream=stream)
    checks["fill_after_timed"] = int(info.fill)
    checks["fill_exact"] = int(info.fill) == n
    clocks = sampler.stop()
    t_clear = float(np.mean([e[0].elapsed_time(e[1]) for e in evs])) / 1e3
    t_ins = float(np.mean([e[1].elapsed_time(e[2]) for e in evs])) / 1e3
    t_q = float(np.mean([e[2].elapsed_time(e[3]) for e in evs])) / 1e3
    ms_per_step = elapsed / args.steps * 1e3
    value = world * 2 * n * args.steps / elapsed / 1e6

    # ---- end-to-end through the public API with pinned host buffers ------
    # Chunked and pipelined: H2D of chunk c+1 (copy stream) overlaps the insert
    # of chunk c (compute stream); the queries' D2H of chunk c overlaps the
    # query of chunk c+1. Every byte of input crosses H2D and every result
    # crosses D2H inside the timed region.
    e2e = None
    if not args.no_e2e:
        h_keys = torch.from_numpy(keys.view(np.int32)).pin_memory()
        h_vals = torch.from_numpy(vals.view(np.int32)).pin_memory()
        h_q = torch.from_numpy(q.view(np.int32)).pin_memory()
        h_out = torch.empty(n, dtype=torch.int32).pin_memory()
        # Several device buffer sets, rotated; a set is reused only after the step that
        # last used it has consumed its inputs and downloaded its results. Two copy
        # streams (--e2e-copy-streams 2): uploads and downloads on their own streams,
        # step k+1's uploads running while step k's kernels do. One copy stream (1):
        # every copy in one order, step k+1's uploads queued before step k's downloads,
        # so the host link carries one direction at a time.
        one_copy = args.e2e_copy_streams == 1
        h2d = torch.cuda.Stream(device=dev)
        d2h = h2d if one_copy else torch.cuda.Stream(device=dev)
        nsets = max(2, args.e2e_sets)
        bufs = [(d_keys, d_vals, d_q, d_out)] + [
            (torch.empty_like(d_keys), torch.empty_like(d_vals), torch.empty_like(d_q), d_out.clone())
            for _ in range(nsets - 1)]
        free = [None] * nsets
        chunks = args.e2e_chunks
        bounds = [(c * n // chunks, (c + 1) * n // chunks) for c in range(chunks)]
        step_no = [0]

        marks = []  # per step: the compute stream at the step's start and at its end
        waits = []  # per step: (before, after) each wait of the compute stream on an upload
        up_spans = []  # per step: the copy stream at the start and the end of its uploads
        down_spans = []  # per step: (start, end) of each download, each start after its wait

        def timing_event(s_):
            e_ = torch.cuda.Event(enable_timing=True)
            e_.record(s_)
            return e_

        def upload(i):
            k = i % nsets
            bk, bv, bq, _ = bufs[k]
            kv_ready, q_ready = [], []
            with torch.cuda.stream(h2d):
                if free[k] is not None:
                    h2d.wait_event(free[k])
                u0 = timing_event(h2d)
                for a, b in bounds:
                    bk[a:b].copy_(h_keys[a:b], non_blocking=True)
                    bv[a:b].copy_(h_vals[a:b], non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(h2d)
                    kv_ready.append(ev)
                for a, b in bounds:
                    bq[a:b].copy_(h_q[a:b], non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(h2d)
                    q_ready.append(ev)
                up_spans.append((u0, timing_event(h2d)))
            return kv_ready, q_ready

        def compute_and_download(i, ready):
            k = i % nsets
            kv_ready, q_ready = ready
            mk = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            bk, bv, bq, bo = bufs[k]
            wl = []
            mk[0].record(stream)
            m.clear(stream=stream)
            for (a, b), ev in zip(bounds, kv_ready):
                w0 = timing_event(stream)
                stream.wait_event(ev)
                wl.append((w0, timing_event(stream)))
                m.insert(bk[a:b], bv[a:b], target_lf=0.5, stream=stream)
            done = []
            for (a, b), ev in zip(bounds, q_ready):
                w0 = timing_event(stream)
                stream.wait_event(ev)
                wl.append((w0, timing_event(stream)))
                m.retrieve(bq[a:b], bo[a:b], stream=stream)
                ev2 = torch.cuda.Event()
                ev2.record(stream)
                done.append(ev2)
            mk[1].record(stream)
            marks.append(mk)
            waits.append(wl)
            with torch.cuda.stream(d2h):
                dl = []
                for (a, b), ev in zip(bounds, done):
                    d2h.wait_event(ev)
                    d0 = timing_event(d2h)
                    h_out[a:b].copy_(bo[a:b], non_blocking=True)
                    dl.append((d0, timing_event(d2h)))
                down_spans.append(dl)
            fin = torch.cuda.Event()
            fin.record(d2h)  # after every kernel of this step (waited on) and its downloads
            free[k] = fin

        def e2e_steps(count):
            """count steps; each step's uploads are queued one step ahead of its kernels."""
            first = step_no[0]
            ready = upload(first)
            for i in range(first, first + count):
                nxt = upload(i + 1) if i + 1 < first + count else None
                compute_and_download(i, ready)
                ready = nxt
            step_no[0] = first + count

        e2e_steps(max(1, args.warmup // 2))
        torch.cuda.synchronize()
        # the host link alone: one step's uploads and downloads as plain pinned copies, best of 3
        link = {}
        for name, fn, nbytes in (("h2d_GB_s", lambda: (bufs[0][0].copy_(h_keys, non_blocking=True),
                                                          bufs[0][1].copy_(h_vals, non_blocking=True),
                                                          bufs[0][2].copy_(h_q, non_blocking=True)), 3 * n * width),
                                 ("d2h_GB_s", lambda: h_out.copy_(bufs[0][3], non_blocking=True), n * width)):
            best = None
            for _ in range(3):
                c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                with torch.cuda.stream(h2d):
                    c0.record(h2d)
                    fn()
                    c1.record(h2d)
                torch.cuda.synchronize()
                t = c0.elapsed_time(c1) / 1e3
                best = t if best is None else min(best, t)
            link[name] = round(nbytes / best / 1e9, 1)
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        h2d.wait_event(s0)  # the first uploads start inside the timed region
        e2e_steps(args.steps)
        stream.wait_event(free[(step_no[0] - 1) % nsets])  # the timed region ends with the last results on the host
        s1.record(stream)
        torch.cuda.synchronize()
        e_el = max_over_ranks(s0.elapsed_time(s1) / 1e3, dev)
        # where the pipeline's time went, from events on the compute and copy streams over the timed
        # steps: the compute stream's time per step, the part of it spent waiting for uploads, the rest
        # (kernels), the upload rate the copy stream achieved while kernels ran, and the idle gap between
        # steps (the host enqueuing late)
        tm = marks[-args.steps:]
        tw = waits[-args.steps:]
        t_stream = float(np.mean([x[0].elapsed_time(x[1]) for x in tm]))
        t_wait = float(np.mean([sum(a.elapsed_time(b) for a, b in wl) for wl in tw]))
        t_up = float(np.median([a.elapsed_time(b) for a, b in up_spans[-args.steps:]]))
        t_down = float(np.median([sum(a.elapsed_time(b) for a, b in dl) for dl in down_spans[-args.steps:]]))
        pipe = {"compute_stream_ms_per_step": round(t_stream, 3),
                "upload_wait_ms_per_step": round(t_wait, 3),
                "kernels_ms_per_step": round(t_stream - t_wait, 3),
                "h2d_GB_s_in_pipeline": round(3 * n * width / (t_up * 1e-3) / 1e9, 1),
                "d2h_GB_s_in_pipeline": round(n * width / (t_down * 1e-3) / 1e9, 1),
                "host_gap_ms_per_step": round(float(np.mean([tm[i][1].elapsed_time(tm[i + 1][0])
                                                             for i in range(len(tm) - 1)])) if len(tm) > 1 else 0.0, 3)}
        # the e2e results (the last step's, on the host) equal the exact expectation
        checks["e2e_exact"] = bool(np.array_equal(h_out.numpy().view(np.uint32), expect))
        e2e = {"value": round(world * 2 * n * args.steps / e_el / 1e6, 3), "unit": "Mkeys/s",
               "h2d_bytes_per_step": 3 * n * width, "d2h_bytes_per_step": n * width,
               "ms_per_step": round(e_el / args.steps * 1e3, 3), "chunks": chunks,
               "api": "hashinator_gb300.Hashmap (libhx C ABI); copies overlapped with the kernels across steps, "
                      f"{nsets} device buffer sets, {args.e2e_copy_streams} copy stream(s)",
               "host_link": link,
               "pipeline": pipe,
               "link_bound_ms_per_step": round(3 * n * width / (link["h2d_GB_s"] * 1e9) * 1e3
                                               + n * width / (link["d2h_GB_s"] * 1e9) * 1e3, 3)}

    # ---- random-access ceilings over 1 GiB: 32-byte sector reads, 64-bit CAS -
    rbuf = torch.empty(1 << 30, dtype=torch.uint8, device=dev)
    n_ops = 1 << 26
    ceil = {}
    for mode in (0, 1):
        rts = []
        for r in range(4):
            rbuf.zero_()
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a0.record(stream)
            hx.diag_random_access(rbuf, rbuf.numel(), n_ops, mode, stream=stream)
            a1.record(stream)
            torch.cuda.synchronize()
            if r:
                rts.append(a0.elapsed_time(a1) / 1e3)
        ceil[mode] = n_ops / min(rts)
    del rbuf

    peak, peak_kind = measured_peak()
    ins_gbs = INSERT_BYTES_PER_KEY[width] * n / t_ins / 1e9
    q_gbs = QUERY_BYTES_PER_KEY[width] * n / t_q / 1e9
    dominant = "insert" if t_ins >= t_q else "query"
    achieved = ins_gbs if dominant == "insert" else q_gbs
    # measured traffic (2^26 keys) exists for the thread-per-key insert and query kernels
    tag = ("insert_u32_lf050" if args.group in (0, 1) else None) if dominant == "insert" else \
        ("query_t1_u32_lf050" if args.group == 1 else ("query_u32_lf050" if args.group == 0 else None))
    traffic = traffic_from_profiles(tag) if tag and args.log_keys == 26 else None
    dom_keys_s = n / (t_ins if dominant == "insert" else t_q)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": f"{peak_kind} hbm_gbs",
                "random_access": {
                    "read32_G_per_s": round(ceil[0] / 1e9, 2), "cas64_G_per_s": round(ceil[1] / 1e9, 2),
                    "frac": round(dom_keys_s / (ceil[1] if dominant == "insert" else ceil[0]), 3),
                    "note": "ceilings measured in this run by hx_diag_random_access over 1 GiB; frac = keys/s of the "
                            "dominant kernel over the ceiling of its one unavoidable random op per key (CAS for "
                            "insert, 32-byte read for query); DRAM transactions, not bytes, bound these kernels"},
                "kernel": (("k_insert_t1 (insert)" if args.group in (0, 1) else "k_insert (insert)")
                           if dominant == "insert" else
                           ("k_find_t1 (query)" if args.group == 1 else "k_retrieve (query)")),
                "algorithmic_bytes_per_launch": (INSERT_BYTES_PER_KEY if dominant == "insert"
                                                 else QUERY_BYTES_PER_KEY)[width] * n,
                "per_op": {"insert": {"ms": round(t_ins * 1e3, 3), "Mkeys_s": round(n / t_ins / 1e6, 1),
                                      "GB_s": round(ins_gbs, 1), "frac": round(ins_gbs / peak, 4)},
                           "query": {"ms": round(t_q * 1e3, 3), "Mkeys_s": round(n / t_q / 1e6, 1),
                                     "GB_s": round(q_gbs, 1), "frac": round(q_gbs / peak, 4)},
                           "clear": {"ms": round(t_clear * 1e3, 3),
                                     "GB_s": round((1 << sp) * 8 / t_clear / 1e9, 1)}}}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline()
    batched = None
    if not args.no_batched:
        batched = run_batched(args, stream, dev)
    serving = None
    if not args.no_serving:
        serving = run_serving(args, dev)
    lf_sweep = streaming = None
    if not args.no_extra:
        if not args.no_lf_sweep:
            lf_sweep = run_lf_sweep(args, stream, dev, peak)
        streaming = run_streaming(args, stream, dev, peak)

    if rank == 0:
        line = {"metric": headline_metric(args.log_keys), "value": round(value, 3), "unit": "Mkeys/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": DATA,
                "config": headline_config(args.log_keys, args.group),
                "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "checks": checks, "clocks": clocks,
                "cpu_baseline": cpu, "large_map_lf_sweep": lf_sweep, "streaming": streaming,
                "batched": batched, "serving": serving}
        line["summary"] = _summary(line)  # last, so that the end of the output carries every headline figure
        print(json.dumps(line), flush=True)
    m.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_case(args):
    """One kernel case on its own, for an ncu capture. --case-kind map: a table of 2^case_log_buckets buckets,
    the case_lf share of them inserted (case_reps times, each after a clear), then the same number of 50%-hit
    queries (case_reps times). --case-kind copy_if / scan: 2^case_log_n uniform u32, copy_if with
    (x % 100) < case_s, or the exclusive scan of x & 15, case_reps times. --case-kind clean: the map case's
    table with 30% of its keys erased, then one clean_tombstones (after a clean with no tombstones has sized
    the map's scratch). Prints one JSON line with the per-launch times."""
    import torch
    import hashinator_gb300 as hx
    from hashinator_gb300 import workloads
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    if args.case_kind in ("copy_if", "scan"):
        n = 1 << args.case_log_n
        g = torch.Generator(device=dev).manual_seed(7)
        x = torch.randint(0, 2**31 - 1, (n,), dtype=torch.int64, device=dev, generator=g)
        x = (x * 2 + (x >> 17 & 1)).to(torch.int32)
        out = torch.empty_like(x)
        stream = torch.cuda.Stream(device=dev)
        if args.case_kind == "copy_if":
            nb = hx.tools.scratch_bytes(hx.SCRATCH_COPY_IF, n)
            sc = torch.empty(nb, dtype=torch.uint8, device=dev)
            dc = torch.zeros(1, dtype=torch.int64, device=dev)
            t = _ev_time(stream, lambda: hx.tools.copy_if(x, out, hx.Pred.mod_lt(100, args.case_s), scratch=sc,
                                                          scratch_bytes=nb, stream=stream, d_count=dc),
                         reps=args.case_reps)
            c = int(dc.item())
            nbytes = 4 * n + 4 * c
        else:
            y = (x & 15).contiguous()
            nb = hx.tools.scratch_bytes(hx.SCRATCH_SCAN, n)
            sc = torch.empty(nb, dtype=torch.uint8, device=dev)
            t = _ev_time(stream, lambda: hx.tools.split_prefix_scan(y, out, scratch=sc, scratch_bytes=nb,
                                                                    stream=stream), reps=args.case_reps)
            nbytes = 8 * n
        print(json.dumps({"case": f"{args.case_kind} 2^{args.case_log_n} u32", "ms": round(t * 1e3, 4),
                          "GB_s": round(nbytes / t / 1e9, 1)}), flush=True)
        return 0
    w, sp = args.case_key_bytes, args.case_log_buckets
    n = int(args.case_lf * (1 << sp))
    keys, vals, q, _ = workloads.large_map_workload(n, w, 31 + w)
    sig = np.int32 if w == 4 else np.int64
    dk, dv, dq = (torch.from_numpy(a.view(sig)).to(dev) for a in (keys, vals, q))
    o = torch.empty_like(dq)
    stream = torch.cuda.Stream(device=dev)
    m = hx.Hashmap(sp, w, stream=stream)
    if args.case_kind == "clean":
        rng = np.random.default_rng(50 + w)
        de = torch.from_numpy(np.ascontiguousarray(keys[workloads.affine_sample(n, int(0.3 * n), rng)]).view(sig))
        de = de.to(dev)
        m.insert(dk, dv, target_lf=0.0, stream=stream)
        m.clean_tombstones(stream=stream)  # no tombstones yet: sizes the scratch, runs no pass
        m.erase(de, stream=stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        m.clean_tombstones(stream=stream)  # once: a second clean finds no tombstones
        e1.record(stream)
        torch.cuda.synchronize()
        t_c = e0.elapsed_time(e1) / 1e3
        inf = m.info(stream=stream)
        print(json.dumps({"case": f"clean_tombstones u{8 * w} 2^{sp} buckets LF {args.case_lf}, 30% erased",
                          "clean_ms": round(t_c * 1e3, 3), "moved": int(inf.last_clean_moved),
                          "fill": int(inf.fill), "tombstones": int(inf.tombstone_counter)}), flush=True)
        m.close()
        return 0
    t_clear = _ev_time(stream, lambda: m.clear(stream=stream), reps=args.case_reps)
    t_ins = _ev_time(stream, lambda: (m.clear(stream=stream), m.insert(dk, dv, target_lf=0.0, stream=stream)),
                     reps=args.case_reps)
    t_q = _ev_time(stream, lambda: m.retrieve(dq, o, stream=stream), reps=args.case_reps)
    inf = m.info(stream=stream)
    print(json.dumps({"case": f"u{8 * w} 2^{sp} buckets LF {args.case_lf}", "keys": n, "fill": int(inf.fill),
                      "clear_ms": round(t_clear * 1e3, 3), "clear_plus_insert_ms": round(t_ins * 1e3, 3),
                      "query_ms": round(t_q * 1e3, 3), "insert_Mkeys_s": round(n / (t_ins - t_clear) / 1e6, 1),
                      "query_Mkeys_s": round(n / t_q / 1e6, 1)}), flush=True)
    m.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--group", type=int, default=0, help="probe-group width (0 = library default)")
    ap.add_argument("--log-keys", type=int, default=26, help="log2 of the key count (table: twice as many buckets)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-chunks", type=int, default=2)
    ap.add_argument("--e2e-sets", type=int, default=3, help="device buffer sets the e2e pipeline rotates")
    ap.add_argument("--e2e-copy-streams", type=int, default=2, choices=[1, 2],
                    help="2: uploads and downloads on their own streams; 1: one copy stream, one direction at a time")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batched-maps", type=int, default=4096)
    ap.add_argument("--batched-tuning", type=int, nargs=3, metavar=("GROUP", "BLOCK", "TILE"),
                    help="fixed lanes-per-key, block size and tile keys instead of the autotuner")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the LF sweep and the streaming primitives")
    ap.add_argument("--no-lf-sweep", action="store_true", help="skip the LF sweep only")
    ap.add_argument("--stream-log-n", type=int, default=28, help="log2 of the streaming-primitive element count")
    ap.add_argument("--serving-maps", type=int, default=1024)
    ap.add_argument("--serving-requests", type=int, default=20000)
    ap.add_argument("--serving-rates", type=float, nargs="+", default=[2.5e5, 5e5, 1e6, 2e6, 4e6])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--case", action="store_true", help="run one hash-kernel case alone (for ncu captures)")
    ap.add_argument("--case-key-bytes", type=int, default=4, choices=[4, 8])
    ap.add_argument("--case-lf", type=float, default=0.5)
    ap.add_argument("--case-log-buckets", type=int, default=27)
    ap.add_argument("--case-reps", type=int, default=1)
    ap.add_argument("--case-kind", default="map", choices=["map", "copy_if", "scan", "clean"])
    ap.add_argument("--case-log-n", type=int, default=26)
    ap.add_argument("--case-s", type=int, default=1, help="copy_if selectivity in percent")
    args = ap.parse_args()
    if args.case:
        return run_case(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
