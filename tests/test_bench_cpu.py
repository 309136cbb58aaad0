"""bench.py's reference arm (the reference's CPU path, restated in the oracle,
on the host cores) runs without a GPU: its JSON line carries every key of the
benchmark contract, and its metric, unit and config are the headline arm's."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line():
    sys.path.insert(0, str(ROOT))
    import bench

    # a 2^22-key headline (the default is 2^26; the arm runs whatever size it is given, in full)
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3", "--log-keys", "22"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 3
    assert d["metric"] == bench.headline_metric(22) and d["unit"] == "Mkeys/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0
    cfg = dict(d["config"])
    assert cfg.pop("reference_host_threads") >= 1 and cfg.pop("reference_sample").endswith("(the full workload)")
    assert cfg == bench.headline_config(22, 0)
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["cores"] >= 1
    assert cb["sample"]
    assert cb["host"]["nproc"] >= cb["cores"] and cb["host"]["cpu_model"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_cpu_streaming_baseline_small():
    sys.path.insert(0, str(ROOT))
    import bench

    d = bench.cpu_streaming(log_n=16, threads=4, reps=1)  # asserts chunked == serial results inside
    assert d["threads"] == 4 and d["kind"] == "port"
    for s, lo, hi in ((1, 0.005, 0.02), (50, 0.45, 0.55), (99, 0.97, 1.0)):
        r = d[f"copy_if_s{s}"]
        assert lo < r["selected"] / (1 << 16) < hi
        assert r["one_core"]["ms"] > 0 and r["all_threads"]["GB_s"] > 0
    assert d["exclusive_scan"]["one_core"]["Gelem_s"] > 0


def test_cpu_batched_baseline_against_a_dict_model():
    sys.path.insert(0, str(ROOT))
    import numpy as np
    import bench
    from hashinator_gb300 import workloads

    w = workloads.batched_workload(48, 7)
    io, qo = w["ins_offsets"].astype(np.int64), w["query_offsets"].astype(np.int64)
    expect = np.full(len(w["queries"]), 0xFFFFFFFF, np.uint32)  # misses keep the pre-fill
    for i in range(48):
        d = dict(zip(w["keys"][io[i]:io[i + 1]].tolist(), w["vals"][io[i]:io[i + 1]].tolist()))
        q = w["queries"][qo[i]:qo[i + 1]].tolist()
        expect[qo[i]:qo[i + 1]] = [d.get(k, 0xFFFFFFFF) for k in q]
    r = bench.cpu_batched(w, expect.view(np.int32), threads=4, reps=1)
    assert r["query_outputs_equal_gpu"] is True and r["Mops_s"] > 0
    bad = expect.copy()
    bad[len(bad) // 2] ^= 1
    assert bench.cpu_batched(w, bad, threads=2, reps=1)["query_outputs_equal_gpu"] is False


def test_cpu_serving_baseline_against_a_dict_model():
    sys.path.insert(0, str(ROOT))
    import numpy as np
    import bench
    from hashinator_gb300 import workloads

    nm, nr = 6, 300
    tr = workloads.serving_trace(nm, nr, 21, init_log=(4.0, 8.0), size_log=(0.0, 7.0), width=8)
    io, ro = tr["init_offsets"], tr["req_offsets"]
    d = [dict(zip(tr["init_keys"][io[m]:io[m + 1]].tolist(), tr["init_vals"][io[m]:io[m + 1]].tolist()))
         for m in range(nm)]
    model = np.zeros(len(tr["req_keys"]), np.uint64)  # a miss may hold anything in the GPU's buffer
    hits = 0
    for i in range(nr):
        m, op = int(tr["req_map"][i]), int(tr["req_op"][i])
        ks = tr["req_keys"][ro[i]:ro[i + 1]].tolist()
        if op == 0:
            d[m].update(zip(ks, tr["req_vals"][ro[i]:ro[i + 1]].tolist()))
        elif op == 1:
            for j, k in enumerate(ks):
                if k in d[m]:
                    model[ro[i] + j] = d[m][k]
                    hits += 1
        else:
            for k in ks:
                d[m].pop(k, None)
    r = bench.cpu_serving(tr, model.view(np.int64), threads=3)
    assert r["query_hits_equal_gpu"] is True and r["query_hits_compared"] == hits > 0
    assert r["rehashes"] > 0  # the trace grows some maps
    bad = model.copy()
    bad[np.flatnonzero(bad)[hits // 2]] ^= np.uint64(1)
    assert bench.cpu_serving(tr, bad, threads=2)["query_hits_equal_gpu"] is False


def test_reference_arm_under_two_ranks():
    """Launched like the multi-GPU runs (torch.distributed.run, 2 processes), the reference arm prints one JSON
    line from rank 0 with n_gpus = 2 and every rank exits 0."""
    import os
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
                        "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--log-keys", "20"],
                       cwd=ROOT, capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
