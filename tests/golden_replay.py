"""Replays the reference-run fixtures of operation sequences (tests/golden/seq/)
and checks the full-size plain-map digests (tests/golden/cfg1_full_u32_sp21.json)
on any map with the Hashmap-like adapter below — the oracle on the CPU and
libhx on the GPU — comparing every recorded result exactly: sizes after each
insert, erase and clean, every query output buffer (same pre-fill), and the
key-sorted mapping. The reference's CPU path reuses tombstones and rehashes
on its own, so bucket layouts and tombstone counts are not compared."""
from __future__ import annotations

import hashlib
import json

import numpy as np

from conftest import GOLDEN

OP_INSERT, OP_QUERY, OP_ERASE, OP_RESIZE, OP_DUMP = 1, 2, 3, 4, 5


def seq_cases():
    return sorted(p.stem for p in (GOLDEN / "seq").glob("*.npz"))


def load_seq(name):
    with np.load(GOLDEN / "seq" / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def replay(g, m):
    """m: insert(keys, vals) (no growth), retrieve(keys, out), erase(keys), clean(sp) (the reference's
    resize(sp): a rehash that drops tombstones), fill() -> int, mapping() -> (keys, vals) sorted by key."""
    dt = np.uint32 if int(g["key_bytes"]) == 4 else np.uint64
    fill = dt(int(g["fill_pattern"]))
    for i, code in enumerate(g["op_codes"].tolist()):
        if code == OP_INSERT:
            m.insert(g[f"op{i}_keys"], g[f"op{i}_vals"])
            assert m.fill() == int(g[f"out{i}_size"]), f"op {i}: size after insert"
        elif code == OP_QUERY:
            out = np.full(len(g[f"op{i}_keys"]), fill, dt)
            m.retrieve(g[f"op{i}_keys"], out)
            np.testing.assert_array_equal(out, g[f"out{i}_vals"], err_msg=f"op {i}: query outputs")
        elif code == OP_ERASE:
            before = m.fill()
            m.erase(g[f"op{i}_keys"])
            assert m.fill() == int(g[f"out{i}_size"]), f"op {i}: size after erase"
            assert before - m.fill() == int(g[f"out{i}_erased"]), f"op {i}: erased count"
        elif code == OP_RESIZE:
            m.clean(int(g[f"op{i}_sp"]))
            assert m.fill() == int(g[f"out{i}_size"]), f"op {i}: size after clean"
        elif code == OP_DUMP:
            k, v = m.mapping()
            np.testing.assert_array_equal(k, g[f"out{i}_map_keys"], err_msg=f"op {i}: mapping keys")
            np.testing.assert_array_equal(v, g[f"out{i}_map_vals"], err_msg=f"op {i}: mapping values")


def cfg1_expected():
    return json.loads((GOLDEN / "cfg1_full_u32_sp21.json").read_text())


def cfg1_inputs(d):
    from hashinator_gb300 import workloads
    return workloads.map_workload(d["n"], 4, d["seed"], hit_frac=0.5, n_queries=d["n_queries"],
                                  erase_frac=d["erase_frac"])


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def check_cfg1(m, d):
    """Insert, query, erase, query, mapping on m (a fresh map of 2^21 buckets); every digest must match."""
    keys, vals, q, e = cfg1_inputs(d)
    assert len(q) == d["n_queries"] and len(e) == d["n_erase"]
    fill = np.uint32(d["fill_pattern"])
    m.insert(keys, vals)
    assert m.fill() == d["size_after_insert"]
    out = np.full(len(q), fill, np.uint32)
    m.retrieve(q, out)
    assert digest(out) == d["sha256"]["q1_vals"]
    m.erase(e)
    assert m.fill() == d["size_after_erase"]
    out = np.full(len(q), fill, np.uint32)
    m.retrieve(q, out)
    assert digest(out) == d["sha256"]["q2_vals"]
    k, v = m.mapping()
    assert digest(k) == d["sha256"]["map_keys"] and digest(v) == d["sha256"]["map_vals"]
