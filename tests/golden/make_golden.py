"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference Hashinator in its own CPU-only mode (oracle/_ref/ref_driver,
built by oracle/build_ref.sh from the reference source tree) on seeded inputs
from hashinator_gb300.workloads and stores inputs and outputs as compressed
.npz files. Needs the reference source tree (only present where the fixtures
are made); the fixtures themselves are committed and read by the tests.

    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py --extra    # only the edge cases in tests/golden/extra/
    python tests/golden/make_golden.py --seq      # operation sequences (tests/golden/seq/) and the
                                                  # full-size plain-map digests (cfg1_full_u32_sp21.json)
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from hashinator_gb300 import workloads  # noqa: E402

DRIVER = ROOT / "oracle" / "_ref" / "ref_driver"
OUT = Path(__file__).resolve().parent

FILL = {4: 0xA5A5A5A5, 8: 0xA5A5A5A5A5A5A5A5}

# name: (key bytes, size power, inserted keys, query hit fraction, erase fraction, seed)
CASES = {
    # the plain single-map workload at 1/256 scale: LF 0.5, 50/50 queries, 25% erased
    "u32_lf050_sp13": (4, 13, 1 << 12, 0.5, 0.25, 11),
    "u32_lf075_sp12": (4, 12, 3072, 0.5, 0.30, 12),
    "u32_lf090_sp12": (4, 12, int(0.9 * 4096), 0.5, 0.30, 13),
    "u64_lf050_sp12": (8, 12, 2048, 0.5, 0.30, 14),
    "u64_lf090_sp12": (8, 12, int(0.9 * 4096), 0.5, 0.30, 15),
}

# Edge cases, written to tests/golden/extra/: the remaining width x load-factor
# pair, queries that all hit or all miss, erasing every key, and tiny tables.
EXTRA_CASES = {
    "u64_lf075_sp12": (8, 12, 3072, 0.5, 0.30, 16),
    "u32_hit100_sp10": (4, 10, 400, 1.0, 0.50, 17),
    "u32_hit0_sp10": (4, 10, 400, 0.0, 0.0, 18),
    "u32_erase_all_sp8": (4, 8, 100, 0.5, 1.0, 19),
    "u32_tiny_sp2": (4, 2, 3, 0.5, 0.34, 20),
    "u64_tiny_sp3": (8, 3, 6, 0.5, 0.5, 22),
    "u64_ragged_sp11": (8, 11, 1001, 0.5, 0.27, 23),
}


def run_driver(width: int, sp: int, keys, vals, q, e) -> dict:
    dt = np.uint32 if width == 4 else np.uint64
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        hdr = np.array([0x48584752, width, sp, len(keys), len(q), len(e), FILL[width]], np.uint64)
        with open(fin, "wb") as f:
            for a in (hdr, keys.astype(dt), vals.astype(dt), q.astype(dt), e.astype(dt)):
                f.write(np.ascontiguousarray(a).tobytes())
        subprocess.run([str(DRIVER), str(fin), str(fout)], check=True)
        raw = fout.read_bytes()
    h = np.frombuffer(raw[:48], np.uint64)
    size_ins, size_er, tomb_er, n_erased, sp_final, n_map = (int(x) for x in h)
    off = 48
    nq = len(q)

    def take(count, dtype):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return a.copy()

    out = {
        "size_after_insert": size_ins, "size_after_erase": size_er, "tombstones_after_erase": tomb_er,
        "n_erased": n_erased, "size_power_final": sp_final,
        "q1_found": take(nq, np.uint8), "q1_vals": take(nq, dt),
        "q2_found": take(nq, np.uint8), "q2_vals": take(nq, dt),
    }
    mk, mv = take(n_map, dt), take(n_map, dt)
    o = np.argsort(mk, kind="stable")
    out["map_keys"], out["map_vals"] = mk[o], mv[o]
    return out


def make_case(name: str, width: int, sp: int, n: int, hit: float, erase: float, seed: int, out_dir: Path = OUT) -> None:
    keys, vals, q, e = workloads.map_workload(n, width, seed, hit_frac=hit, n_queries=2 * n if hit == 0.5 and
                                              name.startswith("u32_lf050") else n, erase_frac=erase)
    res = run_driver(width, sp, keys, vals, q, e)
    out_dir.mkdir(exist_ok=True)
    np.savez_compressed(out_dir / f"{name}.npz", key_bytes=width, size_power=sp,
                        fill_pattern=np.uint64(FILL[width]), seed=seed, keys=keys, vals=vals, queries=q, erase=e,
                        **res)
    print(f"{name}: n={n} size={res['size_after_insert']} erased={res['n_erased']} "
          f"tomb={res['tombstones_after_erase']} sp_final={res['size_power_final']}")


def make_duplicates() -> None:
    """Test_Duplicate_Insertion (unit_tests/hashmap_unit_test/main.cu:1064-1085):
    2^10 unique keys plus 2^10 extra copies of the first key, value = key."""
    width = 4
    keys = workloads.distinct_keys(1 << 10, width, 21)
    keys = np.concatenate([keys, np.full(1 << 10, keys[0], np.uint32)])
    rng = np.random.default_rng(21)
    rng.shuffle(keys)
    vals = keys.copy()
    uq = np.unique(keys)
    res = run_driver(width, 12, keys, vals, uq, uq[:0])
    np.savez_compressed(OUT / "u32_duplicates.npz", key_bytes=width, size_power=12,
                        fill_pattern=np.uint64(FILL[width]), seed=21, keys=keys, vals=vals, queries=uq,
                        erase=uq[:0], **res)
    print(f"u32_duplicates: size={res['size_after_insert']}")


# ---- operation sequences (ref_driver's op-script mode) ----------------------
OP_INSERT, OP_QUERY, OP_ERASE, OP_RESIZE, OP_DUMP = 1, 2, 3, 4, 5


def run_ops(width: int, sp: int, ops) -> list:
    """Runs ops = [(code, payload)] through the reference's CPU build; payloads: INSERT (keys, vals), QUERY keys,
    ERASE keys, RESIZE size power, DUMP None. Returns one result per op."""
    dt = np.uint32 if width == 4 else np.uint64
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as f:
            f.write(np.array([0x48584753, width, sp, len(ops), FILL[width]], np.uint64).tobytes())
            for code, pl in ops:
                if code == OP_INSERT:
                    k, v = pl
                    f.write(np.array([code, len(k)], np.uint64).tobytes())
                    f.write(k.astype(dt).tobytes() + v.astype(dt).tobytes())
                elif code in (OP_QUERY, OP_ERASE):
                    f.write(np.array([code, len(pl)], np.uint64).tobytes() + pl.astype(dt).tobytes())
                elif code == OP_RESIZE:
                    f.write(np.array([code, pl], np.uint64).tobytes())
                else:
                    f.write(np.array([code, 0], np.uint64).tobytes())
        subprocess.run([str(DRIVER), str(fin), str(fout)], check=True)
        raw = fout.read_bytes()
    off = 0

    def take(count, dtype):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return a.copy()

    res = []
    for code, pl in ops:
        if code == OP_INSERT:
            res.append({"size": int(take(1, np.uint64)[0])})
        elif code == OP_QUERY:
            res.append({"found": take(len(pl), np.uint8), "vals": take(len(pl), dt)})
        elif code == OP_ERASE:
            e = take(3, np.uint64)
            res.append({"erased": int(e[0]), "size": int(e[1])})
        elif code == OP_RESIZE:
            r = take(2, np.uint64)
            res.append({"size": int(r[0]), "size_power": int(r[1])})
        else:
            c = int(take(1, np.uint64)[0])
            mk, mv = take(c, dt), take(c, dt)
            o = np.argsort(mk, kind="stable")
            res.append({"map_keys": mk[o], "map_vals": mv[o]})
    assert off == len(raw)
    return res


def seq_ops(name: str):
    """The sequences: re-inserting erased keys after erase, upserting present keys, and clean (the CPU path's
    resize, a rehash that drops tombstones) followed by more inserts. Keys come from the bijective stream
    (distinct); 'absent' keys from a disjoint stretch of it."""
    import zlib
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    if name == "seq_u32_reinsert_after_erase":
        w, sp, seed = 4, 12, 31
        k = workloads.distinct_keys(2000, w, seed)
        v = workloads.values(2000, w, seed)
        absent = workloads.distinct_keys(200, w, seed, offset=4000)
        er = rng.permutation(1500)[:600]
        back = er[:300]
        v2 = workloads.values(300, w, seed + 1)
        ins2_k = np.concatenate([k[back], k[1500:2000]])
        ins2_v = np.concatenate([v2, v[1500:2000]])
        q = np.concatenate([k, absent])[rng.permutation(2200)]
        ops = [(OP_INSERT, (k[:1500], v[:1500])), (OP_ERASE, k[er]), (OP_QUERY, q), (OP_INSERT, (ins2_k, ins2_v)),
               (OP_QUERY, q), (OP_DUMP, None)]
    elif name == "seq_u32_upsert":
        w, sp, seed = 4, 12, 32
        k = workloads.distinct_keys(2200, w, seed)
        v = workloads.values(2200, w, seed)
        up = rng.permutation(2000)[:1000]
        ins2_k = np.concatenate([k[up], k[2000:2200]])
        ins2_v = np.concatenate([workloads.values(1000, w, seed + 1), v[2000:2200]])
        absent = workloads.distinct_keys(300, w, seed, offset=5000)
        q = np.concatenate([k, absent])[rng.permutation(2500)]
        ops = [(OP_INSERT, (k[:2000], v[:2000])), (OP_INSERT, (ins2_k, ins2_v)), (OP_QUERY, q), (OP_DUMP, None)]
    elif name == "seq_u64_erase_clean_upsert":
        w, sp, seed = 8, 12, 33
        k = workloads.distinct_keys(1800, w, seed)
        v = workloads.values(1800, w, seed)
        er = rng.permutation(1800)[:700]
        absent = workloads.distinct_keys(300, w, seed, offset=5000)
        q = np.concatenate([k, absent])[rng.permutation(2100)]
        keep = np.setdiff1d(np.arange(1800), er)
        ins2_k = np.concatenate([k[keep[:250]], k[er[:250]]])
        ins2_v = workloads.values(500, w, seed + 1)
        ops = [(OP_INSERT, (k, v)), (OP_ERASE, k[er]), (OP_RESIZE, sp), (OP_QUERY, q), (OP_INSERT, (ins2_k, ins2_v)),
               (OP_QUERY, q), (OP_DUMP, None)]
    elif name == "seq_u32_clean_then_insert":
        w, sp, seed = 4, 11, 34
        k = workloads.distinct_keys(1600, w, seed)
        v = workloads.values(1600, w, seed)
        er = rng.permutation(1200)[:400]
        absent = workloads.distinct_keys(100, w, seed, offset=3000)
        q = np.concatenate([k, absent])[rng.permutation(1700)]
        ops = [(OP_INSERT, (k[:1200], v[:1200])), (OP_ERASE, k[er]), (OP_RESIZE, sp),
               (OP_INSERT, (k[1200:], v[1200:])), (OP_QUERY, q), (OP_DUMP, None)]
    else:
        raise KeyError(name)
    return w, sp, ops


SEQ_CASES = ("seq_u32_reinsert_after_erase", "seq_u32_upsert", "seq_u64_erase_clean_upsert",
             "seq_u32_clean_then_insert")


def make_seq(name: str) -> None:
    w, sp, ops = seq_ops(name)
    res = run_ops(w, sp, ops)
    arrs = {"key_bytes": w, "size_power": sp, "fill_pattern": np.uint64(FILL[w]),
            "op_codes": np.array([c for c, _ in ops], np.int64)}
    for i, ((code, pl), r) in enumerate(zip(ops, res)):
        if code == OP_INSERT:
            arrs[f"op{i}_keys"], arrs[f"op{i}_vals"] = pl
        elif code in (OP_QUERY, OP_ERASE):
            arrs[f"op{i}_keys"] = pl
        elif code == OP_RESIZE:
            arrs[f"op{i}_sp"] = np.int64(pl)
        for kk, vv in r.items():
            arrs[f"out{i}_{kk}"] = vv
    (OUT / "seq").mkdir(exist_ok=True)
    np.savez_compressed(OUT / "seq" / f"{name}.npz", **arrs)
    print(f"{name}: {[c for c, _ in ops]} sizes {[r.get('size') for r in res]}")


# ---- the plain single-map workload at its full size, as digests -------------
CFG1 = {"n": 1 << 20, "size_power": 21, "seed": 2020, "erase_frac": 0.25}


def digest(a: np.ndarray) -> str:
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def cfg1_inputs():
    """2^20 u32 keys, 2^20 present + 2^20 absent queries (shuffled), a random 25% erased."""
    c = CFG1
    return workloads.map_workload(c["n"], 4, c["seed"], hit_frac=0.5, n_queries=2 * c["n"], erase_frac=c["erase_frac"])


def make_cfg1_full() -> None:
    import json
    keys, vals, q, e = cfg1_inputs()
    r = run_driver(4, CFG1["size_power"], keys, vals, q, e)
    d = dict(CFG1, key_bytes=4, fill_pattern=FILL[4], n_queries=len(q), n_erase=len(e),
             size_after_insert=r["size_after_insert"], size_after_erase=r["size_after_erase"], n_erased=r["n_erased"],
             sha256={"q1_vals": digest(r["q1_vals"]), "q2_vals": digest(r["q2_vals"]),
                     "map_keys": digest(r["map_keys"]), "map_vals": digest(r["map_vals"])},
             about="outputs of the reference's CPU-only build on the plain single-map workload (2^20 u32 keys into "
                   "2^21 buckets, 2^21 queries half present, 25% erased, queries again), as SHA-256 digests of the "
                   "query output arrays (misses keep fill_pattern) and of the key-sorted mapping; inputs are "
                   "regenerated from the seed by hashinator_gb300.workloads.map_workload")
    (OUT / "cfg1_full_u32_sp21.json").write_text(json.dumps(d, indent=1) + "\n")
    print(f"cfg1_full: size {r['size_after_insert']} -> {r['size_after_erase']}")


if __name__ == "__main__":
    if not DRIVER.exists():
        sys.exit(f"{DRIVER} missing: run oracle/build_ref.sh where the reference source tree is present")
    if "--seq" in sys.argv[1:]:
        for nm in SEQ_CASES:
            make_seq(nm)
        make_cfg1_full()
        sys.exit(0)
    if "--extra" not in sys.argv[1:]:
        for nm, args in CASES.items():
            make_case(nm, *args)
        make_duplicates()
    for nm, args in EXTRA_CASES.items():
        make_case(nm, *args, out_dir=OUT / "extra")
