"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference Hashinator in its own CPU-only mode (oracle/_ref/ref_driver,
built by oracle/build_ref.sh from the reference source tree) on seeded inputs
from hashinator_gb300.workloads and stores inputs and outputs as compressed
.npz files. Needs the reference source tree (only present where the fixtures
are made); the fixtures themselves are committed and read by the tests.

    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py --extra    # only the edge cases in tests/golden/extra/
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


if __name__ == "__main__":
    if not DRIVER.exists():
        sys.exit(f"{DRIVER} missing: run oracle/build_ref.sh where the reference source tree is present")
    if "--extra" not in sys.argv[1:]:
        for nm, args in CASES.items():
            make_case(nm, *args)
        make_duplicates()
    for nm, args in EXTRA_CASES.items():
        make_case(nm, *args, out_dir=OUT / "extra")
