"""The tuning variants that the kernels keep behind compile-time switches
still build for sm_103a (no GPU needed): the streaming compaction's per-lane
ranking (HX_STREAM_LANE_CHUNKS) and other slice geometries, and the batched
kernel with several inserts in flight per thread. The product builds none of
them; they stay buildable so that a sweep can time them against the default."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _nvcc():
    from hashinator_gb300 import build
    try:
        return build._nvcc()
    except Exception:  # noqa: BLE001
        pytest.skip("nvcc not found")


@pytest.mark.parametrize("src,defines", [
    ("hx_scan.cu", ["-DHX_STREAM_LANE_CHUNKS=1"]),
    ("hx_scan.cu", ["-DHX_STREAM_BLOCK=1024", "-DHX_STREAM_R=4"]),
    ("hx_scan.cu", ["-DHX_STREAM_R=6", "-DHX_STREAM_STAGES=4", "-DHX_STREAM_DEFER=2"]),
    ("hx_batch.cu", ["-DHX_BATCH_INSERTS_IN_FLIGHT=2"]),
])
def test_variant_builds(tmp_path, src, defines):
    cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", *defines,
           "-c", str(ROOT / "hashinator_gb300" / "csrc" / src), "-o", str(tmp_path / "v.o")]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
