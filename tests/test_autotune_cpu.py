"""Host logic of libhx's batched-maps autotuner, without a GPU: the search
behind hx_batch_autotune (hashinator_gb300/csrc/hx_autotune.h) compiled into
a C++ host program (tests/cpp/test_autotune_host.cpp) that drives it with a
fake plan and a fake clock."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_autotune_search_on_the_host(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "test_autotune_host"
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", str(ROOT / "hashinator_gb300" / "csrc"),
                        str(ROOT / "tests" / "cpp" / "test_autotune_host.cpp"), "-o", str(exe)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "PASSED" in r.stdout, r.stdout[-2000:]


def test_python_caller_passes_the_grid_and_reports_the_best():
    """autotune_batch forwards its grid and reset to BatchPlan.autotune and shapes the result."""
    from hashinator_gb300 import autotune

    class Plan:
        def autotune(self, groups, blocks, tiles, reps, reset, stream):
            self.args = (groups, blocks, tiles, reps, reset, stream)
            return (8, 256, 2048, 1.25), [(1, 128, 512, 3.0), (8, 256, 2048, 1.25)]

    p = Plan()
    res = autotune.autotune_batch(p, None, groups=(1, 8), blocks=(128, 256), tiles=(512, 2048), reps=3, stream="s")
    assert p.args == ((1, 8), (128, 256), (512, 2048), 3, None, "s")
    assert res["best"] == (8, 256, 2048) and res["ms"] == 1.25 and len(res["trials"]) == 2
    assert res["trials"][1] == {"group": 8, "block": 256, "tile": 2048, "ms": 1.25}
