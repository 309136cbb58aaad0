"""The rest of the reference's Hashmap and split::tools surface through the
drop-in header (tests/cpp/test_compat_surface.cu): metadata copy, named
custom sentinels, arena and stack compaction forms, copy_keys_if, the loop
forms, swap / rehash / tombstone_ratio and the printing helpers. Compiled
against include/hashinator_compat.h, linked with libhx.so, run on the GPU."""
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def test_reference_surface_through_compat_header(hx, tmp_path):
    from hashinator_gb300 import build
    exe = tmp_path / "test_compat_surface"
    cmd = [build._nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "--extended-lambda",
           "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "test_compat_surface.cu"), "-o", str(exe),
           "-L", str(hx.LIB_PATH.parent), "-lhx", f"-Xlinker=-rpath,{hx.LIB_PATH.parent}"]
    subprocess.run(cmd, check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout[-4000:], r.stderr[-2000:])
    assert r.returncode == 0 and "PASSED" in r.stdout
