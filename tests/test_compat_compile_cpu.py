"""The drop-in header compiles (no GPU needed): the reference's unit tests
written against it build for sm_103a, and an operation on a map with other
sentinels than the defaults is rejected at compile time."""
import subprocess

import pytest

from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _nvcc():
    from hashinator_gb300 import build
    try:
        return build._nvcc()
    except Exception:  # noqa: BLE001
        pytest.skip("nvcc not found")


def _compile(src: Path, out: Path, lambdas: bool = True):
    cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-I", str(ROOT / "include"),
           "-c", str(src), "-o", str(out)]
    if lambdas:
        cmd.insert(5, "--extended-lambda")
    return subprocess.run(cmd, capture_output=True, text=True, timeout=600)


@pytest.mark.parametrize("name,lambdas", [("test_compat", True), ("test_compat_device", True),
                                          ("test_device_api", False), ("test_compat_surface", True),
                                          ("test_splitvector_device", True)])
def test_cpp_sources_compile_against_the_header(tmp_path, name, lambdas):
    r = _compile(ROOT / "tests" / "cpp" / f"{name}.cu", tmp_path / f"{name}.o", lambdas)
    assert r.returncode == 0, r.stderr[-3000:]


def test_operation_with_custom_sentinels_is_rejected(tmp_path):
    src = tmp_path / "custom_sentinels.cu"
    src.write_text('#include "hashinator_compat.h"\n'
                   "int main() {\n"
                   "  Hashinator::Hashmap<uint32_t, uint32_t, 42, 41> h;\n"
                   "  static_assert(h.get_emptybucket() == 42 && h.get_tombstone() == 41, \"named\");\n"
                   "  uint32_t* k = nullptr;\n"
                   "  h.insert(k, k, 0);\n"
                   "  return 0;\n"
                   "}\n")
    r = _compile(src, tmp_path / "custom_sentinels.o", lambdas=False)
    assert r.returncode != 0
    out = r.stdout + r.stderr
    assert "libhx operates only on tables with the default sentinels" in out
    assert '"named"' not in out  # naming and reporting the sentinels compiles
