"""The reference's own hot-path unit tests (ported to a tiny harness) compiled
against the drop-in C++ header include/hashinator_compat.h and linked with
libhx.so, run on the GPU."""
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def test_reference_unit_tests_through_compat_header(hx, tmp_path):
    from hashinator_gb300 import build
    exe = tmp_path / "test_compat"
    cmd = [build._nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "--extended-lambda",
           "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "test_compat.cu"), "-o", str(exe),
           "-L", str(hx.LIB_PATH.parent), "-lhx", f"-Xlinker=-rpath,{hx.LIB_PATH.parent}"]
    subprocess.run(cmd, check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout[-4000:], r.stderr[-2000:])
    assert r.returncode == 0 and "PASSED" in r.stdout


def test_device_api_from_user_kernels(hx, tmp_path):
    from hashinator_gb300 import build
    exe = tmp_path / "test_device_api"
    cmd = [build._nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
           "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "test_device_api.cu"), "-o", str(exe),
           "-L", str(hx.LIB_PATH.parent), "-lhx", f"-Xlinker=-rpath,{hx.LIB_PATH.parent}"]
    subprocess.run(cmd, check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout[-4000:], r.stderr[-2000:])
    assert r.returncode == 0 and "PASSED" in r.stdout


def test_reference_device_api_tests_through_compat_header(hx, tmp_path):
    """User kernels that take the map's device copy (upload()) and call the
    element, iterator and warp accessors, as the reference's unit tests do."""
    from hashinator_gb300 import build
    exe = tmp_path / "test_compat_device"
    cmd = [build._nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "--extended-lambda",
           "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "test_compat_device.cu"), "-o", str(exe),
           "-L", str(hx.LIB_PATH.parent), "-lhx", f"-Xlinker=-rpath,{hx.LIB_PATH.parent}"]
    subprocess.run(cmd, check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout[-4000:], r.stderr[-2000:])
    assert r.returncode == 0 and "PASSED" in r.stdout


def test_splitvector_device_surface_and_caller_scratch(hx, tmp_path):
    """The SplitVector device surface (upload, device_push_back, device_resize, device_insert) with the
    reference's own device tests and a concurrent device_push_back checked against a host model; the
    preallocated compactions from several host threads and streams with caller scratch and no stream-ordered
    allocation; copy_if_loop reading a device-side size; functor copy_if equal to libhx's descriptor copy_if."""
    from hashinator_gb300 import build
    exe = tmp_path / "test_splitvector_device"
    cmd = [build._nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "--extended-lambda",
           "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "test_splitvector_device.cu"), "-o", str(exe),
           "-L", str(hx.LIB_PATH.parent), "-lhx", f"-Xlinker=-rpath,{hx.LIB_PATH.parent}"]
    subprocess.run(cmd, check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout[-4000:], r.stderr[-2000:])
    assert r.returncode == 0 and "PASSED" in r.stdout
