"""CPU checks of the C-ABI boundary: libhx.so builds, loads, and exports every
entry point declared in include/*.h (no compute calls: no GPU here)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    syms = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"^\s*typedef[^;]*;", "", text, flags=re.M)  # function-pointer types are not entry points
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(hx_[a-z0-9_]+)\s*\(", text, flags=re.M):
            syms.add(m.group(1))
    return sorted(syms)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for must in ("hx_map_create", "hx_insert", "hx_insert_pairs", "hx_retrieve", "hx_retrieve_pairs", "hx_erase",
                 "hx_clean_tombstones", "hx_extract_pattern", "hx_copy_if", "hx_exclusive_scan_u32"):
        assert must in syms


def test_library_exports_every_declared_symbol(hx):
    lib = ctypes.CDLL(str(hx.LIB_PATH))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_status_strings_and_argument_checks(hx):
    lib = hx.lib()
    assert lib.hx_status_string(0) == b"ok"
    # argument validation happens before any device work
    out = ctypes.c_void_p()
    assert lib.hx_map_create(ctypes.byref(out), 4, 8, 10, None) == hx.HX_ERR_INVALID_ARG
    assert lib.hx_map_create(ctypes.byref(out), 4, 4, 0, None) == hx.HX_ERR_INVALID_ARG
    assert lib.hx_map_create(ctypes.byref(out), 4, 4, 32, None) == hx.HX_ERR_INVALID_ARG
    assert lib.hx_insert(None, None, None, 0, 0.5, None) == hx.HX_ERR_INVALID_ARG
    assert lib.hx_retrieve(None, None, None, 0, None) == hx.HX_ERR_INVALID_ARG
    b = ctypes.c_uint64()
    assert lib.hx_scratch_bytes(7, 10, ctypes.byref(b)) == hx.HX_ERR_INVALID_ARG
    assert lib.hx_scratch_bytes(hx.SCRATCH_SCAN, 1 << 20, ctypes.byref(b)) == hx.HX_OK and b.value > 256
    p = hx.Pred.mod_lt(0, 1).c()
    assert lib.hx_copy_if(None, None, 0, 4, ctypes.byref(p), 0, None, None, None, 0, None) == hx.HX_ERR_INVALID_ARG
    assert lib.hx_exclusive_scan_u32(None, None, 0, None, 0, None) == hx.HX_OK  # n == 0 is a no-op


def test_no_cpu_fallback_in_product():
    """The product package must not reach into the oracle."""
    for p in (ROOT / "hashinator_gb300").rglob("*.py"):
        src = p.read_text()
        assert "import oracle" not in src and "from oracle" not in src, p


def test_null_handles_and_outputs_are_rejected(hx):
    """Every entry point that takes a map, batch, plan or server handle returns HX_ERR_INVALID_ARG for a NULL
    handle before any device work, and the create calls reject a NULL output and bad sizes (no GPU here)."""
    lib = hx.lib()
    no_handle = {"hx_status_string", "hx_last_cuda_error", "hx_kernel_launch_count", "hx_set_l2_fetch_granularity",
                 "hx_diag_random_access", "hx_scratch_bytes", "hx_exclusive_scan_u32", "hx_copy_if",
                 "hx_map_create", "hx_batch_create", "hx_server_create", "hx_exclusive_scan_u32_noalloc"}
    names = sorted((set(hx._SIGS) | set(hx._EXTRA_SIGS)) - no_handle)
    assert len(names) >= 40
    for n in names:
        f = getattr(lib, n)
        args = [0 if isinstance(t, type) and issubclass(t, (ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64,
                                                               ctypes.c_int32, ctypes.c_float)) else None
                for t in f.argtypes]
        assert f(*args) == hx.HX_ERR_INVALID_ARG, n
    sp = (ctypes.c_int32 * 2)(10, 10)
    h = ctypes.c_void_p()
    assert lib.hx_map_create(None, 4, 4, 10, None) == hx.HX_ERR_INVALID_ARG
    assert lib.hx_batch_create(None, 2, sp, 4, 4, None) == hx.HX_ERR_INVALID_ARG
    assert lib.hx_batch_create(ctypes.byref(h), 0, sp, 4, 4, None) == hx.HX_ERR_INVALID_ARG
    assert lib.hx_server_create(None, 8, 1 << 30, 0.8, 4, 16, 1 << 20, 2) == hx.HX_ERR_INVALID_ARG
    assert lib.hx_server_create(ctypes.byref(h), 8, 1 << 30, 0.0, 4, 16, 1 << 20, 2) == hx.HX_ERR_INVALID_ARG
    assert lib.hx_exclusive_scan_u32_noalloc(None, None, (1 << 28) + 1, None) == hx.HX_ERR_INVALID_ARG


def test_scratch_sizes_and_undersized_caller_scratch(hx):
    """hx_scratch_bytes: the scan needs the larger of its two kernels' scratch — a 256-byte header and one
    8-byte status per 12288-element tile (buffers that are not 16-byte aligned), or a 256-byte header and
    2 * 1 + 2 count slots of 8 bytes for each CTA, at most one CTA per 16384-element (64 KiB) slice and 1024
    CTAs (the phase-partitioned kernel); copy_if needs at least as much plus a 256-byte count area, never
    shrinking as n grows. A caller buffer smaller than
    the need is rejected before any device work: every call here is one that must be rejected, so the fake
    pointers are never dereferenced."""
    lib = hx.lib()
    b = ctypes.c_uint64()

    def need(op, n):
        assert lib.hx_scratch_bytes(op, n, ctypes.byref(b)) == hx.HX_OK
        return b.value

    for n in (0, 1, 4095, 4096, 4097, 1 << 20, (1 << 28) + 3):
        assert need(hx.SCRATCH_SCAN, n) == max(256 + 8 * max(1, -(-n // 12288)),
                                               256 + 8 * 4 * min(1024, max(1, -(-n // 16384))))
    prev = 0
    for n in (0, 1, 100, 5000, 1 << 16, 1 << 20, 1 << 24):
        c = need(hx.SCRATCH_COPY_IF, n)
        assert c >= prev and c >= 256 + 8 + 256
        prev = c
    fake = ctypes.c_void_p(256)
    n = 5000
    p = hx.Pred.mod_lt(100, 50).c()
    # 256 bytes is below every element width's need (a header, at least one status, the count area)
    for elem in (4, 8, 16):
        assert lib.hx_copy_if(fake, fake, n, elem, ctypes.byref(p), n, None, None, fake, 256, None) == \
            hx.HX_ERR_INVALID_ARG
    assert lib.hx_exclusive_scan_u32(fake, fake, n, fake, need(hx.SCRATCH_SCAN, n) - 1, None) == hx.HX_ERR_INVALID_ARG


def test_header_is_plain_c(tmp_path):
    """include/hx.h compiles as C99 with warnings as errors, so C code and any FFI generator can use it."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        import pytest
        pytest.skip("no C compiler")
    src = tmp_path / "use_hx.c"
    src.write_text('#include "hx.h"\n'
                   "int main(void) {\n"
                   "  hx_map* m = 0; hx_info info; hx_pred p = {HX_PRED_MOD_LT, HX_FIELD_ELEM, 0, 0, 100, 50};\n"
                   "  (void)m; (void)info; (void)p;\n"
                   "  return hx_status_string(HX_OK) ? 0 : 1;\n"
                   "}\n")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", str(ROOT / "include"),
                        "-c", str(src), "-o", str(tmp_path / "use_hx.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_misaligned_device_arrays_are_rejected(hx):
    """Device arrays must start at a multiple of their element size (4-byte words, 8- or 16-byte pairs): a
    misaligned pointer is rejected before any device work. Every call here must be rejected, so the fake
    pointers are never dereferenced; the aligned control calls fail later, on the scratch check, which shows
    that the alignment check is what rejected the others."""
    lib = hx.lib()
    p = hx.Pred.mod_lt(100, 50).c()
    n = 5000
    ok = 1 << 20
    for elem in (4, 8, 16):
        for off in range(1, elem):
            bad = ctypes.c_void_p(ok + off)
            good = ctypes.c_void_p(ok)
            assert lib.hx_copy_if(bad, good, n, elem, ctypes.byref(p), n, None, None, good, 1 << 20, None) == \
                hx.HX_ERR_INVALID_ARG
            assert lib.hx_copy_if(good, bad, n, elem, ctypes.byref(p), n, None, None, good, 1 << 20, None) == \
                hx.HX_ERR_INVALID_ARG
    for off in (1, 2, 3):
        bad, good = ctypes.c_void_p(ok + off), ctypes.c_void_p(ok)
        assert lib.hx_exclusive_scan_u32(bad, good, n, good, 1 << 20, None) == hx.HX_ERR_INVALID_ARG
        assert lib.hx_exclusive_scan_u32(good, bad, n, good, 1 << 20, None) == hx.HX_ERR_INVALID_ARG
        assert lib.hx_exclusive_scan_u32_noalloc(bad, good, n, None) == hx.HX_ERR_INVALID_ARG
        assert lib.hx_exclusive_scan_u32_noalloc(good, bad, n, None) == hx.HX_ERR_INVALID_ARG
    # controls: aligned, with an undersized caller scratch, rejected by the scratch check instead
    good = ctypes.c_void_p(ok)
    assert lib.hx_copy_if(good, good, n, 8, ctypes.byref(p), n, None, None, good, 16, None) == hx.HX_ERR_INVALID_ARG
    assert lib.hx_exclusive_scan_u32(good, good, n, good, 16, None) == hx.HX_ERR_INVALID_ARG
