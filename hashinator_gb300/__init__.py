"""hashinator_gb300 — GB300-native Hashinator hot path.

Python mirror of the reference's accelerated API over the C ABI of libhx.so
(include/hx.h). Names follow Hashinator::Hashmap (hashinator/hashinator.h)
and split::tools (splitvector/split_tools.h):

    m = Hashmap(size_power=21, key_bytes=4)      # Hashmap<uint32_t,uint32_t>(21)
    m.insert(keys, vals, target_lf=0.5)          # insert(keys, vals, len, targetLF)
    m.retrieve(keys, out)                        # retrieve(keys, vals, len)
    m.erase(keys)                                # erase(keys, len)
    m.clean_tombstones()
    n = m.extract_pattern(Pred.value_even(), out)
    tools.copy_if(inp, out, Pred.mod_lt(100, 50))
    tools.split_prefix_scan(inp, out)

Arrays are CUDA tensors (torch) or raw device addresses (int). 4-byte keys
use int32/uint32 tensors, 8-byte keys int64/uint64 tensors; values are
reinterpreted bit-for-bit. The package never falls back to a CPU path: if
libhx.so is missing, every call raises.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

__all__ = ["lib", "HXError", "Hashmap", "Pred", "tools", "Batch", "BatchPlan", "Server", "Request", "Completion",
           "STATUS_SUCCESS", "STATUS_FAIL", "STATUS_INVALID", "LIB_PATH", "Info", "BatchTrial"]

LIB_PATH = Path(__file__).resolve().parent / "libhx.so"

# hx_status
HX_OK, HX_ERR_OVERFLOW, HX_ERR_OOM, HX_ERR_INVALID_ARG, HX_ERR_CUDA, HX_ERR_TIMEOUT, HX_ERR_CAPACITY = range(7)
# Hashinator::status (common.h:85)
STATUS_SUCCESS, STATUS_FAIL, STATUS_INVALID = 0, 1, 2

PRED_ALL, PRED_MOD_LT, PRED_LT, PRED_GE, PRED_EQ, PRED_NE, PRED_MASK_EQ, PRED_RANGE, PRED_VALID, PRED_NOT_HOME = range(10)
FIELD_ELEM, FIELD_KEY, FIELD_VALUE = 0, 1, 2
PRED_SKIP_SENTINELS, PRED_NEGATE = 1, 2
SCRATCH_SCAN, SCRATCH_COPY_IF = 0, 1


class HXError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        msg = _lib_handle.hx_status_string(status).decode() if _lib_handle is not None else str(status)
        extra = ""
        if status == HX_ERR_CUDA and _lib_handle is not None:
            extra = f" (cudaError {_lib_handle.hx_last_cuda_error()})"
        super().__init__(f"{where}: {msg}{extra}")


class Info(ctypes.Structure):
    """hx_info, the host copy of Hashinator::Info (defaults.h:44-54)."""
    _fields_ = [
        ("size_power", ctypes.c_int32),
        ("err", ctypes.c_int32),
        ("fill", ctypes.c_uint64),
        ("current_max_bucket_overflow", ctypes.c_uint64),
        ("tombstone_counter", ctypes.c_uint64),
        ("max_probe", ctypes.c_uint64),
        ("bucket_count", ctypes.c_uint64),
        ("last_clean_moved", ctypes.c_uint64),
    ]


class _CPred(ctypes.Structure):
    _fields_ = [("op", ctypes.c_uint32), ("field", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("a", ctypes.c_uint64), ("b", ctypes.c_uint64)]


class _CBatchWork(ctypes.Structure):
    _fields_ = [("ins_keys", ctypes.c_void_p), ("ins_vals", ctypes.c_void_p),
                ("ins_offsets", ctypes.POINTER(ctypes.c_uint64)),
                ("query_keys", ctypes.c_void_p), ("query_out", ctypes.c_void_p),
                ("query_offsets", ctypes.POINTER(ctypes.c_uint64)),
                ("erase_keys", ctypes.c_void_p), ("erase_offsets", ctypes.POINTER(ctypes.c_uint64)),
                ("clean", ctypes.c_int)]


class Request(ctypes.Structure):
    """hx_request."""
    _fields_ = [("map", ctypes.c_uint32), ("op", ctypes.c_uint32), ("keys", ctypes.c_void_p),
                ("vals", ctypes.c_void_p), ("out", ctypes.c_void_p), ("n", ctypes.c_uint64), ("tag", ctypes.c_uint64)]


class Completion(ctypes.Structure):
    """hx_completion."""
    _fields_ = [("tag", ctypes.c_uint64), ("complete_ns", ctypes.c_uint64), ("status", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


OP_INSERT, OP_QUERY, OP_ERASE = 0, 1, 2


class ServerStats(ctypes.Structure):
    """hx_server_stats."""
    _fields_ = [("rounds", ctypes.c_uint64), ("requests", ctypes.c_uint64), ("keys", ctypes.c_uint64),
                ("growths", ctypes.c_uint64), ("growth_bytes", ctypes.c_uint64), ("rejected", ctypes.c_uint64),
                ("timeouts", ctypes.c_uint64), ("host_ns_step", ctypes.c_uint64), ("max_stage_depth", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]

_lib_handle = None

_SIGS = {
    "hx_map_create": [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p],
    "hx_map_destroy": [ctypes.c_void_p],
    "hx_insert": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_float, ctypes.c_void_p],
    "hx_insert_pairs": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_float, ctypes.c_void_p],
    "hx_retrieve": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p],
    "hx_retrieve_pairs": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p],
    "hx_erase": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p],
    "hx_clean_tombstones": [ctypes.c_void_p, ctypes.c_void_p],
    "hx_extract_pattern": [ctypes.c_void_p, ctypes.POINTER(_CPred), ctypes.c_void_p, ctypes.c_uint64,
                           ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64), ctypes.c_void_p],
    "hx_extract_keys": [ctypes.c_void_p, ctypes.POINTER(_CPred), ctypes.c_void_p, ctypes.c_uint64,
                        ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64), ctypes.c_void_p],
    "hx_map_device_view": [ctypes.c_void_p, ctypes.c_void_p],
    "hx_resize": [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p],
    "hx_insert_index": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_float, ctypes.c_void_p],
    "hx_resize_to_lf": [ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p],
    "hx_perform_cleanup_tasks": [ctypes.c_void_p, ctypes.c_void_p],
    "hx_clear": [ctypes.c_void_p, ctypes.c_void_p],
    "hx_get_info": [ctypes.c_void_p, ctypes.POINTER(Info), ctypes.c_void_p],
    "hx_peek_status": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p],
    "hx_bucket_data": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_uint64)],
    "hx_map_set_tuning": [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int],
    "hx_map_set_insert_mode": [ctypes.c_void_p, ctypes.c_int],
    "hx_map_set_window_bytes": [ctypes.c_void_p, ctypes.c_int],
    "hx_set_l2_fetch_granularity": [ctypes.c_int],
    "hx_diag_random_access": [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p],
    "hx_scratch_bytes": [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)],
    "hx_exclusive_scan_u32": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64,
                              ctypes.c_void_p],
    "hx_copy_if": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(_CPred),
                   ctypes.c_uint64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64), ctypes.c_void_p,
                   ctypes.c_uint64, ctypes.c_void_p],
}
_SIGS.update({
    "hx_batch_create": [ctypes.POINTER(ctypes.c_void_p), ctypes.c_uint32, ctypes.POINTER(ctypes.c_int32), ctypes.c_int,
                        ctypes.c_int, ctypes.c_void_p],
    "hx_batch_destroy": [ctypes.c_void_p],
    "hx_batch_clear": [ctypes.c_void_p, ctypes.c_void_p],
    "hx_batch_map_info": [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(Info), ctypes.c_void_p],
    "hx_batch_bucket_data": [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p),
                             ctypes.POINTER(ctypes.c_uint64)],
    "hx_batch_plan_create": [ctypes.c_void_p, ctypes.POINTER(_CBatchWork), ctypes.POINTER(ctypes.c_void_p),
                             ctypes.c_void_p],
    "hx_batch_plan_destroy": [ctypes.c_void_p],
    "hx_batch_set_tuning": [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p],
    "hx_batch_run": [ctypes.c_void_p, ctypes.c_void_p],
    "hx_batch_run_graph": [ctypes.c_void_p, ctypes.c_void_p],
    "hx_batch_autotune": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_uint32,
                          ctypes.POINTER(ctypes.c_int32), ctypes.c_uint32, ctypes.POINTER(ctypes.c_int32),
                          ctypes.c_uint32, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                          ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p],
    "hx_batch_run_per_map": [ctypes.c_void_p, ctypes.c_void_p],
    "hx_batch_check": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p],
    "hx_batch_inject_stall": [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_void_p],
})
_SIGS.update({
    "hx_server_create": [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_uint64, ctypes.c_float,
                         ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32],
    "hx_server_destroy": [ctypes.c_void_p],
    "hx_server_add_map": [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_uint32)],
    "hx_server_submit": [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.c_uint32],
    "hx_server_step": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)],
    "hx_server_poll": [ctypes.c_void_p, ctypes.POINTER(Completion), ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)],
    "hx_server_drain": [ctypes.c_void_p],
    "hx_server_map_info": [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(Info)],
    "hx_server_bucket_data": [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p),
                              ctypes.POINTER(ctypes.c_uint64)],
    "hx_server_memory": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)],
    "hx_server_get_stats": [ctypes.c_void_p, ctypes.POINTER(ServerStats)],
    "hx_server_run_trace": [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.c_void_p, ctypes.c_uint32,
                            ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)],
})
_EXTRA_SIGS = {
    "hx_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "hx_last_cuda_error": ([], ctypes.c_int),
    "hx_kernel_launch_count": ([], ctypes.c_uint64),
}


def lib(path: str | os.PathLike | None = None) -> ctypes.CDLL:
    """Load libhx.so (once). Raises if it has not been built."""
    global _lib_handle
    if _lib_handle is not None:
        return _lib_handle
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -m hashinator_gb300.build` "
                           "(there is no CPU fallback)")
    h = ctypes.CDLL(str(p))
    for name, args in _SIGS.items():
        f = getattr(h, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    for name, (args, res) in _EXTRA_SIGS.items():
        f = getattr(h, name)
        f.argtypes = args
        f.restype = res
    _lib_handle = h
    for name, (args, res) in _OPTIONAL_SIGS.items():
        f = getattr(h, name, None)
        if f is not None:
            f.argtypes = args
            f.restype = res
    return h


_OPTIONAL_SIGS: dict = {}


def _check(status: int, where: str) -> None:
    if status != HX_OK:
        raise HXError(status, where)


def _ptr(x) -> int:
    """Device address of a CUDA tensor or a raw int address."""
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if not x.is_cuda:
            raise ValueError("libhx takes device memory: pass a CUDA tensor")
        if not x.is_contiguous():
            raise ValueError("libhx takes contiguous arrays")
        return x.data_ptr()
    raise TypeError(f"cannot take a device address of {type(x)!r}")


def _numel(x) -> int:
    return x.numel() if hasattr(x, "numel") else len(x)


def _stream(stream) -> int:
    if stream is None:
        try:
            import torch
            return torch.cuda.current_stream().cuda_stream
        except Exception:
            return 0
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class Pred:
    """hx_pred descriptors for the reference's `Rule` functors."""

    def __init__(self, op: int, field: int = FIELD_ELEM, a: int = 0, b: int = 0, flags: int = 0):
        self.op, self.field, self.a, self.b, self.flags = op, field, a, b, flags

    def c(self) -> _CPred:
        return _CPred(self.op, self.field, self.flags, 0, self.a, self.b)

    # scalar rules
    @staticmethod
    def mod_lt(a: int, s: int) -> "Pred":      # (x % a) < s
        return Pred(PRED_MOD_LT, FIELD_ELEM, a, s)

    @staticmethod
    def even(field: int = FIELD_ELEM) -> "Pred":
        return Pred(PRED_MASK_EQ, field, 1, 0)

    @staticmethod
    def lt(a: int, field: int = FIELD_ELEM) -> "Pred":
        return Pred(PRED_LT, field, a)

    # pair rules (extractPattern)
    @staticmethod
    def value_even(skip_sentinels: bool = True) -> "Pred":
        return Pred(PRED_MASK_EQ, FIELD_VALUE, 1, 0, PRED_SKIP_SENTINELS if skip_sentinels else 0)

    @staticmethod
    def key_lt(a: int) -> "Pred":
        return Pred(PRED_LT, FIELD_KEY, a)

    @staticmethod
    def valid_key() -> "Pred":
        return Pred(PRED_VALID)

    @staticmethod
    def not_home() -> "Pred":
        return Pred(PRED_NOT_HOME)


class Hashmap:
    """Hashinator::Hashmap<K,V> (hashinator.h:59-62) over libhx."""

    def __init__(self, size_power: int = 5, key_bytes: int = 4, val_bytes: int | None = None, stream=None):
        self._h = lib()
        self._m = ctypes.c_void_p()
        self.key_bytes = key_bytes
        self.val_bytes = key_bytes if val_bytes is None else val_bytes
        _check(self._h.hx_map_create(ctypes.byref(self._m), key_bytes, self.val_bytes, size_power,
                                     _stream(stream)), "hx_map_create")

    def close(self) -> None:
        if self._m and self._m.value:
            _check(self._h.hx_map_destroy(self._m), "hx_map_destroy")
            self._m = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> int:
        return self._m.value

    # accelerated API -----------------------------------------------------
    def insert(self, keys, vals, target_lf: float = 0.5, stream=None, n: int | None = None) -> None:
        n = _numel(keys) if n is None else n
        _check(self._h.hx_insert(self._m, _ptr(keys), _ptr(vals), n, target_lf, _stream(stream)), "hx_insert")

    def insert_pairs(self, pairs, n: int | None = None, target_lf: float = 0.5, stream=None) -> None:
        n = _numel(pairs) // 2 if n is None else n
        _check(self._h.hx_insert_pairs(self._m, _ptr(pairs), n, target_lf, _stream(stream)), "hx_insert_pairs")

    def retrieve(self, keys, vals, stream=None, n: int | None = None) -> None:
        n = _numel(keys) if n is None else n
        _check(self._h.hx_retrieve(self._m, _ptr(keys), _ptr(vals), n, _stream(stream)), "hx_retrieve")

    def retrieve_pairs(self, pairs, n: int | None = None, stream=None) -> None:
        n = _numel(pairs) // 2 if n is None else n
        _check(self._h.hx_retrieve_pairs(self._m, _ptr(pairs), n, _stream(stream)), "hx_retrieve_pairs")

    def erase(self, keys, stream=None, n: int | None = None) -> None:
        n = _numel(keys) if n is None else n
        _check(self._h.hx_erase(self._m, _ptr(keys), n, _stream(stream)), "hx_erase")

    def clean_tombstones(self, stream=None) -> None:
        _check(self._h.hx_clean_tombstones(self._m, _stream(stream)), "hx_clean_tombstones")

    def extract_pattern(self, pred: Pred, out, capacity: int | None = None, stream=None, d_count=None) -> int:
        """extractPattern(elements, rule): returns the count (synchronises)
        unless d_count (a device address) is given, then returns -1."""
        cap = (_numel(out) // 2) if capacity is None else capacity
        cp = pred.c()
        if d_count is not None:
            _check(self._h.hx_extract_pattern(self._m, ctypes.byref(cp), _ptr(out), cap, _ptr(d_count), None,
                                              _stream(stream)), "hx_extract_pattern")
            return -1
        cnt = ctypes.c_uint64()
        st = self._h.hx_extract_pattern(self._m, ctypes.byref(cp), _ptr(out), cap, None, ctypes.byref(cnt),
                                        _stream(stream))
        if st not in (HX_OK, HX_ERR_CAPACITY):
            _check(st, "hx_extract_pattern")
        return cnt.value

    def extract_keys_by_pattern(self, pred: Pred, out, capacity: int | None = None, stream=None,
                                d_count=None) -> int:
        """extractKeysByPattern(keys, rule): the keys of the buckets where the
        rule holds, in bucket order; count as for extract_pattern."""
        cap = _numel(out) if capacity is None else capacity
        cp = pred.c()
        if d_count is not None:
            _check(self._h.hx_extract_keys(self._m, ctypes.byref(cp), _ptr(out), cap, _ptr(d_count), None,
                                           _stream(stream)), "hx_extract_keys")
            return -1
        cnt = ctypes.c_uint64()
        st = self._h.hx_extract_keys(self._m, ctypes.byref(cp), _ptr(out), cap, None, ctypes.byref(cnt),
                                     _stream(stream))
        if st not in (HX_OK, HX_ERR_CAPACITY):
            _check(st, "hx_extract_keys")
        return cnt.value

    def extract_all_keys(self, out, capacity: int | None = None, stream=None) -> int:
        """extractAllKeys(keys): every valid key, in bucket order."""
        return self.extract_keys_by_pattern(Pred.valid_key(), out, capacity, stream)

    def resize(self, new_size_power: int, stream=None) -> None:
        _check(self._h.hx_resize(self._m, new_size_power, _stream(stream)), "hx_resize")

    device_rehash = resize

    def resize_to_lf(self, target_lf: float = 0.5, stream=None) -> None:
        _check(self._h.hx_resize_to_lf(self._m, target_lf, _stream(stream)), "hx_resize_to_lf")

    def perform_cleanup_tasks(self, stream=None) -> None:
        _check(self._h.hx_perform_cleanup_tasks(self._m, _stream(stream)), "hx_perform_cleanup_tasks")

    def insert_index(self, keys, target_lf: float = 0.5, stream=None, n: int | None = None) -> None:
        """insertIndex(keys, len, targetLF): keys[i] gets the value i."""
        n = _numel(keys) if n is None else n
        _check(self._h.hx_insert_index(self._m, _ptr(keys), n, target_lf, _stream(stream)), "hx_insert_index")

    def clear(self, stream=None) -> None:
        _check(self._h.hx_clear(self._m, _stream(stream)), "hx_clear")

    def set_tuning(self, group_width: int = 0, keys_per_thread: int = 0, block_size: int = 0) -> None:
        _check(self._h.hx_map_set_tuning(self._m, group_width, keys_per_thread, block_size), "hx_map_set_tuning")

    def set_window_bytes(self, nbytes: int) -> None:
        _check(self._h.hx_map_set_window_bytes(self._m, nbytes), "hx_map_set_window_bytes")

    def set_insert_mode(self, blind_cas: bool) -> None:
        _check(self._h.hx_map_set_insert_mode(self._m, 1 if blind_cas else 0), "hx_map_set_insert_mode")

    # metadata (synchronous) ----------------------------------------------
    def info(self, stream=None) -> Info:
        inf = Info()
        _check(self._h.hx_get_info(self._m, ctypes.byref(inf), _stream(stream)), "hx_get_info")
        return inf

    def size(self) -> int:
        return self.info().fill

    def bucket_count(self) -> int:
        return self.info().bucket_count

    def tombstone_count(self) -> int:
        return self.info().tombstone_counter

    def load_factor(self) -> float:
        i = self.info()
        return i.fill / i.bucket_count

    def getSizePower(self) -> int:
        return self.info().size_power

    def peek_status(self, stream=None) -> int:
        v = ctypes.c_int32()
        _check(self._h.hx_peek_status(self._m, ctypes.byref(v), _stream(stream)), "hx_peek_status")
        return v.value

    def bucket_data(self) -> tuple[int, int]:
        p = ctypes.c_void_p()
        n = ctypes.c_uint64()
        _check(self._h.hx_bucket_data(self._m, ctypes.byref(p), ctypes.byref(n)), "hx_bucket_data")
        return p.value, n.value

    def get_emptybucket(self) -> int:
        return (1 << (8 * self.key_bytes)) - 1

    def get_tombstone(self) -> int:
        return (1 << (8 * self.key_bytes)) - 2


class tools:
    """split::tools (splitvector/split_tools.h)."""

    @staticmethod
    def scratch_bytes(op: int, n: int) -> int:
        b = ctypes.c_uint64()
        _check(lib().hx_scratch_bytes(op, n, ctypes.byref(b)), "hx_scratch_bytes")
        return b.value

    @staticmethod
    def split_prefix_scan(inp, out, n: int | None = None, scratch=None, scratch_bytes: int = 0, stream=None) -> None:
        n = _numel(inp) if n is None else n
        _check(lib().hx_exclusive_scan_u32(_ptr(inp), _ptr(out), n, _ptr(scratch), scratch_bytes, _stream(stream)),
               "hx_exclusive_scan_u32")

    @staticmethod
    def copy_if(inp, out, pred: Pred, elem_bytes: int = 4, n: int | None = None, capacity: int | None = None,
                scratch=None, scratch_bytes: int = 0, stream=None, d_count=None) -> int:
        if n is None:
            n = _numel(inp) * inp.element_size() // elem_bytes
        if capacity is None:
            capacity = _numel(out) * out.element_size() // elem_bytes
        cp = pred.c()
        if d_count is not None:
            _check(lib().hx_copy_if(_ptr(inp), _ptr(out), n, elem_bytes, ctypes.byref(cp), capacity, _ptr(d_count),
                                    None, _ptr(scratch), scratch_bytes, _stream(stream)), "hx_copy_if")
            return -1
        cnt = ctypes.c_uint64()
        st = lib().hx_copy_if(_ptr(inp), _ptr(out), n, elem_bytes, ctypes.byref(cp), capacity, None,
                              ctypes.byref(cnt), _ptr(scratch), scratch_bytes, _stream(stream))
        if st not in (HX_OK, HX_ERR_CAPACITY):
            _check(st, "hx_copy_if")
        return cnt.value


def _offsets(offs):
    if offs is None:
        return None, None
    import numpy as _np
    a = _np.ascontiguousarray(_np.asarray(offs, dtype=_np.uint64))
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))


class Batch:
    """A directory of many independent maps in one device arena (hx_batch)."""

    def __init__(self, size_powers, key_bytes: int = 4, stream=None):
        self._h = lib()
        import numpy as _np
        sp = _np.ascontiguousarray(_np.asarray(size_powers, dtype=_np.int32))
        self.n_maps = len(sp)
        self.size_powers = sp
        self.key_bytes = key_bytes
        self._b = ctypes.c_void_p()
        _check(self._h.hx_batch_create(ctypes.byref(self._b), len(sp), sp.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                       key_bytes, key_bytes, _stream(stream)), "hx_batch_create")

    def close(self) -> None:
        if self._b and self._b.value:
            _check(self._h.hx_batch_destroy(self._b), "hx_batch_destroy")
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def clear(self, stream=None) -> None:
        _check(self._h.hx_batch_clear(self._b, _stream(stream)), "hx_batch_clear")

    def map_info(self, i: int, stream=None) -> Info:
        inf = Info()
        _check(self._h.hx_batch_map_info(self._b, i, ctypes.byref(inf), _stream(stream)), "hx_batch_map_info")
        return inf

    def bucket_data(self, i: int) -> tuple[int, int]:
        p, n = ctypes.c_void_p(), ctypes.c_uint64()
        _check(self._h.hx_batch_bucket_data(self._b, i, ctypes.byref(p), ctypes.byref(n)), "hx_batch_bucket_data")
        return p.value, n.value

    def plan(self, ins_keys=None, ins_vals=None, ins_offsets=None, query_keys=None, query_out=None,
             query_offsets=None, erase_keys=None, erase_offsets=None, clean: bool = False, stream=None) -> "BatchPlan":
        return BatchPlan(self, ins_keys, ins_vals, ins_offsets, query_keys, query_out, query_offsets, erase_keys,
                         erase_offsets, clean, stream)


class BatchTrial(ctypes.Structure):
    """hx_batch_trial: one point of the autotuner's grid and its time."""
    _fields_ = [("group_width", ctypes.c_int32), ("block_size", ctypes.c_int32), ("tile_keys", ctypes.c_int32),
                ("ms", ctypes.c_float)]


# hx_batch_reset_fn: hx_status (*)(void* user, hx_stream stream)
BATCH_RESET_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p)


class BatchPlan:
    """One round of work over a Batch, run as one persistent launch."""

    def __init__(self, batch: Batch, ins_keys, ins_vals, ins_offsets, query_keys, query_out, query_offsets,
                 erase_keys, erase_offsets, clean, stream):
        self.batch = batch
        self._h = batch._h
        self._keep = (ins_keys, ins_vals, query_keys, query_out, erase_keys)
        io, iop = _offsets(ins_offsets)
        qo, qop = _offsets(query_offsets)
        eo, eop = _offsets(erase_offsets)
        w = _CBatchWork(_ptr(ins_keys), _ptr(ins_vals), iop, _ptr(query_keys), _ptr(query_out), qop,
                        _ptr(erase_keys), eop, 1 if clean else 0)
        self._p = ctypes.c_void_p()
        _check(self._h.hx_batch_plan_create(batch._b, ctypes.byref(w), ctypes.byref(self._p), _stream(stream)),
               "hx_batch_plan_create")
        self.tuning = {"group_width": 1, "block_size": 256, "tile_keys": 2048}

    def close(self) -> None:
        if self._p and self._p.value:
            _check(self._h.hx_batch_plan_destroy(self._p), "hx_batch_plan_destroy")
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tuning(self, group_width: int = 0, block_size: int = 0, tile_keys: int = 0, stream=None) -> None:
        _check(self._h.hx_batch_set_tuning(self._p, group_width, block_size, tile_keys, _stream(stream)),
               "hx_batch_set_tuning")
        for k, v in (("group_width", group_width), ("block_size", block_size), ("tile_keys", tile_keys)):
            if v:
                self.tuning[k] = v

    def run(self, stream=None) -> None:
        _check(self._h.hx_batch_run(self._p, _stream(stream)), "hx_batch_run")

    def run_graph(self, stream=None) -> None:
        _check(self._h.hx_batch_run_graph(self._p, _stream(stream)), "hx_batch_run_graph")

    def run_per_map(self, stream=None) -> None:
        _check(self._h.hx_batch_run_per_map(self._p, _stream(stream)), "hx_batch_run_per_map")

    def autotune(self, groups=None, blocks=None, tiles=None, reps: int = 2, reset=None, stream=None):
        """hx_batch_autotune: times the captured-graph replay over the grid (None: libhx's default grid)
        and leaves the plan on the fastest point. reset: None (the maps are cleared before every trial) or
        a callable(stream) that restores the state the round starts from. Returns (best, trials) with
        best = (group, block, tile, ms)."""
        def arr(v):
            if v is None:
                return None, 0
            a = (ctypes.c_int32 * len(v))(*v)
            return a, len(v)

        g, ng = arr(groups)
        b, nb = arr(blocks)
        t, nt = arr(tiles)
        n = (ng or 5) * (nb or 3) * (nt or 3)
        trials = (BatchTrial * n)()
        best = BatchTrial()
        cb = None
        if reset is not None:
            def _reset(user, strm):
                try:
                    reset(stream)
                    return HX_OK
                except Exception:  # noqa: BLE001
                    return HX_ERR_INVALID_ARG
            cb = BATCH_RESET_FN(_reset)
        _check(self._h.hx_batch_autotune(self._p, g, ng, b, nb, t, nt, reps,
                                         ctypes.cast(cb, ctypes.c_void_p) if cb else None, None, _stream(stream),
                                         ctypes.byref(trials), n, ctypes.byref(best)), "hx_batch_autotune")
        self.tuning = {"group_width": best.group_width, "block_size": best.block_size, "tile_keys": best.tile_keys}
        return ((best.group_width, best.block_size, best.tile_keys, best.ms),
                [(x.group_width, x.block_size, x.tile_keys, x.ms) for x in trials])

    def inject_stall(self, map_index: int, phase: int, enable: bool = True, stream=None) -> None:
        """Test hook: make the later phases of one map wait for a tile that never runs."""
        _check(self._h.hx_batch_inject_stall(self._p, map_index, phase, 1 if enable else 0, _stream(stream)),
               "hx_batch_inject_stall")

    def check(self, stream=None) -> int:
        e = ctypes.c_int32()
        st = self._h.hx_batch_check(self._p, ctypes.byref(e), _stream(stream))
        if st not in (HX_OK, HX_ERR_TIMEOUT, HX_ERR_CAPACITY):
            _check(st, "hx_batch_check")
        return e.value


class Server:
    """Serving loop over many resident maps (hx_server)."""

    def __init__(self, key_bytes: int = 8, memory_budget: int = 40 << 30, max_load_factor: float = 0.8,
                 max_maps: int = 4096, max_round_requests: int = 4096, max_round_keys: int = 1 << 24,
                 rounds_in_flight: int = 3):
        self._h = lib()
        self.key_bytes = key_bytes
        self._s = ctypes.c_void_p()
        _check(self._h.hx_server_create(ctypes.byref(self._s), key_bytes, memory_budget, max_load_factor, max_maps,
                                        max_round_requests, max_round_keys, rounds_in_flight), "hx_server_create")

    def close(self) -> None:
        if self._s and self._s.value:
            _check(self._h.hx_server_destroy(self._s), "hx_server_destroy")
            self._s = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_map(self, size_power: int) -> int:
        mid = ctypes.c_uint32()
        _check(self._h.hx_server_add_map(self._s, size_power, ctypes.byref(mid)), "hx_server_add_map")
        return mid.value

    def try_add_map(self, size_power: int):
        mid = ctypes.c_uint32()
        st = self._h.hx_server_add_map(self._s, size_power, ctypes.byref(mid))
        return mid.value if st == HX_OK else None

    @staticmethod
    def requests(reqs) -> "ctypes.Array":
        arr = (Request * len(reqs))()
        for i, r in enumerate(reqs):
            arr[i] = r if isinstance(r, Request) else Request(*r)
        return arr

    def submit(self, reqs) -> None:
        arr = reqs if isinstance(reqs, ctypes.Array) else self.requests(reqs)
        _check(self._h.hx_server_submit(self._s, arr, len(arr)), "hx_server_submit")

    def step(self) -> int:
        n = ctypes.c_uint32()
        _check(self._h.hx_server_step(self._s, ctypes.byref(n)), "hx_server_step")
        return n.value

    def poll(self, capacity: int = 65536) -> list:
        buf = (Completion * capacity)()
        n = ctypes.c_uint32()
        _check(self._h.hx_server_poll(self._s, buf, capacity, ctypes.byref(n)), "hx_server_poll")
        return [(buf[i].tag, buf[i].complete_ns, buf[i].status) for i in range(n.value)]

    def drain(self) -> None:
        _check(self._h.hx_server_drain(self._s), "hx_server_drain")

    def map_info(self, i: int) -> Info:
        inf = Info()
        _check(self._h.hx_server_map_info(self._s, i, ctypes.byref(inf)), "hx_server_map_info")
        return inf

    def bucket_data(self, i: int) -> tuple[int, int]:
        p, n = ctypes.c_void_p(), ctypes.c_uint64()
        _check(self._h.hx_server_bucket_data(self._s, i, ctypes.byref(p), ctypes.byref(n)), "hx_server_bucket_data")
        return p.value, n.value

    def memory(self) -> tuple[int, int]:
        u, b = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self._h.hx_server_memory(self._s, ctypes.byref(u), ctypes.byref(b)), "hx_server_memory")
        return u.value, b.value

    def stats(self) -> dict:
        st = ServerStats()
        _check(self._h.hx_server_get_stats(self._s, ctypes.byref(st)), "hx_server_get_stats")
        return {k: getattr(st, k) for k, _ in ServerStats._fields_ if k != "reserved"}

    def run_trace(self, reqs, arrival_ns):
        """Real-time replay; returns (complete_ns, status) numpy arrays."""
        import numpy as _np
        arr = reqs if isinstance(reqs, ctypes.Array) else self.requests(reqs)
        arrival = _np.ascontiguousarray(arrival_ns, dtype=_np.uint64)
        comp = _np.zeros(len(arr), _np.uint64)
        st = _np.zeros(len(arr), _np.int32)
        t0 = ctypes.c_uint64()
        _check(self._h.hx_server_run_trace(self._s, arr, arrival.ctypes.data, len(arr), comp.ctypes.data,
                                           st.ctypes.data, ctypes.byref(t0)), "hx_server_run_trace")
        return comp, st


def set_l2_fetch_granularity(nbytes: int) -> None:
    """cudaLimitMaxL2FetchGranularity for this process's context (32/64/128)."""
    _check(lib().hx_set_l2_fetch_granularity(nbytes), "hx_set_l2_fetch_granularity")


def diag_random_access(buf, nbytes: int, n_ops: int, mode: int = 0, stream=None) -> None:
    """Launch n_ops random 32-byte sector reads (mode 0) or 64-bit CAS
    (mode 1) over a device buffer: the random-access ceilings."""
    _check(lib().hx_diag_random_access(_ptr(buf), nbytes, n_ops, mode, _stream(stream)), "hx_diag_random_access")


def kernel_launch_count() -> int:
    return lib().hx_kernel_launch_count()
