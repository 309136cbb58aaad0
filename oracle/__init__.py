"""TEST INFRASTRUCTURE ONLY — the parity oracle for libhx.

A serial CPU restatement of the Hashinator hot path (oracle/hx_oracle.c,
compiled into oracle/liboracle.so) with numpy bindings. Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline / reference legs use it,
always as the parity oracle or the timed CPU baseline, never as the product path.

Pinning: tests/test_oracle_golden.py checks this oracle against golden
fixtures produced by the reference's own CPU-only build
(oracle/ref_driver.cpp compiled by oracle/Makefile into oracle/_ref/).
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"


class OxPred(ctypes.Structure):
    _fields_ = [("op", ctypes.c_uint32), ("field", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("a", ctypes.c_uint64), ("b", ctypes.c_uint64)]


_h = None


def build() -> Path:
    src = HERE / "hx_oracle.c"
    if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["gcc", "-O2", "-std=c11", "-shared", "-fPIC", "-o", str(LIB_PATH), str(src)], check=True)
    return LIB_PATH


def lib():
    global _h
    if _h is None:
        build()
        h = ctypes.CDLL(str(LIB_PATH))
        vp, u64 = ctypes.c_void_p, ctypes.c_uint64
        h.ox_map_create.argtypes = [ctypes.c_int, ctypes.c_int]
        h.ox_map_create.restype = vp
        h.ox_map_destroy.argtypes = [vp]
        h.ox_insert.argtypes = [vp, vp, vp, u64, ctypes.c_float]
        h.ox_insert.restype = ctypes.c_int
        h.ox_retrieve.argtypes = [vp, vp, vp, u64]
        h.ox_erase.argtypes = [vp, vp, u64]
        h.ox_clean_tombstones.argtypes = [vp]
        h.ox_resize.argtypes = [vp, ctypes.c_int]
        h.ox_resize.restype = ctypes.c_int
        h.ox_extract.argtypes = [vp, ctypes.POINTER(OxPred), vp, u64]
        h.ox_extract.restype = u64
        h.ox_mapping.argtypes = [vp, vp, vp, u64]
        h.ox_mapping.restype = u64
        h.ox_info.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(u64), ctypes.POINTER(u64),
                              ctypes.POINTER(u64)]
        h.ox_buckets.argtypes = [vp]
        h.ox_buckets.restype = vp
        h.ox_copy_if.argtypes = [vp, vp, u64, ctypes.c_int, ctypes.POINTER(OxPred)]
        h.ox_copy_if.restype = u64
        h.ox_exclusive_scan_u32.argtypes = [vp, vp, u64]
        h.ox_fib_hash32.argtypes = [ctypes.c_uint32, ctypes.c_int]
        h.ox_fib_hash32.restype = ctypes.c_uint32
        h.ox_fib_hash64.argtypes = [ctypes.c_uint64, ctypes.c_int]
        h.ox_fib_hash64.restype = ctypes.c_uint64
        _h = h
    return _h


def _p(a: np.ndarray) -> int:
    assert a.flags.c_contiguous
    return a.ctypes.data


def pred(op: int, field: int = 0, a: int = 0, b: int = 0, flags: int = 0) -> OxPred:
    return OxPred(op, field, flags, 0, a, b)


class OracleMap:
    """Serial restatement of Hashmap<K,V> (K = V = uint32 or uint64)."""

    def __init__(self, size_power: int, key_bytes: int = 4):
        self.kb = key_bytes
        self.dt = np.uint32 if key_bytes == 4 else np.uint64
        self._m = lib().ox_map_create(key_bytes, size_power)
        if not self._m:
            raise ValueError("bad oracle map arguments")

    def __del__(self):
        if getattr(self, "_m", None):
            lib().ox_map_destroy(self._m)
            self._m = None

    def _arr(self, a) -> np.ndarray:
        a = np.ascontiguousarray(a)
        if a.dtype.itemsize != self.kb:
            raise ValueError("key/value width mismatch")
        return a.view(self.dt)

    def insert(self, keys, vals, target_lf: float = 0.5) -> int:
        k, v = self._arr(keys), self._arr(vals)
        return lib().ox_insert(self._m, _p(k), _p(v), len(k), target_lf)

    def retrieve(self, keys, out: np.ndarray) -> None:
        k = self._arr(keys)
        assert out.flags.c_contiguous and out.dtype.itemsize == self.kb
        lib().ox_retrieve(self._m, _p(k), _p(out), len(k))

    def erase(self, keys) -> None:
        k = self._arr(keys)
        lib().ox_erase(self._m, _p(k), len(k))

    def clean_tombstones(self) -> None:
        lib().ox_clean_tombstones(self._m)

    def resize(self, sp: int) -> None:
        assert lib().ox_resize(self._m, sp) == 0

    def info(self) -> dict:
        sp, f, t, mp = ctypes.c_int(), ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        lib().ox_info(self._m, ctypes.byref(sp), ctypes.byref(f), ctypes.byref(t), ctypes.byref(mp))
        return {"size_power": sp.value, "fill": f.value, "tombstones": t.value, "max_probe": mp.value}

    def mapping(self) -> tuple[np.ndarray, np.ndarray]:
        """Valid (keys, values) sorted by key."""
        n = self.info()["fill"]
        k = np.zeros(n, self.dt)
        v = np.zeros(n, self.dt)
        c = lib().ox_mapping(self._m, _p(k), _p(v), n)
        assert c == n, (c, n)
        o = np.argsort(k, kind="stable")
        return k[o], v[o]

    def extract(self, p: OxPred, capacity: int | None = None) -> tuple[int, np.ndarray]:
        if capacity is None:
            capacity = 1 << self.info()["size_power"]
        out = np.zeros(2 * capacity, self.dt)
        c = lib().ox_extract(self._m, ctypes.byref(p), _p(out), capacity)
        return c, out[: 2 * min(c, capacity)].reshape(-1, 2)

    def buckets(self) -> np.ndarray:
        n = 1 << self.info()["size_power"]
        addr = lib().ox_buckets(self._m)
        buf = (ctypes.c_char * (n * 2 * self.kb)).from_address(addr)
        return np.frombuffer(buf, dtype=self.dt).reshape(n, 2).copy()


def copy_if(arr: np.ndarray, elem_bytes: int, p: OxPred) -> np.ndarray:
    arr = np.ascontiguousarray(arr)
    n = arr.nbytes // elem_bytes
    out = np.empty_like(arr)
    c = lib().ox_copy_if(_p(arr), _p(out), n, elem_bytes, ctypes.byref(p))
    words = elem_bytes // arr.dtype.itemsize
    return out[: c * words]


def exclusive_scan_u32(arr: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(arr, dtype=np.uint32)
    out = np.empty_like(a)
    lib().ox_exclusive_scan_u32(_p(a), _p(out), len(a))
    return out


def fib_hash(key: int, sp: int, key_bytes: int) -> int:
    return lib().ox_fib_hash32(key, sp) if key_bytes == 4 else lib().ox_fib_hash64(key, sp)
