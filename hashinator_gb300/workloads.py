"""Seeded synthetic inputs for the Hashinator workloads.

Keys are made distinct by construction: key_i = mix(i + offset), where mix
is a bijection of the key width (the MurmurHash3 32-bit finaliser, or the
SplitMix64 finaliser, each salted by a seed-derived xor constant). Indices
[0, n) give the inserted keys and [n, 2n) keys guaranteed absent. The
EMPTY (all ones) and TOMBSTONE (all ones - 1) sentinels are removed.
Values are uniform from numpy's PCG64 with the same seed. Everything is a
pure function of (n, width, seed), so the oracle and libhx see identical
inputs.
"""
from __future__ import annotations

import numpy as np

M32 = np.uint32(0xFFFFFFFF)


def fmix32(x: np.ndarray) -> np.ndarray:
    x = x.astype(np.uint32, copy=True)
    x ^= x >> np.uint32(16)
    x *= np.uint32(0x85EBCA6B)
    x ^= x >> np.uint32(13)
    x *= np.uint32(0xC2B2AE35)
    x ^= x >> np.uint32(16)
    return x


def fmix64(x: np.ndarray) -> np.ndarray:
    z = x.astype(np.uint64, copy=True)
    z ^= z >> np.uint64(30)
    z *= np.uint64(0xBF58476D1CE4E5B9)
    z ^= z >> np.uint64(27)
    z *= np.uint64(0x94D049BB133111EB)
    z ^= z >> np.uint64(31)
    return z


def _salt(seed: int, width: int) -> int:
    s = np.array([seed * 0x9E3779B97F4A7C15 & 0xFFFFFFFFFFFFFFFF], np.uint64)
    v = int(fmix64(s)[0])
    return v & 0xFFFFFFFF if width == 4 else v


def keys_at(idx: np.ndarray, width: int, seed: int) -> np.ndarray:
    """Bijective key stream: distinct idx -> distinct keys."""
    if width == 4:
        return fmix32(idx.astype(np.uint32) ^ np.uint32(_salt(seed, 4)))
    return fmix64(idx.astype(np.uint64) ^ np.uint64(_salt(seed, 8)))


def distinct_keys(n: int, width: int, seed: int, offset: int = 0) -> np.ndarray:
    """n distinct keys, none equal to EMPTY or TOMBSTONE, from stream
    positions [offset, ...)."""
    empty = (1 << (8 * width)) - 1
    extra = 8
    while True:
        idx = np.arange(offset, offset + n + extra, dtype=np.uint64)
        k = keys_at(idx, width, seed)
        ok = (k != k.dtype.type(empty)) & (k != k.dtype.type(empty - 1))
        k = k[ok]
        if len(k) >= n:
            return np.ascontiguousarray(k[:n])
        extra *= 2


def values(n: int, width: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed + 0x5EED)
    dt = np.uint32 if width == 4 else np.uint64
    return rng.integers(0, np.iinfo(dt).max, size=n, dtype=dt, endpoint=True)


def map_workload(n: int, width: int, seed: int, hit_frac: float = 0.5, n_queries: int | None = None,
                 erase_frac: float = 0.25):
    """Keys/values to insert, a shuffled query set with hit_frac present
    keys, and an erase set (a random erase_frac of the inserted keys)."""
    keys = distinct_keys(n, width, seed)
    vals = values(n, width, seed)
    nq = n if n_queries is None else n_queries
    n_hit = int(round(nq * hit_frac))
    rng = np.random.default_rng(seed + 1)
    hits = keys[rng.choice(n, size=min(n_hit, n), replace=n_hit > n)] if n_hit else keys[:0]
    # absent keys come from a disjoint stretch of the same bijective stream
    misses = distinct_keys(nq - len(hits), width, seed, offset=n + 64)
    q = np.concatenate([hits, misses])
    rng.shuffle(q)
    n_erase = int(round(n * erase_frac))
    erase = keys[rng.permutation(n)[:n_erase]]
    return keys, vals, np.ascontiguousarray(q), np.ascontiguousarray(erase)


def velocity_shell_keys(n: int, centre, r_min: float, r_max: float, rng, grid: int = 200) -> np.ndarray:
    """n distinct velocity-block IDs id = x + grid*(y + grid*z) on a grid^3
    mesh, drawn from the shell r_min <= |p - centre| <= r_max."""
    c = np.asarray(centre, dtype=np.float64)
    lo = np.maximum(np.floor(c - r_max), 0).astype(np.int64)
    hi = np.minimum(np.ceil(c + r_max), grid - 1).astype(np.int64)
    out = np.empty(0, np.uint32)
    need = n
    while need > 0:
        m = max(2 * need, 256)
        p = rng.integers(lo, hi + 1, size=(m, 3))
        d = np.sqrt(((p - c) ** 2).sum(axis=1))
        p = p[(d >= r_min) & (d <= r_max)]
        ids = (p[:, 0] + grid * (p[:, 1] + grid * p[:, 2])).astype(np.uint32)
        out = np.unique(np.concatenate([out, ids]))
        need = n - len(out)
    rng.shuffle(out)
    return np.ascontiguousarray(out[:n])
