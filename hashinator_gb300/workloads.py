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


_SHELL_CACHE: dict = {}


def shell_offsets(r_min: float = 30.0, r_max: float = 60.0) -> np.ndarray:
    """All integer offsets d with r_min <= |d| <= r_max (int16, shape (M, 3))."""
    key = (r_min, r_max)
    if key not in _SHELL_CACHE:
        r = int(np.ceil(r_max))
        ax = np.arange(-r, r + 1, dtype=np.int32)
        x, y, z = np.meshgrid(ax, ax, ax, indexing="ij")
        d2 = x * x + y * y + z * z
        sel = (d2 >= r_min * r_min) & (d2 <= r_max * r_max)
        _SHELL_CACHE[key] = np.stack([x[sel], y[sel], z[sel]], axis=1).astype(np.int16)
    return _SHELL_CACHE[key]


def _coprime(rng, mod: np.ndarray) -> np.ndarray:
    """A random multiplier coprime to each modulus (a bijection j -> a*j mod m)."""
    import math
    out = np.empty(len(mod), np.int64)
    for i, m in enumerate(mod.tolist()):
        m = max(int(m), 1)
        while True:
            a = int(rng.integers(1, max(m, 2)))
            if math.gcd(a, m) == 1:
                out[i] = a
                break
    return out


def _segments(sizes: np.ndarray):
    """(segment id, index within segment) of every element of a concatenation."""
    starts = np.zeros(len(sizes), np.int64)
    starts[1:] = np.cumsum(sizes)[:-1]
    seg = np.repeat(np.arange(len(sizes)), sizes)
    j = np.arange(int(sizes.sum()), dtype=np.int64) - starts[seg]
    return seg, j, starts


def batched_workload(n_maps: int, seed: int, log_lo: float = 6.0, log_hi: float = 16.0, hit_frac: float = 0.7,
                     erase_frac: float = 0.1, grid: int = 200, target_lf: float = 0.5):
    """Many per-cell velocity-block maps: map i gets n_i = round(2^U), U ~ U[log_lo, log_hi], distinct
    velocity-block IDs id = x + grid*(y + grid*z) from the 30-60 cell shell around a random centre in
    [60, 139]^3 (so the shell stays inside the grid), values uniform; size power ceil(log2(n_i / target_lf));
    n_i queries with hit_frac present keys and the rest absent keys from the same shell, in a shuffled
    order; a random erase_frac of the keys erased. Distinct draws use random affine permutations
    j -> (a*j + b) mod M with gcd(a, M) = 1. Returns flat arrays and host offsets."""
    rng = np.random.default_rng(seed)
    shell = shell_offsets()
    m = len(shell)
    n = np.rint(2.0 ** rng.uniform(log_lo, log_hi, size=n_maps)).astype(np.int64)
    sp = np.ceil(np.log2(n / target_lf)).astype(np.int32)
    n_hit = np.rint(n * hit_frac).astype(np.int64)
    n_miss = n - n_hit
    n_er = np.rint(n * erase_frac).astype(np.int64)
    centres = rng.integers(60, 140, size=(n_maps, 3))
    # keys and misses: distinct shell cells per map
    need = n + n_miss
    a = _coprime(rng, np.full(n_maps, m))
    b = rng.integers(0, m, size=n_maps)
    seg, j, _ = _segments(need)
    cell = (a[seg] * j + b[seg]) % m
    pos = shell[cell].astype(np.int64) + centres[seg]
    ids = (pos[:, 0] + grid * (pos[:, 1] + grid * pos[:, 2])).astype(np.uint32)
    is_key = j < n[seg]
    keys = np.ascontiguousarray(ids[is_key])
    misses = ids[~is_key]
    vals = rng.integers(0, 2**32, size=len(keys), dtype=np.uint64).astype(np.uint32)
    _, _, kstart = _segments(n)
    _, _, mstart = _segments(n_miss)
    # queries: n_hit distinct present keys + the misses, shuffled within the map
    c = _coprime(rng, n)
    d = rng.integers(0, np.maximum(n, 1))
    hseg, hj, _ = _segments(n_hit)
    hits = keys[kstart[hseg] + (c[hseg] * hj + d[hseg]) % n[hseg]]
    nq = n_hit + n_miss
    qseg, qj, qstart = _segments(nq)
    vals_q = np.empty(len(qj), np.uint32)
    hit_pos = qj < n_hit[qseg]
    vals_q[hit_pos] = hits
    vals_q[~hit_pos] = misses
    e_mul = _coprime(rng, nq)
    f_add = rng.integers(0, np.maximum(nq, 1))
    queries = np.empty_like(vals_q)
    queries[qstart[qseg] + (e_mul[qseg] * qj + f_add[qseg]) % nq[qseg]] = vals_q
    # erase: a distinct erase_frac of each map's keys
    g = _coprime(rng, n)
    h = rng.integers(0, np.maximum(n, 1))
    eseg, ej, _ = _segments(n_er)
    erase = np.ascontiguousarray(keys[kstart[eseg] + (g[eseg] * ej + h[eseg]) % n[eseg]])

    def offs(sizes):
        o = np.zeros(n_maps + 1, np.uint64)
        o[1:] = np.cumsum(sizes)
        return o

    return {"size_powers": sp, "n": n, "keys": keys, "vals": vals, "ins_offsets": offs(n), "queries": queries,
            "query_offsets": offs(nq), "erase": erase, "erase_offsets": offs(n_er)}


def serving_trace(n_maps: int, n_requests: int, seed: int, init_log=(8.0, 20.0), size_log=(0.0, 16.0),
                  mix=(0.2, 0.7, 0.1), present: float = 0.8, rate_req_s: float = 1e6, width: int = 8,
                  init_lf: float = 0.5):
    """Serving workload: n_maps maps with initial key counts 2^U, U ~ U[init_log], tables sized for
    init_lf; then n_requests requests with Poisson arrivals at rate_req_s, each on a uniform random map,
    2^U keys (U ~ U[size_log], at least 1), op insert/query/erase with probabilities `mix`. Inserts bring
    fresh keys; queries draw `present` of their keys from keys inserted so far and the rest fresh
    (absent); erases draw from keys inserted so far. Map i's keys are positions [i*2^40, ...) of one
    bijective key stream, so with 8-byte keys maps never share keys; with 4-byte keys the positions wrap
    at 2^32 and maps may share keys (each map is a separate table, so that changes no result). The keys
    inserted into one map are distinct. Returns a dict of flat host arrays."""
    rng = np.random.default_rng(seed)
    n0 = np.rint(2.0 ** rng.uniform(init_log[0], init_log[1], size=n_maps)).astype(np.int64)
    sp = np.maximum(np.ceil(np.log2(n0 / init_lf)), 2).astype(np.int32)
    base = np.arange(n_maps, dtype=np.uint64) << np.uint64(40)
    fresh = n0.copy()  # next unused stream position per map
    req_map = rng.integers(0, n_maps, size=n_requests)
    req_op = rng.choice(3, size=n_requests, p=list(mix))
    req_n = np.maximum(np.rint(2.0 ** rng.uniform(size_log[0], size_log[1], size=n_requests)), 1).astype(np.int64)
    pos_parts = []
    for i in range(n_requests):
        m, op, k = int(req_map[i]), int(req_op[i]), int(req_n[i])
        if op == 0:
            pos = np.arange(fresh[m], fresh[m] + k, dtype=np.int64)
            fresh[m] += k
        elif op == 1:
            n_p = int(rng.binomial(k, present))
            pos = np.concatenate([rng.integers(0, fresh[m], size=n_p),
                                  np.arange(fresh[m] + (1 << 30), fresh[m] + (1 << 30) + (k - n_p), dtype=np.int64)])
            rng.shuffle(pos)
        else:
            pos = rng.integers(0, fresh[m], size=k)
        pos_parts.append(pos.astype(np.uint64) + base[m])
    init_pos = np.concatenate([np.arange(n, dtype=np.uint64) + base[m] for m, n in enumerate(n0)])
    init_off = np.zeros(n_maps + 1, np.int64)
    init_off[1:] = np.cumsum(n0)
    req_off = np.zeros(n_requests + 1, np.int64)
    req_off[1:] = np.cumsum(req_n)
    req_pos = np.concatenate(pos_parts) if pos_parts else np.zeros(0, np.uint64)
    gaps = rng.exponential(1e9 / rate_req_s, size=n_requests)
    arrival = np.cumsum(gaps).astype(np.uint64)
    dt = np.uint32 if width == 4 else np.uint64

    def keys_of(pos):
        return keys_at(pos, width, seed).astype(dt) if len(pos) else np.zeros(0, dt)

    return {"size_powers": sp, "n0": n0, "init_keys": keys_of(init_pos),
            "init_vals": values(len(init_pos), width, seed + 11), "init_offsets": init_off,
            "req_map": req_map.astype(np.uint32), "req_op": req_op.astype(np.uint32), "req_n": req_n,
            "req_offsets": req_off, "req_keys": keys_of(req_pos), "req_vals": values(len(req_pos), width, seed + 12),
            "arrival_ns": arrival}


def affine_sample(n: int, k: int, rng) -> np.ndarray:
    """k distinct indices in [0, n) (k <= n) from a random affine permutation, O(k)."""
    import math
    if k == 0 or n == 0:
        return np.zeros(0, np.int64)
    while True:
        a = int(rng.integers(1, max(n, 2)))
        if math.gcd(a, n) == 1:
            break
    b = int(rng.integers(0, n))
    j = np.arange(k, dtype=np.int64)
    return (a * j + b) % n


def query_expectation(keys: np.ndarray, vals: np.ndarray, q: np.ndarray, fill: int):
    """Exact retrieve output for a map holding the distinct keys `keys` with
    `vals`: the value of each query key that is present, `fill` (the output's
    pre-fill, which a miss leaves in place) for the others. Returns (expected
    output, found mask)."""
    out = np.full(len(q), fill, keys.dtype)
    if len(keys) == 0 or len(q) == 0:
        return out, np.zeros(len(q), bool)
    order = np.argsort(keys, kind="stable")
    sk = keys[order]
    pos = np.searchsorted(sk, q)
    pos[pos == len(sk)] = 0
    found = sk[pos] == q
    out[found] = vals[order[pos[found]]]
    return out, found


def large_map_workload(n: int, width: int, seed: int, hit_frac: float = 0.5, erase_frac: float = 0.3):
    """map_workload for very large n without O(n log n) sampling: hits and the
    erase set are affine samples of the inserted keys, the query order an
    affine shuffle."""
    rng = np.random.default_rng(seed + 1)
    keys = distinct_keys(n, width, seed)
    vals = values(n, width, seed)
    n_hit = int(round(n * hit_frac))
    hits = keys[affine_sample(n, n_hit, rng)]
    misses = distinct_keys(n - n_hit, width, seed, offset=n + 64)
    q = np.empty(n, keys.dtype)
    pos = affine_sample(n, n, rng)
    q[pos[:n_hit]] = hits
    q[pos[n_hit:]] = misses
    erase = keys[affine_sample(n, int(round(n * erase_frac)), rng)]
    return keys, vals, q, erase
