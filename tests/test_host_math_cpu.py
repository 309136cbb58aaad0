"""CPU checks of host-side arithmetic the kernels rely on, computed exactly
with Python integers: the direct-remainder method used by the compaction's
`x % d < s` predicate (hx_scan.cuh fastmod_magic / fastmod_u32: with
M = floor((2^64 - 1) / d) + 1 mod 2^64, x mod d is the high 64 bits of
((M * x) mod 2^64) * d, for 32-bit x and 1 <= d < 2^32), the threshold
form of `x % d < s` (hx_scan.cuh PK_MOD_LT_THRESH: for 2 <= d <= 2^31 and
0 < s < d, (x mod d) < s exactly when the high 32 bits of (M * x) mod 2^64
are below the high 32 bits of s * M, the left side computed as
umulhi(M_lo, x) + M_hi * x mod 2^32, as the kernel does), and the build flags
(sm_103a only, with line info)."""
import random

import pytest

M64 = (1 << 64) - 1


def fastmod(x: int, d: int) -> int:
    magic = (M64 // d + 1) & M64
    return (((magic * x) & M64) * d) >> 64


DIVISORS = [1, 2, 3, 5, 7, 10, 31, 32, 100, 641, 1000, 65535, 65536, 65537, 1 << 20, (1 << 31) - 1, 1 << 31,
            (1 << 31) + 1, (1 << 32) - 3, (1 << 32) - 2, (1 << 32) - 1]


@pytest.mark.parametrize("d", DIVISORS)
def test_direct_remainder_matches_modulo(d):
    rng = random.Random(d)
    xs = [0, 1, d - 1, d, d + 1, (1 << 32) - 1, (1 << 32) - 2, (1 << 31), (1 << 31) - 1]
    xs += [rng.randrange(1 << 32) for _ in range(2000)]
    for x in xs:
        if x < (1 << 32):
            assert fastmod(x, d) == x % d, (x, d)


def test_direct_remainder_random_divisors():
    rng = random.Random(7)
    for _ in range(300):
        d = rng.randrange(1, 1 << 32)
        for _ in range(50):
            x = rng.randrange(1 << 32)
            assert fastmod(x, d) == x % d, (x, d)


def thresh_ok(d: int, s: int) -> bool:  # mod_lt_thresh_ok in hx_scan.cuh
    return 2 <= d <= (1 << 31) and 0 < s < d


def mod_lt_by_threshold(x: int, d: int, s: int) -> bool:
    magic = (M64 // d + 1) & M64
    t = s * magic
    assert t <= M64  # s * M fits 64 bits
    m_lo, m_hi = magic & 0xFFFFFFFF, magic >> 32
    hi = (((m_lo * x) >> 32) + m_hi * x) & 0xFFFFFFFF  # umulhi(M_lo, x) + M_hi * x, in 32 bits
    assert hi == ((magic * x) & M64) >> 32
    return hi < (t >> 32)


@pytest.mark.parametrize("d", [d for d in DIVISORS if 2 <= d <= (1 << 31)])
def test_threshold_form_matches_modulo(d):
    rng = random.Random(d + 1)
    ss = sorted({1, 2, d // 2, d - 1} | {rng.randrange(1, d) for _ in range(5)})
    xs = [0, 1, d - 1, d, d + 1, 2 * d - 1, (1 << 32) - 1, (1 << 32) - 2, (1 << 31), (1 << 31) - 1]
    xs += [rng.randrange(1 << 32) for _ in range(1500)]
    xs += [k * d + r for k in (0, 1, rng.randrange(1, (1 << 32) // d)) for r in (0, 1, d - 1) if k * d + r < (1 << 32)]
    for s in ss:
        if not thresh_ok(d, s):
            continue
        for x in xs:
            if x < (1 << 32):
                assert mod_lt_by_threshold(x, d, s) == (x % d < s), (x, d, s)


def test_threshold_form_random_divisors_and_its_limit():
    rng = random.Random(11)
    for _ in range(300):
        d = rng.randrange(2, (1 << 31) + 1)
        s = rng.randrange(1, d)
        for _ in range(40):
            x = rng.randrange(1 << 32)
            assert mod_lt_by_threshold(x, d, s) == (x % d < s), (x, d, s)
    # the argument that the form is exact (q * e < 2^32 < M and no wrap of r*M + q*e) needs d <= 2^31: larger
    # divisors, and s = 0 or s >= d, use the direct remainder instead
    assert not thresh_ok((1 << 31) + 1, 5) and not thresh_ok(100, 0) and not thresh_ok(100, 100)


def test_build_targets_sm103a_with_line_info():
    from hashinator_gb300 import build
    flags = build.NVCC_FLAGS
    i = flags.index("-gencode")
    assert flags[i + 1] == "arch=compute_103a,code=sm_103a"
    assert flags.count("-gencode") == 1 and "-lineinfo" in flags
    assert not any("sm_90" in f or "sm_100" in f for f in flags)
