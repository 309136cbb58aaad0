"""CPU checks of host-side arithmetic the kernels rely on, computed exactly
with Python integers: the direct-remainder method used by the compaction's
`x % d < s` predicate (hx_scan.cuh fastmod_magic / fastmod_u32: with
M = floor((2^64 - 1) / d) + 1 mod 2^64, x mod d is the high 64 bits of
((M * x) mod 2^64) * d, for 32-bit x and 1 <= d < 2^32), and the build
flags (sm_103a only, with line info)."""
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


def test_build_targets_sm103a_with_line_info():
    from hashinator_gb300 import build
    flags = build.NVCC_FLAGS
    i = flags.index("-gencode")
    assert flags[i + 1] == "arch=compute_103a,code=sm_103a"
    assert flags.count("-gencode") == 1 and "-lineinfo" in flags
    assert not any("sm_90" in f or "sm_100" in f for f in flags)
