"""Autotuner for the batched-maps launch: a thin caller of libhx's
hx_batch_autotune, which times the captured-graph replay of a plan over a
grid of probe-group widths (lanes per key), block sizes and keys per tile,
restoring the maps before every trial, and leaves the plan on the fastest
setting. C and C++ hosts call hx_batch_autotune directly.
"""
from __future__ import annotations


def autotune_batch(plan, reset=None, groups=(1, 4, 8, 16, 32), blocks=(128, 256, 512), tiles=(512, 2048, 8192),
                   reps: int = 2, stream=None) -> dict:
    """Returns {"best": (group, block, tile), "ms": best time, "trials": [...]}.

    reset: None (the batch's maps are cleared before every trial: a round that starts from empty maps) or a
    callable(stream) that restores the state the plan's round starts from."""
    best, trials = plan.autotune(groups, blocks, tiles, reps=reps, reset=reset, stream=stream)
    return {"best": best[:3], "ms": round(best[3], 4),
            "trials": [{"group": g, "block": b, "tile": t, "ms": round(ms, 4)} for g, b, t, ms in trials]}
