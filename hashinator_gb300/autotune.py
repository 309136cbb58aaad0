"""Autotuner for the batched-maps launch.

Times the fused persistent launch of a BatchPlan over a grid of probe-group
widths (lanes per key), block shapes and work partitions (keys per tile) on
the live GPU with CUDA events, resetting the maps before every trial, and
leaves the plan on the fastest setting. The grid defaults to group widths
{1, 4, 8, 16, 32} x blocks {128, 256, 512} x tiles {512, 2048, 8192}.
"""
from __future__ import annotations

import itertools


def autotune_batch(plan, reset, groups=(1, 4, 8, 16, 32), blocks=(128, 256, 512), tiles=(512, 2048, 8192),
                   reps: int = 2, stream=None) -> dict:
    """Returns {"best": (group, block, tile), "ms": best time, "trials": [...]}.

    reset: a callable that restores the maps to the state the plan expects
    (for a full round of insert/query/erase/clean: an empty batch)."""
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    trials = []
    best = None
    for g, b, t in itertools.product(groups, blocks, tiles):
        plan.set_tuning(g, b, t, stream=s)
        times = []
        for r in range(reps + 1):
            reset()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            plan.run(stream=s)
            e1.record(s)
            e1.synchronize()
            if r:
                times.append(e0.elapsed_time(e1))
        ms = min(times)
        trials.append({"group": g, "block": b, "tile": t, "ms": round(ms, 4)})
        if best is None or ms < best[1]:
            best = ((g, b, t), ms)
    plan.set_tuning(*best[0], stream=s)
    reset()
    return {"best": best[0], "ms": round(best[1], 4), "trials": trials}
