"""Random map-operation sequences for the fuzz tests, with a plain dict model
kept in step: insert batches (fresh keys and upserts of present ones, keys
plus tombstones held to 85% of the table, since insert never reuses a
tombstone), query batches, erase batches with repeated keys (each present key
counts once), clean_tombstones and resize (same or one size power up)."""
import numpy as np

from hashinator_gb300 import workloads


class Sequence:
    def __init__(self, width: int, seed: int, steps: int = 60):
        self.rng = np.random.default_rng(1000 * width + seed)
        self.width = width
        self.dt = np.uint32 if width == 4 else np.uint64
        self.sp0 = self.sp = int(self.rng.integers(4, 9))
        self.universe = workloads.distinct_keys(1 << self.sp0, width, 500 + seed)  # never more keys than buckets
        self.steps = steps
        self.model: dict[int, int] = {}
        self.tomb = 0
        self.fill = self.dt(np.iinfo(self.dt).max - 3)  # query-output pre-fill

    def expected_mapping(self):
        ks = np.array(sorted(self.model), dtype=self.dt)
        return ks, np.array([self.model[int(x)] for x in ks], dtype=self.dt)

    def ops(self):
        """Yields ("insert", keys, vals), ("query", keys, want), ("erase", keys), ("clean",) or
        ("resize", size_power); the model already holds the state after the yielded op."""
        rng, dt = self.rng, self.dt
        for _ in range(self.steps):
            op = rng.choice(["insert", "query", "erase", "clean", "resize"], p=[0.35, 0.3, 0.2, 0.1, 0.05])
            if op == "insert":
                room = int(0.85 * (1 << self.sp)) - len(self.model) - self.tomb
                present = np.array(sorted(self.model), dtype=dt)
                pool = np.setdiff1d(self.universe, present)
                n_fresh = int(rng.integers(0, max(0, min(room, len(pool))) + 1))
                n_up = int(rng.integers(0, len(present) + 1)) if len(present) else 0
                keys = np.concatenate([rng.choice(pool, n_fresh, replace=False) if n_fresh else pool[:0],
                                       rng.choice(present, n_up, replace=False) if n_up else present[:0]]).astype(dt)
                rng.shuffle(keys)
                vals = rng.integers(0, np.iinfo(dt).max, size=len(keys), dtype=dt, endpoint=True)
                for k, v in zip(keys.tolist(), vals.tolist()):
                    self.model[k] = v
                yield ("insert", keys, vals)
            elif op == "query":
                q = rng.choice(self.universe, int(rng.integers(1, 64)), replace=True).astype(dt)
                want = np.array([self.model.get(int(k), int(self.fill)) for k in q], dtype=dt)
                yield ("query", q, want)
            elif op == "erase":
                e = rng.choice(self.universe, int(rng.integers(1, 32)), replace=True).astype(dt)  # repeats on purpose
                for k in set(e.tolist()):
                    if k in self.model:
                        del self.model[k]
                        self.tomb += 1
                yield ("erase", e)
            elif op == "clean":
                self.tomb = 0
                yield ("clean",)
            else:
                self.sp = int(np.clip(self.sp + rng.integers(0, 2), self.sp0, 12))
                self.tomb = 0
                yield ("resize", self.sp)
