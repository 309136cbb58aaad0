// hx_autotune.h — the search of the batched-maps autotuner, independent of
// how one trial is run and timed (plain C++, so that a host-only test can
// drive it with a fake clock).
//
// For every point of the grid (lanes per key x block size x keys per tile):
// apply it, then run reps + 1 trials, each after restoring the maps to the
// state the round starts from; the first trial of a point is a warm-up (it
// may capture and instantiate the CUDA graph), the point's time is the
// fastest of the others. The plan is left on the fastest point, with the
// maps restored once more.
#pragma once
#include <cstddef>
#include <limits>

#include "../../include/hx.h"

namespace hx {

struct TunePoint {
  int group, block, tile;
};

// Runner: hx_status set(const TunePoint&); hx_status reset(); hx_status timed_run(float* ms).
template <class Runner>
hx_status autotune_grid(Runner& r, const TunePoint* grid, size_t n, int reps, float* trial_ms, TunePoint* best,
                        float* best_ms) {
  if (!grid || n == 0 || reps < 1 || !best || !best_ms) return HX_ERR_INVALID_ARG;
  size_t bi = 0;
  float bm = std::numeric_limits<float>::infinity();
  hx_status st;
  for (size_t i = 0; i < n; ++i) {
    if ((st = r.set(grid[i])) != HX_OK) return st;
    float m = std::numeric_limits<float>::infinity();
    for (int rep = 0; rep <= reps; ++rep) {
      if ((st = r.reset()) != HX_OK) return st;
      float t = 0.f;
      if ((st = r.timed_run(&t)) != HX_OK) return st;
      if (rep > 0 && t < m) m = t;
    }
    if (trial_ms) trial_ms[i] = m;
    if (m < bm) {
      bm = m;
      bi = i;
    }
  }
  if ((st = r.set(grid[bi])) != HX_OK) return st;
  if ((st = r.reset()) != HX_OK) return st;
  *best = grid[bi];
  *best_ms = bm;
  return HX_OK;
}

}  // namespace hx
