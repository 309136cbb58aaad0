// The search of libhx's batched-maps autotuner (hashinator_gb300/csrc/
// hx_autotune.h, behind hx_batch_autotune) driven on the host by a fake plan
// whose run time depends on its tuning and a fake clock: every point of the
// grid is tried, the maps are reset before every trial, each point gets one
// warm-up and `reps` timed runs, the warm-up is not counted, and the plan is
// left on the fastest point with the maps reset once more. Exit code 0 = pass.
#include <cmath>
#include <cstdio>
#include <vector>

#include "hx_autotune.h"

static int g_fail = 0;
#define EXPECT_TRUE(c)                                         \
  do {                                                         \
    if (!(c)) {                                                \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c); \
      ++g_fail;                                                \
    }                                                          \
  } while (0)

struct FakePlan {
  double (*cost)(int, int, int);
  hx::TunePoint tuning{0, 0, 0};
  std::vector<hx::TunePoint> history;
  int runs = 0, resets = 0;
  bool first = true;        // the next run is the first at this tuning (a slow warm-up)
  hx_status set(const hx::TunePoint& p) {
    tuning = p;
    history.push_back(p);
    first = true;
    return HX_OK;
  }
  hx_status reset() {
    ++resets;
    return HX_OK;
  }
  hx_status timed_run(float* ms) {
    ++runs;
    *ms = (float)(cost(tuning.group, tuning.block, tuning.tile) + (first ? 5.0 : 0.0));
    first = false;
    return HX_OK;
  }
};

static double bowl(int g, int b, int t) { return 1.0 + std::abs(g - 8) * 0.1 + std::abs(b - 256) / 1000.0 + std::abs(t - 2048) / 10000.0; }
static double flat(int, int, int) { return 2.5; }

int main() {
  std::vector<hx::TunePoint> grid;
  for (int g : {1, 4, 8, 16})
    for (int b : {128, 256, 512})
      for (int t : {512, 2048, 8192}) grid.push_back({g, b, t});
  {
    FakePlan p{bowl};
    std::vector<float> ms(grid.size());
    hx::TunePoint best{};
    float best_ms = 0;
    EXPECT_TRUE(hx::autotune_grid(p, grid.data(), grid.size(), 2, ms.data(), &best, &best_ms) == HX_OK);
    EXPECT_TRUE(best.group == 8 && best.block == 256 && best.tile == 2048);
    EXPECT_TRUE(p.tuning.group == 8 && p.tuning.block == 256 && p.tuning.tile == 2048);  // left on the winner
    EXPECT_TRUE(p.runs == (int)grid.size() * 3);       // warm-up + 2 timed runs per point
    EXPECT_TRUE(p.resets == p.runs + 1);               // before every run, and once more at the end
    EXPECT_TRUE(p.history.size() == grid.size() + 1);  // every point, then the winner again
    EXPECT_TRUE(std::fabs(best_ms - (float)bowl(8, 256, 2048)) < 1e-6f);  // warm-up excluded
    size_t arg = 0;
    for (size_t i = 0; i < ms.size(); ++i)
      if (ms[i] < ms[arg]) arg = i;
    EXPECT_TRUE(grid[arg].group == best.group && grid[arg].block == best.block && grid[arg].tile == best.tile);
  }
  {
    FakePlan p{flat};
    hx::TunePoint one{1, 128, 2048}, best{};
    float ms = 0, best_ms = 0;
    EXPECT_TRUE(hx::autotune_grid(p, &one, 1, 3, &ms, &best, &best_ms) == HX_OK);
    EXPECT_TRUE(best.group == 1 && best.block == 128 && best.tile == 2048 && std::fabs(best_ms - 2.5f) < 1e-6f);
    EXPECT_TRUE(p.runs == 4);
  }
  {  // arguments checked before anything runs
    FakePlan p{flat};
    hx::TunePoint best{};
    float best_ms = 0;
    EXPECT_TRUE(hx::autotune_grid(p, grid.data(), 0, 2, nullptr, &best, &best_ms) == HX_ERR_INVALID_ARG);
    EXPECT_TRUE(hx::autotune_grid(p, grid.data(), grid.size(), 0, nullptr, &best, &best_ms) == HX_ERR_INVALID_ARG);
    EXPECT_TRUE(p.runs == 0 && p.resets == 0);
  }
  if (g_fail) {
    std::printf("%d FAILED\n", g_fail);
    return 1;
  }
  std::printf("PASSED\n");
  return 0;
}
