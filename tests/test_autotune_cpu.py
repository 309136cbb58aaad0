"""Host logic of the batched-maps autotuner, without a GPU: a fake plan whose
run time depends on its tuning and a fake CUDA event clock. The tuner tries
every point of the grid, resets the maps before every trial, times `reps`
trials after one warm-up, and leaves the plan on the fastest setting."""
import pytest

from hashinator_gb300 import autotune


class FakeClock:
    now = 0.0


class FakeEvent:
    def __init__(self, enable_timing=False):
        self.t = None

    def record(self, stream=None):
        self.t = FakeClock.now

    def synchronize(self):
        pass

    def elapsed_time(self, other):
        return other.t - self.t


class FakePlan:
    def __init__(self, cost):
        self.cost = cost
        self.tuning = None
        self.history = []
        self.runs = 0

    def set_tuning(self, g, b, t, stream=None):
        self.tuning = (g, b, t)
        self.history.append(self.tuning)

    def run(self, stream=None):
        self.runs += 1
        # the first run of each setting is slow (warm-up), later ones cost the model's time
        FakeClock.now += self.cost(*self.tuning) + (5.0 if self.first else 0.0)
        self.first = False


@pytest.fixture
def fake_cuda(monkeypatch):
    torch = pytest.importorskip("torch")
    monkeypatch.setattr(torch.cuda, "Event", FakeEvent)
    return torch


def test_picks_the_fastest_setting_and_leaves_the_plan_on_it(fake_cuda):
    def cost(g, b, t):
        return 1.0 + abs(g - 8) * 0.1 + abs(b - 256) / 1000 + abs(t - 2048) / 10000

    plan = FakePlan(cost)
    resets = []

    class Hook:
        def __call__(self):
            resets.append(plan.tuning)
            plan.first = len(resets) == 1 or resets[-1] != resets[-2]

    res = autotune.autotune_batch(plan, Hook(), groups=(1, 4, 8, 16), blocks=(128, 256, 512),
                                  tiles=(512, 2048, 8192), reps=2, stream=object())
    assert res["best"] == (8, 256, 2048)
    assert plan.tuning == (8, 256, 2048)  # left on the winner
    assert len(res["trials"]) == 4 * 3 * 3
    assert plan.runs == 4 * 3 * 3 * 3  # warm-up + 2 timed runs per setting
    assert len(resets) == plan.runs + 1  # before every run, and once more at the end
    best = min(res["trials"], key=lambda r: r["ms"])
    assert (best["group"], best["block"], best["tile"]) == res["best"]
    assert res["ms"] == pytest.approx(cost(8, 256, 2048))  # warm-up excluded from the timing


def test_single_point_grid(fake_cuda):
    plan = FakePlan(lambda g, b, t: 2.5)

    def reset():
        plan.first = False

    res = autotune.autotune_batch(plan, reset, groups=(1,), blocks=(128,), tiles=(2048,), reps=3, stream=object())
    assert res["best"] == (1, 128, 2048) and res["ms"] == pytest.approx(2.5) and len(res["trials"]) == 1
