"""The autotuners' host logic on CPU: a stand-in kernel and batch whose calls advance a fake clock by
a cost that depends on the tuning state. Each tuner must set only values the C-ABI accepts
(include/dfpt.h's tuning keys) and leave the cheapest candidate set."""
import itertools
import types

import pytest

from dfpt import autotune

# Values dfpt_set_tuning / dfpt_batch_set_tuning accept.
VALID = {
    "trace_config": set(range(18)),
    "primitive_culling": {0, 1, 2},
    "l2_persist": {0, 1},
    "wide_samples": set(range(1, 65)),
    "ray_sort": {0, 1},
    "shadow_defer": {0, 1},
    "tail_bounce": set(range(-1, 33)),
    "tail_blocks": {2, 3, 4},
    "pass_shadow_sort": {0, 1},
    "pass_ray_sort": {0, 3, 6, 9, 12, 15},
    "wave_capacity": None,  # any value >= 1024
}


class Clock:
    def __init__(self):
        self.t = 0.0

    def perf_counter(self):
        return self.t


class FakeTunable:
    """Records set_tuning calls, rejects what the C-ABI rejects, charges cost(state) per unit."""

    def __init__(self, clock, cost, defaults):
        self.clock = clock
        self.cost = cost
        self.state = dict(defaults)
        self.sets = []

    def set_tuning(self, key, value):
        if key not in VALID:
            raise KeyError(key)
        allowed = VALID[key]
        if allowed is None:
            if value < 1024:
                raise ValueError((key, value))
        elif value not in allowed:
            raise ValueError((key, value))
        self.sets.append((key, value))
        self.state[key] = value

    def get_tuning(self, key):
        if key == "trace_configs":
            return 18
        return self.state[key]

    def synchronize(self):
        pass


class FakeKernel(FakeTunable):
    def execute(self, passes):
        self.clock.t += passes * self.cost(self.state)


class FakeBatch(FakeTunable):
    total_samples = 1 << 28

    def clear(self):
        pass

    def render_range(self, first, count):
        self.clock.t += count * self.cost(self.state)


@pytest.fixture
def clock(monkeypatch):
    c = Clock()
    monkeypatch.setattr(autotune, "time", types.SimpleNamespace(perf_counter=c.perf_counter))
    return c


FRAME_DEFAULTS = {"trace_config": 17, "tail_bounce": -1, "tail_blocks": 2, "pass_shadow_sort": 1, "pass_ray_sort": 0}


def frame_cost(best):
    """A frame cost with a unique minimum at `best` (a dict of the tuned keys)."""
    def cost(s):
        c = 3.0
        c += 0.05 * abs(s["trace_config"] - best["trace_config"])
        c += 0.11 * abs(s["tail_bounce"] - best["tail_bounce"])
        # Without a tail launch the blocks do not matter.
        if s["tail_bounce"] >= 0:
            c += 0.07 * abs(s["tail_blocks"] - best["tail_blocks"])
        c += 0.03 * (s["pass_shadow_sort"] != best["pass_shadow_sort"])
        c += 0.02 * abs(s["pass_ray_sort"] - best["pass_ray_sort"]) / 3
        return c * 1e-3
    return cost


@pytest.mark.parametrize("best", [
    {"trace_config": 16, "tail_bounce": 1, "tail_blocks": 4, "pass_shadow_sort": 1, "pass_ray_sort": 0},
    {"trace_config": 17, "tail_bounce": 2, "tail_blocks": 3, "pass_shadow_sort": 0, "pass_ray_sort": 0},
    {"trace_config": 17, "tail_bounce": 3, "tail_blocks": 2, "pass_shadow_sort": 0, "pass_ray_sort": 9},
    {"trace_config": 16, "tail_bounce": 0, "tail_blocks": 3, "pass_shadow_sort": 0, "pass_ray_sort": 0},
    {"trace_config": 16, "tail_bounce": -1, "tail_blocks": 2, "pass_shadow_sort": 1, "pass_ray_sort": 12},
])
def test_tune_frame_picks_the_cheapest_structure(clock, best):
    k = FakeKernel(clock, frame_cost(best), FRAME_DEFAULTS)
    out = autotune.tune_frame(k, configs=(17, 16))
    for key, v in best.items():
        assert k.state[key] == v, (key, k.state, best)
    assert out["trace_config"] == best["trace_config"]
    assert out["tail_bounce"] == best["tail_bounce"]
    assert out["tail_blocks"] == best["tail_blocks"]
    assert out["pass_shadow_sort"] == best["pass_shadow_sort"]
    assert out["pass_ray_sort"] == best["pass_ray_sort"]
    assert set(out["config_ms_per_frame"]) == {16, 17}
    # The reported per-bounce times belong to the chosen blocks and configuration.
    assert min(out["ms_per_frame"], key=out["ms_per_frame"].get) == best["tail_bounce"]
    if best["tail_bounce"] == 0:
        # A tail from the camera rays leaves no bounce-1 queue to bin: the binning is not tried.
        assert all(v == 0 for key, v in k.sets if key == "pass_ray_sort")


def test_tune_frame_picks_the_culling_mode_first(clock):
    best = {"trace_config": 17, "tail_bounce": 1, "tail_blocks": 4, "pass_shadow_sort": 1, "pass_ray_sort": 0}
    base = frame_cost(best)

    def cost(s):
        return base(s) + 1e-3 * abs(s["primitive_culling"] - 2)

    k = FakeKernel(clock, cost, dict(FRAME_DEFAULTS, primitive_culling=0))
    out = autotune.tune_frame(k, culling=True)
    assert k.state["primitive_culling"] == 2 and out["primitive_culling"] == 2
    assert set(out["culling_ms_per_frame"]) == {0, 1, 2}
    assert (out["tail_bounce"], out["tail_blocks"]) == (1, 4)


def test_tune_frame_without_configs_keeps_the_handle_configuration(clock):
    best = {"trace_config": 16, "tail_bounce": 1, "tail_blocks": 4, "pass_shadow_sort": 1, "pass_ray_sort": 0}
    k = FakeKernel(clock, frame_cost(best), FRAME_DEFAULTS)
    out = autotune.tune_frame(k)
    assert k.state["trace_config"] == 17
    assert all(key != "trace_config" for key, _ in k.sets)
    assert out["config_ms_per_frame"] == {}
    assert (out["tail_bounce"], out["tail_blocks"]) == (1, 4)


def test_tune_trace_picks_culling_and_configuration(clock):
    best_cfg, best_cull = 9, 2

    def cost(s):
        return 1e-3 * (5.0 + 0.1 * abs(s["trace_config"] - best_cfg) + 0.2 * abs(s["primitive_culling"] - best_cull)
                       + 0.05 * (1 - s["l2_persist"]))

    k = FakeKernel(clock, cost, {"trace_config": 16, "primitive_culling": 0, "l2_persist": 1})
    out = autotune.tune_trace(k)
    assert k.state == {"trace_config": best_cfg, "primitive_culling": best_cull, "l2_persist": 1}
    assert out["best"] == best_cfg and out["primitive_culling"] == best_cull and out["l2_persist"] == 1
    assert set(out["ms_per_pass"]) == set(range(18))


def test_tune_wide_picks_wave_size_sort_and_shadow_schedule(clock):
    def cost(s):
        return 1e-3 * (2.0 + 0.01 * abs(s["wide_samples"] - 32) + 0.1 * (1 - s["ray_sort"]) + 0.05 * (1 - s["shadow_defer"]))

    k = FakeKernel(clock, cost, {"wide_samples": 8, "ray_sort": 1, "shadow_defer": 0})
    out = autotune.tune_wide(k, passes=64)
    assert k.state == {"wide_samples": 32, "ray_sort": 1, "shadow_defer": 1}
    assert out["best"] == 32 and out["ray_sort"] == 1 and out["shadow_defer"] == 1


def test_tune_batch_maximises_the_sample_rate(clock):
    caps = (1 << 22, 1 << 23, 1 << 24)

    def cost(s):  # seconds per sample: lowest at capacity 2^23, configuration 16, binning on, deferred shadows
        return 1e-9 * (1.0 + 0.1 * abs(caps.index(s["wave_capacity"]) - 1) + 0.02 * abs(s["trace_config"] - 16)
                       + 0.3 * (1 - s["ray_sort"]) + 0.05 * (1 - s["shadow_defer"]))

    b = FakeBatch(clock, cost, {"wave_capacity": 1 << 22, "trace_config": 0, "ray_sort": 1, "shadow_defer": 0})
    out = autotune.tune_batch(b, capacities=caps)
    assert out["best"] == {"wave_capacity": 1 << 23, "trace_config": 16, "ray_sort": 1, "shadow_defer": 1}
    assert b.state == {"wave_capacity": 1 << 23, "trace_config": 16, "ray_sort": 1, "shadow_defer": 1}
    # Every (capacity, configuration) pair the tuner tried is reported.
    assert set(out["m_samples_per_s"]) == {f"{c}/{g}" for c, g in itertools.product(caps, (0, 1, 2, 3, 9, 15, 16, 17))}
