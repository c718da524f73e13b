"""The autotuner's search and table logic with a fake case whose step time
depends on its settings (no GPU)."""
from mphimplicit_gb300 import autotune


class FakeCase:
    clock = [0.0]

    def __init__(self, cost):
        self.cost, self.opts = cost, {}

    def set_option(self, k, v):
        self.opts[k] = v

    def step(self, n):
        FakeCase.clock[0] += n * self.cost(self.opts)

    def close(self):
        pass


def test_coordinate_descent_finds_the_fastest_settings(monkeypatch):
    # fastest: pair_block 256, ct_block 128, chunk 16
    def cost(o):
        return (abs(o["pair_block"] - 256) / 256 + abs(o["ct_block"] - 128) / 128 + abs(o["chunk"] - 16) / 16) + 1.0
    monkeypatch.setattr(autotune.time, "perf_counter", lambda: FakeCase.clock[0])
    out = autotune.tune(lambda: FakeCase(cost), steps=2, warmup=1)
    assert out["settings"] == {"pair_block": 256, "ct_block": 128, "chunk": 16}
    assert len(out["ms_per_step"]) == 3 + 1 + 3   # defaults shared between the coordinates


def test_noise_keeps_the_defaults(monkeypatch):
    # 1% differences stay below the switching margin
    def cost(o):
        return 1.0 - 0.01 * (o["pair_block"] == 128) - 0.01 * (o["chunk"] == 32)
    monkeypatch.setattr(autotune.time, "perf_counter", lambda: FakeCase.clock[0])
    assert autotune.tune(lambda: FakeCase(cost), steps=2, warmup=1)["settings"] == autotune.DEFAULTS


def test_table_choice_by_size_class():
    t = {"2d:12": {"settings": {"pair_block": 256, "ct_block": 128, "chunk": 4}},
         "3d:20": {"settings": {"pair_block": 512, "ct_block": 256, "chunk": 16}}}
    assert autotune.choose(t, 2, 4096)["pair_block"] == 256
    assert autotune.choose(t, 2, 1 << 16)["chunk"] == 4          # nearest 2D class
    assert autotune.choose(t, 3, 1 << 18)["chunk"] == 16
    assert autotune.choose(None, 3, 10) == autotune.DEFAULTS
    assert autotune.choose({}, 2, 10) == autotune.DEFAULTS
