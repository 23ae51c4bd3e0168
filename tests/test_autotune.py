"""The autotuner's search and cache (CPU: a stand-in simulation whose step time depends on the
knobs)."""
import time

from nuclearmpm_gb300 import autotune


class FakeSim:
    def __init__(self, sort_interval=8, graph_steps=0):
        self.cost = 1e-4 * abs(sort_interval - 4) + 1e-5
        self.closed = False

    def advance(self, steps):
        time.sleep(self.cost)

    def close(self):
        self.closed = True


def test_picks_the_fastest_and_caches(tmp_path):
    cache = str(tmp_path / "tune.json")
    made = []

    def make(**opt):
        made.append(opt)
        return FakeSim(**opt)

    best = autotune.tune(make, key="w", candidates={"sort_interval": [1, 4, 16]}, steps=1,
                         repeats=2, cache_path=cache)
    assert best == {"sort_interval": 4}
    n = len(made)
    assert autotune.tune(make, key="w", candidates={"sort_interval": [1, 4, 16]},
                         cache_path=cache) == {"sort_interval": 4}
    assert len(made) == n  # served from the cache


def test_graph_steps_is_carried():
    best = autotune.tune(lambda **o: FakeSim(**o), candidates={"sort_interval": [2, 4]},
                         steps=1, repeats=1, cache_path=None, graph_steps=100)
    assert best == {"graph_steps": 100, "sort_interval": 4}
