"""Autotuner for the runtime knobs of a simulation (plain or batched): the block re-sort
interval, the number of steps per captured CUDA graph and, for single simulations, the
thin-block threshold below which a block's particles skip the shared-memory tile.

The grid tiles of the kernels (4^3 cells in 3D, 8^2 in 2D, 8^3 / 12^2 node tiles) are
compile-time constants fixed by the shared-memory layout and the sort's 64-cell blocks.  The
knobs tuned here, by timing short runs of the workload itself through the public API (the
winner cached per workload signature), trade work against locality at run time: the re-sort
interval, the thin-block threshold, and for batches the threads that step one block together
(128 or 256, each a compiled variant of the fused kernel).

    from nuclearmpm_gb300 import autotune
    best = autotune.tune(lambda **opt: BatchSimulation(scenes, **opt), key="batch256")
    sim = BatchSimulation(scenes, **best)

    best = autotune.tune(lambda **opt: MPMSimulation(state, model, res=res, **opt),
                         key="snow1M", candidates=autotune.PLAIN_CANDIDATES)
"""
from __future__ import annotations

import json
import os
import time

DEFAULT_CANDIDATES = {"sort_interval": [2, 4, 8, 16, 32]}
# single simulations: also the thin-block threshold (particles per block; 0 = every block
# through the tile) and the tail threshold (a block's last pass of fewer particles goes to the
# thin-block chunks; 0 = never); batches ignore both
PLAIN_CANDIDATES = {"sort_interval": [2, 4, 8, 16, 32], "sparse_block_max": [0, 32, 64, 128, 256],
                    "tail_max": [0, 32, 64, 96, 128]}
# batches: re-sort interval, threads per item of the fused kernel (2D: half or whole CTAs),
# thin-block threshold
BATCH_CANDIDATES = {"sort_interval": [4, 8, 16, 32], "batch_item_threads": [128, 256],
                    "sparse_block_max": [0, 16, 32, 64]}
# single simulations small enough for the small-scene kernel: its particles per thread
SMALL_CANDIDATES = {"particles_per_thread": [1, 2, 4]}
CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")


def _load(path: str) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _time(sim, steps: int, repeats: int) -> float:
    sim.advance(steps)  # warm-up: sort, first P2G, graph capture
    best = float("inf")
    for _ in range(repeats):
        t0 = time.perf_counter()
        sim.advance(steps)  # synchronises at its end
        best = min(best, time.perf_counter() - t0)
    return best


def tune(make_sim, *, key: str | None = None, candidates: dict | None = None, steps: int = 32,
         repeats: int = 3, cache_path: str | None = CACHE, graph_steps: int | None = None,
         confirm: int = 0) -> dict:
    """Returns the fastest option set {knob: value}; `make_sim(**options)` builds the
    simulation.  Knobs are tuned one after another (coordinate descent from the defaults).
    With `confirm` > 0, the descent's pick is then timed against the defaults (no knob set)
    in `confirm` alternating rounds, and the defaults win if they are faster: the candidates
    differ by a few percent, so one noisy measurement in the descent can pick a worse set.
    With `key`, results are cached in `cache_path` and reused."""
    cands = dict(DEFAULT_CANDIDATES if candidates is None else candidates)
    cache = _load(cache_path) if (key and cache_path) else {}
    if key and key in cache:
        return dict(cache[key]["best"])
    best: dict = {}
    if graph_steps is not None:
        best["graph_steps"] = graph_steps
    timings = {}
    for knob, values in cands.items():
        scored = []
        for v in values:
            opts = dict(best, **{knob: v})
            sim = make_sim(**opts)
            try:
                t = _time(sim, steps, repeats)
            finally:
                sim.close()
            scored.append((t, v))
            timings[f"{knob}={v}"] = t
        best[knob] = min(scored)[1]
    if confirm > 0:
        base = {} if graph_steps is None else {"graph_steps": graph_steps}
        if best != base:
            t = {0: float("inf"), 1: float("inf")}
            for _ in range(confirm):
                for which, opts in ((0, best), (1, base)):
                    sim = make_sim(**opts)
                    try:
                        t[which] = min(t[which], _time(sim, steps, repeats))
                    finally:
                        sim.close()
            timings["confirm: tuned"], timings["confirm: defaults"] = t[0], t[1]
            if t[1] < t[0]:
                best = dict(base)
    if key and cache_path:
        os.makedirs(os.path.dirname(cache_path), exist_ok=True)
        cache[key] = {"best": best, "seconds": timings, "steps": steps}
        with open(cache_path, "w") as f:
            json.dump(cache, f, indent=1)
    return best
