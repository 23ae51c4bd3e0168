"""Generates the golden fixtures in this directory from the REFERENCE ITSELF.

The reference's src/nclr.h + src/nclr_math.h are compiled unmodified (against the Eigen-API
shim in oracle/ref_shim/) into oracle/_ref/libnclr_ref.so by oracle/build_oracle.py, which
needs the reference tree; this script therefore runs only where that tree exists.  The
fixtures it writes are committed, so the oracle stays pinned on machines without it.

Each .npz holds the input state (x, v, F, C, Jp, mass, volume in the C ABI host layout),
the run parameters, and the reference's output state after each listed step count
(`x@K`, `v@K`, ...), plus the post-update grid after the first step count.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from nuclearmpm_gb300 import scenes  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
FIELDS = ("x", "v", "F", "C", "Jp")


def small_block_3d(seed: int, res: int = 16):
    rng = np.random.default_rng(seed)
    x = scenes.jittered_block(rng, (8, 8, 8), 0.5 / res, (0.35, 0.4, 0.3), 0.25 / res)
    v = rng.normal(0, 0.5, size=x.shape).astype(np.float32)
    return scenes.particles(x, v)


def multiblock_3d(seed: int, res: int = 32, cubes: int = 3, side: int = 20):
    """Several jittered jelly-style lattices (spacing dx/2, jitter +-0.25 cell, one N(0, 0.5^2)
    velocity per cube) on a grid of many 4^3-cell blocks: dense blocks through the shared-memory
    tiles, thin blocks at the cubes' edges, and the block sort all take part."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / res
    edge = side * 0.5 * dx
    parts = []
    for _ in range(cubes):
        lo = rng.uniform(0.2, 0.8 - edge, size=3)
        x = scenes.jittered_block(rng, (side,) * 3, 0.5 * dx, lo, 0.25 * dx)
        v = np.broadcast_to(rng.normal(0.0, 0.5, size=3).astype(np.float32), x.shape)
        parts.append(scenes.particles(x, v))
    return scenes.concat(*parts)


def emit(name: str, state: dict, *, dim: int, model: int, res: int, steps: list[int],
         E: float = 1e4, nu: float = 0.2, gravity: float = -100.0, dt: float = 1e-4):
    out = {k: np.asarray(v, dtype=np.float32) for k, v in state.items()}
    out.update(dim=dim, model=model, res=res, E=E, nu=nu, gravity=gravity, dt=dt,
               steps=np.array(steps))
    cur = state
    done = 0
    for k in steps:
        nxt, grid, st = po.ref_advance(cur, dim=dim, model=model, res=res, dt=dt, E=E, nu=nu,
                                       gravity=gravity, steps=k - done)
        assert st == 0, f"{name}: reference raised out_of_range"
        for f in FIELDS:
            out[f"{f}@{k}"] = nxt[f].astype(np.float32)
        if done == 0:
            out["grid_v"] = grid[0].astype(np.float32)
            out["grid_m"] = grid[1].astype(np.float32)
        cur = {**nxt, "mass": state["mass"], "volume": state["volume"]}
        done = k
    path = os.path.join(OUT, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) // 1024} KiB)")


def main():
    if not po.ref_available():
        from oracle.build_oracle import build
        build()
    if not po.ref_available():
        raise SystemExit("reference tree absent: cannot regenerate golden fixtures")
    readme = scenes.readme_scene()
    emit("readme_snow", readme, dim=2, model=scenes.SNOW, res=64, steps=[1, 100, 101])
    emit("readme_jelly", readme, dim=2, model=scenes.JELLY, res=64, steps=[1, 100])
    emit("readme_liquid", readme, dim=2, model=scenes.LIQUID, res=64, steps=[1, 100])
    for model, tag in ((scenes.SNOW, "snow"), (scenes.JELLY, "jelly"), (scenes.LIQUID, "liquid")):
        emit(f"block3d_{tag}", small_block_3d(7), dim=3, model=model, res=16, steps=[1, 20, 21])
    # many blocks: 3 cubes of 20^3 particles on a 32^3 grid (24,000 particles).  Jelly for
    # 100 steps; snow for 5: under the reference's diag(1,1,0) the clamp lifts sigma_3 to 0.975
    # every step, Jp drops to its floor and the scene flies apart (speeds ~280 after 5 steps),
    # after which FP32 and FP64 runs of the reference's own step diverge by O(1) within 20 steps
    emit("multiblock3d_jelly", multiblock_3d(11), dim=3, model=scenes.JELLY, res=32,
         steps=[1, 100])
    emit("multiblock3d_snow", multiblock_3d(11), dim=3, model=scenes.SNOW, res=32, steps=[1, 5])
    # solver.cpp's defaults (E=1000, nu=0.3) on a jelly cube, 2D
    cube = scenes.particles(scenes.cube(2, 25, 0.3, 0.5))
    emit("cli_cube_jelly", cube, dim=2, model=scenes.JELLY, res=64, steps=[1, 50], E=1000.0,
         nu=0.3)


if __name__ == "__main__":
    main()
