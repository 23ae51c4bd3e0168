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
    # solver.cpp's defaults (E=1000, nu=0.3) on a jelly cube, 2D
    cube = scenes.particles(scenes.cube(2, 25, 0.3, 0.5))
    emit("cli_cube_jelly", cube, dim=2, model=scenes.JELLY, res=64, steps=[1, 50], E=1000.0,
         nu=0.3)


if __name__ == "__main__":
    main()
