"""The measured workloads at their full sizes, on the GPU.
- The 1M-particle 3D jelly scene, the same in snow, and the 4.19M-particle liquid + snow
  scene: one step against the FP32 oracle, run on all host cores.
- The same two scenes conserve their total mass, and with gravity off their total momentum,
  through a step.
- The 256-scene batch: one step of the batch equals every scene stepped alone.

Bound for a step against the oracle: 5e-5 (x, v, F, C, Jp and the grid), as for the seeded
random states of test_gpu_step.py.  The sizes need a few GB of device memory and a few
seconds of host time.
"""
import os

import numpy as np
import pytest

from conftest import DRIFT, FIELDS, field_err
from nuclearmpm_gb300 import BatchSimulation, MPMSimulation, scenes

pytestmark = pytest.mark.gpu

STEP_BOUND = 5e-5
THREADS = max(1, os.cpu_count() or 1)


def gpu_step(state, model, res, steps=1, material=None, **kw):
    sim = MPMSimulation(dict(state), model, res=res, material=material, **kw)
    sim.advance(steps)
    p = sim.particles()
    out = {"x": p.x, "v": p.v, "F": p.F, "C": p.C, "Jp": p.Jp}
    grid = sim.grid()
    sim.close()
    return out, grid


@pytest.mark.parametrize("scene", ["jelly_1M", "snow_1M", "mixed_4M"])
def test_full_size_step_matches_oracle(oracle, scene):
    if scene == "jelly_1M":
        s, mat, model, res = scenes.jelly_cubes_3d(seed=0, res=128), None, scenes.JELLY, 128
    elif scene == "snow_1M":  # the same geometry in snow
        s, mat, model, res = scenes.jelly_cubes_3d(seed=0, res=128), None, scenes.SNOW, 128
    else:
        s, mat = scenes.liquid_snow_boxes_3d(seed=0, res=256)
        model, res = scenes.SNOW, 256
    out, grid = gpu_step(s, model, res, material=mat)
    ref, og, st, _ = oracle.advance(s, dim=3, model=model, res=res, steps=1, material=mat,
                                    threads=THREADS)
    assert st == 0
    for f in FIELDS:
        assert field_err(out[f], ref[f], f) <= STEP_BOUND, (f, field_err(out[f], ref[f], f))
    assert field_err(grid.velocity, og[0], "grid_v") <= STEP_BOUND
    assert field_err(grid.mass, og[1], "grid_m") <= STEP_BOUND


@pytest.mark.parametrize("scene", ["jelly_1M", "mixed_4M"])
def test_full_size_step_conserves_mass_and_momentum(scene):
    """Without gravity and away from the walls, P2G, the grid update and G2P conserve the total
    mass (it all lands on the grid) and the total momentum (the stress is internal)."""
    if scene == "jelly_1M":
        s, mat, model, res = scenes.jelly_cubes_3d(seed=0, res=128), None, scenes.JELLY, 128
    else:
        s, mat = scenes.liquid_snow_boxes_3d(seed=0, res=256)
        model, res = scenes.SNOW, 256
    m = s["mass"].astype(np.float64)
    p0 = (m[:, None] * s["v"].astype(np.float64)).sum(0)
    out, grid = gpu_step(s, model, res, material=mat, gravity=0.0)
    assert abs(float(grid.mass.astype(np.float64).sum()) - m.sum()) <= 1e-5 * m.sum()
    p1 = (m[:, None] * out["v"].astype(np.float64)).sum(0)
    # the scale of the momenta that cancel (the 4M scene starts at rest: then a floor)
    scale = max((m[:, None] * np.abs(s["v"].astype(np.float64))).sum(), 1e-2 * m.sum())
    assert np.abs(p1 - p0).max() <= 1e-5 * scale, (p0, p1)


def test_full_batch_equals_scenes_stepped_alone():
    scs = scenes.batched_scenes_2d(seed=0)
    b = BatchSimulation(scs)
    b.advance(1)
    for i, sc in enumerate(scs):
        state = {k: sc[k] for k in ("x", "v", "F", "C", "Jp", "mass", "volume")}
        alone, _ = gpu_step(state, sc["model"], sc["res"], dt=sc["dt"], E=sc["E"], nu=sc["nu"],
                            gravity=sc["gravity"])
        got = b.particles(i)
        for f in FIELDS:
            assert field_err(got[f], alone[f], f) <= min(DRIFT[f], 1e-5), (i, f)
    b.close()
