"""The measured workloads at their full sizes, on the GPU.
- The 1M-particle 3D jelly scene, the same in snow, and the 4.19M-particle liquid + snow
  scene, under both physics modes: one step from the scene against the FP32 oracle and against
  the FP64 oracle, both run on all host cores, within 1e-5 for every field and the grid; one
  step from the state after 10 steps (F, C and Jp deformed), where FP32 itself lands further
  from FP64 in v and C, within 1e-5 or the FP32 class (conftest.check_fp32_class).
- The same two scenes conserve their total mass, and with gravity off their total momentum,
  through a step.
- The 256-scene batch: one step of the batch equals every scene stepped alone.

The sizes need a few GB of device memory and a few seconds of host time per case.
"""
import os

import numpy as np
import pytest

from conftest import DRIFT, FIELDS, check_fp32_class, field_err
from nuclearmpm_gb300 import BatchSimulation, MPMSimulation, scenes

pytestmark = pytest.mark.gpu

# One step at the measured sizes, normwise per field (conftest.field_err), against the FP32
# and the FP64 oracle alike.  Measured on GB300: at most 3e-6 against either.
STEP_BOUND = 1e-5
THREADS = max(1, os.cpu_count() or 1)


def gpu_step(state, model, res, steps=1, material=None, **kw):
    sim = MPMSimulation(dict(state), model, res=res, material=material, **kw)
    sim.advance(steps)
    p = sim.particles()
    out = {"x": p.x, "v": p.v, "F": p.F, "C": p.C, "Jp": p.Jp}
    grid = sim.grid()
    sim.close()
    return out, grid


# The snow clamp's ill-conditioned points (conftest.check_fp32_class): snow particles whose
# F_hat = M F (M = diag(1) + dt C, with this step's C from the FP64 oracle) has det < 0 and a
# clamp gain f s_1 / (s_p + s_l) of at least CLAMP_ILL_GAIN, ten times the bound of the
# well-conditioned case (1, det > 0).  The deformed reference-physics scenes have C of order
# 1e4, so dt C is of order 1 and C's FP32 rounding moves F_hat by ~1e-3 relative: at such
# gains that is the whole FP32-class budget.
CLAMP_ILL_GAIN = 10.0
CLAMP_LO, CLAMP_HI = 1.0 - 2.5e-2, 1.0 + 4.5e-3
DT = 1e-4


def clamp_ill_rows(state, o64, mat, model, physics):
    def ill(rows):
        rows = np.asarray(rows, dtype=np.int64)
        F = np.asarray(state["F"], np.float64).reshape(-1, 3, 3)[rows]
        C = np.asarray(o64["C"], np.float64).reshape(-1, 3, 3)[rows]
        M = np.broadcast_to(np.eye(3), C.shape).copy()
        if physics == scenes.REFERENCE:
            M[:, 2, 2] = 0.0  # the reference's diag<3>(1) = diag(1, 1, 0)
        Fh = (M + DT * C) @ F
        det = np.linalg.det(Fh)
        sv = np.linalg.svd(Fh, compute_uv=False)
        sp, sl = sv[:, 1], np.where(det < 0, -sv[:, 2], sv[:, 2])
        f = np.clip(sp, CLAMP_LO, CLAMP_HI) + np.clip(sl, CLAMP_LO, CLAMP_HI)
        gain = np.where(det < 0, f * sv[:, 0] / np.maximum(sp + sl, 1e-300), 0.0)
        snow = (np.asarray(mat)[rows] == scenes.SNOW) if mat is not None else \
            np.full(len(rows), model == scenes.SNOW)
        return snow & (det < 0) & (gain >= CLAMP_ILL_GAIN)
    return ill


def full_scene(scene, physics):
    if scene == "jelly_1M":
        return scenes.jelly_cubes_3d(seed=0, res=128, physics=physics), None, scenes.JELLY, 128
    if scene == "snow_1M":  # the same geometry in snow
        return scenes.jelly_cubes_3d(seed=0, res=128, physics=physics), None, scenes.SNOW, 128
    s, mat = scenes.liquid_snow_boxes_3d(seed=0, res=256, physics=physics)
    return s, mat, scenes.SNOW, 256


@pytest.mark.parametrize("start", ["scene", "after_10_steps"])
@pytest.mark.parametrize("physics", [scenes.REFERENCE, scenes.CORRECTED])
@pytest.mark.parametrize("scene", ["jelly_1M", "snow_1M", "mixed_4M"])
def test_full_size_step_matches_oracle(oracle, scene, physics, start):
    s, mat, model, res = full_scene(scene, physics)
    if start == "after_10_steps":  # a deformed state: the GPU's own after 10 steps
        run, _ = gpu_step(s, model, res, steps=10, material=mat, physics=physics)
        s = {**run, "mass": s["mass"], "volume": s["volume"]}
    out, grid = gpu_step(s, model, res, material=mat, physics=physics)
    out = dict(out, grid_v=grid.velocity, grid_m=grid.mass)
    refs = {}
    for fp64 in (False, True):
        ref, og, st, _ = oracle.advance(s, dim=3, model=model, res=res, steps=1, material=mat,
                                        threads=THREADS, physics=physics, fp64=fp64)
        assert st == 0
        refs[fp64] = dict(ref, grid_v=og[0], grid_m=og[1])
    if start == "after_10_steps":  # the FP32 oracle in a second summation order (one thread)
        ref, og, st, _ = oracle.advance(s, dim=3, model=model, res=res, steps=1, material=mat,
                                        threads=1, physics=physics)
        assert st == 0
        refs["fp32_1"] = dict(ref, grid_v=og[0], grid_m=og[1])
    fields = FIELDS + ("grid_v", "grid_m")
    if start == "scene":
        for fp64, ref in refs.items():
            for f in fields:
                e = field_err(out[f], ref[f], f)
                assert e <= STEP_BOUND, (fp64, f, e)
    else:
        # from a deformed state the stiff stress amplifies FP32 rounding of the polar rotation
        # (F - R cancels), and the FP32 oracle itself lands up to a few 1e-5 from FP64 in v
        # and C: those fields are held to the FP32 class, the rest to 1e-5
        check_fp32_class(out, [refs[False], refs["fp32_1"]], refs[True], STEP_BOUND,
                         fields=fields, what=scene,
                         ill=clamp_ill_rows(s, refs[True], mat, model, physics))


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
