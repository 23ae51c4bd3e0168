"""GPU tests of the batched form (nclr_batch_create): every scene of a batch steps exactly as
it does alone, and matches the CPU oracle."""
import numpy as np
import pytest

from conftest import FIELDS, field_err
from nuclearmpm_gb300 import BatchSimulation, MPMSimulation, scenes

pytestmark = pytest.mark.gpu

# One step: the one-step parity bound of the plain step.  Ten steps: the plain step's
# multi-step drift bounds (runs differ only in the atomic summation order, which stiff scenes
# -- E up to 1e5 with unit particle mass and volume -- amplify from step to step), or twice
# the FP32 oracle's own distance to the FP64 oracle over the same steps where that is larger
# (the summation order alone moves a scene that far: 3.3e-3 in v on one scene below).
ONE_STEP = 1e-5
TEN_STEPS = {"x": 2e-5, "v": 3e-3, "F": 3e-4, "C": 1e-2, "Jp": 3e-4}
FP32_SPREAD_FACTOR = 2.0


def small_batch(seed=0, count=6, dim=2):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(200, 3000))
        res = int(rng.choice([32, 64, 128]))
        if dim == 2:
            sc = scenes.random_scene_2d(rng, n, res)
        else:
            side = int(round(n ** (1 / 3)))
            x = scenes.jittered_block(rng, (side,) * 3, 0.5 / res, rng.uniform(0.3, 0.5, 3),
                                      0.25 / res)
            sc = scenes.particles(x, rng.normal(0, 0.3, size=x.shape).astype(np.float32))
        sc.update(model=int(i % 3), res=res, E=float(np.exp(rng.uniform(np.log(1e3), np.log(1e5)))),
                  nu=float(rng.uniform(0.1, 0.4)), dt=1e-4, gravity=-100.0)
        out.append(sc)
    return out


def alone(sc, steps, physics=scenes.REFERENCE):
    sim = MPMSimulation({k: sc[k] for k in ("x", "v", "F", "C", "Jp", "mass", "volume")},
                        sc["model"], res=sc["res"], dt=sc["dt"], E=sc["E"], nu=sc["nu"],
                        gravity=sc["gravity"], physics=physics)
    sim.advance(steps)
    p = sim.particles()
    g = sim.grid()
    sim.close()
    return {f: getattr(p, f) for f in FIELDS}, g


# The batch's step paths: "tile" the block-sorted fused kernel with CUDA graphs (the default;
# 2D items of 128 threads), "tile256" the same with 256 threads per item (the autotuner's other
# item size), "small" all of a call's steps in one cooperative launch with a group of CTAs per
# scene (an option).
PATHS = {"small": {"small_scene_max": 1 << 30}, "tile": {}, "tile256": {"batch_item_threads": 256}}


@pytest.mark.parametrize("path", sorted(PATHS))
@pytest.mark.parametrize("dim,physics,steps", [(2, scenes.REFERENCE, 10),
                                               (3, scenes.REFERENCE, 1),
                                               (3, scenes.CORRECTED, 10)])
def test_batch_matches_scenes_stepped_alone(oracle, dim, physics, steps, path):
    """Ten steps where the physics is well conditioned; under the reference's 3D physics the
    snow scenes clamp a zero singular value every step and their velocities grow towards the
    clip, so two runs that differ only in summation order part after a few steps: one step."""
    scs = small_batch(seed=dim, dim=dim)
    if dim == 3 and physics == scenes.CORRECTED:
        for sc in scs:
            sc["F"] = np.broadcast_to(np.eye(3, dtype=np.float32), sc["F"].shape).copy()
    batch = BatchSimulation(scs, sort_interval=4, graph_steps=8, physics=physics, **PATHS[path])
    batch.advance(steps)
    for i, sc in enumerate(scs):
        ref, rg = alone(sc, steps, physics)
        got = batch.particles(i)
        tol = {f: ONE_STEP for f in FIELDS}
        if steps > 1:
            st = {k: sc[k] for k in ("x", "v", "F", "C", "Jp", "mass", "volume")}
            kw = dict(dim=dim, model=sc["model"], res=sc["res"], dt=sc["dt"], E=sc["E"],
                      nu=sc["nu"], gravity=sc["gravity"], steps=steps, physics=physics,
                      want_grid=False)
            o32, o64 = oracle.advance(st, **kw)[0], oracle.advance(st, fp64=True, **kw)[0]
            tol = {f: max(TEN_STEPS[f], FP32_SPREAD_FACTOR * field_err(o32[f], o64[f], f))
                   for f in FIELDS}
        for f in FIELDS:
            assert field_err(got[f], ref[f], f) <= tol[f], (i, f)
        g = batch.grid(i)
        assert g.mass.shape == rg.mass.shape
        assert batch.status(i) == 0
    batch.close()


@pytest.mark.parametrize("path", sorted(PATHS))
def test_batch_one_step_matches_oracle(oracle, path):
    scs = small_batch(seed=7, count=5)
    batch = BatchSimulation(scs, **PATHS[path])
    batch.advance(1)
    for i, sc in enumerate(scs):
        o, og, st, _ = oracle.advance(sc, dim=2, model=sc["model"], res=sc["res"], dt=sc["dt"],
                                      E=sc["E"], nu=sc["nu"], gravity=sc["gravity"], steps=1)
        assert st == 0
        got = batch.particles(i)
        for f in FIELDS:
            assert field_err(got[f], o[f], f) <= ONE_STEP, (i, f)
        g = batch.grid(i)
        assert field_err(g.velocity, og[0], "grid_v") <= ONE_STEP
        assert field_err(g.mass, og[1], "grid_m") <= ONE_STEP
    batch.close()


def test_batch_graph_of_many_steps_equals_direct_launches():
    scs = small_batch(seed=3, count=4)
    a = BatchSimulation(scs, graph_steps=20, small_scene_max=0)
    a.advance(20)  # exactly one graph, whose last step is the call's final step
    a.advance(25)
    b = BatchSimulation(scs, use_graphs=False, small_scene_max=0)
    b.advance(20)
    b.advance(25)
    c = BatchSimulation(scs, small_scene_max=1 << 30)  # the small-scene kernel
    c.advance(20)
    c2 = BatchSimulation(scs, small_scene_max=0)
    c2.advance(20)
    for i in range(len(scs)):
        pa, pb = a.particles(i), b.particles(i)
        for f in FIELDS:
            assert field_err(pa[f], pb[f], f) <= TEN_STEPS[f], (i, f)
        pc, pc2 = c.particles(i), c2.particles(i)
        for f in FIELDS:
            assert field_err(pc[f], pc2[f], f) <= TEN_STEPS[f], (i, f)
    for sim in (a, b, c, c2):
        sim.close()


@pytest.mark.parametrize("path", sorted(PATHS))
def test_batch_scene_set_get_and_error_isolated(path):
    scs = small_batch(seed=5, count=3)
    bad = dict(scs[1])
    bad["x"] = bad["x"].copy()
    bad["x"][0] = (-0.3, 0.5)  # leaves the grid on the first step
    batch = BatchSimulation([scs[0], bad, scs[2]], **PATHS[path])
    with pytest.raises(IndexError):
        batch.advance(1)
    assert batch.status(0) == 0 and batch.status(1) == 2 and batch.status(2) == 0
    # per-scene upload / download
    p = batch.particles(2)
    batch.set_particles(2, x=scs[2]["x"], Jp=np.full(len(scs[2]["x"]), 2.0, np.float32))
    q = batch.particles(2)
    assert np.array_equal(q["x"], scs[2]["x"]) and np.all(q["Jp"] == 2.0)
    assert np.array_equal(q["F"], p["F"])
    batch.close()
