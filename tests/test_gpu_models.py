"""GPU parity of the model extensions (libnclr_gpu.so through its C ABI) against the CPU
oracle: the neo-Hookean stress (src/nclr.h:339's TODO) and per-particle Young's modulus and
Poisson ratio (nclr_set_moduli).

Tolerances, with errors measured as in test_gpu_step.py:
  * One step from a seeded random state: within 5e-5 of the FP32 oracle. The error against
    the FP64 oracle stays within 2.5x the FP32 oracle's own (or under 1e-5).
  * Several steps, and a modulus change between advance() calls: within the drift bounds of
    conftest.DRIFT.
"""
import numpy as np
import pytest

from conftest import DRIFT, FIELDS, check_fp32_class, field_err, random_state
from nuclearmpm_gb300 import BatchSimulation, MPMSimulation, capi, scenes

pytestmark = pytest.mark.gpu

RANDOM_VS_FP32 = 5e-5
RANDOM_FP64_FACTOR = 2.5
COROTATED, NEOHOOKEAN = capi.STRESS_COROTATED, capi.STRESS_NEOHOOKEAN
# the single-simulation step paths: the small-scene kernel, the tile kernel, and the tile
# kernel with every block stepped particle by particle
PATHS = {"small": {"small_scene_max": 1 << 30},
         "tile": {"small_scene_max": 0, "sparse_block_max": 0},
         "thin": {"small_scene_max": 0, "sparse_block_max": 1 << 30}}
# (dim, physics) pairs the neo-Hookean stress is defined for (det F > 0)
NEO_CASES = [(2, scenes.REFERENCE), (2, scenes.CORRECTED), (3, scenes.CORRECTED)]


def random_moduli(rng, n):
    return (np.exp(rng.uniform(np.log(1e3), np.log(1e5), size=n)).astype(np.float32),
            rng.uniform(0.1, 0.4, size=n).astype(np.float32))


def state_of(sim):
    p = sim.particles()
    return {"x": p.x, "v": p.v, "F": p.F, "C": p.C, "Jp": p.Jp}


def check_one_step(out, grid, o32, og32, o64, og64):
    pairs = [(out[f], o32[f], o64[f], f) for f in FIELDS]
    if grid is not None:
        pairs += [(grid.velocity, og32[0], og64[0], "grid_v"),
                  (grid.mass, og32[1], og64[1], "grid_m")]
    for gpu, ref32, ref64, f in pairs:
        e32, e64, own = field_err(gpu, ref32, f), field_err(gpu, ref64, f), field_err(ref32, ref64, f)
        assert e32 <= RANDOM_VS_FP32, (f, e32)
        assert e64 <= max(RANDOM_FP64_FACTOR * own, 1e-5), (f, e64, own)


@pytest.mark.parametrize("dim,physics", NEO_CASES)
@pytest.mark.parametrize("model", [scenes.SNOW, scenes.JELLY, scenes.LIQUID])
@pytest.mark.parametrize("path", sorted(PATHS))
def test_neohookean_one_step_vs_oracle(oracle, dim, physics, model, path):
    rng = np.random.default_rng(1000 + 100 * dim + 10 * model + physics)
    res = 32
    s = random_state(rng, dim, 2000 if dim == 2 else 4000, res, physics)
    sim = MPMSimulation(dict(s), model, res=res, physics=physics, stress_model=NEOHOOKEAN,
                        **PATHS[path])
    sim.advance(1)
    out, grid = state_of(sim), sim.grid()
    sim.close()
    kw = dict(dim=dim, model=model, res=res, steps=1, physics=physics, stress=NEOHOOKEAN)
    o32, og32, st, _ = oracle.advance(s, **kw)
    o64, og64, _, _ = oracle.advance(s, fp64=True, **kw)
    assert st == 0
    check_one_step(out, grid, o32, og32, o64, og64)


@pytest.mark.parametrize("dim,physics,stress", [(2, scenes.REFERENCE, COROTATED),
                                                (3, scenes.REFERENCE, COROTATED),
                                                (2, scenes.REFERENCE, NEOHOOKEAN),
                                                (3, scenes.CORRECTED, NEOHOOKEAN)])
@pytest.mark.parametrize("path", sorted(PATHS))
def test_per_particle_moduli_one_step_vs_oracle(oracle, dim, physics, stress, path):
    """Every particle with its own E (log-uniform 1e3..1e5) and nu (0.1..0.4), mixed materials."""
    rng = np.random.default_rng(2000 + 10 * dim + stress)
    res, n = 32, 2000 if dim == 2 else 4000
    s = random_state(rng, dim, n, res, physics)
    mat = rng.integers(0, 3, size=n).astype(np.uint8)
    if dim == 3 and physics == scenes.REFERENCE:
        mat[mat == scenes.LIQUID] = scenes.SNOW  # 3D liquid's polar rotation is not unique there
    E, nu = random_moduli(rng, n)
    sim = MPMSimulation(dict(s), scenes.JELLY, res=res, physics=physics, material=mat,
                        stress_model=stress, **PATHS[path])
    sim.set_moduli(E, nu)
    sim.advance(1)
    out, grid = state_of(sim), sim.grid()
    sim.close()
    kw = dict(dim=dim, model=scenes.JELLY, res=res, steps=1, physics=physics, material=mat,
              E_particles=E, nu_particles=nu, stress=stress)
    o32, og32, st, _ = oracle.advance(s, **kw)
    o64, og64, _, _ = oracle.advance(s, fp64=True, **kw)
    assert st == 0
    check_one_step(out, grid, o32, og32, o64, og64)


@pytest.mark.parametrize("path", sorted(PATHS))
@pytest.mark.parametrize("stress", [COROTATED, NEOHOOKEAN])
def test_moduli_follow_particles_and_changes_take_effect(oracle, path, stress):
    """Moduli set, stepped through re-sorts (sort_interval 1), changed between advance() calls
    (the pending P2G of the tile path must be redone), then returned to the scene's pair."""
    dim, res, physics, n = 2, 48, scenes.REFERENCE, 3000
    rng = np.random.default_rng(31 + stress)
    s = random_state(rng, dim, n, res, physics)
    E1, nu1 = random_moduli(rng, n)
    E2, nu2 = random_moduli(rng, n)
    sim = MPMSimulation(dict(s), scenes.SNOW, res=res, physics=physics, sort_interval=1,
                        stress_model=stress, **PATHS[path])
    kw = dict(dim=dim, model=scenes.SNOW, res=res, physics=physics, stress=stress,
              want_grid=False)
    o, o64 = dict(s), dict(s)
    for E, nu, steps in ((E1, nu1, 4), (E2, nu2, 3), (None, None, 3)):
        sim.set_moduli(E, nu)
        sim.advance(steps)
        extra = {} if E is None else dict(E_particles=E, nu_particles=nu)
        nxt, _, st, _ = oracle.advance(o, steps=steps, **kw, **extra)
        nxt64, _, st64, _ = oracle.advance(o64, steps=steps, fp64=True, **kw, **extra)
        assert st == 0 and st64 == 0
        o, o64 = dict(o, **nxt), dict(o64, **nxt64)
        # E up to 1e5 is ten times stiffer than the fixtures DRIFT was derived from
        check_fp32_class(state_of(sim), o, o64, DRIFT, what=steps)
    sim.close()


def test_device_moduli_equal_host_moduli():
    torch = pytest.importorskip("torch")
    dim, res, physics, n = 3, 32, scenes.CORRECTED, 4000
    rng = np.random.default_rng(5)
    s = random_state(rng, dim, n, res, physics)
    E, nu = random_moduli(rng, n)
    outs = []
    for device_arrays in (False, True):
        sim = MPMSimulation(dict(s), scenes.JELLY, res=res, physics=physics, small_scene_max=0,
                            stress_model=NEOHOOKEAN)
        if device_arrays:
            sim.set_moduli(torch.tensor(E, device="cuda"), torch.tensor(nu, device="cuda"))
        else:
            sim.set_moduli(E, nu)
        sim.advance(5)
        outs.append(state_of(sim))
        sim.close()
    for f in FIELDS:
        assert field_err(outs[1][f], outs[0][f], f) <= DRIFT[f], f


@pytest.mark.parametrize("small", [False, True])
@pytest.mark.parametrize("stress", [COROTATED, NEOHOOKEAN])
def test_batch_per_particle_moduli_vs_oracle(oracle, small, stress):
    """A batch of scenes of different sizes, resolutions and materials, moduli set over all of
    them at once (the scenes concatenated): each scene against its own oracle run."""
    rng = np.random.default_rng(77 + stress)
    descs, moduli = [], []
    for i, (n, res, model) in enumerate(((1500, 32, scenes.SNOW), (700, 64, scenes.JELLY),
                                          (2600, 48, scenes.LIQUID))):
        s = random_state(rng, 2, n, res, scenes.REFERENCE)
        descs.append(dict(s, model=model, res=res, E=1e4, nu=0.2))
        moduli.append(random_moduli(rng, n))
    b = BatchSimulation(descs, stress_model=stress,
                        **({"small_scene_max": 1 << 30} if small else {}))
    b.set_moduli(np.concatenate([m[0] for m in moduli]), np.concatenate([m[1] for m in moduli]))
    b.advance(3)
    for i, d in enumerate(descs):
        s = {k: d[k] for k in ("x", "v", "F", "C", "Jp", "mass", "volume")}
        o, _, st, _ = oracle.advance(s, dim=2, model=d["model"], res=d["res"], steps=3,
                                     E_particles=moduli[i][0], nu_particles=moduli[i][1],
                                     stress=stress, want_grid=False)
        assert st == 0
        got = b.particles(i)
        for f in FIELDS:
            assert field_err(got[f], o[f], f) <= DRIFT[f], (i, f)
    b.close()
