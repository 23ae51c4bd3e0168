"""Scene builders on the device (nclr_cube_device / nclr_cubes_device) and simulations created
from device arrays (nclr_create_device): the lattices are bit-equal to the host builders that
reproduce cube<dim>() (src/nclr_math.h:100-129), and a simulation built on the device steps
exactly like one built from host arrays."""
import numpy as np
import pytest

from conftest import DRIFT, FIELDS, field_err
from nuclearmpm_gb300 import MPMSimulation, capi, scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("res,lo,hi", [(50, 0.4, 0.6), (25, 0.1, 0.35), (7, -0.9, 0.2), (1, 0.3, 0.7),
                                       (64, 0.05, 0.95)])
def test_device_cube_is_bit_equal_to_host_builder(dim, res, lo, hi):
    got = scenes.cubes_device(dim, res, [lo], [hi]).cpu().numpy()
    assert np.array_equal(got, scenes.cube(dim, res, lo, hi))


def test_device_cubes_stack_like_generate_cubes():
    los, his = [0.1, 0.5, 0.3], [0.3, 0.7, 0.45]
    got = scenes.cubes_device(2, 25, los, his).cpu().numpy()
    want = np.concatenate([scenes.cube(2, 25, a, b) for a, b in zip(los, his)])
    assert np.array_equal(got, want)


@pytest.mark.parametrize("model", [scenes.SNOW, scenes.JELLY])
def test_simulation_from_device_arrays_matches_host_creation(model):
    x = scenes.cubes_device(2, 50, [0.4, 0.4], [0.6, 0.6])
    x[2500:, 1] -= 0.35  # the README scene's second lattice
    xh = x.cpu().numpy()
    a = MPMSimulation.from_device(x, model)
    b = MPMSimulation(scenes.particles(xh), model)
    pa, pb = a.particles(), b.particles()
    for f in FIELDS:
        assert np.array_equal(getattr(pa, f), getattr(pb, f)), f
    a.advance(20)
    b.advance(20)
    pa, pb = a.particles(), b.particles()
    for f in FIELDS:  # the grid sums are FP32 atomics: equal up to their order
        assert field_err(getattr(pa, f), getattr(pb, f), f) <= DRIFT[f], f
    a.close()
    b.close()


def test_device_creation_with_all_fields_and_materials():
    rng = np.random.default_rng(5)
    n = 3000
    s = scenes.particles(rng.uniform(0.3, 0.7, size=(n, 3)).astype(np.float32))
    s["v"] = rng.normal(0, 0.1, size=(n, 3)).astype(np.float32)
    s["Jp"] = rng.uniform(0.9, 1.1, size=n).astype(np.float32)
    s["mass"] = rng.uniform(0.5, 2.0, size=n).astype(np.float32)
    mat = rng.integers(0, 3, size=n).astype(np.uint8)
    t = {k: torch.tensor(v, device="cuda") for k, v in s.items() if k in
         ("x", "v", "F", "C", "Jp", "mass", "volume")}
    a = MPMSimulation.from_device(t["x"], scenes.SNOW, res=32, v=t["v"], F=t["F"], C=t["C"],
                                  Jp=t["Jp"], mass=t["mass"], volume=t["volume"],
                                  material=torch.tensor(mat, device="cuda"))
    b = MPMSimulation(dict(s), scenes.SNOW, res=32, material=mat)
    a.advance(3)
    b.advance(3)
    pa, pb = a.particles(), b.particles()
    for f in FIELDS:
        assert field_err(getattr(pa, f), getattr(pb, f), f) <= DRIFT[f], f
    a.close()
    b.close()
    bad = mat.copy()
    bad[17] = 7
    with pytest.raises(capi.NclrError):
        MPMSimulation.from_device(t["x"], scenes.SNOW, res=32, material=torch.tensor(bad, device="cuda"))
