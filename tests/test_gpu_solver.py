"""The headless solver (nuclearmpm_gb300/_build/nclr_solver, the reference's src/solver.cpp
over the GPU step) and the device renderer.

* The binary dump holds what the reference's solve_mpm collects (src/solver.cpp:46-61): the
  particles before every advance() and the grid of the previous one (zeros at step 0), equal
  to the same scene stepped through the Python API, in 2D and in the 3D path the reference
  leaves empty.
* A cube without coordinates is an error, as in generate_cubes (src/solver.cpp:140-143).
* nclr_render_device draws exactly the frame of a plain FP32 restatement of its rules (the
  canvas of src/solver.cpp:184-201: background, boundary box, discs painted in order).
"""
import ctypes
import math
import os
import subprocess

import numpy as np
import pytest

from conftest import DRIFT, FIELDS, field_err
from nuclearmpm_gb300 import MPMSimulation, capi, dumpio, scenes
from nuclearmpm_gb300.build import SOLVER

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def solver(*args, cwd=None):
    return subprocess.run([SOLVER, *map(str, args)], capture_output=True, text=True, cwd=cwd,
                          timeout=300)


def api_states(dim, model, cubes, cube_res, steps, E=1000.0, nu=0.3, gravity=-100.0, **kw):
    """The same run through the Python API: particles before each advance, grid after."""
    x = np.concatenate([scenes.cube(dim, cube_res, lo, hi) for lo, hi in cubes])
    sim = MPMSimulation(scenes.particles(x, physics=kw.get("physics", scenes.REFERENCE)), model,
                        res=64, dt=1e-4, E=E, nu=nu, gravity=gravity, **kw)
    out = []
    for _ in range(steps):
        p = sim.particles()
        g = sim.grid()
        out.append(({f: getattr(p, f) for f in FIELDS}, g))
        sim.advance(1)
    sim.close()
    return out


@pytest.mark.parametrize("dim,material,model", [(2, "snow", scenes.SNOW), (3, "jelly", scenes.JELLY)])
def test_dump_equals_the_api_run(tmp_path, dim, material, model):
    cubes = [(0.3, 0.45), (0.5, 0.65)]
    cube_res = 12 if dim == 2 else 6
    steps = 15
    r = solver("--dim", dim, "--steps", steps, "--cubes", 2, "--cube-res", cube_res,
               "--cube0-x", cubes[0][0], "--cube0-y", cubes[0][1], "--cube1-x", cubes[1][0],
               "--cube1-y", cubes[1][1], "--material-model", material, "--dump", "--out", tmp_path)
    assert r.returncode == 0, r.stderr
    res = dumpio.load(str(tmp_path / "dump.nclr"))
    assert sorted(res, key=lambda k: int(k[:-1])) == [f"{s}_" for s in range(steps)]
    ref = api_states(dim, model, cubes, cube_res, steps)
    N = 65
    for s, (p, g) in enumerate(ref):
        got = res[f"{s}_"]
        for f in FIELDS:
            a = getattr(got, f).astype(np.float32)
            if s == 0:
                assert np.array_equal(a, p[f]), (s, f)
            else:  # FP32 atomic sums in both runs: equal up to their order
                assert field_err(a, p[f], f) <= DRIFT[f], (s, f)
        if s == 0:
            assert not got.mass.any() and not got.velocity.any()
        else:
            assert got.mass.shape == (N,) * dim
            assert field_err(got.mass.reshape(-1).astype(np.float32), g.mass, "grid_m") <= 1e-4
            assert field_err(got.velocity.reshape(-1, dim).astype(np.float32), g.velocity,
                             "grid_v") <= DRIFT["v"]
        mu, lam = got.lame[0]
        e = 10.0 if model == scenes.SNOW else 0.3
        sim_mu, sim_lam = 1000.0 / (2 * 1.3), 1000.0 * 0.3 / (1.3 * 0.4)
        assert math.isclose(mu, sim_mu * e, rel_tol=1e-6) and math.isclose(lam, sim_lam * e, rel_tol=1e-6)
        expected_ts = np.float32(1e-4) * np.float32(s) if s > 0 else np.float32(1e-4)
        assert got.timestep[0] == expected_ts


def test_neohookean_dump_equals_the_api_run(tmp_path):
    """--stress neohookean (3D, --physics corrected) steps as the API with the same options."""
    steps, cube_res = 10, 6
    r = solver("--dim", 3, "--steps", steps, "--cube-res", cube_res, "--cube0-x", 0.4,
               "--cube0-y", 0.55, "--material-model", "jelly", "--physics", "corrected",
               "--stress", "neohookean", "--dump", "--out", tmp_path)
    assert r.returncode == 0, r.stderr
    res = dumpio.load(str(tmp_path / "dump.nclr"))
    ref = api_states(3, scenes.JELLY, [(0.4, 0.55)], cube_res, steps,
                     physics=scenes.CORRECTED, stress_model=capi.STRESS_NEOHOOKEAN)
    for s, (p, _) in enumerate(ref):
        for f in FIELDS:
            assert field_err(getattr(res[f"{s}_"], f).astype(np.float32), p[f], f) <= DRIFT[f], (s, f)
    bad = solver("--stress", "hookean", "--cube0-x", 0.4, "--cube0-y", 0.6, "--steps", 1,
                 "--out", tmp_path)
    assert bad.returncode != 0 and "Invalid Option" in bad.stderr


def test_missing_cube_coordinates_is_an_error(tmp_path):
    r = solver("--cubes", 2, "--cube0-x", 0.3, "--cube0-y", 0.4, "--steps", 1, "--out", tmp_path)
    assert r.returncode != 0
    assert "Cube: 1 is missing coordinates" in r.stderr


def test_frames_are_written(tmp_path):
    r = solver("--steps", 3, "--render", "--render-every", 1, "--cube0-x", 0.4, "--cube0-y", 0.6,
               "--out", tmp_path)
    assert r.returncode == 0, r.stderr
    frames = sorted(os.listdir(tmp_path / "frames"))
    assert frames == ["000000.ppm", "000001.ppm", "000002.ppm"]
    data = (tmp_path / "frames" / frames[0]).read_bytes()
    assert data.startswith(b"P6\n800 800\n255\n")
    rgb = np.frombuffer(data[len(b"P6\n800 800\n255\n"):], np.uint8).reshape(800, 800, 3)
    assert (rgb == [0xED, 0x55, 0x3B]).all(axis=2).sum() > 0  # particles drawn


def render_reference(x, w, h, radius, color):
    """The renderer's rules restated in plain FP32 (painter's order)."""
    f = np.float32
    winner = -np.ones(w * h, np.int64)
    r = math.ceil(radius)
    r2 = f(radius) * f(radius)
    for p in range(len(x)):
        px, py = f(x[p, 0]) * f(w), (f(1.0) - f(x[p, 1])) * f(h)
        ci, cj = math.floor(px), math.floor(py)
        for j in range(cj - r, cj + r + 1):
            if j < 0 or j >= h:
                continue
            for i in range(ci - r, ci + r + 1):
                if i < 0 or i >= w:
                    continue
                dx, dy = f(i) + f(0.5) - px, f(j) + f(0.5) - py
                if dx * dx + dy * dy <= r2:
                    winner[j * w + i] = p
    jj, ii = np.divmod(np.arange(w * h), w)
    cx, cy = ii.astype(f) + f(0.5), jj.astype(f) + f(0.5)
    x0, x1, y0, y1 = f(0.04) * f(w), f(0.96) * f(w), f(0.04) * f(h), f(0.96) * f(h)
    rr = f(radius)
    in_x = (cx >= x0 - rr) & (cx <= x1 + rr)
    in_y = (cy >= y0 - rr) & (cy <= y1 + rr)
    near_v = (np.abs(cx - x0) <= rr) | (np.abs(cx - x1) <= rr)
    near_h = (np.abs(cy - y0) <= rr) | (np.abs(cy - y1) <= rr)
    img = np.where((near_v & in_y) | (near_h & in_x), 0x4FB99F, 0x112F41).astype(np.uint32)
    img[winner >= 0] = color
    return img


@pytest.mark.parametrize("dim", [2, 3])
def test_render_matches_restatement(dim):
    rng = np.random.default_rng(6)
    x = rng.uniform(-0.02, 1.02, size=(400, dim)).astype(np.float32)
    w, h, radius = 160, 120, 2.0
    xd = torch.tensor(x, device="cuda")
    img = torch.empty(w * h, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    capi.check(capi.lib().nclr_render_device(ctypes.c_void_p(xd.data_ptr()), len(x), dim, None,
                                             0xED553B, w, h, radius,
                                             ctypes.c_void_p(img.data_ptr()), ctypes.c_void_p(st)))
    torch.cuda.synchronize()
    got = img.cpu().numpy().view(np.uint32)
    assert np.array_equal(got, render_reference(x, w, h, radius, 0xED553B))
