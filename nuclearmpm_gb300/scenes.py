"""Scene builders: the reference's cube<dim>() lattice and the benchmark scenes.

Host-side input generation (numpy, float32).  `cube` follows src/nclr_math.h:100-129 (Eigen
3.4 LinSpaced per axis, x outermost); `readme_scene` is the two-cube snow scene of
src/example.cpp:29-42.  The 3D and batched scenes are seeded synthetic inputs with the
shapes, sizes and distributions of the benchmark configurations (numpy PCG64 streams).

A scene is a dict of host arrays in the C ABI layout (particle-major, row-major matrices):
x (n, dim), v (n, dim), F (n, dim, dim), C (n, dim, dim), Jp (n,), mass (n,), volume (n,).
"""
from __future__ import annotations

import numpy as np

SNOW, JELLY, LIQUID = 0, 1, 2
REFERENCE, CORRECTED = 0, 1


def linspaced(n: int, lo: float, hi: float) -> np.ndarray:
    """Eigen 3.4 LinSpaced(n, lo, hi) in float32 (src/nclr_math.h:103)."""
    lo32, hi32 = np.float32(lo), np.float32(hi)
    if n == 1:
        return np.array([hi32], dtype=np.float32)
    step = np.float32((hi32 - lo32) / np.float32(n - 1))
    i = np.arange(n, dtype=np.float32)
    if abs(hi32) < abs(lo32):
        out = (hi32 - (np.float32(n - 1) - i) * step).astype(np.float32)
        out[0] = lo32
    else:
        out = (lo32 + i * step).astype(np.float32)
        out[-1] = hi32
    return out


def cube(dim: int, n: int, lo: float, hi: float) -> np.ndarray:
    """cube<dim>(n, lo, hi): an n^dim lattice over [lo, hi]^dim, x outermost (nclr_math.h:100-129)."""
    ax = linspaced(n, lo, hi)
    grids = np.meshgrid(*([ax] * dim), indexing="ij")
    return np.stack([g.reshape(-1) for g in grids], axis=1).astype(np.float32)


def cubes_device(dim: int, res: int, los, his, device: int = 0):
    """ncubes lattices cube<dim>(res, lo[c], hi[c]) built on the GPU (nclr_cubes_device), one
    after another: the headless solver's generate_cubes (src/solver.cpp:133-149) without a
    host round trip.  Returns a CUDA tensor (ncubes * res^dim, dim), bit-equal to `cube`."""
    import ctypes

    import torch

    from . import capi
    los = np.ascontiguousarray(np.atleast_1d(los), dtype=np.float32)
    his = np.ascontiguousarray(np.atleast_1d(his), dtype=np.float32)
    if los.shape != his.shape:
        raise ValueError("one (lo, hi) pair per cube")
    out = torch.empty((len(los) * res ** dim, dim), dtype=torch.float32,
                      device=torch.device("cuda", device))
    with torch.cuda.device(device):
        stream = torch.cuda.current_stream().cuda_stream
        capi.check(capi.lib().nclr_cubes_device(dim, len(los), res,
                                                los.ctypes.data_as(ctypes.c_void_p),
                                                his.ctypes.data_as(ctypes.c_void_p),
                                                ctypes.c_void_p(out.data_ptr()),
                                                ctypes.c_void_p(stream)), None)
    return out


def initial_identity(dim: int, physics: int = REFERENCE) -> np.ndarray:
    """Particle<dim>'s initial F = diag<dim>(1) (src/nclr.h:47): diag(1,1,0) in 3D for the
    reference physics (src/nclr_math.h:13-19), the true identity for the corrected physics."""
    I = np.eye(dim, dtype=np.float32)
    if dim == 3 and physics == REFERENCE:
        I[2, 2] = 0.0
    return I


def particles(x: np.ndarray, v: np.ndarray | None = None, *, physics: int = REFERENCE,
              mass: float = 1.0, volume: float = 1.0) -> dict:
    """Particle<dim>(x, c, v=0, mass=1, volume=1) for every row of x (src/nclr.h:46-47)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    n, dim = x.shape
    v = np.zeros_like(x) if v is None else np.ascontiguousarray(v, dtype=np.float32)
    return {
        "x": x, "v": v,
        "F": np.broadcast_to(initial_identity(dim, physics), (n, dim, dim)).copy(),
        "C": np.zeros((n, dim, dim), dtype=np.float32),
        "Jp": np.ones(n, dtype=np.float32),
        "mass": np.full(n, mass, dtype=np.float32),
        "volume": np.full(n, volume, dtype=np.float32),
    }


def concat(*scenes: dict) -> dict:
    return {k: np.concatenate([s[k] for s in scenes]) for k in scenes[0]}


def readme_scene(physics: int = REFERENCE) -> dict:
    """The README / example.cpp scene: two cube<2>(50, 0.4, 0.6) lattices, the second moved
    down by 0.35 in y, zero velocity (src/example.cpp:29-42); 5,000 particles."""
    a = cube(2, 50, 0.4, 0.6)
    b = cube(2, 50, 0.4, 0.6)
    b[:, 1] = (b[:, 1] - np.float32(0.35)).astype(np.float32)
    return particles(np.concatenate([a, b]), physics=physics)


def jittered_block(rng, shape, spacing, origin, jitter):
    """A lattice of `shape` points with `spacing`, corner at `origin`, uniform jitter of
    +-`jitter` per axis."""
    dim = len(shape)
    idx = np.stack(np.meshgrid(*[np.arange(s) for s in shape], indexing="ij"), -1).reshape(-1, dim)
    x = np.asarray(origin, dtype=np.float64) + (idx + 0.5) * spacing
    x += rng.uniform(-jitter, jitter, size=x.shape)
    return x.astype(np.float32)


def jelly_cubes_3d(seed: int = 0, res: int = 128, cubes: int = 4, side: int = 64,
                   physics: int = REFERENCE) -> dict:
    """3D jelly: `cubes` lattices of side^3 particles at spacing dx/2 (edge side*dx/2),
    centres uniform in [0.25, 0.75]^3, jitter +-0.25 cell, per-cube velocity N(0, 0.5^2) per
    axis.  Defaults: 128^3 grid, 4 x 64^3 = 1,048,576 particles."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / res
    spacing = 0.5 * dx
    edge = side * spacing
    parts = []
    for _ in range(cubes):
        centre = rng.uniform(0.25, 0.75, size=3)
        x = jittered_block(rng, (side,) * 3, spacing, centre - edge / 2, 0.25 * dx)
        v = np.broadcast_to(rng.normal(0.0, 0.5, size=3).astype(np.float32), x.shape)
        parts.append(particles(x, v, physics=physics))
    return concat(*parts)


def liquid_snow_boxes_3d(seed: int = 0, res: int = 256, boxes: int = 16,
                         total: int = 4_194_304, physics: int = REFERENCE, margin: float = 0.05):
    """3D mixed liquid + snow: `boxes` axis-aligned boxes with sides uniform in [0.05, 0.2]
    in the upper half of the domain, at least `margin` from the walls, filled with jittered
    lattices whose common spacing makes the particle count `total` (the largest boxes are
    trimmed to hit it exactly); half the boxes liquid, half snow, shuffled.  Returns (scene,
    material per particle).  (A box reaching into the 3-node sticky border, where the
    boundary rule tests the sign of an exactly-zero velocity component, makes the step
    discontinuous in its input: keep `margin` above (3 + 2) / res.)"""
    rng = np.random.default_rng(seed)
    dx = 1.0 / res
    sides = rng.uniform(0.05, 0.2, size=(boxes, 3))
    hi = 1.0 - margin
    lo = np.column_stack([rng.uniform(margin, hi - sides[:, 0]),
                          rng.uniform(0.5, hi - sides[:, 1]),
                          rng.uniform(margin, hi - sides[:, 2])])
    vol = np.prod(sides, axis=1).sum()
    spacing = (vol / total) ** (1.0 / 3.0)
    counts = [np.maximum(1, np.round(s / spacing)).astype(int) for s in sides]
    mats = np.array([LIQUID] * (boxes // 2) + [SNOW] * (boxes - boxes // 2))
    rng.shuffle(mats)
    xs, ms = [], []
    for b in range(boxes):
        x = jittered_block(rng, tuple(counts[b]), spacing, lo[b], 0.25 * min(spacing, dx))
        xs.append(x)
        ms.append(np.full(len(x), mats[b], dtype=np.int32))
    x = np.concatenate(xs)
    m = np.concatenate(ms)
    if len(x) >= total:
        keep = np.sort(rng.permutation(len(x))[:total])
        x, m = x[keep], m[keep]
    else:
        extra = rng.integers(0, len(x), size=total - len(x))
        x = np.concatenate([x, x[extra] + rng.uniform(-0.1, 0.1, (len(extra), 3)).astype(np.float32) * spacing])
        m = np.concatenate([m, m[extra]])
    return particles(x, physics=physics), m


def jelly_block_3d(seed: int = 0, res: int = 64, shape=(64, 64, 32),
                   physics: int = REFERENCE) -> dict:
    """One jittered 3D jelly lattice of prod(shape) particles at spacing dx/2, centred."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / res
    spacing = 0.5 * dx
    edge = np.array(shape) * spacing
    x = jittered_block(rng, shape, spacing, 0.5 - edge / 2, 0.25 * dx)
    return particles(x, physics=physics)


def random_scene_2d(rng, n: int, res: int, physics: int = REFERENCE) -> dict:
    """1-3 jittered 2D cubes holding n particles in total, placed inside the sticky border."""
    dx = 1.0 / res
    ncubes = int(rng.integers(1, 4))
    split = np.diff(np.round(np.linspace(0, n, ncubes + 1)).astype(int))
    xs = []
    for k in split:
        side = int(np.ceil(np.sqrt(k)))
        spacing = 0.5 * dx
        edge = side * spacing
        edge_max = 0.7
        if edge > edge_max:
            spacing = edge_max / side
            edge = edge_max
        lo = rng.uniform(0.1, max(0.1, 0.9 - edge), size=2)
        x = jittered_block(rng, (side, side), spacing, lo, 0.25 * spacing)[:k]
        xs.append(x)
    return particles(np.concatenate(xs), physics=physics)


def batched_scenes_2d(seed: int = 0, count: int = 256, n_min: int = 1000, n_max: int = 65536,
                      physics: int = REFERENCE) -> list:
    """Independent 2D scenes for the batched form: per scene a particle count log-uniform in
    [n_min, n_max], grid resolution from {64, 128, 256}, material uniform over {liquid, snow,
    jelly}, Young's modulus log-uniform in [1e3, 1e5], Poisson ratio uniform in [0.1, 0.4],
    1-3 jittered cubes; dt = 1e-4."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        res = int(rng.choice([64, 128, 256]))
        model = int(rng.choice([LIQUID, SNOW, JELLY]))
        E = float(np.exp(rng.uniform(np.log(1e3), np.log(1e5))))
        nu = float(rng.uniform(0.1, 0.4))
        sc = random_scene_2d(rng, n, res, physics=physics)
        sc.update(model=model, res=res, E=E, nu=nu, dt=1e-4, gravity=-100.0)
        out.append(sc)
    return out
