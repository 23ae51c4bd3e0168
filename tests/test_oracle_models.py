"""The oracle's extensions of the reference's model (CPU): per-particle Young's modulus and
Poisson ratio, and the neo-Hookean stress that src/nclr.h:339 leaves as a TODO.

  * The stress of one particle is read back from its one-step grid: with v = C = 0 and no
    gravity, node i gets velocity A dpos_i / m, so A follows from a least-squares solve over
    the stencil. For the neo-Hookean model it must equal -(dt vol 4 inv_dx^2) tau, where
    tau = (dpsi/dF) F^T. dpsi/dF is taken by FP64 central differences of the energy
    psi = mu/2 (tr F^T F - d) - mu ln J + lambda/2 ln^2 J, with mu and lambda the hardened
    moduli of the scene's or the particle's own E and nu.
  * Per-particle moduli all equal to the simulation's pair reproduce the plain step bit for
    bit.
  * Two particle groups far apart, each with its own moduli, step exactly like two separate
    simulations.
"""
import numpy as np
import pytest

from conftest import FIELDS, random_state
from nuclearmpm_gb300 import scenes

COROTATED, NEOHOOKEAN = 0, 1


def lame(E, nu):
    return E / (2 * (1 + nu)), E * nu / ((1 + nu) * (1 - 2 * nu))


def neohookean_energy(F, mu, lam):
    J = np.linalg.det(F)
    return 0.5 * mu * (np.trace(F.T @ F) - F.shape[0]) - mu * np.log(J) + 0.5 * lam * np.log(J) ** 2


def energy_gradient(F, mu, lam, h=1e-6):
    P = np.zeros_like(F)
    for i in range(F.shape[0]):
        for j in range(F.shape[1]):
            Fp, Fm = F.copy(), F.copy()
            Fp[i, j] += h
            Fm[i, j] -= h
            P[i, j] = (neohookean_energy(Fp, mu, lam) - neohookean_energy(Fm, mu, lam)) / (2 * h)
    return P


def affine_from_grid(x, grid_v, grid_m, res, m):
    """A of a lone particle at x from its one-step grid (v = C = 0, no gravity)."""
    dim = x.size
    N = res + 1
    inv_dx = float(res)
    base = np.trunc(x * inv_dx - 0.5).astype(int)
    fx = x * inv_dx - base
    rows, vals = [], []
    for o in np.ndindex(*(3,) * dim):
        node = base + np.array(o)
        f = node[0] * N + node[1] if dim == 2 else (node[0] * N + node[1]) * N + node[2]
        assert grid_m[f] > 0
        rows.append((np.array(o) - fx) / inv_dx)
        vals.append(grid_v[f] * m)
    At, *_ = np.linalg.lstsq(np.array(rows), np.array(vals), rcond=None)
    return At.T


@pytest.mark.parametrize("dim,physics", [(2, scenes.REFERENCE), (2, scenes.CORRECTED),
                                         (3, scenes.CORRECTED)])
@pytest.mark.parametrize("model,hardening", [(scenes.JELLY, 0.3), (scenes.LIQUID, 1.0),
                                             (scenes.SNOW, 1.0)])
@pytest.mark.parametrize("own_moduli", [False, True])
def test_neohookean_stress_is_the_energy_gradient(oracle, dim, physics, model, hardening,
                                                  own_moduli):
    rng = np.random.default_rng(7 * dim + model)
    res, dt, m, vol = 16, 1e-4, 1.3, 0.7
    E, nu = 1e4, 0.2
    x = np.full((1, dim), 0.5) + rng.uniform(0, 1.0 / res, size=(1, dim))
    F = np.eye(dim) + rng.normal(0, 0.1, size=(dim, dim))
    assert np.linalg.det(F) > 0
    s = {"x": x, "v": np.zeros((1, dim)), "F": F[None], "C": np.zeros((1, dim, dim)),
         "Jp": np.ones(1), "mass": np.full(1, m), "volume": np.full(1, vol)}
    kw = {}
    if own_moduli:
        E, nu = 3.7e3, 0.33
        kw = dict(E_particles=[E], nu_particles=[nu])
    _, (gv, gm), st, _ = oracle.advance(s, dim=dim, model=model, res=res, dt=dt, gravity=0.0,
                                        fp64=True, physics=physics, stress=NEOHOOKEAN, **kw)
    assert st == 0
    A = affine_from_grid(x[0], gv, gm, res, m)
    mu, lam = (hardening * v for v in lame(E, nu))
    tau = energy_gradient(F, mu, lam) @ F.T
    expect = -(dt * vol * 4 * res * res) * tau
    assert np.abs(A - expect).max() <= 1e-6 * np.abs(expect).max(), (A, expect)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("stress", [COROTATED, NEOHOOKEAN])
def test_uniform_per_particle_moduli_match_the_scene_pair(oracle, dim, stress):
    physics = scenes.CORRECTED
    rng = np.random.default_rng(dim)
    n = 600
    s = random_state(rng, dim, n, 32, physics)
    mat = rng.integers(0, 3, size=n).astype(np.uint8)
    kw = dict(dim=dim, model=scenes.JELLY, res=32, E=2.5e3, nu=0.27, steps=3, physics=physics,
              material=mat, stress=stress)
    a, ga, sa, _ = oracle.advance(s, **kw)
    b, gb, sb, _ = oracle.advance(s, E_particles=np.full(n, 2.5e3), nu_particles=np.full(n, 0.27),
                                  **kw)
    assert sa == sb == 0
    for f in FIELDS:
        np.testing.assert_array_equal(a[f], b[f])
    np.testing.assert_array_equal(ga[0], gb[0])
    np.testing.assert_array_equal(ga[1], gb[1])


@pytest.mark.parametrize("stress", [COROTATED, NEOHOOKEAN])
def test_groups_with_their_own_moduli_step_like_separate_simulations(oracle, stress):
    dim, res, physics = 2, 64, scenes.REFERENCE
    rng = np.random.default_rng(11)
    left = random_state(rng, dim, 300, res, physics)
    right = random_state(rng, dim, 300, res, physics)
    left["x"] = (0.1 + 0.3 * (left["x"] - 0.3)).astype(np.float32)   # x in [0.1, 0.22]
    right["x"] = (0.7 + 0.3 * (right["x"] - 0.3)).astype(np.float32)  # x in [0.7, 0.82]
    both = scenes.concat(left, right)
    kw = dict(dim=dim, model=scenes.SNOW, res=res, steps=4, physics=physics, stress=stress,
              want_grid=False)
    Ep = np.r_[np.full(300, 2e3), np.full(300, 4e4)]
    nup = np.r_[np.full(300, 0.15), np.full(300, 0.35)]
    out, _, st, _ = oracle.advance(both, E_particles=Ep, nu_particles=nup, **kw)
    a, _, sa, _ = oracle.advance(left, E=2e3, nu=0.15, **kw)
    b, _, sb, _ = oracle.advance(right, E=4e4, nu=0.35, **kw)
    assert st == sa == sb == 0
    for f in FIELDS:
        np.testing.assert_array_equal(out[f][:300], a[f])
        np.testing.assert_array_equal(out[f][300:], b[f])
