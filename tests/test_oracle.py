"""CPU tests of the oracle: pinned to golden vectors produced by the reference's own step
code, and checked against the analytic invariants of the MLS-MPM step."""
import numpy as np
import pytest

from conftest import DRIFT, FIELDS, field_err, golden_names, load_golden, state_at
from nuclearmpm_gb300 import scenes

# Drift bound over 100 steps (oracle FP32 vs the reference's own FP32 run): the two differ
# only in SVD rounding, which the stress term amplifies (a 1-ulp change of F moves the next
# step's velocities by ~1e-4 of their scale).
ONE_STEP = {"x": 1e-5, "v": 3e-5, "F": 1e-5, "C": 3e-5, "Jp": 1e-5}
DRIFT_100 = {"x": 1e-5, "v": 1e-3, "F": 1e-4, "C": 3e-3, "Jp": 1e-4}


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference_goldens(oracle, name):
    z, state, params, steps = load_golden(name)
    first = steps[0]
    out, grid, status, _ = oracle.advance(state, steps=first, **params)
    assert status == 0
    for f in FIELDS:  # first step from the scene: within 1e-5 relative (FP32 rounding)
        assert field_err(out[f], z[f"{f}@{first}"], f) <= 1e-5, f
    assert field_err(grid[0], z["grid_v"], "grid_v") <= 1e-5
    assert field_err(grid[1], z["grid_m"], "grid_m") <= 1e-6
    for k in steps[1:]:
        out, _, status, _ = oracle.advance(state, steps=k, **params)
        assert status == 0
        for f in FIELDS:
            assert field_err(out[f], z[f"{f}@{k}"], f) <= DRIFT_100[f], (k, f)


def test_drift_bound_follows_reference_fp32_drift(oracle):
    """The drift bound of the GPU tests (conftest.DRIFT) is derived from the reference's own
    FP32 drift: for every golden fixture's scene, the reference's own step (compiled from its
    sources, where the tree exists), the FP32 restatement and the FP64 oracle advance side by
    side, one step at a time, and the distance of each FP32 state to the FP64 one is taken
    after every step.  The largest of these per field must be the recorded REF_FP32_DRIFT (to
    2%), and DRIFT must be DRIFT_FACTOR times it, rounded up by at most a third.  Where the
    reference tree is absent, the FP32 restatement alone bounds it from below."""
    from conftest import DRIFT_FACTOR, REF_FP32_DRIFT
    worst = {f: 0.0 for f in FIELDS}
    have_ref = oracle.ref_available()
    for name in golden_names():
        z, state, params, steps = load_golden(name)
        keep = {"mass": state["mass"], "volume": state["volume"]}
        r, d, o = dict(state), dict(state), dict(state)
        for _ in range(steps[-1]):
            d, _, st64, _ = oracle.advance(d, steps=1, fp64=True, want_grid=False, **params)
            o, _, st32, _ = oracle.advance(o, steps=1, want_grid=False, **params)
            assert st64 == 0 and st32 == 0
            d, o = {**d, **keep}, {**o, **keep}
            if have_ref:
                r, _, st = oracle.ref_advance(r, steps=1, **params)
                assert st == 0
                r = {**r, **keep}
            for f in FIELDS:
                e = field_err(o[f], d[f], f)
                if have_ref:
                    e = max(e, field_err(r[f], d[f], f))
                worst[f] = max(worst[f], e)
    for f in FIELDS:
        if have_ref:
            assert abs(worst[f] - REF_FP32_DRIFT[f]) <= 0.02 * REF_FP32_DRIFT[f], (f, worst[f])
        else:
            assert worst[f] <= 1.02 * REF_FP32_DRIFT[f], (f, worst[f])
        assert DRIFT_FACTOR * REF_FP32_DRIFT[f] <= DRIFT[f] <= 1.34 * DRIFT_FACTOR * REF_FP32_DRIFT[f], f


@pytest.mark.parametrize("name", ["readme_snow", "block3d_snow", "block3d_jelly"])
def test_oracle_one_step_from_reference_state(oracle, name):
    """One step from the reference's own mid-run state: x, F, Jp within 1e-5; v and C
    within 3e-5, because they take the stress of the input F, whose 3D polar SVD rounding
    the stress term amplifies (the reference's own FP32 run is 4e-6 off FP64 there)."""
    z, _, params, steps = load_golden(name)
    a, b = steps[-2], steps[-1]
    assert b == a + 1
    out, _, status, _ = oracle.advance(state_at(z, a), steps=1, **params)
    assert status == 0
    for f in FIELDS:
        assert field_err(out[f], z[f"{f}@{b}"], f) <= ONE_STEP[f], f


@pytest.mark.parametrize("name", ["readme_jelly", "cli_cube_jelly", "block3d_liquid"])
def test_oracle_bit_exact_without_svd(oracle, name):
    """Where no SVD of a full-rank F is involved the restatement reproduces the reference's
    own arithmetic bit for bit (2D jelly uses the closed-form polar; 3D liquid in the
    reference physics resets F to a diagonal every step)."""
    z, state, params, steps = load_golden(name)
    for k in steps:
        out, _, _, _ = oracle.advance(state, steps=k, **params)
        for f in FIELDS:
            assert np.array_equal(out[f].astype(np.float32), z[f"{f}@{k}"]), (k, f)


def test_reference_shim_direct(oracle):
    """Oracle vs the reference's own code on a fresh random 3D case, where the tree exists."""
    if not oracle.ref_available():
        pytest.skip("reference tree not present on this machine")
    rng = np.random.default_rng(3)
    x = scenes.jittered_block(rng, (6, 6, 6), 1 / 64, (0.4, 0.5, 0.4), 0.25 / 32)
    s = scenes.particles(x, rng.normal(0, 0.3, size=x.shape).astype(np.float32))
    for model in (scenes.SNOW, scenes.JELLY, scenes.LIQUID):
        r, rg, st = oracle.ref_advance(s, dim=3, model=model, res=32, steps=1)
        o, og, st2, _ = oracle.advance(s, dim=3, model=model, res=32, steps=1)
        assert st == st2 == 0
        for f in FIELDS:
            assert field_err(o[f], r[f], f) <= 1e-5, (model, f)


def test_cube_matches_linspaced(oracle):
    for n, lo, hi in ((50, 0.4, 0.6), (25, 0.1, 0.9), (7, -0.3, 0.2), (1, 0.2, 0.5)):
        assert np.array_equal(scenes.linspaced(n, lo, hi), oracle.linspaced(n, lo, hi))
    if oracle.ref_available():
        for dim in (2, 3):
            assert np.array_equal(scenes.cube(dim, 13, 0.4, 0.6), oracle.ref_cube(dim, 13, 0.4, 0.6))


def _random_scene(rng, dim, n=300, res=32):
    lo = 0.3
    x = rng.uniform(lo, 1 - lo, size=(n, dim)).astype(np.float32)
    v = rng.normal(0, 0.3, size=(n, dim)).astype(np.float32)
    s = scenes.particles(x, v, physics=scenes.CORRECTED)
    s["F"] = (s["F"] + rng.normal(0, 0.02, size=s["F"].shape)).astype(np.float32)
    s["C"] = rng.normal(0, 1.0, size=s["C"].shape).astype(np.float32)
    s["mass"] = rng.uniform(0.5, 2.0, size=n).astype(np.float32)
    return s


@pytest.mark.parametrize("dim", [2, 3])
def test_p2g_conserves_mass_and_momentum(oracle, dim):
    """B-spline partition of unity: the grid's total mass equals the particles' mass and the
    grid's total momentum (before the update) equals sum(m v), since the affine term sums to
    zero over the stencil.  Checked with gravity 0 and a grid without boundary contact."""
    rng = np.random.default_rng(11 + dim)
    s = _random_scene(rng, dim)
    res = 32
    _, grid, status, _ = oracle.advance(s, dim=dim, model=scenes.JELLY, res=res, steps=1,
                                        gravity=0.0, fp64=True, physics=scenes.CORRECTED)
    assert status == 0
    gv, gm = grid
    assert abs(gm.sum() - s["mass"].astype(np.float64).sum()) < 1e-9 * gm.sum()
    mom = (gv * gm[:, None]).sum(0)
    ref = (s["v"].astype(np.float64) * s["mass"][:, None]).sum(0)
    assert np.allclose(mom, ref, rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("dim", [2, 3])
def test_g2p_reproduces_affine_field(oracle, dim):
    """sum w (x_i - x_p)(x_i - x_p)^T = dx^2/4 I, so G2P of a linear velocity field returns
    the field's value and gradient exactly: a particle cloud moving with v(x) = a + B x keeps
    v = a + B x_p and C = B after one step (FP64, gravity 0, massless stress)."""
    rng = np.random.default_rng(5)
    n, res = 200, 32
    x = rng.uniform(0.35, 0.65, size=(n, dim))
    a = rng.normal(0, 0.1, size=dim)
    B = rng.normal(0, 0.2, size=(dim, dim))
    s = scenes.particles(x.astype(np.float32), physics=scenes.CORRECTED)
    s["x"] = x
    s["v"] = a + x @ B.T
    s["C"] = np.broadcast_to(B, (n, dim, dim)).copy()
    # dense enough that every stencil node is covered: add a filler lattice with the field
    g = np.stack(np.meshgrid(*[np.linspace(0.3, 0.7, 52)] * dim, indexing="ij"), -1).reshape(-1, dim)
    if dim == 3:
        g = np.stack(np.meshgrid(*[np.linspace(0.32, 0.68, 24)] * dim, indexing="ij"), -1).reshape(-1, dim)
    fill = scenes.particles(g.astype(np.float32), physics=scenes.CORRECTED)
    fill["x"] = g
    fill["v"] = a + g @ B.T
    fill["C"] = np.broadcast_to(B, (len(g), dim, dim)).copy()
    allp = {k: np.concatenate([np.asarray(s[k], dtype=np.float64), np.asarray(fill[k], dtype=np.float64)]) for k in s}
    out, _, status, _ = oracle.advance(allp, dim=dim, model=scenes.JELLY, res=res, steps=1,
                                       gravity=0.0, E=0.0, fp64=True, physics=scenes.CORRECTED)
    assert status == 0
    xin = allp["x"][:n]
    assert np.allclose(out["v"][:n], a + xin @ B.T, atol=1e-10)
    assert np.allclose(out["C"][:n], np.broadcast_to(B, (n, dim, dim)), atol=1e-9)


def test_resting_particle_falls_with_gravity(oracle):
    s = scenes.particles(np.array([[0.5, 0.5]], dtype=np.float32), physics=scenes.CORRECTED)
    out, _, status, _ = oracle.advance(s, dim=2, model=scenes.JELLY, steps=1)
    assert status == 0
    assert np.allclose(out["v"][0], [0.0, 1e-4 * -100.0], atol=1e-9)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("physics", [0, 1])
def test_svd_and_polar(oracle, dim, physics):
    rng = np.random.default_rng(dim * 10 + physics)
    for trial in range(200):
        A = rng.normal(size=(dim, dim))
        if trial % 4 == 0:
            A = np.eye(dim) + 1e-4 * rng.normal(size=(dim, dim))  # near-repeated sigma
        U, S, V = oracle.svd(A, physics=physics, fp64=True)
        assert np.allclose(U @ np.diag(S) @ V.T, A, atol=1e-12)
        assert np.allclose(U.T @ U, np.eye(dim), atol=1e-12)
        assert np.allclose(V.T @ V, np.eye(dim), atol=1e-12)
        absS = np.abs(S)
        assert np.all(absS[:-1] >= absS[1:] - 1e-12)
        if dim == 3 or physics == 1:  # sign fix makes U and V rotations
            assert np.linalg.det(U) > 0 and np.linalg.det(V) > 0
        else:  # reference 2D: the out-of-range flips are dropped, sigma >= 0
            assert np.all(S >= 0)
        R = oracle.polar(A, physics=physics, fp64=True)
        assert np.allclose(R.T @ R, np.eye(dim), atol=1e-10)
        if np.linalg.det(A) > 0:
            assert abs(np.linalg.det(R) - 1) < 1e-10
            Sym = R.T @ A
            assert np.allclose(Sym, Sym.T, atol=1e-10)


def test_snow_clamp_keeps_invariants(oracle):
    z, state, params, _ = load_golden("readme_snow")
    out, _, status, _ = oracle.advance(state, steps=50, **params)
    assert status == 0
    assert np.all(out["Jp"] >= 0.6 - 1e-7) and np.all(out["Jp"] <= 20 + 1e-5)
    s = np.linalg.svd(out["F"], compute_uv=False)
    assert np.all(s >= 0.975 - 1e-5) and np.all(s <= 1.0045 + 1e-5)


def test_out_of_range_is_reported(oracle):
    """A particle whose stencil leaves the grid: the reference throws std::out_of_range from
    vector::at (src/nclr.h:163); the oracle reports status 2."""
    s = scenes.particles(np.array([[0.5, 0.5], [-0.2, 0.5]], dtype=np.float32))
    _, _, status, counters = oracle.advance(s, dim=2, model=scenes.JELLY, steps=1)
    assert status == 2 and counters[1] >= 1


@pytest.mark.parametrize("name", ["readme_snow", "block3d_jelly", "block3d_snow"])
def test_threaded_baseline_matches_serial_oracle(oracle, name):
    """The multi-threaded CPU baseline (oracle/nclr_oracle_mt.h: P2G over two colours of
    x-slabs, G2P and the grid update split by range) is the serial step up to the FP32
    summation order of the grid."""
    z, state, params, steps = load_golden(name)
    kw = dict(dim=params["dim"], model=params["model"], res=params["res"], dt=params["dt"],
              E=params["E"], nu=params["nu"], gravity=params["gravity"], steps=steps[0] + 4)
    a, ga, sa, _ = oracle.advance(state, **kw)
    b, gb, sb, _ = oracle.advance(state, threads=4, **kw)
    assert sa == sb == 0
    for f in FIELDS:  # summation order, amplified over the steps like any drift
        assert field_err(b[f], a[f], f) <= DRIFT[f], f
    assert field_err(gb[1], ga[1], "grid_m") <= 1e-4


def test_threaded_baseline_reports_out_of_range(oracle):
    s = scenes.particles(np.array([[0.5, 0.5], [-0.2, 0.5]] * 40, dtype=np.float32))
    _, _, status, counters = oracle.advance(s, dim=2, model=scenes.JELLY, steps=1, threads=3)
    assert status == 2 and counters[1] >= 1
