"""The FP64 CPU adjoint of a jelly rollout (oracle/nclr_adjoint.h) against FP64 central finite
differences.  Loss 1 = |centre of mass of the final positions - target|^2 (gradients with
respect to initial velocities, positions and deformation gradients); internal forces conserve
momentum, so away from the boundary this loss does not depend on the material and its E / nu
gradients vanish -- loss 2 = sum_p m_p |x_p - target_p|^2 over the final positions depends on
the deformation and checks the Young's modulus and Poisson ratio gradients.  Both stress
models: the reference's fixed-corotated one and the neo-Hookean extension (3D under the
corrected physics only: the reference's diag<3>(1) = diag(1,1,0) leaves det F near 0)."""
import numpy as np
import pytest

from nuclearmpm_gb300 import scenes

CASES = [(2, 32, 50, 1024), (3, 16, 10, 216)]  # dim, res, steps, particles
COROTATED, NEOHOOKEAN = 0, 1


def setup(dim, res, n, physics, seed=0):
    rng = np.random.default_rng(seed)
    side = round(n ** (1 / dim))
    x = scenes.jittered_block(rng, (side,) * dim, 0.5 / res, (0.35,) * dim, 0.25 / res)
    s = scenes.particles(x.astype(np.float64), rng.normal(0, 0.5, size=x.shape), physics=physics)
    s = {k: np.asarray(v, np.float64) for k, v in s.items()}
    s["F"] = s["F"] + rng.normal(0, 0.01, size=s["F"].shape)
    target = rng.uniform(0.4, 0.6, size=dim)
    return s, target


def loss_and_seed(xT, mass, target):
    com = (xT * mass[:, None]).sum(0) / mass.sum()
    d = com - target
    return float(d @ d), (2 * d[None, :] * mass[:, None] / mass.sum())


def pointwise(xT, mass, targets):
    d = xT - targets
    return float((mass[:, None] * d * d).sum()), 2 * mass[:, None] * d


def forward_loss(oracle, s, target, dim, res, steps, physics, E=1e4, nu=0.2, loss=loss_and_seed,
                 stress=COROTATED):
    out, _, st, _ = oracle.advance(s, dim=dim, model=scenes.JELLY, res=res, steps=steps, fp64=True,
                                   physics=physics, E=E, nu=nu, want_grid=False, stress=stress)
    assert st == 0
    return loss(out["x"], s["mass"], target)[0]


@pytest.mark.parametrize("dim,res,steps,n", CASES)
@pytest.mark.parametrize("physics", [scenes.REFERENCE, scenes.CORRECTED])
@pytest.mark.parametrize("stress", [COROTATED, NEOHOOKEAN])
def test_oracle_adjoint_matches_finite_differences(oracle, dim, res, steps, n, physics, stress):
    if stress == NEOHOOKEAN and dim == 3 and physics == scenes.REFERENCE:
        pytest.skip("the neo-Hookean stress needs det F > 0")
    s, target = setup(dim, res, n, physics)
    kw = dict(dim=dim, res=res, steps=steps, physics=physics, stress=stress)
    out, _ = oracle.adjoint(s, seed={}, **kw)
    _, seed = loss_and_seed(out["x"], s["mass"], target)
    _, g = oracle.adjoint(s, seed={"x": seed}, **kw)
    rng = np.random.default_rng(1)
    checks = []
    for _ in range(4):
        p, d = int(rng.integers(n)), int(rng.integers(dim))
        checks.append(("v", (p, d), 1e-5))
        checks.append(("x", (p, d), 1e-7))
    checks.append(("F", (int(rng.integers(n)), 0, 1), 1e-6))
    for field, idx, h in checks:
        sp = {k: v.copy() for k, v in s.items()}
        sm = {k: v.copy() for k, v in s.items()}
        sp[field][idx] += h
        sm[field][idx] -= h
        fd = (forward_loss(oracle, sp, target, dim, res, steps, physics, stress=stress) -
              forward_loss(oracle, sm, target, dim, res, steps, physics, stress=stress)) / (2 * h)
        ad = g[field][idx]
        assert abs(ad - fd) <= 1e-6 * max(1.0, abs(fd)) + 1e-4 * abs(fd), (field, idx, ad, fd)
    assert abs(g["E"]) < 1e-15 and abs(g["nu"]) < 1e-12  # momentum conservation
    targets = out["x"] + np.random.default_rng(2).normal(0, 1e-3, size=out["x"].shape)
    _, seed2 = pointwise(out["x"], s["mass"], targets)
    _, g2 = oracle.adjoint(s, seed={"x": seed2}, **kw)
    for name, h in (("E", 1.0), ("nu", 1e-5)):
        kp = {"E": 1e4, "nu": 0.2}
        km = dict(kp)
        kp[name] += h
        km[name] -= h
        fd = (forward_loss(oracle, s, targets, dim, res, steps, physics, loss=pointwise,
                           stress=stress, **kp) -
              forward_loss(oracle, s, targets, dim, res, steps, physics, loss=pointwise,
                           stress=stress, **km)) / (2 * h)
        assert abs(fd) > 0
        assert abs(g2[name] - fd) <= 1e-4 * abs(fd), (name, g2[name], fd)


@pytest.mark.parametrize("stress", [COROTATED, NEOHOOKEAN])
def test_oracle_per_particle_moduli_adjoint_matches_finite_differences(oracle, stress):
    """Every particle with its own E and nu (the nclr_set_moduli extension): each particle's E
    and nu adjoints of a deformation-dependent loss against FP64 central differences."""
    dim, res, steps, n = 2, 32, 30, 1024
    s, _ = setup(dim, res, n, scenes.REFERENCE)
    rng = np.random.default_rng(4)
    Ep = np.exp(rng.uniform(np.log(1e3), np.log(1e4), size=n))
    nup = rng.uniform(0.15, 0.35, size=n)
    kw = dict(dim=dim, res=res, steps=steps, physics=scenes.REFERENCE, stress=stress)
    out, _ = oracle.adjoint(s, seed={}, E_particles=Ep, nu_particles=nup, **kw)
    targets = out["x"] + rng.normal(0, 1e-3, size=out["x"].shape)
    _, seed = pointwise(out["x"], s["mass"], targets)
    _, g = oracle.adjoint(s, seed={"x": seed}, E_particles=Ep, nu_particles=nup, **kw)
    assert g["E"].shape == (n,) and g["nu"].shape == (n,)

    def loss(E_, nu_):
        o, _, st, _ = oracle.advance(s, dim=dim, model=scenes.JELLY, res=res, steps=steps,
                                     fp64=True, physics=scenes.REFERENCE, stress=stress,
                                     want_grid=False, E_particles=E_, nu_particles=nu_)
        assert st == 0
        return pointwise(o["x"], s["mass"], targets)[0]

    for p in rng.choice(n, size=3, replace=False):
        for name, arr, h in (("E", Ep, 1e-2 * Ep[p]), ("nu", nup, 1e-5)):
            plus, minus = arr.copy(), arr.copy()
            plus[p] += h
            minus[p] -= h
            args = (plus, nup) if name == "E" else (Ep, plus)
            argm = (minus, nup) if name == "E" else (Ep, minus)
            fd = (loss(*args) - loss(*argm)) / (2 * h)
            scale = np.abs(g[name]).max()
            assert abs(g[name][p] - fd) <= 1e-4 * abs(fd) + 1e-6 * scale, (name, p, g[name][p], fd)


PLASTIC_CASES = [(2, 32, 30, 1024), (3, 16, 8, 216)]  # dim, res, steps, particles


def plastic_setup(dim, res, n, physics, model, seed=0):
    """A jittered block whose F already sits near the plastic limits: snow with singular values
    scattered across the clamp bounds and Jp away from its own bounds, liquid with a perturbed
    F (the reset keeps only det F)."""
    s, target = setup(dim, res, n, physics, seed)
    rng = np.random.default_rng(seed + 7)
    s["F"] = s["F"] + rng.normal(0, 0.02, size=s["F"].shape)
    s["Jp"] = rng.uniform(0.9, 1.1, size=n)
    return s, target


@pytest.mark.parametrize("dim,res,steps,n", PLASTIC_CASES)
@pytest.mark.parametrize("physics", [scenes.REFERENCE, scenes.CORRECTED])
@pytest.mark.parametrize("model", [scenes.SNOW, scenes.LIQUID])
def test_oracle_plastic_adjoint_matches_finite_differences(oracle, dim, res, steps, n, physics,
                                                           model):
    """The adjoint through the snow clamp (SVD backward with the clamped singular values'
    gradients masked, the Jp update, the Jp-dependent hardening) and through the liquid reset,
    against FP64 central differences: initial velocities, positions, F and Jp with a
    deformation-dependent loss, and E and nu."""
    if dim == 3 and physics == scenes.REFERENCE and model == scenes.LIQUID:
        pytest.skip("3D liquid under the reference physics resets F to diag(J, 1, 0), whose "
                    "polar rotation is not unique: the step is not differentiable there")
    s, _ = plastic_setup(dim, res, n, physics, model)
    kw = dict(dim=dim, res=res, steps=steps, physics=physics, model=model)
    out, _ = oracle.adjoint(s, seed={}, **kw)
    targets = out["x"] + np.random.default_rng(2).normal(0, 1e-3, size=out["x"].shape)
    _, seed = pointwise(out["x"], s["mass"], targets)
    _, g = oracle.adjoint(s, seed={"x": seed}, **kw)

    def loss(st, E=1e4, nu=0.2):
        o, _, status, _ = oracle.advance(st, dim=dim, model=model, res=res, steps=steps,
                                         fp64=True, physics=physics, E=E, nu=nu,
                                         want_grid=False)
        assert status == 0
        return pointwise(o["x"], s["mass"], targets)[0]

    rng = np.random.default_rng(1)
    checks = []
    for _ in range(3):
        p, d = int(rng.integers(n)), int(rng.integers(dim))
        checks += [("v", (p, d), 1e-6), ("x", (p, d), 1e-8)]
    checks += [("F", (int(rng.integers(n)), 0, 1), 1e-7), ("Jp", (int(rng.integers(n)),), 1e-7)]
    scale = max(np.abs(g["v"]).max(), np.abs(g["x"]).max())
    for field, idx, h in checks:
        sp = {k: v.copy() for k, v in s.items()}
        sm = {k: v.copy() for k, v in s.items()}
        sp[field][idx] += h
        sm[field][idx] -= h
        fd = (loss(sp) - loss(sm)) / (2 * h)
        ad = g[field][idx]
        assert abs(ad - fd) <= 1e-4 * abs(fd) + 1e-7 * scale, (field, idx, ad, fd)
    # steps small enough that no particle's clamp switches inside +-h (the loss is piecewise
    # smooth: larger steps cross those kinks and the central difference stops converging)
    for name, h in (("E", 1e-2), ("nu", 1e-7)):
        kp = {"E": 1e4, "nu": 0.2}
        km = dict(kp)
        kp[name] += h
        km[name] -= h
        fd = (loss(s, **kp) - loss(s, **km)) / (2 * h)
        assert abs(g[name] - fd) <= 1e-4 * abs(fd) + 1e-12, (name, g[name], fd)
