"""GPU adjoint of rollouts (nclr_rollout_* / nuclearmpm_gb300.autograd) against the FP64 CPU
adjoint of the oracle and FP64 finite differences of the oracle's forward step: jelly, and the
plastic materials (the snow clamp with its Jp update and Jp-dependent hardening, the liquid
reset).

Bounds: the GPU runs FP32 forward and FP32 adjoint kernels (FP64 only for the E / nu sums),
so its gradients sit within 1e-3 (normwise, relative to each field's largest entry) of the
FP64 adjoint, and directional derivatives within 1e-3 of central differences in FP64."""
import numpy as np
import pytest

from nuclearmpm_gb300 import scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GRAD_TOL = 1e-3


def setup(dim, res, n, physics, seed=0):
    rng = np.random.default_rng(seed)
    side = round(n ** (1 / dim))
    x = scenes.jittered_block(rng, (side,) * dim, 0.5 / res, (0.35,) * dim, 0.25 / res)
    s = scenes.particles(x, rng.normal(0, 0.5, size=x.shape).astype(np.float32), physics=physics)
    s["F"] = (s["F"] + rng.normal(0, 0.01, size=s["F"].shape)).astype(np.float32)
    return s


def gpu_grads(s, dim, res, steps, physics, every, seed_fn, E=1e4, nu=0.2, stress=0,
              model=scenes.JELLY):
    from nuclearmpm_gb300.autograd import Rollout
    roll = Rollout(s["x"], res=res, steps=steps, checkpoint_every=every, physics=physics,
                   stress_model=stress, model=model)
    dev = torch.device("cuda", 0)
    x0 = torch.tensor(s["x"], device=dev, requires_grad=True)
    v0 = torch.tensor(s["v"], device=dev, requires_grad=True)
    F0 = torch.tensor(s["F"], device=dev, requires_grad=True)
    C0 = torch.tensor(s["C"], device=dev, requires_grad=True)
    Et = torch.tensor(E, dtype=torch.float64, requires_grad=True)
    nut = torch.tensor(nu, dtype=torch.float64, requires_grad=True)
    xT, vT = roll(x0, v0, Et, nut, F0, C0)
    loss = seed_fn(xT)
    loss.backward()
    out = {"x": x0.grad.cpu().numpy(), "v": v0.grad.cpu().numpy(), "F": F0.grad.cpu().numpy(),
           "C": C0.grad.cpu().numpy(), "E": Et.grad.detach().cpu().numpy(),
           "nu": nut.grad.detach().cpu().numpy(),
           "xT": xT.detach().cpu().numpy(), "loss": float(loss.detach())}
    out["timing"] = roll.timing()
    roll.close()
    return out


def com_loss(target):
    t = torch.tensor(target, dtype=torch.float32, device="cuda")
    return lambda xT: ((xT.mean(0) - t) ** 2).sum()


def point_loss(targets):
    t = torch.tensor(targets, dtype=torch.float32, device="cuda")
    return lambda xT: ((xT - t) ** 2).sum()


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.mark.parametrize("dim,res,steps,n", [(2, 32, 50, 1024), (3, 16, 10, 512)])
@pytest.mark.parametrize("physics", [scenes.REFERENCE, scenes.CORRECTED])
@pytest.mark.parametrize("stress", [0, 1])  # fixed corotated, neo-Hookean
def test_gpu_adjoint_matches_fp64_adjoint(oracle, dim, res, steps, n, physics, stress):
    if stress == 1 and dim == 3 and physics == scenes.REFERENCE:
        pytest.skip("the neo-Hookean stress needs det F > 0")
    s = setup(dim, res, n, physics)
    rng = np.random.default_rng(3)
    kw = dict(dim=dim, res=res, steps=steps, physics=physics, stress=stress)
    # pointwise loss: depends on the deformation (E / nu gradients non-zero)
    fwd, _ = oracle.adjoint(s, seed={}, **kw)
    targets = (fwd["x"] + rng.normal(0, 1e-3, size=fwd["x"].shape)).astype(np.float32)
    g = gpu_grads(s, dim, res, steps, physics, every=7, seed_fn=point_loss(targets),
                  stress=stress)
    seed = 2 * (g["xT"].astype(np.float64) - targets)  # the GPU's own final state
    _, o = oracle.adjoint(s, seed={"x": seed}, **kw)
    for f in ("x", "v", "F", "C"):
        assert rel(g[f], o[f]) <= GRAD_TOL, (f, rel(g[f], o[f]))
    for p in ("E", "nu"):
        assert abs(g[p] - o[p]) <= GRAD_TOL * abs(o[p]), (p, g[p], o[p])


def test_gpu_gradients_match_finite_differences(oracle):
    """The reduced 2D case: 1,024 particles, 32^2 grid, 50 steps, loss = |COM - target|^2."""
    dim, res, steps, n = 2, 32, 50, 1024
    s = setup(dim, res, n, scenes.CORRECTED, seed=9)
    target = np.array([0.45, 0.4])
    g = gpu_grads(s, dim, res, steps, scenes.CORRECTED, every=50, seed_fn=com_loss(target))

    def loss64(st):
        out, _, status, _ = oracle.advance(st, dim=dim, model=scenes.JELLY, res=res, steps=steps,
                                           fp64=True, physics=scenes.CORRECTED, want_grid=False)
        assert status == 0
        d = out["x"].mean(0) - target
        return float(d @ d)

    rng = np.random.default_rng(11)
    s64 = {k: np.asarray(v, np.float64) for k, v in s.items()}
    for field, h in (("v", 1e-4), ("x", 1e-6)):
        for _ in range(3):
            dirn = rng.normal(size=s64[field].shape)
            sp = dict(s64)
            sm = dict(s64)
            sp[field] = s64[field] + h * dirn
            sm[field] = s64[field] - h * dirn
            fd = (loss64(sp) - loss64(sm)) / (2 * h)
            ad = float((g[field].astype(np.float64) * dirn).sum())
            assert abs(ad - fd) <= GRAD_TOL * abs(fd), (field, ad, fd)


def test_checkpoint_interval_does_not_change_gradients():
    """Recomputing from checkpoints every 3 steps or once: same gradients (a loss on every
    particle's position, so that no field's gradient vanishes by momentum conservation)."""
    dim, res, steps, n = 2, 32, 40, 1024
    s = setup(dim, res, n, scenes.REFERENCE, seed=4)
    loss = point_loss(s["x"] + np.float32(0.01))
    a = gpu_grads(s, dim, res, steps, scenes.REFERENCE, every=40, seed_fn=loss)
    b = gpu_grads(s, dim, res, steps, scenes.REFERENCE, every=3, seed_fn=loss)
    for f in ("x", "v", "F", "C"):
        assert rel(a[f], b[f]) <= GRAD_TOL, f


@pytest.mark.parametrize("dim,res,steps,n,physics,stress", [
    (2, 32, 50, 1024, scenes.REFERENCE, 0),
    (3, 16, 10, 512, scenes.CORRECTED, 1),
])
def test_gpu_per_particle_moduli_gradients_match_fp64_adjoint(oracle, dim, res, steps, n,
                                                              physics, stress):
    """One E and nu per particle (nclr_rollout_forward_moduli / backward_moduli through the
    autograd function with E and nu tensors of n values): every particle's E and nu gradient,
    and those of the initial state, against the FP64 CPU adjoint."""
    s = setup(dim, res, n, physics)
    rng = np.random.default_rng(6)
    Ep = np.exp(rng.uniform(np.log(1e3), np.log(1e4), size=n)).astype(np.float32)
    nup = rng.uniform(0.15, 0.35, size=n).astype(np.float32)
    kw = dict(dim=dim, res=res, steps=steps, physics=physics, stress=stress,
              E_particles=Ep.astype(np.float64), nu_particles=nup.astype(np.float64))
    fwd, _ = oracle.adjoint(s, seed={}, **kw)
    targets = (fwd["x"] + rng.normal(0, 1e-3, size=fwd["x"].shape)).astype(np.float32)
    g = gpu_grads(s, dim, res, steps, physics, every=7, seed_fn=point_loss(targets), E=Ep, nu=nup,
                  stress=stress)
    assert g["E"].shape == (n,) and g["nu"].shape == (n,)
    seed = 2 * (g["xT"].astype(np.float64) - targets)  # the GPU's own final state
    _, o = oracle.adjoint(s, seed={"x": seed}, **kw)
    for f in ("x", "v", "F", "C", "E", "nu"):
        assert rel(g[f], o[f]) <= GRAD_TOL, (f, rel(g[f], o[f]))


def plastic_setup(dim, res, n, physics, seed=0):
    """The jittered block with F perturbed by 2%: singular values on both sides of the snow
    clamp's bounds, so that clamped and free ones both enter."""
    s = setup(dim, res, n, physics, seed)
    rng = np.random.default_rng(seed + 7)
    s["F"] = (s["F"] + rng.normal(0, 0.02, size=s["F"].shape)).astype(np.float32)
    return s


@pytest.mark.parametrize("dim,res,steps,n", [(2, 32, 30, 1024), (3, 16, 8, 512)])
@pytest.mark.parametrize("physics", [scenes.REFERENCE, scenes.CORRECTED])
@pytest.mark.parametrize("model", [scenes.SNOW, scenes.LIQUID])
def test_gpu_plastic_adjoint_matches_fp64_adjoint(oracle, dim, res, steps, n, physics, model):
    """Snow and liquid rollouts: every gradient (initial x, v, F, C; E and nu) against the FP64
    CPU adjoint of the same rollout."""
    if dim == 3 and physics == scenes.REFERENCE and model == scenes.LIQUID:
        pytest.skip("3D liquid under the reference physics resets F to diag(J, 1, 0), whose "
                    "polar rotation is not unique: the step is not differentiable there")
    s = plastic_setup(dim, res, n, physics)
    rng = np.random.default_rng(3)
    kw = dict(dim=dim, res=res, steps=steps, physics=physics, model=model)
    fwd, _ = oracle.adjoint(s, seed={}, **kw)
    targets = (fwd["x"] + rng.normal(0, 1e-3, size=fwd["x"].shape)).astype(np.float32)
    g = gpu_grads(s, dim, res, steps, physics, every=7, seed_fn=point_loss(targets), model=model)
    seed = 2 * (g["xT"].astype(np.float64) - targets)  # the GPU's own final state
    _, o = oracle.adjoint(s, seed={"x": seed}, **kw)
    for f in ("x", "v", "F", "C"):
        assert rel(g[f], o[f]) <= GRAD_TOL, (f, rel(g[f], o[f]))
    for p in ("E", "nu"):
        assert abs(g[p] - o[p]) <= GRAD_TOL * abs(o[p]), (p, g[p], o[p])


def test_gpu_snow_gradients_match_finite_differences(oracle):
    """The reduced 2D case in snow: 1,024 particles, 32^2 grid, 50 steps, a deformation-dependent
    loss; directional derivatives of the initial velocities and positions and the E / nu
    derivatives against FP64 central differences of the oracle's forward rollout (steps small
    enough that no particle's clamp switches inside them: the loss is piecewise smooth).  A
    directional derivative sum_i g_i d_i over random directions cancels (the velocity one by
    about two digits here), so it is held to 1e-3 of its uncancelled scale sum_i |g_i d_i|; the
    E and nu derivatives are sums over particles that cancel too, and are held to 2e-3 of
    sum_p |g_p|, each particle's own derivative (the same rollout with one E and nu per
    particle, all equal, whose gradients must also add up to the scene's).  After every step
    the clamp leaves many snow particles exactly on its bounds; for those whose strain rate is
    near zero, the FP32 and FP64 trajectories can disagree on whether the next step's clamp is
    active, and the gradient -- exact for each trajectory -- jumps there (measured 1.3e-3 of
    that scale for nu)."""
    dim, res, steps, n = 2, 32, 50, 1024
    s = plastic_setup(dim, res, n, scenes.CORRECTED, seed=9)
    fwd, _, st, _ = oracle.advance(s, dim=dim, model=scenes.SNOW, res=res, steps=steps,
                                   fp64=True, physics=scenes.CORRECTED, want_grid=False)
    assert st == 0
    targets = fwd["x"] + np.random.default_rng(5).normal(0, 1e-3, size=fwd["x"].shape)
    g = gpu_grads(s, dim, res, steps, scenes.CORRECTED, every=10,
                  seed_fn=point_loss(targets.astype(np.float32)), model=scenes.SNOW)

    def loss64(st, E=1e4, nu=0.2):
        out, _, status, _ = oracle.advance(st, dim=dim, model=scenes.SNOW, res=res, steps=steps,
                                           fp64=True, physics=scenes.CORRECTED, E=E, nu=nu,
                                           want_grid=False)
        assert status == 0
        return float(((out["x"] - targets) ** 2).sum())

    rng = np.random.default_rng(11)
    s64 = {k: np.asarray(v, np.float64) for k, v in s.items()}
    for field, h in (("v", 1e-6), ("x", 1e-8)):
        for _ in range(3):
            dirn = rng.normal(size=s64[field].shape)
            sp, sm = dict(s64), dict(s64)
            sp[field] = s64[field] + h * dirn
            sm[field] = s64[field] - h * dirn
            fd = (loss64(sp) - loss64(sm)) / (2 * h)
            terms = g[field].astype(np.float64) * dirn
            ad = float(terms.sum())
            assert abs(ad - fd) <= GRAD_TOL * float(np.abs(terms).sum()), (field, ad, fd)
    gp = gpu_grads(s, dim, res, steps, scenes.CORRECTED, every=10,
                   seed_fn=point_loss(targets.astype(np.float32)), model=scenes.SNOW,
                   E=np.full(n, 1e4, np.float32), nu=np.full(n, 0.2, np.float32))
    for name, h in (("E", 1e-2), ("nu", 1e-7)):
        kp, km = {"E": 1e4, "nu": 0.2}, {"E": 1e4, "nu": 0.2}
        kp[name] += h
        km[name] -= h
        fd = (loss64(s64, **kp) - loss64(s64, **km)) / (2 * h)
        scale = float(np.abs(gp[name].astype(np.float64)).sum())
        assert abs(float(gp[name].astype(np.float64).sum()) - float(g[name])) <= GRAD_TOL * scale
        assert abs(float(g[name]) - fd) <= 2 * GRAD_TOL * max(abs(fd), scale), (name, float(g[name]), fd, scale)
