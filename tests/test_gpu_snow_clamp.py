"""The snow plasticity clamp (src/nclr.h:237-250) on near-degenerate singular values, GPU FP32
against the FP64 oracle.

The clamp replaces F_hat = U S V^T by U clamp(S, 1 - 2.5e-2, 1 + 4.5e-3) V^T and updates Jp by the
ratio of determinants, with U, V rotations and the last singular value carrying the sign of
det F_hat.  When two singular values are close, U and V are ill-conditioned, but with det F_hat
> 0 the clamped F is a spectral function of F_hat whose divided differences are at most 1, so
it is as well conditioned as F_hat itself: FP32 suffices, however close the singular values.
With det F_hat < 0 the clamp lifts the negative singular value s_l, and the clamped F changes by
(f(s_p) + f(s_l)) / (s_p + s_l) per unit of F_hat (s_p the one before it): without bound as
|s_l| approaches s_p, where the result is discontinuous.  There the step recomputes the clamp
in FP64 (mpm_step.cuh: snow_clamp_needs_fp64 / snow_clamp_fp64), as the scope asks for the
near-degenerate singular values of the snow clamp.  These tests construct both kinds of case
and hold the GPU to 1e-5 of the FP64 oracle on the same FP32 input.

Construction: each particle sits alone (stencils four cells apart, so no two particles share a
grid node), v = 0, no gravity and a Young's modulus of 0, so there is no stress, the grid
velocities are exactly 0, C = 0 and F_hat = F exactly in FP32 and FP64 alike: the constructed
F = U diag(sigma) V^T (random rotations, stored in FP32) reaches both clamps as built.  (Any
stress would leave a C of order 1e-4 here, and the FP32 product (I + dt C) F would round that
update away while FP64 keeps it -- a difference the discontinuous cases amplify thousands of
times.)  Families of sigma, each with gaps g of 1e-7, 1e-6, 1e-5, 1e-4:
  * all three inside the clamp range, pairwise g apart;
  * a pair straddling the upper bound 1.0045 (1.0045 +- g/2), the third at 1;
  * a pair straddling the lower bound 0.975;
  * a pair g apart just outside either bound, and a triple g apart outside the upper bound;
  * exactly equal pairs and triples on and beyond both bounds;
  * det F_hat < 0 with |s_l| within 1e-4 .. 1e-2 of s_p (the FP64 cases).
3D runs the corrected physics (under the reference's diag(1,1,0) the third column of F_hat
collapses before the clamp sees it); 2D runs both.  Both step paths (tile and small-scene).
"""
import numpy as np
import pytest

from conftest import field_err
from nuclearmpm_gb300 import MPMSimulation, scenes

pytestmark = pytest.mark.gpu

BOUND = 1e-5
LO, HI = 1.0 - 2.5e-2, 1.0 + 4.5e-3
GAPS = (1e-7, 1e-6, 1e-5, 1e-4)


def sigma_families(dim):
    out = []
    for g in GAPS:
        if dim == 3:
            out += [(1.0 + g, 1.0, 1.0 - g), (1.002 + g / 2, 1.002 - g / 2, 0.99),
                    (HI + g / 2, HI - g / 2, 1.0), (LO + g / 2, LO - g / 2, 1.0),
                    (HI + 0.002 + g, HI + 0.002, 1.0), (LO - 0.002, LO - 0.002 - g, 1.0),
                    (HI + 0.001 + g, HI + 0.001, HI + 0.001 - g),
                    (HI + g / 2, HI - g / 2, LO + g / 2)]
        else:
            out += [(1.0 + g, 1.0), (HI + g / 2, HI - g / 2), (LO + g / 2, LO - g / 2),
                    (HI + 0.002 + g, HI + 0.002), (LO - 0.002, LO - 0.002 - g),
                    (HI + g / 2, LO + g / 2)]
    out += [(1.0,) * dim, (HI,) * dim, (LO,) * dim, (HI + 0.003,) * dim, (LO - 0.003,) * dim]
    if dim == 3:
        out += [(HI + 0.003, HI + 0.003, 1.0), (LO - 0.003, LO - 0.003, 1.0), (1.0, 1.0, LO)]
    # det F_hat < 0 with |sigma_last| close to the one before it: the clamp lifts the negative
    # singular value, and its result changes by 2 f / (s_p - |s_l|) per unit of F_hat there
    # (thousands at these gaps); the step recomputes these in FP64
    for g in (1e-4, 1e-3, 1e-2):
        if dim == 3:
            out += [(1.0, 0.5, -(0.5 - g)), (1.2, 0.99, -(0.99 - g)), (2.4, 0.37, -(0.37 - g)),
                    (1.01, HI + g, -HI)]
        else:
            out += [(0.5, -(0.5 - g)), (1.0, -(1.0 - g)), (HI + g, -HI)]
    return out


def rotation(rng, dim):
    q, r = np.linalg.qr(rng.normal(size=(dim, dim)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def constructed_scene(dim, res, seed=0):
    """Isolated particles, one constructed F each (every family with several rotations)."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / res
    axis = np.arange(0.15, 0.85, 4 * dx) + 0.5 * dx  # four cells apart: disjoint stencils
    pts = np.stack(np.meshgrid(*([axis] * dim), indexing="ij"), -1).reshape(-1, dim)
    fams = sigma_families(dim)
    n = len(pts)
    F = np.empty((n, dim, dim))
    for i in range(n):
        sig = np.asarray(fams[i % len(fams)])
        F[i] = rotation(rng, dim) @ np.diag(sig) @ rotation(rng, dim).T
    s = scenes.particles(pts.astype(np.float32), np.zeros((n, dim), np.float32),
                         physics=scenes.CORRECTED)
    s["F"] = F.astype(np.float32)
    return s


CASES = [(2, scenes.REFERENCE), (2, scenes.CORRECTED), (3, scenes.CORRECTED)]
PATHS = {"tile": {"small_scene_max": 0, "sparse_block_max": 0}, "small": {"small_scene_max": 1 << 30}}


@pytest.mark.parametrize("path", sorted(PATHS))
@pytest.mark.parametrize("dim,physics", CASES)
def test_snow_clamp_near_degenerate_sigma_matches_fp64(oracle, dim, physics, path):
    res = 64 if dim == 3 else 256
    s = constructed_scene(dim, res)
    kw = dict(res=res, E=0.0, nu=0.2, gravity=0.0, dt=1e-4)
    sim = MPMSimulation(dict(s), scenes.SNOW, physics=physics, **kw, **PATHS[path])
    sim.advance(1)
    p = sim.particles()
    sim.close()
    o64, _, st, _ = oracle.advance(s, dim=dim, model=scenes.SNOW, steps=1, physics=physics,
                                   fp64=True, want_grid=False, **kw)
    assert st == 0
    # the clamp saw the constructed singular values (F_hat = F to ~1e-9)
    sig_in = np.linalg.svd(s["F"].astype(np.float64), compute_uv=False)
    sig_out64 = np.linalg.svd(o64["F"], compute_uv=False)
    assert np.all(sig_out64 >= LO - 1e-7) and np.all(sig_out64 <= HI + 1e-7)
    assert np.any(sig_in > HI) and np.any(sig_in < LO)
    for f in ("F", "Jp"):
        e = field_err(p.F if f == "F" else p.Jp, o64[f], f)
        assert e <= BOUND, (f, e)
    # elementwise as well: every particle's clamped F within 1e-5 of FP64
    d = np.abs(p.F.astype(np.float64) - o64["F"]).reshape(len(p.F), -1).max(1)
    assert d.max() <= BOUND, (int(d.argmax()), float(d.max()))
    # and the GPU's own result obeys the clamp
    sig_gpu = np.linalg.svd(p.F.astype(np.float64), compute_uv=False)
    assert np.all(sig_gpu >= LO - 1e-6) and np.all(sig_gpu <= HI + 1e-6)
