"""The bounded grid barrier of the small-scene kernels (one cooperative launch per advance()
call).  A CTA that waits at the barrier gives up after a bounded number of polls, flags the
error and leaves the kernel, and so does every other CTA: nothing waits without a bound.

nclr_debug_set_barrier makes every barrier wait for one more CTA than the launch has, a CTA
that never comes, with a short poll limit: the wait runs out on every CTA, the call reports
NCLR_ERR_CUDA with the barrier message within a fraction of a second, and the handle stays
usable -- with the normal barrier back and the half-stepped state replaced, the next step
matches the oracle.  Single scenes and batches (each scene of a batch has its own barrier)."""
import time

import numpy as np
import pytest

from conftest import FIELDS, field_err
from nuclearmpm_gb300 import BatchSimulation, MPMSimulation, capi, scenes

pytestmark = pytest.mark.gpu

SHORT = 1 << 12  # polls of ~64 ns: well under a millisecond per wait


def test_single_scene_barrier_timeout_is_reported_and_handle_recovers(oracle):
    s = scenes.readme_scene()
    sim = MPMSimulation(dict(s), scenes.SNOW, res=64, small_scene_max=1 << 30)
    L = capi.lib()
    assert L.nclr_debug_set_barrier(sim._h, 1, SHORT) == capi.NCLR_OK
    t0 = time.perf_counter()
    with pytest.raises(capi.NclrError) as err:
        sim.advance(3)
    assert err.value.status == capi.NCLR_ERR_CUDA
    assert "barrier" in str(err.value)
    assert time.perf_counter() - t0 < 5.0
    # the normal barrier again; replace the half-stepped state and step once
    assert L.nclr_debug_set_barrier(sim._h, 0, 0) == capi.NCLR_OK
    sim.set_particles(x=s["x"], v=s["v"], F=s["F"], C=s["C"], Jp=s["Jp"])
    sim.advance(1)
    p = sim.particles()
    sim.close()
    ref, _, st, _ = oracle.advance(s, dim=2, model=scenes.SNOW, res=64, steps=1)
    assert st == 0
    for f in FIELDS:
        assert field_err(getattr(p, f), ref[f], f) <= 1e-5, f


def test_batch_barrier_timeout_is_reported_and_handle_recovers():
    scs = scenes.batched_scenes_2d(seed=3, count=4, n_min=1000, n_max=4000)
    b = BatchSimulation(scs, small_scene_max=1 << 30)
    L = capi.lib()
    assert L.nclr_debug_set_barrier(b._h, 1, SHORT) == capi.NCLR_OK
    with pytest.raises(capi.NclrError) as err:
        b.advance(2)
    assert "barrier" in str(err.value)
    assert L.nclr_debug_set_barrier(b._h, 0, 0) == capi.NCLR_OK
    for i, sc in enumerate(scs):
        b.set_particles(i, x=sc["x"], v=sc["v"], F=sc["F"], C=sc["C"], Jp=sc["Jp"])
    b.advance(1)
    for i, sc in enumerate(scs):
        alone = MPMSimulation({k: sc[k] for k in ("x", "v", "F", "C", "Jp", "mass", "volume")},
                              sc["model"], res=sc["res"], dt=sc["dt"], E=sc["E"], nu=sc["nu"],
                              gravity=sc["gravity"], small_scene_max=1 << 30)
        alone.advance(1)
        a = alone.particles()
        alone.close()
        got = b.particles(i)
        for f in FIELDS:
            assert field_err(got[f], getattr(a, f), f) <= 1e-5, (i, f)
    b.close()
