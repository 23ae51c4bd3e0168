"""GPU test of nclr_grid_transfer_noalloc, the entry point for callers that cannot allocate
device memory while they run (an application whose allocator already holds the GPU's memory,
a real-time loop, a plugin inside a runtime that owns every allocation).

The caller owns every array; the transfer's accumulation grid is a static device array inside
the library.  Its output -- the grid after one step's particle-to-grid transfer and grid
update -- must match what the regular entry points give for the same state
(nclr_create + nclr_advance(sim, 1) + nclr_get_grid), within the one-step grid tolerance of the
parity tests, on calls in a row with different scenes and materials (which also shows that
each call starts from a cleared scratch grid), and an empty call in between must give an
all-zero grid.  This file is collected last so that a run stopping at the first failure has
run every other test already.
"""
import ctypes

import numpy as np
import pytest

from conftest import field_err, load_golden
from nuclearmpm_gb300 import MPMSimulation, capi

pytestmark = pytest.mark.gpu

GRID_TOL = {"grid_v": 1e-5, "grid_m": 1e-5}


def _regular_grid(state, params):
    sim = MPMSimulation(dict(state), params["model"], res=params["res"], dt=params["dt"],
                        E=params["E"], nu=params["nu"], gravity=params["gravity"])
    sim.advance(1)
    g = sim.grid()
    sim.close()
    return g.velocity, g.mass


def _noalloc_grid(torch, state, params):
    dim, res = params["dim"], params["res"]
    dev = torch.device("cuda", 0)
    t = {k: torch.as_tensor(np.ascontiguousarray(state[k], dtype=np.float32)).to(dev)
         for k in ("x", "v", "F", "C", "Jp", "mass", "volume")}
    nodes = (res + 1) ** dim
    vel = torch.full((nodes, dim), float("nan"), device=dev)
    mass = torch.full((nodes,), float("nan"), device=dev)
    msg = ctypes.create_string_buffer(256)
    stream = torch.cuda.current_stream(dev).cuda_stream
    st = capi.lib().nclr_grid_transfer_noalloc(
        dim, int(t["x"].shape[0]), t["x"].data_ptr(), t["v"].data_ptr(), t["F"].data_ptr(),
        t["C"].data_ptr(), t["Jp"].data_ptr(), t["mass"].data_ptr(), t["volume"].data_ptr(),
        params["model"], res, params["dt"], params["E"], params["nu"], params["gravity"],
        vel.data_ptr(), mass.data_ptr(), stream, msg, len(msg))
    assert st == capi.NCLR_OK, (st, msg.value)
    return vel.cpu().numpy(), mass.cpu().numpy()


def _empty_call(torch, dim, res):
    """n = 0: no particle arrays; the grid update of a cleared scratch grid is all zeros."""
    dev = torch.device("cuda", 0)
    nodes = (res + 1) ** dim
    vel = torch.full((nodes, dim), float("nan"), device=dev)
    mass = torch.full((nodes,), float("nan"), device=dev)
    msg = ctypes.create_string_buffer(256)
    stream = torch.cuda.current_stream(dev).cuda_stream
    st = capi.lib().nclr_grid_transfer_noalloc(dim, 0, None, None, None, None, None, None, None,
                                               1, res, 1e-4, 1e4, 0.2, -100.0, vel.data_ptr(),
                                               mass.data_ptr(), stream, msg, len(msg))
    assert st == capi.NCLR_OK, (st, msg.value)
    return vel.cpu().numpy(), mass.cpu().numpy()


def test_noalloc_transfer_matches_regular_entry_points_twice():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    # calls in a row: 3D jelly, 2D snow, 2D liquid (different grid sizes and hardening), an
    # empty call over the 3D grid (it must not see the earlier sums), then the 3D scene again
    cases = [load_golden("block3d_jelly"), load_golden("readme_snow"),
             load_golden("readme_liquid"), None, load_golden("block3d_jelly")]
    first = None
    for case in cases:
        if case is None:
            ev, em = _empty_call(torch, 3, first_res)
            assert np.all(ev == 0.0) and np.all(em == 0.0)
            continue
        z, state, params, _ = case
        if first is None:
            first_res = params["res"]
        rv, rm = _regular_grid(state, params)
        nv, nm = _noalloc_grid(torch, state, params)
        assert field_err(nv, rv, "grid_v") <= GRID_TOL["grid_v"]
        assert field_err(nm, rm, "grid_m") <= GRID_TOL["grid_m"]
        # and against the reference's own grid after its first step
        assert field_err(nv, z["grid_v"], "grid_v") <= GRID_TOL["grid_v"]
        assert field_err(nm, z["grid_m"], "grid_m") <= GRID_TOL["grid_m"]
        if first is None:
            first = (nv, nm)
    # the repeated scene: nothing of the 2D call is left in the shared scratch grid
    assert field_err(nv, first[0], "grid_v") <= GRID_TOL["grid_v"]
    assert field_err(nm, first[1], "grid_m") <= GRID_TOL["grid_m"]


def test_noalloc_rejects_grids_beyond_its_static_array():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    x = torch.full((1, 3), 0.5, device=dev)
    msg = ctypes.create_string_buffer(256)
    res = 128  # 129^3 nodes > NCLR_NOALLOC_MAX_NODES
    assert (res + 1) ** 3 > capi.NOALLOC_MAX_NODES
    p = x.data_ptr()
    st = capi.lib().nclr_grid_transfer_noalloc(3, 1, p, p, p, p, p, p, p, 1, res, 1e-4, 1e4, 0.2,
                                               -100.0, p, p, None, msg, len(msg))
    assert st == capi.NCLR_ERR_INVALID
    assert b"at most" in msg.value
