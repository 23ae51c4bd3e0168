"""Reader of the headless solver's binary dump (`nclr_solver --dump` writes <out>/dump.nclr).

The reference's solver dumps every step as text files `tmp/<step>_{timestep,x,v,F,C,Jp,lame,
mass,velocity}.txt` (src/solver.cpp:75-131), and python/ioutils.py:32-102 (`process_tmp`)
loads them into a dict keyed "<step>_" of `SimResult` objects with those nine attributes.  The
binary dump holds the same states (the particles before each advance(), the grid of the
previous advance(), zeros at step 0) at full FP32 precision; `load` returns the same dict,
attribute names and array shapes:

    x, v        (n, dim)          F, C       (n, dim, dim)      Jp        (n,)
    lame        (n, 2)  mu_0 * e, lambda_0 * e with the model's hardening e, per particle
    timestep    (n,)    dt * step (dt at step 0), per particle, as the text dump repeats it
    mass        (N,) * dim        velocity   (N,) * dim + (dim,)     N = res + 1

as float64 arrays (np.loadtxt's type).  With `reference_grid_layout=True`, mass and velocity
reproduce the reference's unload_cells indexing, which reads cell ii * res + jj instead of
ii * (res + 1) + jj (src/solver.cpp:117), so that code written against the reference's
dumps sees the same arrays (2D only, as the reference's dump).

    from nuclearmpm_gb300 import dumpio
    results = dumpio.load("tmp/dump.nclr")
    results["10_"].x          # the particles before the 11th advance()
"""
from __future__ import annotations

import os
import pickle
import struct

import numpy as np

MAGIC = b"NCLRDMP1"
_HEADER = struct.Struct("<8s4Iq4f")  # magic, dim, res, model, physics, n, dt, mu0, lambda0, e
_RECORD_HEAD = struct.Struct("<qff")  # step, timestep, reserved


class SimResult:
    """One dumped step (the attributes of python/ioutils.py's SimResult)."""

    x: np.ndarray
    v: np.ndarray
    F: np.ndarray
    C: np.ndarray
    Jp: np.ndarray
    lame: np.ndarray
    velocity: np.ndarray
    mass: np.ndarray
    timestep: np.ndarray


def read_header(path: str) -> dict:
    with open(path, "rb") as f:
        raw = f.read(_HEADER.size)
    if len(raw) < _HEADER.size:
        raise ValueError(f"{path}: truncated header")
    magic, dim, res, model, physics, n, dt, mu0, lam0, e = _HEADER.unpack(raw)
    if magic != MAGIC:
        raise ValueError(f"{path}: not an nclr_solver dump")
    return dict(dim=dim, res=res, model=model, physics=physics, n=n, dt=dt, mu0=mu0,
                lambda0=lam0, hardening=e)


def _layout(h: dict):
    dim, n, nodes = h["dim"], h["n"], (h["res"] + 1) ** h["dim"]
    sizes = [("x", n * dim), ("v", n * dim), ("F", n * dim * dim), ("C", n * dim * dim),
             ("Jp", n), ("velocity", nodes * dim), ("mass", nodes)]
    return sizes, sum(s for _, s in sizes)


def load(path: str, *, reference_grid_layout: bool = False, dtype=np.float64) -> dict:
    """{"<step>_": SimResult} for every complete record of the dump."""
    h = read_header(path)
    dim, n, res = h["dim"], h["n"], h["res"]
    N = res + 1
    sizes, floats = _layout(h)
    rec = _RECORD_HEAD.size + 4 * floats
    count = (os.path.getsize(path) - _HEADER.size) // rec
    raw = np.memmap(path, dtype=np.uint8, mode="r", offset=_HEADER.size, shape=(count * rec,))
    if reference_grid_layout and dim != 2:
        raise ValueError("the reference's grid dump layout exists in 2D only")
    ii, jj = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
    ref_idx = (ii * res + jj).reshape(-1)  # src/solver.cpp:117 (stride res, not res + 1)
    lame = np.tile(np.array([h["mu0"] * h["hardening"], h["lambda0"] * h["hardening"]],
                            np.float32).astype(dtype), (n, 1))
    out: dict[str, SimResult] = {}
    for k in range(count):
        base = k * rec
        step, ts, _ = _RECORD_HEAD.unpack(bytes(raw[base:base + _RECORD_HEAD.size]))
        data = np.frombuffer(raw[base + _RECORD_HEAD.size:base + rec], dtype=np.float32)
        r = SimResult()
        off = 0
        for name, size in sizes:
            a = data[off:off + size].astype(dtype)
            off += size
            if name in ("x", "v"):
                a = a.reshape(n, dim)
            elif name in ("F", "C"):
                a = a.reshape(n, dim, dim)
            elif name == "velocity":
                a = a.reshape(-1, dim)
                a = (a[ref_idx] if reference_grid_layout else a).reshape((N,) * dim + (dim,))
            elif name == "mass":
                a = (a[ref_idx] if reference_grid_layout else a).reshape((N,) * dim)
            setattr(r, name, a)
        r.lame = lame.copy()
        r.timestep = np.full(n, ts, dtype=np.float32).astype(dtype)
        out[f"{step}_"] = r
    return out


def process_dump(path: str, output: str = "results.pickle", **kw) -> dict:
    """python/ioutils.py's process_tmp for the binary dump: load, then pickle to `output`."""
    results = load(path, **kw)
    with open(output, "wb+") as f:
        pickle.dump(results, f)
    return results
