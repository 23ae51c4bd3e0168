"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module,
and only to check or time against; the GPU library never calls it.

State dictionaries use the C ABI's host layout (particle-major, row-major matrices):
  x (n, dim), v (n, dim), F (n, dim, dim), C (n, dim, dim), Jp (n,), mass (n,), volume (n,).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS: dict[str, ctypes.CDLL] = {}

SNOW, JELLY, LIQUID = 0, 1, 2
REFERENCE, CORRECTED = 0, 1
COROTATED, NEOHOOKEAN = 0, 1  # stress models

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int64)


def _load(name: str, sub: str) -> ctypes.CDLL:
    if name not in _LIBS:
        path = os.path.join(HERE, sub, name)
        if not os.path.isfile(path):
            from oracle.build_oracle import build
            build()
        lib = ctypes.CDLL(path)
        if name.startswith("liboracle"):
            lib.oracle_advance.restype = ctypes.c_int
            lib.oracle_advance.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int64,
                                           _dp, _dp, _dp, _dp, _dp, _dp, _dp, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp,
                                           _dp, _ip, ctypes.c_void_p]
            lib.oracle_advance_threads.restype = ctypes.c_int
            lib.oracle_advance_threads.argtypes = lib.oracle_advance.argtypes + [ctypes.c_int]
            lib.oracle_advance_ex.restype = ctypes.c_int
            lib.oracle_advance_ex.argtypes = lib.oracle_advance.argtypes + [
                _dp, _dp, ctypes.c_int, ctypes.c_int]
            lib.oracle_svd.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp]
            lib.oracle_polar.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp]
            lib.oracle_linspaced.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                             ctypes.POINTER(ctypes.c_float)]
            lib.oracle_adjoint.restype = ctypes.c_int
            lib.oracle_adjoint.argtypes = ([ctypes.c_int, ctypes.c_int, ctypes.c_int64] + [_dp] * 6 +
                                           [ctypes.c_int] + [ctypes.c_double] * 4 + [ctypes.c_int] +
                                           [_dp] * 13 + [ctypes.c_int] + [_dp] * 4)
            lib.oracle_adjoint_model.restype = ctypes.c_int
            lib.oracle_adjoint_model.argtypes = (
                [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int64] + [_dp] * 7 +
                [ctypes.c_int] + [ctypes.c_double] * 4 + [ctypes.c_int] + [_dp] * 16 +
                [ctypes.c_int])
        else:
            lib.ref_advance.restype = ctypes.c_int
            lib.ref_advance.argtypes = [ctypes.c_int, ctypes.c_int64, _dp, _dp, _dp, _dp, _dp, _dp,
                                        _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int, _dp, _dp]
            lib.ref_cube.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                     ctypes.POINTER(ctypes.c_float)]
        _LIBS[name] = lib
    return _LIBS[name]


def oracle_lib(fast: bool = False) -> ctypes.CDLL:
    return _load("liboracle_fast.so" if fast else "liboracle.so", "_build")


def ref_available() -> bool:
    return os.path.isfile(os.path.join(HERE, "_ref", "libnclr_ref.so"))


def ref_lib() -> ctypes.CDLL:
    return _load("libnclr_ref.so", "_ref")


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _prep(state: dict, dim: int):
    n = state["x"].shape[0]
    out = {}
    for k, shape in (("x", (n, dim)), ("v", (n, dim)), ("F", (n, dim, dim)), ("C", (n, dim, dim)),
                     ("Jp", (n,)), ("mass", (n,)), ("volume", (n,))):
        out[k] = np.ascontiguousarray(np.asarray(state[k], dtype=np.float64).reshape(shape)).copy()
    return n, out


def advance(state: dict, *, dim: int, model: int, res: int = 64, dt: float = 1e-4,
            E: float = 1e4, nu: float = 0.2, gravity: float = -100.0, steps: int = 1,
            fp64: bool = False, physics: int = REFERENCE, fast: bool = False,
            want_grid: bool = True, material=None, threads: int = 1, E_particles=None,
            nu_particles=None, stress: int = COROTATED):
    """Runs `steps` reference steps on a copy of `state`; returns (state, grid, status, counters).

    grid = (velocity (nodes, dim), mass (nodes,)) of the last step, post grid update.
    status 0 = ok, 2 = a grid index left the grid (the reference throws std::out_of_range).
    threads > 1 runs the multi-threaded baseline (nclr_oracle_mt.h): the same step up to the
    FP32 summation order of the grid.  E_particles / nu_particles (both or neither) give each
    particle its own moduli; stress picks the fixed-corotated or the neo-Hookean stress.
    """
    n, s = _prep(state, dim)
    mat = None if material is None else np.ascontiguousarray(material, dtype=np.uint8)
    nodes = (res + 1) ** dim
    gv = np.zeros((nodes, dim)) if want_grid else None
    gm = np.zeros((nodes,)) if want_grid else None
    counters = np.zeros(2, dtype=np.int64)
    args = (dim, int(fp64), physics, n, _p(s["x"]), _p(s["v"]), _p(s["F"]), _p(s["C"]),
            _p(s["Jp"]), _p(s["mass"]), _p(s["volume"]), model, res, dt, E, nu, gravity, steps,
            _p(gv) if want_grid else None, _p(gm) if want_grid else None,
            counters.ctypes.data_as(_ip), mat.ctypes.data if mat is not None else None)
    lib = oracle_lib(fast)
    if (E_particles is None) != (nu_particles is None):
        raise ValueError("E_particles and nu_particles go together")
    if E_particles is None and stress == COROTATED:
        st = lib.oracle_advance_threads(*args, threads) if threads > 1 else lib.oracle_advance(*args)
    else:
        Ep = nup = None
        if E_particles is not None:
            Ep = np.ascontiguousarray(np.broadcast_to(np.asarray(E_particles, np.float64), (n,)))
            nup = np.ascontiguousarray(np.broadcast_to(np.asarray(nu_particles, np.float64), (n,)))
        st = lib.oracle_advance_ex(*args, None if Ep is None else _p(Ep),
                                   None if nup is None else _p(nup), int(stress), max(1, threads))
    return s, ((gv, gm) if want_grid else None), st, counters


def _adjoint_model(state, *, dim, res, steps, dt, E, nu, gravity, physics, seed, stress, model):
    n, s = _prep(state, dim)
    out = {k: np.zeros_like(s[k]) for k in ("x", "v", "F", "C", "Jp")}
    g = {k: np.zeros_like(s[k]) for k in ("x", "v", "F", "C", "Jp")}
    sd = {k: (np.ascontiguousarray(seed[k], dtype=np.float64) if k in seed else None)
          for k in ("x", "v", "F", "C", "Jp")}
    ml = np.zeros(2)
    st = oracle_lib().oracle_adjoint_model(
        dim, physics, model, n, _p(s["x"]), _p(s["v"]), _p(s["F"]), _p(s["C"]), _p(s["Jp"]),
        _p(s["mass"]), _p(s["volume"]), res, dt, E, nu, gravity, steps, _p(out["x"]),
        _p(out["v"]), _p(out["F"]), _p(out["C"]), _p(out["Jp"]),
        *(None if sd[k] is None else _p(sd[k]) for k in ("x", "v", "F", "C", "Jp")),
        _p(g["x"]), _p(g["v"]), _p(g["F"]), _p(g["C"]), _p(g["Jp"]), _p(ml), int(stress))
    if st != 0:
        raise RuntimeError(f"oracle adjoint failed ({st})")
    _, _, dmu, dlam = lame(E, nu)
    g["mu0"], g["lambda0"] = float(ml[0]), float(ml[1])
    g["E"] = ml[0] * dmu[0] + ml[1] * dlam[0]
    g["nu"] = ml[0] * dmu[1] + ml[1] * dlam[1]
    return out, g


def ref_advance(state: dict, *, dim: int, model: int, res: int = 64, dt: float = 1e-4,
                E: float = 1e4, nu: float = 0.2, gravity: float = -100.0, steps: int = 1):
    """The reference's own MPMSimulation<dim>::advance() (compiled against the Eigen shim)."""
    n, s = _prep(state, dim)
    nodes = (res + 1) ** dim
    gv = np.zeros((nodes, dim))
    gm = np.zeros((nodes,))
    st = ref_lib().ref_advance(dim, n, _p(s["x"]), _p(s["v"]), _p(s["F"]), _p(s["C"]),
                               _p(s["Jp"]), _p(s["mass"]), _p(s["volume"]), model, res, dt, E,
                               nu, gravity, steps, _p(gv), _p(gm))
    return s, (gv, gm), st


def svd(A: np.ndarray, *, physics: int = REFERENCE, fp64: bool = False):
    A = np.ascontiguousarray(A, dtype=np.float64)
    d = A.shape[0]
    U = np.zeros((d, d)); S = np.zeros(d); V = np.zeros((d, d))
    oracle_lib().oracle_svd(d, int(fp64), physics, _p(A), _p(U), _p(S), _p(V))
    return U, S, V


def polar(A: np.ndarray, *, physics: int = REFERENCE, fp64: bool = False):
    A = np.ascontiguousarray(A, dtype=np.float64)
    d = A.shape[0]
    R = np.zeros((d, d))
    oracle_lib().oracle_polar(d, int(fp64), physics, _p(A), _p(R))
    return R


def linspaced(n: int, lo: float, hi: float) -> np.ndarray:
    out = np.zeros(n, dtype=np.float32)
    oracle_lib().oracle_linspaced(n, lo, hi, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    return out


def ref_cube(dim: int, n: int, lo: float, hi: float) -> np.ndarray:
    out = np.zeros((n ** dim, dim), dtype=np.float32)
    ref_lib().ref_cube(dim, n, lo, hi, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    return out


def lame(E: float, nu: float):
    """mu_0, lambda_0 (src/nclr.h:77-78) and their derivatives with respect to E and nu."""
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    dmu = (1 / (2 * (1 + nu)), -E / (2 * (1 + nu) ** 2))
    dlam = (nu / ((1 + nu) * (1 - 2 * nu)), E * (1 + 2 * nu ** 2) / ((1 + nu) * (1 - 2 * nu)) ** 2)
    return mu, lam, dmu, dlam


def adjoint(state: dict, *, dim: int, res: int, steps: int, dt: float = 1e-4, E: float = 1e4,
            nu: float = 0.2, gravity: float = -100.0, physics: int = REFERENCE, seed: dict,
            stress: int = COROTATED, E_particles=None, nu_particles=None, model: int = JELLY):
    """FP64 rollout and its reverse pass.  `seed` holds the final state's adjoint (keys among
    x, v, F, C, and Jp for the plastic materials).  Returns (final state, adjoint of the
    initial state incl. 'E' and 'nu').  With E_particles / nu_particles (one value per particle,
    jelly), 'E' and 'nu' (and 'mu0', 'lambda0') are arrays: every particle's own adjoints.
    `model` other than jelly (snow, liquid) also carries Jp: the state's 'Jp' (1 if absent) is
    the initial one, and the results hold the final 'Jp' and its initial adjoint 'Jp'."""
    if model != JELLY or "Jp" in seed:
        if E_particles is not None:
            raise ValueError("per-particle moduli are covered for jelly")
        return _adjoint_model(state, dim=dim, res=res, steps=steps, dt=dt, E=E, nu=nu,
                              gravity=gravity, physics=physics, seed=seed, stress=stress,
                              model=model)
    n, s = _prep(state, dim)
    out = {k: np.zeros_like(s[k]) for k in ("x", "v", "F", "C")}
    g = {k: np.zeros_like(s[k]) for k in ("x", "v", "F", "C")}
    sd = {k: (np.ascontiguousarray(seed[k], dtype=np.float64) if k in seed else None)
          for k in ("x", "v", "F", "C")}
    ml = np.zeros(2)
    rows = E_particles is not None
    if rows != (nu_particles is not None):
        raise ValueError("E_particles and nu_particles go together")
    Ep = nup = gmr = glr = None
    if rows:
        Ep = np.ascontiguousarray(np.broadcast_to(np.asarray(E_particles, np.float64), (n,)))
        nup = np.ascontiguousarray(np.broadcast_to(np.asarray(nu_particles, np.float64), (n,)))
        gmr, glr = np.zeros(n), np.zeros(n)
    st = oracle_lib().oracle_adjoint(
        dim, physics, n, _p(s["x"]), _p(s["v"]), _p(s["F"]), _p(s["C"]), _p(s["mass"]),
        _p(s["volume"]), res, dt, E, nu, gravity, steps, _p(out["x"]), _p(out["v"]),
        _p(out["F"]), _p(out["C"]), *(None if sd[k] is None else _p(sd[k]) for k in ("x", "v", "F", "C")),
        _p(g["x"]), _p(g["v"]), _p(g["F"]), _p(g["C"]), _p(ml), int(stress),
        *((_p(Ep), _p(nup), _p(gmr), _p(glr)) if rows else (None,) * 4))
    if st != 0:
        raise RuntimeError(f"oracle adjoint failed ({st})")
    if rows:
        _, _, dmu, dlam = lame(Ep, nup)
        g["mu0"], g["lambda0"] = gmr, glr
        g["E"] = gmr * dmu[0] + glr * dlam[0]
        g["nu"] = gmr * dmu[1] + glr * dlam[1]
        return out, g
    _, _, dmu, dlam = lame(E, nu)
    g["mu0"], g["lambda0"] = float(ml[0]), float(ml[1])
    g["E"] = ml[0] * dmu[0] + ml[1] * dlam[0]
    g["nu"] = ml[0] * dmu[1] + ml[1] * dlam[1]
    return out, g
