"""Python mirror of the reference's solver API (src/nclr.h:20-102) over libnclr_gpu.so.

    Particle(x, c, v=None, mass=1.0, volume=1.0)           src/nclr.h:20-48
    Cell                                                   src/nclr.h:50-55
    MaterialModel.kSnow / kJelly / kLiquid                 src/nclr.h:57-61
    MPMSimulation(particles, model, res=64, dt=1e-4, E=1e4, nu=0.2, gravity=-100)
        .advance()           src/nclr.h:80-84
        .particles()         src/nclr.h:86   (ParticleArrays: SoA numpy views, caller order)
        .grid()              src/nclr.h:87   (GridArrays: post-update grid of the last step;
                                              empty before the first advance, as in the
                                              reference)
        .mu_0, .lambda_0, kBoundary, kSnowHardening, kJellyHardening, kLiquidHardening

Extensions of the model: `material=` (one MaterialModel per particle), `set_moduli(E, nu)`
(one Young's modulus and Poisson ratio per particle) and `stress_model=` (the reference's
fixed-corotated stress, src/nclr.h:313-337, or the neo-Hookean one its TODO names,
src/nclr.h:339).

`particles` may be a list of Particle objects (as the reference takes a
std::vector<Particle<dim>>) or, for large scenes, a dict of arrays in the C ABI host layout
(x (n,dim), v, F (n,dim,dim), C, Jp, mass, volume).  Errors: a stencil that leaves the grid
raises OutOfRange (an IndexError, like the reference's std::out_of_range); CUDA failures
raise NclrError.  All compute runs in libnclr_gpu.so on the GPU.
"""
from __future__ import annotations

import ctypes
import enum
from dataclasses import dataclass, field

import numpy as np

from . import capi


class MaterialModel(enum.IntEnum):
    kSnow = 0
    kJelly = 1
    kLiquid = 2


def diag(dim: int, value: float, corrected: bool = False) -> np.ndarray:
    """diag<dim>(v) (src/nclr_math.h:13-19): only (0,0) and (1,1) are set, so diag<3> is
    diag(v, v, 0); `corrected=True` gives v*I."""
    m = np.zeros((dim, dim), dtype=np.float32)
    m[0, 0] = m[1, 1] = value
    if corrected:
        np.fill_diagonal(m, value)
    return m


@dataclass
class Particle:
    """Particle<dim> (src/nclr.h:20-48): F starts at diag<dim>(1), C at 0, Jp at 1."""
    x: np.ndarray
    c: int = 0
    v: np.ndarray | None = None
    mass: float = 1.0
    volume: float = 1.0
    F: np.ndarray | None = None
    C: np.ndarray | None = None
    Jp: float = 1.0

    def __post_init__(self):
        self.x = np.asarray(self.x, dtype=np.float32).copy()
        dim = self.x.shape[0]
        self.v = np.zeros(dim, np.float32) if self.v is None else np.asarray(self.v, np.float32).copy()
        self.F = diag(dim, 1.0) if self.F is None else np.asarray(self.F, np.float32).copy()
        self.C = np.zeros((dim, dim), np.float32) if self.C is None else np.asarray(self.C, np.float32).copy()


@dataclass
class ParticleArrays:
    """The particle state in the caller's order: x (n,dim), v (n,dim), F (n,dim,dim),
    C (n,dim,dim), Jp (n,), mass (n,), volume (n,), c (n,)."""
    x: np.ndarray
    v: np.ndarray
    F: np.ndarray
    C: np.ndarray
    Jp: np.ndarray
    mass: np.ndarray
    volume: np.ndarray
    c: np.ndarray

    def __len__(self):
        return self.x.shape[0]

    def __getitem__(self, p: int) -> Particle:
        return Particle(self.x[p], int(self.c[p]), self.v[p], float(self.mass[p]),
                        float(self.volume[p]), self.F[p], self.C[p], float(self.Jp[p]))


@dataclass
class GridArrays:
    """The grid in the reference's node order (x-major): velocity (nodes, dim), mass (nodes,)."""
    velocity: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.float32))
    mass: np.ndarray = field(default_factory=lambda: np.zeros((0,), np.float32))

    def __len__(self):
        return self.mass.shape[0]


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _soa_from(particles, dim_hint: int | None):
    if isinstance(particles, dict):
        x = np.ascontiguousarray(particles["x"], dtype=np.float32)
        n, dim = x.shape
        get = lambda k, shape: (None if particles.get(k) is None else  # noqa: E731
                                np.ascontiguousarray(np.asarray(particles[k], np.float32).reshape(shape)))
        return dim, dict(x=x, v=get("v", (n, dim)), F=get("F", (n, dim, dim)),
                         C=get("C", (n, dim, dim)), Jp=get("Jp", (n,)), mass=get("mass", (n,)),
                         volume=get("volume", (n,)),
                         c=np.asarray(particles.get("c", np.zeros(n)), np.int32))
    plist = list(particles)
    if not plist:
        dim = dim_hint or 2
        z = lambda *s: np.zeros(s, np.float32)  # noqa: E731
        return dim, dict(x=z(0, dim), v=z(0, dim), F=z(0, dim, dim), C=z(0, dim, dim), Jp=z(0),
                         mass=z(0), volume=z(0), c=np.zeros(0, np.int32))
    dim = plist[0].x.shape[0]
    return dim, dict(
        x=np.stack([p.x for p in plist]).astype(np.float32),
        v=np.stack([p.v for p in plist]).astype(np.float32),
        F=np.stack([p.F for p in plist]).astype(np.float32),
        C=np.stack([p.C for p in plist]).astype(np.float32),
        Jp=np.array([p.Jp for p in plist], np.float32),
        mass=np.array([p.mass for p in plist], np.float32),
        volume=np.array([p.volume for p in plist], np.float32),
        c=np.array([p.c for p in plist], np.int32))


def _set_moduli(h, n: int, E, nu) -> None:
    L = capi.lib()
    if (E is None) != (nu is None):
        raise ValueError("E and nu go together")
    if E is None:
        capi.check(L.nclr_set_moduli(h, None, None), h)
        return
    try:
        import torch
        on_device = isinstance(E, torch.Tensor) and E.is_cuda
    except ImportError:
        on_device = False
    if on_device:
        for t in (E, nu):
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32
                    and t.is_contiguous() and t.numel() == n):
                raise TypeError("device moduli must be contiguous float32 CUDA tensors of n values")
        capi.check(L.nclr_set_moduli_device(h, ctypes.c_void_p(E.data_ptr()),
                                            ctypes.c_void_p(nu.data_ptr())), h)
        return
    Ea = np.ascontiguousarray(np.broadcast_to(np.asarray(E, np.float32), (n,)))
    nua = np.ascontiguousarray(np.broadcast_to(np.asarray(nu, np.float32), (n,)))
    capi.check(L.nclr_set_moduli(h, _ptr(Ea), _ptr(nua)), h)


class MPMSimulation:
    """MPMSimulation<dim> (src/nclr.h:63-384) running on the GPU."""
    kBoundary = 3
    kSnowHardening = 10.0
    kJellyHardening = 0.3
    kLiquidHardening = 1.0

    def __init__(self, particles, model: MaterialModel | int, res: int = 64, dt: float = 1e-4,
                 E: float = 1e4, nu: float = 0.2, gravity: float = -100.0, *, dim: int | None = None,
                 material: np.ndarray | None = None, physics: int = capi.PHYSICS_REFERENCE,
                 sort_interval: int = 8, particles_per_thread: int = 1, device: int = 0,
                 use_graphs: bool = True, profile: bool = False, graph_steps: int = 0,
                 sparse_block_max: int = -1, small_scene_max: int = -1,
                 stress_model: int = capi.STRESS_COROTATED, tail_max: int = -1):
        L = capi.lib()
        self.dim, soa = _soa_from(particles, dim)
        self._c = soa.pop("c")
        self._mass = soa["mass"] if soa["mass"] is not None else np.ones(len(self._c), np.float32)
        self._volume = soa["volume"] if soa["volume"] is not None else np.ones(len(self._c), np.float32)
        self.n = soa["x"].shape[0]
        self.res = int(res)
        self.model = MaterialModel(int(model))
        mat = None if material is None else np.ascontiguousarray(material, dtype=np.uint8)
        opt = capi.default_options(physics=physics, sort_interval=sort_interval,
                                   p2g_particles_per_thread=particles_per_thread, device=device,
                                   use_graphs=int(use_graphs), profile=int(profile),
                                   graph_steps=graph_steps, sparse_block_max=sparse_block_max,
                                   small_scene_max=small_scene_max, stress_model=stress_model,
                                   tail_max=tail_max)
        h = ctypes.c_void_p()
        st = L.nclr_create(ctypes.byref(h), self.dim, self.n, _ptr(soa["x"]), _ptr(soa["v"]),
                           _ptr(soa["F"]), _ptr(soa["C"]), _ptr(soa["Jp"]), _ptr(soa["mass"]),
                           _ptr(soa["volume"]), _ptr(mat), int(self.model), self.res, float(dt),
                           float(E), float(nu), float(gravity), ctypes.byref(opt))
        capi.check(st, None)
        self._h = h
        mu, lam = ctypes.c_float(), ctypes.c_float()
        capi.check(L.nclr_get_lame(h, ctypes.byref(mu), ctypes.byref(lam)), h)
        self.mu_0, self.lambda_0 = float(mu.value), float(lam.value)
        self._stepped = False

    @classmethod
    def from_device(cls, x, model: MaterialModel | int, res: int = 64, dt: float = 1e-4,
                    E: float = 1e4, nu: float = 0.2, gravity: float = -100.0, *, v=None, F=None,
                    C=None, Jp=None, mass=None, volume=None, material=None,
                    physics: int = capi.PHYSICS_REFERENCE, sort_interval: int = 8,
                    device: int | None = None, use_graphs: bool = True, profile: bool = False,
                    graph_steps: int = 0, sparse_block_max: int = -1,
                    small_scene_max: int = -1,
                    stress_model: int = capi.STRESS_COROTATED, tail_max: int = -1) -> "MPMSimulation":
        """A simulation created from CUDA tensors (nclr_create_device): x (n, dim) and the
        optional fields in the layouts of the constructor, already on the GPU (e.g. from
        scenes.cubes_device), never staged through the host."""
        import torch
        L = capi.lib()
        if not (isinstance(x, torch.Tensor) and x.is_cuda):
            raise TypeError("from_device takes CUDA tensors")
        n, dim = x.shape
        dev = x.device.index if device is None else device

        def ptr(t, dtype=torch.float32):
            if t is None:
                return None
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == dtype and t.is_contiguous()):
                raise TypeError("device arrays must be contiguous CUDA tensors of the field's type")
            return ctypes.c_void_p(t.data_ptr())
        self = cls.__new__(cls)
        self.dim, self.n, self.res = int(dim), int(n), int(res)
        self.model = MaterialModel(int(model))
        self._c = np.zeros(n, np.int32)
        self._mass = (mass.cpu().numpy().astype(np.float32) if mass is not None
                      else np.ones(n, np.float32))
        self._volume = (volume.cpu().numpy().astype(np.float32) if volume is not None
                        else np.ones(n, np.float32))
        opt = capi.default_options(physics=physics, sort_interval=sort_interval, device=dev,
                                   use_graphs=int(use_graphs), profile=int(profile),
                                   graph_steps=graph_steps, sparse_block_max=sparse_block_max,
                                   small_scene_max=small_scene_max, stress_model=stress_model,
                                   tail_max=tail_max)
        h = ctypes.c_void_p()
        st = L.nclr_create_device(ctypes.byref(h), self.dim, self.n, ptr(x.contiguous()), ptr(v),
                                  ptr(F), ptr(C), ptr(Jp), ptr(mass), ptr(volume),
                                  ptr(material, torch.uint8), int(self.model), self.res,
                                  float(dt), float(E), float(nu), float(gravity),
                                  ctypes.byref(opt))
        capi.check(st, None)
        self._h = h
        mu, lam = ctypes.c_float(), ctypes.c_float()
        capi.check(L.nclr_get_lame(h, ctypes.byref(mu), ctypes.byref(lam)), h)
        self.mu_0, self.lambda_0 = float(mu.value), float(lam.value)
        self._stepped = False
        return self

    # -- the reference's API ------------------------------------------------------------
    def advance(self, steps: int = 1) -> None:
        """advance() (src/nclr.h:80-84), `steps` times."""
        capi.check(capi.lib().nclr_advance(self._h, int(steps)), self._h)
        self._stepped = True

    def particles(self) -> ParticleArrays:
        n, d = self.n, self.dim
        x = np.empty((n, d), np.float32); v = np.empty((n, d), np.float32)
        F = np.empty((n, d, d), np.float32); C = np.empty((n, d, d), np.float32)
        Jp = np.empty((n,), np.float32)
        capi.check(capi.lib().nclr_get_particles(self._h, _ptr(x), _ptr(v), _ptr(F), _ptr(C),
                                                 _ptr(Jp)), self._h)
        return ParticleArrays(x, v, F, C, Jp, self._mass.copy(), self._volume.copy(), self._c.copy())

    def grid(self) -> GridArrays:
        if not self._stepped:
            return GridArrays(np.zeros((0, self.dim), np.float32), np.zeros((0,), np.float32))
        nodes = (self.res + 1) ** self.dim
        vel = np.empty((nodes, self.dim), np.float32)
        mass = np.empty((nodes,), np.float32)
        capi.check(capi.lib().nclr_get_grid(self._h, _ptr(vel), _ptr(mass)), self._h)
        return GridArrays(vel, mass)

    # -- extensions ----------------------------------------------------------------------
    def set_particles(self, x=None, v=None, F=None, C=None, Jp=None) -> None:
        """Replaces fields of the particle state (caller order; None keeps a field)."""
        n, d = self.n, self.dim
        arr = lambda a, s: None if a is None else np.ascontiguousarray(np.asarray(a, np.float32).reshape(s))  # noqa: E731
        x, v, F, C, Jp = arr(x, (n, d)), arr(v, (n, d)), arr(F, (n, d, d)), arr(C, (n, d, d)), arr(Jp, (n,))
        capi.check(capi.lib().nclr_set_particles(self._h, _ptr(x), _ptr(v), _ptr(F), _ptr(C),
                                                 _ptr(Jp)), self._h)

    def set_moduli(self, E=None, nu=None) -> None:
        """Per-particle Young's modulus and Poisson ratio (nclr_set_moduli): `E`, `nu` hold one
        value per particle in caller order (numpy arrays or sequences, or contiguous float32
        CUDA tensors); both None return to the simulation's pair."""
        _set_moduli(self._h, self.n, E, nu)

    def get_particles_device(self, x=0, v=0, F=0, C=0, Jp=0) -> None:
        """Device-pointer export (integers = device addresses, 0 skips); stream-ordered."""
        capi.check(capi.lib().nclr_get_particles_device(self._h, x or None, v or None, F or None,
                                                        C or None, Jp or None), self._h)

    def set_particles_device(self, x=0, v=0, F=0, C=0, Jp=0) -> None:
        capi.check(capi.lib().nclr_set_particles_device(self._h, x or None, v or None, F or None,
                                                        C or None, Jp or None), self._h)

    @property
    def stream(self) -> int:
        return int(capi.lib().nclr_stream(self._h) or 0)

    def stats(self) -> tuple[int, int]:
        a, b = ctypes.c_int64(), ctypes.c_int64()
        capi.check(capi.lib().nclr_stats(self._h, ctypes.byref(a), ctypes.byref(b)), self._h)
        return int(a.value), int(b.value)

    def active_nodes(self) -> int:
        """Grid nodes that received mass in the last step's P2G."""
        a = ctypes.c_int64()
        capi.check(capi.lib().nclr_count_active_nodes(self._h, ctypes.byref(a)), self._h)
        return int(a.value)

    def profile(self) -> dict:
        """Per kernel phase: (total device ms, launches) since the last reset (profile=True)."""
        out = {}
        for i, name in enumerate(capi.PHASE_NAMES):
            ms, n = ctypes.c_double(), ctypes.c_int64()
            capi.check(capi.lib().nclr_profile_get(self._h, i, ctypes.byref(ms), ctypes.byref(n)),
                       self._h)
            out[name] = (float(ms.value), int(n.value))
        return out

    def profile_reset(self) -> None:
        capi.check(capi.lib().nclr_profile_reset(self._h), self._h)

    def close(self) -> None:
        if getattr(self, "_h", None):
            capi.lib().nclr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class BatchSimulation:
    """Many independent simulations stepped together (nclr_batch_create): every kernel of a
    step covers all scenes in one launch.  `scenes` is a list of dicts with the particle
    arrays (x, and optionally v, F, C, Jp, mass, volume, material) and the parameters model,
    res, dt, E, nu, gravity (the MPMSimulation defaults apply to missing ones)."""

    def __init__(self, scenes: list, *, dim: int | None = None,
                 physics: int = capi.PHYSICS_REFERENCE, sort_interval: int = 8, device: int = 0,
                 use_graphs: bool = True, graph_steps: int = 0, profile: bool = False,
                 small_scene_max: int = -1, particles_per_thread: int = 1,
                 stress_model: int = capi.STRESS_COROTATED, sparse_block_max: int = -1,
                 batch_item_threads: int = 0):
        L = capi.lib()
        if not scenes:
            raise ValueError("a batch needs at least one scene")
        self._keep = []
        descs = (capi.Scene * len(scenes))()
        self.dims = []
        self.sizes = []
        self.res = []
        for i, sc in enumerate(scenes):
            d, soa = _soa_from(sc, dim)
            self.dims.append(d)
            soa.pop("c")
            mat = sc.get("material")
            mat = None if mat is None else np.ascontiguousarray(mat, dtype=np.uint8)
            self._keep.append((soa, mat))
            descs[i].n = soa["x"].shape[0]
            for k in ("x", "v", "F", "C", "Jp", "mass", "volume"):
                setattr(descs[i], k, _ptr(soa[k]))
            descs[i].material = _ptr(mat)
            descs[i].model = int(sc.get("model", 0))
            descs[i].res = int(sc.get("res", 64))
            descs[i].dt = float(sc.get("dt", 1e-4))
            descs[i].E = float(sc.get("E", 1e4))
            descs[i].nu = float(sc.get("nu", 0.2))
            descs[i].gravity = float(sc.get("gravity", -100.0))
            self.sizes.append(int(descs[i].n))
            self.res.append(int(descs[i].res))
        if len(set(self.dims)) != 1:
            raise ValueError("all scenes of a batch have the same dimension")
        self.dim = self.dims[0]
        opt = capi.default_options(physics=physics, sort_interval=sort_interval, device=device,
                                   use_graphs=int(use_graphs), profile=int(profile),
                                   graph_steps=graph_steps, small_scene_max=small_scene_max,
                                   p2g_particles_per_thread=particles_per_thread,
                                   stress_model=stress_model, sparse_block_max=sparse_block_max,
                                   batch_item_threads=batch_item_threads)
        h = ctypes.c_void_p()
        capi.check(L.nclr_batch_create(ctypes.byref(h), self.dim, len(scenes), descs,
                                       ctypes.byref(opt)), None)
        self._h = h
        self._keep = None
        self._stepped = False

    def __len__(self):
        return len(self.sizes)

    def set_moduli(self, E=None, nu=None) -> None:
        """Per-particle Young's modulus and Poisson ratio of every scene's particles, the
        scenes concatenated in order (see MPMSimulation.set_moduli)."""
        _set_moduli(self._h, sum(self.sizes), E, nu)

    def advance(self, steps: int = 1) -> None:
        capi.check(capi.lib().nclr_advance(self._h, int(steps)), self._h)
        self._stepped = True

    def particles(self, scene: int) -> dict:
        n, d = self.sizes[scene], self.dim
        out = {"x": np.empty((n, d), np.float32), "v": np.empty((n, d), np.float32),
               "F": np.empty((n, d, d), np.float32), "C": np.empty((n, d, d), np.float32),
               "Jp": np.empty((n,), np.float32)}
        capi.check(capi.lib().nclr_scene_get_particles(self._h, scene, *(_ptr(out[k]) for k in
                                                                         ("x", "v", "F", "C", "Jp"))),
                   self._h)
        return out

    def set_particles(self, scene: int, x=None, v=None, F=None, C=None, Jp=None) -> None:
        n, d = self.sizes[scene], self.dim
        arr = lambda a, s: None if a is None else np.ascontiguousarray(np.asarray(a, np.float32).reshape(s))  # noqa: E731
        vals = [arr(x, (n, d)), arr(v, (n, d)), arr(F, (n, d, d)), arr(C, (n, d, d)), arr(Jp, (n,))]
        capi.check(capi.lib().nclr_scene_set_particles(self._h, scene, *(_ptr(a) for a in vals)),
                   self._h)

    def grid(self, scene: int) -> GridArrays:
        if not self._stepped:
            return GridArrays(np.zeros((0, self.dim), np.float32), np.zeros((0,), np.float32))
        nodes = (self.res[scene] + 1) ** self.dim
        vel = np.empty((nodes, self.dim), np.float32)
        mass = np.empty((nodes,), np.float32)
        capi.check(capi.lib().nclr_scene_get_grid(self._h, scene, _ptr(vel), _ptr(mass)), self._h)
        return GridArrays(vel, mass)

    def status(self, scene: int) -> int:
        return int(capi.lib().nclr_scene_status(self._h, scene))

    @property
    def stream(self) -> int:
        return int(capi.lib().nclr_stream(self._h) or 0)

    def stats(self) -> tuple[int, int]:
        a, b = ctypes.c_int64(), ctypes.c_int64()
        capi.check(capi.lib().nclr_stats(self._h, ctypes.byref(a), ctypes.byref(b)), self._h)
        return int(a.value), int(b.value)

    def active_nodes(self) -> int:
        """Grid nodes of all scenes with mass > 0 after the last step."""
        a = ctypes.c_int64()
        capi.check(capi.lib().nclr_count_active_nodes(self._h, ctypes.byref(a)), self._h)
        return int(a.value)

    def profile(self) -> dict:
        out = {}
        for i, name in enumerate(capi.PHASE_NAMES):
            ms, n = ctypes.c_double(), ctypes.c_int64()
            capi.check(capi.lib().nclr_profile_get(self._h, i, ctypes.byref(ms), ctypes.byref(n)),
                       self._h)
            out[name] = (float(ms.value), int(n.value))
        return out

    def profile_reset(self) -> None:
        capi.check(capi.lib().nclr_profile_reset(self._h), self._h)

    def close(self) -> None:
        if getattr(self, "_h", None):
            capi.lib().nclr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
