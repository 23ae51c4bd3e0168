"""ctypes binding of libnclr_gpu.so (include/nclr_gpu.h).

The library is built in-tree by nuclearmpm_gb300/build.py.  There is no fallback: if the
shared library is missing or fails to load, `lib()` raises, and so does everything above it.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnclr_gpu.so")

NCLR_OK, NCLR_ERR_INVALID, NCLR_ERR_OUT_OF_RANGE, NCLR_ERR_CUDA, NCLR_ERR_NO_DEVICE = range(5)
STATUS_NAMES = {0: "NCLR_OK", 1: "NCLR_ERR_INVALID", 2: "NCLR_ERR_OUT_OF_RANGE",
                3: "NCLR_ERR_CUDA", 4: "NCLR_ERR_NO_DEVICE"}
PHYSICS_REFERENCE, PHYSICS_CORRECTED = 0, 1
STRESS_COROTATED, STRESS_NEOHOOKEAN = 0, 1
(PHASE_SORT, PHASE_GRID, PHASE_P2G, PHASE_G2P2G, PHASE_ADJ_G2P, PHASE_ADJ_GRID, PHASE_ADJ_P2G,
 PHASE_SNOW_FIX) = range(8)
PHASE_NAMES = ("sort", "grid", "p2g", "g2p2g", "adj_g2p", "adj_grid", "adj_p2g", "snow_fix")
NOALLOC_MAX_NODES = 1 << 20


class Options(ctypes.Structure):
    _fields_ = [("physics", ctypes.c_int), ("sort_interval", ctypes.c_int),
                ("p2g_particles_per_thread", ctypes.c_int), ("device", ctypes.c_int),
                ("use_graphs", ctypes.c_int), ("profile", ctypes.c_int),
                ("graph_steps", ctypes.c_int), ("sparse_block_max", ctypes.c_int),
                ("small_scene_max", ctypes.c_int), ("stress_model", ctypes.c_int),
                ("batch_item_threads", ctypes.c_int), ("tail_max", ctypes.c_int)]


class Scene(ctypes.Structure):
    """nclr_scene: one simulation of a batch."""
    _fields_ = [("n", ctypes.c_int64), ("x", ctypes.c_void_p), ("v", ctypes.c_void_p),
                ("F", ctypes.c_void_p), ("C", ctypes.c_void_p), ("Jp", ctypes.c_void_p),
                ("mass", ctypes.c_void_p), ("volume", ctypes.c_void_p),
                ("material", ctypes.c_void_p), ("model", ctypes.c_int), ("res", ctypes.c_int),
                ("dt", ctypes.c_float), ("E", ctypes.c_float), ("nu", ctypes.c_float),
                ("gravity", ctypes.c_float)]


_fp = ctypes.POINTER(ctypes.c_float)
_vp = ctypes.c_void_p
_h = ctypes.c_void_p
_i64 = ctypes.c_int64

# name -> (restype, argtypes); every symbol include/nclr_gpu.h declares
SIGNATURES = {
    "nclr_default_options": (None, [ctypes.POINTER(Options)]),
    "nclr_create": (ctypes.c_int, [ctypes.POINTER(_h), ctypes.c_int, _i64, _vp, _vp, _vp, _vp, _vp,
                                   _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                   ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                   ctypes.POINTER(Options)]),
    "nclr_create_device": (ctypes.c_int, [ctypes.POINTER(_h), ctypes.c_int, _i64, _vp, _vp, _vp,
                                          _vp, _vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                          ctypes.c_float, ctypes.POINTER(Options)]),
    "nclr_cube_device": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                        _vp, _vp]),
    "nclr_cubes_device": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp,
                                         _vp]),
    "nclr_get_grid_device": (ctypes.c_int, [_h, _vp, _vp]),
    "nclr_render_device": (ctypes.c_int, [_vp, _i64, ctypes.c_int, _vp, ctypes.c_uint32,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_float, _vp, _vp]),
    "nclr_advance": (ctypes.c_int, [_h, _i64]),
    "nclr_batch_create": (ctypes.c_int, [ctypes.POINTER(_h), ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(Scene), ctypes.POINTER(Options)]),
    "nclr_num_scenes": (ctypes.c_int, [_h]),
    "nclr_scene_get_particles": (ctypes.c_int, [_h, ctypes.c_int, _vp, _vp, _vp, _vp, _vp]),
    "nclr_scene_set_particles": (ctypes.c_int, [_h, ctypes.c_int, _vp, _vp, _vp, _vp, _vp]),
    "nclr_scene_get_grid": (ctypes.c_int, [_h, ctypes.c_int, _vp, _vp]),
    "nclr_scene_status": (ctypes.c_int, [_h, ctypes.c_int]),
    "nclr_get_particles": (ctypes.c_int, [_h, _vp, _vp, _vp, _vp, _vp]),
    "nclr_set_particles": (ctypes.c_int, [_h, _vp, _vp, _vp, _vp, _vp]),
    "nclr_get_grid": (ctypes.c_int, [_h, _vp, _vp]),
    "nclr_get_particles_device": (ctypes.c_int, [_h, _vp, _vp, _vp, _vp, _vp]),
    "nclr_set_particles_device": (ctypes.c_int, [_h, _vp, _vp, _vp, _vp, _vp]),
    "nclr_get_lame": (ctypes.c_int, [_h, _fp, _fp]),
    "nclr_set_moduli": (ctypes.c_int, [_h, _vp, _vp]),
    "nclr_set_moduli_device": (ctypes.c_int, [_h, _vp, _vp]),
    "nclr_num_particles": (_i64, [_h]),
    "nclr_dim": (ctypes.c_int, [_h]),
    "nclr_res": (ctypes.c_int, [_h]),
    "nclr_num_nodes": (_i64, [_h]),
    "nclr_stream": (_vp, [_h]),
    "nclr_stats": (ctypes.c_int, [_h, ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "nclr_count_active_nodes": (ctypes.c_int, [_h, ctypes.POINTER(_i64)]),
    "nclr_profile_get": (ctypes.c_int, [_h, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(_i64)]),
    "nclr_profile_reset": (ctypes.c_int, [_h]),
    "nclr_debug_set_barrier": (ctypes.c_int, [_h, ctypes.c_uint, ctypes.c_uint]),
    "nclr_last_error": (ctypes.c_char_p, [_h]),
    "nclr_destroy": (None, [_h]),
    "nclr_rollout_create": (ctypes.c_int, [ctypes.POINTER(_h), ctypes.c_int, _i64, _vp, _vp, _vp,
                                           ctypes.c_int, ctypes.c_float, ctypes.c_float, _i64,
                                           ctypes.c_int, ctypes.POINTER(Options)]),
    "nclr_rollout_create_model": (ctypes.c_int, [ctypes.POINTER(_h), ctypes.c_int, _i64, _vp, _vp,
                                                 _vp, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                                 ctypes.c_float, _i64, ctypes.c_int,
                                                 ctypes.POINTER(Options)]),
    "nclr_rollout_forward": (ctypes.c_int, [_h, _vp, _vp, _vp, _vp, ctypes.c_float, ctypes.c_float,
                                            _vp, _vp, _vp, _vp]),
    "nclr_rollout_backward": (ctypes.c_int, [_h, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                             ctypes.POINTER(ctypes.c_double),
                                             ctypes.POINTER(ctypes.c_double)]),
    "nclr_rollout_forward_moduli": (ctypes.c_int, [_h, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                                   _vp, _vp]),
    "nclr_rollout_backward_moduli": (ctypes.c_int, [_h, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                                    _vp, _vp]),
    "nclr_rollout_timing": (ctypes.c_int, [_h, ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double)]),
    "nclr_rollout_profile_get": (ctypes.c_int, [_h, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(_i64)]),
    "nclr_rollout_profile_reset": (ctypes.c_int, [_h]),
    "nclr_rollout_stream": (_vp, [_h]),
    "nclr_rollout_error": (ctypes.c_char_p, [_h]),
    "nclr_rollout_destroy": (None, [_h]),
    "nclr_grid_transfer_noalloc": (ctypes.c_int, [ctypes.c_int, _i64, _vp, _vp, _vp, _vp, _vp, _vp,
                                                  _vp, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                                  ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                                  _vp, _vp, _vp, ctypes.c_char_p, ctypes.c_size_t]),
}

_LIB: ctypes.CDLL | None = None


def lib() -> ctypes.CDLL:
    """Loads libnclr_gpu.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.isfile(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                               "`python -m nuclearmpm_gb300.build` (needs nvcc)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


class NclrError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class OutOfRange(NclrError, IndexError):
    """The reference throws std::out_of_range when a stencil leaves the grid (src/nclr.h:163)."""


def check(status: int, handle=None) -> None:
    if status == NCLR_OK:
        return
    msg = (lib().nclr_last_error(handle) or b"").decode(errors="replace")
    if status == NCLR_ERR_OUT_OF_RANGE:
        raise OutOfRange(status, msg)
    raise NclrError(status, msg)


def default_options(**kw) -> Options:
    o = Options()
    lib().nclr_default_options(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, int(v))
    return o
