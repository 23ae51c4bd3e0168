"""CPU checks of the C ABI: the library loads, exports every symbol include/nclr_gpu.h
declares, and reports a missing GPU as an error (no compute without a GPU)."""
import ctypes
import os
import re

import pytest

from nuclearmpm_gb300 import MPMSimulation, NclrError, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "nclr_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nclr_[a-z_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported_and_bound():
    L = capi.lib()
    names = declared_symbols()
    assert len(names) >= 15
    for name in names:
        assert hasattr(L, name), name
        assert name in capi.SIGNATURES, name


def test_default_options():
    o = capi.default_options()
    assert (o.physics, o.sort_interval, o.p2g_particles_per_thread, o.device, o.use_graphs) == (0, 8, 1, 0, 1)
    assert (o.sparse_block_max, o.small_scene_max, o.tail_max) == (-1, -1, -1)
    assert o.stress_model == capi.STRESS_COROTATED


def test_invalid_arguments_are_rejected_before_touching_a_device():
    L = capi.lib()
    h = ctypes.c_void_p()
    assert L.nclr_create(ctypes.byref(h), 4, 0, None, None, None, None, None, None, None, None,
                         0, 64, 1e-4, 1e4, 0.2, -100.0, None) == capi.NCLR_ERR_INVALID
    assert b"dim" in L.nclr_last_error(None)
    assert L.nclr_create(ctypes.byref(h), 2, 5, None, None, None, None, None, None, None, None,
                         0, 64, 1e-4, 1e4, 0.2, -100.0, None) == capi.NCLR_ERR_INVALID
    assert L.nclr_advance(None, 1) == capi.NCLR_ERR_INVALID
    assert L.nclr_set_moduli(None, None, None) == capi.NCLR_ERR_INVALID


@pytest.mark.parametrize("dim,physics,stress", [
    (3, capi.PHYSICS_REFERENCE, capi.STRESS_NEOHOOKEAN),  # det F = 0 under diag(1,1,0)
    (2, capi.PHYSICS_REFERENCE, 7),
    (3, capi.PHYSICS_CORRECTED, -1),
])
def test_stress_model_is_validated_before_touching_a_device(dim, physics, stress):
    L = capi.lib()
    h = ctypes.c_void_p()
    opt = capi.default_options(physics=physics, stress_model=stress)
    assert L.nclr_create(ctypes.byref(h), dim, 0, None, None, None, None, None, None, None, None,
                         1, 16, 1e-4, 1e4, 0.2, -100.0, ctypes.byref(opt)) == capi.NCLR_ERR_INVALID
    assert b"stress" in L.nclr_last_error(None)


@pytest.mark.skipif(os.environ.get("CUDA_VISIBLE_DEVICES") is None and
                    os.path.exists("/dev/nvidia0"), reason="a GPU is present")
def test_no_device_is_an_error_not_a_fallback():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(NclrError) as e:
        MPMSimulation([], 0, dim=2)
    assert e.value.status in (capi.NCLR_ERR_NO_DEVICE, capi.NCLR_ERR_CUDA)
