"""The C-ABI library builds, loads and exports every entry point its header declares.

No GPU is needed: only symbol lookup and argument validation (which returns an
error code before any CUDA call) are exercised.
"""
import ctypes

import pytest

from smilei_gb300 import _lib


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    declared = _lib.declared_symbols()
    assert len(declared) >= 20
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing


def test_every_declared_symbol_has_a_python_signature():
    missing = [s for s in _lib.declared_symbols() if s not in _lib._SIGNATURES]
    assert not missing, missing


def test_invalid_arguments_return_error_codes_without_a_gpu():
    L = _lib.lib()
    cfg = _lib.SimConfig()
    cfg.ndim = 5
    h = ctypes.c_void_p()
    assert L.sg_sim_create(ctypes.byref(cfg), ctypes.byref(h)) == -1
    assert "ndim" in _lib.last_error()
    assert L.sg_push_particles(7, 3, 0.1, 1.0, 10, None, None, None, None, None, None, None) == -1
    assert L.sg_interpolate_fields(None, None, 0, None, None, None, None, None, None) == -1
    g = _lib.GridGeom()
    g.ndim = 3
    assert L.sg_maxwell_ampere(ctypes.byref(g), 0.1, None, None) == -1


def test_check_raises_with_the_library_message():
    L = _lib.lib()
    cfg = _lib.SimConfig()
    cfg.ndim = 3
    cfg.form = 9
    h = ctypes.c_void_p()
    with pytest.raises(_lib.SmileiGPUError, match="unknown form"):
        _lib.check(L.sg_sim_create(ctypes.byref(cfg), ctypes.byref(h)), "sg_sim_create")
