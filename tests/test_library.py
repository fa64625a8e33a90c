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


def _cfg(ndim, form, n_cells, cl=0.1, dt=0.05, bc=None):
    cfg = _lib.SimConfig()
    cfg.ndim = ndim
    cfg.form = form
    for d in range(ndim):
        cfg.n_cells[d] = n_cells[d]
        cfg.cell_length[d] = cl
        cfg.bc[d] = (bc or [0] * ndim)[d]
    cfg.dt = dt
    cfg.capacity_slack = 0.25
    cfg.use_graph = 1
    return cfg


@pytest.mark.parametrize("ndim,n_cells,what", [
    (3, [2049, 64, 64], "too many cells in dimension 0"),   # 11-bit x node of the packed key
    (3, [64, 1025, 64], "too many cells in dimension 1"),   # 10-bit y node
    (3, [64, 64, 1025], "too many cells in dimension 2"),   # 10-bit z node
    (2, [65536, 64], None),                                  # 16 bits: 65536 periodic cells fit
    (3, [4, 64, 64], "at least 8 cells"),
])
def test_grid_limits_of_the_mixed_form_are_checked_before_any_allocation(ndim, n_cells, what):
    """The mixed form packs a particle's node into 32 bits (3D x:11 y:10 z:10, 2D 16:16):
    grids beyond that are refused with a message, before the library touches the GPU."""
    L = _lib.lib()
    h = ctypes.c_void_p()
    r = L.sg_sim_create(ctypes.byref(_cfg(ndim, _lib.FORM_MIXED, n_cells)), ctypes.byref(h))
    if what is None:
        # accepted by the checks: without a GPU the allocation then fails, with a GPU it succeeds
        if r == 0:
            L.sg_sim_destroy(h)
        else:
            assert "too many cells" not in _lib.last_error()
    else:
        assert r == -1 and what in _lib.last_error(), _lib.last_error()


def test_open_2d_grid_limit_counts_the_extra_node():
    L = _lib.lib()
    h = ctypes.c_void_p()
    r = L.sg_sim_create(ctypes.byref(_cfg(2, _lib.FORM_MIXED, [65536, 64], bc=[1, 0])), ctypes.byref(h))
    assert r == -1 and "too many cells in dimension 0" in _lib.last_error()


def test_other_configuration_errors():
    L = _lib.lib()
    h = ctypes.c_void_p()
    assert L.sg_sim_create(ctypes.byref(_cfg(3, _lib.FORM_MIXED, [16, 16, 16], bc=[1, 0, 0])), ctypes.byref(h)) == -1
    assert "open boundaries are implemented in 2D" in _lib.last_error()
    assert L.sg_sim_create(ctypes.byref(_cfg(2, _lib.FORM_FP64, [16, 16], dt=0.2)), ctypes.byref(h)) == -1
    assert "dt must be below every cell length" in _lib.last_error()
    assert L.sg_sim_create(ctypes.byref(_cfg(2, 7, [16, 16])), ctypes.byref(h)) == -1
    assert "unknown form" in _lib.last_error()
