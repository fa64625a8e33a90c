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


def _stream_ranges(nt3, counts, chunks, periodic=True):
    L = _lib.lib()
    nd = len(nt3)
    ntiles = (ctypes.c_int * 3)(*(list(nt3) + [1] * (3 - nd)))
    c = (ctypes.c_int * len(counts))(*[int(v) for v in counts])
    ta, tb, pa = ((ctypes.c_int * (chunks + 1))() for _ in range(3))
    nr = ctypes.c_int()
    _lib.check(L.sg_stream_ranges(nd, ntiles, int(periodic), c, chunks, ta, tb, pa, ctypes.byref(nr)),
               "sg_stream_ranges")
    k = nr.value
    return list(ta[:k]), list(tb[:k]), list(pa[:k])


@pytest.mark.parametrize("nt3", [(4, 4, 4), (3, 4, 4), (5, 3, 7), (8, 2, 2), (6, 5), (3, 9)])
@pytest.mark.parametrize("chunks", [1, 2, 3, 5, 8, 32, 64])
def test_streamed_step_ranges_pack_only_final_tiles(nt3, chunks):
    """The streamed host step packs a tile range only after every tile that can send it
    particles (its 3^D neighbours, periodic wraps included) has stepped, and after every
    range before it in tile order is final (their packed offsets come first).  Checked
    by brute force over the library's own range plan (sg_stream_ranges, host only)."""
    import itertools
    import numpy as np
    rng = np.random.default_rng(len(nt3) * 100 + chunks)
    nt = int(np.prod(nt3))
    for _ in range(3):
        counts = rng.integers(0, 50, nt)
        counts[rng.random(nt) < 0.2] = 0  # empty tiles
        ta, tb, pa = _stream_ranges(nt3, counts, chunks)
        owner = np.full(nt, -1)
        for j, (a, b) in enumerate(zip(ta, tb)):
            assert a <= b
            owner[a:b] = j
        assert (owner >= 0).all()  # every tile in exactly one range
        assert all(0 <= p < len(ta) for p in pa)
        dims = list(nt3)
        for j, (a, b) in enumerate(zip(ta, tb)):
            assert pa[j] >= j
            for t in range(a, b):
                idx = np.unravel_index(t, dims)
                for off in itertools.product((-1, 0, 1), repeat=len(dims)):
                    src = np.ravel_multi_index([(i + o) % n for i, o, n in zip(idx, off, dims)], dims)
                    assert owner[src] <= pa[j], (j, t, int(src))
            for i in range(len(ta)):
                if i != j and tb[i] <= a and tb[i] > ta[i]:
                    assert pa[i] <= pa[j]  # tiles before range j are final no later than it


def test_streamed_step_ranges_without_packing():
    """An open boundary, or fewer than three x-slabs, keeps the copy out after the step."""
    ta, tb, pa = _stream_ranges((4, 4, 4), [1] * 64, 4, periodic=False)
    assert pa == [-1] * 4 and ta[0] == 0 and tb[-1] == 64
    ta, tb, pa = _stream_ranges((2, 4, 4), [1] * 32, 4)
    assert pa == [-1] * 4 and tb[-1] == 32
    with pytest.raises(RuntimeError):
        _stream_ranges((4, 4, 4), [1] * 64, 0)
