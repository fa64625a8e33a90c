"""ctypes binding of libsmileigb300.so (the C ABI declared in include/smilei_gb300.h).

The library is the only compute path: there is no CPU fallback.  If it is
missing it is built with nvcc on first use; if that fails the import error is
raised to the caller.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

SG_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "particle out of reach", -4: "capacity overflow",
          -5: "invalid state", -6: "out of device memory"}

FORM_FP64 = 0
FORM_MIXED = 1
BC_PERIODIC = 0
BC_OPEN = 1
PUSHERS = {"boris": 0, "vay": 1, "higueracary": 2}


class SmileiGPUError(RuntimeError):
    def __init__(self, code: int, where: str, message: str):
        super().__init__(f"{where}: {ERRORS.get(code, code)} ({code}): {message}")
        self.code = code


class GridGeom(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int), ("n_prim", ctypes.c_int * 3), ("domain_begin", ctypes.c_int * 3),
                ("cell_length", ctypes.c_double * 3)]


class SimConfig(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int), ("form", ctypes.c_int), ("n_cells", ctypes.c_int * 3),
                ("cell_length", ctypes.c_double * 3), ("dt", ctypes.c_double), ("tile", ctypes.c_int * 3),
                ("capacity_slack", ctypes.c_double), ("use_graph", ctypes.c_int), ("bc", ctypes.c_int * 3)]


_VP = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_D = ctypes.c_double
_PP = ctypes.POINTER(ctypes.c_void_p)

_SIGNATURES = {
    "sg_last_error": (ctypes.c_char_p, []),
    "sg_version": (_I, []),
    "sg_interpolate_fields": (_I, [ctypes.POINTER(GridGeom), _PP, _I64, _VP, _VP, _VP, _VP, _VP, _VP]),
    "sg_push_particles": (_I, [_I, _I, _D, _D, _I64, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "sg_project_currents": (_I, [_I, ctypes.POINTER(GridGeom), _D, _I64, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _PP,
                                 _VP]),
    "sg_maxwell_ampere": (_I, [ctypes.POINTER(GridGeom), _D, _PP, _VP]),
    "sg_maxwell_faraday": (_I, [ctypes.POINTER(GridGeom), _D, _PP, _VP]),
    "sg_save_magnetic_fields": (_I, [ctypes.POINTER(GridGeom), _PP, _PP, _VP]),
    "sg_center_magnetic_fields": (_I, [ctypes.POINTER(GridGeom), _PP, _PP, _VP]),
    "sg_sort_particles": (_I, [_I, ctypes.POINTER(_I), ctypes.POINTER(_D), ctypes.POINTER(_D), _I64, _PP, _I, _VP,
                               _VP, _VP, _VP, _VP]),
    "sg_sort_particles_noalloc": (_I, [_I, ctypes.POINTER(_I), ctypes.POINTER(_D), ctypes.POINTER(_D), _I64, _PP,
                                       _I, _VP, _VP, _VP, _VP, _VP]),
    "sg_sim_create": (_I, [ctypes.POINTER(SimConfig), ctypes.POINTER(_VP)]),
    "sg_sim_destroy": (_I, [_VP]),
    "sg_sim_add_species": (_I, [_VP, _D, _D, _I, _I64, _VP, _VP, _VP, ctypes.POINTER(_I)]),
    "sg_sim_add_species_device": (_I, [_VP, _D, _D, _I, _I64, _VP, _VP, _VP, ctypes.POINTER(_I)]),
    "sg_sim_set_field": (_I, [_VP, _I, _VP]),
    "sg_sim_get_field": (_I, [_VP, _I, _VP]),
    "sg_sim_field_shape": (_I, [_VP, _I, ctypes.POINTER(_I)]),
    "sg_sim_step": (_I, [_VP, _I]),
    "sg_sim_species_count": (_I, [_VP, _I, ctypes.POINTER(_I64)]),
    "sg_sim_get_species": (_I, [_VP, _I, _VP, _VP, _VP]),
    "sg_sim_species_scalars": (_I, [_VP, _I, _VP]),
    "sg_sim_field_energies": (_I, [_VP, _VP]),
    "sg_sim_add_laser_gaussian2d": (_I, [_VP, _VP]),
    "sg_sim_layout_stats": (_I, [_VP, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "sg_sim_batch_stats": (_I, [_VP, ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_I)]),
    "sg_sim_set_species_photons": (_I, [_VP, _I, _I, _D, _I, _I64]),
    "sg_sim_get_photons": (_I, [_VP, _I, ctypes.POINTER(_I64), _VP, _VP, _VP, _VP, _VP]),
    "sg_sim_set_moving_window": (_I, [_VP, _D, _D, _I]),
    "sg_sim_window_state": (_I, [_VP, ctypes.POINTER(_I64), ctypes.POINTER(_D), ctypes.POINTER(_I64)]),
    "sg_sim_set_species_profile": (_I, [_VP, _I, _VP, _I, _D, ctypes.c_uint64]),
    "sg_sim_fill_species": (_I, [_VP, _I, _I, _I]),
    "sg_sim_set_species_radiation": (_I, [_VP, _I, _VP, _VP, ctypes.c_uint32]),
    "sg_sim_radiation_stats": (_I, [_VP, _I, ctypes.POINTER(_D), ctypes.POINTER(ctypes.c_ulonglong)]),
    "sg_sim_energy": (_I, [_VP, ctypes.POINTER(_D), ctypes.POINTER(_D)]),
    "sg_sim_last_timing": (_I, [_VP, ctypes.POINTER(_D), ctypes.POINTER(_D), ctypes.POINTER(_D),
                                ctypes.POINTER(_I)]),
    "sg_sim_set_stream": (_I, [_VP, _VP]),
    "sg_sim_set_tile_queue": (_I, [_VP, _I]),
    "sg_sim_set_tma_staging": (_I, [_VP, _I]),
    "sg_sim_state_bytes": (_I, [_VP, _I, ctypes.POINTER(ctypes.c_size_t)]),
    "sg_sim_packed_bytes": (_I, [_VP, _I, ctypes.POINTER(ctypes.c_size_t)]),
    "sg_sim_pack_state": (_I, [_VP, _I, _VP]),
    "sg_sim_unpack_state": (_I, [_VP, _I, _VP]),
    "sg_sim_step_host": (_I, [_VP, _I, _VP, _VP, _I]),
    "sg_sim_stream_timing": (_I, [_VP, ctypes.POINTER(ctypes.c_float)]),
    "sg_stream_ranges": (_I, [_I, _VP, _I, _VP, _I, _VP, _VP, _VP, ctypes.POINTER(_I)]),
    "sg_sim_get_rho": (_I, [_VP, _VP]),
    "sg_rad_tables_create": (_I, [_VP, _I, _D, _D, _VP, _I, _I, _D, _D, _VP, _VP, ctypes.POINTER(_VP)]),
    "sg_rad_tables_destroy": (_I, [_VP]),
    "sg_rad_tables_set_fp32_math": (_I, [_VP, _I]),
    "sg_rad_photon_chi": (_I, [_VP, _I64, _VP, _VP, _VP, _VP]),
    "sg_rad_production_yield": (_I, [_VP, _I64, _VP, _VP, _VP, _VP]),
    "sg_rad_monte_carlo": (_I, [_VP, _VP, _I64, _D, _D, _D, _VP, _VP, _VP, _VP, _VP, _VP, ctypes.c_uint32,
                                ctypes.c_uint32, ctypes.c_uint32, _VP, _VP, _VP]),
    "sg_rad_monte_carlo_photons": (_I, [_VP, _VP, _I, _I64, _D, _D, _D, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                                        ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _I, _D, _I, _I64,
                                        _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "sg_push_photons": (_I, [_I, _I64, _D, _VP, _VP, _VP, _VP]),
    "sg_mlp_create": (_I, [_I, ctypes.c_uint32, _D, _D, ctypes.POINTER(_VP)]),
    "sg_mlp_destroy": (_I, [_VP]),
    "sg_mlp_nparams": (_I, [_VP, ctypes.POINTER(_I)]),
    "sg_mlp_get_params": (_I, [_VP, _VP]),
    "sg_mlp_set_params": (_I, [_VP, _VP]),
    "sg_mlp_gradients": (_I, [_VP, _I, _VP, _VP, _VP, _VP]),
    "sg_mlp_train": (_I, [_VP, _VP, _I, _I, ctypes.c_float, ctypes.c_uint32, _VP, _VP]),
    "sg_mlp_validate": (_I, [_VP, _VP, _I, _I, _I, ctypes.c_float, _VP, ctypes.POINTER(_I)]),
    "sg_mlp_photon_chi": (_I, [_VP, _I64, _VP, _VP, _VP, _VP]),
    "sg_mlp_photon_chi_fp32": (_I, [_VP, _I64, _VP, _VP, _VP, _VP]),
    "sg_sim_solve_poisson": (_I, [_VP, _D, _I, ctypes.POINTER(_I), ctypes.POINTER(_D)]),
    "sg_sim_charge_residual": (_I, [_VP, ctypes.POINTER(_D), ctypes.POINTER(_D)]),
    "sg_sim_copy_state": (_I, [_VP, _I, _VP, _I]),
}


def declared_symbols() -> list[str]:
    """Entry points declared in include/smilei_gb300.h (parsed from the header)."""
    import re
    hdr = os.path.join(_build.ROOT, "include", "smilei_gb300.h")
    text = open(hdr).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(sg_\w+)\s*\(", text, re.M)))


def lib() -> ctypes.CDLL:
    """The loaded library (built on first use when missing or stale)."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            L = ctypes.CDLL(path)
            for name, (res, args) in _SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def last_error() -> str:
    return lib().sg_last_error().decode(errors="replace")


def check(code: int, where: str):
    if code != SG_OK:
        raise SmileiGPUError(code, where, last_error())


def ptr(t) -> int | None:
    """Device (or host) address of a torch tensor / numpy array, or None."""
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    return t.ctypes.data


def ptr_array(ts) -> ctypes.Array:
    return (ctypes.c_void_p * len(ts))(*[ptr(t) for t in ts])
