"""Python handle of the resident simulation object (sg_sim in include/smilei_gb300.h).

A ``Simulation`` owns one periodic grid and its species on the GPU and runs
whole timesteps (gather, push, Esirkepov deposit, per-tile sort, J fold, Yee,
B centring) with the fused kernels of smilei_gb300/csrc/sim.cu.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check

FIELD_INDEX = {"Ex": 0, "Ey": 1, "Ez": 2, "Bx": 3, "By": 4, "Bz": 5, "Bx_m": 6, "By_m": 7, "Bz_m": 8,
               "Jx": 9, "Jy": 10, "Jz": 11}


class Simulation:
    def __init__(self, n_cells, cell_length, dt, form="mixed", tile=None, capacity_slack=0.25, use_graph=True,
                 boundaries=None):
        """boundaries: per dimension "periodic" (default) or "open" (2D: Silver-Mueller fields,
        particles removed when they leave)."""
        self.ndim = len(n_cells)
        self.n_cells = [int(n) for n in n_cells]
        self.cell_length = [float(c) for c in cell_length]
        self.dt = float(dt)
        self.form = form
        cfg = _lib.SimConfig()
        cfg.ndim = self.ndim
        cfg.form = _lib.FORM_MIXED if form == "mixed" else _lib.FORM_FP64
        for d in range(self.ndim):
            cfg.n_cells[d] = self.n_cells[d]
            cfg.cell_length[d] = self.cell_length[d]
            cfg.tile[d] = int(tile[d]) if tile else 0
        cfg.dt = self.dt
        cfg.capacity_slack = float(capacity_slack)
        cfg.use_graph = int(bool(use_graph))
        self.boundaries = list(boundaries) if boundaries else ["periodic"] * self.ndim
        for d, b in enumerate(self.boundaries):
            cfg.bc[d] = {"periodic": _lib.BC_PERIODIC, "open": _lib.BC_OPEN}[b]
        h = ctypes.c_void_p()
        check(_lib.lib().sg_sim_create(ctypes.byref(cfg), ctypes.byref(h)), "sg_sim_create")
        self._h = h
        self.species = []

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().sg_sim_destroy(self._h)
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

    def set_tile_queue(self, on: bool = True):
        """Particle kernel as a persistent grid taking tiles from a queue, densest first
        (on), or one CTA per tile (off, the default)."""
        check(_lib.lib().sg_sim_set_tile_queue(self._h, int(bool(on))), "set_tile_queue")

    def set_tma_staging(self, on: bool = True):
        """Field tile staged by the tensor memory accelerator (on: the default of the 3D
        mixed form with 4x4x4 periodic tiles) or by word copies (off)."""
        check(_lib.lib().sg_sim_set_tma_staging(self._h, int(bool(on))), "set_tma_staging")

    # -- species -----------------------------------------------------------
    def add_species(self, mass, charge, pusher, position, momentum, weight, name=None):
        """position[ndim, n], momentum[3, n], weight[n] as float64 numpy arrays (host) or CUDA tensors."""
        idx = ctypes.c_int()
        kind = _lib.PUSHERS[pusher] if isinstance(pusher, str) else int(pusher)
        if hasattr(position, "is_cuda") and position.is_cuda:
            n = int(position.shape[1])
            pos, mom, w = position.contiguous(), momentum.contiguous(), weight.contiguous()
            check(_lib.lib().sg_sim_add_species_device(self._h, float(mass), float(charge), kind, n, pos.data_ptr(),
                                                       mom.data_ptr(), w.data_ptr(), ctypes.byref(idx)),
                  "add_species")
        else:
            pos = np.ascontiguousarray(position, dtype=np.float64)
            mom = np.ascontiguousarray(momentum, dtype=np.float64)
            w = np.ascontiguousarray(weight, dtype=np.float64)
            n = int(pos.shape[1])
            check(_lib.lib().sg_sim_add_species(self._h, float(mass), float(charge), kind, n, pos.ctypes.data,
                                                mom.ctypes.data, w.ctypes.data, ctypes.byref(idx)), "add_species")
        self.species.append(dict(mass=mass, charge=charge, pusher=pusher,
                                 name=name if name is not None else f"species{idx.value}"))
        return idx.value

    def species_count(self, s: int) -> int:
        n = ctypes.c_int64()
        check(_lib.lib().sg_sim_species_count(self._h, s, ctypes.byref(n)), "species_count")
        return n.value

    def get_species(self, s: int):
        n = self.species_count(s)
        pos = np.zeros((self.ndim, n))
        mom = np.zeros((3, n))
        w = np.zeros(n)
        check(_lib.lib().sg_sim_get_species(self._h, s, pos.ctypes.data, mom.ctypes.data, w.ctypes.data),
              "get_species")
        return pos, mom, w

    def state_bytes(self, s: int) -> int:
        b = ctypes.c_size_t()
        check(_lib.lib().sg_sim_state_bytes(self._h, s, ctypes.byref(b)), "state_bytes")
        return b.value

    def packed_bytes(self, s: int) -> int:
        b = ctypes.c_size_t()
        check(_lib.lib().sg_sim_packed_bytes(self._h, s, ctypes.byref(b)), "packed_bytes")
        return b.value

    def pack_state(self, s: int, host_ptr: int):
        """Packed state of species s (tile counts + particles, no slack) to a host buffer of packed_bytes(s)."""
        check(_lib.lib().sg_sim_pack_state(self._h, s, host_ptr), "pack_state")

    def unpack_state(self, s: int, host_ptr: int):
        """Restores a packed state of species s into the current layout."""
        check(_lib.lib().sg_sim_unpack_state(self._h, s, host_ptr), "unpack_state")

    def step_host(self, s: int, host_in_ptr: int, host_out_ptr: int | None = None, chunks: int = 8):
        """One step of species s kept in host memory as a packed state: reads it from
        host_in_ptr, steps (the copy in overlaps the particle kernel over `chunks` tile
        ranges) and writes the new packed state to host_out_ptr (default: in place)."""
        out = host_in_ptr if host_out_ptr is None else host_out_ptr
        check(_lib.lib().sg_sim_step_host(self._h, s, host_in_ptr, out, int(chunks)), "step_host")

    def stream_timing(self):
        """Stage times (ms from the start) of the last step_host that packed while stepping:
        copy in, particle kernels, copy out and field update done."""
        a = (ctypes.c_float * 4)()
        check(_lib.lib().sg_sim_stream_timing(self._h, a), "stream_timing")
        return dict(copy_in=a[0], particles=a[1], copy_out=a[2], fields=a[3])

    def copy_state(self, s: int, host_ptr: int, to_device: bool):
        """Raw state of species s to/from a host buffer of state_bytes(s) bytes (pinned for async)."""
        check(_lib.lib().sg_sim_copy_state(self._h, s, host_ptr, int(bool(to_device))), "copy_state")

    # -- fields ------------------------------------------------------------
    def field_shape(self, name: str):
        sh = (ctypes.c_int * 3)()
        check(_lib.lib().sg_sim_field_shape(self._h, FIELD_INDEX[name], sh), "field_shape")
        return tuple(sh[d] for d in range(self.ndim))

    def get_field(self, name: str) -> np.ndarray:
        a = np.zeros(self.field_shape(name))
        check(_lib.lib().sg_sim_get_field(self._h, FIELD_INDEX[name], a.ctypes.data), "get_field")
        return a

    def set_field(self, name: str, value: np.ndarray):
        a = np.ascontiguousarray(value, dtype=np.float64)
        if a.shape != self.field_shape(name):
            raise ValueError(f"{name}: expected shape {self.field_shape(name)}, got {a.shape}")
        check(_lib.lib().sg_sim_set_field(self._h, FIELD_INDEX[name], a.ctypes.data), "set_field")

    # -- stepping ----------------------------------------------------------
    def step(self, n: int = 1):
        check(_lib.lib().sg_sim_step(self._h, int(n)), "step")

    def energy(self):
        """(Ukin, Uelm) as the reference's scalar diagnostics define them."""
        uk, ue = ctypes.c_double(), ctypes.c_double()
        check(_lib.lib().sg_sim_energy(self._h, ctypes.byref(uk), ctypes.byref(ue)), "energy")
        return uk.value, ue.value

    def species_scalars(self, s: int):
        """(Dens, Ntot, q * Dens, Ukin) of species s, as DiagnosticScalar sums them (FP64 on the device)."""
        a = np.zeros(4)
        check(_lib.lib().sg_sim_species_scalars(self._h, int(s), a.ctypes.data), "species_scalars")
        return tuple(float(v) for v in a)

    def field_energies(self):
        """0.5 V_cell sum F^2 for Ex, Ey, Ez, Bx_m, By_m, Bz_m (FP64 on the device)."""
        a = np.zeros(6)
        check(_lib.lib().sg_sim_field_energies(self._h, a.ctypes.data), "field_energies")
        return a

    def rho(self) -> np.ndarray:
        """FP64 charge density of all species (reference layout, primal, ghosts folded)."""
        a = np.zeros(tuple(n + 5 for n in self.n_cells))
        check(_lib.lib().sg_sim_get_rho(self._h, a.ctypes.data), "rho")
        return a

    def solve_poisson(self, max_error=1e-14, max_iter=50000):
        """Initial E from the particles' charge (FP64 CG); returns (iterations, final r.r/n)."""
        it, ctrl = ctypes.c_int(), ctypes.c_double()
        check(_lib.lib().sg_sim_solve_poisson(self._h, float(max_error), int(max_iter), ctypes.byref(it),
                                              ctypes.byref(ctrl)), "solve_poisson")
        return it.value, ctrl.value

    def charge_residual(self):
        """max|div E - rho| / max|rho| (rho minus its mean) from the current particles, FP64."""
        r, m = ctypes.c_double(), ctypes.c_double()
        check(_lib.lib().sg_sim_charge_residual(self._h, ctypes.byref(r), ctypes.byref(m)), "charge_residual")
        return r.value

    LASER_KEYS = ["a0", "omega", "waist", "focus_x", "focus_y", "polarization_phi", "ellipticity", "phase_offset",
                  "t_start", "t_duration", "t_center", "t_fwhm", "t_order"]

    def add_laser_gaussian2d(self, a0, waist, focus, t_fwhm, t_center=None, t_start=0.0, t_duration=1e300,
                             omega=1.0, polarization_phi=0.0, ellipticity=0.0, phase_offset=0.0, t_order=2.0):
        """Gaussian 2D laser entering through xmin (the reference's LaserGaussian2D with a
        tgaussian time envelope; t_center defaults to sqrt(2) * t_fwhm as in its LWFA example)."""
        vals = dict(a0=a0, omega=omega, waist=waist, focus_x=focus[0], focus_y=focus[1],
                    polarization_phi=polarization_phi, ellipticity=ellipticity, phase_offset=phase_offset,
                    t_start=t_start, t_duration=t_duration, t_center=t_center if t_center is not None else 2 ** 0.5 * t_fwhm,
                    t_fwhm=t_fwhm, t_order=t_order)
        a = np.array([float(vals[k]) for k in self.LASER_KEYS])
        check(_lib.lib().sg_sim_add_laser_gaussian2d(self._h, a.ctypes.data), "add_laser_gaussian2d")
        return vals

    def set_moving_window(self, time_start, velocity_x, shift_cells):
        """The reference's MovingWindow(time_start, velocity_x) moving by ``shift_cells``
        cells (its patch width along x) whenever (time_dual - time_start) * velocity_x
        exceeds the distance already moved."""
        check(_lib.lib().sg_sim_set_moving_window(self._h, float(time_start), float(velocity_x), int(shift_cells)),
              "set_moving_window")

    def window_state(self):
        """(cells moved, distance moved, number of shifts)."""
        n, s = ctypes.c_int64(), ctypes.c_int64()
        x = ctypes.c_double()
        check(_lib.lib().sg_sim_window_state(self._h, ctypes.byref(n), ctypes.byref(x), ctypes.byref(s)),
              "window_state")
        return n.value, x.value, s.value

    def set_species_profile(self, species, n0, ppc, x_vacuum=0.0, x_slope1=0.0, x_plateau=1e300, x_slope2=0.0,
                            temperature=0.0, seed=0):
        """Density profile for particle creation: the reference's trapezoidal(n0, xvacuum,
        xplateau, xslope1, xslope2) along x, ``ppc`` particles per cell at regular
        positions.  Returns the profile tuple (n0, x_vacuum, x_slope1, x_plateau, x_slope2)."""
        prof = np.array([n0, x_vacuum, x_slope1, x_plateau, x_slope2], dtype=np.float64)
        check(_lib.lib().sg_sim_set_species_profile(self._h, int(species), prof.ctypes.data, int(ppc),
                                                    float(temperature), int(seed)), "set_species_profile")
        return tuple(float(v) for v in prof)

    def set_species_radiation(self, species, tables, mlp=None, seed=0):
        """Monte-Carlo radiation reaction of ``species`` in every step (2D mixed form):
        ``tables`` a radiation.RadiationTables, ``mlp`` a validated radiation.PhotonChiMLP
        or None.  Both must stay alive while the simulation runs."""
        self._rad_refs = getattr(self, "_rad_refs", {})
        self._rad_refs[species] = (tables, mlp)
        check(_lib.lib().sg_sim_set_species_radiation(self._h, int(species), tables._h,
                                                      mlp._h if mlp is not None else None, int(seed) & 0xffffffff),
              "set_species_radiation")

    def radiation_stats(self, species):
        """(radiated energy, number of emissions) of a radiating species so far."""
        r, e = ctypes.c_double(), ctypes.c_ulonglong()
        check(_lib.lib().sg_sim_radiation_stats(self._h, int(species), ctypes.byref(r), ctypes.byref(e)),
              "radiation_stats")
        return r.value, e.value

    def set_species_photons(self, species, sampling=1, gamma_threshold=2.0, max_emissions=10, capacity=1 << 20):
        """Macro-photons of a radiating species (sg_sim_set_species_photons): emissions
        above gamma_threshold create `sampling` photons each in a device store of
        `capacity`, pushed every step; capacity 0 removes the store."""
        check(_lib.lib().sg_sim_set_species_photons(self._h, int(species), int(sampling), float(gamma_threshold),
                                                    int(max_emissions), int(capacity)), "set_species_photons")
        if not hasattr(self, "_ph_cap"):
            self._ph_cap = {}
        self._ph_cap[int(species)] = int(capacity)

    def get_photons(self, species):
        """(photons wanted so far, dict(pos[2, n], mom[3, n], weight, chi, tau)) of the n
        stored ones (n = min(count, capacity))."""
        c = ctypes.c_int64()
        check(_lib.lib().sg_sim_get_photons(self._h, int(species), ctypes.byref(c), None, None, None, None, None),
              "get_photons")
        n = min(c.value, getattr(self, "_ph_cap", {}).get(int(species), 0))
        pos, mom = np.zeros((2, n)), np.zeros((3, n))
        w, chi, tau = np.zeros(n), np.zeros(n), np.zeros(n)
        check(_lib.lib().sg_sim_get_photons(self._h, int(species), ctypes.byref(c), pos.ctypes.data, mom.ctypes.data,
                                            w.ctypes.data, chi.ctypes.data, tau.ctypes.data), "get_photons")
        return c.value, dict(pos=pos, mom=mom, weight=w, chi=chi, tau=tau)

    def fill_species(self, species, x0=0, x1=None):
        """Creates the species' particles in window cells [x0, x1) (default: the whole grid)."""
        x1 = self.n_cells[0] if x1 is None else x1
        check(_lib.lib().sg_sim_fill_species(self._h, int(species), int(x0), int(x1)), "fill_species")

    def layout_stats(self):
        """(segment re-layouts so far, particles that went through the spill list)."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        check(_lib.lib().sg_sim_layout_stats(self._h, ctypes.byref(a), ctypes.byref(b)), "layout_stats")
        return a.value, b.value

    def batch_stats(self):
        """(batched graphs launched, steps they made, 1 if the runtime refused batching)."""
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        check(_lib.lib().sg_sim_batch_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
              "batch_stats")
        return a.value, b.value, c.value

    def last_timing(self):
        """Device ms of the last step: (particles, fields, total) and kernel launches per step."""
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        n = ctypes.c_int()
        check(_lib.lib().sg_sim_last_timing(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                            ctypes.byref(n)), "last_timing")
        return a.value, b.value, c.value, n.value
