"""CPU oracle for the PIC-step hot path -- TEST INFRASTRUCTURE ONLY.

This package is the checker.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg import it; the product package
``smilei_gb300`` never does, and fails loudly when its CUDA library is missing
instead of falling back here.

Two back ends with the same Python signatures:

* ``Oracle`` wraps ``oracle/pic_oracle.c`` (``liboracle.so``), a plain-C FP64
  restatement of the reference operators (each C function cites the reference
  file:line it follows);
* ``RefOps`` wraps ``oracle/_ref/libsmilei_ref_ops.so``, the reference's own
  operator sources compiled by ``oracle/build_ref.sh`` (only where the
  reference tree is present; used to make and check the golden fixtures).

Array conventions (the reference's): fields are C-contiguous float64 arrays in
x-major order with ghost cells; particles are SoA ``pos[ndim, n]``,
``mom[3, n]``; interpolator scratch ``E[3, n]``, ``B[3, n]``,
``iold[ndim, n]`` (int32) and ``delta[ndim, n]``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libsmilei_ref_ops.so")

# Yee staggering (dual flag per dimension) of each named component.
STAGGER = {
    "Ex": (1, 0, 0), "Ey": (0, 1, 0), "Ez": (0, 0, 1),
    "Bx": (0, 1, 1), "By": (1, 0, 1), "Bz": (1, 1, 0),
    "Jx": (1, 0, 0), "Jy": (0, 1, 0), "Jz": (0, 0, 1),
    "rho": (0, 0, 0),
}
PUSHERS = {"boris": 0, "vay": 1, "higueracary": 2}


def field_shape(ndim: int, n_prim, comp: str):
    """Extents of component ``comp`` on a grid whose primal extents (with ghosts) are ``n_prim``."""
    st = STAGGER[comp.replace("_m", "")]
    return tuple(int(n_prim[d]) + st[d] for d in range(ndim))


def build(force: bool = False) -> str:
    """Compile ``pic_oracle.c`` into ``liboracle.so`` (gcc, OpenMP, no FP contraction)."""
    src = os.path.join(HERE, "pic_oracle.c")
    srcs = [src, os.path.join(HERE, "rad_oracle.c"), os.path.join(HERE, "bc_oracle.c")]
    srcs = [s for s in srcs if os.path.exists(s)]
    if (not force and os.path.exists(LIB_PATH)
            and all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(s) for s in srcs)):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11",
           "-o", tmp] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def reference_src() -> str | None:
    """The reference's src/ directory: $SMILEI_REFERENCE_SRC, else the reference tree
    beside this checkout's parent, when either exists (it exists only where the
    reference was unpacked, never on a machine that only runs the tests)."""
    cands = [os.environ.get("SMILEI_REFERENCE_SRC"),
             os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference", "src")]
    for c in cands:
        if c and os.path.isdir(c):
            return c
    return None


def build_ref(src: str | None = None) -> str | None:
    """Compile the reference's operator sources (only where the reference tree exists)."""
    script = os.path.join(HERE, "build_ref.sh")
    src = src or reference_src()
    if src is None:
        return None
    subprocess.run(["bash", script, src], check=True, stdout=subprocess.DEVNULL)
    return REF_PATH if os.path.exists(REF_PATH) else None


LASER_KEYS = ["a0", "omega", "waist", "focus_x", "focus_y", "polarization_phi", "ellipticity", "phase_offset",
              "t_start", "t_duration", "t_center", "t_fwhm", "t_order"]


def laser_params(laser: dict) -> list:
    """The 13 numbers of bc_oracle.c's Gaussian 2D laser, in order."""
    return [float(laser[k]) for k in LASER_KEYS]


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _ptrs(arrs):
    return (ctypes.c_void_p * len(arrs))(*[_ptr(a) for a in arrs])


def _i32(v):
    return (ctypes.c_int * len(v))(*[int(x) for x in v])


def _d(v):
    return (ctypes.c_double * len(v))(*[float(x) for x in v])


class _Backend:
    """Shared numpy marshalling for the oracle and the compiled reference."""

    lib: ctypes.CDLL
    prefix: str

    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    # -- Interpolator -------------------------------------------------------
    def interpolate(self, ndim, n_prim, domain_begin, cell_length, fields, pos):
        """fields = [Ex, Ey, Ez, Bx_m, By_m, Bz_m]; returns (E[3,n], B[3,n], iold[ndim,n], delta[ndim,n])."""
        pos = _f64(pos)
        n = pos.shape[1]
        fields = [_f64(f) for f in fields]
        E = np.zeros((3, n)); B = np.zeros((3, n))
        iold = np.zeros((ndim, n), dtype=np.int32); delta = np.zeros((ndim, n))
        self._interpolate(ndim, n_prim, domain_begin, cell_length, fields, n, pos, E, B, iold, delta)
        return E, B, iold, delta

    # -- Pusher -------------------------------------------------------------
    def push(self, kind, ndim, dt, mass, pos, mom, charge, E, B):
        """Returns (pos, mom, invgf) after one push; inputs are not modified."""
        pos = _f64(pos).copy(); mom = _f64(mom).copy()
        charge = np.ascontiguousarray(charge, dtype=np.int16)
        n = mom.shape[1]
        invgf = np.zeros(n)
        k = PUSHERS[kind] if isinstance(kind, str) else int(kind)
        self._fn("push")(k, ndim, ctypes.c_double(dt), ctypes.c_double(mass), self._n(n), _ptr(pos), _ptr(mom),
                         _ptr(charge), _ptr(_f64(E)), _ptr(_f64(B)), _ptr(invgf))
        return pos, mom, invgf


class Oracle(_Backend):
    """The C restatement in ``pic_oracle.c``."""

    prefix = "or_"

    def __init__(self):
        build()
        self.lib = ctypes.CDLL(LIB_PATH)
        self.lib.or_window_shift_particles.restype = ctypes.c_int64
        self.lib.or_create_particles.restype = ctypes.c_int64

    @staticmethod
    def _n(n):
        return ctypes.c_int64(n)

    def _interpolate(self, ndim, n_prim, domain_begin, cell_length, fields, n, pos, E, B, iold, delta):
        dx_inv = [1.0 / c for c in cell_length]
        self.lib.or_interpolate(ndim, _i32(n_prim), _i32(domain_begin), _d(dx_inv), _ptrs(fields),
                                ctypes.c_int64(n), _ptr(pos), _ptr(E), _ptr(B), _ptr(iold), _ptr(delta))

    def project(self, mode, ndim, n_prim, domain_begin, cell_length, dt, pos, mom, weight, charge, invgf,
                iold, delta, J):
        """J = [Jx, Jy, Jz, rho] accumulated in place (arrays may be None when unused)."""
        pos = _f64(pos); n = pos.shape[1]
        J = [_f64(a) if a is not None else None for a in J]
        self.lib.or_project(mode, ndim, _i32(n_prim), _i32(domain_begin), _d(cell_length), ctypes.c_double(dt),
                            ctypes.c_int64(n), _ptr(pos), _ptr(_f64(mom)), _ptr(_f64(weight)),
                            _ptr(np.ascontiguousarray(charge, dtype=np.int16)),
                            _ptr(_f64(invgf) if invgf is not None else None),
                            _ptr(np.ascontiguousarray(iold, dtype=np.int32) if iold is not None else None),
                            _ptr(_f64(delta) if delta is not None else None), _ptrs(J))
        return J

    def maxwell(self, which, ndim, n_prim, cell_length, dt, F, periodic=False, n_cells=None):
        """which 0: Ampere, 1: Faraday.  F = [Ex,Ey,Ez,Bx,By,Bz,Jx,Jy,Jz] updated in place."""
        if which == 0:
            self.lib.or_maxwell_ampere(ndim, _i32(n_prim), _d(cell_length), ctypes.c_double(dt), _ptrs(F))
        else:
            self.lib.or_maxwell_faraday(ndim, _i32(n_prim), _d(cell_length), ctypes.c_double(dt), _ptrs(F),
                                        int(periodic), _i32(n_cells if n_cells is not None else [0, 0, 0]))
        return F

    def fold_periodic(self, ndim, arr, dual, n_cells, oversize=2):
        self.lib.or_fold_periodic(ndim, _i32(arr.shape), _i32(dual), _i32(n_cells), oversize, _ptr(arr))
        return arr

    def pic_step(self, ndim, n_cells, oversize, cell_length, dt, fields, species):
        """fields: dict Ex..Bz, Bx_m..Bz_m, Jx..Jz (float64, updated in place).
        species: list of dicts pos, mom, weight, charge, mass, pusher (pos/mom updated in place)."""
        order = ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Bx_m", "By_m", "Bz_m", "Jx", "Jy", "Jz"]
        farr = [fields[k] for k in order]
        for a in farr:
            assert a.dtype == np.float64 and a.flags.c_contiguous
        ns = len(species)
        npart = (ctypes.c_int64 * ns)(*[s["mom"].shape[1] for s in species])
        mass = _d([s["mass"] for s in species])
        pusher = _i32([PUSHERS[s["pusher"]] for s in species])
        for s in species:
            assert s["pos"].dtype == np.float64 and s["pos"].flags.c_contiguous
            assert s["mom"].dtype == np.float64 and s["mom"].flags.c_contiguous
        self.lib.or_pic_step(ndim, _i32(n_cells), oversize, _d(cell_length), ctypes.c_double(dt), _ptrs(farr),
                             ns, npart, mass, pusher, _ptrs([s["pos"] for s in species]),
                             _ptrs([s["mom"] for s in species]),
                             _ptrs([_f64(s["weight"]) for s in species]),
                             _ptrs([np.ascontiguousarray(s["charge"], dtype=np.int16) for s in species]))

    def pic_step_bc(self, n_cells, oversize, cell_length, dt, fields, species, periodic, laser=None, time_dual=0.0,
                    skip_x=False):
        """2D step with open boundaries (bc_oracle.c or_pic_step_bc).  periodic: (px, py) flags;
        laser: LASER_KEYS dict for a Gaussian laser on xmin, or None; skip_x: the window moves
        at the end of this step (no x boundary).  Species arrays are replaced by their
        compacted survivors (pos, mom, weight, charge)."""
        order = ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Bx_m", "By_m", "Bz_m", "Jx", "Jy", "Jz"]
        farr = [fields[k] for k in order]
        for a in farr:
            assert a.dtype == np.float64 and a.flags.c_contiguous
        ns = len(species)
        npart = (ctypes.c_int64 * ns)(*[s["mom"].shape[1] for s in species])
        mass = _d([s["mass"] for s in species])
        pusher = _i32([PUSHERS[s["pusher"]] for s in species])
        arrs = []
        for s in species:
            s["pos"] = np.ascontiguousarray(s["pos"], dtype=np.float64)
            s["mom"] = np.ascontiguousarray(s["mom"], dtype=np.float64)
            s["weight"] = np.ascontiguousarray(s["weight"], dtype=np.float64)
            s["charge"] = np.ascontiguousarray(s["charge"], dtype=np.int16)
            arrs.append(s)
        lz = _d(laser_params(laser)) if laser is not None else None
        self.lib.or_pic_step_bc(_i32(n_cells), oversize, _d(cell_length), ctypes.c_double(dt), _ptrs(farr), ns, npart,
                                mass, pusher, _ptrs([s["pos"] for s in arrs]), _ptrs([s["mom"] for s in arrs]),
                                _ptrs([s["weight"] for s in arrs]), _ptrs([s["charge"] for s in arrs]),
                                _i32(list(periodic)), lz, ctypes.c_double(time_dual), int(skip_x))
        for k, s in enumerate(arrs):
            m = int(npart[k])
            nd = s["pos"].shape[0]
            s["pos"] = s["pos"].ravel()[: nd * m].reshape(nd, m).copy()
            s["mom"] = s["mom"].ravel()[: 3 * m].reshape(3, m).copy()
            s["weight"] = s["weight"][:m].copy()
            s["charge"] = s["charge"][:m].copy()

    def window_shift(self, n_cells, oversize, cell_length, dt, fields, species, shift, periodic):
        """The moving window's shift by ``shift`` cells (bc_oracle.c or_window_shift_fields and
        or_window_shift_particles), then Silver-Mueller on xmin without laser, as
        SimWindow::shift does after building its new patches (SimWindow.cpp:420-431)."""
        order = ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Bx_m", "By_m", "Bz_m", "Jx", "Jy", "Jz"]
        ndim = len(n_cells)
        farr = [fields[k] for k in order]
        for a in farr:
            assert a.dtype == np.float64 and a.flags.c_contiguous
        assert self.lib.or_window_shift_fields(ndim, _i32(n_cells), oversize, shift, _ptrs(farr)) == 0
        n_prim = [n + 1 + 2 * oversize for n in n_cells]
        self.sm_apply_2d(0, n_prim, cell_length, dt, farr[:6], tmin=int(not periodic[1]), tmax=int(not periodic[1]))
        for s in species:
            n = s["weight"].size
            pos = np.ascontiguousarray(s["pos"], dtype=np.float64)
            mom = np.ascontiguousarray(s["mom"], dtype=np.float64)
            w = np.ascontiguousarray(s["weight"], dtype=np.float64)
            q = np.ascontiguousarray(s["charge"], dtype=np.int16)
            m = self.lib.or_window_shift_particles(ndim, ctypes.c_double(cell_length[0]), shift, ctypes.c_int64(n),
                                                   _ptr(pos), _ptr(mom), _ptr(w), q.ctypes.data_as(ctypes.c_void_p))
            s["pos"] = pos.ravel()[: ndim * m].reshape(ndim, m).copy()
            s["mom"] = mom.ravel()[: 3 * m].reshape(3, m).copy()
            s["weight"] = w[:m].copy()
            s["charge"] = q[:m].copy()

    def create_particles(self, n_cells, cell_length, x0, x1, n_moved, profile, ppc, temperature=0.0, seed=0):
        """Regular-position particles in window cells [x0, x1) (bc_oracle.c or_create_particles);
        profile = (n0, x_vacuum, x_slope1, x_plateau, x_slope2).  Returns (pos, mom, weight)."""
        ndim = len(n_cells)
        cap = max(1, (x1 - x0) * int(np.prod(n_cells[1:])) * ppc)
        pos = np.zeros((ndim, cap)); mom = np.zeros((3, cap)); w = np.zeros(cap)
        n = self.lib.or_create_particles(ndim, _i32(n_cells), _d(cell_length), x0, x1, ctypes.c_int64(n_moved),
                                         _d(list(profile)), ppc, ctypes.c_double(temperature),
                                         ctypes.c_uint64(seed), _ptr(pos), _ptr(mom), _ptr(w), ctypes.c_int64(cap))
        assert n >= 0, "ppc must be a square (2D) or a cube (3D)"
        return pos[:, :n].copy(), mom[:, :n].copy(), w[:n].copy()

    def run_window(self, n_cells, cell_length, dt, fields, species, periodic, nsteps, window, laser=None,
                   profiles=None, state=None):
        """``nsteps`` 2D steps with open boundaries and a moving window, in the order of the
        reference's main loop (Smilei.cpp:483-680): the step at time_dual = (k + 1.5) dt skips
        its x boundaries when the window is due to move (SimWindow::isMoving,
        SimWindow.cpp:93-96), then the window shifts by window["shift"] cells, lasers are
        switched off for good (laserDisabled, SimWindow.cpp:138-145) and the fresh cells
        are filled from each species' profile.  window = {t_start, velocity, shift};
        profiles[s] = (profile, ppc, temperature, seed) or None; state (dict, updated)
        carries step, n_moved, x_moved and laser_off between calls."""
        st = state if state is not None else {}
        st.setdefault("step", 0); st.setdefault("n_moved", 0); st.setdefault("x_moved", 0.0)
        st.setdefault("laser_off", False)
        P = window["shift"]
        for _ in range(nsteps):
            td = (st["step"] + 1.5) * dt
            moving = (td - window["t_start"]) * window["velocity"] > st["x_moved"]
            self.pic_step_bc(n_cells, 2, cell_length, dt, fields, species, periodic,
                             None if st["laser_off"] else laser, td, skip_x=moving)
            if moving:
                st["n_moved"] += P
                st["laser_off"] = True
                self.window_shift(n_cells, 2, cell_length, dt, fields, species, P, periodic)
                for s, pr in zip(species, profiles or [None] * len(species)):
                    if pr is None:
                        continue
                    profile, ppc, temp, seed = pr
                    pos, mom, w = self.create_particles(n_cells, cell_length, n_cells[0] - P, n_cells[0],
                                                        st["n_moved"], profile, ppc, temp, seed)
                    s["pos"] = np.concatenate([s["pos"], pos], axis=1)
                    s["mom"] = np.concatenate([s["mom"], mom], axis=1)
                    s["weight"] = np.concatenate([s["weight"], w])
                    q = int(s["charge"][0]) if s["charge"].size else int(s.get("q", -1))
                    s["charge"] = np.concatenate([s["charge"], np.full(w.size, q, np.int16)])
                st["x_moved"] += cell_length[0] * P
            st["step"] += 1
        return st

    def sm_apply_2d(self, side, n_prim, cell_length, dt, F, b1=None, b2=None, tmin=1, tmax=1, k=None):
        """One Silver-Mueller side on F = [Ex, Ey, Ez, Bx, By, Bz] (updated in place)."""
        kdef = [(1.0, 0.0), (-1.0, 0.0), (0.0, 1.0), (0.0, -1.0)][side]
        self.lib.or_sm_apply_2d(side, _i32(n_prim), _d(cell_length), ctypes.c_double(dt), _d(k or kdef), _ptrs(F),
                                _ptr(b1) if b1 is not None else None, _ptr(b2) if b2 is not None else None, tmin, tmax)

    def laser_gaussian2d(self, laser, y, profile, t):
        """Separable amplitude of a Gaussian 2D laser (profile 0: primal points, 1: dual) at y, time t."""
        y = _f64(y)
        out = np.zeros_like(y)
        self.lib.or_laser_gaussian2d(_d(laser_params(laser)), y.size, _ptr(y), profile, ctypes.c_double(t), _ptr(out))
        return out

    def sort(self, ndim, patch_size, xmin, cell_length, pos):
        """Per-cell sort: returns (keys, first_index, last_index, perm)."""
        pos = _f64(pos); n = pos.shape[1]
        keys = np.zeros(n, dtype=np.int32)
        self.lib.or_sort_keys(ndim, _i32(patch_size), _d(xmin), _d([1.0 / c for c in cell_length]),
                              ctypes.c_int64(n), _ptr(pos), _ptr(keys))
        ncell = int(np.prod([p + 1 for p in patch_size]))
        first = np.zeros(ncell, dtype=np.int32); last = np.zeros(ncell, dtype=np.int32)
        perm = np.zeros(n, dtype=np.int64)
        self.lib.or_sort_bins(ctypes.c_int64(n), _ptr(keys), ncell, _ptr(first), _ptr(last), _ptr(perm))
        return keys, first, last, perm


class RefOps(_Backend):
    """The reference's own operators, compiled by ``build_ref.sh``."""

    prefix = "ref_"

    def __init__(self, path: str = REF_PATH):
        self.lib = ctypes.CDLL(path, mode=os.RTLD_LAZY)

    @staticmethod
    def _n(n):
        return ctypes.c_int(n)

    @staticmethod
    def _patch(ndim, n_prim, oversize=2):
        return _i32([n_prim[d] - 1 - 2 * oversize for d in range(ndim)]), _i32([oversize] * ndim)

    def _interpolate(self, ndim, n_prim, domain_begin, cell_length, fields, n, pos, E, B, iold, delta):
        cells, os_ = self._patch(ndim, n_prim)
        self.lib.ref_interpolate(ndim, cells, os_, _i32(domain_begin), _d(cell_length), _ptrs(fields), n,
                                 _ptr(pos), _ptr(E), _ptr(B), _ptr(iold), _ptr(delta))

    def project(self, mode, ndim, n_prim, domain_begin, cell_length, dt, pos, mom, weight, charge, invgf,
                iold, delta, J):
        pos = _f64(pos); n = pos.shape[1]
        cells, os_ = self._patch(ndim, n_prim)
        J = [_f64(a) for a in J]
        self.lib.ref_project(mode, ndim, cells, os_, _i32(domain_begin), _d(cell_length), ctypes.c_double(dt), n,
                             _ptr(pos), _ptr(_f64(mom)), _ptr(_f64(weight)),
                             _ptr(np.ascontiguousarray(charge, dtype=np.int16)),
                             _ptr(_f64(invgf) if invgf is not None else None),
                             _ptr(np.ascontiguousarray(iold, dtype=np.int32) if iold is not None else None),
                             _ptr(_f64(delta) if delta is not None else None), _ptrs(J))
        return J

    def maxwell(self, which, ndim, n_prim, cell_length, dt, F):
        cells, os_ = self._patch(ndim, n_prim)
        self.lib.ref_maxwell(which, ndim, cells, os_, _d(cell_length), ctypes.c_double(dt), _ptrs(F))
        return F

    def sm_apply_2d(self, side, n_prim, cell_length, dt, F, tmin=1, tmax=1, laser=None, time_dual=0.0):
        """The reference's ElectroMagnBC2D_SM::apply on F = [Ex..Bz] (in place).  laser: dict with
        lt = [start, end, invsigma, center, order], omega, sp1/ph1 (primal points), d1, sp2/ph2 (dual), d2."""
        cells, os_ = self._patch(2, n_prim)
        F = [_f64(a) for a in F]
        if laser is None:
            self.lib.ref_sm_apply_2d(side, cells, os_, _d(cell_length), ctypes.c_double(dt), _ptrs(F), tmin, tmax,
                                     None, ctypes.c_double(1.0), None, None, ctypes.c_double(0.0), None, None,
                                     ctypes.c_double(0.0), ctypes.c_double(time_dual))
        else:
            L = {k: (_f64(v) if isinstance(v, np.ndarray) else v) for k, v in laser.items()}
            self.lib.ref_sm_apply_2d(side, cells, os_, _d(cell_length), ctypes.c_double(dt), _ptrs(F), tmin, tmax,
                                     _d(L["lt"]), ctypes.c_double(L["omega"]), _ptr(L["sp1"]), _ptr(L["ph1"]),
                                     ctypes.c_double(L["d1"]), _ptr(L["sp2"]), _ptr(L["ph2"]), ctypes.c_double(L["d2"]),
                                     ctypes.c_double(time_dual))
        return F

    # -- radiation tables --------------------------------------------------
    def rad_tables(self):
        isz = ctypes.c_int(); imin = ctypes.c_double(); imax = ctypes.c_double()
        xd = (ctypes.c_int * 2)(); xmin = ctypes.c_double(); xmax = ctypes.c_double()
        self.lib.ref_rad_table_info(ctypes.byref(isz), ctypes.byref(imin), ctypes.byref(imax), xd,
                                    ctypes.byref(xmin), ctypes.byref(xmax))
        integ = np.zeros(isz.value); xi = np.zeros((xd[0], xd[1])); amin = np.zeros(xd[0])
        self.lib.ref_rad_table_data(_ptr(integ), _ptr(xi), _ptr(amin))
        return dict(integfochi=integ, integfochi_min=imin.value, integfochi_max=imax.value,
                    xi=xi, xi_min=xmin.value, xi_max=xmax.value, xi_axis1_min=amin)

    def rad_yield(self, chi, gamma, factor):
        chi = _f64(chi); gamma = _f64(gamma); out = np.zeros_like(chi)
        self.lib.ref_rad_yield(len(chi), _ptr(chi), _ptr(gamma), ctypes.c_double(factor), _ptr(out))
        return out

    def rad_photon_chi(self, chi, xi):
        chi = _f64(chi); xi = _f64(xi); out = np.zeros_like(chi)
        self.lib.ref_rad_photon_chi(len(chi), _ptr(chi), _ptr(xi), _ptr(out))
        return out

    def rad_monte_carlo(self, factors, dt, mass, charge, pos, mom, weight, tau, E, B, seeds, sampling=0,
                        threshold=2.0, max_emissions=10):
        """The reference's RadiationMonteCarlo::operator() with the default tables, particle p
        drawing from Random(seeds[p]).  factors: dict(factor_dNph_dt, factor_classical,
        min_chi_continuous, min_chi_discontinuous, inv_norm_E_schwinger).  mom and tau are
        updated in place.  Returns (radiated, chi, photons) with photons = dict(pos, mom,
        weight, chi, tau) in creation order (None without a photon species, sampling = 0)."""
        pos = _f64(pos); ndim, n = pos.shape
        assert mom.dtype == np.float64 and mom.flags.c_contiguous and tau.dtype == np.float64
        chi = np.zeros(n)
        cap = max(1, n * max_emissions * max(sampling, 1))
        ph_pos = np.zeros((ndim, cap)); ph_mom = np.zeros((3, cap)); ph_w = np.zeros(cap)
        ph_chi = np.zeros(cap); ph_tau = np.zeros(cap)
        nph = ctypes.c_long(); rad = ctypes.c_double()
        seeds = np.ascontiguousarray(seeds, dtype=np.uint32)
        f = factors
        self.lib.ref_monte_carlo(ndim, n, ctypes.c_double(dt), ctypes.c_double(mass), ctypes.c_double(charge),
                                 ctypes.c_double(f["factor_dNph_dt"]), ctypes.c_double(f["factor_classical"]),
                                 ctypes.c_double(f["min_chi_continuous"]), ctypes.c_double(f["min_chi_discontinuous"]),
                                 ctypes.c_double(f["inv_norm_E_schwinger"]), _ptr(pos), _ptr(mom),
                                 _ptr(_f64(weight)), _ptr(tau), _ptr(chi), _ptr(_f64(E)), _ptr(_f64(B)),
                                 _ptr(seeds), sampling, ctypes.c_double(threshold), max_emissions,
                                 ctypes.c_long(cap), _ptr(ph_pos), _ptr(ph_mom), _ptr(ph_w), _ptr(ph_chi),
                                 _ptr(ph_tau), ctypes.byref(nph), ctypes.byref(rad))
        photons = None
        if sampling > 0:
            k = int(nph.value)
            assert k <= cap
            photons = dict(pos=ph_pos[:, :k].copy(), mom=ph_mom[:, :k].copy(), weight=ph_w[:k].copy(),
                           chi=ph_chi[:k].copy(), tau=ph_tau[:k].copy())
        return rad.value, chi, photons


class RadTablesC(ctypes.Structure):
    """Mirror of or_rad_tables in rad_oracle.c."""
    _fields_ = [("integ", ctypes.c_void_p), ("n_integ", ctypes.c_int), ("integ_log10_min", ctypes.c_double),
                ("integ_delta", ctypes.c_double), ("integ_inv_delta", ctypes.c_double),
                ("xi", ctypes.c_void_p), ("n_chi", ctypes.c_int), ("n_ph", ctypes.c_int),
                ("xi_log10_min", ctypes.c_double), ("xi_delta", ctypes.c_double), ("xi_inv_delta", ctypes.c_double),
                ("inv_nph_m1", ctypes.c_double), ("axis1_min", ctypes.c_void_p),
                ("factor_dNph_dt", ctypes.c_double), ("factor_classical", ctypes.c_double),
                ("min_chi_continuous", ctypes.c_double), ("min_chi_discontinuous", ctypes.c_double),
                ("inv_norm_E_schwinger", ctypes.c_double)]


class RadTables:
    """Monte-Carlo radiation tables in the reference's conventions (src/Radiation/Table.cpp:77-110).

    integfochi[n] on log10-spaced chi in [integ_min, integ_max]; xi[n_chi, n_ph] with the
    per-row log10 of the minimum photon chi (axis1_min); physical factors as
    RadiationTables::initialization computes them (RadiationTables.cpp:92-103)."""

    def __init__(self, integfochi, integ_min, integ_max, xi, xi_min, xi_max, axis1_min,
                 factor_dNph_dt=1.0, factor_classical=1.0, inv_norm_E_schwinger=1.0,
                 min_chi_continuous=1e-3, min_chi_discontinuous=1e-2):
        self.integfochi = _f64(integfochi)
        self.xi = _f64(xi)
        self.axis1_min = _f64(axis1_min)
        self.integ_min, self.integ_max = float(integ_min), float(integ_max)
        self.xi_min, self.xi_max = float(xi_min), float(xi_max)
        self.factor_dNph_dt = float(factor_dNph_dt)
        self.factor_classical = float(factor_classical)
        self.inv_norm_E_schwinger = float(inv_norm_E_schwinger)
        self.min_chi_continuous = float(min_chi_continuous)
        self.min_chi_discontinuous = float(min_chi_discontinuous)

    @staticmethod
    def axis(vmin, vmax, n):
        lmin = np.log10(vmin) if vmin != 0 else 0.0
        delta = (np.log10(vmax) - lmin) / (n - 1)
        return lmin, delta, 1.0 / delta

    def c_struct(self) -> RadTablesC:
        t = RadTablesC()
        t.integ = self.integfochi.ctypes.data
        t.n_integ = len(self.integfochi)
        t.integ_log10_min, t.integ_delta, t.integ_inv_delta = self.axis(self.integ_min, self.integ_max,
                                                                         len(self.integfochi))
        t.xi = self.xi.ctypes.data
        t.n_chi, t.n_ph = self.xi.shape
        t.xi_log10_min, t.xi_delta, t.xi_inv_delta = self.axis(self.xi_min, self.xi_max, self.xi.shape[0])
        t.inv_nph_m1 = 1.0 / (self.xi.shape[1] - 1)
        t.axis1_min = self.axis1_min.ctypes.data
        t.factor_dNph_dt = self.factor_dNph_dt
        t.factor_classical = self.factor_classical
        t.min_chi_continuous = self.min_chi_continuous
        t.min_chi_discontinuous = self.min_chi_discontinuous
        t.inv_norm_E_schwinger = self.inv_norm_E_schwinger
        return t

    @classmethod
    def from_golden(cls, g, **kw):
        return cls(g["integfochi"], g["integfochi_min"], g["integfochi_max"], g["xi_table"], g["xi_min"],
                   g["xi_max"], g["xi_axis1_min"], **kw)


def _rad_lib():
    L = Oracle().lib
    L.or_rad_monte_carlo.restype = ctypes.c_double
    L.or_rng_init.restype = ctypes.c_uint32
    return L


def rng_seeds(seed, first_id, step, n):
    """Initial xorshift32 state of each particle's random stream (rad_oracle.c or_rng_init)."""
    L = _rad_lib()
    return np.array([L.or_rng_init(ctypes.c_uint32(seed), ctypes.c_uint32((first_id + p) & 0xFFFFFFFF),
                                   ctypes.c_uint32(step)) for p in range(n)], dtype=np.uint32)


def rad_yield(tables: RadTables, chi, gamma):
    chi = _f64(chi); gamma = _f64(gamma); out = np.zeros_like(chi)
    ts = tables.c_struct()
    _rad_lib().or_rad_yield_n(ctypes.byref(ts), ctypes.c_int64(len(chi)), _ptr(chi), _ptr(gamma), _ptr(out))
    return out


def rad_photon_chi(tables: RadTables, chi, xi):
    chi = _f64(chi); xi = _f64(xi); out = np.zeros_like(chi)
    ts = tables.c_struct()
    _rad_lib().or_rad_photon_chi_n(ctypes.byref(ts), ctypes.c_int64(len(chi)), _ptr(chi), _ptr(xi), _ptr(out))
    return out


def rad_monte_carlo_photons(tables: RadTables, dt, mass, charge, pos, mom, weight, tau, E, B, seed, first_id=0,
                            step=0, sampling=1, threshold=2.0, max_emissions=10):
    """Monte-Carlo pass creating macro-photons (rad_oracle.c or_rad_monte_carlo_photons).
    Returns (radiated, n_emissions, chi, photons) with photons = dict(pos, mom, weight, chi, tau)
    in particle order."""
    n = mom.shape[1]
    ndim = pos.shape[0]
    assert mom.dtype == np.float64 and mom.flags.c_contiguous and tau.dtype == np.float64
    chi = np.zeros(n)
    nem, nph = ctypes.c_int64(), ctypes.c_int64()
    cap = max(1, n * max_emissions * sampling)
    ph_pos = np.zeros((ndim, cap)); ph_mom = np.zeros((3, cap)); ph_w = np.zeros(cap)
    ph_chi = np.zeros(cap); ph_tau = np.zeros(cap)
    ts = tables.c_struct()
    L = _rad_lib()
    L.or_rad_monte_carlo_photons.restype = ctypes.c_double
    rad = L.or_rad_monte_carlo_photons(ctypes.byref(ts), ndim, ctypes.c_int64(n), ctypes.c_double(dt),
                                       ctypes.c_double(mass), ctypes.c_double(charge), _ptr(_f64(pos)), _ptr(mom),
                                       _ptr(_f64(weight)), _ptr(tau), _ptr(chi), _ptr(_f64(E)), _ptr(_f64(B)),
                                       ctypes.c_uint32(seed), ctypes.c_uint32(first_id), ctypes.c_uint32(step),
                                       sampling, ctypes.c_double(threshold), max_emissions, ctypes.c_int64(cap),
                                       _ptr(ph_pos), _ptr(ph_mom), _ptr(ph_w), _ptr(ph_chi), _ptr(ph_tau),
                                       ctypes.byref(nph), ctypes.byref(nem))
    k = int(nph.value)
    assert k <= cap
    photons = dict(pos=ph_pos[:, :k].copy(), mom=ph_mom[:, :k].copy(), weight=ph_w[:k].copy(),
                   chi=ph_chi[:k].copy(), tau=ph_tau[:k].copy())
    return rad, nem.value, chi, photons


def push_photons(dt, pos, mom):
    """Rectilinear photon push (rad_oracle.c or_push_photons); pos updated in place, returns 1/|p|."""
    n = mom.shape[1]
    assert pos.dtype == np.float64 and pos.flags.c_contiguous
    inv = np.zeros(n)
    _rad_lib().or_push_photons(pos.shape[0], ctypes.c_int64(n), ctypes.c_double(dt), _ptr(pos), _ptr(_f64(mom)),
                               _ptr(inv))
    return inv


def rad_monte_carlo(tables: RadTables, dt, mass, charge, mom, weight, tau, E, B, seed, first_id=0, step=0):
    """One Monte-Carlo radiation pass; mom and tau updated in place.  Returns (radiated, n_emissions, chi)."""
    n = mom.shape[1]
    assert mom.dtype == np.float64 and mom.flags.c_contiguous and tau.dtype == np.float64
    chi = np.zeros(n)
    nem = ctypes.c_int64()
    ts = tables.c_struct()
    rad = _rad_lib().or_rad_monte_carlo(ctypes.byref(ts), ctypes.c_int64(n), ctypes.c_double(dt),
                                        ctypes.c_double(mass), ctypes.c_double(charge), _ptr(mom),
                                        _ptr(_f64(weight)), _ptr(tau), _ptr(chi), _ptr(_f64(E)), _ptr(_f64(B)),
                                        ctypes.c_uint32(seed), ctypes.c_uint32(first_id), ctypes.c_uint32(step),
                                        ctypes.byref(nem))
    return rad, nem.value, chi
