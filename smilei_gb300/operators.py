"""Operator classes with the reference's interfaces, running the sm_103a kernels.

These mirror the C++ operator classes Species::dynamics and VectorPatch call
(src/Interpolator/Interpolator.h:23, src/Pusher/Pusher.h:22,
src/Projector/Projector.h:44, the Solver operator() of
src/ElectroMagnSolver, ElectroMagn::saveMagneticFields/centerMagneticFields and
Species::sortParticles) so that a dynamics loop written against the reference
reads the same here.  Data live in torch CUDA tensors (FP64, the reference's
layout); every call goes through libsmileigb300.so.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import check, ptr, ptr_array

STAGGER = {
    "Ex": (1, 0, 0), "Ey": (0, 1, 0), "Ez": (0, 0, 1),
    "Bx": (0, 1, 1), "By": (1, 0, 1), "Bz": (1, 1, 0),
    "Jx": (1, 0, 0), "Jy": (0, 1, 0), "Jz": (0, 0, 1), "rho": (0, 0, 0),
}


def _stream(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


class PatchGeometry:
    """A patch's grid: cells per dimension, oversize (ghost width) and origin.

    n_prim = patch_size + 1 + 2*oversize, domain_begin = patch start - oversize
    (src/Patch/Patch.cpp:145-153)."""

    def __init__(self, patch_size, cell_length, patch_start=None, oversize=2):
        self.ndim = len(patch_size)
        self.patch_size = [int(n) for n in patch_size]
        self.cell_length = [float(c) for c in cell_length]
        self.patch_start = [int(s) for s in (patch_start or [0] * self.ndim)]
        self.oversize = int(oversize)
        self.n_prim = [n + 1 + 2 * self.oversize for n in self.patch_size]
        self.domain_begin = [s - self.oversize for s in self.patch_start]

    @classmethod
    def from_arrays(cls, n_prim, domain_begin, cell_length, oversize=2):
        g = cls([n - 1 - 2 * oversize for n in n_prim], cell_length,
                [b + oversize for b in domain_begin], oversize)
        return g

    def shape(self, comp: str):
        st = STAGGER[comp.replace("_m", "")]
        return tuple(self.n_prim[d] + st[d] for d in range(self.ndim))

    def c_geom(self) -> _lib.GridGeom:
        g = _lib.GridGeom()
        g.ndim = self.ndim
        for d in range(self.ndim):
            g.n_prim[d] = self.n_prim[d]
            g.domain_begin[d] = self.domain_begin[d]
            g.cell_length[d] = self.cell_length[d]
        return g


class ElectroMagn:
    """Field container with the reference's member names (src/ElectroMagn/ElectroMagn.h:113)."""

    def __init__(self, geom: PatchGeometry, device="cuda"):
        self.geom = geom
        z = lambda c: torch.zeros(geom.shape(c), dtype=torch.float64, device=device)
        self.Ex_, self.Ey_, self.Ez_ = z("Ex"), z("Ey"), z("Ez")
        self.Bx_, self.By_, self.Bz_ = z("Bx"), z("By"), z("Bz")
        self.Bx_m, self.By_m, self.Bz_m = z("Bx"), z("By"), z("Bz")
        self.Jx_, self.Jy_, self.Jz_ = z("Jx"), z("Jy"), z("Jz")
        self.rho_ = z("rho")

    def restartRhoJ(self):
        for t in (self.Jx_, self.Jy_, self.Jz_, self.rho_):
            t.zero_()

    def saveMagneticFields(self, is_spectral=False, stream=None):
        """B_m <- B (ElectroMagn3D.cpp:1048)."""
        check(_lib.lib().sg_save_magnetic_fields(ctypes.byref(self.geom.c_geom()),
                                                  ptr_array([self.Bx_, self.By_, self.Bz_]),
                                                  ptr_array([self.Bx_m, self.By_m, self.Bz_m]), _stream(stream)),
              "saveMagneticFields")

    def centerMagneticFields(self, stream=None):
        """B_m <- (B + B_m)/2 (ElectroMagn3D.cpp:1191)."""
        check(_lib.lib().sg_center_magnetic_fields(ctypes.byref(self.geom.c_geom()),
                                                    ptr_array([self.Bx_, self.By_, self.Bz_]),
                                                    ptr_array([self.Bx_m, self.By_m, self.Bz_m]), _stream(stream)),
              "centerMagneticFields")


class Particles:
    """SoA particle storage (src/Particles/Particles.h:48): position[ndim, n], momentum[3, n], weight, charge."""

    def __init__(self, position, momentum, weight, charge):
        self.position = position.contiguous()
        self.momentum = momentum.contiguous()
        self.weight = weight.contiguous()
        self.charge = charge.to(torch.int16).contiguous()
        self.first_index = None
        self.last_index = None

    def size(self) -> int:
        return int(self.weight.shape[0])

    numberOfParticles = size


class SmileiMPI:
    """The per-thread dynamics scratch of the reference (src/SmileiMPI/SmileiMPI.h:213-221)."""

    def __init__(self, ndim: int, npart: int, device="cuda"):
        self.resizeBuffers(ndim, npart, device)

    def resizeBuffers(self, ndim, npart, device="cuda"):
        f = lambda *s: torch.zeros(s, dtype=torch.float64, device=device)
        self.dynamics_Epart = f(3, npart)
        self.dynamics_Bpart = f(3, npart)
        self.dynamics_invgf = f(npart)
        self.dynamics_iold = torch.zeros((ndim, npart), dtype=torch.int32, device=device)
        self.dynamics_deltaold = f(ndim, npart)


def _full_range(particles: Particles, istart, iend):
    if istart != 0 or iend != particles.size():
        raise ValueError("operators act on the whole particle range [0, size) of a bin-sorted array")


class Interpolator2D2Order:
    """Order-2 gather (src/Interpolator/Interpolator2D2Order.cpp:158)."""

    ndim = 2

    def __init__(self, geom: PatchGeometry):
        if geom.ndim != self.ndim:
            raise ValueError(f"{type(self).__name__} needs a {self.ndim}D geometry")
        self.geom = geom

    def fieldsWrapper(self, EMfields: ElectroMagn, particles: Particles, smpi: SmileiMPI, istart=0, iend=None,
                      ithread=0, stream=None):
        iend = particles.size() if iend is None else iend
        _full_range(particles, istart, iend)
        f = [EMfields.Ex_, EMfields.Ey_, EMfields.Ez_, EMfields.Bx_m, EMfields.By_m, EMfields.Bz_m]
        check(_lib.lib().sg_interpolate_fields(ctypes.byref(self.geom.c_geom()), ptr_array(f), particles.size(),
                                               ptr(particles.position), ptr(smpi.dynamics_Epart),
                                               ptr(smpi.dynamics_Bpart), ptr(smpi.dynamics_iold),
                                               ptr(smpi.dynamics_deltaold), _stream(stream)), "fieldsWrapper")


class Interpolator3D2Order(Interpolator2D2Order):
    """Order-2 gather (src/Interpolator/Interpolator3D2Order.cpp:163)."""

    ndim = 3


class _Pusher:
    kind = 0

    def __init__(self, dt: float, mass: float, ndim: int):
        self.dt, self.mass, self.ndim = float(dt), float(mass), int(ndim)

    def __call__(self, particles: Particles, smpi: SmileiMPI, istart=0, iend=None, ithread=0,
                 ipart_buffer_offset=0, stream=None):
        iend = particles.size() if iend is None else iend
        _full_range(particles, istart, iend)
        check(_lib.lib().sg_push_particles(self.kind, self.ndim, self.dt, self.mass, particles.size(),
                                           ptr(particles.position), ptr(particles.momentum), ptr(particles.charge),
                                           ptr(smpi.dynamics_Epart), ptr(smpi.dynamics_Bpart),
                                           ptr(smpi.dynamics_invgf), _stream(stream)), type(self).__name__)


class PusherBoris(_Pusher):
    """Boris pusher (src/Pusher/PusherBoris.cpp:23)."""
    kind = 0


class PusherVay(_Pusher):
    """Vay pusher (src/Pusher/PusherVay.cpp:32)."""
    kind = 1


class PusherHigueraCary(_Pusher):
    """Higuera-Cary pusher (src/Pusher/PusherHigueraCary.cpp:32)."""
    kind = 2


def PusherFactory(name: str, dt: float, mass: float, ndim: int) -> _Pusher:
    """Pusher selection by the namelist string (src/Pusher/PusherFactory.h:41-129)."""
    table = {"boris": PusherBoris, "vay": PusherVay, "higueracary": PusherHigueraCary}
    if name not in table:
        raise ValueError(f"For species, pusher must be one of {sorted(table)} (got {name!r})")
    return table[name](dt, mass, ndim)


class Projector2D2Order:
    """Esirkepov deposit (src/Projector/Projector2D2Order.cpp:498)."""

    ndim = 2

    def __init__(self, geom: PatchGeometry, dt: float):
        if geom.ndim != self.ndim:
            raise ValueError(f"{type(self).__name__} needs a {self.ndim}D geometry")
        self.geom, self.dt = geom, float(dt)

    def _run(self, mode, EMfields, particles, smpi, stream):
        J = [EMfields.Jx_, EMfields.Jy_, EMfields.Jz_, EMfields.rho_]
        check(_lib.lib().sg_project_currents(mode, ctypes.byref(self.geom.c_geom()), self.dt, particles.size(),
                                             ptr(particles.position), ptr(particles.momentum),
                                             ptr(particles.weight), ptr(particles.charge),
                                             ptr(smpi.dynamics_invgf) if smpi else None,
                                             ptr(smpi.dynamics_iold) if smpi else None,
                                             ptr(smpi.dynamics_deltaold) if smpi else None, ptr_array(J),
                                             _stream(stream)), "currentsAndDensityWrapper")

    def currentsAndDensityWrapper(self, EMfields, particles, smpi, istart=0, iend=None, ithread=0, diag_flag=False,
                                  is_spectral=False, ispec=0, stream=None):
        iend = particles.size() if iend is None else iend
        _full_range(particles, istart, iend)
        self._run(1 if diag_flag else 0, EMfields, particles, smpi, stream)

    def basic(self, EMfields, particles, stream=None):
        """rho of the current positions (Projector3D2Order::basic, type 0)."""
        self._run(2, EMfields, particles, None, stream)


class Projector3D2Order(Projector2D2Order):
    """Esirkepov deposit (src/Projector/Projector3D2Order.cpp:733)."""

    ndim = 3


class MA_Solver_norm:
    """Ampere (src/ElectroMagnSolver/MA_Solver3D_norm.cpp:18, MA_Solver2D_norm.cpp:18)."""

    def __init__(self, dt: float):
        self.dt = float(dt)

    def __call__(self, fields: ElectroMagn, stream=None):
        F = [fields.Ex_, fields.Ey_, fields.Ez_, fields.Bx_, fields.By_, fields.Bz_, fields.Jx_, fields.Jy_,
             fields.Jz_]
        check(_lib.lib().sg_maxwell_ampere(ctypes.byref(fields.geom.c_geom()), self.dt, ptr_array(F),
                                           _stream(stream)), "MA_Solver")


class MF_Solver_Yee(MA_Solver_norm):
    """Faraday (src/ElectroMagnSolver/MF_Solver3D_Yee.cpp:18, MF_Solver2D_Yee.cpp:18)."""

    def __call__(self, fields: ElectroMagn, stream=None):
        F = [fields.Ex_, fields.Ey_, fields.Ez_, fields.Bx_, fields.By_, fields.Bz_, fields.Jx_, fields.Jy_,
             fields.Jz_]
        check(_lib.lib().sg_maxwell_faraday(ctypes.byref(fields.geom.c_geom()), self.dt, ptr_array(F),
                                            _stream(stream)), "MF_Solver")


def sortParticles(particles: Particles, patch_size, xmin, cell_length, extra=(), stream=None):
    """Per-cell sort (src/Species/SpeciesV.cpp:599): returns (first_index, last_index, cell_keys).

    position, momentum, weight, charge and any tensors in ``extra`` (float64, [n]) are
    permuted in place."""
    ndim = particles.position.shape[0]
    n = particles.size()
    ncell = 1
    for p in patch_size:
        ncell *= int(p) + 1
    dev = particles.weight.device
    first = torch.zeros(ncell, dtype=torch.int32, device=dev)
    last = torch.zeros(ncell, dtype=torch.int32, device=dev)
    keys = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
    props = [particles.position[d] for d in range(ndim)] + [particles.momentum[d] for d in range(3)] + \
        [particles.weight] + list(extra)
    for t in props:
        if not t.is_contiguous():
            raise ValueError("particle properties must be contiguous")
    I3 = ctypes.c_int * ndim
    D3 = ctypes.c_double * ndim
    check(_lib.lib().sg_sort_particles(ndim, I3(*patch_size), D3(*xmin), D3(*cell_length), n, ptr_array(props),
                                       len(props), ptr(particles.charge), ptr(first), ptr(last), ptr(keys),
                                       _stream(stream)), "sortParticles")
    particles.first_index, particles.last_index = first, last
    return first, last, keys[:n]
