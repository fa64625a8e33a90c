"""Smilei-style Python namelists for the resident simulation.

A Smilei namelist is a Python file that calls ``Main(...)``, ``Species(...)``,
``LaserGaussian2D(...)``, ``MovingWindow(...)``, ``DiagScalar(...)`` and so on.
``Namelist`` executes such a file in a namespace that holds this module's
restatement of those blocks (the reference defines them in
src/Python/pyinit.py:77-150 and :156-660, the profiles and lasers in
src/Python/pyprofiles.py), then ``build`` maps the blocks the hot path covers
onto ``simulation.Simulation`` and ``run`` steps it with the diagnostics:

- ``Main``: geometry 2Dcartesian or 3Dcartesian; two of grid_length,
  number_of_cells, cell_length (pyinit.py:296-323); timestep, or
  timestep_over_CFL for the Yee solver (dt = CFL / sqrt(sum 1/dx^2),
  pyinit.py:233-240); simulation_time or number_of_timesteps;
  EM_boundary_conditions periodic or silver-muller (2D); solve_poisson with
  poisson_max_error / poisson_max_iteration; number_of_patches (the window's
  shift is one patch along x); random_seed.
- ``Species``: pusher boris / vay / higueracary; mass, charge; positions and
  weights from a numpy array (ndim + 1, N) and momenta from a numpy array
  (3, N) (the reference's position_initialization / momentum_initialization
  arrays), or "random" / "regular" positions with particles_per_cell and a
  constant or trapezoidal number_density / charge_density, and a
  "maxwell-juettner" / "mj" / "cold" momentum distribution with ``temperature``;
  radiation_model "mc" with a ``RadiationReaction`` block.
- ``LaserGaussian2D`` from xmin with a ``tgaussian`` or ``tconstant`` time
  envelope and ``MovingWindow`` (2D, silver-muller along x).
- ``DiagScalar`` and ``DiagFields`` (diagnostics.py).
Blocks that only tune the reference's own machinery (LoadBalancing,
Vectorization, Checkpoints, DiagPerformances) are accepted and have no effect
here.  Any other block, or an option of a covered block that would change the
physics and is not covered, raises NotImplementedError: a namelist either runs
as written or is refused.

As in the reference, an unknown keyword of a block is an error, a singleton
block may be defined once, and ``Species["name"]`` / ``len(Species)`` work.

Random positions and momenta come from numpy's generator seeded by
``Main.random_seed``: the same namelist gives the same particles every time,
not the reference's random stream.  The Maxwell-Juettner draw is a Gaussian of
variance T / m per momentum component, the non-relativistic limit (T << m c^2).
"""
from __future__ import annotations

import math
import os

import numpy as np


class NamelistError(Exception):
    """Invalid namelist (the reference's ERROR_NAMELIST)."""


class _BlockList(type):
    """Metaclass: each block class keeps the list of its instances."""

    def __iter__(cls):
        return iter(cls._list)

    def __len__(cls):
        return len(cls._list)

    def __getitem__(cls, key):
        for obj in cls._list:
            if getattr(obj, "name", None) == key:
                return obj
        return cls._list[key]


class _Block(metaclass=_BlockList):
    """A namelist block: class attributes are the defaults; keywords must name one."""
    _list: list = []
    _singleton = False

    def __init__(self, **kwargs):
        cls = type(self)
        if cls._singleton and cls._list:
            raise NamelistError(f"cannot define block {cls.__name__}() twice")
        for k, v in kwargs.items():
            if k.startswith("_") or not hasattr(cls, k):
                raise NamelistError(f"cannot define `{k}` in block {cls.__name__}()")
            setattr(self, k, v)
        cls._list.append(self)

    def get(self, k):
        return getattr(self, k)


def _blocks():
    """Fresh block classes for one namelist (no state shared between namelists)."""

    class Main(_Block):
        _list = []
        _singleton = True
        geometry = None
        cell_length = []
        grid_length = []
        number_of_cells = []
        timestep = None
        timestep_over_CFL = None
        simulation_time = None
        number_of_timesteps = None
        interpolation_order = 2
        interpolator = "momentum-conserving"
        custom_oversize = 2
        number_of_patches = None
        patch_arrangement = "hilbertian"
        cluster_width = -1
        cell_sorting = None
        gpu_computing = False
        maxwell_solver = "Yee"
        EM_boundary_conditions = [["periodic"]]
        solve_poisson = True
        poisson_max_iteration = 50000
        poisson_max_error = 1e-14
        time_fields_frozen = 0.0
        reference_angular_frequency_SI = 0.0
        print_every = None
        random_seed = None
        print_expected_disk_usage = True
        every_clean_particles_overhead = 100

        def __init__(self, **kwargs):
            super().__init__(**kwargs)
            _derive_main(self)

    class Species(_Block):
        _list = []
        name = None
        position_initialization = None
        momentum_initialization = ""
        particles_per_cell = None
        regular_number = []
        c_part_max = 1.0
        mass = None
        charge = None
        charge_density = None
        number_density = None
        mean_velocity = []
        temperature = []
        pusher = "boris"
        radiation_model = "none"
        radiation_photon_species = None
        radiation_photon_sampling = 1
        radiation_photon_gamma_threshold = 2.0
        radiation_max_emissions = 10
        time_frozen = 0.0
        radiating = False
        boundary_conditions = [["periodic"]]
        ionization_model = "none"
        is_test = False
        relativistic_field_initialization = False
        merging_method = "none"
        multiphoton_Breit_Wheeler = [None, None]

    class Laser(_Block):
        _list = []
        box_side = "xmin"
        omega = 1.0
        # the parameters of LaserGaussian2D, which builds the reference's Laser block
        a0 = None
        focus = None
        waist = None
        incidence_angle = 0.0
        polarization_phi = 0.0
        ellipticity = 0.0
        time_envelope = None
        phase_offset = 0.0

    class MovingWindow(_Block):
        _list = []
        _singleton = True
        time_start = 0.0
        velocity_x = 1.0
        number_of_additional_shifts = 0
        additional_shifts_time = 0.0

    class RadiationReaction(_Block):
        _list = []
        minimum_chi_discontinuous = 1e-2
        minimum_chi_continuous = 1e-3
        table_path = ""
        Niel_computation_method = "table"

    class DiagScalar(_Block):
        _list = []
        every = None
        precision = 10
        vars = []

    class DiagFields(_Block):
        _list = []
        name = ""
        every = None
        fields = []
        time_average = 1
        subgrid = None
        flush_every = 1
        datatype = "double"

    class LoadBalancing(_Block):
        _list = []
        _singleton = True
        every = 150
        initial_balance = True
        cell_load = 1.0
        frozen_particle_load = 0.1

    class Vectorization(_Block):
        _list = []
        _singleton = True
        mode = "off"
        reconfigure_every = 20
        initial_mode = "off"

    class Checkpoints(_Block):
        _list = []
        _singleton = True
        restart_dir = None
        restart_number = None
        dump_step = 0
        dump_minutes = 0.0
        exit_after_dump = True
        keep_n_dumps = 2
        file_grouping = None
        dump_deflate = 0

    class DiagPerformances(_Block):
        _list = []
        _singleton = True
        every = 0
        flush_every = 1
        patch_information = False

    return dict(Main=Main, Species=Species, Laser=Laser, MovingWindow=MovingWindow,
                RadiationReaction=RadiationReaction, DiagScalar=DiagScalar, DiagFields=DiagFields,
                LoadBalancing=LoadBalancing, Vectorization=Vectorization, Checkpoints=Checkpoints,
                DiagPerformances=DiagPerformances)


def _derive_main(m):
    """Timestep, simulation time and the grid triple, as the reference's Main() does."""
    if m.geometry not in ("2Dcartesian", "3Dcartesian"):
        raise NotImplementedError(f"geometry {m.geometry!r}: this build runs 2Dcartesian and 3Dcartesian")
    have = [len(m.grid_length) > 0, len(m.number_of_cells) > 0, len(m.cell_length) > 0]
    if sum(have) != 2:
        raise NamelistError("you must define exactly two parameters among grid_length, number_of_cells and "
                            "cell_length")
    if not have[0]:
        m.grid_length = [a * b for a, b in zip(m.number_of_cells, m.cell_length)]
    if not have[2]:
        m.cell_length = [a / b for a, b in zip(m.grid_length, m.number_of_cells)]
    if not have[1]:
        m.number_of_cells = [int(round(float(a) / float(b))) for a, b in zip(m.grid_length, m.cell_length)]
        m.grid_length = [a * b for a, b in zip(m.number_of_cells, m.cell_length)]
    if m.timestep is None:
        if m.timestep_over_CFL is None:
            raise NamelistError("timestep and timestep_over_CFL not defined")
        if m.maxwell_solver != "Yee":
            raise NotImplementedError(f"maxwell_solver {m.maxwell_solver!r}: this build has the Yee solver")
        m.timestep = m.timestep_over_CFL / math.sqrt(sum(1.0 / l ** 2 for l in m.cell_length))
    if m.simulation_time is None:
        if m.number_of_timesteps is None:
            raise NamelistError("simulation_time and number_of_timesteps are not defined")
        m.simulation_time = m.timestep * m.number_of_timesteps


# ---- profiles (pyprofiles.py) ------------------------------------------------

class Profile:
    """A space or time profile: callable, with its kind and parameters kept for the GPU."""

    def __init__(self, kind, f, **params):
        self.kind, self._f, self.params = kind, f, params

    def __call__(self, *x):
        return self._f(*x)


def _profiles(blocks):
    Main = blocks["Main"]

    def _need_main(what):
        if len(Main) == 0:
            raise NamelistError(f"{what} profile has been defined before `Main()`")
        return Main[0]

    def constant(value, xvacuum=-float("inf"), yvacuum=-float("inf"), zvacuum=-float("inf")):
        return Profile("constant", lambda *x: value if x[0] >= xvacuum else 0.0, value=value, xvacuum=xvacuum)

    def trapezoidal(max, xvacuum=0.0, xplateau=None, xslope1=0.0, xslope2=0.0, yvacuum=0.0, yplateau=None,
                    yslope1=0.0, yslope2=0.0, zvacuum=0.0, zplateau=None, zslope1=0.0, zslope2=0.0):
        m = _need_main("trapezoidal")
        if xplateau is None:
            xplateau = m.grid_length[0] - xvacuum
        if (yvacuum, yslope1, yslope2) != (0.0, 0.0, 0.0) or yplateau is not None or \
                (zvacuum, zslope1, zslope2) != (0.0, 0.0, 0.0) or zplateau is not None:
            raise NotImplementedError("trapezoidal: this build varies the density along x only")

        def f(x, *rest):
            if x < xvacuum:
                return 0.0
            if x < xvacuum + xslope1:
                return max * (x - xvacuum) / xslope1
            if x < xvacuum + xslope1 + xplateau:
                return max
            if x < xvacuum + xslope1 + xplateau + xslope2:
                return max * (1.0 - (x - (xvacuum + xslope1 + xplateau)) / xslope2)
            return 0.0
        return Profile("trapezoidal", f, value=max, xvacuum=xvacuum, xplateau=xplateau, xslope1=xslope1,
                       xslope2=xslope2)

    def tconstant(start=0.0):
        return Profile("tconstant", lambda t: 1.0 if t >= start else 0.0, start=start)

    def tgaussian(start=0.0, duration=None, fwhm=None, center=None, order=2):
        m = _need_main("tgaussian")
        if duration is None:
            duration = m.simulation_time - start
        if fwhm is None:
            fwhm = duration / 3.0
        if center is None:
            center = start + duration / 2.0
        sigma = (0.5 * fwhm) ** order / math.log(2.0)

        def f(t):
            return math.exp(-(t - center) ** order / sigma) if start <= t < start + duration else 0.0
        return Profile("tgaussian", f, start=start, duration=duration, fwhm=fwhm, center=center, order=order)

    def LaserGaussian2D(box_side="xmin", a0=1.0, omega=1.0, focus=None, waist=3.0, incidence_angle=0.0,
                        polarization_phi=0.0, ellipticity=0.0, time_envelope=None, phase_offset=0.0):
        _need_main("LaserGaussian2D")
        if focus is None or len(focus) != 2:
            raise NamelistError("LaserGaussian2D: focus must be a list of length 2.")
        return blocks["Laser"](box_side=box_side, omega=omega, a0=a0, focus=list(focus), waist=waist,
                               incidence_angle=incidence_angle, polarization_phi=polarization_phi,
                               ellipticity=ellipticity, time_envelope=time_envelope or tconstant(),
                               phase_offset=phase_offset)

    return dict(constant=constant, trapezoidal=trapezoidal, tconstant=tconstant, tgaussian=tgaussian,
                LaserGaussian2D=LaserGaussian2D)


class Namelist:
    """The blocks of one namelist file or string, executed in a fresh namespace."""

    def __init__(self, source: str, is_path: bool | None = None, extra: dict | None = None):
        if is_path is None:
            is_path = os.path.exists(source)
        text = open(source).read() if is_path else source
        self.blocks = _blocks()
        ns = {"__name__": "__namelist__", "np": np, "math": math}
        ns.update(self.blocks)
        ns.update(_profiles(self.blocks))
        ns.update(extra or {})
        exec(compile(text, source if is_path else "<namelist>", "exec"), ns)
        self.ns = ns
        if len(self.blocks["Main"]) == 0:
            raise NamelistError("no Main() block")
        self.main = self.blocks["Main"][0]
        self._check()

    def __getitem__(self, block):
        return self.blocks[block]

    @property
    def ndim(self):
        return int(self.main.geometry[0])

    @property
    def steps(self):
        return int(round(self.main.simulation_time / self.main.timestep))

    def boundaries(self):
        """'periodic' or 'open' per dimension from EM_boundary_conditions (one entry for all
        dimensions, one per dimension, or [min, max] pairs that must agree)."""
        bc = self.main.EM_boundary_conditions
        per = [bc[0]] * self.ndim if len(bc) == 1 else list(bc)
        out = []
        for d in range(self.ndim):
            kinds = set(per[d])
            if kinds == {"periodic"}:
                out.append("periodic")
            elif kinds <= {"silver-muller"} and self.ndim == 2:
                out.append("open")
            else:
                raise NotImplementedError(f"EM_boundary_conditions {per[d]} along dimension {d}: this build has "
                                          "periodic, and silver-muller in 2D")
        return out

    def _check(self):
        m = self.main
        if m.interpolation_order != 2:
            raise NotImplementedError("interpolation_order must be 2")
        if m.time_fields_frozen != 0.0:
            raise NotImplementedError("time_fields_frozen is not covered")
        for s in self.blocks["Species"]:
            if s.pusher not in ("boris", "vay", "higueracary"):
                raise NotImplementedError(f"pusher {s.pusher!r}")
            if s.ionization_model != "none" or s.merging_method != "none" or s.multiphoton_Breit_Wheeler != [None, None]:
                raise NotImplementedError(f"species {s.name}: ionization, merging and pair creation are not covered")
            if s.time_frozen > 0.0 and s.time_frozen < m.simulation_time:
                raise NotImplementedError(f"species {s.name}: a species frozen for part of the run is not covered")
            if s.radiation_model not in ("none", "mc", "Monte-Carlo", "MC"):
                raise NotImplementedError(f"species {s.name}: radiation_model {s.radiation_model!r}")
        for las in self.blocks["Laser"]:
            if las.a0 is None or las.box_side != "xmin" or las.incidence_angle != 0.0:
                raise NotImplementedError("lasers: LaserGaussian2D from xmin at normal incidence")
            if las.time_envelope.kind not in ("tgaussian", "tconstant"):
                raise NotImplementedError(f"laser time envelope {las.time_envelope.kind}")


# ---- from the blocks to the simulation ----------------------------------------

def _momenta(rng, s, n):
    if isinstance(s.momentum_initialization, np.ndarray):
        mom = np.asarray(s.momentum_initialization, dtype=np.float64)
        if mom.shape != (3, n):
            raise NamelistError(f"species {s.name}: momentum_initialization must have shape (3, {n})")
        return mom
    kind = s.momentum_initialization
    if kind in ("", "cold"):
        return np.zeros((3, n))
    if kind in ("maxwell-juettner", "mj"):
        T = list(s.temperature) if s.temperature else [1e-10]
        T = (T * 3)[:3] if len(T) == 1 else T
        sig = [math.sqrt(t / s.mass) for t in T]
        mom = np.stack([rng.normal(0.0, sig[d], n) for d in range(3)])
        if s.mean_velocity:
            raise NotImplementedError(f"species {s.name}: a drifting Maxwellian is not covered")
        return mom
    raise NotImplementedError(f"species {s.name}: momentum_initialization {kind!r}")


def _density(s):
    d = s.number_density if s.number_density is not None else s.charge_density
    if d is None:
        raise NamelistError(f"species {s.name}: number_density or charge_density required")
    scale = 1.0 if s.number_density is not None else 1.0 / abs(s.charge)
    if isinstance(d, (int, float)):
        return "constant", dict(value=float(d) * scale, xvacuum=-float("inf"))
    if isinstance(d, Profile) and d.kind in ("constant", "trapezoidal"):
        p = dict(d.params)
        p["value"] = p["value"] * scale
        return d.kind, p
    raise NotImplementedError(f"species {s.name}: density profiles other than constant and trapezoidal")


def species_plan(nl: Namelist):
    """Per species: how its particles are made -- ('arrays', pos, mom, w) or
    ('profile', dict(n0, ppc, x_vacuum, x_slope1, x_plateau, x_slope2, temperature))."""
    m = nl.main
    rng = np.random.default_rng(m.random_seed if m.random_seed is not None else 0)
    nd = nl.ndim
    out = []
    for s in nl["Species"]:
        if isinstance(s.position_initialization, np.ndarray):
            a = np.asarray(s.position_initialization, dtype=np.float64)
            if a.ndim != 2 or a.shape[0] != nd + 1:
                raise NamelistError(f"species {s.name}: position_initialization must have shape (ndim + 1, N)")
            n = a.shape[1]
            out.append(("arrays", np.ascontiguousarray(a[:nd]), _momenta(rng, s, n), np.ascontiguousarray(a[nd])))
            continue
        kind, prof = _density(s)
        ppc = int(s.particles_per_cell)
        if s.position_initialization == "regular":
            if round(ppc ** (1.0 / nd)) ** nd != ppc:
                raise NotImplementedError(f"species {s.name}: regular positions need a perfect-power ppc")
            if s.momentum_initialization not in ("", "cold", "maxwell-juettner", "mj"):
                raise NotImplementedError(f"species {s.name}: momentum_initialization {s.momentum_initialization!r}")
            T = s.temperature[0] if s.temperature else 0.0
            if s.temperature and len(set(s.temperature)) > 1:
                raise NotImplementedError(f"species {s.name}: anisotropic temperature with regular positions")
            if kind == "constant":
                x_vac, sl1, plat, sl2 = max(prof["xvacuum"], 0.0), 0.0, 1e300, 0.0
            else:
                x_vac, sl1, plat, sl2 = prof["xvacuum"], prof["xslope1"], prof["xplateau"], prof["xslope2"]
            out.append(("profile", dict(n0=prof["value"], ppc=ppc, x_vacuum=x_vac, x_slope1=sl1, x_plateau=plat,
                                        x_slope2=sl2, temperature=T / s.mass if T else 0.0)))
            continue
        if s.position_initialization != "random":
            raise NotImplementedError(f"species {s.name}: position_initialization {s.position_initialization!r}")
        if kind != "constant":
            raise NotImplementedError(f"species {s.name}: random positions with a constant density only")
        n_cells, cl = m.number_of_cells, m.cell_length
        ncell = int(np.prod(n_cells))
        n = ncell * ppc
        idx = np.repeat(np.arange(ncell, dtype=np.int64), ppc)
        strides = [int(np.prod(n_cells[d + 1:])) for d in range(nd)]
        pos = np.empty((nd, n))
        for d in range(nd):
            pos[d] = ((idx // strides[d]) % n_cells[d] + rng.random(n)) * cl[d]
        del idx
        w = np.full(n, prof["value"] * float(np.prod(cl)) / ppc)
        out.append(("arrays", pos, _momenta(rng, s, n), w))
    return out


def build(nl: Namelist, form: str = "mixed", radiation_tables=None, tile=None):
    """The Simulation a namelist describes, with its species, lasers, window and initial field."""
    from . import simulation
    m = nl.main
    sim = simulation.Simulation(m.number_of_cells, m.cell_length, m.timestep, form=form, tile=tile,
                                boundaries=nl.boundaries())
    for las in nl["Laser"]:
        te = las.time_envelope
        if te.kind == "tgaussian":
            p = te.params
            sim.add_laser_gaussian2d(a0=las.a0, waist=las.waist, focus=las.focus, t_fwhm=p["fwhm"],
                                     t_center=p["center"], t_start=p["start"], t_duration=p["duration"],
                                     omega=las.omega, polarization_phi=las.polarization_phi,
                                     ellipticity=las.ellipticity, phase_offset=las.phase_offset,
                                     t_order=float(p["order"]))
        else:  # tconstant: a flat envelope from its start on
            sim.add_laser_gaussian2d(a0=las.a0, waist=las.waist, focus=las.focus, t_fwhm=1e300, t_center=0.0,
                                     t_start=te.params["start"], t_duration=1e300, omega=las.omega,
                                     polarization_phi=las.polarization_phi, ellipticity=las.ellipticity,
                                     phase_offset=las.phase_offset)
    plans = species_plan(nl)
    for k, (s, plan) in enumerate(zip(nl["Species"], plans)):
        if plan[0] == "arrays":
            _, pos, mom, w = plan
            sim.add_species(s.mass, s.charge, s.pusher, pos, mom, w, name=s.name)
        else:
            p = plan[1]
            sim.add_species(s.mass, s.charge, s.pusher, np.zeros((nl.ndim, 0)), np.zeros((3, 0)), np.zeros(0),
                            name=s.name)
            sim.set_species_profile(k, p["n0"], p["ppc"], x_vacuum=p["x_vacuum"], x_slope1=p["x_slope1"],
                                    x_plateau=p["x_plateau"], x_slope2=p["x_slope2"],
                                    temperature=p["temperature"], seed=int(m.random_seed or 0) + k)
            sim.fill_species(k)
        if s.radiation_model != "none":
            if radiation_tables is None:
                raise NamelistError(f"species {s.name}: radiation_model needs the radiation tables (pass "
                                    "radiation_tables, or RadiationReaction(table_path=...))")
            sim.set_species_radiation(k, radiation_tables, seed=int(m.random_seed or 0) + k)
    if len(nl["MovingWindow"]):
        w = nl["MovingWindow"][0]
        patches = m.number_of_patches[0] if m.number_of_patches else 1
        sim.set_moving_window(w.time_start, w.velocity_x, max(1, m.number_of_cells[0] // patches))
    if m.solve_poisson and any(plan[0] == "arrays" for plan in plans) and not len(nl["Laser"]):
        sim.solve_poisson(max_error=m.poisson_max_error, max_iter=m.poisson_max_iteration)
    return sim


def load_radiation_tables(nl: Namelist):
    """Tables for a radiating species from RadiationReaction(table_path=<.npz>): the
    reference's table arrays (integfochi, xi, their ranges, the minimum-photon-chi axis)."""
    rr = nl["RadiationReaction"]
    if not len(rr) or not rr[0].table_path:
        return None
    from . import radiation
    g = np.load(rr[0].table_path)
    omega = nl.main.reference_angular_frequency_SI
    if not omega:
        raise NamelistError("radiation reaction needs Main.reference_angular_frequency_SI")
    f_dn, f_cl, inv_es = radiation.normalised_factors(omega)
    return radiation.RadiationTables(g["integfochi"], float(g["integfochi_min"]), float(g["integfochi_max"]),
                                     g["xi"], float(g["xi_min"]), float(g["xi_max"]), g["xi_axis1_min"], f_dn, f_cl,
                                     inv_es, min_chi_continuous=rr[0].minimum_chi_continuous,
                                     min_chi_discontinuous=rr[0].minimum_chi_discontinuous)


def run(source, form="mixed", output_dir=".", steps=None, radiation_tables=None, tile=None):
    """Executes the namelist, builds the simulation and runs number_of_timesteps (or
    ``steps``) with its DiagScalar / DiagFields output under output_dir; returns the
    simulation (still open) and the namelist."""
    from . import diagnostics
    nl = source if isinstance(source, Namelist) else Namelist(source)
    tables = radiation_tables if radiation_tables is not None else load_radiation_tables(nl)
    sim = build(nl, form=form, radiation_tables=tables, tile=tile)
    os.makedirs(output_dir, exist_ok=True)
    diags = []
    for d in nl["DiagScalar"]:
        diags.append(diagnostics.DiagScalar(sim, os.path.join(output_dir, "scalars.txt"), every=d.every or 1,
                                            precision=d.precision, vars=d.vars or None))
    for i, d in enumerate(nl["DiagFields"]):
        diags.append(diagnostics.DiagFields(sim, os.path.join(output_dir, f"Fields{i}"), every=d.every or 1,
                                            fields=d.fields or None, time_average=d.time_average,
                                            subgrid=d.subgrid))
    n = nl.steps if steps is None else int(steps)
    for it in range(n + 1):
        for d in diags:
            d(it)
        if it < n:
            sim.step(1)
    sim._namelist_tables = tables
    return sim, nl
