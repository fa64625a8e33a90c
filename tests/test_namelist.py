"""The namelist front end on the CPU: blocks, derived parameters, particle plans, refusals.

The namelists here are written in the reference's idiom (Main, Species,
LaserGaussian2D, MovingWindow, DiagScalar blocks; src/Python/pyinit.py and
pyprofiles.py define them there).  Nothing here needs a GPU: the tests check what
the namelist resolves to, which is what smilei_gb300.namelist.build hands to the
simulation.
"""
import math

import numpy as np
import pytest

from smilei_gb300 import namelist

THERMAL_3D = """
import math as m
TkeV = 10.
T = TkeV / 511.
dx = 0.1
Main(
    geometry = "3Dcartesian",
    interpolation_order = 2,
    timestep_over_CFL = 0.95,
    number_of_timesteps = 40,
    cell_length = [dx, dx, dx],
    grid_length = [1.6, 1.6, 0.8],
    number_of_patches = [2, 2, 1],
    EM_boundary_conditions = [["periodic"]],
    random_seed = 3,
)
LoadBalancing(every = 20)
Vectorization(mode = "off")
Species(
    name = "electron",
    position_initialization = POS,
    momentum_initialization = MOM,
    mass = 1.0,
    charge = -1.0,
    pusher = "higueracary",
)
DiagScalar(every = 10, vars = ["Utot", "Ukin", "Uelm"])
"""

WAKE_2D = """
dx, dy = 0.1, 1.5
Main(
    geometry = "2Dcartesian",
    timestep = 0.095,
    simulation_time = 50 * 0.095,
    cell_length = [dx, dy],
    number_of_cells = [384, 64],
    number_of_patches = [12, 2],
    EM_boundary_conditions = [["silver-muller"], ["silver-muller"]],
    solve_poisson = False,
)
MovingWindow(time_start = 20.0, velocity_x = 1.0)
LaserGaussian2D(
    a0 = 2.0, omega = 1.0, focus = [0.0, 48.0], waist = 30.0,
    time_envelope = tgaussian(fwhm = 60.0, center = 60.0 * 2 ** 0.5),
)
Species(
    name = "electron",
    position_initialization = "regular",
    momentum_initialization = "cold",
    particles_per_cell = 4,
    mass = 1.0,
    charge = -1.0,
    number_density = trapezoidal(0.003, xvacuum = 2.0, xslope1 = 10.0),
    pusher = "vay",
)
"""


def _thermal_arrays(n=1000, seed=1):
    rng = np.random.default_rng(seed)
    pos = np.vstack([rng.uniform(0, 1.6, n), rng.uniform(0, 1.6, n), rng.uniform(0, 0.8, n), np.full(n, 2e-4)])
    mom = rng.normal(0, 0.14, (3, n))
    return pos, mom


def test_thermal_namelist_resolves_like_the_reference():
    pos, mom = _thermal_arrays()
    nl = namelist.Namelist(THERMAL_3D, extra=dict(POS=pos, MOM=mom))
    m = nl.main
    assert nl.ndim == 3
    assert m.number_of_cells == [16, 16, 8]
    # dt = CFL / sqrt(sum 1/dx^2) for the Yee solver (pyinit.py:233-240)
    assert m.timestep == pytest.approx(0.95 / math.sqrt(3 / 0.01), rel=1e-15)
    assert nl.steps == 40 and m.simulation_time == pytest.approx(40 * m.timestep)
    assert nl.boundaries() == ["periodic"] * 3
    assert nl["Species"]["electron"].pusher == "higueracary" and len(nl["Species"]) == 1
    (kind, p, q, w), = namelist.species_plan(nl)
    assert kind == "arrays"
    assert np.array_equal(p, pos[:3]) and np.array_equal(q, mom) and np.array_equal(w, pos[3])
    assert nl["DiagScalar"][0].every == 10


def test_wakefield_namelist_resolves_to_profile_laser_and_window():
    nl = namelist.Namelist(WAKE_2D)
    assert nl.ndim == 2 and nl.boundaries() == ["open", "open"]
    assert nl.steps == 50
    assert nl.main.grid_length == pytest.approx([38.4, 96.0])
    las, = list(nl["Laser"])
    assert las.a0 == 2.0 and las.focus == [0.0, 48.0] and las.waist == 30.0
    te = las.time_envelope
    assert te.kind == "tgaussian" and te.params["fwhm"] == 60.0
    assert te.params["duration"] == pytest.approx(nl.main.simulation_time)
    (kind, p), = namelist.species_plan(nl)
    assert kind == "profile"
    # the plateau reaches the end of the box: grid_length - xvacuum (pyprofiles.py:21-30)
    assert p == dict(n0=0.003, ppc=4, x_vacuum=2.0, x_slope1=10.0, x_plateau=nl.main.grid_length[0] - 2.0,
                     x_slope2=0.0, temperature=0.0)
    w = nl["MovingWindow"][0]
    assert (w.time_start, w.velocity_x) == (20.0, 1.0)


def test_random_positions_are_seeded_and_uniform_per_cell():
    text = THERMAL_3D.replace("position_initialization = POS", "position_initialization = 'random'") \
        .replace("momentum_initialization = MOM", "momentum_initialization = 'mj', temperature = [T]") \
        .replace("pusher = \"higueracary\",", "pusher = \"higueracary\", particles_per_cell = 8, "
                                               "number_density = 1.0,")
    a = namelist.species_plan(namelist.Namelist(text))[0]
    b = namelist.species_plan(namelist.Namelist(text))[0]
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    _, pos, mom, w = a
    assert pos.shape == (3, 16 * 16 * 8 * 8)
    cells = np.floor(pos / 0.1).astype(int)
    flat = (cells[0] * 16 + cells[1]) * 8 + cells[2]
    assert np.all(np.bincount(flat, minlength=2048) == 8)
    assert np.allclose(w, 1e-3 / 8)
    assert abs(mom.std() - math.sqrt(10 / 511)) < 0.01


def test_namelist_errors_like_the_reference():
    with pytest.raises(namelist.NamelistError, match="cannot define `dx`"):
        namelist.Namelist("Main(geometry='2Dcartesian', dx=0.1)")
    with pytest.raises(namelist.NamelistError, match="twice"):
        namelist.Namelist("Main(geometry='2Dcartesian', cell_length=[.1,.1], number_of_cells=[8,8], timestep=.05,"
                          " number_of_timesteps=1)\nMain()")
    with pytest.raises(namelist.NamelistError, match="exactly two"):
        namelist.Namelist("Main(geometry='2Dcartesian', cell_length=[.1,.1], timestep=.05, number_of_timesteps=1)")
    with pytest.raises(NotImplementedError, match="geometry"):
        namelist.Namelist("Main(geometry='AMcylindrical', cell_length=[.1,.1], number_of_cells=[8,8], timestep=.05,"
                          " number_of_timesteps=1)")
    with pytest.raises(NotImplementedError, match="pusher"):
        namelist.Namelist("Main(geometry='2Dcartesian', cell_length=[.1,.1], number_of_cells=[8,8], timestep=.05,"
                          " number_of_timesteps=1)\nSpecies(name='e', pusher='borisnr', mass=1., charge=-1.)")
