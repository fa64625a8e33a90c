"""Namelist-driven runs against the same runs built through the direct API (GPU).

A 3D thermal-plasma namelist (particles given as arrays, the reference's
position_initialization / momentum_initialization arrays) and a 2D wakefield
namelist (LaserGaussian2D with a tgaussian envelope, a trapezoidal density at
regular positions, MovingWindow, silver-muller boundaries) must give the fields
and particles of the hand-built Simulation: FP64 within 1e-12 relative, the split
form within 1e-5 (the deposit's atomics add in a run-dependent order).  The
thermal run also writes scalars.txt through its DiagScalar block.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FIELDS = ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Jx", "Jy", "Jz"]


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from smilei_gb300 import namelist, simulation, synthetic
    import test_namelist as tn
    return namelist, simulation, synthetic, tn


def _fields_close(a, b, tol):
    for k in FIELDS:
        fa, fb = a.get_field(k), b.get_field(k)
        err = float(np.abs(fa - fb).max() / max(np.abs(fb).max(), 1e-300))
        assert err <= tol, (k, err)


@pytest.mark.parametrize("form,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
def test_thermal_namelist_matches_direct_api(mods, form, tol, tmp_path):
    namelist, simulation, synthetic, tn = mods
    pos, mom = tn._thermal_arrays(n=16 * 16 * 8 * 8, seed=4)
    nl = namelist.Namelist(tn.THERMAL_3D, extra=dict(POS=pos, MOM=mom))
    sim_nl, _ = namelist.run(nl, form=form, output_dir=str(tmp_path), steps=3)
    m = nl.main
    ref = simulation.Simulation([16, 16, 8], [0.1] * 3, 0.95 / np.sqrt(300.0), form=form)
    ref.add_species(1.0, -1.0, "higueracary", pos[:3], mom, pos[3])
    ref.solve_poisson(max_error=m.poisson_max_error, max_iter=m.poisson_max_iteration)
    ref.step(3)
    _fields_close(sim_nl, ref, tol)
    assert sim_nl.species_count(0) == ref.species_count(0) == pos.shape[1]
    assert os.path.exists(tmp_path / "scalars.txt")
    sim_nl.close()
    ref.close()


def test_wakefield_namelist_matches_direct_api(mods):
    namelist, simulation, synthetic, tn = mods
    nl = namelist.Namelist(tn.WAKE_2D)
    sim_nl = namelist.build(nl, form="fp64")
    m = nl.main
    ref = simulation.Simulation([384, 64], [0.1, 1.5], 0.095, form="fp64", boundaries=("open", "open"))
    ref.add_laser_gaussian2d(a0=2.0, waist=30.0, focus=[0.0, 48.0], t_fwhm=60.0, t_center=60.0 * 2 ** 0.5,
                             t_start=0.0, t_duration=m.simulation_time)
    ref.add_species(1.0, -1.0, "vay", np.zeros((2, 0)), np.zeros((3, 0)), np.zeros(0))
    ref.set_species_profile(0, 0.003, 4, x_vacuum=2.0, x_slope1=10.0, x_plateau=m.grid_length[0] - 2.0)
    ref.fill_species(0)
    ref.set_moving_window(20.0, 1.0, 32)
    assert sim_nl.species_count(0) == ref.species_count(0) > 0
    sim_nl.step(1)
    ref.step(1)
    _fields_close(sim_nl, ref, 1e-12)
    # through the first window shift (time_start 20 is step 211): the atomics' order
    # differs between the runs, and 230 steps amplify its last bits
    for _ in range(229):
        sim_nl.step(1)
        ref.step(1)
    assert sim_nl.window_state() == ref.window_state()
    assert sim_nl.window_state()[2] >= 1
    assert sim_nl.species_count(0) == ref.species_count(0)
    _fields_close(sim_nl, ref, 1e-9)
    sim_nl.close()
    ref.close()
