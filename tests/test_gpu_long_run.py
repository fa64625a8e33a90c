"""1000 steps of a 3D thermal plasma in both forms: energy drift and charge residual.

The split-precision form must track the FP64 form over a long run: total
energy (kinetic + field) of the two runs within 1 % of each other at every
checkpoint, and the charge-conservation residual max|div E - (rho - <rho>)| /
max|rho - <rho>| at most 1e-6 after 1000 steps (RESIDUAL_TOL below).  Both runs start from the same
seeded particles and an FP64 Poisson solve, so the only difference is the
form's arithmetic.  20^3 cells x 8 particles per cell, T = 10 keV, dt = 0.95 CFL,
Higuera-Cary; each run takes a few seconds on one GPU.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

STEPS = 1000
CHECK_EVERY = 100
DRIFT_TOL = 0.01       # relative difference of total energy, mixed vs FP64
# Charge-conservation residual of the mixed form after STEPS (the target for the form).
RESIDUAL_TOL = 1e-6


@pytest.fixture(scope="module")
def runs():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from smilei_gb300 import simulation, synthetic
    n_cells = [20, 20, 20]
    cl = [0.1] * 3
    dt = 0.95 / np.sqrt(sum(1.0 / c ** 2 for c in cl))
    pos, mom, w = synthetic.thermal_plasma(n_cells, cl, 8, np.sqrt(10.0 / 511.0), 11)
    out = {}
    for form in ("fp64", "mixed"):
        sim = simulation.Simulation(n_cells, cl, dt, form=form)
        sim.add_species(1.0, -1.0, "higueracary", pos, mom, w)
        sim.solve_poisson(max_error=1e-26)
        r0 = sim.charge_residual()
        energies = [sum(sim.energy())]
        for _ in range(STEPS // CHECK_EVERY):
            sim.step(CHECK_EVERY)
            energies.append(sum(sim.energy()))
        out[form] = dict(energy=np.array(energies), r0=r0, r1=sim.charge_residual())
        sim.close()
    return out


def test_mixed_energy_tracks_fp64_over_1000_steps(runs):
    e64, e32 = runs["fp64"]["energy"], runs["mixed"]["energy"]
    rel = np.abs(e32 - e64) / np.abs(e64)
    assert rel.max() <= DRIFT_TOL, rel
    # the FP64 run itself conserves energy to the scheme's accuracy
    assert abs(e64[-1] - e64[0]) / e64[0] < 0.05, e64


def test_mixed_charge_residual_after_1000_steps(runs):
    assert runs["fp64"]["r1"] <= 1e-9, runs["fp64"]
    assert runs["mixed"]["r1"] <= RESIDUAL_TOL, runs["mixed"]
