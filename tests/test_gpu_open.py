"""GPU parity of the 2D open boundaries with the oracle (bc_oracle.c).

Silver-Mueller fields on the open axes, a Gaussian laser entering through
xmin, particles removed when they leave, J ghosts not folded along open axes.
The oracle is pinned to the reference's compiled boundary and its own laser
profiles (tests/test_oracle_boundaries.py).  Step k of the simulation applies
the boundary at time (k + 1.5) dt, the reference's time_dual of iteration k+1.
Tolerances: 1e-12 relative (FP64 form), 1e-5 (mixed form).
"""
import numpy as np
import pytest

from conftest import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FIELDS = ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Bx_m", "By_m", "Bz_m", "Jx", "Jy", "Jz"]


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from smilei_gb300 import simulation, synthetic
    return simulation, synthetic


def zero_fields(n_cells):
    from smilei_gb300 import synthetic
    st = synthetic.STAGGER
    out = {}
    for k in FIELDS:
        s = st[k.replace("_m", "")]
        out[k] = np.zeros(tuple(n_cells[d] + 5 + s[d] for d in range(2)))
    return out


def run(mods, cpu_oracle, form, boundaries, nsteps, with_plasma, with_laser, seed=9):
    simulation, synthetic = mods
    n_cells, cl = [32, 24], [0.1, 0.15]
    dt = 0.95 / np.sqrt(sum(1.0 / c ** 2 for c in cl))
    periodic = [b == "periodic" for b in boundaries]
    fields = zero_fields(n_cells) if with_laser else synthetic.periodic_em(seed, n_cells)
    sim = simulation.Simulation(n_cells, cl, dt, form=form, boundaries=boundaries)
    for k in FIELDS:
        sim.set_field(k, fields[k])
    laser = None
    if with_laser:
        laser = sim.add_laser_gaussian2d(a0=0.8, waist=0.9, focus=[0.3, 1.8], t_fwhm=0.5, t_center=0.6,
                                         polarization_phi=0.4, ellipticity=0.2)
    species = []
    if with_plasma:
        pos, mom, w = synthetic.thermal_plasma(n_cells, cl, 4, 0.5, seed + 1, unique_weights=True)
        sim.add_species(1.0, -1.0, "vay", pos, mom, w)
        species.append(dict(pos=pos.copy(), mom=mom.copy(), weight=w.copy(),
                            charge=np.full(w.shape, -1, np.int16), mass=1.0, pusher="vay"))
    sim.step(nsteps)
    ref = {k: v.copy() for k, v in fields.items()}
    for k in range(nsteps):
        cpu_oracle.pic_step_bc(n_cells, 2, cl, dt, ref, species, periodic, laser, (k + 1.5) * dt)
    got = {k: sim.get_field(k) for k in FIELDS}
    parts = None
    if with_plasma:
        p, m, w = sim.get_species(0)
        s = species[0]
        assert sim.species_count(0) == s["weight"].size == w.size
        og = np.argsort(w, kind="stable")
        orf = np.argsort(s["weight"].astype(np.float32) if form == "mixed" else s["weight"], kind="stable")
        parts = (p[:, og], m[:, og], s["pos"][:, orf], s["mom"][:, orf])
    sim.close()
    return got, ref, parts


@pytest.mark.parametrize("boundaries", [("open", "periodic"), ("open", "open")])
def test_laser_in_vacuum_matches_oracle(mods, cpu_oracle, boundaries):
    got, ref, _ = run(mods, cpu_oracle, "fp64", boundaries, 40, False, True)
    assert np.abs(ref["Bz"]).max() > 1e-3  # the pulse has entered
    for k in FIELDS:
        assert rel_err(got[k], ref[k]) <= 1e-12, k


@pytest.mark.parametrize("form,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
def test_open_plasma_with_laser_matches_oracle(mods, cpu_oracle, form, tol):
    got, ref, (pg, mg, pr, mr) = run(mods, cpu_oracle, form, ("open", "open"), 6, True, True)
    for k in FIELDS:
        assert rel_err(got[k], ref[k]) <= tol, (k, rel_err(got[k], ref[k]))
    assert rel_err(mg, mr) <= tol
    assert np.abs(pg - pr).max() <= (1e-10 if form == "fp64" else 1e-5)


def test_particles_leave_through_open_boundaries(mods, cpu_oracle):
    # hot plasma, periodic y: particles leave only through x
    got, ref, (pg, mg, pr, mr) = run(mods, cpu_oracle, "fp64", ("open", "periodic"), 8, True, False)
    for k in FIELDS:
        assert rel_err(got[k], ref[k]) <= 1e-12, k
    assert pg.shape[1] < 4 * 32 * 24  # some left
    assert rel_err(mg, mr) <= 1e-12
