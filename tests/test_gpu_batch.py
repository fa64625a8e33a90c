"""Batched steps: sg_sim_step with graphs runs up to 8 steps as one graph, each step
behind a conditional node that a gate kernel arms from the previous step's device
flags, and the host waits once per batch.

- The same run stepped in batches and one step at a time agrees: FP64 within 1e-12,
  the mixed form within 1e-4 after 10 steps (the deposit's atomics add in a
  run-dependent order, which the plasma amplifies); 2D and 3D, full batches and a
  remainder.
- A spill inside a batch stops it on the device; the host re-lays out the species and
  goes on: after 11 steps the run still matches the oracle at 1e-12.
- The moving window: the steps at which it shifts run one by one and the others in
  batches; window state, particle counts and fields as with single steps.
"""
import numpy as np
import pytest

from conftest import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FIELDS = ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Bx_m", "By_m", "Bz_m", "Jx", "Jy", "Jz"]


@pytest.fixture(scope="module")
def sim_mod():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from smilei_gb300 import simulation, synthetic
    import test_gpu_sim as tg
    return simulation, synthetic, tg


def _build(simulation, n_cells, cl, dt, form, fields, species, **kw):
    sim = simulation.Simulation(n_cells, cl, dt, form=form, use_graph=True, **kw)
    for k in FIELDS:
        sim.set_field(k, fields[k])
    for s in species:
        sim.add_species(s["mass"], s["q"], s["pusher"], s["pos"], s["mom"], s["weight"])
    return sim


@pytest.mark.parametrize("ndim,form,nsteps,tol,queue", [(3, "fp64", 19, 1e-12, False), (2, "fp64", 19, 1e-12, False),
                                                        (3, "mixed", 10, 1e-4, False), (2, "mixed", 10, 1e-4, False),
                                                        (3, "mixed", 10, 1e-4, True)])
def test_batched_steps_match_single_steps(sim_mod, ndim, form, nsteps, tol, queue):
    """queue: the persistent tile-queue kernel, whose counter is reset inside each step."""
    simulation, synthetic, tg = sim_mod
    spec = [(1.0, -1, "boris", 4, 0.3), (1836.0, 1, "higueracary", 2, 0.01)]
    n_cells, cl, dt, fields, species = tg.make_case(synthetic, ndim, 7, spec)
    a = _build(simulation, n_cells, cl, dt, form, fields, species)
    b = _build(simulation, n_cells, cl, dt, form, fields, species)
    if queue:
        a.set_tile_queue(True)
        b.set_tile_queue(True)
    a.step(nsteps)
    for _ in range(nsteps):
        b.step(1)
    batches, steps, unsupported = a.batch_stats()
    assert unsupported == 0
    assert steps == nsteps and batches == (nsteps + 7) // 8
    assert b.batch_stats()[:2] == (0, 0)
    assert a.last_timing()[2] == -1.0 and b.last_timing()[2] > 0.0
    for k in FIELDS:
        assert rel_err(a.get_field(k), b.get_field(k)) <= tol, k
    for i in range(len(species)):
        assert a.species_count(i) == b.species_count(i) == species[i]["weight"].size
        pa, ma, wa = a.get_species(i)
        pb, mb, wb = b.get_species(i)
        oa, ob = np.argsort(wa, kind="stable"), np.argsort(wb, kind="stable")
        assert np.array_equal(wa[oa], wb[ob])
        assert rel_err(ma[:, oa], mb[:, ob]) <= tol
        assert tg.position_error(pa[:, oa], pb[:, ob], cl, n_cells) <= tol * 100
    a.close()
    b.close()


def test_spill_inside_a_batch_relayouts_and_matches_oracle(sim_mod, cpu_oracle):
    """Hot particles and zero slack: tiles overflow within batches."""
    simulation, synthetic, tg = sim_mod
    spec = [(1.0, -1, "boris", 3, 2.0)]
    n_cells, cl, dt, fields, species = tg.make_case(synthetic, 3, 11, spec)
    sim = _build(simulation, n_cells, cl, dt, "fp64", fields, species, tile=[2, 2, 2], capacity_slack=1e-6)
    sim.step(11)
    relayouts, spilled = sim.layout_stats()
    batches, steps, unsupported = sim.batch_stats()
    assert unsupported == 0 and relayouts > 0 and spilled > 0
    # a spill ends its batch after that step; a last single step runs on its own
    assert batches >= 2 and 8 < steps <= 11
    ref = {k: v.copy() for k, v in fields.items()}
    ref_sp = [dict(s, pos=s["pos"].copy(), mom=s["mom"].copy()) for s in species]
    for _ in range(11):
        cpu_oracle.pic_step(3, n_cells, 2, cl, dt, ref, ref_sp)
    for k in FIELDS:
        assert rel_err(sim.get_field(k), ref[k]) <= 1e-12, k
    pos, mom, w = sim.get_species(0)
    assert pos.shape[1] == species[0]["pos"].shape[1]
    o, r = np.argsort(w), np.argsort(ref_sp[0]["weight"])
    assert rel_err(mom[:, o], ref_sp[0]["mom"][:, r]) <= 1e-12
    sim.close()


def _wake(simulation):
    sim = simulation.Simulation([384, 64], [0.1, 1.5], 0.095, form="fp64", boundaries=("open", "open"))
    sim.add_laser_gaussian2d(a0=2.0, waist=30.0, focus=[0.0, 48.0], t_fwhm=60.0, t_center=60.0 * 2 ** 0.5,
                             t_start=0.0, t_duration=400.0)
    sim.add_species(1.0, -1.0, "vay", np.zeros((2, 0)), np.zeros((3, 0)), np.zeros(0))
    sim.set_species_profile(0, 0.003, 4, x_vacuum=2.0, x_slope1=10.0, x_plateau=36.4)
    sim.fill_species(0)
    sim.set_moving_window(20.0, 1.0, 32)
    return sim


def test_moving_window_batches_around_the_shifts(sim_mod):
    simulation, _, _ = sim_mod
    a, b = _wake(simulation), _wake(simulation)
    a.step(260)
    for _ in range(260):
        b.step(1)
    assert a.window_state() == b.window_state()
    assert a.window_state()[2] >= 1
    assert a.species_count(0) == b.species_count(0) > 0
    batches, steps, unsupported = a.batch_stats()
    assert unsupported == 0 and 0 < steps < 260
    for k in ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Jx", "Jy", "Jz"]:
        fa, fb = a.get_field(k), b.get_field(k)
        assert float(np.abs(fa - fb).max() / max(np.abs(fb).max(), 1e-300)) <= 1e-9, k
    a.close()
    b.close()
