"""The 2D thermal plasma at its full size against the oracle's timestep.

256 x 256 cells, dx = dy = 0.1, dt = 0.95 CFL, periodic; electrons and protons
(mass 1836) at 16 particles per cell each (2,097,152 particles), T = 10 keV in
each species' own momentum unit, Boris pusher (PusherBoris.cpp:23), order-2
gather, Esirkepov deposit (Projector2D2Order.cpp:49), Yee -- the 2D thermal
workload of bench.py.  Random periodic E and B to start, so the gather and the
push see fields from the first step.

- FP64 form, one step: fields and every particle (matched by a unique weight)
  within 1e-12 relative (max|a - b| / max|b|) of oracle/pic_oracle.c.
- Mixed form, one step: the same within 1e-5.
- FP64 form, 200 steps: still within 1e-8 of the oracle after 200 steps (the
  deposit's atomic order changes the last bits, which the plasma amplifies).
- FP64 form from an FP64 Poisson solve, 200 steps: charge residual below 1e-9,
  every particle and the total weight kept.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N = [256, 256]
CL = [0.1, 0.1]
DT = 0.95 * 0.1 / np.sqrt(2.0)
PPC = 16
SIG = np.sqrt(10.0 / 511.0)
SPECIES = [(1.0, -1, SIG), (1836.0, 1, SIG / np.sqrt(1836.0))]
NAMES = ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Bx_m", "By_m", "Bz_m", "Jx", "Jy", "Jz"]


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import oracle
    from smilei_gb300 import simulation, synthetic
    return oracle, simulation, synthetic


def _setup(synthetic, seed=5):
    fields = synthetic.periodic_em(seed, N, 0.05, 0.05)
    sp = []
    for k, (m, q, sig) in enumerate(SPECIES):
        pos, mom, w = synthetic.thermal_plasma(N, CL, PPC, sig, seed + 100 * k, unique_weights=True)
        sp.append(dict(pos=pos, mom=mom, weight=w, charge=np.full(w.shape, q, np.int16), mass=m, pusher="boris"))
    return fields, sp


def _gpu(simulation, form, fields, sp):
    sim = simulation.Simulation(N, CL, DT, form=form)
    for k in NAMES:
        sim.set_field(k, fields[k])
    for s in sp:
        sim.add_species(s["mass"], float(s["charge"][0]), "boris", s["pos"], s["mom"], s["weight"])
    return sim


def _compare(sim, fields, sp, tol):
    for k in NAMES:
        got = sim.get_field(k)
        err = float(np.abs(got - fields[k]).max() / max(np.abs(fields[k]).max(), 1e-300))
        assert err <= tol, (k, err)
    for k, s in enumerate(sp):
        p, m, w = sim.get_species(k)
        assert w.size == s["weight"].size
        o1, o2 = np.argsort(s["weight"]), np.argsort(w)
        assert np.allclose(w[o2], s["weight"][o1], rtol=1e-6, atol=0)
        merr = float(np.abs(m[:, o2] - s["mom"][:, o1]).max() / np.abs(s["mom"]).max())
        assert merr <= tol, ("momenta", k, merr)
        # positions: the GPU wraps into [0, L); compare on the periodic circle, relative to a cell
        L = np.array([n * c for n, c in zip(N, CL)])[:, None]
        dpos = np.abs(p[:, o2] - s["pos"][:, o1])
        dpos = np.minimum(dpos, L - dpos) / np.array(CL)[:, None]
        assert float(dpos.max()) <= tol * 10, ("positions", k, float(dpos.max()))


def test_thermal2d_fp64_one_step_and_200_steps_match_oracle(mods):
    oracle, simulation, synthetic = mods
    fields, sp = _setup(synthetic)
    sim = _gpu(simulation, "fp64", fields, sp)
    O = oracle.Oracle()
    sim.step(1)
    O.pic_step(2, N, 2, CL, DT, fields, sp)
    _compare(sim, fields, sp, 1e-12)
    sim.step(199)
    for _ in range(199):
        O.pic_step(2, N, 2, CL, DT, fields, sp)
    _compare(sim, fields, sp, 1e-8)
    sim.close()


def test_thermal2d_mixed_one_step_matches_oracle(mods):
    oracle, simulation, synthetic = mods
    fields, sp = _setup(synthetic)
    sim = _gpu(simulation, "mixed", fields, sp)
    sim.step(1)
    oracle.Oracle().pic_step(2, N, 2, CL, DT, fields, sp)
    _compare(sim, fields, sp, 1e-5)
    sim.close()


def test_thermal2d_fp64_200_steps_charge_and_counts(mods):
    _, simulation, synthetic = mods
    _, sp = _setup(synthetic, seed=9)
    sim = simulation.Simulation(N, CL, DT, form="fp64")
    for s in sp:
        sim.add_species(s["mass"], float(s["charge"][0]), "boris", s["pos"], s["mom"], s["weight"])
    sim.solve_poisson(max_error=1e-24)  # far below the default, so the residual measures the steps
    before = [sim.species_scalars(k) for k in range(2)]
    sim.step(200)
    assert sim.charge_residual() <= 1e-9
    for k in range(2):
        after = sim.species_scalars(k)
        assert sim.species_count(k) == sp[k]["weight"].size
        assert after[1] == before[k][1]
        assert abs(after[0] - before[k][0]) <= 1e-12 * before[k][0]
    sim.close()
