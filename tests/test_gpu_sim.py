"""GPU parity of the resident timestep (sg_sim) with the oracle's full PIC step.

The oracle step (or_pic_step: gather, push, Esirkepov deposit, periodic wrap,
J ghost fold, Ampere, Faraday, B centring) runs on the same seeded plasma and
fields; particles are matched by their (unique) weights.  FP64 form: 1e-12
relative on every field and on momenta/positions.  Mixed form (int cell +
FP32 offset, FP32 arithmetic): 1e-5 relative after one step.
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
    return simulation, synthetic


def make_case(synthetic, ndim, seed, species_spec):
    n_cells = [16, 12, 8][:ndim] if ndim == 3 else [32, 24]
    cl = [0.1, 0.12, 0.09][:ndim]
    dt = 0.95 / np.sqrt(sum(1.0 / c ** 2 for c in cl))
    fields = synthetic.periodic_em(seed, n_cells)
    species = []
    for k, (mass, charge, pusher, ppc, sigma) in enumerate(species_spec):
        pos, mom, w = synthetic.thermal_plasma(n_cells, cl, ppc, sigma, seed + 10 + k, unique_weights=True)
        species.append(dict(pos=pos, mom=mom, weight=w, charge=np.full(w.shape, int(charge), np.int16),
                            mass=mass, pusher=pusher, q=charge))
    return n_cells, cl, dt, fields, species


def run_pair(sim_mod, cpu_oracle, ndim, form, nsteps, species_spec, seed=5, tile=None, tile_queue=False, tma=False):
    simulation, synthetic = sim_mod
    n_cells, cl, dt, fields, species = make_case(synthetic, ndim, seed, species_spec)
    sim = simulation.Simulation(n_cells, cl, dt, form=form, tile=tile, use_graph=True)
    for k in FIELDS:
        sim.set_field(k, fields[k])
    for s in species:
        sim.add_species(s["mass"], s["q"], s["pusher"], s["pos"], s["mom"], s["weight"])
    if tile_queue:
        sim.set_tile_queue(True)
    if ndim == 3 and form == "mixed" and tile in (None, [4, 4, 4]):
        sim.set_tma_staging(tma)  # TMA is this case's default: off tests the word copies
    sim.step(nsteps)
    ref = {k: v.copy() for k, v in fields.items()}
    ref_sp = [dict(s, pos=s["pos"].copy(), mom=s["mom"].copy()) for s in species]
    for _ in range(nsteps):
        cpu_oracle.pic_step(ndim, n_cells, 2, cl, dt, ref, ref_sp)
    got = {k: sim.get_field(k) for k in FIELDS}
    parts = []
    for i, s in enumerate(ref_sp):
        pos, mom, w = sim.get_species(i)
        assert pos.shape[1] == s["pos"].shape[1]
        order_got = np.argsort(w, kind="stable")
        order_ref = np.argsort(s["weight"].astype(np.float32) if form == "mixed" else s["weight"], kind="stable")
        parts.append((pos[:, order_got], mom[:, order_got], s["pos"][:, order_ref], s["mom"][:, order_ref], cl,
                      n_cells))
    sim.close()
    return got, ref, parts


def position_error(p_got, p_ref, cl, n_cells):
    """Largest periodic distance between matched particles, in cells."""
    err = 0.0
    for d in range(p_got.shape[0]):
        L = n_cells[d] * cl[d]
        dd = np.abs(p_got[d] - p_ref[d])
        dd = np.minimum(dd, L - dd) / cl[d]
        err = max(err, float(dd.max()))
    return err


@pytest.mark.parametrize("ndim,pusher", [(3, "higueracary"), (3, "boris"), (2, "boris"), (2, "vay")])
def test_fp64_step_matches_oracle(sim_mod, cpu_oracle, ndim, pusher):
    spec = [(1.0, -1, pusher, 4, 0.3), (1836.0, 1, pusher, 2, 0.01)]
    got, ref, parts = run_pair(sim_mod, cpu_oracle, ndim, "fp64", 3, spec)
    for k in FIELDS:
        assert rel_err(got[k], ref[k]) <= 1e-12, k
    for pg, mg, pr, mr, cl, nc in parts:
        assert rel_err(mg, mr) <= 1e-12
        assert position_error(pg, pr, cl, nc) <= 1e-10


# ppc 64 (3D) and 96 (2D) put 4096 / 6144 particles in a tile: several chunks of the
# per-cell mode's shared planes per tile
@pytest.mark.parametrize("ndim,pusher,ppc", [(3, "higueracary", 4), (2, "boris", 4), (3, "boris", 64),
                                             (2, "vay", 96)])
def test_mixed_step_matches_fp64_oracle(sim_mod, cpu_oracle, ndim, pusher, ppc):
    spec = [(1.0, -1, pusher, ppc, 0.3)]
    got, ref, parts = run_pair(sim_mod, cpu_oracle, ndim, "mixed", 1, spec)
    for k in FIELDS:
        assert rel_err(got[k], ref[k]) <= 1e-5, k
    for pg, mg, pr, mr, cl, nc in parts:
        assert rel_err(mg, mr) <= 1e-5
        assert position_error(pg, pr, cl, nc) <= 1e-5


def test_fp64_step_with_tile_spill_and_relayout(sim_mod, cpu_oracle):
    """Hot particles and zero slack force spills and re-layouts; results must not change."""
    simulation, synthetic = sim_mod
    spec = [(1.0, -1, "boris", 3, 2.0)]
    n_cells, cl, dt, fields, species = make_case(synthetic, 3, 11, spec)
    sim = simulation.Simulation(n_cells, cl, dt, form="fp64", tile=[2, 2, 2], capacity_slack=1e-6, use_graph=True)
    for k in FIELDS:
        sim.set_field(k, fields[k])
    s = species[0]
    sim.add_species(s["mass"], s["q"], s["pusher"], s["pos"], s["mom"], s["weight"])
    sim.step(4)
    ref = {k: v.copy() for k, v in fields.items()}
    ref_sp = [dict(s, pos=s["pos"].copy(), mom=s["mom"].copy())]
    for _ in range(4):
        cpu_oracle.pic_step(3, n_cells, 2, cl, dt, ref, ref_sp)
    for k in FIELDS:
        assert rel_err(sim.get_field(k), ref[k]) <= 1e-12, k
    pos, mom, w = sim.get_species(0)
    assert pos.shape[1] == s["pos"].shape[1]
    o = np.argsort(w)
    r = np.argsort(ref_sp[0]["weight"])
    assert rel_err(mom[:, o], ref_sp[0]["mom"][:, r]) <= 1e-12
    sim.close()


def test_energy_diagnostic_matches_numpy(sim_mod):
    simulation, synthetic = sim_mod
    n_cells, cl = [16, 16, 8], [0.1, 0.1, 0.1]
    fields = synthetic.periodic_em(3, n_cells, 0.2, 0.3)
    pos, mom, w = synthetic.thermal_plasma(n_cells, cl, 2, 0.2, 4)
    sim = simulation.Simulation(n_cells, cl, 0.05, form="fp64")
    for k in FIELDS:
        sim.set_field(k, fields[k])
    sim.add_species(1.0, -1.0, "boris", pos, mom, w)
    uk, ue = sim.energy()
    uk_ref = np.sum(w * (np.sqrt(1 + (mom ** 2).sum(0)) - 1.0))
    ue_ref = 0.0
    for k in ("Ex", "Ey", "Ez", "Bx_m", "By_m", "Bz_m"):
        a = fields[k][2:2 + n_cells[0], 2:2 + n_cells[1], 2:2 + n_cells[2]]
        ue_ref += 0.5 * np.prod(cl) * np.sum(a * a)
    assert abs(uk - uk_ref) <= 1e-12 * abs(uk_ref)
    assert abs(ue - ue_ref) <= 1e-12 * abs(ue_ref)
    sim.close()


def test_autotune_times_every_candidate_and_keeps_the_fastest(sim_mod):
    simulation, synthetic = sim_mod
    from smilei_gb300 import autotune
    n_cells, cl = [16, 16, 16], [0.1, 0.1, 0.1]
    dt = 0.95 / np.sqrt(sum(1.0 / c ** 2 for c in cl))
    pos, mom, w, ppc_p = synthetic.uneven_plasma(n_cells, cl, [8, 8, 8], 8, 1.5, 64, 0.14, 4)
    assert ppc_p.max() > ppc_p.min()

    def build(tile):
        sim = simulation.Simulation(n_cells, cl, dt, form="mixed", tile=list(tile))
        sim.add_species(1.0, -1.0, "boris", pos, mom, w)
        return sim

    best, times = autotune.tune_tiles(build, ndim=3, warmup=1, steps=2)
    assert set(times) == set(autotune.CANDIDATES_3D)
    assert best == min(times, key=times.get) and all(t > 0 for t in times.values())
    # the (tile, queue, staging) search: TMA staging is tried for the 4x4x4 tile only
    best3, times3 = autotune.tune(build, ndim=3, tiles=[(4, 4, 4), (8, 4, 2)], warmup=1, steps=1)
    assert set(times3) == {((4, 4, 4), q, t) for q in (False, True) for t in (True, False)} | \
        {((8, 4, 2), q, False) for q in (False, True)}
    assert best3 == min(times3, key=times3.get)


@pytest.mark.parametrize("form,n_cells", [("mixed", [16, 16, 16]), ("fp64", [16, 16, 16]), ("mixed", [8, 16, 16])])
def test_step_host_matches_unpack_step_pack(sim_mod, form, n_cells):
    """sg_sim_step_host (the copy in overlapped with the particle kernel over tile
    ranges, and with 3 or more x-slabs of tiles the copy out overlapped too) gives the
    particles of unpack -> step -> pack: identical after the first step, equal to
    rounding afterwards (the order of the deposit's atomics differs)."""
    simulation, synthetic = sim_mod
    cl = [0.1, 0.1, 0.1]
    dt = 0.95 * 0.1 / np.sqrt(3.0)
    pos, mom, w = synthetic.thermal_plasma(n_cells, cl, 8, 0.14, 4, unique_weights=True)

    def make():
        sim = simulation.Simulation(n_cells, cl, dt, form=form)
        sim.add_species(1.0, -1.0, "higueracary", pos, mom, w)
        return sim

    def particles(sim):
        p, m, wt = sim.get_species(0)
        o = np.argsort(wt)
        return p[:, o], m[:, o], wt[o]

    a, b = make(), make()
    nb = a.packed_bytes(0)
    ha = np.zeros(nb, dtype=np.uint8)
    a.pack_state(0, ha.ctypes.data)
    torch.cuda.synchronize()
    hb = ha.copy()  # the order inside a tile is not deterministic: both start from the same one
    b.unpack_state(0, hb.ctypes.data)
    tol = dict(rtol=0, atol=1e-10) if form == "fp64" else dict(rtol=0, atol=2e-6)
    for it, chunks in enumerate([5, 1, 64, 3]):
        a.unpack_state(0, ha.ctypes.data)
        a.step(1)
        a.pack_state(0, ha.ctypes.data)
        torch.cuda.synchronize()
        b.step_host(0, hb.ctypes.data, chunks=chunks)
        # the per-tile counts are deterministic
        nt = int(np.prod(n_cells)) // 64
        assert np.array_equal(ha[:8 + 4 * nt], hb[:8 + 4 * nt])
        pa, ma, wa = particles(a)
        pb, mb, wb = particles(b)
        assert np.array_equal(wa, wb)
        if it == 0:
            assert np.array_equal(pa, pb) and np.array_equal(ma, mb)
        else:
            np.testing.assert_allclose(pb, pa, **tol)
            np.testing.assert_allclose(mb, ma, **tol)
    ua, ub = a.energy(), b.energy()
    np.testing.assert_allclose(ub, ua, rtol=1e-5 if form == "mixed" else 1e-10)
    # the streamed step left the sums of its new state; a fresh pass gives the same
    b.step(0)
    np.testing.assert_allclose(b.energy(), ub, rtol=1e-12)
    with pytest.raises(RuntimeError):
        b.step_host(0, hb.ctypes.data, chunks=0)
    bad = hb.copy()
    bad[:8] = np.frombuffer(np.int64(len(w) + 1).tobytes(), dtype=np.uint8)
    with pytest.raises(RuntimeError):
        b.step_host(0, bad.ctypes.data)
    a.close()
    b.close()


def test_step_host_refuses_a_tile_over_its_segment_and_leaves_the_input(sim_mod):
    """A packed state whose tile holds more particles than its segment in the current
    layout is refused before anything is copied: host_in (here also host_out) keeps
    its bytes, and the simulation can still step the valid state afterwards."""
    simulation, synthetic = sim_mod
    n_cells, cl = [16, 16, 16], [0.1, 0.1, 0.1]
    dt = 0.95 * 0.1 / np.sqrt(3.0)
    pos, mom, w = synthetic.thermal_plasma(n_cells, cl, 8, 0.14, 4, unique_weights=True)
    sim = simulation.Simulation(n_cells, cl, dt, form="mixed")
    sim.add_species(1.0, -1.0, "higueracary", pos, mom, w)
    host = np.zeros(sim.packed_bytes(0), dtype=np.uint8)
    sim.pack_state(0, host.ctypes.data)
    torch.cuda.synchronize()
    nt = int(np.prod(n_cells)) // 64
    counts = host[8:8 + 4 * nt].view(np.int32)
    bad = host.copy()
    bc = bad[8:8 + 4 * nt].view(np.int32)
    moved = int(counts[1]) // 2 + 300  # tile 0 far over its capacity; the total is unchanged
    moved = min(moved, int(counts[1]))
    bc[0] += moved
    bc[1] -= moved
    before = bad.copy()
    with pytest.raises(RuntimeError, match="segment"):
        sim.step_host(0, bad.ctypes.data, chunks=4)
    assert np.array_equal(bad, before)
    sim.step_host(0, host.ctypes.data, chunks=4)
    assert sim.species_count(0) == len(w)
    sim.close()


@pytest.mark.parametrize("form", ["mixed", "fp64"])
def test_packed_state_round_trip(sim_mod, form):
    """pack -> (one more step) -> unpack restores the packed particles exactly; the
    packed bytes carry no segment slack."""
    simulation, synthetic = sim_mod
    n_cells, cl = [16, 16, 16], [0.1, 0.1, 0.1]
    dt = 0.95 * 0.1 / np.sqrt(3.0)
    pos, mom, w = synthetic.thermal_plasma(n_cells, cl, 8, 0.14, 4, unique_weights=True)
    sim = simulation.Simulation(n_cells, cl, dt, form=form)
    sim.add_species(1.0, -1.0, "higueracary", pos, mom, w)
    sim.step(2)
    nb = sim.packed_bytes(0)
    assert nb < sim.state_bytes(0)
    host = np.zeros(nb, dtype=np.uint8)
    sim.pack_state(0, host.ctypes.data)
    torch.cuda.synchronize()
    p1, m1, w1 = sim.get_species(0)
    sim.step(1)
    p2, _, _ = sim.get_species(0)
    assert not np.array_equal(np.sort(p2[0]), np.sort(p1[0]))
    sim.unpack_state(0, host.ctypes.data)
    p3, m3, w3 = sim.get_species(0)
    o1, o3 = np.lexsort((p1[0], w1)), np.lexsort((p3[0], w3))
    assert np.array_equal(w1[o1], w3[o3])
    assert np.array_equal(p1[:, o1], p3[:, o3]) and np.array_equal(m1[:, o1], m3[:, o3])
    sim.close()


@pytest.mark.parametrize("ndim,form,tol", [(3, "mixed", 1e-5), (3, "fp64", 1e-12), (2, "mixed", 1e-5)])
def test_tile_queue_step_matches_oracle(sim_mod, cpu_oracle, ndim, form, tol):
    """The persistent particle kernel (CTAs take tiles from a device queue, densest first)
    gives the oracle's step like the one-CTA-per-tile launch, over 3 steps (the third
    and later steps replay the captured graph, with the queue counter reset inside it)."""
    spec = [(1.0, -1.0, "higueracary" if ndim == 3 else "vay", 6, 0.14)]
    got, ref, parts = run_pair(sim_mod, cpu_oracle, ndim, form, 3, spec, tile_queue=True)
    for k in FIELDS:
        assert rel_err(got[k], ref[k]) <= tol * 10, k
    for pg, mg, pr, mr, cl, n_cells in parts:
        assert rel_err(mg, mr) <= tol * 10
        assert position_error(pg, pr, cl, n_cells) <= tol * 10


@pytest.mark.parametrize("pusher,ppc,queue", [("higueracary", 6, False), ("boris", 64, False), ("vay", 40, True)])
def test_tma_staging_step_matches_oracle(sim_mod, cpu_oracle, pusher, ppc, queue):
    """The field tile staged by TMA (tensor copies of padded E and B_m, one mbarrier per
    tile) gives the oracle's step like the word copies: 3 graph-replayed steps of the
    16 x 12 x 8 grid (tiles at every grid edge, so boxes reach past the arrays and read
    the tensor maps' zero fill), and dense cases whose tiles take several chunks (each
    chunk after the first stages the field tile again: the previous chunk kept its
    node-changing list there), one of them with the persistent tile queue."""
    spec = [(1.0, -1.0, pusher, ppc, 0.14)]
    got, ref, parts = run_pair(sim_mod, cpu_oracle, 3, "mixed", 3 if ppc < 32 else 1, spec, tma=True,
                               tile_queue=queue)
    tol = 1e-4 if ppc < 32 else 1e-5
    for k in FIELDS:
        assert rel_err(got[k], ref[k]) <= tol, k
    for pg, mg, pr, mr, cl, n_cells in parts:
        assert rel_err(mg, mr) <= tol
        assert position_error(pg, pr, cl, n_cells) <= tol


def test_tma_copies_follow_fields_set_between_steps(sim_mod):
    """With TMA staging the field kernels keep the padded copies of E and B_m that the
    tensor maps read; a field set from the host between (graph-replayed) steps makes the
    next step copy them again.  The same sequence with word copies (which read the arrays
    themselves) must give the same fields and momenta: 2 steps, new E and B_m from the
    host, 2 more steps (1e-5: the deposit's atomics add in another order)."""
    simulation, synthetic = sim_mod
    n_cells, cl, dt, fields, species = make_case(synthetic, 3, 9, [(1.0, -1.0, "boris", 6, 0.14)])
    fields2 = synthetic.periodic_em(17, n_cells)
    out = []
    for tma in (True, False):
        sim = simulation.Simulation(n_cells, cl, dt, form="mixed", use_graph=True)
        sim.set_tma_staging(tma)
        for k in FIELDS:
            sim.set_field(k, fields[k])
        s = species[0]
        sim.add_species(s["mass"], s["q"], s["pusher"], s["pos"], s["mom"], s["weight"])
        sim.step(2)
        for k in ("Ex", "Ey", "Ez", "Bx_m", "By_m", "Bz_m"):
            sim.set_field(k, fields2[k])
        sim.step(2)
        p, m, w = sim.get_species(0)
        o = np.argsort(w)
        out.append(({k: sim.get_field(k) for k in FIELDS}, m[:, o]))
        sim.close()
    (fa, ma), (fb, mb) = out
    for k in FIELDS:
        assert rel_err(fa[k], fb[k]) <= 1e-5, k
    assert rel_err(ma, mb) <= 1e-5
