"""GPU parity of the drop-in operators with the oracle, on the golden inputs.

Each operator runs through libsmileigb300.so (C ABI) on the inputs stored in
tests/golden/operators.npz; its output is compared with the C oracle on the
same inputs and with the reference's own output stored in the fixture.
Tolerance: 1e-12 relative (max|a-b| / max|b|), the FP64 parity bar.
"""
import numpy as np
import pytest

from conftest import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12
EB = ["Ex", "Ey", "Ez", "Bx", "By", "Bz"]


def cu(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


@pytest.fixture(scope="module")
def ops():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from smilei_gb300 import operators
    return operators


@pytest.mark.parametrize("ndim", [2, 3])
def test_interpolator(ops, golden_ops, cpu_oracle, ndim):
    g = golden_ops[f"interp{ndim}d"]
    geom = ops.PatchGeometry.from_arrays(g["n_prim"], g["domain_begin"], g["cell_length"])
    em = ops.ElectroMagn(geom)
    em.Ex_.copy_(cu(g["Ex"])); em.Ey_.copy_(cu(g["Ey"])); em.Ez_.copy_(cu(g["Ez"]))
    em.Bx_m.copy_(cu(g["Bx"])); em.By_m.copy_(cu(g["By"])); em.Bz_m.copy_(cu(g["Bz"]))
    n = g["pos"].shape[1]
    part = ops.Particles(cu(g["pos"]), torch.zeros(3, n, dtype=torch.float64, device="cuda"),
                         torch.ones(n, dtype=torch.float64, device="cuda"), torch.ones(n, dtype=torch.int16, device="cuda"))
    smpi = ops.SmileiMPI(ndim, n)
    interp = (ops.Interpolator3D2Order if ndim == 3 else ops.Interpolator2D2Order)(geom)
    interp.fieldsWrapper(em, part, smpi, 0, n)
    torch.cuda.synchronize()
    E, B, iold, delta = cpu_oracle.interpolate(ndim, g["n_prim"], g["domain_begin"], g["cell_length"],
                                               [g[k] for k in EB], g["pos"])
    assert rel_err(smpi.dynamics_Epart.cpu().numpy(), E) <= TOL
    assert rel_err(smpi.dynamics_Bpart.cpu().numpy(), B) <= TOL
    assert rel_err(smpi.dynamics_Epart.cpu().numpy(), g["E"]) <= TOL
    assert np.array_equal(smpi.dynamics_iold.cpu().numpy(), iold)
    assert rel_err(smpi.dynamics_deltaold.cpu().numpy(), delta) <= TOL


def test_pushers(ops, golden_ops, cpu_oracle):
    names = sorted(k for k in golden_ops if k.startswith("push_"))
    for c in names:
        g = golden_ops[c]
        nd = int(g["ndim"]); n = g["mom"].shape[1]
        part = ops.Particles(cu(g["pos"]), cu(g["mom"]), torch.ones(n, dtype=torch.float64, device="cuda"),
                             cu(g["charge"], torch.int16))
        smpi = ops.SmileiMPI(nd, n)
        smpi.dynamics_Epart.copy_(cu(g["E"])); smpi.dynamics_Bpart.copy_(cu(g["B"]))
        ops.PusherFactory(str(g["kind"]), float(g["dt"]), float(g["mass"]), nd)(part, smpi)
        torch.cuda.synchronize()
        pos, mom, invgf = cpu_oracle.push(str(g["kind"]), nd, float(g["dt"]), float(g["mass"]), g["pos"], g["mom"],
                                          g["charge"], g["E"], g["B"])
        assert rel_err(part.momentum.cpu().numpy(), mom) <= TOL, c
        assert rel_err(part.momentum.cpu().numpy(), g["mom_out"]) <= TOL, c
        assert rel_err(part.position.cpu().numpy(), pos) <= TOL, c
        assert rel_err(smpi.dynamics_invgf.cpu().numpy(), invgf) <= TOL, c


@pytest.mark.parametrize("ndim", [2, 3])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_projector(ops, golden_ops, cpu_oracle, ndim, mode):
    g = golden_ops[f"project{ndim}d_mode{mode}"]
    geom = ops.PatchGeometry.from_arrays(g["n_prim"], g["domain_begin"], g["cell_length"])
    em = ops.ElectroMagn(geom)
    for k, t in (("Jx", em.Jx_), ("Jy", em.Jy_), ("Jz", em.Jz_), ("rho", em.rho_)):
        t.copy_(cu(g[k + "_in"]))
    n = g["pos"].shape[1]
    part = ops.Particles(cu(g["pos"]), cu(g["mom"]), cu(g["weight"]), cu(g["charge"], torch.int16))
    smpi = ops.SmileiMPI(ndim, n)
    smpi.dynamics_invgf.copy_(cu(g["invgf"]))
    smpi.dynamics_iold.copy_(cu(g["iold"], torch.int32))
    smpi.dynamics_deltaold.copy_(cu(g["delta"]))
    proj = (ops.Projector3D2Order if ndim == 3 else ops.Projector2D2Order)(geom, float(g["dt"]))
    if mode == 2:
        proj.basic(em, part)
    else:
        proj.currentsAndDensityWrapper(em, part, smpi, 0, n, 0, diag_flag=(mode == 1))
    torch.cuda.synchronize()
    J = [g[k + "_in"].copy() for k in ("Jx", "Jy", "Jz", "rho")]
    cpu_oracle.project(mode, ndim, g["n_prim"], g["domain_begin"], g["cell_length"], float(g["dt"]), g["pos"],
                       g["mom"], g["weight"], g["charge"], g["invgf"], g["iold"], g["delta"], J)
    for t, ref, k in zip((em.Jx_, em.Jy_, em.Jz_, em.rho_), J, ("Jx", "Jy", "Jz", "rho")):
        got = t.cpu().numpy() - g[k + "_in"]
        assert rel_err(got, ref - g[k + "_in"]) <= TOL, k
        assert rel_err(got, g[k] - g[k + "_in"]) <= TOL, k


@pytest.mark.parametrize("ndim", [2, 3])
def test_maxwell_and_centring(ops, golden_ops, cpu_oracle, ndim):
    names = ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Jx", "Jy", "Jz"]
    for which in (0, 1):
        g = golden_ops[f"maxwell{ndim}d_{'ampere' if which == 0 else 'faraday'}"]
        geom = ops.PatchGeometry.from_arrays(g["n_prim"], [0] * ndim, g["cell_length"])
        em = ops.ElectroMagn(geom)
        tens = [em.Ex_, em.Ey_, em.Ez_, em.Bx_, em.By_, em.Bz_, em.Jx_, em.Jy_, em.Jz_]
        for t, k in zip(tens, names):
            t.copy_(cu(g[k + "_in"]))
        em.saveMagneticFields()
        (ops.MA_Solver_norm if which == 0 else ops.MF_Solver_Yee)(float(g["dt"]))(em)
        em.centerMagneticFields()
        torch.cuda.synchronize()
        F = [g[k + "_in"].copy() for k in names]
        cpu_oracle.maxwell(which, ndim, g["n_prim"], g["cell_length"], float(g["dt"]), F)
        for t, ref, k in zip(tens, F, names):
            assert rel_err(t.cpu().numpy(), ref) <= TOL, (which, k)
            assert rel_err(t.cpu().numpy(), g[k]) <= TOL, (which, k)
        for t, k in zip((em.Bx_m, em.By_m, em.Bz_m), ("Bx", "By", "Bz")):
            assert rel_err(t.cpu().numpy(), 0.5 * (g[k] + g[k + "_in"])) <= TOL


@pytest.mark.parametrize("ndim", [2, 3])
def test_per_cell_sort(ops, cpu_oracle, ndim):
    rng = np.random.default_rng(7 + ndim)
    patch = [9, 7, 6][:ndim]
    cl = [0.1, 0.2, 0.15][:ndim]
    xmin = [3 * c for c in cl]
    n = 5000
    pos = np.stack([xmin[d] + rng.uniform(-0.49, patch[d] + 0.49, n) * cl[d] for d in range(ndim)])
    mom = rng.normal(0, 1, (3, n))
    w = rng.uniform(0.5, 1.5, n)
    q = rng.choice(np.array([-1, 1], dtype=np.int16), n)
    part = ops.Particles(cu(pos), cu(mom), cu(w), cu(q, torch.int16))
    first, last, keys = ops.sortParticles(part, patch, xmin, cl)
    torch.cuda.synchronize()
    k_ref, f_ref, l_ref, perm = cpu_oracle.sort(ndim, patch, xmin, cl, pos)
    assert np.array_equal(first.cpu().numpy(), f_ref)
    assert np.array_equal(last.cpu().numpy(), l_ref)
    assert np.array_equal(keys.cpu().numpy(), k_ref[perm])
    assert np.array_equal(part.position.cpu().numpy(), pos[:, perm])
    assert np.array_equal(part.momentum.cpu().numpy(), mom[:, perm])
    assert np.array_equal(part.weight.cpu().numpy(), w[perm])
    assert np.array_equal(part.charge.cpu().numpy(), q[perm])
    assert np.all(np.diff(keys.cpu().numpy()) >= 0)


def test_sort_rejects_particles_outside_the_patch(ops):
    from smilei_gb300 import SmileiGPUError
    pos = np.array([[0.05, 5.0]])
    part = ops.Particles(cu(pos), cu(np.zeros((3, 2))), cu(np.ones(2)), cu(np.ones(2), torch.int16))
    with pytest.raises(SmileiGPUError, match="outside"):
        ops.sortParticles(part, [8], [0.0], [0.1])


def test_empty_inputs_are_no_ops(ops):
    """Zero particles (an empty bin or species): every operator returns without touching
    the fields; the sort returns empty bins."""
    geom = ops.PatchGeometry([8, 8, 8], [0.1, 0.1, 0.1])
    em = ops.ElectroMagn(geom)
    for comp in ("Ex_", "By_m", "Jx_"):
        getattr(em, comp).fill_(1.5)
    part = ops.Particles(torch.zeros((3, 0), dtype=torch.float64, device="cuda"),
                         torch.zeros((3, 0), dtype=torch.float64, device="cuda"),
                         torch.zeros(0, dtype=torch.float64, device="cuda"),
                         torch.zeros(0, dtype=torch.int16, device="cuda"))
    smpi = ops.SmileiMPI(3, 0)
    ops.Interpolator3D2Order(geom).fieldsWrapper(em, part, smpi)
    ops.PusherFactory("boris", 0.05, 1.0, 3)(part, smpi)
    ops.Projector3D2Order(geom, 0.05).currentsAndDensityWrapper(em, part, smpi)
    first, last, keys = ops.sortParticles(part, [8, 8, 8], [0.0, 0.0, 0.0], [0.1, 0.1, 0.1])
    torch.cuda.synchronize()
    assert float(em.Jx_.min()) == 1.5 and float(em.Jx_.max()) == 1.5
    assert keys.numel() == 0 and int(first.sum()) == 0 and int(last.sum()) == 0


def test_resident_step_with_an_empty_species(ops):
    """A species without particles steps alongside a populated one; the result equals
    the populated species alone."""
    from smilei_gb300 import simulation, synthetic
    n_cells, cl = [16, 16], [0.1, 0.1]
    dt = 0.95 / np.sqrt(2 / 0.01)
    pos, mom, w = synthetic.thermal_plasma(n_cells, cl, 4, 0.1, 3)
    out = []
    for with_empty in (False, True):
        sim = simulation.Simulation(n_cells, cl, dt, form="fp64")
        if with_empty:
            sim.add_species(1.0, -1.0, "boris", np.zeros((2, 0)), np.zeros((3, 0)), np.zeros(0))
        sim.add_species(1.0, -1.0, "boris", pos, mom, w)
        sim.step(5)
        out.append(sim.get_field("Jx"))
        assert sim.species_count(1 if with_empty else 0) == w.size
        sim.close()
    assert rel_err(out[1], out[0]) <= 1e-12


@pytest.mark.parametrize("ndim", [2, 3])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("order", ["sorted", "shuffled"])
def test_projector_many_particles_sorted_and_shuffled(ops, cpu_oracle, ndim, mode, order):
    """200,000 particles in a 32 x 24 x 16-cell patch, sorted by cell (as the reference
    sorts them every step) or shuffled: the deposit matches the oracle at 1e-12 either
    way (many particles add into each node, in an order the atomics decide)."""
    rng = np.random.default_rng(17 + ndim + 10 * mode)
    cells = [32, 24, 16][:ndim]
    cl = [0.1, 0.12, 0.09][:ndim]
    n_prim = [c + 5 for c in cells]
    dom = [-2] * ndim
    dt = 0.95 / np.sqrt(sum(1.0 / c ** 2 for c in cl))
    n = 200_000
    pos0 = np.stack([rng.uniform(0.0, cells[d], n) * cl[d] for d in range(ndim)])
    stag = ([1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 1, 1], [1, 0, 1], [1, 1, 0])  # Ex Ey Ez Bx By Bz
    zeros = [np.zeros(tuple(n_prim[d] + st[d] for d in range(ndim))) for st in stag]
    _, _, iold, delta = cpu_oracle.interpolate(ndim, n_prim, dom, cl, zeros, pos0)
    mom = rng.normal(0.0, 0.3, (3, n))
    invgf = 1.0 / np.sqrt(1.0 + (mom ** 2).sum(0))
    pos = pos0 + mom[:ndim] * invgf * dt
    w = rng.uniform(0.5, 1.5, n)
    q = rng.choice(np.array([-1, 1], np.int16), n)
    if order == "sorted":
        o = np.lexsort(iold[::-1])
    else:
        o = rng.permutation(n)
    pos, mom, w, q, invgf, iold, delta = (pos[:, o], mom[:, o], w[o], q[o], invgf[o], iold[:, o], delta[:, o])
    geom = ops.PatchGeometry.from_arrays(n_prim, dom, cl)
    em = ops.ElectroMagn(geom)
    part = ops.Particles(cu(pos), cu(mom), cu(w), cu(q, torch.int16))
    smpi = ops.SmileiMPI(ndim, n)
    smpi.dynamics_invgf.copy_(cu(invgf))
    smpi.dynamics_iold.copy_(cu(iold, torch.int32))
    smpi.dynamics_deltaold.copy_(cu(delta))
    proj = (ops.Projector3D2Order if ndim == 3 else ops.Projector2D2Order)(geom, float(dt))
    proj.currentsAndDensityWrapper(em, part, smpi, 0, n, 0, diag_flag=(mode == 1))
    torch.cuda.synchronize()
    J = [np.zeros(tuple(t.shape)) for t in (em.Jx_, em.Jy_, em.Jz_, em.rho_)]
    cpu_oracle.project(mode, ndim, n_prim, dom, cl, float(dt), pos, mom, w, q, invgf, iold, delta, J)
    names = ("Jx", "Jy", "Jz", "rho") if mode == 1 else ("Jx", "Jy", "Jz")
    for t, ref, k in zip((em.Jx_, em.Jy_, em.Jz_, em.rho_), J, names):
        assert rel_err(t.cpu().numpy(), ref) <= TOL, k
