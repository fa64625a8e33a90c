"""GPU Monte-Carlo radiation: table kernels, the Monte-Carlo pass and the MLP surrogate.

Tables are the reference's default tables (tests/golden/radiation.npz, dumped
from the reference's RadiationTablesDefault).  Table kernels must reproduce the
reference's outputs; the Monte-Carlo pass must reproduce the oracle's pass
drawing the same per-particle random streams, and the reference's own operator
(tests/golden/monte_carlo.npz); the network's gradients must
match the FP64 oracle's; the trained network is checked against the table: its
per-bin error decides where it is used, and the emitted spectrum and mean
energy loss of a Monte-Carlo pass using it are compared with the table-only pass.
"""
import numpy as np
import pytest

import oracle
from conftest import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rad(golden_rad):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from smilei_gb300 import radiation
    g = golden_rad
    f_dn, f_cl, inv_es = radiation.normalised_factors(2.0 * np.pi * 299792458.0 / 1e-6)  # lambda_r = 1 um
    T = radiation.RadiationTables(g["integfochi"], g["integfochi_min"], g["integfochi_max"], g["xi_table"],
                                  g["xi_min"], g["xi_max"], g["xi_axis1_min"], f_dn, f_cl, inv_es)
    Tc = oracle.RadTables.from_golden(g, factor_dNph_dt=f_dn, factor_classical=f_cl, inv_norm_E_schwinger=inv_es)
    return radiation, T, Tc


def cu(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def test_table_kernels_match_reference(rad, golden_rad):
    radiation, T, _ = rad
    g = golden_rad
    pc = T.photon_chi(cu(g["chi"]), cu(g["xi"])).cpu().numpy()
    assert np.max(np.abs(pc / g["photon_chi"] - 1.0)) <= 1e-12
    Ty = radiation.RadiationTables(g["integfochi"], g["integfochi_min"], g["integfochi_max"], g["xi_table"],
                                   g["xi_min"], g["xi_max"], g["xi_axis1_min"], float(g["factor"]), 1.0, 1.0)
    y = Ty.production_yield(cu(g["chi"]), cu(g["gamma"])).cpu().numpy()
    assert rel_err(y, g["yield_"]) <= 1e-12


def beam(n, seed):
    """An electron beam (gamma ~ 2000) in a strong field: chi spans about 0.1 - 10."""
    rng = np.random.default_rng(seed)
    mom = np.ascontiguousarray(np.stack([rng.normal(-2000, 40, n), rng.normal(0, 4, n), rng.normal(0, 4, n)]))
    E = rng.normal(0, 60, (3, n))
    B = rng.normal(0, 60, (3, n))
    return mom, E, B, np.ones(n)


def test_monte_carlo_pass_matches_oracle(rad):
    radiation, T, Tc = rad
    n = 20000
    mom, E, B, w = beam(n, 1)
    tau = np.full(n, -1.0)
    m_gpu, tau_gpu = cu(mom), cu(tau)
    chi_gpu = torch.zeros(n, dtype=torch.float64, device="cuda")
    total_g = total_o = 0.0
    nem_g = nem_o = 0
    for step in range(3):
        r_g, e_g = radiation.monte_carlo(T, 0.1, 1.0, -1.0, m_gpu, cu(w), tau_gpu, cu(E), cu(B), seed=99,
                                         step=step, chi_out=chi_gpu)
        r_o, e_o, chi_o = oracle.rad_monte_carlo(Tc, 0.1, 1.0, -1.0, mom, w, tau, E, B, seed=99, step=step)
        total_g += r_g; total_o += r_o; nem_g += e_g; nem_o += e_o
    assert nem_g == nem_o and nem_g > 1000
    assert abs(total_g - total_o) <= 1e-10 * total_o
    assert rel_err(m_gpu.cpu().numpy(), mom) <= 1e-12
    assert rel_err(chi_gpu.cpu().numpy(), chi_o) <= 1e-12
    assert 0.05 < chi_o.mean() < 20.0


def test_monte_carlo_photons_match_oracle(rad):
    """Macro-photon creation: the same emissions, photons and recoils as the oracle
    (photons come out in slot order on the GPU: compared sorted by chi)."""
    radiation, T, Tc = rad
    n = 20000
    mom, E, B, w = beam(n, 3)
    rng = np.random.default_rng(4)
    pos = np.ascontiguousarray(np.stack([rng.uniform(0, 10, n), rng.uniform(0, 5, n)]))
    w = rng.uniform(0.5, 1.5, n)
    tau = np.full(n, -1.0)
    m_gpu, tau_gpu = cu(mom), cu(tau)
    for step in range(2):
        r_g, e_g, ph_g = radiation.monte_carlo_photons(T, 0.1, 1.0, -1.0, cu(pos), m_gpu, cu(w), tau_gpu, cu(E), cu(B),
                                                       seed=5, step=step, sampling=2, gamma_threshold=20.0,
                                                       max_emissions=3)
        r_o, e_o, _, ph_o = oracle.rad_monte_carlo_photons(Tc, 0.1, 1.0, -1.0, pos, mom, w, tau, E, B, seed=5,
                                                           step=step, sampling=2, threshold=20.0, max_emissions=3)
        assert e_g == e_o and ph_o["weight"].size == ph_g["weight"].numel() > 1000
        assert abs(r_g - r_o) <= 1e-10 * max(abs(r_o), 1.0)
        og = np.lexsort((ph_g["weight"].cpu().numpy(), ph_g["chi"].cpu().numpy()))
        oo = np.lexsort((ph_o["weight"], ph_o["chi"]))
        for k in ["pos", "mom", "weight", "chi", "tau"]:
            a = ph_g[k].cpu().numpy()[..., og]
            assert rel_err(a, ph_o[k][..., oo]) <= 1e-12, k
    assert rel_err(m_gpu.cpu().numpy(), mom) <= 1e-12
    # photons then move in straight lines at c
    p_gpu = ph_g["pos"].contiguous().clone()
    radiation.push_photons(0.5, p_gpu, ph_g["mom"].contiguous())
    p_ref = ph_g["pos"].cpu().numpy().copy()
    oracle.push_photons(0.5, p_ref, ph_g["mom"].cpu().numpy())
    assert rel_err(p_gpu.cpu().numpy(), p_ref) <= 1e-15


@pytest.fixture(scope="module")
def golden_mc():
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "monte_carlo.npz"))
    return {k: z[k] for k in z.files}


def test_monte_carlo_pass_matches_reference_operator(rad, golden_rad, golden_mc):
    """The FP64 pass against the reference's own RadiationMonteCarlo::operator() outputs
    (tests/golden/monte_carlo.npz: each particle drew from a reference Random started at its
    stream's state): momenta, optical depths, final chi, radiated energy and the photons of the
    photon-species run (compared sorted by chi, the GPU takes slots atomically)."""
    radiation = rad[0]
    g, gr = golden_mc, golden_rad
    T = radiation.RadiationTables(gr["integfochi"], gr["integfochi_min"], gr["integfochi_max"], gr["xi_table"],
                                  gr["xi_min"], gr["xi_max"], gr["xi_axis1_min"], float(g["f_factor_dNph_dt"]),
                                  float(g["f_factor_classical"]), float(g["f_inv_norm_E_schwinger"]),
                                  float(g["f_min_chi_continuous"]), float(g["f_min_chi_discontinuous"]))
    n = g["weight"].size
    kw = dict(seed=int(g["seed"]), first_id=int(g["first_id"]), step=int(g["step"]))
    args = (float(g["dt"]), float(g["mass"]), float(g["charge"]))
    m_gpu, tau_gpu = cu(g["mom"]), cu(g["tau"])
    chi_gpu = torch.zeros(n, dtype=torch.float64, device="cuda")
    r_g, _ = radiation.monte_carlo(T, *args, m_gpu, cu(g["weight"]), tau_gpu, cu(g["E"]), cu(g["B"]), chi_out=chi_gpu,
                                   **kw)
    assert rel_err(m_gpu.cpu().numpy(), g["rad_mom"]) <= 1e-12
    assert np.max(np.abs(tau_gpu.cpu().numpy() - g["rad_tau"])) <= 1e-10
    assert rel_err(chi_gpu.cpu().numpy(), g["rad_chi"]) <= 1e-12
    assert abs(r_g - float(g["rad_radiated"])) <= 1e-11 * abs(float(g["rad_radiated"]))

    m_gpu, tau_gpu = cu(g["mom"]), cu(g["tau"])
    r_g, _, ph = radiation.monte_carlo_photons(T, *args, cu(g["pos"]), m_gpu, cu(g["weight"]), tau_gpu, cu(g["E"]),
                                               cu(g["B"]), sampling=int(g["sampling"]),
                                               gamma_threshold=float(g["threshold"]),
                                               max_emissions=int(g["max_emissions"]), **kw)
    assert ph["weight"].numel() == g["ph_photon_weight"].size > 100
    og = np.lexsort((ph["weight"].cpu().numpy(), ph["chi"].cpu().numpy()))
    oo = np.lexsort((g["ph_photon_weight"], g["ph_photon_chi"]))
    for k in ["pos", "mom", "weight", "chi", "tau"]:
        assert rel_err(ph[k].cpu().numpy()[..., og], g["ph_photon_" + k][..., oo]) <= 1e-12, k
    assert rel_err(m_gpu.cpu().numpy(), g["ph_mom"]) <= 1e-12
    assert abs(r_g - float(g["ph_radiated"])) <= 1e-11 * abs(float(g["ph_radiated"]))
    T.close()


def test_fp32_math_pass_agrees_with_fp64(rad):
    """The FP32-math pass draws the same random numbers as the FP64 pass and uses the
    same tables in FP32: the same emissions up to rare threshold flips, the same radiated
    energy and spectrum to well under a percent, and most particles' momenta at FP32
    rounding level.  It is also faster (FP64 is slow on this GPU)."""
    from smilei_gb300 import radiation as R
    radiation, T, _ = rad
    g = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "radiation.npz"))
    f_dn, f_cl, inv_es = R.normalised_factors(2.0 * np.pi * 299792458.0 / 1e-6)
    T32 = R.RadiationTables(g["integfochi"], g["integfochi_min"], g["integfochi_max"], g["xi_table"], g["xi_min"],
                            g["xi_max"], g["xi_axis1_min"], f_dn, f_cl, inv_es)
    T32.set_fp32_math(True)
    n = 400000
    mom, E, B, w = beam(n, 5)
    res, times = {}, {}
    for name, tab in (("fp64", T), ("fp32", T32)):
        m, tau = cu(mom), cu(np.full(n, -1.0))
        tot, nem = 0.0, 0
        radiation.monte_carlo(tab, 0.3, 1.0, -1.0, m.clone(), cu(w), tau.clone(), cu(E), cu(B), seed=3, step=99)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for step in range(6):  # several emissions per particle and pass
            r, e = radiation.monte_carlo(tab, 0.3, 1.0, -1.0, m, cu(w), tau, cu(E), cu(B), seed=3, step=step)
            tot += r
            nem += e
        e1.record()
        torch.cuda.synchronize()
        times[name] = e0.elapsed_time(e1)
        res[name] = (tot, nem, m.cpu().numpy())
        # no optical depth left at a tiny positive residual: such a particle would never emit again
        tv = tau.cpu().numpy()
        assert not np.any((tv > 0) & (tv < 1e-38)), name
    (t64, n64, m64), (t32, n32, m32) = res["fp64"], res["fp32"]
    assert abs(n32 - n64) <= 0.002 * n64, (n32, n64)
    assert abs(t32 - t64) <= 0.005 * t64, (t32, t64)
    dp = np.abs(m32 - m64).max(axis=0) / np.abs(m64).max(axis=0)
    assert np.mean(dp < 1e-4) > 0.95, np.mean(dp < 1e-4)
    g64 = np.sqrt(1 + (m64 ** 2).sum(axis=0))
    g32 = np.sqrt(1 + (m32 ** 2).sum(axis=0))
    h64, edges = np.histogram(g64, bins=40)
    h32, _ = np.histogram(g32, bins=edges)
    assert np.abs(h32 - h64).sum() <= 0.02 * n
    assert times["fp32"] < times["fp64"], times
    print(f"\nMonte Carlo 6 passes over {n}: fp64 {times['fp64']:.2f} ms, fp32 math {times['fp32']:.2f} ms")
    T32.close()


def test_mlp_gradients_match_cpu_oracle(rad):
    radiation, _, _ = rad
    from oracle import mlp as M
    net = radiation.PhotonChiMLP(hidden=64, seed=3)
    p = net.params().astype(np.float64)
    rng = np.random.default_rng(5)
    X = rng.uniform(-1, 1, (512, 2))
    Y = rng.normal(0, 1, 512)
    g_gpu, l_gpu = net.gradients(X, Y)
    g_ref, l_ref = M.gradients(p, 64, X.astype(np.float32).astype(np.float64), Y.astype(np.float32).astype(np.float64))
    assert abs(l_gpu - l_ref) <= 1e-5 * l_ref
    assert rel_err(g_gpu, g_ref) <= 2e-5
    fd = M.fd_gradients(p, 64, X, Y, idx=[0, 200, 1000, 3000, net.nparams - 1])
    for k, v in fd.items():
        assert abs(g_ref[k] - v) <= 1e-6 * max(1.0, abs(v))
    net.close()


def test_trained_mlp_with_table_fallback(rad):
    radiation, T, _ = rad
    net = radiation.PhotonChiMLP(hidden=64, seed=1)
    l0 = net.train(T, steps=1, batch=4096)
    l1 = net.train(T, steps=3000, batch=8192, lr=2e-3)
    assert l1 < 0.05 * l0
    err, n_masked = net.validate(T, tol=0.05)
    assert n_masked < err.size  # the network is used somewhere
    # Monte-Carlo with the network (table where masked) vs table only: same draws
    n = 100000
    mom, E, B, w = beam(n, 2)
    res = {}
    for name, m in (("table", None), ("mlp", net)):
        mm = cu(mom)
        tau = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
        tot, nem = 0.0, 0
        for step in range(4):
            r, e = radiation.monte_carlo(T, 0.1, 1.0, -1.0, mm, cu(w), tau, cu(E), cu(B), seed=5, step=step, mlp=m)
            tot += r; nem += e
        g = torch.sqrt(1 + (mm ** 2).sum(0)).cpu().numpy()
        res[name] = (tot, nem, g)
    (t_tab, n_tab, g_tab), (t_mlp, n_mlp, g_mlp) = res["table"], res["mlp"]
    assert abs(n_mlp - n_tab) <= 0.05 * n_tab
    assert abs(t_mlp - t_tab) / t_tab < 0.05  # mean energy loss within 5 %
    h_tab, edges = np.histogram(np.log10(g_tab), bins=40)
    h_mlp, _ = np.histogram(np.log10(g_mlp), bins=edges)
    assert np.abs(h_mlp - h_tab).sum() / h_tab.sum() < 0.1  # final energy spectrum
    net.close()


def test_what_the_trained_network_gains_over_the_table(rad):
    """The learned inverse CDF -- the 3-layer, 64-wide network of the radiation
    workload -- against the table it was trained on, on this GPU.

    Gain 1, memory: the network's FP32 parameters are a small fraction of the table's
    FP64 entries (and fit in a block's shared memory).  Gain 2, speed: batched over 4M
    samples, the network's 64 x 64 layer runs on the tensor cores (mma.sync, FP16
    operands, FP32 accumulation) and the whole network evaluates them several times
    faster than the table, which needs two binary searches and FP64 log/exp
    interpolation.  The tensor-core outputs stay within 0.01 decades of the same network
    on the FP32 cores (a fifth of the validation tolerance).  Price, accuracy: the network passes the 0.05-decade validation
    on a third or more of the (chi, xi) bins (the table serves the rest); its median
    deviation from the table over all samples, masked bins included, is under 8 %; the
    spectrum of emitted photon chi it samples (log-binned) and the mean photon chi (the
    mean energy an emission takes) are compared with the table's.  Training: Adam with
    a step-down learning rate, on the GPU."""
    radiation, T, _ = rad
    net = radiation.PhotonChiMLP(hidden=64, seed=3)
    for steps, lr in ((4000, 2e-3), (6000, 1e-3), (6000, 3e-4), (6000, 1e-4)):
        net.train(T, steps=steps, batch=8192, lr=lr)
    err, n_masked = net.validate(T, tol=0.05)
    table_bytes = T.nbytes
    net_bytes = net.nparams * 4
    assert net_bytes * 25 < table_bytes, (net_bytes, table_bytes)  # 17,668 B against 528,384 B
    n = 1 << 22
    rng = np.random.default_rng(11)
    chi = cu(10.0 ** rng.uniform(-1.0, 1.0, n))
    xi = cu(rng.uniform(0.0, 1.0, n))
    times = {}
    for name, fn in (("table", T.photon_chi), ("mlp", net.photon_chi),
                     ("mlp_fp32_cores", lambda c, x: net.photon_chi(c, x, tensor_cores=False))):
        fn(chi, xi)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(10):
            fn(chi, xi)
        e1.record()
        torch.cuda.synchronize()
        times[name] = e0.elapsed_time(e1) / 10
    ref = T.photon_chi(chi, xi)
    got = net.photon_chi(chi, xi)
    got32 = net.photon_chi(chi, xi, tensor_cores=False)
    tc_dev = torch.abs(torch.log10(got) - torch.log10(got32)).max().item()
    assert tc_dev < 0.01, tc_dev  # a fifth of the validation tolerance
    used = err.size - n_masked
    assert used * 3 >= err.size, (used, err.size)
    rel = (torch.abs(got - ref) / torch.abs(ref)).median().item()
    assert rel < 0.08, rel
    assert times["mlp"] * 2 <= times["table"], times
    # the emitted photon chi: spectrum (40 log bins) and mean, network against table
    lg, lr_ = torch.log10(got).cpu().numpy(), torch.log10(ref).cpu().numpy()
    h_ref, edges = np.histogram(lr_, bins=40)
    h_got, _ = np.histogram(lg, bins=edges)
    spec_dev = np.abs(h_got - h_ref).sum() / h_ref.sum()
    mean_dev = (got.mean() / ref.mean()).item() - 1.0
    assert spec_dev < 0.1, spec_dev
    assert abs(mean_dev) < 0.05, mean_dev
    print(f"\nMLP inverse CDF (64 wide): {net_bytes} B vs table {table_bytes} B; 4M samples: mlp tensor cores "
          f"{times['mlp']:.3f} ms, mlp FP32 cores {times['mlp_fp32_cores']:.3f} ms, table {times['table']:.3f} ms; "
          f"median rel dev {rel:.4f}; photon-chi spectrum L1 dev {spec_dev:.4f}, mean photon chi dev {mean_dev:+.4f}; "
          f"tensor cores vs FP32 cores {tc_dev:.2e} decades; network used on {used}/{err.size} bins")
    net.close()


def test_resident_radiation_matches_the_operator_loop(rad):
    """Radiation inside the resident 2D mixed step against the drop-in operator loop
    (FP64 interpolate, Monte Carlo, push, deposit, Maxwell) on the same electrons in the
    same uniform crossed fields (E_y = B_z = 50, electrons at gamma 1000 moving towards
    -x: chi about 0.25).  Different random streams (the resident pass keys them on the
    buffer slot): emissions and radiated energy agree to 2 %, and the tallies of a run
    whose fields make chi zero are zero with the momenta untouched by radiation."""
    radiation, _, _ = rad
    from smilei_gb300 import operators as O, simulation
    g = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "radiation.npz"))
    f_dn, f_cl, inv_es = radiation.normalised_factors(2.0 * np.pi * 299792458.0 / 1e-6)
    T32 = radiation.RadiationTables(g["integfochi"], g["integfochi_min"], g["integfochi_max"], g["xi_table"],
                                    g["xi_min"], g["xi_max"], g["xi_axis1_min"], f_dn, f_cl, inv_es)
    T32.set_fp32_math(True)
    n_cells, cl, dt, steps = [32, 32], [0.5, 0.5], 0.3, 8
    rng = np.random.default_rng(21)
    n = 200000
    L = [n_cells[0] * cl[0], n_cells[1] * cl[1]]
    pos = np.stack([rng.uniform(0, L[0], n), rng.uniform(0, L[1], n)])
    mom = np.stack([np.full(n, -1000.0), rng.normal(0, 1, n), np.zeros(n)])
    w = np.full(n, 1e-9)  # test particles: their current does not disturb the fields

    def uniform_fields(E0):
        from smilei_gb300 import synthetic
        st = synthetic.STAGGER
        f = {}
        for k in ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Bx_m", "By_m", "Bz_m", "Jx", "Jy", "Jz"]:
            f[k] = np.zeros(tuple(n_cells[d] + 5 + st[k.replace("_m", "")][d] for d in range(2)))
        for k in ("Ey", "Bz", "Bz_m"):
            f[k][:] = E0
        return f

    def resident(E0):
        sim = simulation.Simulation(n_cells, cl, dt, form="mixed")
        for k, a in uniform_fields(E0).items():
            sim.set_field(k, a)
        sim.add_species(1.0, -1.0, "vay", pos, mom, w)
        sim.set_species_radiation(0, T32, None, seed=5)
        sim.step(steps)
        r, e = sim.radiation_stats(0)
        p, m, _ = sim.get_species(0)
        sim.close()
        return r, e, m

    def operators(E0):
        geom = O.PatchGeometry(n_cells, cl)
        em = O.ElectroMagn(geom)
        for k, a in uniform_fields(E0).items():
            name = k + "_" if not k.endswith("_m") else k
            if hasattr(em, name):
                getattr(em, name).copy_(torch.as_tensor(a, device="cuda"))
        part = O.Particles(cu(pos), cu(mom), cu(w), torch.full((n,), -1, device="cuda"))
        smpi = O.SmileiMPI(2, n)
        tau = cu(np.full(n, -1.0))
        interp, push = O.Interpolator2D2Order(geom), O.PusherVay(dt, 1.0, 2)
        tot, nem = 0.0, 0
        for it in range(steps):
            interp.fieldsWrapper(em, part, smpi)
            r, e = radiation.monte_carlo(T32, dt, 1.0, -1.0, part.momentum, part.weight, tau, smpi.dynamics_Epart,
                                         smpi.dynamics_Bpart, seed=5, step=it)
            tot += r
            nem += e
            push(part, smpi)
            # periodic wrap (the operators act on one patch)
            for d in range(2):
                part.position[d] = torch.remainder(part.position[d], L[d])
        return tot, nem

    r_res, e_res, _ = resident(50.0)
    r_op, e_op = operators(50.0)
    assert e_op > 100000
    assert abs(e_res - e_op) <= 0.02 * e_op, (e_res, e_op)
    assert abs(r_res - r_op) <= 0.02 * r_op, (r_res, r_op)
    r0, e0, m0 = resident(0.0)
    assert r0 == 0.0 and e0 == 0
    assert np.allclose(np.sort(m0[0]), np.sort(mom[0]), rtol=1e-6)
    T32.close()


def test_resident_photons_carry_the_emitted_energy(rad):
    """Macro-photons of the resident step (sg_sim_set_species_photons) in a uniform
    magnetic field (B_z = 50, no E: the push changes no particle energy, so only the
    radiation does): over one step the electrons' kinetic energy falls by the radiated
    tally plus the photons' energy (sum w_ph |p_ph|); every photon carries w / sampling,
    tau = -1, a positive chi and at least the threshold energy, and sits in the box.  A
    second step moves each photon of the first by dt p / |p| (wrapped) and appends the
    new ones after them."""
    radiation, _, _ = rad
    from smilei_gb300 import simulation, synthetic
    g = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "radiation.npz"))
    f_dn, f_cl, inv_es = radiation.normalised_factors(2.0 * np.pi * 299792458.0 / 1e-6)
    T32 = radiation.RadiationTables(g["integfochi"], g["integfochi_min"], g["integfochi_max"], g["xi_table"],
                                    g["xi_min"], g["xi_max"], g["xi_axis1_min"], f_dn, f_cl, inv_es)
    T32.set_fp32_math(True)
    n_cells, cl, dt = [32, 32], [0.5, 0.5], 0.3
    L = np.array([n_cells[0] * cl[0], n_cells[1] * cl[1]])
    rng = np.random.default_rng(31)
    n = 200000
    pos = np.stack([rng.uniform(0, L[0], n), rng.uniform(0, L[1], n)])
    mom = np.stack([np.full(n, -1000.0), rng.normal(0, 1, n), np.zeros(n)])
    w = np.full(n, 1e-9)
    sim = simulation.Simulation(n_cells, cl, dt, form="mixed")
    st = synthetic.STAGGER
    for k in ("Bz", "Bz_m"):
        sim.set_field(k, np.full(tuple(n_cells[d] + 5 + st["Bz"][d] for d in range(2)), 50.0))
    sim.add_species(1.0, -1.0, "boris", pos, mom, w)  # Boris keeps |p| in a pure magnetic field
    # a photon store needs a radiating species; reading one needs a store
    with pytest.raises(RuntimeError):
        sim.set_species_photons(0, sampling=2, gamma_threshold=20.0, capacity=1000)
    with pytest.raises(RuntimeError):
        sim.get_photons(0)
    sim.set_species_radiation(0, T32, None, seed=11)
    sampling, threshold = 2, 20.0
    sim.set_species_photons(0, sampling=sampling, gamma_threshold=threshold, max_emissions=3, capacity=2_000_000)
    uk0 = sim.energy()[0]
    sim.step(1)
    uk1 = sim.energy()[0]
    rad_e, nem = sim.radiation_stats(0)
    count1, ph1 = sim.get_photons(0)
    assert nem > 10000 and 0 < count1 <= 2_000_000 and count1 % sampling == 0
    e_ph = float(np.sum(ph1["weight"] * np.sqrt((ph1["mom"] ** 2).sum(0))))
    assert e_ph > 0.5 * rad_e  # most of the emitted energy goes into photons above the threshold
    assert abs((uk0 - uk1) - (rad_e + e_ph)) <= 1e-4 * (uk0 - uk1), (uk0 - uk1, rad_e, e_ph)
    assert np.allclose(ph1["weight"], 1e-9 / sampling, rtol=1e-6)
    assert np.all(ph1["tau"] == -1.0) and np.all(ph1["chi"] > 0.0)
    assert np.all(np.sqrt((ph1["mom"] ** 2).sum(0)) >= threshold * (1 - 1e-6))
    assert np.all((ph1["pos"] >= 0.0) & (ph1["pos"] < L[:, None]))
    sim.step(1)
    count2, ph2 = sim.get_photons(0)
    assert count2 > count1
    p = ph1["mom"]
    moved = ph1["pos"] + dt * p[:2] / np.sqrt((p ** 2).sum(0))
    moved = np.where(moved >= L[:, None], moved - L[:, None], np.where(moved < 0.0, moved + L[:, None], moved))
    assert np.allclose(ph2["pos"][:, :count1], moved, rtol=0, atol=1e-12)
    assert np.array_equal(ph2["mom"][:, :count1], ph1["mom"])
    sim.close()
    T32.close()
