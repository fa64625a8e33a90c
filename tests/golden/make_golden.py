"""Generate the golden fixtures in tests/golden from the reference's own operators.

Run where the reference tree is present:

    python tests/golden/make_golden.py [reference_src_dir]

(default: $SMILEI_REFERENCE_SRC, else ../reference/src beside the checkout).

It compiles the reference's operator sources (oracle/build_ref.sh), feeds them
seeded inputs, and stores inputs and outputs as .npz files next to this script.
The tests compare the C oracle (oracle/pic_oracle.c) against these files on any
machine, and the GPU kernels against the oracle; nothing at test time reads the
reference tree.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

REF_SRC = sys.argv[1] if len(sys.argv) > 1 else oracle.reference_src()

FIELDS_EB = ["Ex", "Ey", "Ez", "Bx", "By", "Bz"]


def geometry(ndim, cells, patch_start, oversize=2):
    n_prim = [cells[d] + 1 + 2 * oversize for d in range(ndim)]
    domain_begin = [patch_start[d] - oversize for d in range(ndim)]
    return n_prim, domain_begin


def random_fields(rng, ndim, n_prim, names, scale=1.0):
    return {k: rng.normal(0.0, scale, oracle.field_shape(ndim, n_prim, k)) for k in names}


def random_positions(rng, ndim, cells, patch_start, cell_length, n):
    """Uniform positions inside the patch, plus a few exactly on half-cell points (rounding edge)."""
    pos = np.zeros((ndim, n))
    for d in range(ndim):
        lo = patch_start[d] * cell_length[d]
        pos[d] = lo + rng.uniform(0.0, cells[d], n) * cell_length[d]
    # Put some particles exactly on half-integer node coordinates, where round()'s
    # half-away-from-zero rule matters.
    k = max(1, n // 16)
    for d in range(ndim):
        idx = rng.integers(0, cells[d], k)
        pos[d, :k] = (patch_start[d] + idx + 0.5) * cell_length[d]
    return pos


def case_interpolate(ref, rng, ndim):
    cells = [6, 5, 4][:ndim]
    start = [3, -1, 2][:ndim] if ndim == 3 else [4, 2]
    cell_length = [0.1, 0.15, 0.2][:ndim]
    n_prim, db = geometry(ndim, cells, start)
    F = random_fields(rng, ndim, n_prim, FIELDS_EB)
    pos = random_positions(rng, ndim, cells, start, cell_length, 600)
    E, B, iold, delta = ref.interpolate(ndim, n_prim, db, cell_length, [F[k] for k in FIELDS_EB], pos)
    return dict(ndim=ndim, n_prim=n_prim, domain_begin=db, cell_length=cell_length, pos=pos,
                **{k: F[k] for k in FIELDS_EB}, E=E, B=B, iold=iold, delta=delta)


def case_push(ref, rng, ndim, kind, mass, field_scale):
    n = 500
    pos = rng.uniform(0.0, 2.0, (ndim, n))
    mom = rng.normal(0.0, 1.0, (3, n)) * np.where(rng.uniform(size=n) < 0.3, 30.0, 0.2)
    charge = rng.choice(np.array([-2, -1, 1, 2], dtype=np.int16), n)
    E = rng.normal(0.0, field_scale, (3, n))
    B = rng.normal(0.0, field_scale, (3, n))
    dt = 0.05
    pos1, mom1, invgf = ref.push(kind, ndim, dt, mass, pos, mom, charge, E, B)
    return dict(kind=kind, ndim=ndim, dt=dt, mass=mass, pos=pos, mom=mom, charge=charge, E=E, B=B,
                pos_out=pos1, mom_out=mom1, invgf=invgf)


def case_project(ref, rng, ndim, mode):
    cells = [7, 6, 5][:ndim]
    start = [2, 4, -3][:ndim]
    cell_length = [0.1, 0.12, 0.09][:ndim]
    dt = 0.05
    n_prim, db = geometry(ndim, cells, start)
    n = 400
    # Keep old positions one cell away from the patch edges so the 5-point stencil stays inside.
    pos_old = np.zeros((ndim, n))
    for d in range(ndim):
        pos_old[d] = (start[d] + 1 + rng.uniform(0.0, cells[d] - 2, n)) * cell_length[d]
    zeros = random_fields(rng, ndim, n_prim, FIELDS_EB, 0.0)
    _, _, iold, delta = ref.interpolate(ndim, n_prim, db, cell_length, [zeros[k] for k in FIELDS_EB], pos_old)
    disp = rng.uniform(-0.95, 0.95, (ndim, n)) * np.array(cell_length)[:, None]
    pos = pos_old + disp
    mom = rng.normal(0.0, 0.5, (3, n))
    invgf = 1.0 / np.sqrt(1.0 + (mom ** 2).sum(0))
    weight = rng.uniform(0.5, 1.5, n)
    charge = rng.choice(np.array([-1, 1, 2], dtype=np.int16), n)
    J0 = random_fields(rng, ndim, n_prim, ["Jx", "Jy", "Jz", "rho"], 0.1)
    Jin = [J0[k].copy() for k in ["Jx", "Jy", "Jz", "rho"]]
    Jout = ref.project(mode, ndim, n_prim, db, cell_length, dt, pos, mom, weight, charge, invgf, iold, delta,
                       [a.copy() for a in Jin])
    return dict(mode=mode, ndim=ndim, n_prim=n_prim, domain_begin=db, cell_length=cell_length, dt=dt, pos=pos,
                mom=mom, weight=weight, charge=charge, invgf=invgf, iold=iold, delta=delta,
                Jx_in=Jin[0], Jy_in=Jin[1], Jz_in=Jin[2], rho_in=Jin[3],
                Jx=Jout[0], Jy=Jout[1], Jz=Jout[2], rho=Jout[3])


def case_maxwell(ref, rng, ndim, which):
    cells = [6, 7, 5][:ndim]
    cell_length = [0.1, 0.12, 0.08][:ndim]
    dt = 0.04
    n_prim, _ = geometry(ndim, cells, [0, 0, 0][:ndim])
    names = FIELDS_EB + ["Jx", "Jy", "Jz"]
    F = random_fields(rng, ndim, n_prim, names)
    Fin = [F[k].copy() for k in names]
    Fout = ref.maxwell(which, ndim, n_prim, cell_length, dt, [a.copy() for a in Fin])
    out = dict(which=which, ndim=ndim, n_prim=n_prim, cell_length=cell_length, dt=dt)
    for k, a, b in zip(names, Fin, Fout):
        out[k + "_in"] = a
        out[k] = b
    return out


def case_radiation(ref, rng):
    t = ref.rad_tables()
    n = 4000
    # particle chi across and beyond the table range, xi in [0, 1)
    chi = 10.0 ** rng.uniform(-4.5, 3.5, n)
    xi = rng.uniform(0.0, 1.0, n)
    xi[:50] = 0.0
    gamma = 1.0 + 10.0 ** rng.uniform(0.0, 4.0, n)
    factor = 3.7e3
    y = ref.rad_yield(chi, gamma, factor)
    pc = ref.rad_photon_chi(chi, xi)
    return dict(chi=chi, xi=xi, gamma=gamma, factor=factor, yield_=y, photon_chi=pc,
                integfochi=t["integfochi"], integfochi_min=t["integfochi_min"],
                integfochi_max=t["integfochi_max"], xi_table=t["xi"], xi_min=t["xi_min"], xi_max=t["xi_max"],
                xi_axis1_min=t["xi_axis1_min"])


MC_FACTORS = dict(factor_dNph_dt=5e3, factor_classical=2e-3, min_chi_continuous=1e-3, min_chi_discontinuous=1e-2,
                  inv_norm_E_schwinger=2e-6)


def case_monte_carlo(ref):
    """The reference's RadiationMonteCarlo::operator() on seeded particles, particle p drawing
    from Random(state p) with state p = oracle.rng_seeds(seed, first_id, step)[p], so that the
    oracle's per-particle streams are the same draws.  A third of the particles sit in strong
    fields (discontinuous emissions, several per step), a third in weak ones (continuous loss
    and no emission), a few are slow (gamma < 1.1); half start with a spent optical depth.
    Run once without and once with a photon species (sampling 2, threshold 50, at most 3
    photon groups per particle)."""
    rng = np.random.default_rng(1234)
    n = 1500
    mom = np.stack([rng.normal(-2000, 800, n), rng.normal(0, 50, n), rng.normal(0, 50, n)])
    E = rng.normal(0, 50, (3, n))
    B = rng.normal(0, 50, (3, n))
    k = n // 3
    E[:, k:2 * k] *= 0.02
    B[:, k:2 * k] *= 0.02
    mom[:, 2 * k:2 * k + 40] *= 1e-4
    w = rng.uniform(0.5, 2.0, n)
    tau = np.where(rng.uniform(size=n) < 0.5, -1.0, rng.exponential(1.0, n))
    pos = rng.uniform(0.0, 10.0, (2, n))
    seed, first_id, step, dt = 7, 100, 3, 0.05
    seeds = oracle.rng_seeds(seed, first_id, step, n)
    out = dict(mom=mom, E=E, B=B, weight=w, tau=tau, pos=pos, seed=seed, first_id=first_id, step=step, dt=dt,
               mass=1.0, charge=-1.0, sampling=2, threshold=50.0, max_emissions=3,
               **{"f_" + a: b for a, b in MC_FACTORS.items()})
    for tag, sampling in (("rad", 0), ("ph", 2)):
        m, t = np.ascontiguousarray(mom.copy()), tau.copy()
        r, chi, ph = ref.rad_monte_carlo(MC_FACTORS, dt, 1.0, -1.0, pos, m, w, t, E, B, seeds, sampling=sampling,
                                         threshold=50.0, max_emissions=3)
        out.update({f"{tag}_mom": m, f"{tag}_tau": t, f"{tag}_chi": chi, f"{tag}_radiated": r})
        if ph is not None:
            out.update({f"{tag}_photon_{a}": b for a, b in ph.items()})
    return out


def reference_laser_gaussian2d(cfg):
    """Runs the reference's own pyinit.py and pyprofiles.py (pure Python, from the reference
    tree) to build LaserGaussian2D and returns its Laser component."""
    ns = {}
    for f in ("pyinit.py", "pyprofiles.py"):
        path = os.path.join(REF_SRC, "Python", f)
        exec(compile(open(path).read(), path, "exec"), ns)
    ns["Main"](geometry="2Dcartesian", interpolation_order=2, timestep=cfg["dt"], simulation_time=cfg["t_sim"],
               cell_length=list(cfg["cell_length"]), grid_length=list(cfg["grid_length"]), number_of_patches=[1, 1])
    ns["LaserGaussian2D"](box_side="xmin", a0=cfg["a0"], omega=cfg["omega"], focus=list(cfg["focus"]),
                          waist=cfg["waist"], polarization_phi=cfg["polarization_phi"], ellipticity=cfg["ellipticity"],
                          time_envelope=ns["tgaussian"](center=cfg["t_center"], fwhm=cfg["t_fwhm"]))
    return ns["Laser"][0]


def case_silver_mueller(ref, rng, side, tmin, tmax, laser_cfg=None, time_dual=0.0):
    """One side of the reference's 2D Silver-Mueller condition on random fields, with or
    without a Gaussian laser on xmin (space and phase from the reference's Python profiles)."""
    cells, cl, dt, os_ = [9, 7], [0.1, 0.3], 0.08, 2
    n_prim = [c + 1 + 2 * os_ for c in cells]
    F = random_fields(rng, 2, n_prim, FIELDS_EB)
    out = dict(side=side, tmin=tmin, tmax=tmax, n_prim=n_prim, cell_length=cl, dt=dt, time_dual=time_dual,
               **{k + "_in": F[k].copy() for k in FIELDS_EB})
    laser = None
    if laser_cfg is not None:
        L = reference_laser_gaussian2d(dict(laser_cfg, dt=dt, cell_length=cl,
                                            grid_length=[cells[0] * cl[0], cells[1] * cl[1]]))
        te = L.time_envelope
        yp = (np.arange(n_prim[1]) - os_) * cl[1]
        yd = (np.arange(n_prim[1] + 1) - 0.5 - os_) * cl[1]
        laser = dict(lt=[te.start, te.start + te.duration, 1.0 / te.sigma, te.center, te.order], omega=L.omega,
                     sp1=np.array([L.space_envelope[0](y) for y in yp]), ph1=np.array([L.phase[0](y) for y in yp]),
                     d1=L.delay_phase[0], sp2=np.array([L.space_envelope[1](y) for y in yd]),
                     ph2=np.array([L.phase[1](y) for y in yd]), d2=L.delay_phase[1])
        out.update({"laser_" + k: np.asarray(v) for k, v in laser.items()})
        out.update({"cfg_" + k: np.asarray(v) for k, v in laser_cfg.items()})
        out["t_duration"] = te.duration
    res = ref.sm_apply_2d(side, n_prim, cl, dt, [F[k] for k in FIELDS_EB], tmin, tmax, laser, time_dual)
    out.update({k: res[i] for i, k in enumerate(FIELDS_EB)})
    return out


def boundary_cases(ref):
    rng = np.random.default_rng(20261205)
    cases = {}
    for side in range(4):
        for tmin, tmax in ((1, 1), (0, 0)):
            cases[f"sm_side{side}_t{tmin}{tmax}"] = case_silver_mueller(ref, rng, side, tmin, tmax)
    lasers = {
        "linear_focus0": dict(a0=2.0, omega=1.0, focus=[0.0, 1.05], waist=0.8, polarization_phi=0.0,
                              ellipticity=0.0, t_center=0.5, t_fwhm=0.6, t_sim=3.0),
        "elliptic_focus_inside": dict(a0=1.3, omega=2.0, focus=[0.4, 0.9], waist=0.6, polarization_phi=0.7,
                                      ellipticity=0.3, t_center=0.8, t_fwhm=0.9, t_sim=3.0),
    }
    for name, cfg in lasers.items():
        for k, t in enumerate((0.3, 0.55, 1.7)):
            cases[f"laser_{name}_{k}"] = case_silver_mueller(ref, rng, 0, 1, 1, cfg, t)
    return cases


def main():
    path = oracle.build_ref(REF_SRC)
    if path is None:
        raise SystemExit("reference tree not found; the fixtures cannot be regenerated here")
    ref = oracle.RefOps(path)
    rng = np.random.default_rng(20261204)
    cases = {}
    for ndim in (2, 3):
        cases[f"interp{ndim}d"] = case_interpolate(ref, rng, ndim)
        for kind in ("boris", "vay", "higueracary"):
            for mass, scale in ((1.0, 0.5), (1836.0, 30.0)):
                cases[f"push_{kind}_{ndim}d_m{int(mass)}"] = case_push(ref, rng, ndim, kind, mass, scale)
        for mode in (0, 1, 2):
            cases[f"project{ndim}d_mode{mode}"] = case_project(ref, rng, ndim, mode)
        for which in (0, 1):
            cases[f"maxwell{ndim}d_{'ampere' if which == 0 else 'faraday'}"] = case_maxwell(ref, rng, ndim, which)
    np.savez_compressed(os.path.join(HERE, "operators.npz"),
                        **{f"{c}/{k}": np.asarray(v) for c, d in cases.items() for k, v in d.items()})
    rad = case_radiation(ref, rng)
    np.savez_compressed(os.path.join(HERE, "radiation.npz"), **{k: np.asarray(v) for k, v in rad.items()})
    mc = case_monte_carlo(ref)
    np.savez_compressed(os.path.join(HERE, "monte_carlo.npz"), **{k: np.asarray(v) for k, v in mc.items()})
    bcases = boundary_cases(ref)
    np.savez_compressed(os.path.join(HERE, "boundaries.npz"),
                        **{f"{c}/{k}": np.asarray(v) for c, d in bcases.items() for k, v in d.items()})
    print("wrote", len(cases), "operator cases, the radiation and Monte-Carlo cases and", len(bcases), "boundary cases")


if __name__ == "__main__":
    main()
