"""Pins the radiation oracle (oracle/rad_oracle.c) to the reference's own table functions.

tests/golden/radiation.npz holds the reference's default tables
(RadiationTablesDefault::setDefault) and the outputs of its compiled
computePhotonProductionYield and computeRandomPhotonChiWithInterpolation on
seeded (chi, xi, gamma) samples spanning and exceeding the table range;
tests/golden/monte_carlo.npz holds inputs and outputs of its compiled
RadiationMonteCarlo::operator() (tests/golden/make_golden.py case_monte_carlo).
"""
import os

import numpy as np
import pytest

import oracle
from conftest import rel_err


def test_photon_chi_matches_reference(golden_rad):
    t = oracle.RadTables.from_golden(golden_rad)
    got = oracle.rad_photon_chi(t, golden_rad["chi"], golden_rad["xi"])
    assert np.max(np.abs(got / golden_rad["photon_chi"] - 1.0)) <= 1e-14


def test_production_yield_matches_reference(golden_rad):
    t = oracle.RadTables.from_golden(golden_rad, factor_dNph_dt=float(golden_rad["factor"]))
    got = oracle.rad_yield(t, golden_rad["chi"], golden_rad["gamma"])
    assert rel_err(got, golden_rad["yield_"]) <= 1e-15


def test_monte_carlo_conserves_energy_bookkeeping(golden_rad):
    """gamma lost by the particles equals the tallied radiated energy (unit weights)."""
    t = oracle.RadTables.from_golden(golden_rad, factor_dNph_dt=5e3, factor_classical=2e-3,
                                     inv_norm_E_schwinger=2e-6)
    rng = np.random.default_rng(3)
    n = 2000
    mom = np.ascontiguousarray(np.stack([rng.normal(-2000, 50, n), rng.normal(0, 5, n), rng.normal(0, 5, n)]))
    E = rng.normal(0, 50, (3, n)); B = rng.normal(0, 50, (3, n))
    w = np.ones(n)
    tau = np.full(n, -1.0)
    g0 = np.sqrt(1 + (mom ** 2).sum(0))
    rad, nem, chi = oracle.rad_monte_carlo(t, 0.05, 1.0, -1.0, mom, w, tau, E, B, seed=11)
    g1 = np.sqrt(1 + (mom ** 2).sum(0))
    assert nem > 0
    assert abs(np.sum(g0 - g1) - rad) <= 1e-9 * rad
    assert chi.max() > 0.01


@pytest.fixture(scope="module")
def golden_mc():
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "monte_carlo.npz"))
    return {k: z[k] for k in z.files}


def mc_tables(golden_rad, g):
    return oracle.RadTables.from_golden(golden_rad, factor_dNph_dt=float(g["f_factor_dNph_dt"]),
                                        factor_classical=float(g["f_factor_classical"]),
                                        inv_norm_E_schwinger=float(g["f_inv_norm_E_schwinger"]),
                                        min_chi_continuous=float(g["f_min_chi_continuous"]),
                                        min_chi_discontinuous=float(g["f_min_chi_discontinuous"]))


def test_monte_carlo_pass_matches_reference_operator(golden_rad, golden_mc):
    """tests/golden/monte_carlo.npz: the reference's RadiationMonteCarlo::operator() with each
    particle drawing from Random(its stream's initial state).  The oracle's pass draws the same
    numbers, so momenta, optical depths and the final chi agree to rounding (bit for bit where
    both are built with the same compiler), across discontinuous emissions, continuous loss,
    slow particles (gamma < 1.1) and particles below the continuous threshold."""
    g = golden_mc
    t = mc_tables(golden_rad, g)
    mom, tau = np.ascontiguousarray(g["mom"].copy()), g["tau"].copy()
    rad, nem, chi = oracle.rad_monte_carlo(t, float(g["dt"]), float(g["mass"]), float(g["charge"]), mom, g["weight"],
                                           tau, g["E"], g["B"], seed=int(g["seed"]), first_id=int(g["first_id"]),
                                           step=int(g["step"]))
    assert nem > 100
    # every branch of the pass is exercised
    changed = np.abs(mom - g["mom"]).max(0) > 0
    assert changed.sum() > 300 and (~changed).sum() > 100
    assert rel_err(mom, g["rad_mom"]) <= 1e-13
    assert np.max(np.abs(tau - g["rad_tau"])) <= 1e-12
    assert rel_err(chi, g["rad_chi"]) <= 1e-13
    assert abs(rad - float(g["rad_radiated"])) <= 1e-13 * abs(float(g["rad_radiated"]))


def test_monte_carlo_photons_match_reference_operator(golden_rad, golden_mc):
    """The same pass with a photon species (sampling 2, threshold 50, at most 3 photon groups
    per particle): photons in the reference's creation order."""
    g = golden_mc
    t = mc_tables(golden_rad, g)
    mom, tau = np.ascontiguousarray(g["mom"].copy()), g["tau"].copy()
    rad, nem, chi, ph = oracle.rad_monte_carlo_photons(
        t, float(g["dt"]), float(g["mass"]), float(g["charge"]), g["pos"], mom, g["weight"], tau, g["E"], g["B"],
        seed=int(g["seed"]), first_id=int(g["first_id"]), step=int(g["step"]), sampling=int(g["sampling"]),
        threshold=float(g["threshold"]), max_emissions=int(g["max_emissions"]))
    assert ph["weight"].size == g["ph_photon_weight"].size > 100
    for k in ("pos", "mom", "weight", "chi", "tau"):
        assert rel_err(ph[k], g["ph_photon_" + k]) <= 1e-13, k
    assert rel_err(mom, g["ph_mom"]) <= 1e-13
    assert rel_err(chi, g["ph_chi"]) <= 1e-13
    assert abs(rad - float(g["ph_radiated"])) <= 1e-13 * abs(float(g["ph_radiated"]))
