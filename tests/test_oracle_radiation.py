"""Pins the radiation oracle (oracle/rad_oracle.c) to the reference's own table functions.

tests/golden/radiation.npz holds the reference's default tables
(RadiationTablesDefault::setDefault) and the outputs of its compiled
computePhotonProductionYield and computeRandomPhotonChiWithInterpolation on
seeded (chi, xi, gamma) samples spanning and exceeding the table range.
"""
import numpy as np

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
