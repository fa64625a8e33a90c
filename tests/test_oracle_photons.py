"""The oracle's macro-photon creation and photon pusher (rad_oracle.c), on CPU.

RadiationMonteCarlo.cpp:425-545 creates `sampling` photons per emission whose
photon gamma reaches the threshold, at most max_emissions groups per particle and
pass, with momentum photon_gamma p / |p| after the recoil and weight w / sampling;
the recoil is along p, so the macro-particles' total momentum sum w p is conserved
by every emission that makes photons.  These follow from the reference's formulas;
the Monte-Carlo draws are this repository's own stream (parity unpinned against
the reference's generator, as for the pass without photons).
"""
import numpy as np
import pytest

import oracle


@pytest.fixture(scope="module")
def tables(golden_rad):
    from smilei_gb300.radiation import normalised_factors
    f_dn, f_cl, inv_es = normalised_factors(2.0 * np.pi * 299792458.0 / 1e-6)  # lambda_r = 1 um
    return oracle.RadTables.from_golden(golden_rad, factor_dNph_dt=f_dn, factor_classical=f_cl,
                                        inv_norm_E_schwinger=inv_es)


def beam(n, seed):
    rng = np.random.default_rng(seed)
    mom = np.ascontiguousarray(np.stack([rng.normal(-2000, 40, n), rng.normal(0, 4, n), rng.normal(0, 4, n)]))
    pos = np.ascontiguousarray(np.stack([rng.uniform(0, 10, n), rng.uniform(0, 5, n)]))
    return pos, mom, rng.normal(0, 60, (3, n)), rng.normal(0, 60, (3, n)), rng.uniform(0.5, 1.5, n)


def test_photons_conserve_momentum_and_follow_the_rules(tables):
    n = 3000
    pos, mom, E, B, w = beam(n, 2)
    tau = np.full(n, -1.0)
    m0 = mom.copy()
    thr, samp, mx = 50.0, 3, 2
    rad, nem, chi, ph = oracle.rad_monte_carlo_photons(tables, 0.1, 1.0, -1.0, pos, mom, w, tau, E, B, seed=7,
                                                       sampling=samp, threshold=thr, max_emissions=mx)
    k = ph["weight"].size
    assert nem > 100 and k > 0 and k % samp == 0
    # photon energies reach the threshold; groups of `sampling` identical photons
    g = np.sqrt((ph["mom"] ** 2).sum(axis=0))
    assert g.min() >= thr
    groups = ph["mom"].reshape(3, -1, samp)
    assert np.array_equal(groups, np.repeat(groups[:, :, :1], samp, axis=2))
    assert np.all(ph["tau"] == -1.0) and np.all(ph["chi"] > 0)
    # photons sit at their particle's position, weight w / sampling: match positions back
    key = {tuple(np.round(pos[:, i], 12)): i for i in range(n)}
    src = np.array([key[tuple(np.round(ph["pos"][:, j], 12))] for j in range(k)])
    np.testing.assert_allclose(ph["weight"], w[src] / samp, rtol=1e-15)
    # at most max_emissions groups per particle
    assert np.bincount(src, minlength=n).max() <= mx * samp
    # photon momentum along the particle's (recoiled) momentum
    d = mom[:, src] / np.sqrt((mom[:, src] ** 2).sum(axis=0))
    np.testing.assert_allclose(ph["mom"] / g, d, atol=1e-12)


def test_momentum_conserved_when_every_emission_makes_photons(tables):
    n = 2000
    pos, mom, E, B, w = beam(n, 3)
    tau = np.full(n, -1.0)
    before = (w * mom).sum(axis=1)
    rad, nem, chi, ph = oracle.rad_monte_carlo_photons(tables, 0.1, 1.0, -1.0, pos, mom, w, tau, E, B, seed=8,
                                                       sampling=2, threshold=0.0, max_emissions=1000)
    assert rad == 0.0 and ph["weight"].size == 2 * nem  # no emission tallied, every one made photons
    after = (w * mom).sum(axis=1) + (ph["weight"] * ph["mom"]).sum(axis=1)
    np.testing.assert_allclose(after, before, rtol=1e-12)


def test_photon_push_is_rectilinear():
    rng = np.random.default_rng(4)
    pos = rng.uniform(0, 1, (3, 100))
    mom = rng.normal(0, 10, (3, 100))
    p0 = pos.copy()
    inv = oracle.push_photons(0.3, pos, mom)
    np.testing.assert_allclose(inv, 1.0 / np.sqrt((mom ** 2).sum(axis=0)), rtol=1e-15)
    np.testing.assert_allclose(np.sqrt(((pos - p0) ** 2).sum(axis=0)), 0.3, rtol=1e-14)
