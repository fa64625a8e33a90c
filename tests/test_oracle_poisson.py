"""The CPU Poisson oracle solves Laplacian(phi) = -rho and yields div E = rho."""
import numpy as np

import oracle.poisson as P


def test_poisson_oracle_converges_and_satisfies_gauss():
    rng = np.random.default_rng(0)
    rho = rng.normal(size=(12, 10, 8))
    cl = [0.1, 0.12, 0.09]
    phi, E, it, ctrl = P.solve_poisson(rho, cl, max_error=1e-26)
    assert ctrl <= 1e-26 and it < 500
    assert P.charge_residual(E, rho, cl) < 1e-11
    for e in E:
        assert abs(e.mean()) < 1e-14


def test_poisson_oracle_reference_tolerance_stops_early():
    rng = np.random.default_rng(1)
    rho = rng.normal(size=(16, 16))
    _, _, it14, c14 = P.solve_poisson(rho, [0.1, 0.1])
    _, _, it26, c26 = P.solve_poisson(rho, [0.1, 0.1], max_error=1e-26)
    assert c14 <= 1e-14 and it14 < it26
