"""FP64 conjugate-gradient Poisson solve and charge residual -- TEST INFRASTRUCTURE ONLY.

Restates VectorPatch::solvePoisson (src/Patch/VectorPatch.cpp:1523-1620) with
the ElectroMagn3D helpers initPoisson / compute_r / compute_Ap / update_pand_r /
update_p / initE (src/ElectroMagn/ElectroMagn3D.cpp:255-560) for one periodic
domain, vectorised with numpy:

    phi = 0, r = -rho, p = r
    while r.r / n_nodes > max_error and it < max_iter:
        Ap = Laplacian(p)            (7-point, periodic)
        alpha = r.r / p.Ap;  phi += alpha p;  r -= alpha Ap
        beta = r_new.r_new / r.r;  p = r + beta p
    E_d(dual i) = (phi(i-1) - phi(i)) / dx_d, then each component's mean removed
    (the reference's "centering" of the electrostatic field).

The periodic Laplacian is singular; the plasma is neutral (or neutralised by a
uniform background), so the mean of rho is removed first.  Arrays here hold the
N^ndim physical nodes only (no ghosts).
"""
from __future__ import annotations

import numpy as np


def laplacian(p, cell_length):
    out = np.zeros_like(p)
    for d, h in enumerate(cell_length):
        out += (np.roll(p, 1, axis=d) + np.roll(p, -1, axis=d) - 2.0 * p) / (h * h)
    return out


def solve_poisson(rho, cell_length, max_error=1e-14, max_iter=50000):
    """Returns (phi, E list per dimension on the dual nodes, iterations, final ctrl)."""
    rho = np.asarray(rho, dtype=np.float64)
    rho = rho - rho.mean()
    n_nodes = rho.size
    phi = np.zeros_like(rho)
    r = -rho.copy()
    p = r.copy()
    rr = float(np.sum(r * r))
    ctrl = rr / n_nodes
    it = 0
    while ctrl > max_error and it < max_iter:
        it += 1
        Ap = laplacian(p, cell_length)
        pAp = float(np.sum(p * Ap))
        alpha = rr / pAp
        phi += alpha * p
        r -= alpha * Ap
        rnew = float(np.sum(r * r))
        p = r + (rnew / rr) * p
        rr = rnew
        ctrl = rr / n_nodes
    E = []
    for d, h in enumerate(cell_length):
        e = (np.roll(phi, 1, axis=d) - phi) / h
        E.append(e - e.mean())
    return phi, E, it, ctrl


def charge_residual(E, rho, cell_length):
    """max |div E - rho| / max |rho| on the periodic lattice (E on dual nodes, rho on primal)."""
    div = np.zeros_like(rho)
    for d, h in enumerate(cell_length):
        div += (np.roll(E[d], -1, axis=d) - E[d]) / h
    r = rho - rho.mean()
    return float(np.max(np.abs(div - r)) / max(np.max(np.abs(r)), 1e-300))
