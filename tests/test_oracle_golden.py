"""Pins the C oracle (oracle/pic_oracle.c) to the reference's own operators.

The fixtures in tests/golden/operators.npz were produced by the reference's
compiled Interpolator/Pusher/Projector/Solver classes
(tests/golden/make_golden.py).  The oracle must reproduce them to FP64
round-off: bit-exact except where the summation order of the Esirkepov
running sums differs (<= 1e-15 relative).
"""
import numpy as np
import pytest

from conftest import rel_err

TOL = 1e-15
EB = ["Ex", "Ey", "Ez", "Bx", "By", "Bz"]
JR = ["Jx", "Jy", "Jz", "rho"]


def _cases(golden, prefix):
    return sorted(k for k in golden if k.startswith(prefix))


@pytest.mark.parametrize("ndim", [2, 3])
def test_interpolate_matches_reference(golden_ops, cpu_oracle, ndim):
    g = golden_ops[f"interp{ndim}d"]
    E, B, iold, delta = cpu_oracle.interpolate(ndim, g["n_prim"], g["domain_begin"], g["cell_length"],
                                               [g[k] for k in EB], g["pos"])
    assert rel_err(E, g["E"]) <= TOL
    assert rel_err(B, g["B"]) <= TOL
    assert np.array_equal(iold, g["iold"])
    assert rel_err(delta, g["delta"]) <= TOL


def test_push_matches_reference(golden_ops, cpu_oracle):
    names = _cases(golden_ops, "push_")
    assert len(names) == 12
    for c in names:
        g = golden_ops[c]
        pos, mom, invgf = cpu_oracle.push(str(g["kind"]), int(g["ndim"]), float(g["dt"]), float(g["mass"]),
                                          g["pos"], g["mom"], g["charge"], g["E"], g["B"])
        assert rel_err(pos, g["pos_out"]) <= TOL, c
        assert rel_err(mom, g["mom_out"]) <= TOL, c
        assert rel_err(invgf, g["invgf"]) <= TOL, c


def test_project_matches_reference(golden_ops, cpu_oracle):
    names = _cases(golden_ops, "project")
    assert len(names) == 6
    for c in names:
        g = golden_ops[c]
        J = [g[k + "_in"].copy() for k in JR]
        cpu_oracle.project(int(g["mode"]), int(g["ndim"]), g["n_prim"], g["domain_begin"], g["cell_length"],
                           float(g["dt"]), g["pos"], g["mom"], g["weight"], g["charge"], g["invgf"], g["iold"],
                           g["delta"], J)
        for a, k in zip(J, JR):
            # compare the deposited increment, which is what the operator produces
            assert rel_err(a - g[k + "_in"], g[k] - g[k + "_in"]) <= 1e-15, (c, k)


def test_maxwell_matches_reference(golden_ops, cpu_oracle):
    names = ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Jx", "Jy", "Jz"]
    for c in _cases(golden_ops, "maxwell"):
        g = golden_ops[c]
        F = [g[k + "_in"].copy() for k in names]
        cpu_oracle.maxwell(int(g["which"]), int(g["ndim"]), g["n_prim"], g["cell_length"], float(g["dt"]), F)
        for a, k in zip(F, names):
            assert rel_err(a, g[k]) <= TOL, (c, k)


def test_charge_conservation_of_oracle_deposit(golden_ops, cpu_oracle):
    """Esirkepov's defining property: div J = -d rho/dt to round-off (3D, one step)."""
    g = golden_ops["project3d_mode0"]
    nd = 3
    n_prim, db, cl, dt = g["n_prim"], g["domain_begin"], g["cell_length"], float(g["dt"])
    zeros = [np.zeros(np.array(n_prim) + np.array(s)) for s in [(1, 0, 0), (0, 1, 0), (0, 0, 1), (0, 0, 0)]]
    pos_old = np.zeros_like(g["pos"])
    for d in range(nd):
        pos_old[d] = (g["iold"][d] + db[d] + g["delta"][d]) * cl[d]
    J = [z.copy() for z in zeros]
    cpu_oracle.project(0, nd, n_prim, db, cl, dt, g["pos"], g["mom"], g["weight"], g["charge"], g["invgf"],
                       g["iold"], g["delta"], J)
    rho0 = zeros[3].copy(); rho1 = zeros[3].copy()
    cpu_oracle.project(2, nd, n_prim, db, cl, dt, pos_old, g["mom"], g["weight"], g["charge"], None, None, None,
                       [None, None, None, rho0])
    cpu_oracle.project(2, nd, n_prim, db, cl, dt, g["pos"], g["mom"], g["weight"], g["charge"], None, None, None,
                       [None, None, None, rho1])
    Jx, Jy, Jz = J[:3]
    div = ((Jx[1:, :, :] - Jx[:-1, :, :]) / cl[0] + (Jy[:, 1:, :] - Jy[:, :-1, :]) / cl[1]
           + (Jz[:, :, 1:] - Jz[:, :, :-1]) / cl[2])
    drho = (rho1 - rho0) / dt
    assert rel_err(div, -drho) < 1e-12
