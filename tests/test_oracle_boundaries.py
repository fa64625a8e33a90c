"""The C oracle's open boundaries against the reference's own code (CPU).

tests/golden/boundaries.npz holds the reference's ElectroMagnBC2D_SM::apply,
compiled from the reference tree, on random 2D fields: every side, with and
without boundary tangent ends, and on xmin with Gaussian lasers whose space
envelope and phase come from the reference's own LaserGaussian2D
(pyprofiles.py) and whose time envelope is the compiled tgaussian.  The
oracle (bc_oracle.c) restates both the boundary and the laser; they must agree
to rounding (1e-13 of the largest field value).
"""
import numpy as np
import pytest

from conftest import rel_err

FIELDS_EB = ["Ex", "Ey", "Ez", "Bx", "By", "Bz"]


@pytest.fixture(scope="module")
def golden_bc():
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "boundaries.npz")
    z = np.load(path)
    cases = {}
    for k in z.files:
        c, name = k.split("/", 1)
        cases.setdefault(c, {})[name] = z[k]
    return cases


def laser_from_case(g):
    return dict(a0=float(g["cfg_a0"]), omega=float(g["cfg_omega"]), waist=float(g["cfg_waist"]),
                focus_x=float(g["cfg_focus"][0]), focus_y=float(g["cfg_focus"][1]),
                polarization_phi=float(g["cfg_polarization_phi"]), ellipticity=float(g["cfg_ellipticity"]),
                phase_offset=0.0, t_start=0.0, t_duration=float(g["t_duration"]), t_center=float(g["cfg_t_center"]),
                t_fwhm=float(g["cfg_t_fwhm"]), t_order=2.0)


def test_silver_mueller_and_laser_match_reference(golden_bc, cpu_oracle):
    assert len(golden_bc) == 14
    for name, g in golden_bc.items():
        F = [g[k + "_in"].copy() for k in FIELDS_EB]
        n_prim = [int(v) for v in g["n_prim"]]
        b1 = b2 = None
        if "laser_sp1" in g:
            L = laser_from_case(g)
            t = float(g["time_dual"])
            os_ = 2
            yp = (np.arange(n_prim[1]) - os_) * g["cell_length"][1]
            yd = (np.arange(n_prim[1] + 1) - 0.5 - os_) * g["cell_length"][1]
            b1 = cpu_oracle.laser_gaussian2d(L, yp, 0, t)
            b2 = cpu_oracle.laser_gaussian2d(L, yd, 1, t)
            assert np.abs(b1).max() + np.abs(b2).max() > 0.0, name  # the laser is on at these times
        cpu_oracle.sm_apply_2d(int(g["side"]), n_prim, list(g["cell_length"]), float(g["dt"]), F, b1, b2,
                               int(g["tmin"]), int(g["tmax"]))
        for k, a in zip(FIELDS_EB, F):
            assert rel_err(a, g[k]) <= 1e-13, (name, k, rel_err(a, g[k]))
        # the boundary changed something (the case is not vacuous)
        assert any(rel_err(F[i], g[k + "_in"]) > 1e-3 for i, k in enumerate(FIELDS_EB[3:], start=3)), name
