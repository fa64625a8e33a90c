"""scalars.txt layout (CPU, with a stand-in simulation) and its values (GPU).

Layout rules of the reference's DiagnosticScalar (src/Diagnostic/
DiagnosticScalar.cpp:350-400): a numbered list of the columns, "#", then one
header line with "time" right-aligned in precision+9 characters after the "#"
and each name right-aligned in 2 + max(len(name), precision+8); each row has
the time (step * dt) in precision+10 characters and every value in scientific
notation with `precision` digits, location columns as integers.
"""
import numpy as np
import pytest

from smilei_gb300 import diagnostics as D


class FakeSim:
    ndim = 2
    n_cells = [4, 3]
    dt = 0.5
    species = [dict(name="eon", mass=1.0, charge=-1.0)]

    def species_scalars(self, s):
        return (2.0, 24.0, -2.0, 0.75)

    def field_energies(self):
        return np.array([1.0, 2.0, 0.0, 0.0, 0.0, 0.5])

    def get_field(self, name):
        a = np.zeros((9, 8))
        a[2 + 1, 2 + 2] = 3.0 if name == "Ex" else 0.0
        a[2 + 3, 2 + 0] = -4.0 if name == "Ex" else 0.0
        return a

    def rho(self):
        return np.ones((9, 8))


def test_header_and_row_layout(tmp_path):
    path = tmp_path / "scalars.txt"
    d = D.DiagScalar(FakeSim(), path=str(path), precision=10, vars=["Utot", "Ukin_eon", "ExMin", "ExMax"])
    d(0)
    d(0)  # already written: no second row
    d(2)
    lines = path.read_text().splitlines()
    assert lines[:8] == ["# 1 time", "# 2 Utot", "# 3 Ukin_eon", "# 4 ExMin", "# 5 ExMinCell", "# 6 ExMax",
                         "# 7 ExMaxCell", "#"]
    w = 2 + max(len("Utot"), 18)
    assert lines[8] == "#" + "time".rjust(19) + "Utot".rjust(w) + "Ukin_eon".rjust(w) + "ExMin".rjust(w) + \
        "ExMinCell".rjust(w) + "ExMax".rjust(w) + "ExMaxCell".rjust(w)
    row = lines[9]
    assert row[:20] == f"{0.0:.10e}".rjust(20)
    utot = 0.75 + 3.5
    assert row[20:20 + w] == f"{utot:.10e}".rjust(w)
    assert row[20 + 2 * w:20 + 3 * w] == f"{-4.0:.10e}".rjust(w)
    assert row[20 + 3 * w:20 + 4 * w] == str(3 * 3 + 0).rjust(w)  # i * N1 + j over the physical points
    assert row[20 + 5 * w:20 + 6 * w] == str(1 * 3 + 2).rjust(w)
    assert len(lines) == 11 and lines[10].startswith(f"{1.0:.10e}".rjust(20))
    cols = D.read_scalars(str(path))
    assert list(cols) == ["time", "Utot", "Ukin_eon", "ExMin", "ExMinCell", "ExMax", "ExMaxCell"]
    assert cols["time"].tolist() == [0.0, 1.0]
    assert cols["ExMaxCell"].tolist() == [5.0, 5.0]


def test_all_columns_in_reference_order():
    d = D.DiagScalar(FakeSim(), path="/dev/null")
    names = [c[0] for c in d.columns()]
    assert names[:15] == D.GENERAL
    assert names[15:20] == ["Dens_eon", "Ntot_eon", "Zavg_eon", "Ukin_eon", "Urad_eon"]
    assert names[20:26] == ["Uelm_Ex", "Uelm_Ey", "Uelm_Ez", "Uelm_Bx_m", "Uelm_By_m", "Uelm_Bz_m"]
    assert names[26:28] == ["ExMin", "ExMax"] and names[44:46] == ["RhoMin", "RhoMax"]
    assert names[46:] == ["PoyXmin", "PoyXminInst", "PoyYmin", "PoyYminInst", "PoyXmax", "PoyXmaxInst",
                          "PoyYmax", "PoyYmaxInst"]


def test_energy_balance():
    d = D.DiagScalar(FakeSim(), path="/dev/null")
    v0 = d.values(0)
    assert v0["Utot"] == pytest.approx(0.75 + 3.5) and v0["Ubal"] == 0.0 and v0["Uexp"] == v0["Utot"]
    assert v0["Zavg_eon"] == -1.0 and v0["Ntot_eon"] == 24.0


@pytest.mark.gpu
def test_scalar_values_match_numpy_on_gpu(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from smilei_gb300 import simulation, synthetic
    n_cells, cl = [16, 12, 8], [0.1, 0.1, 0.1]
    dt = 0.95 / np.sqrt(sum(1.0 / c ** 2 for c in cl))
    pos, mom, w = synthetic.thermal_plasma(n_cells, cl, 4, 0.2, 5)
    sim = simulation.Simulation(n_cells, cl, dt, form="fp64")
    sim.add_species(1.0, -1.0, "boris", pos, mom, w, name="eon")
    sim.solve_poisson()
    sim.step(3)
    d = D.DiagScalar(sim, path=str(tmp_path / "scalars.txt"))
    v = d.values(3)
    p, m, ww = sim.get_species(0)
    gam = np.sqrt(1 + (m ** 2).sum(0))
    assert v["Dens_eon"] == pytest.approx(ww.sum(), rel=1e-12)
    assert v["Ukin_eon"] == pytest.approx((ww * (gam - 1)).sum(), rel=1e-12)
    vol = np.prod(cl)
    for f in D.ENERGY_FIELDS:
        a = d._interior(sim.get_field(f))
        assert v["Uelm_" + f] == pytest.approx(0.5 * vol * (a ** 2).sum(), rel=1e-12, abs=1e-300)
    uk, ue = sim.energy()
    assert v["Ukin"] == pytest.approx(uk, rel=1e-12) and v["Uelm"] == pytest.approx(ue, rel=1e-12)
    ex = d._interior(sim.get_field("Ex"))
    assert v["ExMax"] == ex.max() and np.unravel_index(v["ExMaxCell"], ex.shape) == np.unravel_index(ex.argmax(), ex.shape)
    sim.close()


class FieldSim:
    """A stand-in simulation whose fields encode their array indices."""
    n_cells = [4, 3]

    def __init__(self):
        self.t = 0

    def get_field(self, name):
        from smilei_gb300 import synthetic
        st = synthetic.STAGGER[name.replace("_m", "")]
        shape = tuple(self.n_cells[d] + 5 + st[d] for d in range(2))
        i, j = np.indices(shape)
        return 100.0 * i + j + 1000.0 * self.t

    def window_state(self):
        return (8, 0.8, 2)


def test_field_dump_layout_and_time_average(tmp_path):
    """N + 1 points per dimension from array index oversize, whatever the staggering
    (DiagnosticFields2D.cpp:20-55,150-190); time_average T sums the T steps from each
    selected step and writes at step k*every + T - 1 (DiagnosticFields.cpp:262-292)."""
    sim = FieldSim()
    d = D.DiagFields(sim, path=str(tmp_path / "F"), every=5, fields=["Ex", "By_m", "Jz"])
    for t in range(11):
        sim.t = t
        d(t)
    got = D.read_fields(str(tmp_path / "F"))
    assert sorted(got) == [0, 5, 10]
    a = got[5]["Ex"]
    assert a.shape == (5, 4)
    assert a[0, 0] == 100.0 * 2 + 2 + 5000.0 and a[4, 3] == 100.0 * 6 + 5 + 5000.0
    assert got[5]["By_m"].shape == (5, 4) and got[10]["x_moved"] == 0.8
    d2 = D.DiagFields(sim, path=str(tmp_path / "G"), every=5, fields=["Ex"], time_average=3)
    for t in range(11):
        sim.t = t
        d2(t)
    got = D.read_fields(str(tmp_path / "G"))
    assert sorted(got) == [2, 7]
    np.testing.assert_allclose(got[7]["Ex"][0, 0], 100.0 * 2 + 2 + 1000.0 * (5 + 6 + 7) / 3)
