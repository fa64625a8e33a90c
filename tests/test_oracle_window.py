"""The oracle's moving window and particle creation (bc_oracle.c), on CPU.

The reference's SimWindow and ParticleCreator need its whole patch and Python
machinery, so these restatements are not run against compiled reference code
(parity unpinned); the tests check the properties that the reference's code
gives by construction: the shifted grid equals the old grid moved by the shift
with zeros in the fresh cells, particles keep their order and lose only those
below x = 0, created particles sit at the regular positions of their cells
with weights n dV / ppc, and the window moves when time_dual (v) passes x_moved.
"""
import numpy as np
import pytest

FIELDS = ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Bx_m", "By_m", "Bz_m", "Jx", "Jy", "Jz"]
STAG_X = {"Ex": 1, "Ey": 0, "Ez": 0, "Bx": 0, "By": 1, "Bz": 1, "Jx": 1, "Jy": 0, "Jz": 0}


def random_fields(n_cells, seed):
    from oracle import STAGGER
    rng = np.random.default_rng(seed)
    out = {}
    for k in FIELDS:
        st = STAGGER[k.replace("_m", "")]
        out[k] = rng.standard_normal(tuple(n_cells[d] + 5 + st[d] for d in range(2)))
    return out


def test_field_shift_moves_contents_and_zeroes_fresh_cells(cpu_oracle):
    n_cells, P = [20, 12], 4
    f = random_fields(n_cells, 3)
    old = {k: v.copy() for k, v in f.items()}
    sp = []
    cpu_oracle.window_shift(n_cells, 2, [0.1, 0.2], 0.05, f, sp, P, (False, True))
    for k in FIELDS:
        s = STAG_X[k.replace("_m", "")]
        keep = n_cells[0] - P + 2 + s
        a = f[k]
        if k in ("By", "Bz"):  # xmin boundary layer rewritten by Silver-Mueller
            np.testing.assert_array_equal(a[1:keep], old[k][1 + P:keep + P])
            assert not np.array_equal(a[0], old[k][P])
        else:
            np.testing.assert_array_equal(a[:keep], old[k][P:keep + P])
        assert not a[keep:].any(), k
        # the last kept point is in front of the fresh region: position < (N - P) dx
        assert (keep - 1 - 2 - 0.5 * s) < n_cells[0] - P


def test_particle_shift_removes_dropped_cells_keeps_order(cpu_oracle):
    n_cells, cl, P = [20, 12], [0.1, 0.2], 4
    rng = np.random.default_rng(5)
    n = 400
    pos = np.stack([rng.uniform(0, n_cells[0] * cl[0], n), rng.uniform(0, n_cells[1] * cl[1], n)])
    mom = rng.standard_normal((3, n))
    w = rng.uniform(1, 2, n)
    sp = [dict(pos=pos.copy(), mom=mom.copy(), weight=w.copy(), charge=np.full(n, -1, np.int16))]
    f = random_fields(n_cells, 4)
    cpu_oracle.window_shift(n_cells, 2, cl, 0.05, f, sp, P, (False, True))
    keep = pos[0] - P * cl[0] >= 0.0
    np.testing.assert_array_equal(sp[0]["pos"][0], pos[0][keep] - P * cl[0])
    np.testing.assert_array_equal(sp[0]["pos"][1], pos[1][keep])
    np.testing.assert_array_equal(sp[0]["mom"], mom[:, keep])
    np.testing.assert_array_equal(sp[0]["weight"], w[keep])


def test_created_particles_regular_positions_and_weights(cpu_oracle):
    n_cells, cl = [24, 6], [0.1, 0.15]
    prof = (0.7, 0.5, 0.8, 1e300, 0.0)  # vacuum to 0.5, ramp 0.8 long, plateau
    n_moved = 3
    pos, mom, w = cpu_oracle.create_particles(n_cells, cl, 2, 24, n_moved, prof, 4, 0.0, 0)
    xc = (n_moved + np.arange(2, 24) + 0.5) * cl[0] - prof[1]
    dens = prof[0] * np.clip(xc / prof[2], 0.0, 1.0) * (xc > 0)
    cells = np.nonzero(dens > 0)[0]
    assert w.size == cells.size * n_cells[1] * 4
    # weights: n dV / ppc per cell, cells in x order
    np.testing.assert_allclose(np.unique(w), np.unique(dens[cells] * cl[0] * cl[1] / 4), rtol=1e-15)
    # regular sub-positions 0.975 (0.5 + m) / 2 of the cell along each axis
    fx = pos[0] / cl[0] - np.floor(pos[0] / cl[0])
    fy = pos[1] / cl[1] - np.floor(pos[1] / cl[1])
    np.testing.assert_allclose(np.unique(np.round(fx, 9)), [0.24375, 0.73125])
    np.testing.assert_allclose(np.unique(np.round(fy, 9)), [0.24375, 0.73125])
    assert not mom.any()


def test_created_momenta_are_maxwellian(cpu_oracle):
    _, mom, _ = cpu_oracle.create_particles([64, 64], [0.1, 0.1], 0, 64, 0, (1.0, 0.0, 0.0, 1e300, 0.0), 4, 0.01, 11)
    assert mom.shape[1] == 64 * 64 * 4
    np.testing.assert_allclose(mom.std(axis=1), 0.1, rtol=0.03)
    np.testing.assert_allclose(mom.mean(axis=1), 0.0, atol=0.005)
    # a different seed gives different momenta; the same seed the same
    _, m2, _ = cpu_oracle.create_particles([64, 64], [0.1, 0.1], 0, 64, 0, (1.0, 0.0, 0.0, 1e300, 0.0), 4, 0.01, 11)
    _, m3, _ = cpu_oracle.create_particles([64, 64], [0.1, 0.1], 0, 64, 0, (1.0, 0.0, 0.0, 1e300, 0.0), 4, 0.01, 12)
    np.testing.assert_array_equal(mom, m2)
    assert not np.array_equal(mom, m3)


def test_non_power_ppc_is_refused(cpu_oracle):
    with pytest.raises(AssertionError):
        cpu_oracle.create_particles([8, 8], [0.1, 0.1], 0, 8, 0, (1.0, 0.0, 0.0, 1e300, 0.0), 3)


def test_window_moves_when_time_passes_distance(cpu_oracle):
    n_cells, cl = [16, 8], [0.1, 0.2]
    dt = 0.95 / np.sqrt(sum(1.0 / c ** 2 for c in cl))
    f = {k: np.zeros_like(v) for k, v in random_fields(n_cells, 1).items()}
    win = dict(t_start=0.3, velocity=1.0, shift=4)
    st = cpu_oracle.run_window(n_cells, cl, dt, f, [], (False, True), 30, win)
    td = (np.arange(30) + 1.5) * dt
    # expected shifts: step k moves when (td_k - t_start) v > x_moved
    x_moved, n = 0.0, 0
    for t in td:
        if (t - win["t_start"]) * win["velocity"] > x_moved:
            x_moved += cl[0] * win["shift"]
            n += 1
    assert st["n_moved"] == n * 4 and n >= 3
    assert st["x_moved"] == x_moved
