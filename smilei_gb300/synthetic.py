"""Seeded synthetic plasmas with the shapes of the benchmark configurations.

Positions are uniform inside each cell, ``ppc`` per cell (the reference's
``position_initialization="random"``, src/Particles/ParticleCreator.cpp:615);
momenta are Gaussian per component with sigma = sqrt(T / m c^2) (a Maxwellian
at non-relativistic temperature); weights are n0 * V_cell / ppc
(ParticleCreator.cpp:933-939).  The same arrays feed the GPU path and the CPU
oracle, so their results can be compared particle by particle.
"""
from __future__ import annotations

import numpy as np


def thermal_plasma(n_cells, cell_length, ppc, sigma_p, seed, density=1.0, unique_weights=False, dtype=np.float64):
    """Returns pos[ndim, n], mom[3, n], weight[n] (n = ppc * prod(n_cells))."""
    ndim = len(n_cells)
    rng = np.random.default_rng(seed)
    ncell = int(np.prod(n_cells))
    n = ncell * int(ppc)
    idx = np.repeat(np.arange(ncell, dtype=np.int64), ppc)
    pos = np.empty((ndim, n), dtype=dtype)
    rem = idx
    strides = [int(np.prod(n_cells[d + 1:])) for d in range(ndim)]
    for d in range(ndim):
        c = rem // strides[d]
        rem = rem % strides[d]
        pos[d] = (c + rng.random(n)) * cell_length[d]
    mom = rng.normal(0.0, sigma_p, (3, n)).astype(dtype)
    vol = float(np.prod(cell_length))
    w = np.full(n, density * vol / ppc, dtype=dtype)
    if unique_weights:
        # exactly representable in FP32 for n < 2^20: lets results be matched particle by particle
        w = w * (1.0 + np.arange(n, dtype=np.float64) * 2.0 ** -21)
    return pos, mom, w


def periodic_field(rng, ndim, n_cells, dual, scale=1.0, oversize=2):
    """Random field on a single periodic patch with ghosts: every copy of a node holds the same value."""
    shape = tuple(n_cells[d] + 1 + 2 * oversize + dual[d] for d in range(ndim))
    phys = rng.normal(0.0, scale, tuple(n_cells[:ndim]))
    index = np.ix_(*[(np.arange(shape[d]) - oversize) % n_cells[d] for d in range(ndim)])
    return np.ascontiguousarray(phys[index])


STAGGER = {
    "Ex": (1, 0, 0), "Ey": (0, 1, 0), "Ez": (0, 0, 1),
    "Bx": (0, 1, 1), "By": (1, 0, 1), "Bz": (1, 1, 0),
    "Jx": (1, 0, 0), "Jy": (0, 1, 0), "Jz": (0, 0, 1),
}


def periodic_em(seed, n_cells, e_scale=0.05, b_scale=0.05):
    """E, B and B_m = B, consistent over the periodic ghosts, for a single-patch grid."""
    ndim = len(n_cells)
    rng = np.random.default_rng(seed)
    out = {}
    for k in ("Ex", "Ey", "Ez", "Bx", "By", "Bz"):
        st = STAGGER[k][:ndim]
        out[k] = periodic_field(rng, ndim, n_cells, st, e_scale if k[0] == "E" else b_scale)
    for k in ("Bx", "By", "Bz"):
        out[k + "_m"] = out[k].copy()
    for k in ("Jx", "Jy", "Jz"):
        st = STAGGER[k][:ndim]
        out[k] = np.zeros(tuple(n_cells[d] + 5 + st[d] for d in range(ndim)))
    return out


def patch_ppc(n_patches, median_ppc, sigma_ln, ppc_max, seed):
    """Particles per cell of each patch: median_ppc * exp(N(0, sigma_ln)), floored, clipped to [0, ppc_max]."""
    rng = np.random.default_rng(seed)
    z = rng.normal(0.0, sigma_ln, int(np.prod(n_patches)))
    return np.clip(np.floor(median_ppc * np.exp(z)), 0, ppc_max).astype(np.int64).reshape(tuple(n_patches))


def uneven_plasma(n_cells, cell_length, patch, median_ppc, sigma_ln, ppc_max, sigma_p, seed, density=1.0):
    """Plasma whose particles per cell vary by patch (log-normal, clipped): pos, mom, weight, ppc per patch.

    Every macro-particle carries the weight of the median density, so a patch's
    density is proportional to its particles per cell."""
    ndim = len(n_cells)
    n_patches = [n_cells[d] // patch[d] for d in range(ndim)]
    ppc_p = patch_ppc(n_patches, median_ppc, sigma_ln, ppc_max, seed)
    rng = np.random.default_rng(seed + 1)
    grids = np.meshgrid(*[np.arange(n) for n in n_cells], indexing="ij")
    cell_ppc = ppc_p[tuple(g // patch[d] for d, g in enumerate(grids))].ravel()
    cells = np.repeat(np.arange(int(np.prod(n_cells)), dtype=np.int64), cell_ppc)
    n = cells.size
    pos = np.empty((ndim, n))
    rem = cells
    strides = [int(np.prod(n_cells[d + 1:])) for d in range(ndim)]
    for d in range(ndim):
        c = rem // strides[d]
        rem = rem % strides[d]
        pos[d] = (c + rng.random(n)) * cell_length[d]
    mom = rng.normal(0.0, sigma_p, (3, n))
    w = np.full(n, density * float(np.prod(cell_length)) / median_ppc)
    return pos, mom, w, ppc_p
