"""The per-cell sort entry point that allocates no device memory.

sg_sort_particles_noalloc exists for callers that cannot call cudaMalloc: a host
code that takes all of the GPU's memory into its own pool at start-up leaves none
for the library, and one that gives each library a fixed device-memory budget
cannot let a call grow it.  It sorts on a fixed scratch array in the library's
device image instead.  These tests call it through the C ABI and require results
identical to sg_sort_particles, the allocating entry point, on two calls in a row
with different shapes (the shared array keeps the previous call's contents, which
must not leak into the next result), and at its stated limits.  The file is
named to be collected last.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from smilei_gb300 import _lib
    return _lib


def _inputs(seed, ndim, patch, n):
    rng = np.random.default_rng(seed)
    cl = [0.1, 0.2, 0.15][:ndim]
    xmin = [3 * c for c in cl]
    pos = np.stack([xmin[d] + rng.uniform(-0.49, patch[d] + 0.49, n) * cl[d] for d in range(ndim)])
    mom = rng.normal(0, 1, (3, n))
    w = rng.uniform(0.5, 1.5, n)
    q = rng.choice(np.array([-1, 1], dtype=np.int16), n)
    return cl, xmin, pos, mom, w, q


def _sort(lib, fn, ndim, patch, cl, xmin, pos, mom, w, q):
    """Runs one sort entry point on fresh device copies; returns every output on the host."""
    n = pos.shape[1]
    ncell = int(np.prod([p + 1 for p in patch]))
    dev = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a)).to("cuda", dt)  # noqa: E731
    props = [dev(pos[d]) for d in range(ndim)] + [dev(mom[d]) for d in range(3)] + [dev(w)]
    charge = dev(q, torch.int16)
    first = torch.full((ncell,), -7, dtype=torch.int32, device="cuda")
    last = torch.full((ncell,), -7, dtype=torch.int32, device="cuda")
    keys = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    I = ctypes.c_int * ndim
    D = ctypes.c_double * ndim
    rc = getattr(lib.lib(), fn)(ndim, I(*patch), D(*xmin), D(*cl), n, lib.ptr_array(props), len(props),
                                lib.ptr(charge), lib.ptr(first), lib.ptr(last), lib.ptr(keys),
                                torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.lib().sg_last_error().decode()
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in props + [charge, first, last, keys]]


def test_noalloc_sort_matches_allocating_sort_twice_in_a_row(lib):
    cases = [(3, [9, 7, 6], 20000, 11), (2, [30, 17], 3000, 12)]  # larger first, then a smaller, other shape
    for ndim, patch, n, seed in cases:
        cl, xmin, pos, mom, w, q = _inputs(seed, ndim, patch, n)
        got = _sort(lib, "sg_sort_particles_noalloc", ndim, patch, cl, xmin, pos, mom, w, q)
        ref = _sort(lib, "sg_sort_particles", ndim, patch, cl, xmin, pos, mom, w, q)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b), (ndim, patch, n)
        assert np.all(np.diff(got[-1]) >= 0)


def test_noalloc_sort_at_its_limits_matches_allocating_sort(lib):
    """Exactly SG_SORT_NOALLOC_MAX_PARTICLES particles on a 32 x 32 x 32 node lattice,
    exactly SG_SORT_NOALLOC_MAX_CELLS: the fixed scratch holds the whole layout."""
    ndim, patch, n = 3, [31, 31, 31], 262144
    cl, xmin, pos, mom, w, q = _inputs(13, ndim, patch, n)
    for _ in range(2):
        got = _sort(lib, "sg_sort_particles_noalloc", ndim, patch, cl, xmin, pos, mom, w, q)
        ref = _sort(lib, "sg_sort_particles", ndim, patch, cl, xmin, pos, mom, w, q)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)


def test_noalloc_sort_rejects_sizes_beyond_its_scratch(lib):
    n = 262144 + 1  # one particle past SG_SORT_NOALLOC_MAX_PARTICLES: rejected before any GPU work
    I = ctypes.c_int * 1
    D = ctypes.c_double * 1
    null = ctypes.c_void_p()
    rc = lib.lib().sg_sort_particles_noalloc(1, I(8), D(0.0), D(0.1), n, lib.ptr_array([]), 1, null, null, null,
                                             null, None)
    assert rc == -1
    assert b"scratch limit" in lib.lib().sg_last_error()
    small = [torch.zeros(16, dtype=torch.float64, device="cuda") for _ in range(3)]
    idx = torch.zeros(16, dtype=torch.int32, device="cuda")
    rc = lib.lib().sg_sort_particles_noalloc(3, (ctypes.c_int * 3)(40, 40, 40), (ctypes.c_double * 3)(0, 0, 0),
                                             (ctypes.c_double * 3)(0.1, 0.1, 0.1), 10, lib.ptr_array(small), 3, null,
                                             lib.ptr(idx), lib.ptr(idx), null, None)
    assert rc == -1  # 41^3 cells > SG_SORT_NOALLOC_MAX_CELLS
    assert b"scratch limit" in lib.lib().sg_last_error()
