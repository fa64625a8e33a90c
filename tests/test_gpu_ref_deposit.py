"""The reference's own CUDA current deposits (DepositCurrentDensity_3D_Order2,
src/Projector/Projector3D2OrderGPUKernelCUDAHIP.cu:136-516, and
DepositCurrentDensity_2D_Order2, Projector2D2OrderGPUKernelCUDAHIP.cu:545-870), compiled
from the reference tree by oracle/build_ref.sh and run here through
oracle/ref_gpu_deposit.py.

- Driven as currentDepositionKernel3D drives it, its currents match the oracle's
  Esirkepov deposit (oracle/pic_oracle.c or_project) within 1e-12 on a 16x12x8 patch
  with particles sorted by 4^3 bin, for particles whose nearest node does not
  increase; for one whose node increases along d it drops the fifth stencil row of
  the currents transverse to d (a difference of the reference's CUDA kernel from its
  CPU projector, which the oracle follows).
- On the 256^3 x 8 ppc thermal plasma (134,217,728 particles) its deposit alone is
  timed against this project's whole particle kernel (gather, push, deposit and
  re-binning; mixed and FP64 forms) on the same plasma; the line printed holds the
  times.

- The 2D kernel matches the oracle within 1e-12 for particles moving either way, and is
  timed on the 2D thermal plasma (256 x 256, electrons and protons at 16 ppc each)
  against this project's particle kernels of a step.

Skipped where the cubins were not built (no reference tree when build() ran).
"""
import json

import numpy as np
import pytest

from conftest import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import ref_gpu_deposit
    if not ref_gpu_deposit.available():
        pytest.skip("the reference's CUDA deposit was not compiled (oracle/build_ref.sh)")
    torch.zeros(1, device="cuda")  # the runtime's primary context first
    return ref_gpu_deposit.RefGpuDeposit()


def _cu(a, dtype=None):
    return torch.as_tensor(np.ascontiguousarray(a if dtype is None else a.astype(dtype)), device="cuda")


def _patch_case(plus):
    """Particles on a 16x12x8 patch (origin 0, oversize 2) sorted by 4^3 bin, each moving
    less than half a cell; plus[d] False drops those whose nearest node increases along d."""
    rng = np.random.default_rng(17)
    cells = np.array([16, 12, 8])
    cl = np.array([0.1, 0.12, 0.09])
    nb = cells // 4
    n = int(cells.prod()) * 4
    cell = rng.integers(0, cells, size=(n, 3))
    frac = rng.uniform(0, 1, (n, 3))
    disp = rng.uniform(-0.45, 0.45, (n, 3))
    shift = np.floor(cell + frac + disp + 0.5) - np.floor(cell + frac + 0.5)
    keep = np.ones(n, bool)
    for d in range(3):
        if not plus[d]:
            keep &= shift[:, d] <= 0
    cell, frac, disp = cell[keep], frac[keep], disp[keep]
    binid = ((cell[:, 0] // 4) * nb[1] + cell[:, 1] // 4) * nb[2] + cell[:, 2] // 4
    order = np.argsort(binid, kind="stable")
    cell, frac, disp, binid = cell[order], frac[order], disp[order], binid[order]
    n = cell.shape[0]
    xold = ((cell + frac) * cl).T.copy()
    xnew = ((cell + frac + disp) * cl).T.copy()
    db = [-2, -2, -2]
    # iold, deltaold planes [d * n + p] of the old positions (the interpolator's round)
    iold = np.zeros(3 * n, np.int32)
    delta = np.zeros(3 * n)
    for d in range(3):
        xn = xold[d] / cl[d]
        ip = np.floor(xn + 0.5)
        iold[d * n:(d + 1) * n] = (ip - db[d]).astype(np.int32)
        delta[d * n:(d + 1) * n] = xn - ip
        # the kernel's shared tiles stay in bounds: the old node lies in the bin's window
        ipo = iold[d * n:(d + 1) * n] - 2 - 4 * (cell[:, d] // 4)
        assert ipo.min() >= 0 and ipo.max() <= 4
    w = rng.uniform(0.5, 1.5, cell.shape[0])
    q = np.where(rng.uniform(size=n) < 0.5, -1, 1).astype(np.int16)
    return dict(cells=cells, cl=cl, nb=nb, n=n, binid=binid, xnew=xnew, iold=iold, delta=delta, w=w, q=q, db=db,
                n_prim=(cells + 5).tolist(), dt=0.05)


def _both(ref, cpu_oracle, c):
    n_prim, cl, n = c["n_prim"], c["cl"], c["n"]
    shapes = [(n_prim[0] + 1, n_prim[1], n_prim[2]), (n_prim[0], n_prim[1] + 1, n_prim[2]),
              (n_prim[0], n_prim[1], n_prim[2] + 1)]
    J = cpu_oracle.project(0, 3, n_prim, c["db"], cl, c["dt"], c["xnew"], np.zeros((3, n)), c["w"], c["q"],
                           np.ones(n), c["iold"], c["delta"], [np.zeros(s) for s in shapes] + [None])[:3]
    Jd = [torch.zeros(s, dtype=torch.float64, device="cuda") for s in shapes]
    pos = [_cu(c["xnew"][d]) for d in range(3)]
    bin_index = _cu(np.cumsum(np.bincount(c["binid"], minlength=int(c["nb"].prod()))), np.int32)
    qd, wd, invgf, iold, delta = _cu(c["q"]), _cu(c["w"]), _cu(np.ones(n)), _cu(c["iold"]), _cu(c["delta"])
    ref.launch(c["nb"], J=[a.data_ptr() for a in Jd], J_sizes=[a.numel() for a in Jd],
               pos=[p.data_ptr() for p in pos], charge=qd.data_ptr(), weight=wd.data_ptr(),
               bin_index=bin_index.data_ptr(), invgf=invgf.data_ptr(), iold=iold.data_ptr(),
               deltaold=delta.data_ptr(), inv_cell_volume=1.0 / float(np.prod(cl)), dx_inv=list(1.0 / cl),
               dx_ov_dt=list(cl / c["dt"]), domain_begin=c["db"], nprimy=n_prim[1], nprimz=n_prim[2])
    torch.cuda.synchronize()
    return [float(rel_err(Jd[k].cpu().numpy(), J[k])) for k in range(3)]


def test_reference_gpu_deposit_matches_oracle(ref, cpu_oracle):
    """Particles whose nearest node does not increase: the reference kernel and the oracle
    agree to rounding."""
    err = _both(ref, cpu_oracle, _patch_case((False, False, False)))
    assert max(err) <= 1e-12, err


@pytest.mark.parametrize("d", [0, 1, 2])
def test_reference_gpu_deposit_drops_the_fifth_transverse_point(ref, cpu_oracle, d):
    """A particle whose nearest node increases along d has a nonzero S1[4] along d
    (init_S1, :114-131), but the kernel's loops over the transverse stencil points run
    0..3 (Jx :302-365, Jy :367-427, Jz :429-490), so the currents transverse to d miss
    that row; the current along d is whole (its fifth cumulative value is zero).  The
    oracle and the reference's CPU projector (Projector3D2Order.cpp:81-90, loops 0..4)
    keep it.  Measured here: the current
    along d still agrees to rounding, the two transverse ones differ by about 1 %."""
    err = _both(ref, cpu_oracle, _patch_case(tuple(k == d for k in range(3))))
    assert err[d] <= 1e-12, err
    assert all(err[k] > 1e-3 for k in range(3) if k != d), err


def test_fused_step_against_reference_gpu_deposit_at_256(ref):
    from smilei_gb300 import simulation, _lib
    N, ppc, dx = 256, 8, 0.1
    dt = 0.95 * dx / np.sqrt(3.0)
    sigma = np.sqrt(10.0 / 511.0)
    n = N ** 3 * ppc
    nb = N // 4
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    # particles in bin order: bin-major, then the 64 cells of the bin, ppc per cell
    cb = torch.arange(n, device="cuda", dtype=torch.int64) // ppc
    b, loc = cb // 64, cb % 64
    del cb
    cell = [(b // (nb * nb)) * 4 + loc // 16, ((b // nb) % nb) * 4 + (loc // 4) % 4, (b % nb) * 4 + loc % 4]
    del b, loc
    xold = torch.empty((3, n), dtype=torch.float64, device="cuda")
    for d in range(3):
        xold[d] = (cell[d].to(torch.float64) + torch.rand(n, generator=g, device="cuda", dtype=torch.float64)) * dx
    del cell
    mom = torch.randn((3, n), generator=g, device="cuda", dtype=torch.float64) * sigma
    invgf = 1.0 / torch.sqrt(1.0 + (mom * mom).sum(0))
    xnew = xold + mom * invgf * dt
    ip = torch.floor(xold / dx + 0.5)
    iold = (ip + 2).to(torch.int32).reshape(-1).contiguous()
    delta = (xold / dx - ip).reshape(-1).contiguous()
    del ip
    w = torch.full((n,), dx ** 3 / ppc, dtype=torch.float64, device="cuda")
    q = torch.full((n,), -1, dtype=torch.int16, device="cuda")
    bin_index = ((torch.arange(nb ** 3, device="cuda", dtype=torch.int64) + 1) * 64 * ppc).to(torch.int32)
    npr = N + 5
    shapes = [(npr + 1, npr, npr), (npr, npr + 1, npr), (npr, npr, npr + 1)]
    Jd = [torch.zeros(s, dtype=torch.float64, device="cuda") for s in shapes]
    stream = torch.cuda.current_stream()
    kw = dict(J=[a.data_ptr() for a in Jd], J_sizes=[a.numel() for a in Jd],
              pos=[xnew[d].data_ptr() for d in range(3)], charge=q.data_ptr(), weight=w.data_ptr(),
              bin_index=bin_index.data_ptr(), invgf=invgf.data_ptr(), iold=iold.data_ptr(), deltaold=delta.data_ptr(),
              inv_cell_volume=1.0 / dx ** 3, dx_inv=[1.0 / dx] * 3, dx_ov_dt=[dx / dt] * 3, domain_begin=[-2] * 3,
              nprimy=npr, nprimz=npr, stream=stream.cuda_stream)
    ref_ms = {}
    for sorting in (False, True):
        ref.launch([nb] * 3, cell_sorting=sorting, **kw)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            ref.launch([nb] * 3, cell_sorting=sorting, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
        ref_ms["cell_sorting" if sorting else "default"] = e0.elapsed_time(e1) / 3
    assert float(Jd[0].abs().sum()) > 0.0
    del Jd, xnew, iold, delta, invgf, q, bin_index
    torch.cuda.empty_cache()
    # this project's particle kernel on the same plasma (old positions, momenta, weights),
    # in the mixed form and in the FP64 form (the reference kernel computes in FP64)
    ours = {}
    for form in ("mixed", "fp64"):
        s = torch.cuda.Stream()
        sim = simulation.Simulation([N] * 3, [dx] * 3, dt, form=form)
        _lib.check(_lib.lib().sg_sim_set_stream(sim._h, s.cuda_stream), "set_stream")
        sim.add_species(1.0, -1.0, "higueracary", xold, mom, w)
        torch.cuda.empty_cache()
        with torch.cuda.stream(s):
            sim.step(2)
            tp = []
            for _ in range(3):
                sim.step(1)
                tp.append(sim.last_timing()[0])
        sim.close()
        torch.cuda.empty_cache()
        ours[form] = float(np.mean(tp))
    line = {"particles": n, "reference_deposit_ms": ref_ms, "fused_particle_kernel_ms": ours,
            "reference_default_over_fused_mixed": ref_ms["default"] / ours["mixed"],
            "reference_default_over_fused_fp64": ref_ms["default"] / ours["fp64"]}
    print("REF_GPU_DEPOSIT " + json.dumps(line))
    assert ours["mixed"] < ref_ms["default"] and ours["fp64"] < ref_ms["default"]


@pytest.fixture(scope="module")
def ref2():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import ref_gpu_deposit
    if not ref_gpu_deposit.available(2):
        pytest.skip("the reference's 2D CUDA deposit was not compiled (oracle/build_ref.sh)")
    torch.zeros(1, device="cuda")
    return ref_gpu_deposit.RefGpuDeposit(ndim=2)


def _launch2d(ref2, c, J, pos, momz, q, w, bin_index, invgf, iold, delta, stream=0, cell_sorting=False):
    ref2.launch2d(c["nb"], J=[a.data_ptr() for a in J], J_sizes=[a.numel() for a in J], pos=pos, momz=momz, charge=q,
                  weight=w, bin_index=bin_index, invgf=invgf, iold=iold, deltaold=delta,
                  inv_cell_volume=1.0 / float(np.prod(c["cl"])), dx_inv=[1.0 / v for v in c["cl"]],
                  dx_ov_dt=[v / c["dt"] for v in c["cl"]], domain_begin=[-2, -2], nprimy=c["n_prim"][1],
                  cell_sorting=cell_sorting, stream=stream)


def test_reference_gpu_deposit_2d_matches_oracle(ref2, cpu_oracle):
    """The 2D kernel's loops run over the whole 5 x 5 stencil: its three currents match the
    oracle's for particles moving either way."""
    rng = np.random.default_rng(23)
    cells = np.array([16, 12])
    cl = np.array([0.1, 0.15])
    nb = cells // 4
    n = int(cells.prod()) * 6
    cell = rng.integers(0, cells, size=(n, 2))
    binid = (cell[:, 0] // 4) * nb[1] + cell[:, 1] // 4
    order = np.argsort(binid, kind="stable")
    cell, binid = cell[order], binid[order]
    frac = rng.uniform(0, 1, (n, 2))
    xold = ((cell + frac) * cl).T.copy()
    xnew = ((cell + frac + rng.uniform(-0.45, 0.45, (n, 2))) * cl).T.copy()
    mom = rng.normal(0, 0.3, (3, n))
    invgf = 1.0 / np.sqrt(1.0 + (mom ** 2).sum(0))
    w = rng.uniform(0.5, 1.5, n)
    q = np.where(rng.uniform(size=n) < 0.5, -1, 1).astype(np.int16)
    iold = np.zeros(2 * n, np.int32)
    delta = np.zeros(2 * n)
    for d in range(2):
        xn = xold[d] / cl[d]
        ip = np.floor(xn + 0.5)
        iold[d * n:(d + 1) * n] = (ip + 2).astype(np.int32)
        delta[d * n:(d + 1) * n] = xn - ip
        ipo = iold[d * n:(d + 1) * n] - 2 - 4 * (cell[:, d] // 4)
        assert ipo.min() >= 0 and ipo.max() <= 4
    n_prim = (cells + 5).tolist()
    c = dict(nb=nb, cl=cl, dt=0.05, n_prim=n_prim)
    shapes = [(n_prim[0] + 1, n_prim[1]), (n_prim[0], n_prim[1] + 1), (n_prim[0], n_prim[1])]
    J = cpu_oracle.project(0, 2, n_prim, [-2, -2], cl, c["dt"], xnew, mom, w, q, invgf, iold, delta,
                           [np.zeros(s) for s in shapes] + [None])[:3]
    Jd = [torch.zeros(s, dtype=torch.float64, device="cuda") for s in shapes]
    t = [_cu(xnew[0]), _cu(xnew[1]), _cu(mom[2]), _cu(q), _cu(w), _cu(np.cumsum(np.bincount(binid, minlength=int(nb.prod()))), np.int32),
         _cu(invgf), _cu(iold), _cu(delta)]
    _launch2d(ref2, c, Jd, [t[0].data_ptr(), t[1].data_ptr()], *[a.data_ptr() for a in t[2:]])
    torch.cuda.synchronize()
    for k in range(3):
        assert rel_err(Jd[k].cpu().numpy(), J[k]) <= 1e-12, k


def test_fused_step_against_reference_gpu_deposit_2d_thermal(ref2):
    """The 2D thermal plasma of the bench (256 x 256 cells, electrons and protons at 16 ppc
    each, Boris): the reference's deposit of both species against this project's particle
    kernels of a step (gather, push, deposit and re-binning of both species)."""
    from smilei_gb300 import simulation, _lib
    N, ppc, dx = 256, 16, 0.1
    dt = 0.95 * dx / np.sqrt(2.0)
    sig = np.sqrt(10.0 / 511.0)
    species = [(1.0, -1, sig), (1836.0, 1, sig / np.sqrt(1836.0))]
    nb = N // 4
    n = N * N * ppc
    c = dict(nb=[nb, nb], cl=[dx, dx], dt=dt, n_prim=[N + 5, N + 5])
    stream = torch.cuda.current_stream()
    shapes = [(N + 6, N + 5), (N + 5, N + 6), (N + 5, N + 5)]
    Jd = [torch.zeros(s, dtype=torch.float64, device="cuda") for s in shapes]
    g = torch.Generator(device="cuda")
    g.manual_seed(9)
    plasma, launches = [], []
    for k, (mass, charge, sigma) in enumerate(species):
        cb = torch.arange(n, device="cuda", dtype=torch.int64) // ppc
        b, loc = cb // 16, cb % 16
        cell = [(b // nb) * 4 + loc // 4, (b % nb) * 4 + loc % 4]
        xold = torch.empty((2, n), dtype=torch.float64, device="cuda")
        for d in range(2):
            xold[d] = (cell[d].to(torch.float64) + torch.rand(n, generator=g, device="cuda", dtype=torch.float64)) * dx
        mom = torch.randn((3, n), generator=g, device="cuda", dtype=torch.float64) * sigma
        invgf = 1.0 / torch.sqrt(1.0 + (mom * mom).sum(0))
        xnew = (xold + mom[:2] * invgf * dt).contiguous()
        ip = torch.floor(xold / dx + 0.5)
        iold = (ip + 2).to(torch.int32).reshape(-1).contiguous()
        delta = (xold / dx - ip).reshape(-1).contiguous()
        w = torch.full((n,), dx * dx / ppc, dtype=torch.float64, device="cuda")
        q = torch.full((n,), charge, dtype=torch.int16, device="cuda")
        bin_index = ((torch.arange(nb * nb, device="cuda", dtype=torch.int64) + 1) * 16 * ppc).to(torch.int32)
        momz = mom[2].contiguous()
        keep = [xnew, iold, delta, w, q, bin_index, momz, invgf]
        launches.append((keep, [xnew[0].data_ptr(), xnew[1].data_ptr()], momz.data_ptr(), q.data_ptr(), w.data_ptr(),
                         bin_index.data_ptr(), invgf.data_ptr(), iold.data_ptr(), delta.data_ptr()))
        plasma.append((mass, float(charge), xold, mom, w))
    ref_ms = {}
    for sorting in (False, True):
        for _, pos, *ptrs in launches:
            _launch2d(ref2, c, Jd, pos, *ptrs, stream=stream.cuda_stream, cell_sorting=sorting)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(5):
            for _, pos, *ptrs in launches:
                _launch2d(ref2, c, Jd, pos, *ptrs, stream=stream.cuda_stream, cell_sorting=sorting)
        e1.record(stream)
        torch.cuda.synchronize()
        ref_ms["cell_sorting" if sorting else "default"] = e0.elapsed_time(e1) / 5
    assert float(Jd[2].abs().sum()) > 0.0
    ours = {}
    for form in ("mixed", "fp64"):
        s = torch.cuda.Stream()
        sim = simulation.Simulation([N, N], [dx, dx], dt, form=form)
        _lib.check(_lib.lib().sg_sim_set_stream(sim._h, s.cuda_stream), "set_stream")
        for mass, charge, xold, mom, w in plasma:
            sim.add_species(mass, charge, "boris", xold, mom, w)
        with torch.cuda.stream(s):
            sim.step(3)
            tp = []
            for _ in range(5):
                sim.step(1)
                tp.append(sim.last_timing()[0])
        sim.close()
        ours[form] = float(np.mean(tp))
    line = {"particles": 2 * n, "reference_deposit_ms_both_species": ref_ms, "fused_particle_kernels_ms": ours,
            "reference_default_over_fused_mixed": ref_ms["default"] / ours["mixed"],
            "reference_default_over_fused_fp64": ref_ms["default"] / ours["fp64"]}
    print("REF_GPU_DEPOSIT_2D " + json.dumps(line))
    assert ours["mixed"] < ref_ms["default"]
