"""Benchmark: particle-steps/s of the resident PIC timestep on one GB300 (and replicas on N GPUs).

Workload (default): the 3D thermal plasma -- 256^3 cells, dx = 0.1 c/omega_p,
dt = 0.95 CFL, periodic, electrons only over an immobile neutralising
background, 8 particles per cell (134,217,728 particles), Maxwellian
T = 10 keV (sigma_p = sqrt(10/511)), Higuera-Cary pusher, order-2 gather and
Esirkepov deposit, Yee solver -- in the split-precision form (int cell index +
FP32 offset, FP32 arithmetic); ``--form fp64`` runs the plain FP64 form.
Synthetic seeded inputs are generated on the device.

One step = gather + push + deposit + per-tile sort of every particle, J ghost
fold, Ampere, Faraday and B centring (sg_sim_step).  ``value`` is the
device-timed throughput with the state resident in HBM (134M particles, far
larger than L2); ``e2e`` drives the same step through the C ABI from host
buffers: each step copies the particle state host->device, steps, copies it
back and reads the energy scalars.

``--impl reference`` times the CPU restatement of the reference operators
(oracle/pic_oracle.c, OpenMP on every host core) on a bounded sample of the
same workload; it is the reference arm because the reference's OpenACC GPU
build needs a compiler that is not installed and the reference tree is not
present on the GPU host.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300 (mixed vs FP64 form), % of HBM roofline"
UNIT = "particle-steps/s"
# the step's result read back every e2e step: the 16 FP64 energy sums (sg_sim_energy)
ENERGY_READBACK_BYTES = 16 * 8
SIGMA_10KEV = float(np.sqrt(10.0 / 511.0))


def workload_cfg(args):
    dx = 0.1
    dt = 0.95 * dx / np.sqrt(3.0)
    if getattr(args, "workload", "thermal") == "thermal2d":
        # 2D thermal plasma: 256 x 256 cells, electrons and protons (mass 1836) at 16 ppc each,
        # T = 10 keV in each species' own momentum unit (sigma = sqrt(T / m c^2)), Boris
        return dict(n_cells=[256, 256], cell_length=[dx, dx], dt=float(0.95 * dx / np.sqrt(2.0)), ppc=16,
                    pusher="boris", sigma=SIGMA_10KEV,
                    species=[dict(mass=1.0, charge=-1.0, sigma=SIGMA_10KEV),
                             dict(mass=1836.0, charge=1.0, sigma=SIGMA_10KEV / np.sqrt(1836.0))])
    if getattr(args, "workload", "thermal") == "uneven":
        # batched uneven patches: 512 x 256 x 256 cells in 1024 patches of 32^3, particles per
        # cell per patch 8 * exp(N(0, 1.5)) floored and clipped to [0, 64], T = 5 keV, Boris
        return dict(n_cells=[512, 256, 256], cell_length=[dx, dx, dx], dt=float(dt), ppc=8, pusher="boris",
                    sigma=float(np.sqrt(5.0 / 511.0)), patch=[32, 32, 32], sigma_ln=1.5, ppc_max=64)
    n = args.cells
    return dict(n_cells=[n, n, n], cell_length=[dx, dx, dx], dt=float(dt), ppc=args.ppc, pusher="higueracary",
                sigma=SIGMA_10KEV)


# DRAM bytes read + written per particle by one k_step_particles launch: one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of the 3D thermal case at
# 128^3 cells x 8 ppc, divided by its 16,777,216 particles; a launch over N particles
# at the same ppc moves N times this.  None where no capture has been taken.
NCU_TRAFFIC_BYTES_PER_PARTICLE = {"mixed": (693.389568e6 + 557.328640e6) / 16777216, "fp64": None}


def bytes_alg_per_particle_step(form, ppc, ndim=3):
    """B_alg = S_state + 24 * s / ppc (state read+write once; 24 grid values per cell per step).
    S_state: 3D 60 B mixed, 104 B FP64; 2D3V 52 B mixed, 88 B FP64."""
    if form == "mixed":
        st = 60.0 if ndim == 3 else 52.0
        return st + 24 * 4 / ppc, st, 4
    st = 104.0 if ndim == 3 else 88.0
    return st + 24 * 8 / ppc, st, 8


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join("/tmp", f"sg_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None:
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        except OSError:
            return None
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_uniform_2d(cfg, sigma, seed, device):
    """ppc particles per cell at uniform random positions, Maxwellian momenta of width sigma,
    weight n0 dV / ppc (n0 = 1), 2D, on the device."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    n_cells, cl, ppc = cfg["n_cells"], cfg["cell_length"], cfg["ppc"]
    n = int(np.prod(n_cells)) * ppc
    cell = torch.arange(n, device=device, dtype=torch.int64) // ppc
    pos = torch.empty((2, n), dtype=torch.float64, device=device)
    pos[0] = ((cell // n_cells[1]).to(torch.float64) + torch.rand(n, generator=g, device=device,
                                                                   dtype=torch.float64)) * cl[0]
    pos[1] = ((cell % n_cells[1]).to(torch.float64) + torch.rand(n, generator=g, device=device,
                                                                  dtype=torch.float64)) * cl[1]
    mom = torch.randn((3, n), generator=g, device=device, dtype=torch.float64) * sigma
    w = torch.full((n,), float(np.prod(cl)) / ppc, dtype=torch.float64, device=device)
    return pos, mom, w


def add_plasma(sim, cfg, seed, device):
    """Adds the workload's species to sim; returns the particle count."""
    if "species" in cfg:
        n = 0
        for k, sp in enumerate(cfg["species"]):
            pos, mom, w = make_uniform_2d(cfg, sp["sigma"], seed + 7919 * k, device)
            sim.add_species(sp["mass"], sp["charge"], cfg["pusher"], pos, mom, w)
            n += int(w.shape[0])
        return n
    pos, mom, w = make_plasma(cfg, seed, device)
    sim.add_species(1.0, -1.0, cfg["pusher"], pos, mom, w)
    return int(w.shape[0])


def make_plasma(cfg, seed, device):
    """Seeded plasma generated on the device (FP64 positions, momenta, weights).

    Uniform ppc, or for the uneven workload a particles-per-cell count per patch
    (smilei_gb300.synthetic.patch_ppc); every particle has the median density's weight."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    n_cells, cl, ppc = cfg["n_cells"], cfg["cell_length"], cfg["ppc"]
    ncell = int(np.prod(n_cells))
    if "patch" in cfg:
        from smilei_gb300 import synthetic
        patch = cfg["patch"]
        npat = [n_cells[d] // patch[d] for d in range(3)]
        ppc_p = torch.as_tensor(synthetic.patch_ppc(npat, ppc, cfg["sigma_ln"], cfg["ppc_max"], seed), device=device)
        ids = torch.arange(ncell, device=device, dtype=torch.int64)
        pidx = ((ids // (n_cells[1] * n_cells[2])) // patch[0]) * npat[1] * npat[2] + \
            (((ids // n_cells[2]) % n_cells[1]) // patch[1]) * npat[2] + ((ids % n_cells[2]) // patch[2])
        cell = torch.repeat_interleave(ids, ppc_p.reshape(-1)[pidx])
        del ids, pidx
        n = int(cell.numel())
    else:
        n = ncell * ppc
        cell = torch.arange(n, device=device, dtype=torch.int64) // ppc
    pos = torch.empty((3, n), dtype=torch.float64, device=device)
    strides = [n_cells[1] * n_cells[2], n_cells[2], 1]
    for d in range(3):
        c = (cell // strides[d]) % n_cells[d]
        pos[d] = (c.to(torch.float64) + torch.rand(n, generator=g, device=device, dtype=torch.float64)) * cl[d]
        del c
    del cell
    mom = torch.randn((3, n), generator=g, device=device, dtype=torch.float64) * cfg["sigma"]
    w = torch.full((n,), float(np.prod(cl)) / ppc, dtype=torch.float64, device=device)
    return pos, mom, w


def max_over_ranks(x: float, device) -> float:
    """The largest of every rank's x (the job's time is its slowest replica's)."""
    import torch
    import torch.distributed as td
    if not (td.is_available() and td.is_initialized()) or td.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(particles_per_rank: int, world: int, steps: int, ms: float) -> float:
    """Particle-steps/s of the whole job: every replica's particles over the slowest replica's time."""
    return particles_per_rank * world * steps / (ms / 1e3)


def time_batched(sim, steps, stream, device):
    """The same steps through one sg_sim_step(steps) call: batched graphs of up to 8 steps,
    one host wait per batch (the timed loops above wait after every step, to read each
    step's stage times).  Returns (ms per step, batched graphs launched)."""
    import torch
    sim.step(2)  # untimed: builds the batched graph (an even count keeps the parity the timed steps start from)
    b0 = sim.batch_stats()[0]
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sim.step(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    return max_over_ranks(e0.elapsed_time(e1), device) / steps, sim.batch_stats()[0] - b0


def run_gpu(args, rank, world, local_rank):
    import torch
    from smilei_gb300 import simulation
    device = f"cuda:{local_rank}"
    torch.cuda.set_device(local_rank)
    cfg = workload_cfg(args)
    # a dedicated stream: the step is captured as a CUDA graph, which the legacy default stream does not allow
    stream = torch.cuda.Stream(device=device)
    torch.cuda.set_stream(stream)
    from smilei_gb300 import _lib

    def build(tile):
        sm = simulation.Simulation(cfg["n_cells"], cfg["cell_length"], cfg["dt"], form=args.form,
                                   tile=list(tile) if tile else None, use_graph=True, capacity_slack=args.slack)
        _lib.check(_lib.lib().sg_sim_set_stream(sm._h, stream.cuda_stream), "set_stream")
        add_plasma(sm, cfg, args.seed + rank, device)
        torch.cuda.empty_cache()
        return sm

    ndim = len(cfg["n_cells"])
    tile, tuning, queue = ([args.tile] * ndim if args.tile else None), None, args.tile_queue
    # TMA staging is the default of the 3D mixed form with 4x4x4 tiles; --no-tma turns it off
    tma_choice = not args.no_tma
    if args.autotune:
        from smilei_gb300 import autotune
        (best, queue, tma_choice), times = autotune.tune(build, ndim=ndim,
                                                         stagings=(False,) if args.no_tma else (True, False))
        tile = list(best)
        tuning = {"x".join(map(str, k)) + (" queue" if q else "") + (" tma" if t else ""): round(v, 3)
                  for (k, q, t), v in times.items()}
    sim = build(tile)
    sim.set_tile_queue(queue)
    tma = len(cfg["n_cells"]) == 3 and args.form == "mixed" and list(tile or [4, 4, 4]) == [4, 4, 4]
    if tma and not tma_choice:
        sim.set_tma_staging(False)
        tma = False
    nspec = len(cfg.get("species", [None]))
    n = sum(sim.species_count(k) for k in range(nspec))
    # initial E from the charge (FP64 CG, as the reference's solve_poisson): the charge
    # residual then measures what the steps add
    poisson = sim.solve_poisson(max_error=POISSON_MAX_ERROR) if args.poisson else None
    res0 = sim.charge_residual() if args.poisson else None
    uk0, ue0 = sim.energy()
    for _ in range(args.warmup):
        sim.step(1)
    dist = world > 1
    if dist:
        import torch.distributed as td
        td.barrier()
    torch.cuda.synchronize()
    t_part = []
    launches = 0
    with ClockSampler(local_rank) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        wall0 = time.perf_counter()
        ev0.record(stream)
        for _ in range(args.steps):
            sim.step(1)
            tp, tf, tt, launches = sim.last_timing()
            t_part.append(tp)
        ev1.record(stream)
        torch.cuda.synchronize()
        wall1 = time.perf_counter()
    if dist:
        td.barrier()
    ms = max_over_ranks(ev0.elapsed_time(ev1), device)
    uk1, ue1 = sim.energy()
    res1 = sim.charge_residual() if args.poisson else None
    relayouts = sim.layout_stats()
    # the run's fields after the warm-up and timed steps, for the comparison with the FP64 form
    fields_mixed = None
    if args.compare_fp64 and args.form == "mixed" and args.workload in ("thermal", "thermal2d"):
        fields_mixed = {k: sim.get_field(k) for k in COMPARE_FIELDS}

    # e2e: the same step driven from host buffers through the C ABI
    e2e = None
    if not args.no_e2e and nspec > 1:
        # every species' packed state host->device, the step, and back (no streamed variant
        # for several species)
        nb = [sim.packed_bytes(k) for k in range(nspec)]
        hosts = [torch.empty(b, dtype=torch.uint8, pin_memory=True) for b in nb]
        for k in range(nspec):
            sim.pack_state(k, hosts[k].data_ptr())
        torch.cuda.synchronize()
        ke = max(1, min(args.steps, args.e2e_steps))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(ke):
            for k in range(nspec):
                sim.unpack_state(k, hosts[k].data_ptr())
            sim.step(1)
            for k in range(nspec):
                sim.pack_state(k, hosts[k].data_ptr())
            sim.energy()
        e1.record(stream)
        torch.cuda.synchronize()
        ems = max_over_ranks(e0.elapsed_time(e1), device)
        e2e = {"value": whole_job_rate(n, world, ke, ems), "unit": UNIT, "h2d_bytes_per_step": int(sum(nb)),
               "d2h_bytes_per_step": int(sum(nb) + ENERGY_READBACK_BYTES), "steps": ke}
        del hosts
    elif not args.no_e2e:
        nbytes = sim.packed_bytes(0)
        host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        sim.pack_state(0, host.data_ptr())
        torch.cuda.synchronize()
        if args.e2e_chunks > 0:
            sim.step_host(0, host.data_ptr(), chunks=args.e2e_chunks)  # untimed: its staging buffers
            torch.cuda.synchronize()
        ke = max(1, min(args.steps, args.e2e_steps))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        if dist:
            td.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(ke):
            if args.e2e_chunks > 0:
                # the copy in overlaps the particle kernel over tile ranges
                sim.step_host(0, host.data_ptr(), chunks=args.e2e_chunks)
            else:
                sim.unpack_state(0, host.data_ptr())
                sim.step(1)
                sim.pack_state(0, host.data_ptr())
            sim.energy()
        e1.record(stream)
        torch.cuda.synchronize()
        ems = max_over_ranks(e0.elapsed_time(e1), device)
        e2e = {"value": whole_job_rate(n, world, ke, ems), "unit": UNIT, "h2d_bytes_per_step": int(nbytes),
               "d2h_bytes_per_step": int(nbytes + ENERGY_READBACK_BYTES), "steps": ke}
        if args.e2e_chunks > 0:
            e2e["last_step_stages_ms"] = sim.stream_timing()
        del host
    bms, nb = time_batched(sim, args.steps, stream, device)
    batched = {"ms_per_step": bms, "value": whole_job_rate(n, world, 1, bms), "steps": args.steps, "graphs": nb}
    sim.close()
    fp64 = None
    if fields_mixed is not None:
        fp64 = run_fp64_compare(args, cfg, rank, device, stream, fields_mixed, (uk0 + ue0, uk1 + ue1))
        del fields_mixed
    ncell_all = int(np.prod(cfg["n_cells"]))
    B_alg, s_state, s = bytes_alg_per_particle_step(args.form, n / ncell_all, len(cfg["n_cells"]))
    ncell = int(np.prod(cfg["n_cells"]))
    kernel_bytes = n * s_state + ncell * 9 * s  # state read+write; gather E,B_m and J write per cell
    t_kernel = float(np.mean(t_part)) / 1e3
    peak, peak_kind = measured_peak()
    value = whole_job_rate(n, world, args.steps, ms)
    return dict(n=n, ms=ms, value=value, wall_ms_per_step=(wall1 - wall0) * 1e3 / args.steps, e2e=e2e,
                kernel_bytes=kernel_bytes, t_kernel=t_kernel, peak=peak, peak_kind=peak_kind, B_alg=B_alg,
                launches=launches, clocks=clk.summary(), energy=(uk0, ue0, uk1, ue1), cfg=cfg, tile=tile,
                tuning=tuning, relayouts=relayouts, fp64=fp64, queue=bool(queue), tma=tma, batched=batched,
                residual=None if res0 is None else {"after_poisson": res0, "after_steps": res1,
                                                    "poisson_iterations": poisson[0]})


COMPARE_FIELDS = ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Jx", "Jy", "Jz"]
# r.r / n of the initial Poisson solve: far below the reference's default 1e-14, so that the
# charge residual after the steps measures the steps, not the start
POISSON_MAX_ERROR = 1e-24


def rel_l2(a_list, b_list):
    """sqrt(sum |a - b|^2 / sum |b|^2) over a group of arrays (b the FP64 run)."""
    num = sum(float(np.sum((a - b) ** 2)) for a, b in zip(a_list, b_list))
    den = sum(float(np.sum(b ** 2)) for b in b_list)
    return (num / den) ** 0.5 if den > 0 else num ** 0.5


def run_fp64_compare(args, cfg, rank, device, stream, fields_mixed, utot_mixed):
    """The plain FP64 form on the same seeded plasma, the same number of steps: its
    throughput (the mixed form's target is 2x it) and the mixed run's errors against it
    (relative L2 of E, B and J after the steps, energy drift, charge residual)."""
    import torch
    from smilei_gb300 import simulation, _lib
    sim = simulation.Simulation(cfg["n_cells"], cfg["cell_length"], cfg["dt"], form="fp64", use_graph=True,
                                capacity_slack=args.slack)
    _lib.check(_lib.lib().sg_sim_set_stream(sim._h, stream.cuda_stream), "set_stream")
    n = add_plasma(sim, cfg, args.seed + rank, device)
    torch.cuda.empty_cache()
    if args.poisson:
        sim.solve_poisson(max_error=POISSON_MAX_ERROR)
    uk0, ue0 = sim.energy()
    for _ in range(args.warmup):
        sim.step(1)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        sim.step(1)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    uk1, ue1 = sim.energy()
    res1 = sim.charge_residual() if args.poisson else None
    f64 = {k: sim.get_field(k) for k in COMPARE_FIELDS}
    sim.close()
    err = {"E_rel_l2": rel_l2([fields_mixed[k] for k in COMPARE_FIELDS[:3]], [f64[k] for k in COMPARE_FIELDS[:3]]),
           "B_rel_l2": rel_l2([fields_mixed[k] for k in COMPARE_FIELDS[3:6]], [f64[k] for k in COMPARE_FIELDS[3:6]]),
           "J_rel_l2": rel_l2([fields_mixed[k] for k in COMPARE_FIELDS[6:]], [f64[k] for k in COMPARE_FIELDS[6:]]),
           "energy_drift_mixed": (utot_mixed[1] - utot_mixed[0]) / utot_mixed[0],
           "energy_drift_fp64": (uk1 + ue1 - uk0 - ue0) / (uk0 + ue0),
           "energy_mixed_vs_fp64": (utot_mixed[1] - (uk1 + ue1)) / (uk1 + ue1),
           "charge_residual_fp64": res1}
    return {"value": n * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps, "steps": args.steps,
            "warmup": args.warmup, "errors": err}


LWFA = dict(n_cells=[3840, 512], cell_length=[0.1, 1.5], dt=0.095, ppc=4, pusher="vay", n0=0.003, ramp=100.0,
            a0=2.0, waist=30.0, t_fwhm=60.0, shift=32)


def lwfa_t_start():
    """The window starts once the pulse has entered: 2 x its envelope centre sqrt(2) x FWHM."""
    return 2.0 * 2 ** 0.5 * LWFA["t_fwhm"]


def run_gpu_lwfa(args, rank, world, local_rank):
    """2D laser wakefield with a moving window: the Gaussian pulse is injected from xmin,
    the window starts moving at c once the pulse is in (laser then off, as in the
    reference), and the timed steps run with the window moving and plasma injected."""
    import torch
    from smilei_gb300 import simulation, _lib
    device = f"cuda:{local_rank}"
    torch.cuda.set_device(local_rank)
    stream = torch.cuda.Stream(device=device)
    torch.cuda.set_stream(stream)
    c = LWFA

    def make(tile):
        sm = simulation.Simulation(c["n_cells"], c["cell_length"], c["dt"], form=args.form,
                                   boundaries=("open", "open"), tile=list(tile) if tile else None, use_graph=True,
                                   capacity_slack=args.slack)
        _lib.check(_lib.lib().sg_sim_set_stream(sm._h, stream.cuda_stream), "set_stream")
        ly = c["n_cells"][1] * c["cell_length"][1]
        sm.add_laser_gaussian2d(a0=c["a0"], waist=c["waist"], focus=[0.0, ly / 2], t_fwhm=c["t_fwhm"])
        sm.add_species(1.0, -1.0, c["pusher"], np.zeros((2, 0)), np.zeros((3, 0)), np.zeros(0))
        sm.set_species_profile(0, c["n0"], c["ppc"], x_vacuum=0.0, x_slope1=c["ramp"])
        sm.fill_species(0)
        return sm

    # 8x16 tiles unless asked otherwise: the autotuner's pick for this workload
    tile, tuning = ([args.tile] * 2 if args.tile else [8, 16]), None
    if args.autotune:
        from smilei_gb300 import autotune
        best, times = autotune.tune_tiles(make, ndim=2)
        tile, tuning = list(best), {"x".join(map(str, k)): round(v, 3) for k, v in times.items()}
    sim = make(tile)
    t_start = lwfa_t_start()
    sim.set_moving_window(t_start, 1.0, c["shift"])
    # untimed: run until the window moves (or --preroll-steps, for small profiling runs), then the warm-up steps
    pre = int(np.ceil(t_start / c["dt"])) + 1 if args.preroll_steps < 0 else args.preroll_steps
    sim.step(pre)
    for _ in range(args.warmup):
        sim.step(1)
    torch.cuda.synchronize()
    n0 = sim.species_count(0)
    t_part, counts = [], []
    with ClockSampler(local_rank) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        wall0 = time.perf_counter()
        ev0.record(stream)
        for _ in range(args.steps):
            counts.append(sim.species_count(0))
            sim.step(1)
            tp, tf, tt, launches = sim.last_timing()
            t_part.append(tp)
        ev1.record(stream)
        torch.cuda.synchronize()
        wall1 = time.perf_counter()
    ms = max_over_ranks(ev0.elapsed_time(ev1), device)
    n_moved, x_moved, shifts = sim.window_state()
    relayouts = sim.layout_stats()
    particle_steps = float(sum(counts))
    nb0 = sim.species_count(0)
    bms, nb = time_batched(sim, args.steps, stream, device)
    nb_mean = 0.5 * (nb0 + sim.species_count(0))
    batched = {"ms_per_step": bms, "value": nb_mean * world / (bms / 1e3), "steps": args.steps, "graphs": nb}
    sim.close()
    ncell = int(np.prod(c["n_cells"]))
    s_state = 52.0 if args.form == "mixed" else 88.0
    s = 4 if args.form == "mixed" else 8
    n_mean = particle_steps / args.steps
    kernel_bytes = n_mean * s_state + ncell * 9 * s
    t_kernel = float(np.mean(t_part)) / 1e3
    peak, peak_kind = measured_peak()
    return dict(n=int(round(n_mean)), ms=ms, value=particle_steps * world / (ms / 1e3),
                wall_ms_per_step=(wall1 - wall0) * 1e3 / args.steps, kernel_bytes=kernel_bytes, t_kernel=t_kernel,
                peak=peak, peak_kind=peak_kind, B_alg=s_state + 24 * s / c["ppc"], launches=launches,
                clocks=clk.summary(), window=dict(n_moved=n_moved, x_moved=x_moved, shifts=shifts, pre_steps=pre,
                                                  particles_at_start=n0),
                cfg=c, energy=None, tile=tile or "default 8x8", tuning=tuning, relayouts=relayouts, batched=batched,
                e2e=None, e2e_note="not measured for this workload: the state size changes at every window shift")


def run_cpu_sample_lwfa(args):
    """The oracle's 2D open-boundary step with the moving window on a bounded sample: the
    first 1920 x 256 cells of the workload (same cell size, density ramp, 4 ppc), window moving."""
    import oracle
    c = LWFA
    n_cells = [1920, 256]
    O = oracle.Oracle()
    prof = (c["n0"], 0.0, c["ramp"], 1e300, 0.0)
    pos, mom, w = O.create_particles(n_cells, c["cell_length"], 0, n_cells[0], 0, prof, c["ppc"])
    sp = [dict(pos=pos, mom=mom, weight=w, charge=np.full(w.shape, -1, np.int16), mass=1.0, pusher="vay")]
    from smilei_gb300 import synthetic
    st = synthetic.STAGGER
    fields = {k: np.zeros(tuple(n_cells[d] + 5 + st[k.replace("_m", "")][d] for d in range(2)))
              for k in ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Bx_m", "By_m", "Bz_m", "Jx", "Jy", "Jz"]}
    win = dict(t_start=0.0, velocity=1.0, shift=c["shift"])
    steps = args.cpu_steps * 3
    state = {}
    O.run_window(n_cells, c["cell_length"], c["dt"], fields, sp, (False, False), 1, win,
                 profiles=[(prof, c["ppc"], 0.0, 0)], state=state)
    t0 = time.perf_counter()
    npart = 0
    for _ in range(steps):
        npart += sp[0]["weight"].size
        O.run_window(n_cells, c["cell_length"], c["dt"], fields, sp, (False, False), 1, win,
                     profiles=[(prof, c["ppc"], 0.0, 0)], state=state)
    t1 = time.perf_counter()
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return dict(value=npart / (t1 - t0), unit=UNIT, cores=cores, kind="port", steps=steps, warmup=1,
                ms_per_step=(t1 - t0) * 1e3 / steps,
                sample=f"2D wakefield sample 1920x256 cells x 4 ppc ({w.size} electrons), Vay, window moving, "
                       f"{steps} FP64 steps of oracle/bc_oracle.c + pic_oracle.c")


RAD = dict(n_cells=[2048, 512], ppw=16, npart=10_000_000, gamma=2000.0, sigma_wavelengths=2.0, a0=100.0)


def rad_setup(n_cells, npart, seed):
    """Head-on collision: a Gaussian electron bunch (gamma 2000, sigma_x = sigma_y = 2 lambda)
    moving towards -x through a plane wave of a0 = 100 moving towards +x; 16 cells per
    wavelength (lambda = 2 pi), dt = 0.95 CFL."""
    lam = 2.0 * np.pi
    dx = lam / RAD["ppw"]
    dt = 0.95 / np.sqrt(2.0 / dx ** 2)
    rng = np.random.default_rng(seed)
    L = [n_cells[0] * dx, n_cells[1] * dx]
    sig = RAD["sigma_wavelengths"] * lam
    pos = np.stack([np.clip(rng.normal(L[0] / 2, sig, npart), 4 * dx, L[0] - 4 * dx),
                    np.clip(rng.normal(L[1] / 2, sig, npart), 4 * dx, L[1] - 4 * dx)])
    p0 = np.sqrt(RAD["gamma"] ** 2 - 1.0)
    mom = np.stack([np.full(npart, -p0), np.zeros(npart), np.zeros(npart)])
    return dict(dx=dx, dt=dt, pos=np.ascontiguousarray(pos), mom=np.ascontiguousarray(mom),
                w=np.ones(npart), lam=lam)


def plane_wave(shape_fn, n_cells, dx, a0):
    """Ey = Bz = a0 sin(k x) on their own staggered x positions (a wave moving towards +x)."""
    out = {}
    for comp, stag_x in (("Ey", 0), ("Bz", 1)):
        shp = shape_fn(comp)
        x = (np.arange(shp[0]) - 2 - 0.5 * stag_x) * dx
        out[comp] = np.repeat((a0 * np.sin(x))[:, None], shp[1], axis=1)
    return out


def run_gpu_radiation(args, rank, world, local_rank):
    """Monte-Carlo radiation reaction in the PIC loop through the drop-in operators (FP64):
    per step interpolate, radiate (RadiationMonteCarlo), push (Vay), deposit (Esirkepov),
    then B save, Ampere, Faraday, B centring, in the order of Species::dynamics.  Photon
    chi from the table, or from the MLP where its validation passed (--mlp)."""
    import torch
    from smilei_gb300 import operators as O, radiation as R, _lib
    device = f"cuda:{local_rank}"
    torch.cuda.set_device(local_rank)
    n_cells = RAD["n_cells"]
    st = rad_setup(n_cells, RAD["npart"], args.seed + rank)
    geom = O.PatchGeometry(n_cells, [st["dx"], st["dx"]])
    EM = O.ElectroMagn(geom, device=device)
    for comp, arr in plane_wave(geom.shape, n_cells, st["dx"], RAD["a0"]).items():
        getattr(EM, comp + "_").copy_(torch.as_tensor(arr, device=device))
    EM.Bz_m.copy_(EM.Bz_)
    cu = lambda a: torch.as_tensor(a, dtype=torch.float64, device=device).contiguous()
    P = O.Particles(cu(st["pos"]), cu(st["mom"]), cu(st["w"]), torch.full((RAD["npart"],), -1, device=device))
    del st["pos"], st["mom"]
    smpi = O.SmileiMPI(2, P.size(), device=device)
    tau = torch.full((P.size(),), -1.0, dtype=torch.float64, device=device)
    g = np.load(os.path.join(ROOT, "tests", "golden", "radiation.npz"))
    f_dn, f_cl, inv_es = R.normalised_factors(2.0 * np.pi * 299792458.0 / 1e-6)
    T = R.RadiationTables(g["integfochi"], g["integfochi_min"], g["integfochi_max"], g["xi_table"], g["xi_min"],
                          g["xi_max"], g["xi_axis1_min"], f_dn, f_cl, inv_es)
    if args.rad_math == "fp32":
        T.set_fp32_math(True)
    mlp, used = None, None
    if args.mlp:
        mlp = R.PhotonChiMLP(hidden=64, seed=3)
        for steps, lr in ((4000, 2e-3), (4000, 1e-3), (4000, 3e-4)):
            mlp.train(T, steps=steps, batch=8192, lr=lr)
        err, n_masked = mlp.validate(T, tol=0.05)
        used = f"{err.size - n_masked}/{err.size} (chi, xi) bins"
    dt = st["dt"]
    interp = O.Interpolator2D2Order(geom)
    push = O.PusherVay(dt, 1.0, 2)
    proj = O.Projector2D2Order(geom, dt)
    ma, mf = O.MA_Solver_norm(dt), O.MF_Solver_Yee(dt)
    acc = torch.zeros(2, dtype=torch.float64, device=device)
    stream = torch.cuda.current_stream()
    L = _lib.lib()

    def step(it):
        interp.fieldsWrapper(EM, P, smpi)
        _lib.check(L.sg_rad_monte_carlo(T._h, mlp._h if mlp is not None else None, P.size(), dt, 1.0, -1.0,
                                        P.momentum.data_ptr(), P.weight.data_ptr(), tau.data_ptr(), None,
                                        smpi.dynamics_Epart.data_ptr(), smpi.dynamics_Bpart.data_ptr(), 7, 0, it,
                                        acc.data_ptr(), acc.data_ptr() + 8, stream.cuda_stream), "monte_carlo")
        push(P, smpi)
        EM.restartRhoJ()
        proj.currentsAndDensityWrapper(EM, P, smpi)
        EM.saveMagneticFields()
        ma(EM)
        mf(EM)
        EM.centerMagneticFields()

    for it in range(args.warmup):
        step(it)
    torch.cuda.synchronize()
    acc.zero_()
    with ClockSampler(local_rank) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        wall0 = time.perf_counter()
        e0.record()
        for it in range(args.steps):
            step(args.warmup + it)
        e1.record()
        torch.cuda.synchronize()
        wall1 = time.perf_counter()
    ms = max_over_ranks(e0.elapsed_time(e1), device)
    radiated = float(acc[0].item())
    n_emit = int(acc[1:].view(torch.int64).item())
    n = P.size()
    # bytes the operator chain moves per particle-step (FP64): interpolate 88, radiate 120, push 138, deposit 82
    b_per = 88.0 + 120.0 + 138.0 + 82.0
    peak, peak_kind = measured_peak()
    value = whole_job_rate(n, world, args.steps, ms)
    if mlp is not None:
        mlp.close()
    return dict(n=n, ms=ms, value=value, wall_ms_per_step=(wall1 - wall0) * 1e3 / args.steps, clocks=clk.summary(),
                b_per=b_per, peak=peak, peak_kind=peak_kind, radiated=radiated, emissions=n_emit, mlp_used=used)


def run_gpu_radiation_resident(args, rank, world, local_rank):
    """The same collision in the resident 2D mixed-form step: FP32 push and deposit, the
    radiation pass of the species (FP32 arithmetic, table or network) before each push."""
    import torch
    from smilei_gb300 import simulation, radiation as R, _lib, synthetic
    device = f"cuda:{local_rank}"
    torch.cuda.set_device(local_rank)
    stream = torch.cuda.Stream(device=device)
    torch.cuda.set_stream(stream)
    n_cells = RAD["n_cells"]
    st = rad_setup(n_cells, RAD["npart"], args.seed + rank)
    stag = synthetic.STAGGER
    shape = lambda c: tuple(n_cells[d] + 5 + stag[c.replace("_m", "")][d] for d in range(2))
    wave = plane_wave(shape, n_cells, st["dx"], RAD["a0"])

    def make(tile, tables=None, net=None):
        sm = simulation.Simulation(n_cells, [st["dx"], st["dx"]], st["dt"], form="mixed", use_graph=True,
                                   tile=list(tile) if tile else None)
        _lib.check(_lib.lib().sg_sim_set_stream(sm._h, stream.cuda_stream), "set_stream")
        for comp in ("Ey", "Bz"):
            sm.set_field(comp, wave[comp])
        sm.set_field("Bz_m", wave["Bz"])
        sm.add_species(1.0, -1.0, "vay", st["pos"], st["mom"], st["w"])
        if tables is not None:
            sm.set_species_radiation(0, tables, net, seed=7)
        return sm

    g = np.load(os.path.join(ROOT, "tests", "golden", "radiation.npz"))
    f_dn, f_cl, inv_es = R.normalised_factors(2.0 * np.pi * 299792458.0 / 1e-6)
    T = R.RadiationTables(g["integfochi"], g["integfochi_min"], g["integfochi_max"], g["xi_table"], g["xi_min"],
                          g["xi_max"], g["xi_axis1_min"], f_dn, f_cl, inv_es)
    T.set_fp32_math(True)
    mlp, used = None, None
    if args.mlp:
        mlp = R.PhotonChiMLP(hidden=64, seed=3)
        for steps, lr in ((4000, 2e-3), (4000, 1e-3), (4000, 3e-4)):
            mlp.train(T, steps=steps, batch=8192, lr=lr)
        err, n_masked = mlp.validate(T, tol=0.05)
        used = f"{err.size - n_masked}/{err.size} (chi, xi) bins"
    tile, tuning = ([args.tile] * 2 if args.tile else None), None
    if args.autotune:
        from smilei_gb300 import autotune
        best, times = autotune.tune_tiles(lambda t: make(t, T, mlp), ndim=2)
        tile, tuning = list(best), {"x".join(map(str, k)): round(v, 3) for k, v in times.items()}
    sim = make(tile, T, mlp)
    del st["pos"], st["mom"]
    for _ in range(args.warmup):
        sim.step(1)
    torch.cuda.synchronize()
    r0, e0 = sim.radiation_stats(0)
    n = sim.species_count(0)
    t_part = []
    with ClockSampler(local_rank) as clk:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        wall0 = time.perf_counter()
        ev0.record(stream)
        for _ in range(args.steps):
            sim.step(1)
            tp, tf, tt, launches = sim.last_timing()
            t_part.append(tp)
        ev1.record(stream)
        torch.cuda.synchronize()
        wall1 = time.perf_counter()
    ms = max_over_ranks(ev0.elapsed_time(ev1), device)
    r1, e1 = sim.radiation_stats(0)
    sim.close()
    if mlp is not None:
        mlp.close()
    peak, peak_kind = measured_peak()
    return dict(n=n, ms=ms, value=whole_job_rate(n, world, args.steps, ms),
                wall_ms_per_step=(wall1 - wall0) * 1e3 / args.steps, clocks=clk.summary(),
                b_per=52.0 + 8.0 + 24 * 4 / (n / float(np.prod(n_cells))), peak=peak, peak_kind=peak_kind,
                radiated=r1 - r0, emissions=e1 - e0, mlp_used=used, launches=launches, tile=tile or "default 8x8",
                tuning=tuning)


def run_cpu_sample_radiation(args):
    """The oracle's interpolate, Monte-Carlo radiation, Vay push and deposit on a bounded
    sample: 200,000 electrons of the same bunch on a 512 x 128-cell grid (FP64)."""
    import oracle
    n_cells = [512, 128]
    st = rad_setup(n_cells, 200_000, args.seed)
    O = oracle.Oracle()
    from smilei_gb300 import synthetic
    stag = synthetic.STAGGER
    shape = lambda c: tuple(n_cells[d] + 5 + stag[c.replace("_m", "")][d] for d in range(2))
    f = {c: np.zeros(shape(c)) for c in ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Jx", "Jy", "Jz"]}
    f.update(plane_wave(shape, n_cells, st["dx"], RAD["a0"]))
    n_prim = [n + 5 for n in n_cells]
    dom = [-2, -2]
    cl = [st["dx"], st["dx"]]
    g = np.load(os.path.join(ROOT, "tests", "golden", "radiation.npz"))
    from smilei_gb300.radiation import normalised_factors
    f_dn, f_cl, inv_es = normalised_factors(2.0 * np.pi * 299792458.0 / 1e-6)
    Tc = oracle.RadTables.from_golden(g, factor_dNph_dt=f_dn, factor_classical=f_cl, inv_norm_E_schwinger=inv_es)
    pos, mom, w = st["pos"], st["mom"], st["w"]
    q = np.full(w.size, -1, np.int16)
    tau = np.full(w.size, -1.0)
    steps = max(2, args.cpu_steps)
    t0 = time.perf_counter()
    for it in range(steps):
        E, B, iold, delta = O.interpolate(2, n_prim, dom, cl, [f["Ex"], f["Ey"], f["Ez"], f["Bx"], f["By"], f["Bz"]],
                                          pos)
        oracle.rad_monte_carlo(Tc, st["dt"], 1.0, -1.0, mom, w, tau, E, B, seed=7, step=it)
        pos, mom, invgf = O.push("vay", 2, st["dt"], 1.0, pos, mom, q, E, B)
        J = [np.zeros_like(f["Jx"]), np.zeros_like(f["Jy"]), np.zeros_like(f["Jz"]), None]
        O.project(0, 2, n_prim, dom, cl, st["dt"], pos, mom, w, q, invgf, iold, delta, J)
    t1 = time.perf_counter()
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return dict(value=w.size * steps / (t1 - t0), unit=UNIT, cores=cores, kind="port", steps=steps, warmup=0,
                ms_per_step=(t1 - t0) * 1e3 / steps,
                sample=f"radiation sample: 200000 electrons (gamma 2000, a0 = 100 plane wave) on 512x128 cells, "
                       f"{steps} FP64 steps of interpolate + Monte-Carlo radiation + Vay push + Esirkepov "
                       f"(oracle/pic_oracle.c, rad_oracle.c; fields held fixed)")


def run_cpu_sample_2d(args, steps=None, warmup=1):
    """The oracle's FP64 2D timestep on the whole 2D thermal workload (electrons and protons,
    256 x 256 cells, 16 ppc each; all host cores)."""
    import oracle
    from smilei_gb300 import synthetic
    cfg = workload_cfg(args)
    n_cells, cl = cfg["n_cells"], cfg["cell_length"]
    sp = []
    for k, spc in enumerate(cfg["species"]):
        pos, mom, w = synthetic.thermal_plasma(n_cells, cl, cfg["ppc"], spc["sigma"], args.seed + 7919 * k)
        sp.append(dict(pos=pos, mom=mom, weight=w, charge=np.full(w.shape, int(spc["charge"]), np.int16),
                       mass=spc["mass"], pusher=cfg["pusher"]))
    fields = synthetic.periodic_em(args.seed, n_cells, 0.0, 0.0)
    O = oracle.Oracle()
    steps = steps or args.cpu_steps
    for _ in range(max(1, warmup)):
        O.pic_step(2, n_cells, 2, cl, cfg["dt"], fields, sp)
    t0 = time.perf_counter()
    for _ in range(steps):
        O.pic_step(2, n_cells, 2, cl, cfg["dt"], fields, sp)
    t1 = time.perf_counter()
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    npart = sum(s_["weight"].size for s_ in sp)
    return dict(value=npart * steps / (t1 - t0), unit=UNIT, cores=cores, kind="port", steps=steps,
                warmup=max(1, warmup), ms_per_step=(t1 - t0) * 1e3 / steps, particles=int(npart),
                cells=int(np.prod(n_cells)),
                sample=f"2D thermal 256x256 cells, electrons + protons x 16 ppc ({npart} particles), Boris, "
                       f"{steps} FP64 steps of oracle/pic_oracle.c (OpenMP)")


def run_cpu_sample(args, steps=None, warmup=1):
    """The oracle's FP64 timestep on a bounded sample of the workload (all host cores)."""
    import oracle
    n = args.cpu_cells
    dx = 0.1
    dt = 0.95 * dx / np.sqrt(3.0)
    from smilei_gb300 import synthetic
    if getattr(args, "workload", "thermal") == "thermal2d":
        return run_cpu_sample_2d(args, steps, warmup)
    if getattr(args, "workload", "thermal") == "uneven":
        # the same patch statistics on an n^3 grid cut into 8^3-cell patches
        pos, mom, w, _ = synthetic.uneven_plasma([n, n, n], [dx] * 3, [8, 8, 8], 8, 1.5, 64, np.sqrt(5.0 / 511.0),
                                                 args.seed)
        pusher, what = "boris", f"3D uneven patches {n}^3 cells in 8^3 patches"
    else:
        pos, mom, w = synthetic.thermal_plasma([n, n, n], [dx] * 3, args.ppc, SIGMA_10KEV, args.seed)
        pusher, what = "higueracary", f"3D thermal {n}^3 cells x {args.ppc} ppc"
    fields = synthetic.periodic_em(args.seed, [n, n, n], 0.0, 0.0)
    sp = [dict(pos=pos, mom=mom, weight=w, charge=np.full(w.shape, -1, np.int16), mass=1.0, pusher=pusher)]
    O = oracle.Oracle()
    steps = steps or args.cpu_steps
    for _ in range(max(1, warmup)):
        O.pic_step(3, [n] * 3, 2, [dx] * 3, dt, fields, sp)
    t0 = time.perf_counter()
    for _ in range(steps):
        O.pic_step(3, [n] * 3, 2, [dx] * 3, dt, fields, sp)
    t1 = time.perf_counter()
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    value = pos.shape[1] * steps / (t1 - t0)
    return dict(value=value, unit=UNIT, cores=cores, kind="port", steps=steps, warmup=max(1, warmup),
                ms_per_step=(t1 - t0) * 1e3 / steps, particles=int(pos.shape[1]), cells=n ** 3,
                sample=f"{what} ({pos.shape[1]} electrons), {pusher}, "
                       f"{steps} FP64 steps of oracle/pic_oracle.c (OpenMP)")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--cells", type=int, default=256)
    ap.add_argument("--ppc", type=int, default=8)
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--cpu-cells", type=int, default=0,
                    help="cells per dimension of the 3D CPU legs (default: the thermal workload's own 256; "
                         "a 64^3 sample for the uneven workload)")
    ap.add_argument("--no-poisson", dest="poisson", action="store_false",
                    help="thermal workloads: skip the initial FP64 Poisson solve (and the charge residual)")
    ap.add_argument("--no-compare-fp64", dest="compare_fp64", action="store_false",
                    help="3D thermal, mixed form: skip the FP64-form run on the same plasma")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--e2e-chunks", type=int, default=32,
                    help="tile ranges of the streamed host step (0: unpack, step, pack one after another)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="thermal", choices=["thermal", "thermal2d", "uneven", "lwfa", "radiation"])
    ap.add_argument("--mlp", action="store_true", help="radiation workload: photon chi from the trained MLP")
    ap.add_argument("--resident", action="store_true",
                    help="radiation workload: the resident mixed-form step instead of the drop-in operators")
    ap.add_argument("--rad-math", default="fp32", choices=["fp32", "fp64"],
                    help="radiation workload: arithmetic of the Monte-Carlo table lookups and draws")
    ap.add_argument("--autotune", action="store_true",
                    help="pick the tile shape (and, for the 3D and 2D thermal and uneven workloads, the tile "
                         "queue) by timing candidates first")
    ap.add_argument("--no-tma", action="store_true",
                    help="3D mixed form, 4x4x4 tiles: stage the field tile with word copies instead of the "
                         "tensor memory accelerator")
    ap.add_argument("--tile-queue", action="store_true",
                    help="particle kernel as a persistent grid draining a tile queue, densest tile first")
    ap.add_argument("--slack", type=float, default=0.25,
                    help="segment capacity slack: room per tile beyond its particle count, as a fraction")
    ap.add_argument("--preroll-steps", type=int, default=-1,
                    help="wakefield workload: untimed steps before the warm-up (default: until the window moves)")
    args = ap.parse_args()
    if args.cpu_cells <= 0:
        args.cpu_cells = args.cells if args.workload == "thermal" else 64
    # the uneven plasma is far from neutral patch by patch: a Poisson start would give it
    # fields that empty the dense patches, another workload than the batched-patch one
    if args.workload not in ("thermal", "thermal2d"):
        args.poisson = False

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload == "radiation":
        workload = ("2D Monte-Carlo radiation reaction: 2048x512 cells (16 per wavelength), 1e7 electrons gamma=2000 "
                    "in a Gaussian bunch (sigma_x = sigma_y = 2 lambda) head-on with a plane wave a0=100, Vay, " +
                    ("resident mixed-form step (FP32 push, deposit and Monte Carlo)" if args.resident else
                     "drop-in FP64 operators, Monte-Carlo lookups in " + args.rad_math) + ", photon chi from the " +
                    ("MLP (table where its validation failed)" if args.mlp else "table"))
    elif args.workload == "lwfa":
        c = LWFA
        workload = (f"2D laser wakefield with a moving window: {c['n_cells'][0]}x{c['n_cells'][1]} cells, dx=0.1, "
                    f"dy=1.5, dt=0.095, Gaussian laser a0=2 waist 30 FWHM 60 from xmin, electrons n=0.003 with a "
                    f"100-long ramp then plateau at 4 ppc (regular positions), Vay, window at c from "
                    f"t={lwfa_t_start():.1f} moving {c['shift']} cells per shift, Silver-Mueller on all sides")
    elif args.workload == "uneven":
        workload = ("3D uneven patches: 512x256x256 cells in 1024 patches of 32^3, particles per cell per patch "
                    "8*exp(N(0,1.5)) floored and clipped to [0,64], T=5 keV electrons, Boris, dt=0.95 CFL, periodic")
    elif args.workload == "thermal2d":
        workload = ("2D thermal plasma 256x256 cells, dx=dy=0.1, dt=0.95 CFL, periodic, electrons and protons "
                    "(mass 1836) at 16 ppc each (2097152 particles), T=10 keV, Boris")
    else:
        workload = (f"3D thermal plasma {args.cells}^3 cells, {args.ppc} ppc electrons "
                    f"({args.cells ** 3 * args.ppc} particles per GPU), Higuera-Cary, dt=0.95 CFL, periodic")

    if args.impl == "reference":
        if rank != 0:
            return
        # the 3D sample runs the requested warm-up and timed steps (each one FP64 step of the
        # bounded sample); the 2D samples keep their own bounded step counts
        r = (run_cpu_sample_lwfa(args) if args.workload == "lwfa" else
             run_cpu_sample_radiation(args) if args.workload == "radiation" else
             run_cpu_sample(args, steps=max(1, args.steps), warmup=args.warmup))
        line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
                "steps": r["steps"], "warmup": r["warmup"], "ms_per_step": r["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, host)",
                "config": {"workload": workload, "sample": r["sample"], "form": "fp64",
                           **({"global_particles": r["particles"], "cells": r["cells"]} if "particles" in r else {})},
                "cpu_baseline": r,
                "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch.distributed as td
        td.init_process_group("nccl")
    if args.workload == "radiation":
        res = (run_gpu_radiation_resident if args.resident else run_gpu_radiation)(args, rank, world, local_rank)
        cpu = None
        if rank == 0 and world == 1 and not args.no_cpu_baseline:
            cpu = run_cpu_sample_radiation(args)
        if rank == 0:
            achieved = res["b_per"] * res["value"] / 1e9
            print(json.dumps({
                "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": res["ms"] / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.resident else "f64",
                "data": "synthetic (seeded bunch, host)",
                "config": {"workload": workload, "form": "mixed, resident step" if args.resident else "fp64 operators",
                           "global_particles": res["n"] * world,
                           "wall_ms_per_step": res["wall_ms_per_step"], "radiated_energy": res["radiated"],
                           "emissions": res["emissions"], "mlp_used_on": res["mlp_used"],
                           "tile": res.get("tile"), "autotune_ms_per_step": res.get("tuning"),
                           "l2": "inputs larger than L2"},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": res["peak"], "unit": "GB/s",
                             "frac": achieved / res["peak"], "traffic": None,
                             "kernel": "resident step (radiation pass, particle kernel, fields)" if args.resident
                             else "operator chain",
                             "algorithmic_bytes_per_particle_step": res["b_per"],
                             "peak_source": res["peak_kind"]},
                "cpu_baseline": cpu, "e2e": None,
                "gpu_launches": res.get("launches", 9) * args.steps, "clocks": res["clocks"]}))
        if world > 1:
            import torch.distributed as td
            td.destroy_process_group()
        return
    if args.workload == "lwfa":
        res = run_gpu_lwfa(args, rank, world, local_rank)
    else:
        res = run_gpu(args, rank, world, local_rank)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = run_cpu_sample_lwfa(args) if args.workload == "lwfa" else run_cpu_sample(args)
        except Exception as e:  # the baseline is reported, not required
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {e}"}
    if rank != 0:
        if world > 1:
            import torch.distributed as td
            td.destroy_process_group()
        return
    achieved = res["kernel_bytes"] / res["t_kernel"] / 1e9
    tpp = NCU_TRAFFIC_BYTES_PER_PARTICLE.get(args.form)
    traffic = tpp * res["n"] if (tpp is not None and args.ppc == 8 and args.workload == "thermal") else None
    step_gbs = res["B_alg"] * res["value"] / 1e9
    line = {
        "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+i32" if args.form == "mixed" else "f64",
        "data": "synthetic (seeded Maxwellian, generated on device)",
        "config": {"workload": workload, "form": args.form, "global_particles": res["n"] * world,
                   "capacity_slack": args.slack,
                   "cells": int(np.prod(res["cfg"]["n_cells"])), "parallelism": f"replicas x{world}", "l2": "inputs larger than L2",
                   "B_alg_bytes_per_particle_step": res["B_alg"],
                   "hbm_fraction_of_step": step_gbs / res["peak"], "wall_ms_per_step": res["wall_ms_per_step"],
                   "energy_ukin_uelm_before_after": res["energy"], "tile": res["tile"] or "default 4x4x4",
                   "tile_queue": res.get("queue", False), "tma_staging": res.get("tma", False),
                   "autotune_ms_per_step": res["tuning"],
                   "relayouts_spilled_over_run": res["relayouts"],
                   "batched_steps": res.get("batched"),
                   **({"charge_residual": res["residual"]} if res.get("residual") else {}),
                   **({"fp64_value": res["fp64"]["value"], "fp64_ms_per_step": res["fp64"]["ms_per_step"],
                       "fp64_steps": res["fp64"]["steps"], "mixed_over_fp64": res["value"] / res["fp64"]["value"],
                       "errors_vs_fp64": res["fp64"]["errors"]} if res.get("fp64") else {}),
                   **({"window": res["window"], "e2e_note": res["e2e_note"]} if "window" in res else {})},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": res["peak"], "unit": "GB/s",
                     "frac": achieved / res["peak"], "traffic": traffic, "kernel": "k_step_particles",
                     "algorithmic_bytes_per_launch": res["kernel_bytes"], "peak_source": res["peak_kind"]},
        "cpu_baseline": cpu,
        "e2e": res["e2e"],
        "gpu_launches": res["launches"] * args.steps,
        "clocks": res["clocks"],
    }
    print(json.dumps(line))
    if world > 1:
        import torch.distributed as td
        td.destroy_process_group()


if __name__ == "__main__":
    main()
