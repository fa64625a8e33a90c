"""Autotuner for the resident step: tile (bin) shape and how tiles reach the CTAs.

The tile shape decides the work of one CTA of the particle kernel: the field and
current tiles it stages, the cells the per-cell deposit walks, and how a dense
region is cut into work items.  The tiles reach the CTAs either one CTA per tile
through the hardware block scheduler, or through a device queue that a persistent
grid drains, densest tile first (Simulation.set_tile_queue).  A 4x4x4 tile of the 3D
mixed form stages its fields by TMA or by word copies (Simulation.set_tma_staging).  The best choice
depends on the density and its spread, so it is measured: every candidate builds
the same simulation, runs a few warm-up steps and a few timed steps (CUDA events
on the simulation's stream), and the fastest is kept.  Candidates whose shape does
not divide the grid are adjusted by the library exactly as a user's choice would be.
"""
from __future__ import annotations

import time

# 3D shapes of at most 64 cells (the per-cell deposit's limit with two thread
# groups per cell) and 2D shapes of at most 128 cells.
CANDIDATES_3D = [(4, 4, 4), (2, 4, 8), (8, 4, 2), (4, 4, 2), (4, 2, 4)]
CANDIDATES_2D = [(8, 8), (4, 16), (16, 4), (8, 16), (4, 8), (4, 4)]


def tune_tiles(build, candidates=None, ndim=3, warmup=2, steps=3, log=None):
    """build(tile) -> Simulation with its particles added (closed here after timing).

    Returns (best_tile, {tile: mean step ms})."""
    import torch
    cands = candidates or (CANDIDATES_3D if ndim == 3 else CANDIDATES_2D)
    times = {}
    for tile in cands:
        t0 = time.perf_counter()
        sim = build(tuple(tile))
        try:
            for _ in range(warmup):
                sim.step(1)
            torch.cuda.synchronize()
            ms = []
            for _ in range(steps):
                sim.step(1)
                ms.append(sim.last_timing()[2])
            times[tuple(tile)] = sum(ms) / len(ms)
        finally:
            sim.close()
            torch.cuda.empty_cache()
        if log:
            log(f"tile {tile}: {times[tuple(tile)]:.3f} ms/step (trial {time.perf_counter() - t0:.1f} s)")
    best = min(times, key=times.get)
    return best, times


def tune(build, ndim=3, tiles=None, queues=(False, True), stagings=(True, False), warmup=2, steps=3, log=None):
    """Every (tile shape, tile queue, TMA staging) triple: build(tile) -> Simulation, then
    the queue and staging settings, timed as in tune_tiles.  TMA staging is tried only
    where the simulation accepts it (3D mixed form, 4x4x4 periodic tiles); elsewhere the
    word copies.  Returns ((best_tile, best_queue, best_tma), {(tile, queue, tma): ms})."""
    import torch
    from ._lib import SmileiGPUError
    cands = tiles or (CANDIDATES_3D if ndim == 3 else CANDIDATES_2D)
    times = {}
    for tile in cands:
        for q in queues:
            for tma in stagings:
                t0 = time.perf_counter()
                sim = build(tuple(tile))
                try:
                    try:
                        sim.set_tma_staging(tma)
                    except SmileiGPUError:
                        continue  # this simulation stages by word copies only
                    sim.set_tile_queue(q)
                    for _ in range(warmup):
                        sim.step(1)
                    torch.cuda.synchronize()
                    ms = []
                    for _ in range(steps):
                        sim.step(1)
                        ms.append(sim.last_timing()[2])
                    times[(tuple(tile), bool(q), bool(tma))] = sum(ms) / len(ms)
                finally:
                    sim.close()
                    torch.cuda.empty_cache()
                if log:
                    log(f"tile {tile} queue {q} tma {tma}: {times[(tuple(tile), bool(q), bool(tma))]:.3f} ms/step "
                        f"(trial {time.perf_counter() - t0:.1f} s)")
    best = min(times, key=times.get)
    return best, times
