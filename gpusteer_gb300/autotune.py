"""Autotuner for the batched engine.

Picks the cell size of the shared per-scene grid, the threads per block of
the fused launches, the candidate capacity of the fused KNN scan, the form
of the step (separate launches, or one persistent launch where that build
exists) and the number of parts (consecutive scene ranges, each a batch on
its own stream, stepped concurrently so the GPU overlaps one part's kernels
with another's) by timing a few batched steps of each candidate on the
actual scenes.  Block size, capacity, form and parts never change results.  The cell size does (it sets the
reference's 3 x 3 neighbour-cell box), so the tuner only tries cells at
least as large as the scenario's own, and whatever it picks is applied
identically to any per-scene run that is compared with the batch.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from .groups import Batch, set_block, set_knn_capacity, set_persistent
from .scenario import StepParams
from .state import AgentState


@dataclass
class TuneResult:
    params: StepParams   # the scenario's parameters with the chosen grid
    block: int
    capacity: int        # 0: chosen by the library from the crowd's density
    ms_per_step: float
    persistent: bool = False  # one persistent launch per step
    parts: int = 1            # batches (scene ranges) stepped concurrently
    trials: list = field(default_factory=list)


def batch_for(states, gaps, p: StepParams, walls_rows) -> Batch:
    """A batch of the given scenes on p's grid, state uploaded."""
    b = Batch([s.n for s in states], p.k, p.world_cells, p.world_size, p.search_radius)
    for i, g in enumerate(gaps):
        b.set_walls(i, walls_rows(g))
    b.upload(AgentState.concat(states))
    return b


def scene_cuts(states, parts: int):
    """(first, end) scene ranges, `parts` of them at most, of about equal
    agent counts."""
    n = sum(s.n for s in states)
    cum = np.cumsum([s.n for s in states])
    cuts = [0] + [int(np.searchsorted(cum, n * i / parts, side="right"))
                  for i in range(1, parts)] + [len(states)]
    cuts = sorted(set(cuts))
    return list(zip(cuts[:-1], cuts[1:]))


def batch_parts(states, gaps, p: StepParams, walls_rows, parts: int) -> list:
    """The scenes as `parts` batches (scene_cuts), each on its own stream."""
    return [batch_for(states[lo:hi], gaps[lo:hi], p, walls_rows)
            for lo, hi in scene_cuts(states, parts)]


def configure(batch: Batch, tr: "TuneResult", capacity: int | None = None) -> None:
    """Applies a tuning result's block, capacity and form to a batch."""
    set_block(batch.group, tr.block)
    set_knn_capacity(batch.group, tr.capacity if capacity is None else capacity)
    set_persistent(batch.group, tr.persistent)


def time_parts(parts: list, p: StepParams, steps: int) -> float:
    """Host wall-clock ms per step of all parts, each part's steps queued on
    its own stream, every stream synchronised on both sides."""
    for b in parts:
        b.group.synchronize()
    t0 = time.perf_counter()
    for b in parts:
        b.step(p, steps)
    for b in parts:
        b.group.synchronize()
    return (time.perf_counter() - t0) * 1e3 / steps


def time_steps(batch: Batch, p: StepParams, steps: int) -> float:
    """Host wall-clock ms per step over `steps` steps, stream synchronised on
    both sides (graph replay after the first step of a configuration)."""
    batch.group.synchronize()
    t0 = time.perf_counter()
    batch.step(p, steps)
    batch.group.synchronize()
    return (time.perf_counter() - t0) * 1e3 / steps


def grid_for(base: StepParams, cell: float) -> StepParams:
    """base with square 2D cells of side `cell` (rounded to whole cells)."""
    wx, _, wz = base.world_size
    cx = max(1, int(round(wx / cell)))
    cz = max(1, int(round(wz / cell)))
    return base.replace(world_cells=(cx, base.world_cells[1], cz))


def tune_batched(states, gaps, base: StepParams, walls_rows, cell_scales=(1.0, 1.25, 1.5),
                 blocks=(128, 256), capacities=(0, 256), part_counts=(1, 2, 3, 4), steps: int = 4,
                 warmup: int = 2) -> TuneResult:
    """Times every (cell size, block, capacity, form) on the batch; cell
    sizes are the scenario's cell times `cell_scales` (all >= 1).  The
    persistent form runs 256-thread blocks, so it is tried with those.  The
    best of those is then timed on fresh batches split into each of
    `part_counts` parts, from the same initial state (the crowds' density,
    and so the step time, changes over a run)."""
    cell0 = base.world_size[0] / base.world_cells[0]
    trials, best = [], None
    for scale in cell_scales:
        if scale < 1.0:
            raise ValueError("cells smaller than the scenario's change its neighbourhoods")
        p = grid_for(base, cell0 * scale)
        b = batch_for(states, gaps, p, walls_rows)
        b.step(p, warmup)
        for blk in blocks:
            for cap in capacities:
                for pers in ((False, True) if blk == 256 else (False,)):
                    set_block(b.group, blk)
                    set_knn_capacity(b.group, cap)
                    set_persistent(b.group, pers)
                    b.step(p, 1)  # new configuration: eager step and graph capture
                    ms = time_steps(b, p, steps)
                    trials.append({"cell": cell0 * scale, "cells": list(p.world_cells),
                                   "block": blk, "capacity": cap, "persistent": pers, "ms": ms})
                    if best is None or ms < best.ms_per_step:
                        best = TuneResult(params=p, block=blk, capacity=cap, ms_per_step=ms,
                                          persistent=pers)
        del b
    best_parts = None
    for parts in part_counts:
        if parts < 1 or parts > len(states):
            continue
        bs = batch_parts(states, gaps, best.params, walls_rows, parts)
        for b in bs:
            configure(b, best)
            b.step(best.params, warmup)
        ms = time_parts(bs, best.params, steps)
        trials.append({"cell": best.params.world_size[0] / best.params.world_cells[0],
                       "block": best.block, "capacity": best.capacity,
                       "persistent": best.persistent, "parts": len(bs), "ms": ms})
        if best_parts is None or ms < best_parts[1]:
            best_parts = (len(bs), ms)
        del bs
    if best_parts is not None:
        best.parts = best_parts[0]
    best.trials = trials
    return best
