"""Autotuner for the batched engine.

Picks the cell size of the shared per-scene grid, the threads per block of
the fused launches, the candidate capacity of the fused KNN scan and the
form of the step (separate launches, or one persistent launch where that
build exists) by timing a few batched steps of each candidate on the
actual scenes.  Block size, capacity and form never change results.  The cell size does (it sets the
reference's 3 x 3 neighbour-cell box), so the tuner only tries cells at
least as large as the scenario's own, and whatever it picks is applied
identically to any per-scene run that is compared with the batch.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

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
    trials: list = field(default_factory=list)


def batch_for(states, gaps, p: StepParams, walls_rows) -> Batch:
    """A batch of the given scenes on p's grid, state uploaded."""
    b = Batch([s.n for s in states], p.k, p.world_cells, p.world_size, p.search_radius)
    for i, g in enumerate(gaps):
        b.set_walls(i, walls_rows(g))
    b.upload(AgentState.concat(states))
    return b


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
                 blocks=(128, 256), capacities=(0, 256), steps: int = 4,
                 warmup: int = 2) -> TuneResult:
    """Times every (cell size, block, capacity, form) on the batch; cell
    sizes are the scenario's cell times `cell_scales` (all >= 1).  The
    persistent form runs 256-thread blocks, so it is tried with those."""
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
    best.trials = trials
    return best
