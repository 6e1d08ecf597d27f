"""Autotuner for the batched choke-point engine.

Picks the grid (cells per axis of the shared world) and the threads per block
of the fused launches by timing a few batched steps of each candidate with
CUDA events (per-phase profiling of the batch's group).  The block size never
changes results; the grid does (it sets the reference's 3 x 3 neighbour-cell
box), so whatever is picked is applied identically to the per-scene runs it
is compared with.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from . import _lib
from .groups import Batch, set_block
from .scenario import StepParams
from .state import AgentState


@dataclass
class TuneResult:
    cells: int
    block: int
    ms_per_step: float
    trials: list


def batch_for(states, gaps, p: StepParams, walls_rows) -> Batch:
    b = Batch([s.n for s in states], p.k, p.world_cells, p.world_size, p.search_radius)
    for i, g in enumerate(gaps):
        b.set_walls(i, walls_rows(g))
    b.upload(AgentState.concat(states))
    return b


def step_ms(batch: Batch, p: StepParams, steps: int) -> float:
    """Average ms per step over `steps` steps (sum of the phase timings)."""
    _lib.call("gs_group_set_profiling", batch.group.handle, 1)
    batch.step(p, steps)
    ms = (C.c_float * 4)()
    n = (C.c_uint * 4)()
    _lib.call("gs_group_phase_times", batch.group.handle, ms, n, 4)
    _lib.call("gs_group_set_profiling", batch.group.handle, 0)
    return sum(ms) / steps


def tune_batched(states, gaps, base: StepParams, walls_rows, cell_sizes=(2.0, 2.5, 3.0, 4.0),
                 blocks=(128, 256), steps: int = 3, warmup: int = 2) -> TuneResult:
    """Times every (cell size, block) pair on the batch; cell sizes are
    rounded to a whole number of cells across the (square, 2D) world."""
    world = base.world_size[0]
    trials = []
    best = None
    for cs in cell_sizes:
        cells = max(1, int(round(world / cs)))
        p = base.replace(world_cells=(cells, 1, cells))
        b = batch_for(states, gaps, p, walls_rows)
        b.step(p, warmup)
        for blk in blocks:
            set_block(b.group, blk)
            b.step(p, 1)
            ms = step_ms(b, p, steps)
            trials.append({"cells": cells, "cell_size": world / cells, "block": blk, "ms": ms})
            if best is None or ms < best[2]:
                best = (cells, blk, ms)
        del b
    return TuneResult(cells=best[0], block=best[1], ms_per_step=best[2], trials=trials)
