"""FP32 trajectories against an FP64 rerun of the same scenario.

The GPU path is bit-identical to the FP32 oracle (the GPU parity tests), so
the oracle's FP32 run stands for it here; orc_run_d is the same restatement
in binary64 (its KNN also in binary64).  Run as a script to print the
divergence table for the boids (4,096 agents, k = 7) and choke-point
(10,000 agents, k = 16) configurations over 100 steps."""
import sys
from pathlib import Path

import numpy as np

if __name__ == "__main__":  # run as a script from anywhere
    here = Path(__file__).resolve().parent
    sys.path[:0] = [str(here.parent), str(here)]

import oracle_lib as ol  # noqa: E402
from gpusteer_gb300 import scenario as sc  # noqa: E402
from gpusteer_gb300.state import AgentState  # noqa: E402


def as64(s: AgentState) -> AgentState:
    out = {}
    for k in AgentState.names():
        a = getattr(s, k)
        out[k] = np.ascontiguousarray(a.astype(np.float64) if a.dtype == np.float32 else a)
    return AgentState(**out)


def divergence(name, steps=100, marks=(1, 10, 50, 100)):
    if name == "boids":
        s = sc.boids_sphere(4096, seed=0)
        p = sc.boids_params(k=7)
        walls = None
    else:
        s = sc.chokepoint_agents(10000, seed=0)
        s.speed[:] = np.float32(0.5)  # a defined heading from the first step
        p = sc.chokepoint_params()
        walls = ol.split_walls(*sc.walls_from_rows(sc.chokepoint_walls(10.0)), p.world_size,
                               p.world_cells)
    a, b = s.copy(), as64(s)
    rows, done = [], 0
    for m in marks:
        ol.run(a, p, m - done, walls=walls)
        ol.run_d(b, p, m - done, walls=walls)
        done = m
        d = np.linalg.norm(a.position[:, :3].astype(np.float64) - b.position[:, :3], axis=1)
        rows.append((m, float(np.median(d)), float(np.percentile(d, 99)), float(d.max()),
                     float(np.mean(d > 1e-3))))
    return rows


def test_first_step_agrees_with_fp64_within_1e5():
    """One step: FP32 state within 1e-5 (relative to the world's scale) of
    the FP64 rerun for every agent."""
    for name in ("boids", "chokepoint"):
        rows = divergence(name, marks=(1,))
        assert rows[0][3] < 1e-5 * 100.0, (name, rows)


if __name__ == "__main__":
    for name in ("boids", "chokepoint"):
        print(f"{name}: step, median |dp|, p99 |dp|, max |dp|, fraction > 1e-3")
        for r in divergence(name):
            print("  %4d  %.3e  %.3e  %.3e  %.4f" % r)
        sys.stdout.flush()
