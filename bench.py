"""Throughput benchmark of the per-step agent update on GB300.

Default workload (the headline): 256 independent 2D choke-point scenes
advanced together, one CUDA-graph replay per step (gs_batch_step), against
the same 256 scenes stepped one gs_step call per scene.  Gap half-widths are
drawn from {7.5, 10, ..., 32.5}, agent counts uniformly from [1,000, 20,000];
k = 16, walls k = 3, cell size and block shape from the autotuner, FP32.

Other workloads: `large` (1,048,576 3D boids in a 512^3 cube, k = 16, cell
4.0), `chokepoint` (one 10,000-agent scene), `boids` (4,096 boids, k = 7).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gs|reference]
                  [--workload batched|large|chokepoint|boids]

Prints one JSON line (rank 0).  `value` is whole-job agent-steps/s with the
state resident in HBM, timed with CUDA events on the engine's stream; `e2e`
is the same metric through the upload / step / download calls with the
state copied from and back to page-locked host memory every step.  Under
torchrun every rank runs an independent replica on its own GPU (scenes and
flocks are not split across GPUs: replicas only).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

WORKLOADS = {
    # name: (description, n, builder)
    "large": "large plain flock: 1,048,576 3D boids in a 512^3 cube, k=16, cell 4.0",
    "chokepoint": "2D choke point: 10,000 agents, gap half-width 10, k=16, knw=3, cell 2.0",
    "boids": "plain 3D flock: 4,096 boids in a sphere of radius 50, k=7, cell 4.0",
    "brute": "brute-force KNN: 65,536 agents uniform in a 512^3 cube, k=16, FP32 (one query "
             "per agent against all agents)",
    "batched": "256 independent 2D choke-point scenes (gap half-widths 7.5..32.5, 1,000-20,000 "
               "agents each), k=16, knw=3, 512x512 world per scene, cell size (2.0 or larger), "
               "block shape and KNN capacity from the autotuner",
}


def make_workload(name):
    from gpusteer_gb300 import scenario as sc

    if name == "large":
        s = sc.boids_cube(1 << 20, size=512.0, seed=0)
        p = sc.boids_params(k=16, world=512.0, cell=4.0)
        return s, p, None
    if name == "chokepoint":
        s = sc.chokepoint_agents(10000, seed=0)
        p = sc.chokepoint_params()
        return s, p, sc.chokepoint_walls(10.0)
    if name == "boids":
        return sc.boids_sphere(4096, seed=0), sc.boids_params(k=7), None
    raise SystemExit(f"unknown workload {name}")


def make_batched(n_scenes=256, seed=0):
    """(states, gaps, params, walls_rows(gap)) of the batched workload."""
    from gpusteer_gb300 import scenario as sc

    states, gaps = sc.batched_chokepoint(n_scenes, seed=seed)
    return states, gaps, sc.chokepoint_params(), sc.chokepoint_walls


def batched_config(p, scenes: int, n: int, world: int) -> dict:
    """The batched workload's config, as both arms print it."""
    return {"workload": WORKLOADS["batched"] if scenes == 256 else
            WORKLOADS["batched"].replace("256", str(scenes), 1),
            "scenes": scenes, "agents": n, "k": p.k, "knw": p.knw,
            "cell": p.world_size[0] / p.world_cells[0],
            "cells_per_scene": int(np.prod(p.world_cells)),
            "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (about 270 MB of bucketed state per step)"}


def single_config(name: str, p, n: int, world: int) -> dict:
    """A single-group workload's config, as both arms print it."""
    cfg = {"workload": WORKLOADS[name], "agents": n, "k": p.k,
           "cell": p.world_size[0] / p.world_cells[0], "cells": int(np.prod(p.world_cells)),
           "parallelism": f"replicas x{world}"}
    if name == "large":
        cfg["l2"] = "inputs larger than L2 (about 200 MB of bucketed state per step)"
    return cfg


def brute_config(n: int, k: int, world: int) -> dict:
    return {"workload": WORKLOADS["brute"], "agents": n, "k": k,
            "parallelism": f"replicas x{world}",
            "l2": "1 MB of positions, L2-resident by design (compute-bound)"}


def fused_bytes_per_agent(p) -> int:
    """Algorithmic DRAM bytes of the dominant fused kernel(s) per agent: its own
    bucketed state read once (5 float4 = 80 B), the new state written once
    (80 B) and the next step's (cell, rank) pair (8 B).  Neighbour and
    candidate reads hit the same bucketed arrays and are counted once.  With
    avoid-walls the step is split in two launches that also write and read
    the wall-phase state (3 float4) and the neighbour slots (4 B each; plus
    the KNN distances, 4 B each, when avoid-close-neighbours needs them)."""
    from gpusteer_gb300 import scenario as sc

    if sc.B_AVOID_WALLS in p.order:
        lists = 4 * p.k * (2 if (sc.B_AVOID_NEIGHBORS in p.order and p.avoid_close) else 1)
        walls_half = 80 + lists + 48
        rest_half = 48 + 48 + lists + 80 + 8
        return walls_half + rest_half
    return 80 + 80 + 8


def step_model_bytes(n, k, cells) -> int:
    """Whole-step bytes of the reference decomposition (bin rebuild + KNN +
    steering): (216 + 12k) N + 8 C."""
    return (216 + 12 * k) * n + 8 * cells


# ---- clocks ------------------------------------------------------------------------

REASON_BITS = {
    0x1: "gpu_idle", 0x2: "applications_clocks_setting", 0x4: "sw_power_cap",
    0x8: "hw_slowdown", 0x10: "sync_boost", 0x20: "sw_thermal_slowdown",
    0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown",
    0x100: "display_clock_setting",
}


class ClockSampler:
    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if not self.lines:
                # a timed region shorter than the sampling period: one reading
                # right after it
                try:
                    out = subprocess.run(
                        ["nvidia-smi", "-i", str(self.index),
                         "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active",
                         "--format=csv,noheader,nounits"],
                        capture_output=True, text=True, timeout=10).stdout
                    self.lines = [ln.strip() for ln in out.splitlines() if ln.strip()]
                    self.after = True
                except (OSError, subprocess.TimeoutExpired):
                    pass

    def summary(self):
        sm, mx, reasons = [], [], set()
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 4:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
                bits = int(parts[3], 16) if parts[3].startswith("0x") else int(parts[3])
            except ValueError:
                continue
            for b, name in REASON_BITS.items():
                if bits & b and name not in ("gpu_idle",):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
               "samples": len(sm)}
        if getattr(self, "after", False):
            out["sampled"] = "once, right after the timed region (shorter than the 200 ms period)"
        return out


# ---- distributed plumbing ---------------------------------------------------------

def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1, 0
    import torch.distributed as dist

    dist.init_process_group("gloo")
    return dist, dist.get_rank(), ws, int(os.environ.get("LOCAL_RANK", "0"))


def allreduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ---- CPU legs (oracle) -------------------------------------------------------------

def cpu_sample(state, p, walls_rows, seconds: float):
    """Times the CPU oracle on the workload (all host threads), stepping until
    about `seconds` have elapsed; returns (agent-steps/s, steps, threads, n)."""
    sys.path.insert(0, str(REPO / "tests"))
    import oracle_lib as ol
    from gpusteer_gb300 import scenario as sc

    s = state.copy()
    walls = None
    if walls_rows is not None:
        walls = ol.split_walls(*sc.walls_from_rows(walls_rows), p.world_size, p.world_cells)
    threads = ol.threads_available()
    ol.run(s, p, 1, walls=walls, threads=threads)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while True:
        ol.run(s, p, 1, walls=walls, threads=threads)
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return state.n * steps / el, steps, threads, state.n


class BatchedOracle:
    """The batched workload on the CPU oracle: every scene stepped in turn
    (one scene at a time, all host threads per scene)."""

    def __init__(self, states, gaps, p, walls_rows):
        sys.path.insert(0, str(REPO / "tests"))
        import oracle_lib as ol
        from gpusteer_gb300 import scenario as sc

        self.ol = ol
        self.p = p
        self.states = [s.copy() for s in states]
        cache = {}
        self.walls = []
        for g in gaps:
            if g not in cache:
                cache[g] = ol.split_walls(*sc.walls_from_rows(walls_rows(g)), p.world_size,
                                          p.world_cells)
            self.walls.append(cache[g])
        self.threads = ol.threads_available()
        self.n = sum(s.n for s in states)

    def step_scene(self, i):
        self.ol.run(self.states[i], self.p, 1, walls=self.walls[i], threads=self.threads)
        return self.states[i].n

    def step(self):
        for i in range(len(self.states)):
            self.step_scene(i)


def cpu_sample_batched(states, gaps, p, walls_rows, seconds: float):
    """Oracle agent-steps/s over whole batched steps (scene after scene),
    stopping after about `seconds`; returns (value, scene steps, threads)."""
    bo = BatchedOracle(states, gaps, p, walls_rows)
    bo.step_scene(0)  # warm-up
    done, agents, t0 = 0, 0, time.perf_counter()
    while True:
        agents += bo.step_scene(done % len(states))
        done += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return agents / el, done, bo.threads


def run_reference(args, dist, rank):
    """--impl reference: the reference's CPU path.  The reference itself
    cannot run here (legacy CUDA texture references, Windows/cutil build),
    so this is the oracle's restatement of its kernels on the host cores."""
    if rank != 0:
        return
    if args.workload == "batched":
        return run_reference_batched(args)
    if args.workload == "brute":
        return run_reference_brute(args)
    state, p, walls_rows = make_workload(args.workload)
    sys.path.insert(0, str(REPO / "tests"))
    import oracle_lib as ol
    from gpusteer_gb300 import scenario as sc

    walls = None
    if walls_rows is not None:
        walls = ol.split_walls(*sc.walls_from_rows(walls_rows), p.world_size, p.world_cells)
    threads = ol.threads_available()
    s = state.copy()
    t0 = time.perf_counter()
    warm = min(args.warmup, 3)
    for _ in range(warm):
        ol.run(s, p, 1, walls=walls, threads=threads)
    per_step = (time.perf_counter() - t0) / max(1, warm)
    # a bounded sample: at most about a minute of host time
    steps = max(1, min(args.steps, int(60.0 / max(per_step, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(steps):
        ol.run(s, p, 1, walls=walls, threads=threads)
    el = time.perf_counter() - t0
    v = state.n * steps / el
    line = {
        "impl": "reference", "metric": "agent-steps/s", "value": v, "unit": "agent-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": single_config(args.workload, p, state.n, args.gpus),
        "cpu_baseline": {"value": v, "unit": "agent-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} whole steps of the {state.n}-agent workload "
                                   f"(CPU oracle restating the reference kernels)"},
        "e2e": {"value": v, "unit": "agent-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference_brute(args):
    """The oracle's brute-force KNN on the host cores: a bounded sample of the
    65,536 queries per step (about 10 s of work in all)."""
    sys.path.insert(0, str(REPO / "tests"))
    import oracle_lib as ol
    from gpusteer_gb300 import scenario as sc

    n, k = 65536, 16
    pos = sc.boids_cube(n, size=512.0, seed=0).position
    threads = ol.threads_available()
    t0 = time.perf_counter()
    ol.knn_brute(pos[:1024], pos, False, k, threads=threads)
    per_query = (time.perf_counter() - t0) / 1024
    m = int(max(256, min(n, 10.0 / max(1, args.steps) / max(per_query, 1e-9))))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ol.knn_brute(pos[:m], pos, False, k, threads=threads)
    el = time.perf_counter() - t0
    v = m * args.steps / el
    line = {
        "impl": "reference", "metric": "agent-queries/s", "value": v, "unit": "agent-queries/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / args.steps * n / m, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": brute_config(n, k, args.gpus),
        "cpu_baseline": {"value": v, "unit": "agent-queries/s", "cores": threads, "kind": "port",
                         "sample": f"{m} of the {n} queries per step against all {n} agents "
                                   f"(CPU oracle restating KNNBruteForceCUDAV2, {threads} threads)"},
        "e2e": {"value": v, "unit": "agent-queries/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference_batched(args):
    states, gaps, p, walls_rows = make_batched(args.scenes)
    bo = BatchedOracle(states, gaps, p, walls_rows)
    t0 = time.perf_counter()
    bo.step()  # one whole warm-up step of all scenes
    per_step = time.perf_counter() - t0
    # a bounded sample: at most about a minute of host time
    steps = max(1, min(args.steps, int(60.0 / max(per_step, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(steps):
        bo.step()
    el = time.perf_counter() - t0
    v = bo.n * steps / el
    line = {
        "impl": "reference", "metric": "agent-steps/s", "value": v, "unit": "agent-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": batched_config(p, len(states), bo.n, args.gpus),
        "cpu_baseline": {"value": v, "unit": "agent-steps/s", "cores": bo.threads,
                         "kind": "port",
                         "sample": f"{steps} whole steps of all {len(states)} scenes "
                                   f"({bo.n} agents; CPU oracle restating the reference "
                                   f"kernels, scene after scene, {bo.threads} threads)"},
        "e2e": {"value": v, "unit": "agent-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---- GPU arm ------------------------------------------------------------------------

def pinned_state(lib, n):
    """AgentState whose arrays live in page-locked host memory, in the
    library's three blocks (one pitched copy per block); freed with the state."""
    import gpusteer_gb300 as gs

    return gs.pinned_state(n), []


def read_peaks():
    pk_path = REPO / "MEASURED_PEAKS.json"
    peaks = json.loads(pk_path.read_text()) if pk_path.exists() else {}
    return peaks.get("hbm_gbs", 6800.0), ("measured" if "hbm_gbs" in peaks else "fallback")


def read_traffic(workload):
    tr_path = REPO / "profiles" / f"traffic_{workload}.json"
    if tr_path.exists():
        return json.loads(tr_path.read_text()).get("fused_bytes_per_launch")
    return None


def phase_times(lib, group, run, steps):
    """Per-launch ms of the four step phases over `steps` profiled steps."""
    from gpusteer_gb300._lib import check

    check(lib.gs_group_set_profiling(group.handle, 1))
    run(steps)
    phase_ms = (C.c_float * 4)()
    phase_n = (C.c_uint * 4)()
    check(lib.gs_group_phase_times(group.handle, phase_ms, phase_n, 4))
    check(lib.gs_group_set_profiling(group.handle, 0))
    return {name: (phase_ms[i] / phase_n[i] if phase_n[i] else None)
            for i, name in enumerate(["scan", "permute", "fused", "fused_rest"])}


def adjoint_timing(reps: int = 5):
    """Forward rollout vs adjoint pass of the differentiable fit's
    configuration: 65,536 3D boids in a 200^3 cube, k = 16, 64 steps,
    checkpoints every 8.  Host clock around each synchronised call, median
    of `reps`; the plain fused step (gs_step, graph replay) alongside."""
    import torch

    import gpusteer_gb300 as gs
    from gpusteer_gb300 import scenario as sc

    n, steps, every = 65536, 64, 8
    s = sc.boids_cube(n, size=200.0, seed=0)
    p = sc.boids_params(k=16, world=256.0, cell=4.0)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    g = gs.AgentGroup(p.k, n)
    r = gs.Rollout(g, bins, steps, every)
    gen = torch.Generator(device="cuda").manual_seed(0)
    seed = torch.randn(n, 4, device="cuda", generator=gen) * 1e-3
    gv = torch.zeros(n, 4, device="cuda")
    gp = torch.zeros(n, 4, device="cuda")
    fwd, bwd, plain = [], [], []
    for it in range(reps + 1):
        g.upload(s)
        g.synchronize()
        t0 = time.perf_counter()
        r.forward(p)
        g.synchronize()
        t1 = time.perf_counter()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        r.backward(seed.data_ptr(), None, gp.data_ptr(), gv.data_ptr())
        t3 = time.perf_counter()
        g.upload(s)
        gs.step(g, bins, None, p, 1)
        g.synchronize()
        t4 = time.perf_counter()
        gs.step(g, bins, None, p, steps)
        g.synchronize()
        t5 = time.perf_counter()
        if it > 0:
            fwd.append((t1 - t0) * 1e3 / steps)
            bwd.append((t3 - t2) * 1e3 / steps)
            plain.append((t5 - t4) * 1e3 / steps)
    f, b, pl = statistics.median(fwd), statistics.median(bwd), statistics.median(plain)
    return {"config": "65,536 3D boids in a 200^3 cube, k=16, 64 steps, checkpoints every 8",
            "fwd_ms_per_step": f, "bwd_ms_per_step": b, "bwd_over_fwd": b / f,
            "plain_step_ms": pl, "bwd_over_plain_step": b / pl,
            "timing": f"host clock around synchronised calls, median of {reps}"}


def gpu_batched_line(args, dist, rank, world, local_rank):
    """The headline: 256 choke-point scenes batched, against per-scene
    launches, end to end through host memory, with the large-flock and
    brute-force records beside it.  Returns the JSON line (rank 0)."""
    import torch

    import gpusteer_gb300 as gs
    from gpusteer_gb300 import autotune
    from gpusteer_gb300._lib import check
    from gpusteer_gb300.state import AgentState

    lib = gs.load()
    check(lib.gs_set_device(local_rank))
    torch.cuda.set_device(local_rank)
    states, gaps, base, walls_rows = make_batched(args.scenes)
    n = sum(s.n for s in states)

    # autotune cell size, block shape and KNN capacity on the scenes themselves
    t0 = time.perf_counter()
    if args.fixed_config:
        tr = autotune.TuneResult(params=base, block=args.block or 256, capacity=0,
                                 ms_per_step=0.0, persistent=args.persistent,
                                 parts=max(1, args.parts))
    else:
        tr = autotune.tune_batched(states, gaps, base, walls_rows)
    tune_s = time.perf_counter() - t0
    p = tr.params
    def configure(grp, capacity=None):
        gs.set_block(grp, tr.block)
        gs.set_knn_capacity(grp, tr.capacity if capacity is None else capacity)
        gs.set_persistent(grp, tr.persistent)

    b = autotune.batch_for(states, gaps, p, walls_rows)
    configure(b.group)
    stream = torch.cuda.ExternalStream(b.group.stream)
    # the timed batches: the scenes in tr.parts consecutive ranges, each a
    # batch on its own stream, stepped concurrently (one batch when 1)
    run = [b] if tr.parts <= 1 else autotune.batch_parts(states, gaps, p, walls_rows, tr.parts)
    for x in run:
        configure(x.group)
    streams = [torch.cuda.ExternalStream(x.group.stream) for x in run]

    # warm-up, then K timed steps (one graph replay per batch each, state
    # resident in HBM); the other streams start after ev0 and ev1 waits for
    # all of them
    for x in run:
        x.step(p, args.warmup)
    for x in run:
        x.group.synchronize()
    barrier(dist)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        torch.cuda.synchronize()
        torch.cuda.profiler.start()  # ncu --profile-from-start off sees the timed steps only
        ev0.record(streams[0])
        for st_ in streams[1:]:
            st_.wait_event(ev0)
        for _ in range(args.steps):
            for x in run:
                x.step(p, 1)
        for st_ in streams[1:]:
            done = torch.cuda.Event()
            done.record(st_)
            streams[0].wait_event(done)
        ev1.record(streams[0])
        ev1.synchronize()
        torch.cuda.profiler.stop()
        torch.cuda.synchronize()
    barrier(dist)
    ms_max = allreduce_max(dist, ev0.elapsed_time(ev1))
    value = n * args.steps * world / (ms_max / 1e3)
    parts_identical = None
    if len(run) > 1:
        # the parts against the whole batch stepped as often
        b.step(p, args.warmup + args.steps)
        want = b.download()
        got = AgentState.concat([x.download() for x in run])
        parts_identical = all(np.array_equal(getattr(got, k), getattr(want, k))
                              for k in got.names())
    del run
    phases = phase_times(lib, b.group, lambda k: b.step(p, k), max(3, min(args.steps, 10)))
    launches_per_step = gs.step_launches(b.group, True) * max(1, tr.parts)
    measured_cap = gs.knn_capacity(b.group)  # the scan the resident steps used
    # both forms of the step on the same batch: separate launches (one graph
    # replay per step) and one persistent launch per step
    forms = {}
    for pers in (False, True):
        gs.set_persistent(b.group, pers)
        gs.set_knn_capacity(b.group, measured_cap)
        b.step(p, 3)
        b.group.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.steps):
            b.step(p, 1)
        f1.record(stream)
        f1.synchronize()
        forms["persistent" if pers else "separate"] = {
            "ms_per_step": f0.elapsed_time(f1) / args.steps,
            "launches_per_step": gs.step_launches(b.group, True)}
    del b

    # the same scenes, one gs_step call per scene per step (same grid, block,
    # capacity; each scene's group keeps its CUDA graph).  "sequential": all
    # scenes' groups on one stream, one scene's step after another, as the
    # reference's plugins run on the default stream; "concurrent": each
    # group on its own stream, so the GPU may overlap scenes.
    ps_steps = max(3, min(args.steps, 50))

    def per_scene_run(shared: bool):
        groups, first = [], None
        for s, g in zip(states, gaps):
            bins = gs.KNNBinData(p.world_cells, p.world_size, p.search_radius)
            walls = gs.WallGroup(walls_rows(g), bins=bins, knw=p.knw)
            grp = gs.AgentGroup(p.k, s.n, stream=first.stream if (shared and first) else None)
            first = first or grp
            grp.upload(s)
            configure(grp)
            groups.append((grp, bins, walls))
        for grp, bins, walls in groups:
            gs.step(grp, bins, walls, p, args.warmup)
        for grp, _, _ in groups:
            grp.synchronize()
        barrier(dist)
        t0 = time.perf_counter()
        for _ in range(ps_steps):
            for grp, bins, walls in groups:
                gs.step(grp, bins, walls, p, 1)
        for grp, _, _ in groups:
            grp.synchronize()
        el = allreduce_max(dist, time.perf_counter() - t0)
        return n * ps_steps * world / el, 1e3 * el / ps_steps, groups

    total = args.warmup + ps_steps
    b2 = autotune.batch_for(states, gaps, p, walls_rows)
    configure(b2.group)
    per_scene, identical, identical_other = None, None, None
    if not args.no_per_scene:
        per_seq, per_seq_ms, groups = per_scene_run(shared=True)
        del groups
        per_conc, per_conc_ms, per = per_scene_run(shared=False)
        # identical results: a fresh batch stepped as often as the per-scene groups
        b2.step(p, total)
        got = b2.download()
        want = AgentState.concat([grp.download() for grp, _, _ in per])
        identical = all(np.array_equal(getattr(got, k), getattr(want, k)) for k in got.names())
        # the other form of the step gives the same state
        b3 = autotune.batch_for(states, gaps, p, walls_rows)
        configure(b3.group, measured_cap)
        gs.set_persistent(b3.group, not tr.persistent)
        b3.step(p, total)
        got3 = b3.download()
        identical_other = all(np.array_equal(getattr(got3, k), getattr(want, k))
                              for k in got3.names())
        del b3
        del per
        per_scene = {
            "value": per_seq, "unit": "agent-steps/s", "steps": ps_steps,
            "ms_per_step": per_seq_ms,
            "launch": "one gs_step per scene per step, all scenes on one stream",
            "timing": "host clock, streams synchronised on both sides",
            "batched_over_per_scene": value / per_seq,
            "concurrent": {"value": per_conc, "ms_per_step": per_conc_ms,
                           "launch": "one gs_step per scene per step, each scene on its own "
                                     "stream",
                           "batched_over": value / per_conc}}

    # end to end: every step, the whole page-locked host state goes to the
    # device, is stepped once and comes back.  One batch: upload, step and
    # download one after another (gs_batch_upload / _step / _download).  Parts:
    # the scenes in `e2e_parts` consecutive ranges, each a batch on its own
    # stream, stepped with gs_batches_step_host, which overlaps one part's
    # copies with another part's step; the headline e2e is the parts' number.
    hio, keep = pinned_state(lib, n)
    init = AgentState.concat(states)
    for k in hio.names():
        getattr(hio, k)[...] = getattr(init, k)
    e2e_steps = max(3, min(args.steps, 20))
    b2.upload(hio)
    b2.step(p, 1)
    b2.download(hio)
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        b2.upload(hio)
        b2.step(p, 1)
        b2.download(hio)
    one_s = allreduce_max(dist, time.perf_counter() - t0)
    e2e_one = n * e2e_steps * world / one_s
    # the parts: scene ranges of about equal agent counts
    K = max(1, min(args.e2e_parts, len(states)))
    ranges = autotune.scene_cuts(states, K)
    cuts = [lo for lo, _ in ranges] + [ranges[-1][1]]
    parts = []
    for lo, hi in ranges:
        bp = autotune.batch_for(states[lo:hi], gaps[lo:hi], p, walls_rows)
        # a fixed capacity (the host-stepping graph needs one): the one the
        # resident batch used
        configure(bp.group, tr.capacity or measured_cap or 256)
        parts.append(bp)
    # one step from the initial state: the parts equal the single batch
    for k in hio.names():
        getattr(hio, k)[...] = getattr(init, k)
    b2.upload(hio)
    b2.step(p, 1)
    want = b2.download()
    gs.batches_step_host(parts, p, 1, hio, hio)
    parts_identical = all(np.array_equal(getattr(hio, k), getattr(want, k)) for k in want.names())
    gs.batches_step_host(parts, p, 1, hio, hio)
    barrier(dist)
    # each call is synchronous (its results are in host memory when it
    # returns): timed one by one, the median per step discounts a host-side
    # stall in one call; the mean is reported beside it
    step_s = []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        gs.batches_step_host(parts, p, 1, hio, hio)
        step_s.append(time.perf_counter() - t0)
    e2e_med = allreduce_max(dist, statistics.median(step_s))
    e2e_mean = allreduce_max(dist, sum(step_s) / len(step_s))
    e2e = n * world / e2e_med
    bytes_state = n * (16 * 3 + 12 * 2 + 4 * 5 + 4)
    # in place, the four per-agent constants (16 B) are not copied back
    bytes_back = n * (16 * 3 + 12 * 2 + 4 * 2)
    del parts
    for ptr in keep:
        lib.gs_host_free(ptr)
    del b2

    floor_ms = copy_floor_ms([s.n for s in states], cuts)
    adjoint = adjoint_timing() if not args.no_adjoint else None
    # the other throughput configurations, as records of this line
    large = brute = choke = boids = None
    if not args.no_sub:
        sub = argparse.Namespace(**vars(args))
        sub.workload, sub.steps, sub.warmup = "large", args.large_steps, args.large_warmup
        sub.cpu_seconds = min(args.cpu_seconds, 5.0)
        large = gpu_single_line(sub, dist, rank, world, local_rank)
        sub = argparse.Namespace(**vars(args))
        sub.workload, sub.steps, sub.warmup = "brute", 5, 3
        brute = gpu_brute_line(sub, dist, rank, world, local_rank)
        sub = argparse.Namespace(**vars(args))
        sub.workload, sub.steps, sub.warmup, sub.block = "chokepoint", 500, 10, None
        sub.cpu_seconds = min(args.cpu_seconds, 3.0)
        choke = gpu_single_line(sub, dist, rank, world, local_rank)
        sub = argparse.Namespace(**vars(args))
        sub.workload, sub.steps, sub.warmup, sub.block = "boids", 100, 10, None
        sub.cpu_seconds = min(args.cpu_seconds, 3.0)
        boids = gpu_single_line(sub, dist, rank, world, local_rank)
        if boids is not None:
            boids["bruteforce_dropin"] = boids_bruteforce_dropin(100, 10)
    if rank != 0:
        return None
    peak, peak_src = read_peaks()
    fused_ms = phases["fused"] + (phases["fused_rest"] or 0.0)
    fbytes = fused_bytes_per_agent(p) * n
    achieved = fbytes / (fused_ms / 1e3) / 1e9
    cpu = None
    if world == 1 and not args.no_cpu:
        v, done, threads = cpu_sample_batched(states, gaps, p, walls_rows, args.cpu_seconds)
        cpu = {"value": v, "unit": "agent-steps/s", "cores": threads, "kind": "port",
               "sample": f"{done} scene-steps of the batched workload (scenes in order), "
                         f"CPU oracle, {threads} threads"}
    cells = int(np.prod(p.world_cells))
    line = {
        "metric": "agent-steps/s",
        "value": value,
        "unit": "agent-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": batched_config(p, len(states), n, world),
        "tuned": {"block": tr.block, "knn_capacity": tr.capacity or "auto",
                  "cell": p.world_size[0] / p.world_cells[0], "persistent": tr.persistent,
                  "parts": tr.parts},
        "parts": {"count": tr.parts, "identical_to_one_batch": parts_identical,
                  "launch": "the scenes in consecutive ranges of about equal agent counts, "
                            "each a batch on its own stream, stepped concurrently"},
        "forms": forms,
        "per_scene": per_scene,
        "identical_to_per_scene": None if identical is None else {
            "equal": bool(identical), "steps": total,
            "compared": "every state array of every agent",
            "other_form_equal": bool(identical_other)},
        "autotune": {"seconds": tune_s, "trials": tr.trials},
        "adjoint": adjoint,
        "e2e": {"value": e2e, "unit": "agent-steps/s", "h2d_bytes_per_step": bytes_state,
                "d2h_bytes_per_step": bytes_back, "ms_per_step": e2e_med * 1e3,
                "ms_per_step_mean": e2e_mean * 1e3,
                "timing": f"median of {e2e_steps} host-timed calls, one step each",
                "api": f"gs_batches_step_host over {len(cuts) - 1} parts (scene ranges) in "
                       "place, one graph: each part's copies in, steps and copies out, "
                       "overlapped across the parts",
                "copy_floor_ms": floor_ms,
                "e2e_over_copy_floor": e2e_med * 1e3 / floor_ms,
                "copy_floor": "the same bytes in and out of the same page-locked arrays "
                              "alone: one cudaMemcpyAsync per block and part, each part on "
                              "its own stream (copies out after its copies in), no steps",
                "identical_to_one_batch": parts_identical,
                "one_batch": {"value": e2e_one, "ms_per_step": one_s * 1e3 / e2e_steps,
                              "api": "gs_batch_upload, gs_batch_step, gs_batch_download"}},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": read_traffic("batched"),
                     "kernel": "k_fused_walls+k_fused_rest",
                     "algorithmic_bytes_per_launch": fbytes, "peak_source": peak_src},
        "phases_ms": phases,
        # the committed instruction count is the 256-scene workload's
        "issue": (issue_rate("batched", fused_ms, clocks.summary(), local_rank)
                  if len(states) == 256 else None),
        "step_model_gbs": step_model_bytes(n, p.k, cells * len(states)) /
                          (ms_max / args.steps / 1e3) / 1e9,
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
        "large_flock": large,
        "brute": brute,
        "chokepoint": choke,
        "boids": boids,
    }
    return line


def boids_bruteforce_dropin(steps: int, warmup: int) -> dict:
    """Config 1 through brute-force KNN: 4,096 boids, k = 7, the drop-in call
    sequence of BoidsGroupBruteForce's update (wrap, brute-force KNN,
    separation, cohesion, alignment, update), `steps` steps timed with CUDA
    events on the group's stream after `warmup`."""
    import torch

    import gpusteer_gb300 as gs
    from gpusteer_gb300 import scenario as sc

    p = sc.boids_params(k=7)
    s = sc.boids_sphere(4096, seed=0)
    g = gs.AgentGroup(p.k, s.n)
    g.upload(s)
    knn = gs.KNNData(s.n, p.k)
    stream = torch.cuda.ExternalStream(g.stream)

    def frame():
        gs.wrapWorld(g, p.world_size, p.wrap_mode)
        gs.findKNearestNeighborsBruteForce(g, knn, g)
        gs.steerForSeparation(g, knn, g, p.sep_min, p.sep_max, p.sep_cos, p.w_sep, p.mask_sep)
        gs.steerForCohesion(g, knn, g, p.coh_min, p.coh_max, p.coh_cos, p.w_coh, p.mask_coh)
        gs.steerForAlignment(g, knn, g, p.ali_min, p.ali_max, p.ali_cos, p.w_ali, p.mask_ali)
        gs.updateGroup(g, p.dt)

    for _ in range(warmup):
        frame()
    g.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        frame()
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    return {"ms_per_step": ms, "value": s.n / (ms / 1e3), "unit": "agent-steps/s", "steps": steps,
            "calls": "gs_wrap_world, gs_knn_bruteforce, gs_steer_for_separation / cohesion / "
                     "alignment, gs_update_group per step (per-function launches)"}


def copy_floor_ms(agents, cuts, reps: int = 5) -> float:
    """Milliseconds to move the end-to-end step's bytes alone, with no steps:
    per part (scene range cuts[i]..cuts[i+1]) the three state blocks in
    (float4 x3, float3 x2, 4-byte x6: 96 B/agent) and out (80 B/agent: the
    four per-agent constants stay), one cudaMemcpyAsync per block, each part
    on its own stream.  Median of `reps`."""
    import torch

    blocks_in, blocks_out = (48, 24, 24), (48, 24, 8)
    parts = []
    for lo, hi in zip(cuts[:-1], cuts[1:]):
        na = int(sum(agents[lo:hi]))
        host = [torch.empty(na * b, dtype=torch.uint8, pin_memory=True) for b in blocks_in]
        dev = [torch.empty(na * b, dtype=torch.uint8, device="cuda") for b in blocks_in]
        parts.append((host, dev, torch.cuda.Stream(), na))
    times = []
    for _ in range(reps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for host, dev, st, na in parts:
            with torch.cuda.stream(st):
                for h, d in zip(host, dev):
                    d.copy_(h, non_blocking=True)
                for h, d, b in zip(host, dev, blocks_out):
                    h[:na * b].copy_(d[:na * b], non_blocking=True)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    return statistics.median(times[1:]) * 1e3


def issue_rate(workload: str, kernel_ms: float, clocks: dict, device: int):
    """Warp instructions the dominant kernel(s) issue per launch (from the
    committed ncu capture, profiles/issue_<workload>.json) over what the SMs
    can issue in the measured time: SMs x 4 schedulers x median SM clock x
    time.  An instruction-bound kernel is measured against this ceiling."""
    path = REPO / "profiles" / f"issue_{workload}.json"
    if not path.exists() or not kernel_ms or not clocks.get("sm_mhz"):
        return None
    import torch

    rec = json.loads(path.read_text())
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    slots = sms * 4 * clocks["sm_mhz"] * 1e6 * kernel_ms / 1e3
    return {"warp_instructions_per_launch": rec["warp_instructions_per_launch"],
            "kernels": rec.get("kernels"), "sm_count": sms, "sm_mhz": clocks["sm_mhz"],
            "kernel_ms": kernel_ms, "frac": rec["warp_instructions_per_launch"] / slots,
            "source": f"profiles/issue_{workload}.json"}


def fp32_peak_tflops():
    """Measured FP32 peak: cuBLAS SGEMM with TF32 off (FP32 FMA pipe),
    8192^3, best of 5, CUDA events."""
    import torch

    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        n = 8192
        a = torch.randn(n, n, device="cuda")
        b = torch.randn(n, n, device="cuda")
        torch.matmul(a, b)
        best = None
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        return 2.0 * n ** 3 / (best / 1e3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def gpu_brute_line(args, dist, rank, world, local_rank):
    """gs_knn_bruteforce (KNNBruteForceCUDAV2) over 65,536 agents, k = 16.
    Returns the JSON line (rank 0; None elsewhere)."""
    import torch

    import gpusteer_gb300 as gs
    from gpusteer_gb300 import scenario as sc
    from gpusteer_gb300._lib import check

    lib = gs.load()
    check(lib.gs_set_device(local_rank))
    torch.cuda.set_device(local_rank)
    n, k = 65536, 16
    s = sc.boids_cube(n, size=512.0, seed=0)
    g = gs.AgentGroup(k, n)
    g.upload(s)
    knn = gs.KNNData(n, k)
    stream = torch.cuda.ExternalStream(g.stream)
    for _ in range(args.warmup):
        gs.findKNearestNeighborsBruteForce(g, knn, g)
    g.synchronize()
    barrier(dist)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        ev0.record(stream)
        for _ in range(args.steps):
            gs.findKNearestNeighborsBruteForce(g, knn, g)
        ev1.record(stream)
        ev1.synchronize()
        torch.cuda.profiler.stop()
    barrier(dist)
    ms_max = allreduce_max(dist, ev0.elapsed_time(ev1))
    per = ms_max / args.steps
    pairs_all = float(n) * (n - 1)
    # the pairs the distance filter ran on: the bucketed scan skips chunks of
    # candidates beyond every bound of a warp's queries
    pairs = float(gs.bruteforce_pairs(g))
    tflops = 8.0 * pairs / (per / 1e3) / 1e12
    peak = fp32_peak_tflops()
    # end to end: positions up, lists down, every query
    hp = s.copy()
    t0 = time.perf_counter()
    e2e_steps = max(3, min(args.steps, 20))
    for _ in range(e2e_steps):
        g.upload(hp)
        gs.findKNearestNeighborsBruteForce(g, knn, g)
        knn.download(g)
    e2e_s = allreduce_max(dist, time.perf_counter() - t0)
    if rank != 0:
        return None
    cpu = None
    if world == 1 and not args.no_cpu:
        sys.path.insert(0, str(REPO / "tests"))
        import oracle_lib as ol

        threads = ol.threads_available()
        sub = s.position[:4096]
        t0 = time.perf_counter()
        ol.knn_brute(sub, s.position, False, k, threads=threads)
        el = time.perf_counter() - t0
        cpu = {"value": 4096 / el, "unit": "agent-queries/s", "cores": threads, "kind": "port",
               "sample": f"4,096 of the 65,536 queries against all 65,536 agents, CPU oracle, "
                         f"{threads} threads"}
    line = {
        "metric": "agent-queries/s", "value": n * world / (per / 1e3), "unit": "agent-queries/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": per,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": brute_config(n, k, world),
        "e2e": {"value": n * e2e_steps * world / e2e_s, "unit": "agent-queries/s",
                "h2d_bytes_per_step": n * 96, "d2h_bytes_per_step": n * k * 8},
        # per call: the extent, the seed database (count, three scan
        # launches, scatter), the seed, chunk and stage boxes, the scan
        # (profiles/k_knn_brute3_65536_agents.md lists them)
        "gpu_launches": 10 * args.steps,
        "roofline": {"bound": "fp32", "achieved": tflops, "peak": peak, "unit": "TFLOP/s",
                     "frac": tflops / peak, "traffic": None, "kernel": "k_knn_brute3_bucketed",
                     "algorithmic_flops_per_launch": 8.0 * pairs,
                     "pairs_evaluated": pairs, "pairs_all": pairs_all,
                     "time": "the whole call (extent, seed databases and search, chunk "
                             "boxes, scan)",
                     "peak_source": "measured here: cuBLAS SGEMM 8192^3 with TF32 off"},
        "issue": issue_rate("brute", per, clocks.summary(), local_rank),
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
    }
    return line


def run_gpu(args, dist, rank, world, local_rank):
    if args.workload == "batched":
        line = gpu_batched_line(args, dist, rank, world, local_rank)
    elif args.workload == "brute":
        line = gpu_brute_line(args, dist, rank, world, local_rank)
    else:
        line = gpu_single_line(args, dist, rank, world, local_rank)
    if line is not None:
        print(json.dumps(line), flush=True)


def gpu_single_line(args, dist, rank, world, local_rank):
    """One group of the `large`, `chokepoint` or `boids` workload stepped K
    times.  Returns the JSON line (rank 0; None elsewhere)."""
    import torch

    import gpusteer_gb300 as gs
    from gpusteer_gb300 import scenario as sc
    from gpusteer_gb300._lib import check

    lib = gs.load()
    check(lib.gs_set_device(local_rank))
    torch.cuda.set_device(local_rank)
    state, p, walls_rows = make_workload(args.workload)
    n = state.n
    bins = gs.KNNBinData(p.world_cells, p.world_size, p.search_radius)
    walls = gs.WallGroup(walls_rows, bins=bins, knw=p.knw) if walls_rows is not None else None
    group = gs.AgentGroup(p.k, n)
    group.upload(state)
    if getattr(args, "block", None):
        gs.set_block(group, args.block)
    stream = torch.cuda.ExternalStream(group.stream)
    has_walls = walls is not None

    # warm-up, then K timed steps (state resident in HBM)
    gs.step(group, bins, walls, p, args.warmup)
    group.synchronize()
    barrier(dist)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        torch.cuda.synchronize()
        torch.cuda.profiler.start()  # ncu --profile-from-start off sees the timed steps only
        ev0.record(stream)
        for _ in range(args.steps):
            gs.step(group, bins, walls, p, 1)
        ev1.record(stream)
        ev1.synchronize()
        torch.cuda.profiler.stop()
        torch.cuda.synchronize()
    barrier(dist)
    ms = ev0.elapsed_time(ev1)
    ms_max = allreduce_max(dist, ms)
    value = n * args.steps * world / (ms_max / 1e3)

    # dominant kernel: phase timing with CUDA events on the group's stream
    phases = phase_times(lib, group, lambda k: gs.step(group, bins, walls, p, k),
                         max(3, min(args.steps, 20)))
    fused_ms = phases["fused"] + (phases["fused_rest"] or 0.0)
    fbytes = fused_bytes_per_agent(p) * n
    peak, peak_src = read_peaks()
    achieved = fbytes / (fused_ms / 1e3) / 1e9
    traffic = read_traffic(args.workload)

    # end to end: host state in page-locked memory, copied in and out every step
    hin, keep_in = pinned_state(lib, n)
    hout, keep_out = pinned_state(lib, n)
    for k in hin.names():
        getattr(hin, k)[...] = getattr(state, k)
    e2e_steps = max(3, min(args.steps, 20))
    gs.step_host(group, bins, walls, p, 1, hin, hout)  # warm-up
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        gs.step_host(group, bins, walls, p, 1, hout, hout)
    e2e_s = allreduce_max(dist, time.perf_counter() - t0)
    e2e = n * e2e_steps * world / e2e_s
    bytes_state = n * (16 * 3 + 12 * 2 + 4 * 5 + 4)
    # in place, the four per-agent constants no step changes are not copied back
    bytes_back = bytes_state - n * 16
    for ptr in keep_in + keep_out:
        lib.gs_host_free(ptr)

    if rank != 0:
        return None
    cpu = None
    if world == 1 and not args.no_cpu:
        v, steps, threads, n_cpu = cpu_sample(state, p, walls_rows, args.cpu_seconds)
        cpu = {"value": v, "unit": "agent-steps/s", "cores": threads, "kind": "port",
               "sample": f"{steps} whole steps of the full {n_cpu}-agent workload, "
                         f"CPU oracle, {threads} threads"}
    cells = int(np.prod(p.world_cells))
    step_model_gbs = step_model_bytes(n, p.k, cells) / (ms_max / args.steps / 1e3) / 1e9
    line = {
        "metric": "agent-steps/s",
        "value": value,
        "unit": "agent-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": single_config(args.workload, p, n, world),
        "e2e": {"value": e2e, "unit": "agent-steps/s", "h2d_bytes_per_step": bytes_state,
                "d2h_bytes_per_step": bytes_back,
                "api": "gs_step_host in place: page-locked host state copied in, one step, "
                       "copied out (the per-agent constants stay on the host)"},
        "gpu_launches": gs.step_launches(group, has_walls) * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "k_fused" + ("_walls+k_fused_rest" if has_walls else ""),
                     "algorithmic_bytes_per_launch": fbytes, "peak_source": peak_src},
        "phases_ms": phases,
        "step_model_gbs": step_model_gbs,
        "step_model_frac": step_model_gbs / peak,
        "issue": issue_rate(args.workload, fused_ms, clocks.summary(), local_rank),
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
    }
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: the workload's own step count)")
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gs", choices=["gs", "reference"])
    ap.add_argument("--workload", default="batched", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the differentiable rollout's forward / backward timing")
    ap.add_argument("--scenes", type=int, default=256, help="batched workload: scene count")
    ap.add_argument("--fixed-config", action="store_true",
                    help="batched workload: the scenario's grid, 256 threads, KNN capacity "
                         "from the density (no autotuning)")
    ap.add_argument("--e2e-parts", type=int, default=8,
                    help="batched workload: scene ranges overlapped in the end-to-end run")
    ap.add_argument("--no-per-scene", action="store_true",
                    help="batched workload: skip the per-scene baselines")
    ap.add_argument("--block", type=int, default=None,
                    help="threads per block of the fused launches (large/chokepoint/boids "
                         "workloads, and the batched workload with --fixed-config)")
    ap.add_argument("--parts", type=int, default=1,
                    help="batched workload with --fixed-config: scene ranges stepped "
                         "concurrently, each a batch on its own stream")
    ap.add_argument("--persistent", action="store_true",
                    help="batched workload with --fixed-config: one persistent launch per step")
    ap.add_argument("--no-sub", action="store_true",
                    help="batched workload: skip the large-flock and brute-force records")
    ap.add_argument("--large-steps", type=int, default=200,
                    help="large-flock record: timed steps")
    ap.add_argument("--large-warmup", type=int, default=100,
                    help="large-flock record: untimed steps before (the flock clusters)")
    args = ap.parse_args()
    if args.steps is None:
        from gpusteer_gb300 import scenario as sc

        args.steps = sc.default_steps(args.workload)
    if args.warmup < 3:
        args.warmup = 3
    dist, rank, world, local_rank = dist_setup()
    if args.impl == "reference":
        run_reference(args, dist, rank)
    else:
        run_gpu(args, dist, rank, world, local_rank)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
