"""Throughput benchmark of the fused per-step agent update on GB300.

Default workload: the large plain flock - 1,048,576 3D boids uniform in a
512^3 cube, k = 16, spatial bins of cell 4.0 (128^3 cells), FP32, symmetric
world wrap.  A step is one whole update of every agent (wrap, bin rebuild,
KNN, separation / cohesion / alignment, integration) through gs_step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gs|reference]
                  [--workload large|chokepoint|boids]

Prints one JSON line (rank 0).  `value` is whole-job agent-steps/s with the
state resident in HBM, timed with CUDA events on the group's stream; `e2e`
is the same metric through gs_step_host with the state copied from and back
to page-locked host memory every step.  Under torchrun every rank runs an
independent replica on its own GPU (the flock is one world: replicas only).
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
    "batched": "256 independent 2D choke-point scenes (gap half-widths 7.5..32.5, 1,000-20,000 "
               "agents each), k=16, knw=3, 256x256 world, autotuned cell size and block shape",
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


def fused_bytes_per_agent(p) -> int:
    """Algorithmic DRAM bytes of the dominant fused kernel(s) per agent: its own
    bucketed state read once (5 float4 = 80 B), the new state written once
    (80 B) and the next step's (cell, rank) pair (8 B).  Neighbour and
    candidate reads hit the same bucketed arrays and are counted once.  With
    avoid-walls the step is split in two launches that also write and read
    the wall-phase state (3 float4) and the neighbour list (slot + distance
    per neighbour)."""
    from gpusteer_gb300 import scenario as sc

    if sc.B_AVOID_WALLS in p.order:
        walls_half = 80 + 48 + 8 * p.k
        rest_half = 48 + 48 + 8 * p.k + 80 + 8
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
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


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


def run_reference(args, dist, rank):
    """--impl reference: the reference's CPU path.  The reference itself
    cannot run here (legacy CUDA texture references, Windows/cutil build),
    so this is the oracle's restatement of its kernels on the host cores."""
    if rank != 0:
        return
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
        "config": {"workload": WORKLOADS[args.workload], "agents": state.n, "k": p.k},
        "cpu_baseline": {"value": v, "unit": "agent-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} whole steps of the {state.n}-agent workload "
                                   f"(CPU oracle restating the reference kernels)"},
        "e2e": {"value": v, "unit": "agent-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---- GPU arm ------------------------------------------------------------------------

def pinned_state(lib, n):
    """AgentState whose arrays live in page-locked host memory."""
    from gpusteer_gb300.state import AgentState

    shapes = {"position": (n, 4), "direction": (n, 4), "steering": (n, 4), "side": (n, 3),
              "up": (n, 3), "speed": (n,), "max_speed": (n,), "max_force": (n,),
              "radius": (n,), "mass": (n,), "applied": (n,)}
    arrays, ptrs = {}, []
    for k, shp in shapes.items():
        count = int(np.prod(shp))
        p = C.c_void_p()
        from gpusteer_gb300._lib import check

        check(lib.gs_host_alloc(count * 4, C.byref(p)))
        ptrs.append(p)
        ctype = C.c_uint if k == "applied" else C.c_float
        buf = (ctype * count).from_address(p.value)
        arrays[k] = np.ctypeslib.as_array(buf).reshape(shp)
    return AgentState(**arrays), ptrs


def run_gpu(args, dist, rank, world, local_rank):
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
    stream = torch.cuda.ExternalStream(group.stream)
    has_walls = walls is not None
    launches_per_step = 3 + 1 + (2 if has_walls else 1)

    # warm-up, then K timed steps (state resident in HBM)
    gs.step(group, bins, walls, p, args.warmup)
    group.synchronize()
    barrier(dist)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            gs.step(group, bins, walls, p, 1)
        ev1.record(stream)
        ev1.synchronize()
        torch.cuda.synchronize()
    barrier(dist)
    ms = ev0.elapsed_time(ev1)
    ms_max = allreduce_max(dist, ms)
    value = n * args.steps * world / (ms_max / 1e3)

    # dominant kernel: phase timing with CUDA events on the group's stream
    check(lib.gs_group_set_profiling(group.handle, 1))
    prof_steps = max(3, min(args.steps, 20))
    gs.step(group, bins, walls, p, prof_steps)
    phase_ms = (C.c_float * 4)()
    phase_n = (C.c_uint * 4)()
    check(lib.gs_group_phase_times(group.handle, phase_ms, phase_n, 4))
    check(lib.gs_group_set_profiling(group.handle, 0))
    phases = {name: (phase_ms[i] / phase_n[i] if phase_n[i] else None)
              for i, name in enumerate(["scan", "permute", "fused", "fused_rest"])}
    fused_ms = phases["fused"] + (phases["fused_rest"] or 0.0)
    fbytes = fused_bytes_per_agent(p) * n
    peaks = {}
    pk_path = REPO / "MEASURED_PEAKS.json"
    if pk_path.exists():
        peaks = json.loads(pk_path.read_text())
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = fbytes / (fused_ms / 1e3) / 1e9
    traffic = None
    tr_path = REPO / "profiles" / f"traffic_{args.workload}.json"
    if tr_path.exists():
        traffic = json.loads(tr_path.read_text()).get("fused_bytes_per_launch")

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
    for ptr in keep_in + keep_out:
        lib.gs_host_free(ptr)

    if rank != 0:
        return
    cpu = None
    if world == 1 and not args.no_cpu:
        v, steps, threads, n_cpu = cpu_sample(state, p, walls_rows, args.cpu_seconds)
        cpu = {"value": v, "unit": "agent-steps/s", "cores": threads, "kind": "port",
               "sample": f"{steps} whole steps of the full {n_cpu}-agent workload, "
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
        "config": {"workload": WORKLOADS[args.workload], "agents_per_gpu": n, "k": p.k,
                   "cells": cells, "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (about 200 MB of bucketed state per step)"},
        "e2e": {"value": e2e, "unit": "agent-steps/s", "h2d_bytes_per_step": bytes_state,
                "d2h_bytes_per_step": bytes_state},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "k_fused" + ("_walls+k_fused_rest" if has_walls else ""),
                     "algorithmic_bytes_per_launch": fbytes,
                     "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"},
        "phases_ms": phases,
        "step_model_gbs": step_model_bytes(n, p.k, cells) / (ms_max / args.steps / 1e3) / 1e9,
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gs", choices=["gs", "reference"])
    ap.add_argument("--workload", default="large", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
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
