"""Plugins written against the C++ drop-in (include/GroupSteerLibrary.h),
run by the headless driver (gpusteer_gb300/plugins/headless.cpp): the
reference's BoidsGroup and choke-point updates, call for call, give the
fused step's and the oracle's results bit for bit."""
import subprocess

import numpy as np
import pytest

import gpusteer_gb300 as gs
import oracle_lib as ol
from gpusteer_gb300 import build as gb
from gpusteer_gb300 import scenario as sc
from gpusteer_gb300.state import AgentState

pytestmark = pytest.mark.gpu
FIELDS = ("position", "direction", "steering", "side", "up", "speed", "max_speed", "max_force",
          "radius", "mass", "applied")


def write_state(path, s: AgentState):
    with open(path, "wb") as f:
        np.array([s.n], np.uint32).tofile(f)
        for k in FIELDS:
            np.ascontiguousarray(getattr(s, k)).tofile(f)


def read_state(path) -> AgentState:
    raw = open(path, "rb").read()
    n = int(np.frombuffer(raw[:4], np.uint32)[0])
    out, off = AgentState.zeros(n), 4
    for k in FIELDS:
        a = getattr(out, k)
        nb = a.nbytes
        a[...] = np.frombuffer(raw[off:off + nb], a.dtype).reshape(a.shape)
        off += nb
    return out


def f32(x) -> str:
    return np.format_float_positional(np.float32(x), unique=True, trim="0")


def v3(v) -> str:
    return ",".join(f32(x) for x in v)


def run_driver(tmp_path, plugin, s, frames, params):
    gb.build()
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    write_state(fin, s)
    args = [str(gb.HEADLESS), plugin, str(fin), str(fout), str(frames)]
    args += [f"{k}={v}" for k, v in params.items()]
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return read_state(fout)


def flock_args(p: sc.StepParams):
    d = {"world": v3(p.world_size), "cells": ",".join(str(c) for c in p.world_cells),
         "k": p.k, "radius": p.search_radius, "dt": f32(p.dt)}
    for b in ("sep", "ali", "coh"):
        d[f"{b}_min"] = f32(getattr(p, f"{b}_min"))
        d[f"{b}_max"] = f32(getattr(p, f"{b}_max"))
        d[f"{b}_cos"] = f32(getattr(p, f"{b}_cos"))
        d[f"w_{b}"] = f32(getattr(p, f"w_{b}"))
        d[f"mask_{b}"] = getattr(p, f"mask_{b}")
    return d


@pytest.mark.parametrize("masks", [False, True])
def test_boids_plugin_equals_fused_step_and_oracle(tmp_path, masks):
    s = sc.boids_sphere(4096, seed=0)
    p = sc.boids_params(k=7, masks=masks).replace(wrap_mode=sc.WRAP_REFERENCE)
    got = run_driver(tmp_path, "Boids", s, 30, flock_args(p))
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    g = gs.AgentGroup(p.k, s.n)
    g.upload(s)
    gs.step(g, bins, None, p, 30)
    fused = g.download()
    want = s.copy()
    ol.run(want, p, 30)
    for k in FIELDS:
        np.testing.assert_array_equal(getattr(got, k), getattr(fused, k), err_msg=k)
        if k != "side":
            np.testing.assert_array_equal(getattr(got, k), getattr(want, k), err_msg=k)


def test_chokepoint_plugin_equals_fused_step_and_oracle(tmp_path):
    s = sc.chokepoint_agents(10000, seed=0)
    s.speed[:] = np.float32(0.5)
    p = sc.chokepoint_params()
    rows = sc.chokepoint_walls(10.0)
    mp = tmp_path / "ChokePoint10.map"
    mp.write_text("\n".join(" ".join(f32(x) for x in r) for r in rows) + "\n")
    args = flock_args(p)
    args.update({"knw": p.knw, "map": str(mp), "min_time_wall": f32(p.min_time_to_wall),
                 "w_walls": f32(p.w_walls), "mask_walls": p.mask_walls,
                 "min_time_col": f32(p.min_time_to_collision),
                 "min_sep": f32(p.min_separation_distance), "avoid_close": p.avoid_close,
                 "w_avoid": f32(p.w_avoid), "mask_avoid": p.mask_avoid,
                 "seek": v3(p.seek_target), "w_seek": f32(p.w_seek), "mask_seek": p.mask_seek})
    got = run_driver(tmp_path, "ChokePoint", s, 30, args)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    walls = gs.WallGroup(rows, bins=bins, knw=p.knw)
    g = gs.AgentGroup(p.k, s.n)
    g.upload(s)
    gs.step(g, bins, walls, p, 30)
    fused = g.download()
    want = s.copy()
    ol.run(want, p, 30, walls=walls.download())
    for k in FIELDS:
        np.testing.assert_array_equal(getattr(got, k), getattr(fused, k), err_msg=k)
        np.testing.assert_array_equal(getattr(got, k), getattr(want, k), err_msg=k)
