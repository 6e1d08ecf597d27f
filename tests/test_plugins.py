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


def test_chokepoint_new_plugin_with_path_and_antipenetration(tmp_path):
    """CtfGroup::update as ChokePointNew.cpp:586-630 runs it (path following,
    seek to the path's second point, anti-penetration after the update):
    without anti-penetration it equals the fused step and the oracle, with it
    the per-function sequence through the Python binding."""
    import test_gpu_parity as tp

    p, pts, radius = tp.chokepoint_with_path()
    s = sc.chokepoint_agents(6000, seed=17)
    s.speed[:] = np.float32(1.0)
    rows = sc.chokepoint_walls(10.0)
    mp = tmp_path / "ChokePoint10.map"
    mp.write_text("\n".join(" ".join(f32(x) for x in r) for r in rows) + "\n")
    args = flock_args(p)
    args.update({"knw": p.knw, "map": str(mp), "min_time_wall": f32(p.min_time_to_wall),
                 "w_walls": f32(p.w_walls), "mask_walls": p.mask_walls,
                 "path": ";".join(v3(q) for q in pts), "path_radius": f32(radius),
                 "path_time": f32(p.path_prediction_time), "w_path": f32(p.w_path),
                 "mask_path": p.mask_path, "w_seek": f32(p.w_seek), "mask_seek": p.mask_seek})
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    walls = gs.WallGroup(rows, bins=bins, knw=p.knw)
    path = gs.Path(pts, radius)
    # without anti-penetration: the fused step and the oracle
    got = run_driver(tmp_path, "ChokePointNew", s, 20, dict(args, antipen=0))
    g = gs.AgentGroup(p.k, s.n)
    g.upload(s)
    gs.step(g, bins, walls, p, 20, path=path)
    fused = g.download()
    want = s.copy()
    ol.run(want, p, 20, walls=walls.download(), path=ol.path_init(pts, radius, False))
    for k in FIELDS:
        np.testing.assert_array_equal(getattr(got, k), getattr(fused, k), err_msg=k)
        np.testing.assert_array_equal(getattr(got, k), getattr(want, k), err_msg=k)
    # with anti-penetration: the per-function sequence
    got = run_driver(tmp_path, "ChokePointNew", s, 20, dict(args, antipen=1))
    g2 = gs.AgentGroup(p.k, s.n)
    g2.upload(s)
    knn = gs.KNNData(s.n, p.k)
    knw = gs.KNNData(s.n, p.knw)
    for _ in range(20):
        gs.wrapWorld(g2, p.world_size, p.wrap_mode)
        gs.updateKNNDatabase(g2, bins)
        gs.findKNearestNeighbors(g2, knn, bins, g2, 1)
        gs.findKNearestNeighbors(g2, knw, bins, walls, 1)
        gs.steerToAvoidWalls(g2, knw, walls, p.min_time_to_wall, p.w_walls, p.mask_walls)
        gs.steerForSeparation(g2, knn, g2, p.sep_min, p.sep_max, p.sep_cos, p.w_sep, p.mask_sep)
        gs.steerForAlignment(g2, knn, g2, p.ali_min, p.ali_max, p.ali_cos, p.w_ali, p.mask_ali)
        gs.steerForCohesion(g2, knn, g2, p.coh_min, p.coh_max, p.coh_cos, p.w_coh, p.mask_coh)
        gs.steerToFollowPath(g2, path, p.path_prediction_time, p.w_path, p.mask_path)
        gs.steerForSeek(g2, p.seek_target, p.w_seek, p.mask_seek)
        gs.updateGroup(g2, p.dt)
        gs.antiPenetrationAgents(g2, knn, g2, 0)
    dropin = g2.download()
    for k in FIELDS:
        np.testing.assert_array_equal(getattr(got, k), getattr(dropin, k), err_msg=k)


# CtfEnemyGroup's values (plugins/ChokePointGroup.cpp:148-203): weights, masks,
# neighbourhoods; the path and the goal are the test's.
CPG = {"min_time_wall": 10.0, "w_walls": 1.0, "mask_walls": 0, "path_time": 5.0, "w_path": 1.0,
       "mask_path": 16, "w_seek": 1.0, "mask_seek": 256, "sep_min": 0.5, "sep_max": 1.2,
       "sep_cos": -0.8660254, "w_sep": 10.0, "mask_sep": 4096, "ali_min": 0.5, "ali_max": 7.0,
       "ali_cos": -0.8660254, "w_ali": 2.5, "mask_ali": 272, "coh_min": 0.5, "coh_max": 7.0,
       "coh_cos": -0.8660254, "w_coh": 1.0, "mask_coh": 272, "mask_antipen": 4352}


def oracle_chokepoint_group(s, p, walls, path, goal, frames, dt):
    """CtfEnemyGroup::update (ChokePointGroup.cpp:683-728), one oracle call per
    reference call, on a copy of s."""
    C = ol.C
    o = ol.oracle()
    st, mid, en, nm = walls
    W = ol.walls_struct(st, mid, en, nm)
    s = s.copy()
    n, k, kw = s.n, p.k, p.knw
    c = CPG
    f = C.c_float
    for _ in range(frames):
        G = C.byref(ol.group_struct(s))
        o.orc_wrap_world(G, ol.f3(p.world_size), sc.WRAP_REFERENCE)
        s.applied[:] = 0
        idx, dist = ol.knn_binned(s.position, s.position, True, p.world_size, p.world_cells, 1, k)
        widx, _ = ol.knn_binned(s.position, mid, False, p.world_size, p.world_cells, 1, kw)
        ip, wp = ol.ptr(idx, C.c_uint), ol.ptr(widx, C.c_uint)
        o.orc_steer_avoid_walls(G, wp, kw, C.byref(W), f(c["min_time_wall"]), f(c["w_walls"]),
                                c["mask_walls"])
        o.orc_steer_follow_path(G, C.byref(path), f(c["path_time"]), f(c["w_path"]),
                                c["mask_path"])
        o.orc_steer_seek(G, ol.f3(goal), f(c["w_seek"]), c["mask_seek"])
        o.orc_steer_separation(G, ip, k, ol.ptr(s.position), n, f(c["sep_min"]),
                               f(c["sep_max"]), f(c["sep_cos"]), f(c["w_sep"]), c["mask_sep"])
        o.orc_steer_alignment(G, ip, k, ol.ptr(s.position), ol.ptr(s.direction), n,
                              f(c["ali_min"]), f(c["ali_max"]), f(c["ali_cos"]), f(c["w_ali"]),
                              c["mask_ali"])
        o.orc_steer_cohesion(G, ip, k, ol.ptr(s.position), n, f(c["coh_min"]), f(c["coh_max"]),
                             f(c["coh_cos"]), f(c["w_coh"]), c["mask_coh"])
        o.orc_update_with_antipenetration(G, wp, kw, C.byref(W), f(dt))
        pb, rb, ab = s.position.copy(), s.radius.copy(), s.applied.copy()
        o.orc_antipenetration_agents(G, ip, ol.ptr(dist), ol.ptr(pb), ol.ptr(rb),
                                     ol.ptr(ab, C.c_uint), n, c["mask_antipen"])
    return s


def test_chokepoint_group_plugin_with_wall_antipenetration(tmp_path):
    """CtfEnemyGroup::update (ChokePointGroup.cpp:683-728) through the C++
    drop-in: the applied bits cleared by the plugin's own cudaMemset on the
    group's device array, updateGroupWithAntiPenetration and
    antiPenetrationAgents; bit for bit the oracle composed call for call."""
    p = sc.chokepoint_params()
    pts, radius, goal, dt, frames = [(0.0, 0.0, 13.5), (0.0, 0.0, -1650.0)], 23.5, \
        (0.0, 0.0, -93.5), 0.1, 25
    s = sc.chokepoint_agents(5000, x_range=(-45.0, 45.0), z_range=(14.0, 44.0), seed=23)
    s.speed[:] = np.float32(2.0)
    rows = sc.chokepoint_walls(10.0)
    mp = tmp_path / "ChokePoint10.map"
    mp.write_text("\n".join(" ".join(f32(x) for x in r) for r in rows) + "\n")
    args = {"world": v3(p.world_size), "cells": ",".join(str(c) for c in p.world_cells),
            "k": p.k, "knw": p.knw, "map": str(mp), "path": ";".join(v3(q) for q in pts),
            "path_radius": f32(radius), "goal": v3(goal), "dt": f32(dt)}
    args.update({key: (f32(v) if isinstance(v, float) else v) for key, v in CPG.items()})
    got = run_driver(tmp_path, "ChokePointGroup", s, frames, args)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    walls = gs.WallGroup(rows, bins=bins, knw=p.knw).download()
    want = oracle_chokepoint_group(s, p, walls, ol.path_init(pts, radius, False), goal, frames,
                                   np.float32(dt))
    for k in FIELDS:
        np.testing.assert_array_equal(getattr(got, k), getattr(want, k), err_msg=k)
    # the frame's wall anti-penetration and agent anti-penetration both fired
    assert ((want.applied & 4096) != 0).sum() > 20
    assert ((want.applied & 8192) != 0).sum() > 20


SCENARIO = """# choke-point scenario: the values of the reference's data/ChokePoint.params
# on a 512 x 512 world
    seed = 1
    knn = 16
    knw = 3
    searchRadius = 1
    minTimeToWall = 10
    pathPredictionTime = 5
    minSeparationDistance = 0.5
    maxSeparationDistance = 1.2
    minFlockingDistance = 0.5
    maxFlockingDistance = 7
    cosMaxFlockingAngle = -0.86602540378443864676372317075294
    weightAlignment = 2.5   # per-value comment
    weightCohesion = 1
    weightSeparation = 10
    weightSeek = 1.5
    weightFollowPath = 1
    weightAvoidWalls = 1
    maskAlignment = 272
    maskAntiPenetrationAgents = 4096
    maskCohesion = 272
    maskSeparation = 4096
    maskSeek = 4480
    maskFollowPath = 16
    maskAvoidWalls = 0
    <world>
        dimensions = 512 10 512
        cells = 256 1 256
        obstacleCount = 0
        mapFilename = ChokePoint10.map
    </world>
    <group>
        numAgents = 6000
        maxSpeed = 3
        maxForce = 3
        <path>
            point = 0 0 13.5
            point = 0 0 -1650
            cyclic = 0
            radius = 20
        </path>
    </group>
</simulation>
"""


def test_chokepoint_new_plugin_from_params_file(tmp_path):
    """ChokePointNew configured by a .params file, read by the C++ plugin through
    include/SimulationParams.h and by the Python reader for gs_step
    (scenario.chokepoint_new_from_file): the plugin, the fused step and the
    oracle agree bit for bit (closing anti-penetration off)."""
    pf = tmp_path / "scenario.params"
    pf.write_text(SCENARIO)
    rows = sc.chokepoint_walls(10.0)
    (tmp_path / "ChokePoint10.map").write_text(
        "\n".join(" ".join(f32(x) for x in r) for r in rows) + "\n")
    dt = np.float32(1.0 / 30.0)
    p, pts, radius, cyclic = sc.chokepoint_new_from_file(sc.load_params(SCENARIO), float(dt))
    assert p.k == 16 and p.mask_seek == 4480 and radius == 20.0 and not cyclic
    s = sc.chokepoint_agents(6000, seed=29)
    s.speed[:] = np.float32(1.0)
    frames = 20
    got = run_driver(tmp_path, "ChokePointNew", s, frames,
                     {"params": str(pf), "antipen": 0, "dt": f32(dt)})
    bins = gs.KNNBinData(p.world_cells, p.world_size, p.search_radius)
    walls = gs.WallGroup(rows, bins=bins, knw=p.knw)
    g = gs.AgentGroup(p.k, s.n)
    g.upload(s)
    gs.step(g, bins, walls, p, frames, path=gs.Path(pts, radius, cyclic))
    fused = g.download()
    want = s.copy()
    ol.run(want, p, frames, walls=walls.download(), path=ol.path_init(pts, radius, cyclic))
    for k in FIELDS:
        np.testing.assert_array_equal(getattr(got, k), getattr(fused, k), err_msg=k)
        np.testing.assert_array_equal(getattr(got, k), getattr(want, k), err_msg=k)


def test_multigroup_plugin_equals_fused_multigroup_frames(tmp_path):
    """MultiGroupSimulation::update (MultiGroup.cpp:545-610) through the C++
    drop-in, call for call over three groups with two paths, against
    gs_multigroup_step on the same groups: bit for bit."""
    p = sc.boids_params(k=8, world=96.0, cell=4.0)
    states = [sc.boids_sphere(2200, radius=16.0, seed=61), sc.boids_sphere(1500, radius=16.0, seed=62),
              sc.boids_sphere(700, radius=12.0, seed=63)]
    for s in states:
        s.radius[:] = np.float32(0.9)
    pts = [[(0.0, 0.0, 0.0), (30.0, 5.0, -20.0)], None, [(5.0, -5.0, 5.0), (-25.0, 0.0, 10.0)]]
    radius, dt, frames = 6.0, np.float32(1.0 / 30.0), 8
    mp = dict(world_size=p.world_size, wrap_mode=sc.WRAP_REFERENCE, min_time_to_collision=2.0,
              min_separation_distance=0.5, avoid_close=1, w_avoid=1.0, mask_avoid=0,
              sep_min=p.sep_min, sep_max=p.sep_max, sep_cos=p.sep_cos, w_sep=p.w_sep,
              mask_sep=4096, ali_min=p.ali_min, ali_max=p.ali_max, ali_cos=p.ali_cos,
              w_ali=p.w_ali, mask_ali=272, coh_min=p.coh_min, coh_max=p.coh_max,
              coh_cos=p.coh_cos, w_coh=p.w_coh, mask_coh=272, path_prediction_time=5.0,
              w_path=1.0, mask_path=16, w_seek=1.5, mask_seek=4480, mask_antipen=4096,
              dt=float(dt))
    ins = [tmp_path / f"in{i}.bin" for i in range(3)]
    outs = [tmp_path / f"out{i}.bin" for i in range(3)]
    for f, s in zip(ins, states):
        write_state(f, s)
    args = {"world": v3(p.world_size), "cells": ",".join(str(c) for c in p.world_cells),
            "k": p.k, "radius": 1, "min_time_col": f32(2.0), "min_sep": f32(0.5),
            "avoid_close": 1, "w_avoid": f32(1.0), "mask_avoid": 0, "sep_min": f32(p.sep_min),
            "sep_max": f32(p.sep_max), "sep_cos": f32(p.sep_cos), "w_sep": f32(p.w_sep),
            "mask_sep": 4096, "ali_min": f32(p.ali_min), "ali_max": f32(p.ali_max),
            "ali_cos": f32(p.ali_cos), "w_ali": f32(p.w_ali), "mask_ali": 272,
            "coh_min": f32(p.coh_min), "coh_max": f32(p.coh_max), "coh_cos": f32(p.coh_cos),
            "w_coh": f32(p.w_coh), "mask_coh": 272, "path_time": f32(5.0), "w_path": f32(1.0),
            "mask_path": 16, "w_seek": f32(1.5), "mask_seek": 4480, "mask_antipen": 4096,
            "path_radius": f32(radius), "dt": f32(dt),
            "path0": ";".join(v3(q) for q in pts[0]), "path2": ";".join(v3(q) for q in pts[2])}
    gb.build()
    cmd = [str(gb.HEADLESS), "MultiGroup", ",".join(map(str, ins)), ",".join(map(str, outs)),
           str(frames)] + [f"{k}={v}" for k, v in args.items()]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    got = [read_state(f) for f in outs]
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    groups = []
    for s in states:
        g = gs.AgentGroup(p.k, s.n)
        g.upload(s)
        groups.append(g)
    knns = [[gs.KNNData(states[i].n, p.k) for _ in range(3)] for i in range(3)]
    paths = [gs.Path(q, radius) if q is not None else None for q in pts]
    gs.multigroup_step(groups, bins, knns, gs.MultiGroupParams(**mp), frames, paths=paths)
    for i in range(3):
        want = groups[i].download()
        for k in FIELDS:
            np.testing.assert_array_equal(getattr(got[i], k), getattr(want, k), err_msg=f"{i} {k}")
