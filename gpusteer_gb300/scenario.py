"""Seeded synthetic scenarios and scenario input formats.

* A portable counter-based RNG (splitmix64 -> binary32 in [0, 1) from the top
  24 bits) so that every machine generates identical agents.
* Initial states for the plain 3D flock and the 2D choke-point crowd, following
  ``randomizeStartingPositionAndHeading{2D,3D}`` (plugins/PluginCommon.cpp:5-32)
  and the agent defaults of ``SimpleVehicle::reset``
  (include/OpenSteer/SimpleVehicle.h:100-113: radius 0.5, mass 1).
* The choke-point wall map as a function of the gap half-width; it reproduces
  the reference's ``data/ChokePoint{X}.map`` files (six segments, 9 floats per
  line as read by WallGroupData::LoadFromFile, WallGroupData.cu:73-106).
* A reader for the reference's ``.params`` format (SimulationParams::load,
  src/Simulation.cpp:7-250).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .state import AgentState, KERNEL_ANTI_PENETRATION_WALL

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """Outputs offset..offset+count-1 of the splitmix64 stream seeded with seed."""
    with np.errstate(over="ignore"):
        i = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform01(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """binary32 uniforms in [0, 1) with 24 random bits each."""
    bits = splitmix64(seed, count, offset) >> np.uint64(40)
    return (bits.astype(np.float64) * (1.0 / (1 << 24))).astype(np.float32)


def hash_seed(seed: int, stream: int) -> int:
    """A derived seed for sub-stream `stream` (one scene of a batch, ...)."""
    return int(splitmix64(seed ^ 0x5DEECE66D, 1, stream)[0])


class Stream:
    """Sequential draws from one splitmix64 stream."""

    def __init__(self, seed: int):
        self.seed = int(seed)
        self.pos = 0

    def take(self, count: int) -> np.ndarray:
        out = uniform01(self.seed, count, self.pos)
        self.pos += count
        return out


def _unit_vectors_in_ball(stream: Stream, n: int, dims: int = 3) -> np.ndarray:
    """n points uniform in the unit ball (rejection sampling in [-1, 1]^dims)."""
    out = np.zeros((n, 3), np.float32)
    filled = 0
    while filled < n:
        need = n - filled
        draw = max(64, int(need * 2.2))
        u = stream.take(draw * dims).reshape(draw, dims).astype(np.float32) * np.float32(2) - np.float32(1)
        ok = (u.astype(np.float64) ** 2).sum(1) < 1.0
        acc = u[ok][:need]
        if dims == 3:
            out[filled:filled + len(acc)] = acc
        else:
            out[filled:filled + len(acc), 0] = acc[:, 0]
            out[filled:filled + len(acc), 2] = acc[:, 1]
        filled += len(acc)
    return out


def _normalize(v: np.ndarray) -> np.ndarray:
    n = np.sqrt((v.astype(np.float64) ** 2).sum(1, keepdims=True))
    n[n == 0] = 1.0
    return (v / n).astype(np.float32)


def _frame(direction: np.ndarray):
    """side = normalize(dir x up0), up = side x dir with up0 = (0, 1, 0)."""
    up0 = np.array([0, 1, 0], np.float64)
    d = direction.astype(np.float64)
    side = np.cross(d, up0)
    bad = (side ** 2).sum(1) < 1e-12
    side[bad] = np.array([1, 0, 0])
    side = side / np.sqrt((side ** 2).sum(1, keepdims=True))
    up = np.cross(side, d)
    return side.astype(np.float32), up.astype(np.float32)


def _finish(n, pos, direction, speed, max_speed, max_force, radius=0.5, mass=1.0) -> AgentState:
    s = AgentState.zeros(n)
    s.position[:, :3] = pos
    s.direction[:, :3] = direction
    s.side[:], s.up[:] = _frame(direction)
    s.speed[:] = speed
    s.max_speed[:] = max_speed
    s.max_force[:] = max_force
    s.radius[:] = radius
    s.mass[:] = mass
    return s


def boids_sphere(n: int, radius: float = 50.0, speed_max: float = 9.0, max_speed: float = 9.0,
                 max_force: float = 27.0, seed: int = 0) -> AgentState:
    """3D flock: positions uniform in a ball, random unit headings, speed U[0, speed_max]."""
    st = Stream(seed)
    pos = _unit_vectors_in_ball(st, n) * np.float32(radius)
    direction = _normalize(_unit_vectors_in_ball(st, n) + np.float32(1e-7))
    speed = st.take(n) * np.float32(speed_max)
    return _finish(n, pos, direction, speed, max_speed, max_force)


def boids_cube(n: int, size: float = 512.0, speed_max: float = 9.0, max_speed: float = 9.0,
               max_force: float = 27.0, seed: int = 0) -> AgentState:
    """3D flock: positions uniform in a cube of side `size` centred at the origin."""
    st = Stream(seed)
    u = st.take(3 * n).reshape(n, 3)
    half = np.float32(size * 0.5)
    pos = (u * np.float32(size) - half).astype(np.float32)
    direction = _normalize(_unit_vectors_in_ball(st, n) + np.float32(1e-7))
    speed = st.take(n) * np.float32(speed_max)
    return _finish(n, pos, direction, speed, max_speed, max_force)


def chokepoint_agents(n: int, x_range=(-50.0, 50.0), z_range=(13.5, 113.5), max_speed=3.0,
                      max_force=3.0, seed: int = 0) -> AgentState:
    """2D crowd uniform in a rectangle on the inflow side of the gap, speed 0
    (CtfGroup::reset, plugins/ChokePointNew.cpp:455-476), headings on the XZ plane."""
    st = Stream(seed)
    u = st.take(2 * n).reshape(n, 2)
    pos = np.zeros((n, 3), np.float32)
    pos[:, 0] = np.float32(x_range[0]) + u[:, 0] * np.float32(x_range[1] - x_range[0])
    pos[:, 2] = np.float32(z_range[0]) + u[:, 1] * np.float32(z_range[1] - z_range[0])
    direction = _normalize(_unit_vectors_in_ball(st, n, dims=2) + np.float32(1e-7) * np.array([1, 0, 0], np.float32))
    return _finish(n, pos, direction, 0.0, max_speed, max_force)


def chokepoint_walls(gap: float, far_x: float = 1232.5, far_z: float = 293.5,
                     wall_z: float = 13.5) -> np.ndarray:
    """Wall segments of data/ChokePoint{gap}.map as a (6, 9) float32 array of
    start(3), end(3), normal(3): a funnel on each side of a channel of
    half-width `gap` through a wall of half-depth `wall_z`."""
    g, fx, fz, wz = float(gap), far_x, far_z, wall_z
    rows = [
        [-fx, 0, fz, -g, 0, wz, 0, 0, 1],
        [-fx, 0, -fz, -g, 0, -wz, 0, 0, -1],
        [-g, 0, -wz, -g, 0, wz, 1, 0, 0],
        [g, 0, wz, fx, 0, fz, 0, 0, 1],
        [g, 0, -wz, fx, 0, -fz, 0, 0, -1],
        [g, 0, wz, g, 0, -wz, -1, 0, 0],
    ]
    return np.array(rows, np.float32)


def read_map(path: str) -> np.ndarray:
    """Read a .map file: whitespace separated, 9 floats per segment."""
    with open(path) as f:
        vals = f.read().split()
    n = len(vals) // 9
    return np.array([float(v) for v in vals[: 9 * n]], np.float32).reshape(n, 9)


def walls_from_rows(rows: np.ndarray):
    """(start4, mid4, end4, normal4) arrays as WallGroupData stores them, with
    mid = 0.5 * (start + end) (WallGroupData.cu:87-89)."""
    n = rows.shape[0]
    start = np.zeros((n, 4), np.float32)
    end = np.zeros((n, 4), np.float32)
    normal = np.zeros((n, 4), np.float32)
    start[:, :3] = rows[:, 0:3]
    end[:, :3] = rows[:, 3:6]
    normal[:, :3] = rows[:, 6:9]
    mid = np.zeros((n, 4), np.float32)
    mid[:, :3] = np.float32(0.5) * (start[:, :3] + end[:, :3])
    return start, mid, end, normal


# ---- step parameters -----------------------------------------------------------

B_AVOID_WALLS, B_AVOID_NEIGHBORS, B_SEPARATION, B_ALIGNMENT, B_COHESION, B_SEEK = 1, 2, 3, 4, 5, 6
B_FOLLOW_PATH = 7
WRAP_REFERENCE, WRAP_SYMMETRIC, WRAP_NONE = 0, 1, 2
KNN_BINNED, KNN_BRUTEFORCE = 0, 1


@dataclass
class StepParams:
    """Everything one step needs; field meanings follow SimulationParams
    (include/OpenSteer/Simulation.h:64-117) and the plugin update functions."""

    world_size: tuple = (160.0, 160.0, 160.0)
    world_cells: tuple = (40, 40, 40)
    search_radius: int = 1
    wrap_mode: int = WRAP_SYMMETRIC
    knn_mode: int = KNN_BINNED
    k: int = 7
    clear_applied: int = 0
    knw: int = 3
    min_time_to_wall: float = 5.0
    w_walls: float = 1.0
    mask_walls: int = 0
    min_time_to_collision: float = 2.0
    min_separation_distance: float = 1.0
    avoid_close: int = 0
    w_avoid: float = 1.0
    mask_avoid: int = 0
    sep_min: float = 0.5
    sep_max: float = 2.0
    sep_cos: float = -0.98480775301220805936674302458952
    w_sep: float = 5.0
    mask_sep: int = 0
    ali_min: float = 0.5
    ali_max: float = 7.0
    ali_cos: float = -0.98480775301220805936674302458952
    w_ali: float = 8.0
    mask_ali: int = 0
    coh_min: float = 0.5
    coh_max: float = 7.0
    coh_cos: float = -0.98480775301220805936674302458952
    w_coh: float = 4.0
    mask_coh: int = 0
    seek_target: tuple = (0.0, 0.0, 0.0)
    w_seek: float = 1.0
    mask_seek: int = 0
    order: tuple = (B_SEPARATION, B_COHESION, B_ALIGNMENT)
    dt: float = 1.0 / 60.0
    # path following (ChokePoint.params: pathPredictionTime, weightFollowPath,
    # maskFollowPath); the path itself is passed beside the parameters
    path_prediction_time: float = 3.0
    w_path: float = 1.0
    mask_path: int = 0

    def replace(self, **kw) -> "StepParams":
        d = dict(self.__dict__)
        d.update(kw)
        return StepParams(**d)


def boids_params(k: int = 7, world: float = 160.0, cell: float = 4.0, masks: bool = False,
                 knn_mode: int = KNN_BINNED) -> StepParams:
    """Plain 3D flock (plugins/BoidsGroup.cpp:606-637: separation, cohesion,
    alignment, update) with the distances of data/BoidsGroup.params:13-17,
    weights 5/8/4 (separation/alignment/cohesion) and symmetric wrapping."""
    c = int(round(world / cell))
    p = StepParams(world_size=(world, world, world), world_cells=(c, c, c), k=k,
                   knn_mode=knn_mode, order=(B_SEPARATION, B_COHESION, B_ALIGNMENT),
                   dt=1.0 / 60.0)
    if masks:  # data/BoidsGroup.params:43-44
        p = p.replace(mask_ali=16, mask_coh=16)
    return p


def chokepoint_params(k: int = 16, knw: int = 3, world: float = 512.0, cell: float = 2.0,
                      goal=(0.0, 0.0, -93.5)) -> StepParams:
    """2D choke point: avoid walls, avoid neighbours, separation, seek, update,
    with the values of data/ChokePoint.params:3-55 and dt = 1/30
    (plugins/ChokePointNew.cpp:692)."""
    c = int(round(world / cell))
    return StepParams(
        world_size=(world, 10.0, world), world_cells=(c, 1, c), search_radius=1,
        wrap_mode=WRAP_REFERENCE, k=k, knw=knw, clear_applied=1,
        min_time_to_wall=10.0, w_walls=1.0, mask_walls=0,
        min_time_to_collision=2.0, min_separation_distance=0.5, avoid_close=0,
        w_avoid=1.0, mask_avoid=0,
        sep_min=0.5, sep_max=1.2, sep_cos=-0.86602540378443864676372317075294, w_sep=10.0,
        mask_sep=KERNEL_ANTI_PENETRATION_WALL,
        seek_target=tuple(goal), w_seek=1.5, mask_seek=4480,
        order=(B_AVOID_WALLS, B_AVOID_NEIGHBORS, B_SEPARATION, B_SEEK), dt=1.0 / 30.0)


# ---- .params reader (src/Simulation.cpp:7-250) ---------------------------------

_SIM_KEYS = {
    "seed": int, "knn": int, "kno": int, "knw": int, "searchRadius": int,
    "maxPursuitPredictionTime": float, "minTimeToCollision": float,
    "minTimeToObstacle": float, "minTimeToWall": float, "pathPredictionTime": float,
    "minSeparationDistance": float, "maxSeparationDistance": float,
    "minFlockingDistance": float, "maxFlockingDistance": float,
    "cosMaxFlockingAngle": float, "avoidCloseNeighbors": int,
    "weightAlignment": float, "weightCohesion": float, "weightSeparation": float,
    "weightPursuit": float, "weightSeek": float, "weightFollowPath": float,
    "weightAvoidObstacles": float, "weightAvoidWalls": float, "weightAvoidNeighbors": float,
    "maskAlignment": int, "maskAntiPenetrationAgents": int, "maskCohesion": int,
    "maskSeparation": int, "maskSeek": int, "maskFlee": int, "maskPursuit": int,
    "maskEvade": int, "maskFollowPath": int, "maskAvoidObstacles": int,
    "maskAvoidWalls": int, "maskAvoidNeighbors": int,
}


@dataclass
class SimulationParams:
    values: dict = field(default_factory=dict)
    world: dict = field(default_factory=dict)
    groups: list = field(default_factory=list)


class ParamsError(ValueError):
    pass


def load_params(text: str) -> SimulationParams:
    """Parse the whitespace key/value format.  Like the reference, a token that
    starts with '#' comments out the rest of its line and an unknown key is an
    error (the reference asserts)."""
    lines = text.splitlines()
    toks = []
    for line in lines:
        for t in line.split():
            if t.startswith("#"):
                break
            toks.append(t)
    out = SimulationParams()
    i = 0

    def take(n):
        nonlocal i
        v = toks[i:i + n]
        if len(v) < n:
            raise ParamsError("unexpected end of file")
        i += n
        return v

    while i < len(toks):
        key = take(1)[0]
        if key == "</simulation>":
            break
        if key == "<world>":
            while True:
                k2 = take(1)[0]
                if k2 == "</world>":
                    break
                take(1)  # delimiter
                if k2 == "dimensions":
                    out.world["dimensions"] = tuple(float(v) for v in take(3))
                elif k2 == "cells":
                    out.world["cells"] = tuple(int(v) for v in take(3))
                elif k2 == "obstacleCount":
                    out.world["obstacleCount"] = int(take(1)[0])
                elif k2 == "mapFilename":
                    out.world["mapFilename"] = take(1)[0]
                else:
                    raise ParamsError(f"unknown world key {k2!r}")
            continue
        if key == "<group>":
            g = {"path": []}
            while True:
                k2 = take(1)[0]
                if k2 == "</group>":
                    break
                if k2 == "<path>":
                    while True:
                        k3 = take(1)[0]
                        if k3 == "</path>":
                            break
                        take(1)
                        if k3 == "point":
                            g["path"].append(tuple(float(v) for v in take(3)))
                        elif k3 == "cyclic":
                            g["cyclic"] = int(take(1)[0])
                        elif k3 == "radius":
                            g["pathRadius"] = float(take(1)[0])
                        else:
                            raise ParamsError(f"unknown path key {k3!r}")
                    continue
                take(1)
                if k2 == "numAgents":
                    g["numAgents"] = int(take(1)[0])
                elif k2 == "startPosition":
                    g["startPosition"] = tuple(float(v) for v in take(3))
                elif k2 in ("minStartRadius", "maxStartRadius", "maxSpeed", "maxForce"):
                    g[k2] = float(take(1)[0])
                elif k2 == "bodyColor":
                    g["bodyColor"] = tuple(float(v) for v in take(3))
                else:
                    raise ParamsError(f"unknown group key {k2!r}")
            out.groups.append(g)
            continue
        if key == "<simulation>":
            continue
        take(1)  # delimiter
        if key not in _SIM_KEYS:
            raise ParamsError(f"unknown key {key!r}")
        out.values[key] = _SIM_KEYS[key](take(1)[0])
    return out


def params_from_file(sim: SimulationParams, dt: float) -> StepParams:
    """The flock step a BoidsGroup plugin runs for a parsed .params file."""
    v = sim.values
    dims = sim.world.get("dimensions", (160.0, 160.0, 160.0))
    cells = sim.world.get("cells", (40, 40, 40))
    cos = v.get("cosMaxFlockingAngle", -0.98480775301220805936674302458952)
    return StepParams(
        world_size=dims, world_cells=cells, search_radius=v.get("searchRadius", 1),
        k=v.get("knn", 7), knw=v.get("knw", 3),
        sep_min=v.get("minFlockingDistance", 0.5), sep_max=v.get("maxSeparationDistance", 2.0),
        sep_cos=cos, w_sep=v.get("weightSeparation", 1.0), mask_sep=v.get("maskSeparation", 0),
        ali_min=v.get("minFlockingDistance", 0.5), ali_max=v.get("maxFlockingDistance", 7.0),
        ali_cos=cos, w_ali=v.get("weightAlignment", 1.0), mask_ali=v.get("maskAlignment", 0),
        coh_min=v.get("minFlockingDistance", 0.5), coh_max=v.get("maxFlockingDistance", 7.0),
        coh_cos=cos, w_coh=v.get("weightCohesion", 1.0), mask_coh=v.get("maskCohesion", 0),
        dt=dt)


def chokepoint_new_from_file(sim: SimulationParams, dt: float = 1.0 / 30.0, group: int = 0):
    """CtfGroup::update (plugins/ChokePointNew.cpp:586-630) with a parsed
    .params file: (StepParams, path points, path radius, cyclic).  Walls,
    separation (mask KERNEL_ANTI_PENETRATION_WALL, as the plugin passes it,
    :615), alignment, cohesion, follow path, seek the path's second point;
    the closing antiPenetrationAgents takes maskAntiPenetrationAgents."""
    v, w, g = sim.values, sim.world, sim.groups[group]
    pts = [tuple(float(c) for c in q) for q in g["path"]]
    if len(pts) < 2:
        raise ParamsError("the group needs a path of at least two points")
    cos = v["cosMaxFlockingAngle"]
    p = StepParams(
        world_size=tuple(w["dimensions"]), world_cells=tuple(w["cells"]),
        search_radius=v["searchRadius"], wrap_mode=WRAP_REFERENCE, k=v["knn"], knw=v["knw"],
        clear_applied=1,
        min_time_to_wall=v["minTimeToWall"], w_walls=v["weightAvoidWalls"],
        mask_walls=v["maskAvoidWalls"],
        sep_min=v["minSeparationDistance"], sep_max=v["maxSeparationDistance"], sep_cos=cos,
        w_sep=v["weightSeparation"], mask_sep=KERNEL_ANTI_PENETRATION_WALL,
        ali_min=v["minFlockingDistance"], ali_max=v["maxFlockingDistance"], ali_cos=cos,
        w_ali=v["weightAlignment"], mask_ali=v["maskAlignment"],
        coh_min=v["minFlockingDistance"], coh_max=v["maxFlockingDistance"], coh_cos=cos,
        w_coh=v["weightCohesion"], mask_coh=v["maskCohesion"],
        seek_target=pts[1], w_seek=v["weightSeek"], mask_seek=v["maskSeek"],
        path_prediction_time=v["pathPredictionTime"], w_path=v["weightFollowPath"],
        mask_path=v["maskFollowPath"],
        order=(B_AVOID_WALLS, B_SEPARATION, B_ALIGNMENT, B_COHESION, B_FOLLOW_PATH, B_SEEK),
        dt=dt)
    return p, pts, float(g.get("pathRadius", 0.0)), bool(g.get("cyclic", 0))


CHOKEPOINT_GAPS = (7.5, 10.0, 12.5, 15.0, 17.5, 20.0, 22.5, 25.0, 27.5, 30.0, 32.5)


def batched_chokepoint(n_scenes: int = 256, seed: int = 0, n_range=(1000, 20000),
                       gaps=CHOKEPOINT_GAPS):
    """Independent choke-point scenes: per scene s, a gap half-width drawn
    uniformly from `gaps` (the data/ChokePoint{X}.map set) and an agent count
    uniform in n_range, agents seeded with hash_seed(seed, s).
    Returns (states, gaps_per_scene)."""
    u = uniform01(seed ^ 0xB47C4, 2 * n_scenes).reshape(n_scenes, 2).astype(np.float64)
    lo, hi = n_range
    counts = (lo + np.floor(u[:, 0] * (hi - lo + 1))).astype(np.int64).clip(lo, hi)
    picks = np.floor(u[:, 1] * len(gaps)).astype(np.int64).clip(0, len(gaps) - 1)
    states = [chokepoint_agents(int(counts[s]), seed=hash_seed(seed, s)) for s in range(n_scenes)]
    return states, [float(gaps[i]) for i in picks]


def default_steps(name: str) -> int:
    return {"boids": 100, "chokepoint": 500, "large": 1000, "batched": 300, "adjoint": 64,
            "brute": 20}[name]


def isqrt_cells(world: float, cell: float) -> int:
    return int(math.floor(world / cell + 0.5))
