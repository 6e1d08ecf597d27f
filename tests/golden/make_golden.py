"""Generate the golden fixtures in this directory from the reference itself.

Runs PsychoLogicAu/GPUSteer's own CUDA kernel sources, compiled for the CPU by
oracle/ref (make -C oracle/ref REF=<reference tree>), on seeded inputs and
stores inputs and outputs as .npz files.  The fixtures pin the CPU oracle
(tests/test_oracle_golden.py) and, through it, the sm_103a kernels.

Usage:  python tests/golden/make_golden.py [--ref /path/to/GPUSteer]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "tests"))

from gpusteer_gb300 import scenario as sc  # noqa: E402
from gpusteer_gb300.state import AgentState  # noqa: E402
import oracle_lib as ol  # noqa: E402

fp = lambda a: ol.ptr(a)  # noqa: E731
up = lambda a: ol.ptr(a, C.c_uint)  # noqa: E731


def save(name, meta, **arrays):
    np.savez_compressed(HERE / f"{name}.npz", meta=np.array(json.dumps(meta)), **arrays)
    print("wrote", name, {k: v.shape for k, v in arrays.items()})


def state_arrays(prefix, s: AgentState):
    return {f"{prefix}{k}": np.array(v, copy=True) for k, v in s.arrays().items()}


def ref_knn_binned(ref, posA, posB, self_, ws, wc, r, k):
    nA, nB = posA.shape[0], posB.shape[0]
    idx = np.empty(k * nA, np.uint32)
    dist = np.empty(k * nA, np.float32)
    rc = ref.gsref_knn_binned(fp(posA), nA, fp(posB), nB, int(self_), ol.f3(ws), ol.u3(wc), r, k,
                              up(idx), fp(dist))
    assert rc == 0, rc
    return idx, dist


def ref_knn_brute(ref, posA, posB, self_, k):
    nA, nB = posA.shape[0], posB.shape[0]
    idx = np.empty(k * nA, np.uint32)
    dist = np.empty(k * nA, np.float32)
    assert ref.gsref_knn_brute(fp(posA), nA, fp(posB), nB, int(self_), k, up(idx), fp(dist)) == 0
    return idx, dist


def pos_uniform(seed, n, lo, hi, dims=3):
    u = sc.uniform01(seed, 3 * n).reshape(n, 3)
    p = np.zeros((n, 4), np.float32)
    lo, hi = np.asarray(lo, np.float32), np.asarray(hi, np.float32)
    p[:, :3] = lo + u * (hi - lo)
    if dims == 2:
        p[:, 1] = 0
    return p


def knn_cases(ref):
    # 3D, self, k = 7 and a cross-group case; some agents outside the world.
    ws, wc = (64.0, 64.0, 64.0), (16, 16, 16)
    pa = pos_uniform(11, 1500, (-34, -34, -34), (34, 34, 34))
    i1, d1 = ref_knn_binned(ref, pa, pa, True, ws, wc, 1, 7)
    pb = pos_uniform(12, 400, (-30, -30, -30), (30, 30, 30))
    pc = pos_uniform(13, 700, (-30, -30, -30), (30, 30, 30))
    i2, d2 = ref_knn_binned(ref, pc, pb, False, ws, wc, 1, 5)
    save("knn_binned_3d", {"ws": ws, "wc": wc, "r": 1, "k_self": 7, "k_cross": 5},
         pos_self=pa, idx_self=i1, dist_self=d1, pos_a=pc, pos_b=pb, idx_cross=i2, dist_cross=d2)
    # 2D, k = 16 with search radius 1 and 2.
    ws2, wc2 = (128.0, 10.0, 128.0), (64, 1, 64)
    p2 = pos_uniform(21, 1500, (-60, 0, -60), (60, 0, 60), dims=2)
    i3, d3 = ref_knn_binned(ref, p2, p2, True, ws2, wc2, 1, 16)
    i4, d4 = ref_knn_binned(ref, p2, p2, True, ws2, wc2, 2, 16)
    save("knn_binned_2d", {"ws": ws2, "wc": wc2, "k": 16},
         pos=p2, idx_r1=i3, dist_r1=d3, idx_r2=i4, dist_r2=d4)
    # brute force.
    p5 = pos_uniform(31, 1000, (-20, -20, -20), (20, 20, 20))
    i5, d5 = ref_knn_brute(ref, p5, p5, True, 16)
    p6 = pos_uniform(32, 300, (-20, -20, -20), (20, 20, 20))
    i6, d6 = ref_knn_brute(ref, p5[:500].copy(), p6, False, 7)
    save("knn_brute", {"k_self": 16, "k_cross": 7}, pos=p5, idx_self=i5, dist_self=d5,
         pos_b=p6, idx_cross=i6, dist_cross=d6)


def g_args(s: AgentState):
    return s.position, s.direction, s.steering, s.applied


def flock_case(ref):
    """Separation, cohesion and alignment one kernel at a time, then update,
    on a dense 3D flock, with and without masks."""
    s0 = sc.boids_sphere(1024, radius=9.0, seed=5)
    s0.applied[:] = (sc.uniform01(77, s0.n) < 0.2).astype(np.uint32) * 16
    ws, wc, k = (64.0, 64.0, 64.0), (16, 16, 16), 7
    idx, dist = ref_knn_binned(ref, s0.position, s0.position, True, ws, wc, 1, k)
    s = s0.copy()
    n = s.n
    cos = np.float32(-0.98480775301220805936674302458952)
    ref.gsref_separation(fp(s.position), fp(s.direction), fp(s.steering), up(s.applied), n,
                         up(idx), k, fp(s.position), n, C.c_float(0.5), C.c_float(2.0),
                         C.c_float(cos), C.c_float(5.0), 0)
    after_sep = s.copy()
    ref.gsref_cohesion(fp(s.position), fp(s.direction), fp(s.steering), up(s.applied), n, up(idx),
                       k, fp(s.position), n, C.c_float(0.5), C.c_float(7.0), C.c_float(cos),
                       C.c_float(4.0), 16)
    after_coh = s.copy()
    ref.gsref_alignment(fp(s.position), fp(s.direction), fp(s.steering), up(s.applied), n, up(idx),
                        k, fp(s.position), fp(s.direction), n, C.c_float(0.5), C.c_float(7.0),
                        C.c_float(cos), C.c_float(8.0), 16)
    after_ali = s.copy()
    ref.gsref_seek(fp(s.position), fp(s.direction), fp(s.steering), up(s.applied), n,
                   ol.f3((3.0, -2.0, 1.0)), C.c_float(1.5), 64)
    after_seek = s.copy()
    ref.gsref_update(fp(s.side), fp(s.up), fp(s.direction), fp(s.position), fp(s.steering),
                     fp(s.speed), fp(s.max_force), fp(s.max_speed), fp(s.mass),
                     C.c_float(1.0 / 60.0), n, up(s.applied))
    after_update = s.copy()
    w = s.copy()
    w.position[:, :3] = pos_uniform(8, n, (-120, -120, -120), (120, 120, 120))[:, :3]
    wrap_in = w.copy()
    ref.gsref_wrap(fp(w.position), ol.f3((160.0, 160.0, 160.0)), n)
    save("flock_stages", {"ws": ws, "wc": wc, "k": k, "seek_target": [3.0, -2.0, 1.0]},
         knn_idx=idx, knn_dist=dist, **state_arrays("in_", s0), **state_arrays("sep_", after_sep),
         **state_arrays("coh_", after_coh), **state_arrays("ali_", after_ali),
         **state_arrays("seek_", after_seek), **state_arrays("upd_", after_update),
         wrap_in=wrap_in.position, wrap_out=w.position)


def choke_walls(gap, ws, wc):
    rows = sc.chokepoint_walls(gap)
    st, mid, en, nm = sc.walls_from_rows(rows)
    return ol.split_walls(st, mid, en, nm, ws, wc)


def avoid_case(ref):
    """Avoid walls and avoid neighbours (with and without the close-neighbour
    pass) on agents around a choke point, and anti-penetration after update."""
    ws, wc = (128.0, 10.0, 128.0), (64, 1, 64)
    walls = choke_walls(10.0, ws, wc)
    n = 1200
    s0 = sc.chokepoint_agents(n, x_range=(-30, 30), z_range=(-25, 40), seed=3)
    s0.speed[:] = sc.uniform01(99, n) * np.float32(3.0)
    k, kw = 16, 3
    idx, dist = ref_knn_binned(ref, s0.position, s0.position, True, ws, wc, 1, k)
    widx, wdist = ref_knn_binned(ref, s0.position, walls[1], False, ws, wc, 1, kw)
    out = {}
    s = s0.copy()
    ref.gsref_avoid_walls(fp(s.position), fp(s.direction), fp(s.side), fp(s.speed), fp(s.radius),
                          fp(s.steering), up(s.applied), n, up(widx), kw, fp(walls[0]),
                          fp(walls[2]), fp(walls[3]), walls[0].shape[0], C.c_float(10.0),
                          C.c_float(1.0), 0)
    out.update(state_arrays("walls_", s))
    for close in (0, 1):
        s = s0.copy()
        ref.gsref_avoid_neighbors(fp(s.position), fp(s.direction), fp(s.side), fp(s.speed),
                                  fp(s.radius), fp(s.steering), up(s.applied), n, up(idx),
                                  fp(dist), k, fp(s.position), fp(s.direction), fp(s.speed),
                                  fp(s.radius), n, C.c_float(2.0), C.c_float(0.5), close,
                                  C.c_float(1.0), 0)
        out.update(state_arrays(f"avoid{close}_", s))
    # Anti-penetration (AntiPenetrationAgentsCUDAKernel.cu:57-109) on a
    # crowded copy; masked agents have bit 12 set.
    s = s0.copy()
    s.applied[:] = (sc.uniform01(5, n) < 0.3).astype(np.uint32) * 4096
    ap_in = s.copy()
    ref.gsref_antipenetration_agents(fp(s.position), fp(s.radius), n, up(idx), fp(dist), k,
                                     fp(s0.position), fp(s.radius), up(ap_in.applied), n,
                                     up(s.applied), 4096)
    save("avoid_stages", {"ws": ws, "wc": wc, "k": k, "knw": kw, "min_time_wall": 10.0,
                          "min_time": 2.0, "min_sep": 0.5},
         knn_idx=idx, knn_dist=dist, knw_idx=widx, knw_dist=wdist, wall_start=walls[0],
         wall_mid=walls[1], wall_end=walls[2], wall_normal=walls[3], **state_arrays("in_", s0),
         **out, ap_in_applied=ap_in.applied, ap_out_position=s.position,
         ap_out_applied=s.applied)


def wall_antipen_case(ref):
    """updateGroupWithAntiPenetration (UpdateCUDAKernelNew.cu:95-268) and
    antiPenetrationWall (AntiPenetrationWallCUDAKernel.cu:52-134) on agents
    moving at and along the choke point's walls.  Both kernels read the wall
    list row-major; each runs on the wall KNN as findKNearestNeighbors writes
    it (column-major) and on its transpose, with which every agent tests its
    own nearest walls."""
    ws, wc = (128.0, 10.0, 128.0), (64, 1, 64)
    walls = choke_walls(10.0, ws, wc)
    nl = walls[0].shape[0]
    n = 1500
    s0 = sc.chokepoint_agents(n, x_range=(-24, 24), z_range=(-16, 16), seed=61)
    u = sc.uniform01(62, 4 * n).reshape(4, n)
    s0.speed[:] = u[0] * np.float32(4.0)
    s0.steering[:, 0] = (u[1] - np.float32(0.5)) * np.float32(6.0)
    s0.steering[:, 2] = (u[2] - np.float32(0.5)) * np.float32(6.0)
    s0.radius[:] = np.float32(0.3) + u[3] * np.float32(0.6)
    s0.applied[:] = (u[3] < 0.25).astype(np.uint32) * 256
    kw, dt = 4, 0.5
    widx, _ = ref_knn_binned(ref, s0.position, walls[1], False, ws, wc, 1, kw)
    widx_t = np.ascontiguousarray(widx.reshape(kw, n).T).ravel()
    out = {}
    for name, knl in (("col", widx), ("row", widx_t)):
        s = s0.copy()
        rc = ref.gsref_update_antipen_wall(
            fp(s.side), fp(s.up), fp(s.direction), fp(s.position), fp(s.steering), fp(s.speed),
            fp(s.max_force), fp(s.max_speed), fp(s.mass), fp(s.radius), up(knl), kw,
            fp(walls[0]), fp(walls[2]), fp(walls[3]), nl, C.c_float(dt), n, up(s.applied))
        assert rc == 0
        out.update(state_arrays(f"upd_{name}_", s))
        s = s0.copy()
        rc = ref.gsref_antipenetration_wall(
            fp(s.position), fp(s.direction), fp(s.speed), up(knl), kw, fp(walls[0]),
            fp(walls[2]), fp(walls[3]), nl, C.c_float(dt), n, up(s.applied))
        assert rc == 0
        out.update(state_arrays(f"apw_{name}_", s))
    save("wall_antipen", {"ws": ws, "wc": wc, "knw": kw, "dt": dt},
         knw_col=widx, knw_row=widx_t, wall_start=walls[0], wall_mid=walls[1],
         wall_end=walls[2], wall_normal=walls[3], **state_arrays("in_", s0), **out)


def flock_steps(ref):
    """20 whole flock steps (KNN, separation, cohesion, alignment, update),
    each kernel the reference's, composed as BoidsGroup::update."""
    p = sc.boids_params(k=7, world=64.0, cell=4.0)
    s = sc.boids_sphere(600, radius=10.0, seed=9)
    s_in = s.copy()
    n, k = s.n, p.k
    for _ in range(20):
        idx, dist = ref_knn_binned(ref, s.position, s.position, True, p.world_size,
                                   p.world_cells, 1, k)
        ref.gsref_separation(fp(s.position), fp(s.direction), fp(s.steering), up(s.applied), n,
                             up(idx), k, fp(s.position), n, C.c_float(p.sep_min),
                             C.c_float(p.sep_max), C.c_float(p.sep_cos), C.c_float(p.w_sep), 0)
        ref.gsref_cohesion(fp(s.position), fp(s.direction), fp(s.steering), up(s.applied), n,
                           up(idx), k, fp(s.position), n, C.c_float(p.coh_min),
                           C.c_float(p.coh_max), C.c_float(p.coh_cos), C.c_float(p.w_coh), 0)
        ref.gsref_alignment(fp(s.position), fp(s.direction), fp(s.steering), up(s.applied), n,
                            up(idx), k, fp(s.position), fp(s.direction), n, C.c_float(p.ali_min),
                            C.c_float(p.ali_max), C.c_float(p.ali_cos), C.c_float(p.w_ali), 0)
        ref.gsref_update(fp(s.side), fp(s.up), fp(s.direction), fp(s.position), fp(s.steering),
                         fp(s.speed), fp(s.max_force), fp(s.max_speed), fp(s.mass),
                         C.c_float(p.dt), n, up(s.applied))
    save("flock_steps", {"steps": 20, "world": 64.0, "cell": 4.0, "k": 7},
         **state_arrays("in_", s_in), **state_arrays("out_", s), knn_idx=idx, knn_dist=dist)


def choke_steps(ref):
    """20 whole choke-point steps: wrap (reference mode), KNN, wall KNN, avoid
    walls, separation, seek, update (ChokePointNew.cpp:586-630 without path
    following)."""
    ws, wc = (128.0, 10.0, 128.0), (64, 1, 64)
    walls = choke_walls(10.0, ws, wc)
    p = sc.chokepoint_params(world=128.0, cell=2.0)
    s = sc.chokepoint_agents(700, x_range=(-20, 20), z_range=(2, 30), seed=4)
    # Non-zero initial speeds: UpdateCUDAKernel writes an uninitialised side
    # vector for agents whose new speed is 0 (UpdateCUDAKernel.cu:75,114).
    s.speed[:] = np.float32(0.5) + sc.uniform01(44, s.n) * np.float32(2.5)
    s_in = s.copy()
    n, k, kw = s.n, p.k, p.knw
    for _ in range(20):
        ref.gsref_wrap(fp(s.position), ol.f3(ws), n)
        s.applied[:] = 0
        idx, dist = ref_knn_binned(ref, s.position, s.position, True, ws, wc, 1, k)
        widx, _ = ref_knn_binned(ref, s.position, walls[1], False, ws, wc, 1, kw)
        ref.gsref_avoid_walls(fp(s.position), fp(s.direction), fp(s.side), fp(s.speed),
                              fp(s.radius), fp(s.steering), up(s.applied), n, up(widx), kw,
                              fp(walls[0]), fp(walls[2]), fp(walls[3]), walls[0].shape[0],
                              C.c_float(p.min_time_to_wall), C.c_float(p.w_walls), 0)
        ref.gsref_separation(fp(s.position), fp(s.direction), fp(s.steering), up(s.applied), n,
                             up(idx), k, fp(s.position), n, C.c_float(p.sep_min),
                             C.c_float(p.sep_max), C.c_float(p.sep_cos), C.c_float(p.w_sep),
                             p.mask_sep)
        ref.gsref_seek(fp(s.position), fp(s.direction), fp(s.steering), up(s.applied), n,
                       ol.f3(p.seek_target), C.c_float(p.w_seek), p.mask_seek)
        ref.gsref_update(fp(s.side), fp(s.up), fp(s.direction), fp(s.position), fp(s.steering),
                         fp(s.speed), fp(s.max_force), fp(s.max_speed), fp(s.mass),
                         C.c_float(p.dt), n, up(s.applied))
    save("choke_steps", {"steps": 20, "world": 128.0, "cell": 2.0},
         **state_arrays("in_", s_in), **state_arrays("out_", s), wall_start=walls[0],
         wall_mid=walls[1], wall_end=walls[2], wall_normal=walls[3])


PATH_CASES = [
    # name, points, radius, cyclic, prediction time, weight, mask
    ("line", [(0.0, 0.0, 13.5), (0.0, 0.0, -1650.0)], 20.0, 0, 5.0, 1.0, 16),  # ChokePoint.params
    ("loop", [(-40.0, 0.0, -40.0), (40.0, 0.0, -40.0), (40.0, 0.0, 40.0), (-40.0, 0.0, 40.0)],
     6.0, 1, 2.0, 1.5, 0),
    ("bend", [(0.0, 0.0, 100.0), (0.0, 0.0, 0.0), (60.0, 0.0, -30.0), (60.0, 0.0, -200.0)],
     4.0, 0, -1.0, 1.0, 0),
]


def path_case(ref):
    """FollowPathCUDAKernel on 2D crowds around three paths: the choke
    point's straight path, a cyclic square and a bent path followed with a
    negative prediction time; some agents masked, some at speed 0."""
    for ci, (name, pts, radius, cyclic, pt, w, mask) in enumerate(PATH_CASES):
        s = sc.chokepoint_agents(1500, x_range=(-70.0, 70.0), z_range=(-120.0, 140.0),
                                 seed=40 + ci)
        u = sc.uniform01(50 + ci, 3 * s.n).reshape(3, s.n)
        s.speed[:] = np.where(u[0] < 0.05, 0.0, 3.0 * u[1]).astype(np.float32)
        s.steering[:, :3] = (sc.uniform01(60 + ci, 3 * s.n).reshape(s.n, 3) - 0.5).astype(np.float32)
        s.applied[:] = np.where(u[2] < 0.25, 16, 0).astype(np.uint32)
        P = ol.path_init(pts, radius, cyclic)
        po, ln, nm, tot = P.arrays
        po, ln, nm = np.ascontiguousarray(po), np.ascontiguousarray(ln), np.ascontiguousarray(nm)
        out = s.copy()
        ref.gsref_follow_path(fp(out.position), fp(out.direction), fp(out.speed), fp(out.steering),
                              up(out.applied), out.n, fp(po), fp(ln), fp(nm), int(P.n),
                              C.c_float(radius), int(cyclic), C.c_float(tot), C.c_float(pt),
                              C.c_float(w), mask)
        save(f"path_{name}", {"points": pts, "radius": radius, "cyclic": cyclic,
                              "prediction_time": pt, "weight": w, "mask": mask},
             path_points=po, path_lengths=ln, path_normals=nm,
             path_total=np.array([tot], np.float32), **state_arrays("in_", s),
             out_steering=out.steering, out_applied=out.applied)


def cell_diag_case(ref):
    """ExtractData's ComputeCellDensity / ComputeAvgCellVelocity
    (ProcessData.cu:51-237) on the reference's database: a 2D crowd (some
    agents outside the world, clamped into edge cells) and a 3D flock."""
    arrays = {}
    cases = {
        "crowd2d": (sc.chokepoint_agents(3000, seed=21), (128.0, 10.0, 128.0), (64, 1, 64), 5),
        "flock3d": (sc.boids_sphere(4000, radius=20.0, seed=24), (64.0, 64.0, 64.0),
                    (16, 16, 16), 6),
    }
    meta = {}
    for name, (s, ws, wc, sseed) in cases.items():
        s.speed[:] = (sc.uniform01(sseed, s.n) * 3.0).astype(np.float32)
        if name == "crowd2d":
            s.position[:40, 0] = np.float32(70.0)  # beyond the +x face
        C_ = wc[0] * wc[1] * wc[2]
        dens = np.empty(C_, np.uint32)
        vel = np.empty((C_, 3), np.float32)
        rc = ref.gsref_cell_diagnostics(fp(s.position), fp(s.direction), fp(s.speed), s.n,
                                        ol.f3(ws), ol.u3(wc), up(dens), fp(vel))
        assert rc == 0, rc
        assert dens.max() >= 4
        arrays.update({f"{name}_position": s.position, f"{name}_direction": s.direction,
                       f"{name}_speed": s.speed, f"{name}_density": dens,
                       f"{name}_avg_velocity": vel})
        meta[name] = {"ws": ws, "wc": wc}
    save("cell_diag", meta, **arrays)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=str(ol.reference_root()))
    ap.add_argument("--only", nargs="*", default=None, help="case functions to run")
    a = ap.parse_args()
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle" / "ref"), f"REF={a.ref}"], check=True)
    ref = ol.ref_harness()
    assert ref is not None
    cases = [knn_cases, flock_case, avoid_case, flock_steps, choke_steps, path_case,
             wall_antipen_case, cell_diag_case]
    for case in cases:
        if a.only is None or case.__name__ in a.only:
            case(ref)


if __name__ == "__main__":
    main()
