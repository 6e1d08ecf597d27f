"""The CPU oracle against golden vectors produced by the reference's own
kernel sources (tests/golden/make_golden.py).  CPU only.

Expected exceptions, each a documented oracle decision:
* binned KNN breaks exact distance ties by agent index (the reference by cell
  visit order); the fixtures are random, so no ties occur and the check is
  exact;
* avoid-neighbours, "parallel" branch: the reference reads an uninitialised
  threat position, so agents that took that branch are excluded;
* update with a new speed of 0 keeps the side vector (the reference writes
  uninitialised shared memory); those agents' side vectors are excluded.
"""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as ol
from gpusteer_gb300 import scenario as sc
from gpusteer_gb300.state import AgentState

GOLD = Path(__file__).resolve().parent / "golden"


def load(name):
    z = np.load(GOLD / f"{name}.npz")
    return z, json.loads(str(z["meta"]))


def state(z, prefix) -> AgentState:
    return AgentState(**{k: np.array(z[prefix + k], copy=True) for k in AgentState.names()})


def assert_state_equal(got: AgentState, want: AgentState, exclude_side=None):
    for k in AgentState.names():
        a, b = getattr(got, k), getattr(want, k)
        if k == "side" and exclude_side is not None:
            a, b = a[~exclude_side], b[~exclude_side]
        np.testing.assert_array_equal(a, b, err_msg=k)


def test_knn_binned_3d_matches_reference():
    z, m = load("knn_binned_3d")
    i, d = ol.knn_binned(z["pos_self"], z["pos_self"], True, m["ws"], m["wc"], m["r"], m["k_self"])
    np.testing.assert_array_equal(i, z["idx_self"])
    np.testing.assert_array_equal(d, z["dist_self"])
    i, d = ol.knn_binned(z["pos_a"], z["pos_b"], False, m["ws"], m["wc"], m["r"], m["k_cross"])
    np.testing.assert_array_equal(i, z["idx_cross"])
    np.testing.assert_array_equal(d, z["dist_cross"])


def test_knn_binned_2d_matches_reference():
    z, m = load("knn_binned_2d")
    for r in (1, 2):
        i, d = ol.knn_binned(z["pos"], z["pos"], True, m["ws"], m["wc"], r, m["k"])
        np.testing.assert_array_equal(i, z[f"idx_r{r}"])
        np.testing.assert_array_equal(d, z[f"dist_r{r}"])


def test_knn_brute_matches_reference():
    z, m = load("knn_brute")
    i, d = ol.knn_brute(z["pos"], z["pos"], True, m["k_self"])
    np.testing.assert_array_equal(i, z["idx_self"])
    np.testing.assert_array_equal(d, z["dist_self"])
    i, d = ol.knn_brute(z["pos"][:500].copy(), z["pos_b"], False, m["k_cross"])
    np.testing.assert_array_equal(i, z["idx_cross"])
    np.testing.assert_array_equal(d, z["dist_cross"])


def test_flocking_stages_match_reference():
    z, m = load("flock_stages")
    o = ol.oracle()
    s = state(z, "in_")
    g = ol.group_struct(s)
    idx, k = z["knn_idx"], m["k"]
    cos = C.c_float(-0.98480775301220805936674302458952)
    o.orc_steer_separation(C.byref(g), ol.ptr(idx, C.c_uint), k, ol.ptr(s.position), s.n,
                           C.c_float(0.5), C.c_float(2.0), cos, C.c_float(5.0), 0)
    assert_state_equal(s, state(z, "sep_"))
    o.orc_steer_cohesion(C.byref(g), ol.ptr(idx, C.c_uint), k, ol.ptr(s.position), s.n,
                         C.c_float(0.5), C.c_float(7.0), cos, C.c_float(4.0), 16)
    assert_state_equal(s, state(z, "coh_"))
    o.orc_steer_alignment(C.byref(g), ol.ptr(idx, C.c_uint), k, ol.ptr(s.position),
                          ol.ptr(s.direction), s.n, C.c_float(0.5), C.c_float(7.0), cos,
                          C.c_float(8.0), 16)
    assert_state_equal(s, state(z, "ali_"))
    o.orc_steer_seek(C.byref(g), ol.f3(m["seek_target"]), C.c_float(1.5), 64)
    assert_state_equal(s, state(z, "seek_"))
    o.orc_update(C.byref(g), C.c_float(1.0 / 60.0))
    want = state(z, "upd_")
    assert_state_equal(s, want, exclude_side=want.speed == 0)
    w = AgentState.zeros(s.n)
    w.position[:] = z["wrap_in"]
    o.orc_wrap_world(C.byref(ol.group_struct(w)), ol.f3((160.0, 160.0, 160.0)), sc.WRAP_REFERENCE)
    np.testing.assert_array_equal(w.position, z["wrap_out"])


def test_avoid_stages_match_reference():
    z, m = load("avoid_stages")
    o = ol.oracle()
    walls = ol.walls_struct(z["wall_start"], z["wall_mid"], z["wall_end"], z["wall_normal"])
    s = state(z, "in_")
    o.orc_steer_avoid_walls(C.byref(ol.group_struct(s)), ol.ptr(z["knw_idx"], C.c_uint), m["knw"],
                            C.byref(walls), C.c_float(m["min_time_wall"]), C.c_float(1.0), 0)
    assert_state_equal(s, state(z, "walls_"))
    want0 = state(z, "walls_")
    assert (want0.applied & 4096).any() and (want0.applied & 256).any()
    for close in (0, 1):
        s = state(z, "in_")
        branch = np.zeros(s.n, np.uint32)
        o.orc_steer_avoid_neighbors_dbg(
            C.byref(ol.group_struct(s)), ol.ptr(z["knn_idx"], C.c_uint), ol.ptr(z["knn_dist"]),
            m["k"], ol.ptr(s.position), ol.ptr(s.direction), ol.ptr(s.speed), ol.ptr(s.radius),
            s.n, C.c_float(m["min_time"]), C.c_float(m["min_sep"]), close, C.c_float(1.0), 0,
            ol.ptr(branch, C.c_uint))
        want = state(z, f"avoid{close}_")
        keep = branch != 2
        if close:
            # Agents whose close-neighbour steering fired leave the main kernel
            # before its coalesced side-vector read (CUDAKernelGlobals.cuh:35-46,
            # SteerToAvoidNeighborsCUDAKernel.cu:265,291): in full blocks, float
            # f of the block's side vectors is loaded by thread f % 256, so an
            # agent's side is garbage in the reference when a loader exited.
            exited = (want.applied & 1024) != 0
            full = (s.n // 256) * 256
            t = np.arange(full) % 256
            base = np.arange(full) - t
            loaders = [base + (3 * t + j) % 256 for j in range(3)]
            stale = np.zeros(s.n, bool)
            stale[:full] = exited[loaders[0]] | exited[loaders[1]] | exited[loaders[2]]
            keep &= ~stale | exited
        else:
            assert keep.sum() > 0.5 * s.n
            assert (branch == 1).any() and (branch == 3).any()
        for k in AgentState.names():
            np.testing.assert_array_equal(getattr(s, k)[keep], getattr(want, k)[keep], err_msg=k)
        if close:
            assert (want.applied & 1024).any()


def test_agent_antipenetration_matches_reference():
    """antiPenetrationAgents on the choke-point crowd, a third of it masked."""
    z, m = load("avoid_stages")
    s = state(z, "in_")
    s.applied[:] = z["ap_in_applied"]
    pos_b, rad_b, app_b = s.position.copy(), s.radius.copy(), s.applied.copy()
    ol.oracle().orc_antipenetration_agents(
        C.byref(ol.group_struct(s)), ol.ptr(z["knn_idx"], C.c_uint), ol.ptr(z["knn_dist"]),
        ol.ptr(pos_b), ol.ptr(rad_b), ol.ptr(app_b, C.c_uint), s.n, 4096)
    np.testing.assert_array_equal(s.position, z["ap_out_position"])
    np.testing.assert_array_equal(s.applied, z["ap_out_applied"])
    assert ((s.applied & 8192) != 0).sum() > 20


def test_wall_antipenetration_matches_reference():
    """updateGroupWithAntiPenetration and antiPenetrationWall, bit for bit,
    on the wall KNN as written (column-major) and on its transpose."""
    z, m = load("wall_antipen")
    o = ol.oracle()
    walls = ol.walls_struct(z["wall_start"], z["wall_mid"], z["wall_end"], z["wall_normal"])
    for layout in ("col", "row"):
        knl = ol.ptr(z[f"knw_{layout}"], C.c_uint)
        s = state(z, "in_")
        o.orc_update_with_antipenetration(C.byref(ol.group_struct(s)), knl, m["knw"],
                                          C.byref(walls), C.c_float(m["dt"]))
        want = state(z, f"upd_{layout}_")
        assert (want.speed > 0).all()
        assert_state_equal(s, want)
        s = state(z, "in_")
        o.orc_antipenetration_wall(C.byref(ol.group_struct(s)), knl, m["knw"], C.byref(walls),
                                   C.c_float(m["dt"]))
        assert_state_equal(s, state(z, f"apw_{layout}_"))
    # the transposed lists reach the walls: both kernels fire on many agents
    assert ((z["upd_row_applied"] & 4096) != 0).sum() > 50
    assert ((z["apw_row_applied"] & 4096) != 0).sum() > 30


def test_flock_steps_match_reference():
    z, m = load("flock_steps")
    s = state(z, "in_")
    p = sc.boids_params(k=m["k"], world=m["world"], cell=m["cell"]).replace(wrap_mode=sc.WRAP_NONE)
    idx, dist = ol.run(s, p, m["steps"], want_knn=True)
    want = state(z, "out_")
    assert_state_equal(s, want, exclude_side=want.speed == 0)
    np.testing.assert_array_equal(idx, z["knn_idx"])
    np.testing.assert_array_equal(dist, z["knn_dist"])


def test_choke_steps_match_reference():
    z, m = load("choke_steps")
    s = state(z, "in_")
    p = sc.chokepoint_params(world=m["world"], cell=m["cell"]).replace(
        order=(sc.B_AVOID_WALLS, sc.B_SEPARATION, sc.B_SEEK))
    walls = (z["wall_start"], z["wall_mid"], z["wall_end"], z["wall_normal"])
    ol.run(s, p, m["steps"], walls=walls)
    want = state(z, "out_")
    assert_state_equal(s, want, exclude_side=want.speed == 0)


def test_wall_split_is_cell_bounded():
    ws, wc = (128.0, 10.0, 128.0), (64, 1, 64)
    st, mid, en, nm = sc.walls_from_rows(sc.chokepoint_walls(10.0))
    s2, m2, e2, n2 = ol.split_walls(st, mid, en, nm, ws, wc)
    assert s2.shape[0] > st.shape[0]
    # each split piece inside the world spans at most one cell per axis
    step = 2.0
    inside = (np.abs(s2[:, 0]) < 60) & (np.abs(s2[:, 2]) < 60) & (np.abs(e2[:, 0]) < 60) & (np.abs(e2[:, 2]) < 60)
    assert inside.any()
    span = np.abs(s2[inside, :3] - e2[inside, :3])
    assert (span[:, [0, 2]] <= step + 1e-3).all()
    np.testing.assert_array_equal(n2[:, 3], 0)


@pytest.mark.parametrize("gap", ["7.5", "10", "20", "32.5"])
def test_chokepoint_map_generator_matches_reference_files(gap):
    path = ol.reference_root() / "data" / f"ChokePoint{gap}.map"
    if not path.exists():
        pytest.skip("reference data not mounted")
    np.testing.assert_array_equal(sc.read_map(str(path)), sc.chokepoint_walls(float(gap)))


# ---- path following (SteerToFollowPathCUDAKernel.cu, PolylinePathwayCUDA.cu) ----------

def fixture_path(z, m):
    P = ol.OrcPath()
    po = np.ascontiguousarray(z["path_points"])
    ln = np.ascontiguousarray(z["path_lengths"])
    nm = np.ascontiguousarray(z["path_normals"])
    P.points, P.lengths, P.normals = ol.ptr(po), ol.ptr(ln), ol.ptr(nm)
    P.n, P.radius, P.cyclic = po.shape[0], m["radius"], m["cyclic"]
    P.total_length = float(z["path_total"][0])
    P._keep = (po, ln, nm)
    return P


@pytest.mark.parametrize("name", ["line", "loop", "bend"])
def test_follow_path_matches_reference(name):
    z, m = load(f"path_{name}")
    s = state(z, "in_")
    ol.oracle().orc_steer_follow_path(C.byref(ol.group_struct(s)), C.byref(fixture_path(z, m)),
                                      C.c_float(m["prediction_time"]), C.c_float(m["weight"]),
                                      m["mask"])
    np.testing.assert_array_equal(s.steering, z["out_steering"])
    np.testing.assert_array_equal(s.applied, z["out_applied"])
    assert (s.applied & (1 << 11)).any(), "no agent steered"


@pytest.mark.parametrize("name", ["line", "loop", "bend"])
def test_path_initialize_restates_the_pathway(name):
    """PolylinePathwayCUDA::Initialize: segment vectors, their lengths
    (sqrt of the dot product) and unit normals, in binary32."""
    z, m = load(f"path_{name}")
    P = ol.path_init(m["points"], m["radius"], m["cyclic"])
    po, ln, nm, tot = P.arrays
    pts = np.array(m["points"], np.float32)
    if m["cyclic"]:
        pts = np.concatenate([pts, pts[:1]])
    np.testing.assert_array_equal(po, pts)
    seg = (pts[1:] - pts[:-1]).astype(np.float32)
    lens = np.sqrt((seg[:, 0] * seg[:, 0] + seg[:, 1] * seg[:, 1]) + seg[:, 2] * seg[:, 2])
    np.testing.assert_array_equal(ln[1:], lens)
    np.testing.assert_array_equal(nm[1:], seg / lens[:, None])
    total = np.float32(0)
    for v in lens:
        total = np.float32(total + v)
    assert np.float32(tot) == total
    np.testing.assert_array_equal(po, z["path_points"])


# ---- ExtractData diagnostics (ProcessData.cu:132-237) ---------------------------------

@pytest.mark.parametrize("case", ["crowd2d", "flock3d"])
def test_cell_diagnostics_match_reference_golden(case):
    """Agents per cell and mean cell velocity against the reference's own
    ComputeCellDensityKernel / ComputeAvgCellVelocityKernel run on its own
    database (tests/golden/cell_diag.npz), bit for bit."""
    z, m = load("cell_diag")
    ws, wc = m[case]["ws"], m[case]["wc"]
    pos = z[f"{case}_position"]
    np.testing.assert_array_equal(ol.cell_density(pos, ws, wc), z[f"{case}_density"])
    got = ol.cell_avg_velocity(pos, z[f"{case}_direction"], z[f"{case}_speed"], ws, wc)
    np.testing.assert_array_equal(got.reshape(-1, 3), z[f"{case}_avg_velocity"])


def test_cell_diagnostics_restate_processdata():
    """Agents per cell and the mean cell velocity, summed in ascending agent
    index (the stable sort's order) in binary32, against a plain loop."""
    s = sc.chokepoint_agents(3000, seed=21)
    s.speed[:] = (sc.uniform01(5, s.n) * 3.0).astype(np.float32)
    ws, wc = (128.0, 10.0, 128.0), (64, 1, 64)
    cells = ol.cell_index(s.position, ws, wc)
    dens = ol.cell_density(s.position, ws, wc)
    np.testing.assert_array_equal(dens, np.bincount(cells, minlength=64 * 64))
    avg = ol.cell_avg_velocity(s.position, s.direction, s.speed, ws, wc)
    acc = np.zeros((64 * 64, 3), np.float32)
    for i in range(s.n):
        acc[cells[i]] = (acc[cells[i]] + s.direction[i, :3] * s.speed[i]).astype(np.float32)
    want = np.zeros_like(acc)
    nz = dens > 0
    want[nz] = acc[nz] / dens[nz].astype(np.float32)[:, None]
    np.testing.assert_array_equal(avg, want)
    assert dens.max() >= 5
