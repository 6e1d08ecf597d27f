"""sm_103a kernels against the CPU oracle and the reference's golden vectors,
through the C ABI.  Bit-exact: every result is compared with
np.testing.assert_array_equal (KNN indices and distances, forces, state)."""
import json
from pathlib import Path

import numpy as np
import pytest

import gpusteer_gb300 as gs
import oracle_lib as ol
from gpusteer_gb300 import scenario as sc
from gpusteer_gb300.state import AgentState

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def load(name):
    z = np.load(GOLD / f"{name}.npz")
    return z, json.loads(str(z["meta"]))


def gstate(z, prefix):
    return AgentState(**{k: np.array(z[prefix + k], copy=True) for k in AgentState.names()})


def assert_state(got: AgentState, want: AgentState, skip_side=None, fields=None):
    for k in fields or AgentState.names():
        a, b = getattr(got, k), getattr(want, k)
        if k == "side" and skip_side is not None:
            a, b = a[~skip_side], b[~skip_side]
        np.testing.assert_array_equal(a, b, err_msg=k)


def group_of(s: AgentState, k=16):
    g = gs.AgentGroup(k, max(1, s.n))
    g.upload(s)
    return g


def pos_state(pos4):
    s = AgentState.zeros(pos4.shape[0])
    s.position[:] = pos4
    return s


# ---- KNN ----------------------------------------------------------------------------

def gpu_knn_binned(posA, posB, self_, ws, wc, r, k):
    bins = gs.KNNBinData(wc, ws, r)
    A = group_of(pos_state(posA), k)
    gs.updateKNNDatabase(A, bins)
    if self_:
        B = A
    else:
        B = group_of(pos_state(posB), k)
        gs.updateKNNDatabase(B, bins)
    knn = gs.KNNData(posA.shape[0], k)
    gs.findKNearestNeighbors(A, knn, bins, B, r)
    return knn.download(A)


def test_knn_binned_matches_reference_golden_3d():
    z, m = load("knn_binned_3d")
    i, d = gpu_knn_binned(z["pos_self"], z["pos_self"], True, m["ws"], m["wc"], 1, m["k_self"])
    np.testing.assert_array_equal(i, z["idx_self"])
    np.testing.assert_array_equal(d, z["dist_self"])
    i, d = gpu_knn_binned(z["pos_a"], z["pos_b"], False, m["ws"], m["wc"], 1, m["k_cross"])
    np.testing.assert_array_equal(i, z["idx_cross"])
    np.testing.assert_array_equal(d, z["dist_cross"])


def test_knn_binned_matches_reference_golden_2d():
    z, m = load("knn_binned_2d")
    for r in (1, 2):
        i, d = gpu_knn_binned(z["pos"], z["pos"], True, m["ws"], m["wc"], r, m["k"])
        np.testing.assert_array_equal(i, z[f"idx_r{r}"])
        np.testing.assert_array_equal(d, z[f"dist_r{r}"])


@pytest.mark.parametrize("k", [1, 7, 16, 24, 33, 64])
def test_knn_binned_matches_oracle_all_k(k):
    p = sc.boids_sphere(3000, radius=20.0, seed=k).position
    ws, wc = (64.0, 64.0, 64.0), (16, 16, 16)
    i, d = gpu_knn_binned(p, p, True, ws, wc, 1, k)
    oi, od = ol.knn_binned(p, p, True, ws, wc, 1, k)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


def test_knn_ties_break_by_lower_index():
    # integer lattice with duplicated points: many exactly equal distances
    g = np.stack(np.meshgrid(np.arange(6), np.arange(6), np.arange(6), indexing="ij"), -1)
    g = g.reshape(-1, 3).astype(np.float32) - 3.0
    pts = np.concatenate([g, g[::7]])  # duplicates at distance 0
    p = np.zeros((pts.shape[0], 4), np.float32)
    p[:, :3] = pts
    ws, wc = (16.0, 16.0, 16.0), (8, 8, 8)
    for k in (6, 16):
        i, d = gpu_knn_binned(p, p, True, ws, wc, 1, k)
        oi, od = ol.knn_binned(p, p, True, ws, wc, 1, k)
        np.testing.assert_array_equal(i, oi)
        np.testing.assert_array_equal(d, od)
        bi, bd = ol.knn_brute(p, p, True, k)
        # every agent has its 26-neighbourhood inside the 27-cell box here only
        # for interior agents; compare those with brute force
        n = p.shape[0]
        sel = (np.abs(pts) <= 1).all(1)
        for s in range(k):
            np.testing.assert_array_equal(i[s * n:(s + 1) * n][sel], bi[s * n:(s + 1) * n][sel])


def test_knn_edge_cases():
    ws, wc = (32.0, 32.0, 32.0), (8, 8, 8)
    # fewer candidates than k: padding is (UINT_MAX, FLT_MAX); agents outside
    # the world clamp into the edge cells.
    p = np.array([[0, 0, 0, 0], [1, 0, 0, 0], [100, 100, 100, 0], [-100, 5, 5, 0],
                  [15.9, 15.9, 15.9, 0]], np.float32)
    i, d = gpu_knn_binned(p, p, True, ws, wc, 1, 8)
    oi, od = ol.knn_binned(p, p, True, ws, wc, 1, 8)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)
    assert (i == 0xFFFFFFFF).sum() > 0 and (d[i == 0xFFFFFFFF] == np.finfo(np.float32).max).all()
    # a single agent
    i, d = gpu_knn_binned(p[:1], p[:1], True, ws, wc, 1, 4)
    assert (i == 0xFFFFFFFF).all()


def test_knn_bruteforce_matches_reference_golden():
    z, m = load("knn_brute")
    A = group_of(pos_state(z["pos"]))
    knn = gs.KNNData(A.size, m["k_self"])
    gs.findKNearestNeighborsBruteForce(A, knn, A)
    i, d = knn.download(A)
    np.testing.assert_array_equal(i, z["idx_self"])
    np.testing.assert_array_equal(d, z["dist_self"])
    A2 = group_of(pos_state(z["pos"][:500].copy()))
    B2 = group_of(pos_state(z["pos_b"]))
    knn2 = gs.KNNData(500, m["k_cross"])
    gs.findKNearestNeighborsBruteForce(A2, knn2, B2)
    i, d = knn2.download(A2)
    np.testing.assert_array_equal(i, z["idx_cross"])
    np.testing.assert_array_equal(d, z["dist_cross"])


def test_knn_bruteforce_matches_oracle_larger():
    p = sc.boids_cube(20000, size=128.0, seed=4).position
    A = group_of(pos_state(p))
    for k in (7, 16):
        knn = gs.KNNData(A.size, k)
        gs.findKNearestNeighborsBruteForce(A, knn, A)
        i, d = knn.download(A)
        oi, od = ol.knn_brute(p, p, True, k)
        np.testing.assert_array_equal(i, oi)
        np.testing.assert_array_equal(d, od)
        # the bucketed scan skips most chunks of candidates
        assert 0 < gs.bruteforce_pairs(A) < A.size * A.size // 4


@pytest.mark.parametrize("k", [1, 8, 16, 24, 32, 33, 40, 64])
def test_knn_bruteforce_sizes_ties_and_cross_groups(k):
    """Group sizes that are not multiples of the 64-query block or of the
    eight candidate slices, an integer lattice with duplicated points (exact
    distance ties, broken by the lower index), and a cross-group search; k
    past 32 keeps two list entries per lane."""
    rng = np.random.default_rng(k)
    g3 = np.stack(np.meshgrid(np.arange(9), np.arange(9), np.arange(9), indexing="ij"), -1)
    lat = g3.reshape(-1, 3).astype(np.float32) - 4.0
    lat = np.concatenate([lat, lat[::3]])                 # 972 points, duplicates
    pa = np.zeros((lat.shape[0], 4), np.float32)
    pa[:, :3] = lat
    pb = np.zeros((1999, 4), np.float32)
    pb[:, :3] = rng.uniform(-6, 6, (1999, 3)).astype(np.float32)
    A, B = group_of(pos_state(pa)), group_of(pos_state(pb))
    for (G, O, P, Q, self_) in ((A, A, pa, pa, True), (A, B, pa, pb, False), (B, A, pb, pa, False)):
        knn = gs.KNNData(G.size, k)
        gs.findKNearestNeighborsBruteForce(G, knn, O)
        i, d = knn.download(G)
        oi, od = ol.knn_brute(P, Q, self_, k)
        np.testing.assert_array_equal(i, oi)
        np.testing.assert_array_equal(d, od)


@pytest.mark.parametrize("k", [8, 16, 32, 48, 64])
def test_knn_bruteforce_seeded_large_groups(k):
    """Groups of 4,096 and more take the seeded filter (k-th distance of a
    binned search on an automatic grid): a lattice with duplicates (ties), a
    flat 2D crowd, and a cross-group search with queries outside the other
    group's extent all give the oracle's lists."""
    g3 = np.stack(np.meshgrid(np.arange(17), np.arange(17), np.arange(17), indexing="ij"), -1)
    lat = g3.reshape(-1, 3).astype(np.float32) - 8.0
    lat = np.concatenate([lat, lat[::7]])
    pa = np.zeros((lat.shape[0], 4), np.float32)
    pa[:, :3] = lat
    crowd = sc.chokepoint_agents(6000, seed=k).position.copy()
    rng = np.random.default_rng(k)
    pb = np.zeros((5000, 4), np.float32)
    pb[:, :3] = rng.uniform(-30, 30, (5000, 3)).astype(np.float32)
    pb[:2000, 0] += 100.0
    for P, Q, self_ in ((pa, pa, True), (crowd, crowd, True), (pb, pa, False), (pa, pb, False)):
        A = group_of(pos_state(P))
        B = A if self_ else group_of(pos_state(Q))
        knn = gs.KNNData(A.size, k)
        gs.findKNearestNeighborsBruteForce(A, knn, B)
        i, d = knn.download(A)
        oi, od = ol.knn_brute(P, Q, self_, k)
        np.testing.assert_array_equal(i, oi)
        np.testing.assert_array_equal(d, od)
        # a second call reuses the seed databases
        gs.findKNearestNeighborsBruteForce(A, knn, B)
        i2, d2 = knn.download(A)
        np.testing.assert_array_equal(i2, oi)


def test_knn_bruteforce_fewer_candidates_than_k():
    pa = np.zeros((70, 4), np.float32)
    pa[:, 0] = np.arange(70, dtype=np.float32)
    pb = pa[:5].copy()
    A, B = group_of(pos_state(pa)), group_of(pos_state(pb))
    knn = gs.KNNData(70, 16)
    gs.findKNearestNeighborsBruteForce(A, knn, B)
    i, d = knn.download(A)
    oi, od = ol.knn_brute(pa, pb, False, 16)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)
    assert (i.reshape(16, 70)[5:] == 0xFFFFFFFF).all()
    assert gs.bruteforce_pairs(A) == 70 * 5  # a small call scans every pair


# ---- behaviours, one per launch -----------------------------------------------------

def test_flocking_stages_match_reference_golden():
    z, m = load("flock_stages")
    s = gstate(z, "in_")
    g = group_of(s, m["k"])
    knn = gs.KNNData(s.n, m["k"])
    # use the reference's own KNN result for the stage inputs
    bins = gs.KNNBinData(m["wc"], m["ws"], 1)
    gs.updateKNNDatabase(g, bins)
    gs.findKNearestNeighbors(g, knn, bins, g, 1)
    i, _ = knn.download(g)
    np.testing.assert_array_equal(i, z["knn_idx"])
    cos = -0.98480775301220805936674302458952
    gs.steerForSeparation(g, knn, g, 0.5, 2.0, cos, 5.0, 0)
    assert_state(g.download(), gstate(z, "sep_"))
    gs.steerForCohesion(g, knn, g, 0.5, 7.0, cos, 4.0, 16)
    assert_state(g.download(), gstate(z, "coh_"))
    gs.steerForAlignment(g, knn, g, 0.5, 7.0, cos, 8.0, 16)
    assert_state(g.download(), gstate(z, "ali_"))
    gs.steerForSeek(g, m["seek_target"], 1.5, 64)
    assert_state(g.download(), gstate(z, "seek_"))
    gs.updateGroup(g, 1.0 / 60.0)
    want = gstate(z, "upd_")
    assert_state(g.download(), want, skip_side=want.speed == 0)
    w = AgentState.zeros(s.n)
    w.position[:] = z["wrap_in"]
    gw = group_of(w)
    gs.wrapWorld(gw, (160.0, 160.0, 160.0), sc.WRAP_REFERENCE)
    np.testing.assert_array_equal(gw.download().position, z["wrap_out"])


def test_avoid_stages_match_oracle_on_golden_inputs():
    z, m = load("avoid_stages")
    s0 = gstate(z, "in_")
    n, k, kw = s0.n, m["k"], m["knw"]
    rows = np.concatenate([z["wall_start"][:, :3], z["wall_end"][:, :3],
                           z["wall_normal"][:, :3]], 1)
    walls = gs.WallGroup(rows, bins=None, knw=kw)  # already split
    bins = gs.KNNBinData(m["wc"], m["ws"], 1)
    g = group_of(s0, k)
    gs.updateKNNDatabase(g, bins)
    knw = gs.KNNData(n, kw)
    gs.findKNearestNeighbors(g, knw, bins, walls, 1)
    wi, wd = knw.download(g)
    np.testing.assert_array_equal(wi, z["knw_idx"])
    np.testing.assert_array_equal(wd, z["knw_dist"])
    gs.steerToAvoidWalls(g, knw, walls, m["min_time_wall"], 1.0, 0)
    assert_state(g.download(), gstate(z, "walls_"))
    for close in (0, 1):
        g = group_of(s0, k)
        gs.updateKNNDatabase(g, bins)
        knn = gs.KNNData(n, k)
        gs.findKNearestNeighbors(g, knn, bins, g, 1)
        gs.steerToAvoidNeighbors(g, knn, g, m["min_time"], m["min_sep"], close, 1.0, 0)
        want = s0.copy()
        ol.oracle().orc_steer_avoid_neighbors(
            ol.C.byref(ol.group_struct(want)), ol.ptr(z["knn_idx"], ol.C.c_uint),
            ol.ptr(z["knn_dist"]), k, ol.ptr(s0.position), ol.ptr(s0.direction),
            ol.ptr(s0.speed), ol.ptr(s0.radius), n, ol.C.c_float(m["min_time"]),
            ol.C.c_float(m["min_sep"]), close, ol.C.c_float(1.0), 0)
        assert_state(g.download(), want)
    # anti-penetration (the next ChokePoint stage)
    g = group_of(s0, k)
    st = s0.copy()
    st.applied[:] = z["ap_in_applied"]
    g.upload(st)
    gs.updateKNNDatabase(g, bins)
    knn = gs.KNNData(n, k)
    gs.findKNearestNeighbors(g, knn, bins, g, 1)
    gs.antiPenetrationAgents(g, knn, g, 4096)
    out = g.download()
    np.testing.assert_array_equal(out.position, z["ap_out_position"])
    np.testing.assert_array_equal(out.applied, z["ap_out_applied"])


def test_wall_antipenetration_matches_reference_golden():
    """updateGroupWithAntiPenetration and antiPenetrationWall against the
    reference kernels' outputs, bit for bit: on the wall lists as
    findKNearestNeighbors writes them (found here on the GPU) and on their
    transpose (uploaded), both read row-major as the reference kernels do."""
    z, m = load("wall_antipen")
    s0 = gstate(z, "in_")
    n, kw, dt = s0.n, m["knw"], m["dt"]
    rows = np.concatenate([z["wall_start"][:, :3], z["wall_end"][:, :3],
                           z["wall_normal"][:, :3]], 1)
    walls = gs.WallGroup(rows, bins=None, knw=kw)  # already split
    bins = gs.KNNBinData(m["wc"], m["ws"], 1)
    calls = {"upd": lambda g, knw: gs.updateGroupWithAntiPenetration(g, knw, walls, dt),
             "apw": lambda g, knw: gs.antiPenetrationWall(g, knw, walls, dt, 0)}
    for layout in ("col", "row"):
        for name, call in calls.items():
            g = group_of(s0)
            knw = gs.KNNData(n, kw)
            if layout == "col":
                gs.updateKNNDatabase(g, bins)
                gs.findKNearestNeighbors(g, knw, bins, walls, 1)
                np.testing.assert_array_equal(knw.download(g)[0], z["knw_col"])
            else:
                knw.upload(z["knw_row"], None, g)
                np.testing.assert_array_equal(knw.download(g)[0], z["knw_row"])
            call(g, knw)
            assert_state(g.download(), gstate(z, f"{name}_{layout}_"))


def test_wall_split_matches_oracle():
    for gap in (7.5, 10.0, 32.5):
        for ws, wc in (((128.0, 10.0, 128.0), (64, 1, 64)), ((512.0, 10.0, 512.0), (256, 1, 256))):
            bins = gs.KNNBinData(wc, ws, 1)
            w = gs.WallGroup(sc.chokepoint_walls(gap), bins=bins, knw=3)
            got = w.download()
            want = ol.split_walls(*sc.walls_from_rows(sc.chokepoint_walls(gap)), ws, wc)
            for a, b in zip(got, want):
                np.testing.assert_array_equal(a, b)


# ---- whole steps --------------------------------------------------------------------

def dropin_flock_step(g, knn, bins, p: sc.StepParams):
    gs.wrapWorld(g, p.world_size, p.wrap_mode)
    gs.updateKNNDatabase(g, bins)
    gs.findKNearestNeighbors(g, knn, bins, g, p.search_radius)
    for b in p.order:
        if b == sc.B_SEPARATION:
            gs.steerForSeparation(g, knn, g, p.sep_min, p.sep_max, p.sep_cos, p.w_sep, p.mask_sep)
        elif b == sc.B_COHESION:
            gs.steerForCohesion(g, knn, g, p.coh_min, p.coh_max, p.coh_cos, p.w_coh, p.mask_coh)
        elif b == sc.B_ALIGNMENT:
            gs.steerForAlignment(g, knn, g, p.ali_min, p.ali_max, p.ali_cos, p.w_ali, p.mask_ali)
    gs.updateGroup(g, p.dt)


def test_flock_steps_match_reference_golden():
    z, m = load("flock_steps")
    s = gstate(z, "in_")
    p = sc.boids_params(k=m["k"], world=m["world"], cell=m["cell"]).replace(wrap_mode=sc.WRAP_NONE)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    want = gstate(z, "out_")
    # drop-in sequence
    g = group_of(s, p.k)
    knn = gs.KNNData(s.n, p.k)
    for _ in range(m["steps"]):
        dropin_flock_step(g, knn, bins, p)
    assert_state(g.download(), want, skip_side=want.speed == 0)
    # fused
    g2 = group_of(s, p.k)
    gs.step(g2, bins, None, p, m["steps"])
    assert_state(g2.download(), want, skip_side=want.speed == 0)


def test_choke_steps_match_reference_golden():
    z, m = load("choke_steps")
    s = gstate(z, "in_")
    p = sc.chokepoint_params(world=m["world"], cell=m["cell"]).replace(
        order=(sc.B_AVOID_WALLS, sc.B_SEPARATION, sc.B_SEEK))
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    rows = np.concatenate([z["wall_start"][:, :3], z["wall_end"][:, :3],
                           z["wall_normal"][:, :3]], 1)
    walls = gs.WallGroup(rows, bins=None, knw=p.knw)
    g = group_of(s, p.k)
    gs.step(g, bins, walls, p, m["steps"])
    want = gstate(z, "out_")
    assert_state(g.download(), want, skip_side=want.speed == 0)


@pytest.mark.parametrize("masks", [False, True])
def test_boids_config_fused_matches_oracle(masks):
    """4,096 3D boids, k = 7, cell 4.0, 100 steps (bins), bit-exact."""
    s = sc.boids_sphere(4096, seed=0)
    p = sc.boids_params(k=7, masks=masks)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    g = group_of(s, p.k)
    gs.step(g, bins, None, p, 100)
    want = s.copy()
    ol.run(want, p, 100)
    assert_state(g.download(), want, skip_side=want.speed == 0)


@pytest.mark.parametrize("capacity", [32, 64, 128, 256])
def test_fused_step_on_a_lattice_with_exact_ties(capacity):
    """Agents on an integer lattice, some duplicated: many neighbours at
    exactly equal distances, so the KNN order depends on the index
    tie-break (the fused kernels' exact fallback path), for the collecting
    (32, 64) and streaming (128, 256) scans."""
    g3 = np.stack(np.meshgrid(np.arange(12), np.arange(12), np.arange(12), indexing="ij"), -1)
    pts = g3.reshape(-1, 3).astype(np.float32) - 6.0
    pts = np.concatenate([pts, pts[::5]])
    s = sc.boids_sphere(pts.shape[0], seed=3)
    s.position[:, :3] = pts
    for k in (7, 16, 20):
        p = sc.boids_params(k=k, world=64.0, cell=2.0)
        bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
        g = group_of(s, p.k)
        gs.set_knn_capacity(g, capacity)
        gs.step(g, bins, None, p, 3)
        want = s.copy()
        ol.run(want, p, 3)
        assert_state(g.download(), want, skip_side=want.speed == 0)


@pytest.mark.parametrize("capacity", [0, 32, 64, 128, 256])
def test_knn_capacity_does_not_change_results(capacity):
    """Dense 2D crowds (4 and 8 agents per cell, 36 and 72 candidates on
    average) overflow the small capacities into the exact redo; every
    capacity gives the oracle's result bit for bit."""
    p = sc.chokepoint_params()
    bins, walls = choke_walls(p)
    for n in (10000, 20000):
        s = sc.chokepoint_agents(n, seed=5)
        g = group_of(s, p.k)
        gs.set_knn_capacity(g, capacity)
        gs.step(g, bins, walls, p, 20)
        want = s.copy()
        ol.run(want, p, 20, walls=walls.download())
        assert_state(g.download(), want, skip_side=want.speed == 0)


@pytest.mark.parametrize("case", ["lattice_past_list_cap", "crowd_warp_lists", "clump_thread_lists"])
def test_exact_redo_routes(case):
    """Every route of the exact redo after the streaming scan (capacity 128)
    gives the oracle's result bit for bit: lists found by one warp per agent
    (boxes of up to 256 candidates), lists left to the redo's own thread
    (larger boxes), and redo entries past the 16,384 stored lists (a
    27,000-agent lattice, 216 candidates per box: every agent overflows into
    the redo), with and without walls.  The collecting scans' redo (capacity
    32 and 64, no stored lists) is covered by the lattice test above."""
    if case == "lattice_past_list_cap":
        g3 = np.stack(np.meshgrid(*(np.arange(30),) * 3, indexing="ij"), -1)
        pts = g3.reshape(-1, 3).astype(np.float32) - 15.0
        s = sc.boids_sphere(pts.shape[0], seed=4)
        s.position[:, :3] = pts
        p = sc.boids_params(k=16, world=64.0, cell=2.0)
        bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
        g = group_of(s, p.k)
        gs.set_knn_capacity(g, 128)
        gs.step(g, bins, None, p, 2)
        want = s.copy()
        ol.run(want, p, 2)
    else:
        # 4,000 agents in a square: about 20 per cell (184 candidates, past
        # the streaming scan's 128) or 40 per cell (360, past the warp's 256)
        p = sc.chokepoint_params()
        bins, walls = choke_walls(p)
        half = 10.0 if case == "clump_thread_lists" else 14.0
        s = sc.chokepoint_agents(4000, x_range=(-half, half), z_range=(20.0, 20.0 + 2 * half),
                                 seed=6)
        g = group_of(s, p.k)
        gs.set_knn_capacity(g, 128)
        gs.step(g, bins, walls, p, 3)
        want = s.copy()
        ol.run(want, p, 3, walls=walls.download())
    assert_state(g.download(), want, skip_side=want.speed == 0)


def test_knn_capacity_reads_back():
    """The capacity a step used: the fixed one, or the measured choice
    (streaming scan for a dense crowd, collecting scan for a sparse flock);
    the step's launch count follows it."""
    p = sc.chokepoint_params()
    bins, walls = choke_walls(p)
    g = group_of(sc.chokepoint_agents(10000, seed=5), p.k)
    assert gs.knn_capacity(g) == 0
    gs.step(g, bins, walls, p, 1)
    assert gs.knn_capacity(g) in (128, 256)
    # scan, permute, wall phase, warp-per-agent lists, rest phase
    assert gs.step_launches(g, True) == 5
    gs.set_knn_capacity(g, 64)
    assert gs.knn_capacity(g) == 64
    assert gs.step_launches(g, True) == 4
    s = sc.boids_sphere(4096, seed=0)
    pb = sc.boids_params(k=7)
    fb = group_of(s, pb.k)
    gs.step(fb, gs.KNNBinData(pb.world_cells, pb.world_size, 1), None, pb, 1)
    assert gs.knn_capacity(fb) in (32, 64)
    assert gs.step_launches(fb, False) == 3


@pytest.mark.parametrize("cell,want", [(2.0, 128), (3.0, 256)])
def test_knn_capacity_follows_the_dense_scenes_of_a_batch(cell, want):
    """The automatic capacity weighs cells by their agents: a batch whose
    densest scenes see more than 128 candidates per box (cell 3.0) takes the
    256-candidate scan, the same scenes at cell 2.0 the 128-candidate one."""
    states, gaps = sc.batched_chokepoint(24, seed=0)
    p = sc.chokepoint_params(cell=cell)
    b = gs.Batch([s.n for s in states], p.k, p.world_cells, p.world_size, p.search_radius)
    for i, gap in enumerate(gaps):
        b.set_walls(i, sc.chokepoint_walls(gap))
    b.upload(AgentState.concat(states))
    b.step(p, 1)
    assert gs.knn_capacity(b.group) == want


@pytest.mark.parametrize("capacity", [128, 256])
def test_flat_streaming_scan_without_walls(capacity):
    """A 2D crowd (grid one cell high) without walls: the 3-row build of the
    streaming scan in the single fused kernel gives the oracle's result."""
    p = sc.chokepoint_params().replace(order=(sc.B_AVOID_NEIGHBORS, sc.B_SEPARATION, sc.B_SEEK))
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    s = sc.chokepoint_agents(10000, seed=9)
    g = group_of(s, p.k)
    gs.set_knn_capacity(g, capacity)
    gs.step(g, bins, None, p, 10)
    want = s.copy()
    ol.run(want, p, 10)
    assert_state(g.download(), want, skip_side=want.speed == 0)


@pytest.mark.parametrize("wide", [False, True])
def test_scan_over_tiles_near_agents(wide):
    """The step's scan writes starts only for the cell tiles within reach of
    agents.  A flock in one corner of a large grid leaves most tiles empty
    and unwritten; on a grid whose box spans more tiles than a block can
    test (1024 x 4 x 1024 cells: y rows are a million labels apart) every
    tile is written.  Both against the oracle over the steps' moves across
    tiles."""
    if wide:
        p = sc.boids_params(k=16, world=2048.0, cell=2.0).replace(
            world_size=(2048.0, 8.0, 2048.0), world_cells=(1024, 4, 1024))
        s = sc.boids_sphere(4096, radius=30.0, seed=12)
        s.position[:, 1] *= np.float32(0.1)  # a disc inside the 8-unit-high world
    else:
        p = sc.boids_params(k=16, world=512.0, cell=4.0)
        s = sc.boids_sphere(8192, radius=30.0, seed=12)
        s.position[:, :3] += np.float32(200.0)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    g = group_of(s, p.k)
    gs.step(g, bins, None, p, 6)
    want = s.copy()
    ol.run(want, p, 6)
    assert_state(g.download(), want, skip_side=want.speed == 0)


def test_streaming_scan_in_3d_matches_oracle():
    s = sc.boids_sphere(20000, radius=25.0, seed=8)
    p = sc.boids_params(k=16, world=64.0, cell=2.0)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    g = group_of(s, p.k)
    gs.set_knn_capacity(g, 128)
    gs.step(g, bins, None, p, 5)
    want = s.copy()
    ol.run(want, p, 5)
    assert_state(g.download(), want, skip_side=want.speed == 0)


def test_boids_fused_equals_dropin_sequence():
    s = sc.boids_sphere(2000, radius=15.0, seed=11)
    p = sc.boids_params(k=16, world=64.0)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    g1 = group_of(s, p.k)
    knn = gs.KNNData(s.n, p.k)
    for _ in range(10):
        dropin_flock_step(g1, knn, bins, p)
    g2 = group_of(s, p.k)
    gs.step(g2, bins, None, p, 10)
    assert_state(g2.download(), g1.download())


def choke_walls(p):
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    walls = gs.WallGroup(sc.chokepoint_walls(10.0), bins=bins, knw=p.knw)
    return bins, walls


@pytest.mark.parametrize("avoid_close", [0, 1])
def test_chokepoint_config_fused_matches_oracle(avoid_close):
    """2D choke point: walls, neighbour avoidance, separation, seek; 10,000
    agents, k = 16, cell 2.0, 60 steps, bit-exact."""
    p = sc.chokepoint_params().replace(avoid_close=avoid_close)
    s = sc.chokepoint_agents(10000, seed=0)
    bins, walls = choke_walls(p)
    g = group_of(s, p.k)
    gs.step(g, bins, walls, p, 60)
    want = s.copy()
    ol.run(want, p, 60, walls=walls.download())
    assert_state(g.download(), want, skip_side=want.speed == 0)


def test_fused_steps_resume_across_calls_and_downloads():
    p = sc.chokepoint_params()
    s = sc.chokepoint_agents(3000, seed=5)
    bins, walls = choke_walls(p)
    g = group_of(s, p.k)
    gs.step(g, bins, walls, p, 7)
    mid = g.download()
    gs.step(g, bins, walls, p, 8)
    want = s.copy()
    ol.run(want, p, 7, walls=walls.download())
    assert_state(mid, want, skip_side=want.speed == 0)
    ol.run(want, p, 8, walls=walls.download())
    assert_state(g.download(), want, skip_side=want.speed == 0)


def test_step_host_is_upload_step_download():
    p = sc.boids_params(k=7)
    s = sc.boids_sphere(3000, seed=2)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    g = gs.AgentGroup(p.k, s.n)
    out = AgentState.zeros(s.n)
    gs.step_host(g, bins, None, p, 5, s, out)
    want = s.copy()
    ol.run(want, p, 5)
    assert_state(out, want, skip_side=want.speed == 0)
    # in place: the state stepped in its own arrays, five more steps one call
    # at a time (the constants stay on the host)
    inplace = want.copy()
    for _ in range(5):
        gs.step_host(g, bins, None, p, 1, inplace, inplace)
    ol.run(want, p, 5)
    assert_state(inplace, want, skip_side=want.speed == 0)


def test_large_flock_two_steps_match_oracle():
    """The full 1,048,576-agent, k = 16 flock of the throughput benchmark,
    two fused steps against the oracle."""
    n = 1 << 20
    s = sc.boids_cube(n, size=512.0, seed=0)
    p = sc.boids_params(k=16, world=512.0, cell=4.0)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    g = group_of(s, p.k)
    gs.step(g, bins, None, p, 2)
    want = s.copy()
    ol.run(want, p, 2)
    assert_state(g.download(), want, skip_side=want.speed == 0)


# ---- errors -----------------------------------------------------------------------

def test_invalid_arguments_are_reported_not_fatal():
    s = sc.boids_sphere(100, seed=1)
    g = group_of(s, 7)
    bins = gs.KNNBinData((8, 8, 8), (32.0, 32.0, 32.0), 1)
    knn = gs.KNNData(50, 7)  # wrong size
    gs.updateKNNDatabase(g, bins)
    with pytest.raises(gs.GpuSteerError) as e:
        gs.findKNearestNeighbors(g, knn, bins, g, 1)
    assert e.value.status == 1
    with pytest.raises(gs.GpuSteerError) as e:
        gs.updateGroup(g, float("nan"))
    assert e.value.status == 5
    with pytest.raises(gs.GpuSteerError):
        gs.AgentGroup(65, 10)
    with pytest.raises(gs.GpuSteerError):
        big = sc.boids_sphere(200, seed=1)
        g.upload(big)  # over capacity
    p = sc.boids_params(k=7).replace(order=(sc.B_SEPARATION, sc.B_AVOID_WALLS))
    with pytest.raises(gs.GpuSteerError) as e:
        gs.step(g, gs.KNNBinData(p.world_cells, p.world_size, 1), None, p, 1)
    assert e.value.status == 7
    # the group still works afterwards
    gs.step(g, gs.KNNBinData((40, 40, 40), (160.0,) * 3, 1), None, sc.boids_params(k=7), 1)
    assert g.download().n == 100


def test_empty_group_steps():
    g = gs.AgentGroup(7, 16)
    g.upload(AgentState.zeros(0))
    p = sc.boids_params(k=7)
    gs.step(g, gs.KNNBinData(p.world_cells, p.world_size, 1), None, p, 3)
    assert g.download().n == 0


# ---- batched scenes ---------------------------------------------------------------

def batch_setup(states, gaps, p, graphs=True, block=256):
    b = gs.Batch([s.n for s in states], p.k, p.world_cells, p.world_size, p.search_radius)
    for i, g in enumerate(gaps):
        b.set_walls(i, sc.chokepoint_walls(g))
    b.upload(AgentState.concat(states))
    gs.set_graphs(b.group, graphs)
    gs.set_block(b.group, block)
    return b


def per_scene(states, gaps, p, steps):
    outs = []
    for s, g in zip(states, gaps):
        bins = gs.KNNBinData(p.world_cells, p.world_size, p.search_radius)
        walls = gs.WallGroup(sc.chokepoint_walls(g), bins=bins, knw=p.knw)
        grp = group_of(s, p.k)
        gs.step(grp, bins, walls, p, steps)
        outs.append(grp.download())
    return AgentState.concat(outs)


def test_batches_step_host_equals_one_batch():
    """gs_batches_step_host over three parts of a workload (host state in,
    steps, host state out, copies and steps overlapped across the parts'
    streams) equals one batch of all scenes, also called twice in place."""
    states, gaps = sc.batched_chokepoint(7, seed=9, n_range=(300, 3000))
    p = sc.chokepoint_params(world=256.0, cell=2.0)
    whole = batch_setup(states, gaps, p)
    whole.step(p, 3)
    want = whole.download()
    cuts = [(0, 3), (3, 5), (5, 7)]
    parts = []
    for lo, hi in cuts:
        b = batch_setup(states[lo:hi], gaps[lo:hi], p)
        gs.set_knn_capacity(b.group, 256)
        parts.append(b)
    host = AgentState.concat(states)
    out = AgentState.zeros(host.n)
    gs.batches_step_host(parts, p, 3, host, out)  # pageable arrays: queued call by call
    assert_state(out, want)
    whole.step(p, 3)
    gs.batches_step_host(parts, p, 3, out, out)
    assert_state(out, whole.download())
    # page-locked arrays: each part's upload, steps and download as one graph,
    # captured on the first call and replayed on the next ones
    pin = gs.pinned_state(host.n)
    for k in host.names():
        getattr(pin, k)[...] = getattr(host, k)
    whole = batch_setup(states, gaps, p)
    for _ in range(3):
        gs.batches_step_host(parts, p, 2, pin, pin)
        whole.step(p, 2)
        assert_state(pin, whole.download())
    # separate page-locked output arrays (every field written), then the
    # parts' own state read back through the batch API
    out_pin = gs.pinned_state(host.n)
    gs.batches_step_host(parts, p, 1, pin, out_pin)
    whole.step(p, 1)
    want = whole.download()
    assert_state(out_pin, want)
    got = AgentState.concat([b.download() for b in parts])
    assert_state(got, want)


def test_batched_scenes_equal_per_scene_runs():
    states, gaps = sc.batched_chokepoint(7, seed=3, n_range=(300, 3000))
    p = sc.chokepoint_params(world=256.0, cell=2.0)
    want = per_scene(states, gaps, p, 15)
    for graphs, block in ((True, 256), (False, 256), (True, 128)):
        b = batch_setup(states, gaps, p, graphs=graphs, block=block)
        b.step(p, 5)
        b.step(p, 10)  # resumes across calls (graph replay)
        assert_state(b.download(), want)


def test_batched_scene_matches_oracle():
    states, gaps = sc.batched_chokepoint(3, seed=9, n_range=(500, 2000))
    p = sc.chokepoint_params(world=256.0, cell=2.0)
    b = batch_setup(states, gaps, p)
    b.step(p, 12)
    got = b.download()
    off = 0
    for s, g in zip(states, gaps):
        want = s.copy()
        walls = ol.split_walls(*sc.walls_from_rows(sc.chokepoint_walls(g)), p.world_size,
                               p.world_cells)
        ol.run(want, p, 12, walls=walls)
        assert_state(got.subset(slice(off, off + s.n)), want, skip_side=want.speed == 0)
        off += s.n


@pytest.mark.parametrize("capacity", [0, 128])
def test_ragged_batch_with_empty_and_single_agent_scenes(capacity):
    """Scenes of 0, 1, 17 and 3,000 agents in one batch (and an empty last
    scene): every non-empty scene equals the oracle stepped alone."""
    counts = [0, 1, 17, 3000, 0]
    states = [sc.chokepoint_agents(n, seed=40 + i) for i, n in enumerate(counts)]
    gaps = [10.0, 7.5, 20.0, 12.5, 30.0]
    p = sc.chokepoint_params(world=256.0, cell=2.0)
    b = batch_setup(states, gaps, p)
    gs.set_knn_capacity(b.group, capacity)
    b.step(p, 15)
    got = b.download()
    assert got.n == sum(counts)
    off = 0
    for st, g in zip(states, gaps):
        if st.n:
            want = st.copy()
            walls = ol.split_walls(*sc.walls_from_rows(sc.chokepoint_walls(g)), p.world_size,
                                   p.world_cells)
            ol.run(want, p, 15, walls=walls)
            assert_state(got.subset(slice(off, off + st.n)), want, skip_side=want.speed == 0)
        off += st.n


def test_persistent_step_equals_separate_launches():
    """One cooperative persistent launch per step (scan, permute, wall phase,
    exact lists, redo and rest phase between grid-wide barriers) equals the
    separate launches bit for bit, with graphs on and off, resumed across
    calls."""
    states, gaps = sc.batched_chokepoint(7, seed=3, n_range=(300, 3000))
    p = sc.chokepoint_params(world=256.0, cell=2.0)
    want = per_scene(states, gaps, p, 15)
    for graphs in (True, False):
        b = batch_setup(states, gaps, p, graphs=graphs)
        gs.set_knn_capacity(b.group, 256)
        gs.set_persistent(b.group, True)
        b.step(p, 5)
        b.step(p, 10)
        assert_state(b.download(), want)
        assert gs.step_launches(b.group, True) == 1


def test_persistent_step_through_the_redo_routes():
    """A crowd of about 20 agents per cell (184 candidates per box, past the
    streaming scan's 128): most agents go through the persistent step's
    warp-per-agent lists and redo phase; the result is the oracle's."""
    p = sc.chokepoint_params()
    bins, walls = choke_walls(p)
    s = sc.chokepoint_agents(4000, x_range=(-14.0, 14.0), z_range=(20.0, 48.0), seed=6)
    g = group_of(s, p.k)
    gs.set_knn_capacity(g, 128)
    gs.set_persistent(g, True)
    gs.step(g, bins, walls, p, 3)
    want = s.copy()
    ol.run(want, p, 3, walls=walls.download())
    assert_state(g.download(), want, skip_side=want.speed == 0)


def test_persistent_barrier_timeout_is_reported():
    """A grid barrier whose wait runs out (a limit of one poll) makes every
    block return without feeding the next phase; synchronize reports
    GS_ERR_TIMEOUT and the group steps correctly again after an upload."""
    p = sc.chokepoint_params()
    bins, walls = choke_walls(p)
    s = sc.chokepoint_agents(10000, seed=0)
    g = group_of(s, p.k)
    gs.set_knn_capacity(g, 256)
    gs.set_persistent(g, True)
    gs.set_barrier_limit(g, 1)
    gs.step(g, bins, walls, p, 1)
    with pytest.raises(gs.GpuSteerError) as e:
        g.synchronize()
    assert e.value.status == 4  # GS_ERR_TIMEOUT
    gs.set_barrier_limit(g, 0)
    g.upload(s)
    gs.step(g, bins, walls, p, 2)
    want = s.copy()
    ol.run(want, p, 2, walls=walls.download())
    assert_state(g.download(), want, skip_side=want.speed == 0)


def test_graph_replay_equals_eager_single_group():
    p = sc.boids_params(k=16, world=64.0)
    s = sc.boids_sphere(5000, radius=20.0, seed=21)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    g1 = group_of(s, p.k)
    gs.set_graphs(g1, False)
    gs.step(g1, bins, None, p, 12)
    g2 = group_of(s, p.k)
    gs.step(g2, bins, None, p, 4)
    gs.step(g2, bins, None, p, 8)
    assert_state(g2.download(), g1.download())


# ---- MultiGroup: cross-group KNN and steering (plugins/MultiGroup.cpp:545-610) ------

def test_multigroup_cross_group_steps_match_oracle():
    """Two groups in one world, stepped as MultiGroupSimulation::update does:
    every group wraps and rebuilds its database first (Group::preUpdate),
    then each group in turn runs KNN against every group, avoids the other
    group, separates from every group, aligns and coheres with itself and
    integrates.  A later group's KNN reads an earlier group's database built
    before that group moved, while the steering reads its current state."""
    p = sc.boids_params(k=8, world=96.0, cell=4.0)
    min_time, min_sep, w_avoid = 2.0, 0.5, 1.0
    states = [sc.boids_sphere(3000, radius=18.0, seed=31), sc.boids_sphere(2000, radius=18.0, seed=32)]
    G = len(states)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    groups = [group_of(s, p.k) for s in states]
    knns = [[gs.KNNData(states[i].n, p.k) for _ in range(G)] for i in range(G)]
    want = [s.copy() for s in states]
    o = ol.oracle()
    f = ol.C.c_float
    for _ in range(6):
        for g in groups:
            gs.wrapWorld(g, p.world_size, sc.WRAP_REFERENCE)
            gs.updateKNNDatabase(g, bins)
        for s in want:
            o.orc_wrap_world(ol.C.byref(ol.group_struct(s)), ol.f3(p.world_size), sc.WRAP_REFERENCE)
        snap = [s.position.copy() for s in want]  # the databases' positions
        for i, g in enumerate(groups):
            for j, other in enumerate(groups):
                gs.findKNearestNeighbors(g, knns[i][j], bins, other, 1)
            lists = [ol.knn_binned(snap[i], snap[j], i == j, p.world_size, p.world_cells, 1, p.k)
                     for j in range(G)]
            for j in range(G):
                gi, gd = knns[i][j].download(g)
                np.testing.assert_array_equal(gi, lists[j][0])
                np.testing.assert_array_equal(gd, lists[j][1])
            me = ol.group_struct(want[i])
            for j, other in enumerate(groups):
                if j == i:
                    continue
                gs.steerToAvoidNeighbors(g, knns[i][j], other, min_time, min_sep, 1, w_avoid, 0)
                ob = want[j]
                o.orc_steer_avoid_neighbors(
                    ol.C.byref(me), ol.ptr(lists[j][0], ol.C.c_uint), ol.ptr(lists[j][1]), p.k,
                    ol.ptr(ob.position), ol.ptr(ob.direction), ol.ptr(ob.speed), ol.ptr(ob.radius),
                    ob.n, f(min_time), f(min_sep), 1, f(w_avoid), 0)
            for j, other in enumerate(groups):
                gs.steerForSeparation(g, knns[i][j], other, p.sep_min, p.sep_max, p.sep_cos,
                                      p.w_sep, p.mask_sep)
                ob = want[j]
                o.orc_steer_separation(ol.C.byref(me), ol.ptr(lists[j][0], ol.C.c_uint), p.k,
                                       ol.ptr(ob.position), ob.n, f(p.sep_min), f(p.sep_max),
                                       f(p.sep_cos), f(p.w_sep), p.mask_sep)
            gs.steerForAlignment(g, knns[i][i], g, p.ali_min, p.ali_max, p.ali_cos, p.w_ali,
                                 p.mask_ali)
            o.orc_steer_alignment(ol.C.byref(me), ol.ptr(lists[i][0], ol.C.c_uint), p.k,
                                  ol.ptr(want[i].position), ol.ptr(want[i].direction), want[i].n,
                                  f(p.ali_min), f(p.ali_max), f(p.ali_cos), f(p.w_ali), p.mask_ali)
            gs.steerForCohesion(g, knns[i][i], g, p.coh_min, p.coh_max, p.coh_cos, p.w_coh,
                                p.mask_coh)
            o.orc_steer_cohesion(ol.C.byref(me), ol.ptr(lists[i][0], ol.C.c_uint), p.k,
                                 ol.ptr(want[i].position), want[i].n, f(p.coh_min), f(p.coh_max),
                                 f(p.coh_cos), f(p.w_coh), p.mask_coh)
            gs.updateGroup(g, p.dt)
            o.orc_update(ol.C.byref(me), f(p.dt))
    for g, s in zip(groups, want):
        assert_state(g.download(), s, skip_side=s.speed == 0)


def test_multigroup_batched_knn_equals_per_pair_calls():
    """gs_find_knn_groups: every group pair's lists in one launch, taken at the
    start of a MultiGroup frame, equal the per-pair findKNearestNeighbors calls
    that Group::update makes in turn after the earlier groups have moved, and
    the oracle's.  Pairs carry different k, one pair is skipped, and one group
    appears twice (its pairs with itself are self searches)."""
    p = sc.boids_params(k=8, world=96.0, cell=4.0)
    states = [sc.boids_sphere(3000, radius=18.0, seed=41), sc.boids_sphere(2000, radius=18.0, seed=42),
              sc.boids_sphere(1200, radius=12.0, seed=43)]
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    groups = [group_of(s, 16) for s in states]
    seq = groups + [groups[1]]  # group 1 listed twice
    sizes = [st.n for st in states] + [states[1].n]
    G = len(seq)
    kk = [[16 if (i + j) % 2 else 8 for j in range(G)] for i in range(G)]
    for frame in range(4):
        for g in groups:
            gs.wrapWorld(g, p.world_size, sc.WRAP_REFERENCE)
            gs.updateKNNDatabase(g, bins)
        snap = [g.download().position.copy() for g in seq]
        batched = [[gs.KNNData(sizes[i], kk[i][j]) if (i, j) != (2, 0) else None
                    for j in range(G)] for i in range(G)]
        gs.findKNearestNeighborsGroups(seq, bins, batched)
        for i in range(G):
            for j in range(G):
                if batched[i][j] is None:
                    continue
                single = gs.KNNData(sizes[i], kk[i][j])
                gs.findKNearestNeighbors(seq[i], single, bins, seq[j], 1)
                bi, bd = batched[i][j].download(seq[i])
                si, sd = single.download(seq[i])
                np.testing.assert_array_equal(bi, si)
                np.testing.assert_array_equal(bd, sd)
                if frame == 0 and i < 3:
                    oi, od = ol.knn_binned(snap[i], snap[j], seq[i] is seq[j], p.world_size,
                                           p.world_cells, 1, kk[i][j])
                    np.testing.assert_array_equal(bi, oi)
                    np.testing.assert_array_equal(bd, od)
            if i < 3:  # this group steps before the next group's per-pair calls
                gs.steerForSeparation(seq[i], batched[i][i], seq[i], p.sep_min, p.sep_max,
                                      p.sep_cos, p.w_sep, 0)
                gs.updateGroup(seq[i], p.dt)


def test_multigroup_fused_frames_equal_per_function_frames():
    """gs_multigroup_step (one steering launch per group) against the same
    frames through the per-function API, call for call as MultiGroup.cpp:545-610
    runs them: three groups, two with paths, close-neighbour avoidance and
    anti-penetration between all groups; bit for bit over six frames."""
    p = sc.boids_params(k=8, world=96.0, cell=4.0)
    states = [sc.boids_sphere(2500, radius=16.0, seed=51), sc.boids_sphere(1800, radius=16.0, seed=52),
              sc.boids_sphere(900, radius=12.0, seed=53)]
    for st in states:
        st.radius[:] = np.float32(0.9)
    G = len(states)
    pts = [[(0.0, 0.0, 0.0), (30.0, 5.0, -20.0), (-10.0, 20.0, 30.0)], None,
           [(5.0, -5.0, 5.0), (-25.0, 0.0, 10.0)]]
    mp = dict(world_size=p.world_size, wrap_mode=sc.WRAP_REFERENCE, min_time_to_collision=2.0,
              min_separation_distance=0.5, avoid_close=1, w_avoid=1.0, mask_avoid=0,
              sep_min=p.sep_min, sep_max=p.sep_max, sep_cos=p.sep_cos, w_sep=p.w_sep,
              mask_sep=4096, ali_min=p.ali_min, ali_max=p.ali_max, ali_cos=p.ali_cos,
              w_ali=p.w_ali, mask_ali=272, coh_min=p.coh_min, coh_max=p.coh_max,
              coh_cos=p.coh_cos, w_coh=p.w_coh, mask_coh=272, path_prediction_time=5.0,
              w_path=1.0, mask_path=16, w_seek=1.5, mask_seek=4480, mask_antipen=4096,
              dt=1.0 / 30.0)
    frames = 6
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    paths = [gs.Path(q, 6.0) if q is not None else None for q in pts]
    # fused
    fused = [group_of(s, p.k) for s in states]
    kf = [[gs.KNNData(states[i].n, p.k) for _ in range(G)] for i in range(G)]
    gs.multigroup_step(fused, bins, kf, gs.MultiGroupParams(**mp), frames, paths=paths)
    # per function
    groups = [group_of(s, p.k) for s in states]
    kp = [[gs.KNNData(states[i].n, p.k) for _ in range(G)] for i in range(G)]
    m = mp
    for _ in range(frames):
        for g in groups:
            gs.wrapWorld(g, p.world_size, sc.WRAP_REFERENCE)
            st = g.download()
            st.applied[:] = 0
            g.upload(st)
            gs.updateKNNDatabase(g, bins)
        for i, g in enumerate(groups):
            for j, o in enumerate(groups):
                gs.findKNearestNeighbors(g, kp[i][j], bins, o, 1)
            for j, o in enumerate(groups):
                if j != i:
                    gs.steerToAvoidNeighbors(g, kp[i][j], o, m["min_time_to_collision"],
                                             m["min_separation_distance"], m["avoid_close"],
                                             m["w_avoid"], m["mask_avoid"])
            for j, o in enumerate(groups):
                gs.steerForSeparation(g, kp[i][j], o, m["sep_min"], m["sep_max"], m["sep_cos"],
                                      m["w_sep"], m["mask_sep"])
            gs.steerForAlignment(g, kp[i][i], g, m["ali_min"], m["ali_max"], m["ali_cos"],
                                 m["w_ali"], m["mask_ali"])
            gs.steerForCohesion(g, kp[i][i], g, m["coh_min"], m["coh_max"], m["coh_cos"],
                                m["w_coh"], m["mask_coh"])
            if paths[i] is not None:
                gs.steerToFollowPath(g, paths[i], m["path_prediction_time"], m["w_path"],
                                     m["mask_path"])
                gs.steerForSeek(g, pts[i][1], m["w_seek"], m["mask_seek"])
            gs.updateGroup(g, m["dt"])
            for j, o in enumerate(groups):
                gs.antiPenetrationAgents(g, kp[i][j], o, m["mask_antipen"])
    for i in range(G):
        assert_state(fused[i].download(), groups[i].download())
        np.testing.assert_array_equal(kf[i][(i + 1) % G].download(fused[i])[0],
                                      kp[i][(i + 1) % G].download(groups[i])[0])
    got = fused[0].download()
    assert ((got.applied & 8192) != 0).sum() > 50  # anti-penetration fired


# ---- path following (SteerToFollowPathCUDAKernel.cu, PolylinePathwayCUDA.cu) ----------

@pytest.mark.parametrize("name", ["line", "loop", "bend"])
def test_follow_path_matches_reference_golden(name):
    z, m = load(f"path_{name}")
    path = gs.Path(m["points"], m["radius"], m["cyclic"])
    po, ln, nm, tot = path.arrays()
    np.testing.assert_array_equal(po, z["path_points"])
    np.testing.assert_array_equal(ln, z["path_lengths"])
    np.testing.assert_array_equal(nm, z["path_normals"])
    assert np.float32(tot) == z["path_total"][0]
    s = gstate(z, "in_")
    g = group_of(s)
    gs.steerToFollowPath(g, path, m["prediction_time"], m["weight"], m["mask"])
    out = g.download()
    np.testing.assert_array_equal(out.steering, z["out_steering"])
    np.testing.assert_array_equal(out.applied, z["out_applied"])


def chokepoint_with_path():
    """CtfGroup::update's behaviours (ChokePointNew.cpp:603-624): walls,
    separation, alignment, cohesion, follow path, seek the path's second
    point, update; path and weights of data/ChokePoint.params."""
    pts = [(0.0, 0.0, 13.5), (0.0, 0.0, -1650.0)]
    p = sc.chokepoint_params().replace(
        order=(sc.B_AVOID_WALLS, sc.B_SEPARATION, sc.B_ALIGNMENT, sc.B_COHESION,
               sc.B_FOLLOW_PATH, sc.B_SEEK),
        ali_min=0.5, ali_max=7.0, w_ali=2.0, coh_min=0.5, coh_max=7.0, w_coh=1.0,
        seek_target=pts[1], path_prediction_time=5.0, w_path=1.0, mask_path=16)
    return p, pts, 20.0


def test_fused_step_with_path_matches_dropin_and_oracle():
    p, pts, radius = chokepoint_with_path()
    s = sc.chokepoint_agents(8000, seed=13)
    s.speed[:] = np.float32(1.0)
    bins, walls = choke_walls(p)
    path = gs.Path(pts, radius)
    g = group_of(s, p.k)
    gs.step(g, bins, walls, p, 25, path=path)
    fused = g.download()
    # the same frames through the per-function API
    g2 = group_of(s, p.k)
    knn = gs.KNNData(s.n, p.k)
    knw = gs.KNNData(s.n, p.knw)
    for _ in range(25):
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
    assert_state(fused, g2.download())
    want = s.copy()
    ol.run(want, p, 25, walls=walls.download(), path=ol.path_init(pts, radius, False))
    assert_state(fused, want)
    assert (fused.position[:, 2] < s.position[:, 2]).mean() > 0.5  # heading down the path


# ---- ExtractData diagnostics ----------------------------------------------------------

@pytest.mark.parametrize("case", ["crowd2d", "flock3d"])
def test_cell_diagnostics_match_oracle(case):
    if case == "crowd2d":
        s = sc.chokepoint_agents(20000, seed=23)
        s.speed[:] = (sc.uniform01(6, s.n) * 3.0).astype(np.float32)
        ws, wc = (512.0, 10.0, 512.0), (256, 1, 256)
    else:
        s = sc.boids_sphere(30000, radius=40.0, seed=24)
        ws, wc = (160.0, 160.0, 160.0), (40, 40, 40)
    bins = gs.KNNBinData(wc, ws, 1)
    g = group_of(s)
    gs.updateKNNDatabase(g, bins)
    from gpusteer_gb300.groups import cell_avg_velocity, cell_density

    np.testing.assert_array_equal(cell_density(g, bins), ol.cell_density(s.position, ws, wc))
    np.testing.assert_array_equal(cell_avg_velocity(g, bins),
                                  ol.cell_avg_velocity(s.position, s.direction, s.speed, ws, wc))


@pytest.mark.parametrize("case", ["crowd2d", "flock3d"])
def test_cell_diagnostics_match_reference_golden(case):
    """gs_cell_density / gs_cell_avg_velocity against the reference's own
    ProcessData.cu kernels on the reference's database (cell_diag.npz)."""
    from gpusteer_gb300.groups import cell_avg_velocity, cell_density

    z, m = load("cell_diag")
    ws, wc = m[case]["ws"], m[case]["wc"]
    s = AgentState.zeros(z[f"{case}_position"].shape[0])
    s.position[:] = z[f"{case}_position"]
    s.direction[:] = z[f"{case}_direction"]
    s.speed[:] = z[f"{case}_speed"]
    bins = gs.KNNBinData(wc, ws, 1)
    g = group_of(s)
    gs.updateKNNDatabase(g, bins)
    np.testing.assert_array_equal(cell_density(g, bins), z[f"{case}_density"])
    np.testing.assert_array_equal(cell_avg_velocity(g, bins).reshape(-1, 3),
                                  z[f"{case}_avg_velocity"])


def frame_diagnostics_oracle(s, p, walls, steps):
    """ExtractData after `steps` frames: the database the last frame built
    (positions after its wrap) and the velocities after that frame."""
    pre = s.copy()
    if steps > 1:
        ol.run(pre, p, steps - 1, walls=walls)
    db = pre.copy()
    ol.oracle().orc_wrap_world(ol.C.byref(ol.group_struct(db)), ol.f3(p.world_size), p.wrap_mode)
    post = pre.copy()
    ol.run(post, p, 1, walls=walls)
    return (ol.cell_density(db.position, p.world_size, p.world_cells),
            ol.cell_avg_velocity(db.position, post.direction, post.speed, p.world_size,
                                 p.world_cells))


def test_cell_diagnostics_of_a_fused_frame():
    """After gs_step, ExtractData reads the step's own buckets (the database the
    reference's plugin builds at the start of the frame) and the agents' new
    velocities, with no rebuild; once gs_update_knn_database runs again, its
    database takes over.  The same per scene after gs_batch_step."""
    from gpusteer_gb300.groups import cell_avg_velocity, cell_density

    p = sc.chokepoint_params(world=256.0, cell=2.0)
    s = sc.chokepoint_agents(12000, seed=31)
    s.speed[:] = (sc.uniform01(7, s.n) * 2.0).astype(np.float32)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    walls = gs.WallGroup(sc.chokepoint_walls(10.0), bins=bins, knw=p.knw)
    g = group_of(s, p.k)
    steps = 12
    gs.step(g, bins, walls, p, steps)
    want_d, want_v = frame_diagnostics_oracle(s, p, walls.download(), steps)
    got_d = cell_density(g, bins)
    np.testing.assert_array_equal(got_d, want_d)
    np.testing.assert_array_equal(cell_avg_velocity(g, bins), want_v)
    assert got_d.max() >= 4
    gs.updateKNNDatabase(g, bins)
    cur = g.download()
    np.testing.assert_array_equal(cell_density(g, bins),
                                  ol.cell_density(cur.position, p.world_size, p.world_cells))
    # batched: every scene's frame at once
    states, gaps = sc.batched_chokepoint(4, seed=5, n_range=(800, 4000))
    b = batch_setup(states, gaps, p)
    b.step(p, steps)
    dens, vel = b.cell_density(), b.cell_avg_velocity()
    for i, (st, gap) in enumerate(zip(states, gaps)):
        wb = gs.KNNBinData(p.world_cells, p.world_size, 1)
        sw = gs.WallGroup(sc.chokepoint_walls(gap), bins=wb, knw=p.knw).download()
        wd, wv = frame_diagnostics_oracle(st, p, sw, steps)
        np.testing.assert_array_equal(dens[i], wd)
        np.testing.assert_array_equal(vel[i], wv.reshape(-1, 3))
