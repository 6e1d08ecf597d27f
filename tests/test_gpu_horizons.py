"""Parity at the benchmark configurations' own sizes and step counts.

Every comparison is bit-exact (np.testing.assert_array_equal) against the CPU
oracle, through the C ABI:

- the 10,000-agent choke point for all 500 of its steps;
- the 4,096-boid flock for 100 steps through brute-force KNN, in the drop-in
  call sequence of plugins/BoidsGroupBruteForce.cpp:459-489 (wrap, KNN,
  separation, cohesion, alignment, update);
- the 1,048,576-boid flock for 10 steps from its initial state, and for 5
  steps from the clustered state it reaches after 300 steps;
- the benchmark's own 256-scene batch, with 16 scenes spread over the gap set
  checked against the oracle, and batches at the autotuner's other cell sizes.

The only agents excluded are those whose speed is 0, whose side vector the
reference leaves undefined (UpdateCUDAKernel.cu:75,114).
"""
import numpy as np
import pytest

import gpusteer_gb300 as gs
import oracle_lib as ol
from gpusteer_gb300 import scenario as sc
from gpusteer_gb300.state import AgentState

pytestmark = pytest.mark.gpu


def assert_state(got: AgentState, want: AgentState, skip_side=None):
    for k in AgentState.names():
        a, b = getattr(got, k), getattr(want, k)
        if k == "side" and skip_side is not None:
            a, b = a[~skip_side], b[~skip_side]
        np.testing.assert_array_equal(a, b, err_msg=k)


def group_of(s: AgentState, k: int):
    g = gs.AgentGroup(k, max(1, s.n))
    g.upload(s)
    return g


@pytest.mark.parametrize("avoid_close", [0, 1])
def test_chokepoint_config_all_500_steps(avoid_close):
    """10,000 agents, gap 10, k = 16, knw = 3, cell 2.0: the whole 500-step run."""
    p = sc.chokepoint_params().replace(avoid_close=avoid_close)
    s = sc.chokepoint_agents(10000, seed=0)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    walls = gs.WallGroup(sc.chokepoint_walls(10.0), bins=bins, knw=p.knw)
    g = group_of(s, p.k)
    want = s.copy()
    for chunk in (100, 150, 250):  # checked along the way, resumed across calls
        gs.step(g, bins, walls, p, chunk)
        ol.run(want, p, chunk, walls=walls.download())
        assert_state(g.download(), want, skip_side=want.speed == 0)


def test_boids_config_brute_force_dropin_100_steps():
    """4,096 boids, k = 7, 100 steps, KNN by brute force through the drop-in
    functions, as BoidsGroupBruteForce's update calls them."""
    p = sc.boids_params(k=7)
    s = sc.boids_sphere(4096, seed=0)
    g = group_of(s, p.k)
    knn = gs.KNNData(s.n, p.k)
    for _ in range(100):
        gs.wrapWorld(g, p.world_size, p.wrap_mode)
        gs.findKNearestNeighborsBruteForce(g, knn, g)
        gs.steerForSeparation(g, knn, g, p.sep_min, p.sep_max, p.sep_cos, p.w_sep, p.mask_sep)
        gs.steerForCohesion(g, knn, g, p.coh_min, p.coh_max, p.coh_cos, p.w_coh, p.mask_coh)
        gs.steerForAlignment(g, knn, g, p.ali_min, p.ali_max, p.ali_cos, p.w_ali, p.mask_ali)
        gs.updateGroup(g, p.dt)
    want = s.copy()
    idx, dist = ol.run(want, p.replace(knn_mode=sc.KNN_BRUTEFORCE), 100, want_knn=True)
    got_i, got_d = knn.download(g)
    np.testing.assert_array_equal(got_i, idx.reshape(got_i.shape))
    np.testing.assert_array_equal(got_d, dist.reshape(got_d.shape))
    assert_state(g.download(), want, skip_side=want.speed == 0)


def test_large_flock_ten_steps_then_clustered_restart():
    """1,048,576 boids in a 512^3 cube, k = 16, cell 4.0: 10 steps from the
    initial state; then, after 300 steps in all, 5 more steps from the
    clustered state, the oracle starting from the GPU's downloaded state."""
    n = 1 << 20
    s = sc.boids_cube(n, size=512.0, seed=0)
    p = sc.boids_params(k=16, world=512.0, cell=4.0)
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    g = group_of(s, p.k)
    gs.step(g, bins, None, p, 10)
    want = s.copy()
    ol.run(want, p, 10)
    assert_state(g.download(), want, skip_side=want.speed == 0)
    gs.step(g, bins, None, p, 290)
    start = g.download()
    # the flock has clustered: more agents per occupied cell than at the start
    def per_cell(st):
        return n / np.unique(ol.cell_index(st.position, p.world_size, p.world_cells)).size

    assert per_cell(start) > per_cell(s)
    gs.step(g, bins, None, p, 5)
    want = start.copy()
    ol.run(want, p, 5)
    assert_state(g.download(), want, skip_side=want.speed == 0)


def batch_of(states, gaps, p, block=256):
    b = gs.Batch([s.n for s in states], p.k, p.world_cells, p.world_size, p.search_radius)
    for i, gap in enumerate(gaps):
        b.set_walls(i, sc.chokepoint_walls(gap))
    b.upload(AgentState.concat(states))
    gs.set_block(b.group, block)
    return b


def check_scenes(got, states, gaps, p, steps, picks):
    offs = np.concatenate([[0], np.cumsum([s.n for s in states])])
    for i in picks:
        want = states[i].copy()
        walls = ol.split_walls(*sc.walls_from_rows(sc.chokepoint_walls(gaps[i])), p.world_size,
                               p.world_cells)
        ol.run(want, p, steps, walls=walls)
        assert_state(got.subset(slice(int(offs[i]), int(offs[i + 1]))), want,
                     skip_side=want.speed == 0)


def spread_picks(gaps, count):
    """`count` scene indices covering every gap width, then evenly spaced."""
    first = {gaps.index(gap) for gap in set(gaps)}
    picks, m = set(first), 2
    while len(picks) < min(count, len(gaps)):
        picks = first | {int(i) for i in np.linspace(0, len(gaps) - 1, m).astype(int)}
        m += 1
    return sorted(picks)


def test_benchmark_batch_of_256_scenes_matches_oracle():
    """The benchmark's batch: 256 choke-point scenes (gaps 7.5..32.5, 1,000 to
    20,000 agents), cell 2.0, 5 steps; 16 scenes covering every gap width are
    stepped by the oracle on their own and compared."""
    states, gaps = sc.batched_chokepoint(256, seed=0)
    p = sc.chokepoint_params()
    b = batch_of(states, gaps, p)
    b.step(p, 5)
    picks = spread_picks(gaps, 16)
    assert len(picks) >= 16 and len({gaps[i] for i in picks}) == len(set(gaps))
    check_scenes(b.download(), states, gaps, p, 5, picks)


@pytest.mark.parametrize("cell", [2.5, 3.0])
def test_batch_at_the_autotuners_other_cell_sizes(cell):
    """The autotuner also tries cells of 2.5 and 3.0 (205^2 and 171^2 cells
    per scene): results at those sizes against the oracle on the same grid."""
    states, gaps = sc.batched_chokepoint(24, seed=0)
    p = sc.chokepoint_params(cell=cell)
    b = batch_of(states, gaps, p)
    gs.set_knn_capacity(b.group, 256)  # the streaming scan the bench's trials also time
    b.step(p, 6)
    check_scenes(b.download(), states, gaps, p, 6, spread_picks(gaps, 8))
