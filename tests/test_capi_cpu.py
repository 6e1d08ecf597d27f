"""CPU-only checks of the C ABI library and the host-side logic."""
import re
from pathlib import Path

import numpy as np
import pytest

import gpusteer_gb300 as gs
from gpusteer_gb300 import _lib, scenario as sc
from gpusteer_gb300.state import AgentState

import oracle_lib as ol

REPO = Path(__file__).resolve().parents[1]


def header_functions():
    text = (REPO / "include" / "gpusteer.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gs_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function():
    lib = _lib.load()
    names = header_functions()
    assert len(names) > 30
    for n in names:
        assert hasattr(lib, n), n


def test_bindings_cover_the_header():
    assert set(header_functions()) == set(_lib.SIGNATURES)


def test_status_strings_and_version():
    lib = _lib.load()
    assert lib.gs_version() >= 1
    assert lib.gs_status_string(0) == b"ok"
    assert lib.gs_status_string(1) == b"invalid argument"
    assert lib.gs_max_k() == 64


def test_bins_host_side_matches_reference_cell_layout():
    b = gs.KNNBinData((8, 1, 4), (16.0, 10.0, 8.0), 1)
    assert b.num_cells == 32
    lo, hi, c = b.hv_cells()
    # bin_cell order: width fastest, then depth, then height (KNNBinDataV2.cu:103-116)
    np.testing.assert_allclose(lo[0], [-8.0, -5.0, -4.0])
    np.testing.assert_allclose(lo[1], [-6.0, -5.0, -4.0])
    np.testing.assert_allclose(lo[8], [-8.0, -5.0, -2.0])
    np.testing.assert_allclose(hi[31], [8.0, 5.0, 4.0])
    np.testing.assert_allclose(c[0], [-7.0, 0.0, -3.0])


@pytest.mark.parametrize("cells,size", [((0, 1, 1), (1, 1, 1)), ((1, 1, 1), (0, 1, 1)),
                                        ((1, 1, 1), (float("nan"), 1, 1)),
                                        # 2^31 * 2^31 * 4 wraps a 64-bit product to 0
                                        ((1 << 31, 1 << 31, 4), (1, 1, 1)),
                                        ((1 << 20, 1 << 11, 1), (1, 1, 1))])
def test_bins_reject_bad_grids(cells, size):
    with pytest.raises(gs.GpuSteerError) as e:
        gs.KNNBinData(cells, size, 1)
    assert e.value.status == 1


@pytest.mark.parametrize("parts", [1, 2, 3, 4, 8, 300])
def test_scene_cuts_cover_the_scenes_in_balanced_ranges(parts):
    """The concurrent batches of the batched workload: consecutive scene
    ranges covering every scene once, of about equal agent counts."""
    from gpusteer_gb300 import autotune

    states, _ = sc.batched_chokepoint(40, seed=3)
    ranges = autotune.scene_cuts(states, parts)
    assert ranges[0][0] == 0 and ranges[-1][1] == len(states)
    assert all(a < b for a, b in ranges)
    assert all(ranges[i][1] == ranges[i + 1][0] for i in range(len(ranges) - 1))
    assert len(ranges) <= min(parts, len(states))
    if parts <= 4:
        agents = [sum(s.n for s in states[a:b]) for a, b in ranges]
        n = sum(agents)
        # each range ends at the first scene that reaches its share
        assert max(agents) <= n / len(ranges) + max(s.n for s in states)


def test_splitmix_stream_is_fixed():
    # first outputs of splitmix64 seeded with 0 (published test values)
    v = sc.splitmix64(0, 3)
    assert [hex(int(x)) for x in v] == ["0xe220a8397b1dcdaf", "0x6e789e6aa1b965f4",
                                        "0x6c45d188009454f"]
    u = sc.uniform01(7, 1000)
    assert u.dtype == np.float32 and u.min() >= 0 and u.max() < 1


def test_scenarios_are_deterministic_and_in_range():
    a = sc.boids_sphere(500, seed=3)
    b = sc.boids_sphere(500, seed=3)
    for k in AgentState.names():
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k))
    r = np.linalg.norm(a.position[:, :3], axis=1)
    assert r.max() < 50 and np.allclose(np.linalg.norm(a.direction[:, :3], axis=1), 1, atol=1e-5)
    c = sc.chokepoint_agents(300, seed=1)
    assert (c.position[:, 1] == 0).all() and (c.speed == 0).all()
    assert c.position[:, 2].min() >= 13.5 and c.position[:, 2].max() <= 113.5
    q = sc.boids_cube(1000, size=512.0, seed=2)
    assert np.abs(q.position[:, :3]).max() <= 256


def test_params_reader_parses_reference_format():
    text = """# comment
    seed = 12345
    knn = 6
    cosMaxFlockingAngle = -0.5
    maskAlignment = 272 # trailing comment
    <world>
        dimensions = 2048 10 2048
        cells = 512 1 512
        # mapFilename = none
    </world>
    <group>
        numAgents = 10
        <path>
            point = 0 0 1
            point = 0 0 -2
            cyclic = 0
        </path>
    </group>
    </simulation>"""
    p = sc.load_params(text)
    assert p.values["seed"] == 12345 and p.values["knn"] == 6
    assert p.values["maskAlignment"] == 272
    assert p.world["cells"] == (512, 1, 512)
    assert p.groups[0]["numAgents"] == 10 and len(p.groups[0]["path"]) == 2
    with pytest.raises(sc.ParamsError):
        sc.load_params("bogusKey = 1\n</simulation>")


def test_reference_params_files_parse():
    data = ol.reference_root() / "data"
    if not data.exists():
        pytest.skip("reference data not mounted")
    for name in ("BoidsGroup.params", "ChokePoint.params", "MultiGroup.params"):
        p = sc.load_params((data / name).read_text())
        assert "knn" in p.values and p.groups
    sp = sc.params_from_file(sc.load_params((data / "BoidsGroup.params").read_text()), 1 / 60)
    assert sp.k == 6 and sp.mask_ali == 16 and sp.world_cells == (94, 94, 94)


def test_step_params_struct_roundtrip():
    p = sc.chokepoint_params()
    c = gs.groups.step_params_c(p)
    assert c.k == 16 and c.knw == 3 and c.n_order == 4
    assert list(c.order)[:4] == [1, 2, 3, 6]
    assert abs(c.dt - 1 / 30) < 1e-7 and c.mask_seek == 4480


def test_cpp_facade_has_the_reference_signatures(tmp_path):
    """include/GroupSteerLibrary.h declares the reference's free functions
    with their parameter lists (GroupSteerLibrary.cuh:43-223); a plugin's
    calls bind to them as written."""
    import shutil
    import subprocess

    from gpusteer_gb300 import build as gb

    src = tmp_path / "sig.cpp"
    src.write_text(r'''
#include "GroupSteerLibrary.h"
using namespace OpenSteer;
void (*a)(AgentGroup*, float3 const&) = wrapWorld;
void (*b)(AgentGroup*, float3 const&, float const, uint const) = steerForSeek;
void (*c)(AgentGroup*, KNNData*, AgentGroup*, const float, float const, bool const, float const,
          uint const) = steerToAvoidNeighbors;
void (*d)(AgentGroup*, KNNData*, WallGroup*, float const, float const, uint const) = steerToAvoidWalls;
void (*e)(BaseGroup*, KNNBinData*) = updateKNNDatabase;
void (*f)(AgentGroup*, KNNData*, KNNBinData*, BaseGroup*, uint const) = findKNearestNeighbors;
void (*g1)(AgentGroup*, KNNData*, AgentGroup*, float const, float const, float const, float const,
           uint const) = steerForSeparation;
void (*g2)(AgentGroup*, KNNData*, AgentGroup*, float const, float const, float const, float const,
           uint const) = steerForAlignment;
void (*g3)(AgentGroup*, KNNData*, AgentGroup*, float const, float const, float const, float const,
           uint const) = steerForCohesion;
void (*h)(AgentGroup*, const float) = updateGroup;
void (*i)(AgentGroup*, KNNData*, AgentGroup*, uint const) = antiPenetrationAgents;
void (*j)(AgentGroup*, PolylinePathwayCUDA*, float const, float const, uint const) =
    steerToFollowPath;
void (*k1)(AgentGroup*, KNNData*, WallGroup*, const float) = updateGroupWithAntiPenetration;
void (*k2)(AgentGroup*, KNNData*, WallGroup*, float const, uint const) = antiPenetrationWall;
int main() {
    AgentGroup* grp = nullptr;
    (void)grp;
    AgentData ad;
    ad.id = 0;
    ad.appliedKernels = KERNEL_SEPARATION_BIT | KERNEL_ANTI_PENETRATION_WALL;
    return int(ad.appliedKernels & 1u);
}
''')
    cuda_inc = Path(gb.nvcc()).resolve().parent.parent / "include"
    cxx = shutil.which("g++")
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-fsyntax-only",
                        "-I", str(REPO / "include"), "-I", str(cuda_inc), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_headless_driver_builds_and_links():
    import subprocess

    from gpusteer_gb300 import build as gb

    gb.build()
    r = subprocess.run([str(gb.HEADLESS)], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


PARAMS_DUMP = r'''
#include <cstdio>
#include "SimulationParams.h"
using namespace OpenSteer;
static void f3(const char* k, float3 v) { std::printf("%s %.9g %.9g %.9g\n", k, v.x, v.y, v.z); }
int main(int argc, char** argv) {
    SimulationParams p;
    try {
        p.load(argv[1]);
    } catch (ParamsError const& e) {
        std::printf("error %s\n", e.what());
        return 0;
    }
#define U(m, k) std::printf("%s %u\n", k, unsigned(p.m));
#define F(m, k) std::printf("%s %.9g\n", k, p.m);
    U(m_nSeed, "seed") U(m_nKNN, "knn") U(m_nKNO, "kno") U(m_nKNW, "knw")
    U(m_nSearchRadius, "searchRadius") U(m_bAvoidCloseNeighbors, "avoidCloseNeighbors")
    F(m_fMaxPursuitPredictionTime, "maxPursuitPredictionTime")
    F(m_fMinTimeToCollision, "minTimeToCollision") F(m_fMinTimeToObstacle, "minTimeToObstacle")
    F(m_fMinTimeToWall, "minTimeToWall") F(m_fPathPredictionTime, "pathPredictionTime")
    F(m_fMinSeparationDistance, "minSeparationDistance")
    F(m_fMaxSeparationDistance, "maxSeparationDistance")
    F(m_fMinFlockingDistance, "minFlockingDistance") F(m_fMaxFlockingDistance, "maxFlockingDistance")
    F(m_fCosMaxFlockingAngle, "cosMaxFlockingAngle")
    F(m_fWeightAlignment, "weightAlignment") F(m_fWeightCohesion, "weightCohesion")
    F(m_fWeightSeparation, "weightSeparation") F(m_fWeightPursuit, "weightPursuit")
    F(m_fWeightSeek, "weightSeek") F(m_fWeightFollowPath, "weightFollowPath")
    F(m_fWeightAvoidObstacles, "weightAvoidObstacles") F(m_fWeightAvoidWalls, "weightAvoidWalls")
    F(m_fWeightAvoidNeighbors, "weightAvoidNeighbors")
    U(m_nMaskAlignment, "maskAlignment") U(m_nMaskAntiPenetrationAgents, "maskAntiPenetrationAgents")
    U(m_nMaskCohesion, "maskCohesion") U(m_nMaskSeparation, "maskSeparation")
    U(m_nMaskSeek, "maskSeek") U(m_nMaskFlee, "maskFlee") U(m_nMaskPursuit, "maskPursuit")
    U(m_nMaskEvade, "maskEvade") U(m_nMaskFollowPath, "maskFollowPath")
    U(m_nMaskAvoidObstacles, "maskAvoidObstacles") U(m_nMaskAvoidWalls, "maskAvoidWalls")
    U(m_nMaskAvoidNeighbors, "maskAvoidNeighbors")
    f3("world.dimensions", p.m_WorldParams.m_f3Dimensions);
    std::printf("world.cells %u %u %u\n", p.m_WorldParams.m_u3Cells.x, p.m_WorldParams.m_u3Cells.y,
                p.m_WorldParams.m_u3Cells.z);
    std::printf("world.obstacleCount %u\n", p.m_WorldParams.m_nObstacleCount);
    std::printf("world.mapFilename %s\n", p.m_WorldParams.m_strMapFilename.c_str());
    for (GroupParams const& g : p.m_vecGroupParams) {
        std::printf("group %u %.9g %.9g %.9g %.9g %.9g %u\n", g.m_nNumAgents, g.m_fMaxSpeed,
                    g.m_fMaxForce, g.m_fMinStartRadius, g.m_fMaxStartRadius, g.m_fPathRadius,
                    unsigned(g.m_bPathIsCyclic));
        f3("group.startPosition", g.m_f3StartPosition);
        f3("group.bodyColor", g.m_f3BodyColor);
        for (float3 const& q : g.m_vecPathPoints) f3("group.point", q);
    }
    return 0;
}
'''


def _params_dump_binary(tmp_path):
    import shutil
    import subprocess

    from gpusteer_gb300 import build as gb

    src = tmp_path / "dump.cpp"
    src.write_text(PARAMS_DUMP)
    exe = tmp_path / "dump"
    cuda_inc = Path(gb.nvcc()).resolve().parent.parent / "include"
    r = subprocess.run([shutil.which("g++"), "-std=c++17", "-Wall", "-Werror", "-O1",
                        "-I", str(REPO / "include"), "-I", str(cuda_inc), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _python_dump(p) -> list:
    f32 = lambda x: float(np.float32(x))  # noqa: E731
    g9 = lambda x: f"{f32(x):.9g}"  # noqa: E731
    v = p.values
    lines = []
    for k in ("seed", "knn", "kno", "knw", "searchRadius", "avoidCloseNeighbors"):
        lines.append(f"{k} {int(v.get(k, 0))}")
    for k in ("maxPursuitPredictionTime", "minTimeToCollision", "minTimeToObstacle",
              "minTimeToWall", "pathPredictionTime", "minSeparationDistance",
              "maxSeparationDistance", "minFlockingDistance", "maxFlockingDistance",
              "cosMaxFlockingAngle", "weightAlignment", "weightCohesion", "weightSeparation",
              "weightPursuit", "weightSeek", "weightFollowPath", "weightAvoidObstacles",
              "weightAvoidWalls", "weightAvoidNeighbors"):
        lines.append(f"{k} {g9(v.get(k, 0.0))}")
    for k in ("maskAlignment", "maskAntiPenetrationAgents", "maskCohesion", "maskSeparation",
              "maskSeek", "maskFlee", "maskPursuit", "maskEvade", "maskFollowPath",
              "maskAvoidObstacles", "maskAvoidWalls", "maskAvoidNeighbors"):
        lines.append(f"{k} {int(v.get(k, 0))}")
    w = p.world
    lines.append("world.dimensions " + " ".join(g9(x) for x in w.get("dimensions", (0, 0, 0))))
    lines.append("world.cells " + " ".join(str(x) for x in w.get("cells", (0, 0, 0))))
    lines.append(f"world.obstacleCount {w.get('obstacleCount', 0)}")
    lines.append(f"world.mapFilename {w.get('mapFilename', '')}")
    for g in p.groups:
        lines.append(f"group {g.get('numAgents', 0)} {g9(g.get('maxSpeed', 0))} "
                     f"{g9(g.get('maxForce', 0))} {g9(g.get('minStartRadius', 0))} "
                     f"{g9(g.get('maxStartRadius', 0))} {g9(g.get('pathRadius', 0))} "
                     f"{int(g.get('cyclic', 0))}")
        lines.append("group.startPosition " + " ".join(g9(x) for x in g.get("startPosition", (0, 0, 0))))
        lines.append("group.bodyColor " + " ".join(g9(x) for x in g.get("bodyColor", (0, 0, 0))))
        for q in g["path"]:
            lines.append("group.point " + " ".join(g9(x) for x in q))
    return lines


def test_cpp_simulation_params_loader_matches_python_reader(tmp_path):
    """include/SimulationParams.h (SimulationParams::load, Simulation.cpp:7-250)
    and the Python reader agree on every value of a scenario file, and of the
    reference's own data/*.params files where the reference tree is present."""
    import subprocess

    exe = _params_dump_binary(tmp_path)
    text = """# header
    seed = 7
    knn = 6 # comment after a value
    cosMaxFlockingAngle = -0.86602540378443864676372317075294
    avoidCloseNeighbors = 1
    maskSeek = 4480
    weightSeek = 1.5
    <world>
        dimensions = 2048 10 2048
        cells = 512 1 512
        mapFilename = ChokePoint20.map
    </world>
    <group>
        numAgents = 100
        maxSpeed = 3
        <path>
            point = 0 0 13.5
            #radius = 5
            point = 0 0 -1650
            radius = 20
            cyclic = 0
        </path>
        bodyColor = 0.4 0.4 0.6 # Bluish
    </group>
    </simulation>
    """
    files = [tmp_path / "synthetic.params"]
    files[0].write_text(text)
    data = ol.reference_root() / "data"
    if data.exists():
        files += sorted(data.glob("*.params"))
    for f in files:
        got = subprocess.run([str(exe), str(f)], capture_output=True, text=True).stdout.split("\n")
        want = _python_dump(sc.load_params(f.read_text()))
        assert got[:len(want)] == want, f.name
    bad = tmp_path / "bad.params"
    bad.write_text("bogusKey = 1\n</simulation>\n")
    out = subprocess.run([str(exe), str(bad)], capture_output=True, text=True).stdout
    assert out.startswith("error unknown key bogusKey")


def test_parameter_blocks_match_the_header(tmp_path):
    """The ctypes mirrors of gs_step_params and gs_multigroup_params have the C
    header's size and field offsets."""
    import ctypes
    import shutil
    import subprocess

    from gpusteer_gb300 import build as gb
    from gpusteer_gb300.groups import MultiGroupParams, _StepParamsC

    checks = {"gs_multigroup_params": MultiGroupParams, "gs_step_params": _StepParamsC}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "gpusteer.h"', "int main(void) {"]
    for cname, cls in checks.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    cuda_inc = Path(gb.nvcc()).resolve().parent.parent / "include"
    r = subprocess.run([shutil.which("gcc"), "-std=c99", "-Wall", "-I", str(REPO / "include"),
                        "-I", str(cuda_inc), str(src), "-o", str(exe)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True).stdout.split("\n")
    got = {tuple(line.split()[:2]): int(line.split()[2]) for line in out if line.strip()}
    for cname, cls in checks.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for field, _ in cls._fields_:
            assert got[(cname, field)] == getattr(cls, field).offset, (cname, field)


def test_chunk_box_distance_bounds_every_inside_candidate():
    """The bucketed brute force skips a chunk of candidates when the squared
    distance from a query to the chunk's bounding box, in the reference's
    unfused binary32 operations, exceeds the filter bound.  That is safe
    because the box's value is at most every inside candidate's exact squared
    distance: per axis fl(lo - q) or fl(q - hi) is at most |fl(q - c)|
    (rounding is monotone), and so are the squares and the sums.  Checked
    here in float32 numpy arithmetic on boxes that are points, on ones that
    straddle the query, and across magnitudes from 1e-3 to 1e18."""
    rng = np.random.default_rng(5)
    f = np.float32
    for scale in (1e-3, 1.0, 512.0, 1e6, 1e18):
        q = (rng.uniform(-1, 1, (4000, 3)) * scale).astype(f)
        c = (rng.uniform(-1, 1, (4000, 32, 3)) * scale).astype(f)
        c[::7] = c[::7, :1]                      # every candidate at one point
        c[1::7] += q[1::7, None, :] - c[1::7, :1]  # the query on the box's corner
        lo, hi = c.min(axis=1), c.max(axis=1)
        zero = f(0)
        gap = np.maximum(np.maximum(lo - q, q - hi), zero)
        box = (gap[:, 0] * gap[:, 0] + gap[:, 1] * gap[:, 1]) + gap[:, 2] * gap[:, 2]
        o = q[:, None, :] - c
        d2 = (o[..., 0] * o[..., 0] + o[..., 1] * o[..., 1]) + o[..., 2] * o[..., 2]
        assert box.dtype == np.float32 and d2.dtype == np.float32
        finite = np.isfinite(d2)
        assert (box[:, None] <= d2)[finite].all()


def _ru_mul(a, b):
    """binary32 a * b rounded up (the float64 product of two binary32 values
    is exact)."""
    prod = np.float64(a) * np.float64(b)
    x = np.float32(prod)
    return np.nextafter(x, np.float32(np.inf)) if np.float64(x) < prod else x


def _bucketed_brute_lists(pos, k, per_axis):
    """A restatement of the bucketed brute force's pruning for self searches:
    per query the seed (k-th distance among the candidates of its 3 x 3 x 3
    cells, widened to 5 x 5 x 5 and 9 x 9 x 9 when they hold fewer than k),
    the filter bound rounded up from it, chunks of 64 bucketed candidates
    skipped for a warp of four bucketed queries when their box's squared
    distance exceeds every query's bound; then each query's (distance, index)
    top k among the candidates of the chunks its warp kept."""
    f = np.float32
    p = pos[:, :3].astype(f)
    n = p.shape[0]
    lo_w, hi_w = p.min(0), p.max(0)
    cell3 = np.clip(((p - lo_w) / (hi_w - lo_w + f(1e-3)) * per_axis).astype(np.int64), 0,
                    per_axis - 1)
    cell = (cell3[:, 1] * per_axis + cell3[:, 2]) * per_axis + cell3[:, 0]
    order = np.argsort(cell, kind="stable")          # bucket order
    bp, bc3 = p[order], cell3[order]

    def dist(q, c):
        o = q - c
        return np.sqrt((o[..., 0] * o[..., 0] + o[..., 1] * o[..., 1]) + o[..., 2] * o[..., 2])

    bound = np.empty(n, f)
    for s in range(n):
        for r in (1, 2, 4):
            near = np.all(np.abs(bc3 - bc3[s]) <= r, axis=1)
            near[s] = False
            d = dist(bp[s], bp[near])
            if d.size >= k:
                kth = np.partition(d, k - 1)[k - 1]
                bound[s] = _ru_mul(_ru_mul(kth, kth), f(1.000004))
                break
        else:
            bound[s] = np.inf
    chunks = (n + 63) // 64
    clo = np.stack([bp[c * 64:(c + 1) * 64].min(0) for c in range(chunks)])
    chi = np.stack([bp[c * 64:(c + 1) * 64].max(0) for c in range(chunks)])
    out_idx = np.empty((k, n), np.uint32)
    out_dist = np.empty((k, n), f)
    kept = 0
    for w0 in range(0, n, 4):
        qs = range(w0, min(w0 + 4, n))
        keep = np.zeros(chunks, bool)
        for s in qs:
            gap = np.maximum(np.maximum(clo - bp[s], bp[s] - chi), f(0))
            box = (gap[:, 0] * gap[:, 0] + gap[:, 1] * gap[:, 1]) + gap[:, 2] * gap[:, 2]
            keep |= box <= bound[s]
        kept += int(keep.sum())
        cand = np.concatenate([np.arange(c * 64, min(c * 64 + 64, n))
                               for c in np.flatnonzero(keep)])
        for s in qs:
            c = cand[cand != s]
            d = dist(bp[s], bp[c])
            ids = order[c].astype(np.uint32)
            pick = np.lexsort((ids, d))[:k]
            a = order[s]
            out_idx[:, a] = ids[pick]
            out_dist[:, a] = d[pick]
    return out_idx.reshape(-1), out_dist.reshape(-1), kept / (chunks * ((n + 3) // 4))


@pytest.mark.parametrize("case", ["cube", "lattice", "flat", "clusters"])
def test_bucketed_brute_force_pruning_keeps_every_list(case):
    """The bucketed brute force's seed and chunk skipping, restated on the CPU,
    give the oracle's full-scan lists: uniform, lattice with duplicated
    points (distance ties broken by the lower index), flat 2D crowd and
    tight clusters, at k = 8, 16 and 40."""
    rng = np.random.default_rng(11)
    if case == "cube":
        pos = sc.boids_cube(2500, size=64.0, seed=3).position
    elif case == "lattice":
        g3 = np.stack(np.meshgrid(*(np.arange(12),) * 3, indexing="ij"), -1)
        lat = g3.reshape(-1, 3).astype(np.float32) - 6.0
        lat = np.concatenate([lat, lat[::5]])
        pos = np.zeros((lat.shape[0], 4), np.float32)
        pos[:, :3] = lat
    elif case == "flat":
        pos = sc.chokepoint_agents(2500, seed=4).position
    else:
        centres = rng.uniform(-200, 200, (6, 3))
        pts = centres[rng.integers(0, 6, 2400)] + rng.normal(0, 2.0, (2400, 3))
        pos = np.zeros((2400, 4), np.float32)
        pos[:, :3] = pts
    pos = np.ascontiguousarray(pos, np.float32)
    for k in (8, 16, 40):
        want_i, want_d = ol.knn_brute(pos, pos, True, k)
        got_i, got_d, kept = _bucketed_brute_lists(pos, k, per_axis=11)
        np.testing.assert_array_equal(got_i, want_i)
        np.testing.assert_array_equal(got_d, want_d)
        assert kept < 0.5, kept  # the pruning is not vacuous
