"""gs_knn_binned_noalloc against gs_update_knn_database + gs_find_knn.

The no-allocation entry point serves callers that cannot let the library
allocate device memory (pre-sized pools, real-time loops, external
allocation accounting): it works out of a fixed array inside the library.
Its results must be identical to the regular path's, and stay identical on a
second call that reuses the array left behind by the first.  This file is
collected last so that a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

import gpusteer_gb300 as gs
from gpusteer_gb300 import _lib, scenario as sc
from gpusteer_gb300.state import AgentState

pytestmark = pytest.mark.gpu


def regular_knn(state, cells, size, r, k):
    g = gs.AgentGroup(k, state.n)
    g.upload(state)
    bins = gs.KNNBinData(cells, size, r)
    gs.updateKNNDatabase(g, bins)
    knn = gs.KNNData(state.n, k)
    gs.findKNearestNeighbors(g, knn, bins, g, r)
    return knn.download(g)


def noalloc_knn(state, cells, size, r, k):
    lib = _lib.load()
    g = gs.AgentGroup(k, state.n)  # holds the input positions on the device
    g.upload(state)
    pos = g.device_arrays()["position"]
    out = gs.KNNData(state.n, k)  # holds the outputs on the device
    idx, dist = C.POINTER(C.c_uint)(), C.POINTER(C.c_float)()
    _lib.check(lib.gs_knn_device_arrays(out.handle, C.byref(idx), C.byref(dist)))
    _lib.check(lib.gs_knn_binned_noalloc(
        C.c_void_p(pos), state.n, (C.c_uint * 3)(*cells), (C.c_float * 3)(*size), r, k,
        C.cast(idx, C.c_void_p), C.cast(dist, C.c_void_p), C.c_void_p(g.stream)))
    return out.download(g)


@pytest.mark.parametrize("k", [7, 16])
@pytest.mark.parametrize("r", [1, 2])
def test_noalloc_knn_equals_regular_path_on_two_calls(k, r):
    cases = [
        (sc.boids_sphere(20000, radius=40.0, seed=1), (32, 32, 32), (128.0, 128.0, 128.0)),
        # a flat grid (one cell high): the 2D worlds on the x-z plane
        (sc.chokepoint_agents(15000, seed=2), (128, 1, 128), (256.0, 10.0, 256.0)),
    ]
    for state, cells, size in cases:  # two calls in a row on the shared array
        want_i, want_d = regular_knn(state, cells, size, r, k)
        got_i, got_d = noalloc_knn(state, cells, size, r, k)
        np.testing.assert_array_equal(got_i, want_i)
        np.testing.assert_array_equal(got_d, want_d)


def test_noalloc_knn_rejects_problems_beyond_its_array():
    lib = _lib.load()
    s = AgentState.zeros(4)
    g = gs.AgentGroup(4, 4)
    g.upload(s)
    out = gs.KNNData(4, 4)
    idx, dist = C.POINTER(C.c_uint)(), C.POINTER(C.c_float)()
    _lib.check(lib.gs_knn_device_arrays(out.handle, C.byref(idx), C.byref(dist)))
    cells = (1024, 1024, 16)  # 16.7 M cells: far beyond the fixed array
    st = lib.gs_knn_binned_noalloc(C.c_void_p(g.device_arrays()["position"]), 4,
                                   (C.c_uint * 3)(*cells), (C.c_float * 3)(64.0, 64.0, 64.0), 1,
                                   4, C.cast(idx, C.c_void_p), C.cast(dist, C.c_void_p),
                                   C.c_void_p(g.stream))
    assert st == 1  # GS_ERR_INVALID_ARG, nothing launched
    assert b"32 MiB" in lib.gs_last_error()
    # a cell count whose 64-bit product wraps (2^31 * 2^31 * 4 = 2^64) is
    # rejected before anything is launched
    st = lib.gs_knn_binned_noalloc(C.c_void_p(g.device_arrays()["position"]), 4,
                                   (C.c_uint * 3)(1 << 31, 1 << 31, 4),
                                   (C.c_float * 3)(64.0, 64.0, 64.0), 1, 4,
                                   C.cast(idx, C.c_void_p), C.cast(dist, C.c_void_p),
                                   C.c_void_p(g.stream))
    assert st == 1
    assert b"too many cells" in lib.gs_last_error()
