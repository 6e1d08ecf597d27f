"""Python mirror of the reference's group API over the C ABI.

Classes follow the reference objects (AgentGroup, KNNData, KNNBinData,
WallGroup) and the free functions keep the names and argument order of
include/OpenSteer/CUDA/GroupSteerLibrary.cuh:43-223, so a plugin's update
(e.g. plugins/BoidsGroup.cpp:606-637) reads the same here.  Failures raise
GpuSteerError instead of aborting the process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import AgentArrays, StepParams as _StepParamsC, call
from .scenario import StepParams, WRAP_REFERENCE
from .state import AgentState

_fp = C.POINTER(C.c_float)
_up = C.POINTER(C.c_uint)


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


def _u3(v):
    return (C.c_uint * 3)(*[int(x) for x in v])


def _ptr(a: np.ndarray, t=C.c_float):
    if not a.flags.c_contiguous:
        raise ValueError("arrays must be C-contiguous")
    return a.ctypes.data_as(C.POINTER(t))


def host_arrays(s: AgentState) -> AgentArrays:
    """AgentArrays pointing at the numpy arrays of `s` (kept alive by the caller)."""
    a = AgentArrays()
    for k in AgentState.float_names():
        arr = getattr(s, k)
        if arr.dtype != np.float32:
            raise TypeError(f"{k} must be float32")
        setattr(a, k, _ptr(arr))
    if s.applied.dtype != np.uint32:
        raise TypeError("applied must be uint32")
    a.applied = _ptr(s.applied, C.c_uint)
    return a


def step_params_c(p: StepParams, path=None) -> _StepParamsC:
    """The C parameter block; `path` (a Path) serves GS_B_FOLLOW_PATH."""
    s = _StepParamsC()
    for name, _ in _StepParamsC._fields_:
        if name in ("order", "n_order", "path"):
            continue
        v = getattr(p, name)
        if isinstance(v, (tuple, list)):
            arr = getattr(s, name)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(s, name, v)
    if len(p.order) > 8:
        raise ValueError("at most 8 behaviours")
    for i, b in enumerate(p.order):
        s.order[i] = int(b)
    s.n_order = len(p.order)
    if path is not None:
        s.path = path.handle.value
    return s


class Path:
    """PolylinePathwayCUDA(points, radius, cyclic) (PolylinePathwayCUDA.cu:7-56)."""

    def __init__(self, points, radius: float, cyclic: bool = False):
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        h = C.c_void_p()
        call("gs_path_create", _ptr(pts), pts.shape[0], float(radius), int(bool(cyclic)),
             C.byref(h))
        self._h = h
        self.radius = float(radius)
        self.cyclic = bool(cyclic)
        self.points_in = pts

    @property
    def handle(self):
        return self._h

    def arrays(self):
        """(points (n, 3), lengths (n,), normals (n, 3), total length)."""
        n = C.c_uint()
        call("gs_path_get", self._h, None, None, None, 0, C.byref(n), None)
        po = np.zeros((n.value, 3), np.float32)
        ln = np.zeros(n.value, np.float32)
        nm = np.zeros((n.value, 3), np.float32)
        tot = np.zeros(1, np.float32)
        call("gs_path_get", self._h, _ptr(po), _ptr(ln), _ptr(nm), n.value, C.byref(n),
             _ptr(tot))
        return po, ln, nm, float(tot[0])

    def __del__(self):
        if getattr(self, "_h", None) and _lib._lib is not None:
            _lib._lib.gs_path_destroy(self._h)
            self._h = None


class KNNBinData:
    """KNNBinDataV2(worldCells, worldSize, searchRadius), KNNBinDataV2.cu:30-42."""

    def __init__(self, world_cells, world_size, search_radius: int = 1):
        h = C.c_void_p()
        call("gs_bins_create", _u3(world_cells), _f3(world_size), int(search_radius), C.byref(h))
        self._h = h
        self.world_cells = tuple(int(x) for x in world_cells)
        self.world_size = tuple(float(x) for x in world_size)
        self.search_radius = int(search_radius)

    @property
    def handle(self):
        return self._h

    @property
    def num_cells(self) -> int:
        n = C.c_uint()
        call("gs_bins_num_cells", self._h, C.byref(n))
        return n.value

    def hv_cells(self):
        """(min, max, centre) float3 per cell in bin_cell order."""
        n = self.num_cells
        lo, hi, c = (np.zeros((n, 3), np.float32) for _ in range(3))
        call("gs_bins_get_cells", self._h, _ptr(lo), _ptr(hi), _ptr(c), n)
        return lo, hi, c

    def __del__(self):
        if getattr(self, "_h", None) and _lib._lib is not None:
            _lib._lib.gs_bins_destroy(self._h)
            self._h = None


class AgentGroup:
    """AgentGroup(worldCells, knn) (src/AgentGroup.cpp:8-11) with its device
    arrays and binning database."""

    def __init__(self, k: int, capacity: int, stream: int | None = None):
        h = C.c_void_p()
        call("gs_group_create", int(k), int(capacity), C.c_void_p(stream) if stream else None,
             C.byref(h))
        self._h = h
        self.k = int(k)
        self.capacity = int(capacity)

    @property
    def handle(self):
        return self._h

    def upload(self, s: AgentState) -> None:
        """Clear + AddAgent* + SyncDevice."""
        a = host_arrays(s)
        call("gs_group_upload", self._h, C.byref(a), s.n)
        # the copies are asynchronous: keep the host arrays alive until done
        call("gs_group_synchronize", self._h)

    def download(self) -> AgentState:
        """SyncHost: the whole state as host arrays."""
        out = AgentState.zeros(self.size)
        a = host_arrays(out)
        call("gs_group_download", self._h, C.byref(a))
        return out

    @property
    def size(self) -> int:
        n = C.c_uint()
        call("gs_group_size", self._h, C.byref(n))
        return n.value

    def device_arrays(self) -> dict:
        """pdPosition()/pdDirection()/...: device addresses (ints)."""
        a = AgentArrays()
        call("gs_group_device_arrays", self._h, C.byref(a))
        return {name: C.cast(getattr(a, name), C.c_void_p).value for name, _ in AgentArrays._fields_}

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        call("gs_group_stream", self._h, C.byref(s))
        return s.value or 0

    def synchronize(self) -> None:
        call("gs_group_synchronize", self._h)

    def __del__(self):
        if getattr(self, "_h", None) and _lib._lib is not None:
            _lib._lib.gs_group_destroy(self._h)
            self._h = None


class KNNData:
    """KNNData(nSize, nK): column-major k x n indices and distances."""

    def __init__(self, n: int, k: int):
        h = C.c_void_p()
        call("gs_knn_create", int(n), int(k), C.byref(h))
        self._h = h
        self.n, self.k = int(n), int(k)

    @property
    def handle(self):
        return self._h

    def download(self, group: AgentGroup | None = None):
        idx = np.empty(self.k * self.n, np.uint32)
        dist = np.empty(self.k * self.n, np.float32)
        call("gs_knn_download", self._h, group.handle if group else None, _ptr(idx, C.c_uint),
             _ptr(dist))
        return idx, dist

    def upload(self, idx: np.ndarray | None, dist: np.ndarray | None = None,
               group: AgentGroup | None = None) -> None:
        """Writes the lists (column-major, k * n) from the host, as a caller of
        the reference writes pdKNNIndices() / pdKNNDistances()."""
        cnt = self.k * self.n
        i = None if idx is None else np.ascontiguousarray(idx, np.uint32).reshape(-1)
        d = None if dist is None else np.ascontiguousarray(dist, np.float32).reshape(-1)
        if (i is not None and i.size != cnt) or (d is not None and d.size != cnt):
            raise ValueError(f"KNN arrays must hold k * n = {cnt} entries")
        call("gs_knn_upload", self._h, group.handle if group else None,
             None if i is None else _ptr(i, C.c_uint), None if d is None else _ptr(d))

    def __del__(self):
        if getattr(self, "_h", None) and _lib._lib is not None:
            _lib._lib.gs_knn_destroy(self._h)
            self._h = None


class WallGroup:
    """WallGroup: LoadFromFile + SplitWalls + SyncDevice (ChokePointNew.cpp:107-119)."""

    def __init__(self, rows: np.ndarray | None = None, bins: KNNBinData | None = None,
                 knw: int = 3, path: str | None = None):
        h = C.c_void_p()
        if path is not None:
            call("gs_walls_load", path.encode(), bins.handle if bins else None, int(knw),
                 C.byref(h))
        else:
            rows = np.asarray(rows, np.float32).reshape(-1, 9)
            n = rows.shape[0]
            st = np.zeros((n, 4), np.float32)
            en = np.zeros((n, 4), np.float32)
            nm = np.zeros((n, 4), np.float32)
            st[:, :3], en[:, :3], nm[:, :3] = rows[:, 0:3], rows[:, 3:6], rows[:, 6:9]
            call("gs_walls_create", _ptr(st), _ptr(en), _ptr(nm), n,
                 bins.handle if bins else None, int(knw), C.byref(h))
        self._h = h
        self.knw = int(knw)

    @property
    def handle(self):
        return self._h

    @property
    def size(self) -> int:
        n = C.c_uint()
        call("gs_walls_size", self._h, C.byref(n))
        return n.value

    def download(self):
        n = self.size
        out = [np.zeros((n, 4), np.float32) for _ in range(4)]
        call("gs_walls_download", self._h, *[_ptr(o) for o in out], n)
        return tuple(out)

    def __del__(self):
        if getattr(self, "_h", None) and _lib._lib is not None:
            _lib._lib.gs_walls_destroy(self._h)
            self._h = None


class _GroupRef:
    """A non-owning view of a group handle (e.g. a batch's underlying group)."""

    def __init__(self, handle, k: int):
        self._h = handle
        self.k = int(k)

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        st = C.c_void_p()
        call("gs_group_stream", self._h, C.byref(st))
        return st.value or 0

    def synchronize(self) -> None:
        call("gs_group_synchronize", self._h)


def set_graphs(group, enable: bool) -> None:
    call("gs_group_set_graphs", group.handle, int(bool(enable)))


def set_block(group, threads: int) -> None:
    call("gs_group_set_block", group.handle, int(threads))


def set_persistent(group, enable: bool) -> None:
    """One persistent launch per supported step (avoid-walls first, 9 <= k <=
    16, a flat world, the streaming KNN scan) instead of separate launches;
    results equal the separate launches bit for bit."""
    call("gs_group_set_persistent", group.handle, int(bool(enable)))
    group.persistent = bool(enable)


def set_barrier_limit(group, polls: int) -> None:
    """Polls a persistent step's barrier wait makes before it gives up (0:
    the default); a step that gave up is void and the next synchronize raises
    GS_ERR_TIMEOUT."""
    call("gs_group_set_barrier_limit", group.handle, int(polls))


def set_knn_capacity(group, capacity: int) -> None:
    """0 = from the crowd's density; 32/64 collecting scan; 128/256 streaming."""
    call("gs_group_set_knn_capacity", group.handle, int(capacity))


def knn_capacity(group) -> int:
    """The capacity the fused step uses (the fixed one, else the one measured
    at the last step; 0 before the first step)."""
    out = C.c_uint(0)
    call("gs_group_knn_capacity", group.handle, C.byref(out))
    return int(out.value)


def step_launches(group, walls: bool) -> int:
    """Kernel launches of one fused step: the counting-sort scan, the
    permute, the fused kernel (two with walls), and with the streaming scan
    (capacity 128 or 256) the warp-per-agent exact lists, plus, without
    walls, the exact redo (with walls the lists go straight to the second
    half; the collecting scan redoes its rare agents inline)."""
    cap = knn_capacity(group)
    if getattr(group, "persistent", False) and walls and cap > 64 and 8 < group.k <= 16:
        return 1
    redo = (1 if walls else 2) if cap > 64 else 0
    return 1 + 1 + (2 if walls else 1) + redo


class Batch:
    """Many independent scenes advanced together (gs_batch_*): agents are
    concatenated in scene order, each scene keeps scene-local indices, cells
    and walls, and its result equals stepping it alone."""

    def __init__(self, counts, k: int, world_cells, world_size, search_radius: int = 1,
                 stream: int | None = None):
        counts = np.ascontiguousarray(counts, np.uint32)
        h = C.c_void_p()
        call("gs_batch_create", len(counts), _ptr(counts, C.c_uint), int(k), _u3(world_cells),
             _f3(world_size), int(search_radius), C.c_void_p(stream) if stream else None,
             C.byref(h))
        self._h = h
        self.counts = counts
        self.n = int(counts.sum())
        self.cells_per_scene = int(np.prod(np.asarray(world_cells, np.uint64)))
        g = C.c_void_p()
        call("gs_batch_group", h, C.byref(g))
        self.group = _GroupRef(g, k)

    @property
    def handle(self):
        return self._h

    def set_walls(self, scene: int, rows: np.ndarray) -> None:
        rows = np.asarray(rows, np.float32).reshape(-1, 9)
        n = rows.shape[0]
        st = np.zeros((n, 4), np.float32)
        en = np.zeros((n, 4), np.float32)
        nm = np.zeros((n, 4), np.float32)
        st[:, :3], en[:, :3], nm[:, :3] = rows[:, 0:3], rows[:, 3:6], rows[:, 6:9]
        call("gs_batch_set_walls", self._h, int(scene), _ptr(st), _ptr(en), _ptr(nm), n)

    def upload(self, s: AgentState) -> None:
        if s.n != self.n:
            raise ValueError("state size differs from the batch")
        a = host_arrays(s)
        call("gs_batch_upload", self._h, C.byref(a))
        self.group.synchronize()

    def download(self, out: AgentState | None = None) -> AgentState:
        """All scenes' agents in scene order (into `out` when given)."""
        if out is None:
            out = AgentState.zeros(self.n)
        elif out.n != self.n:
            raise ValueError("state size differs from the batch")
        a = host_arrays(out)
        call("gs_batch_download", self._h, C.byref(a))
        return out

    def step(self, params: StepParams, steps: int = 1) -> None:
        p = step_params_c(params)
        call("gs_batch_step", self._h, C.byref(p), int(steps))

    def cell_density(self) -> np.ndarray:
        """Agents per cell of the last step's frame, (scenes, cells)."""
        out = np.zeros((len(self.counts), self.cells_per_scene), np.uint32)
        call("gs_batch_cell_density", self._h, _ptr(out, C.c_uint))
        return out

    def cell_avg_velocity(self) -> np.ndarray:
        """Mean velocity per cell of the last step's frame, (scenes, cells, 3)."""
        out = np.zeros((len(self.counts), self.cells_per_scene, 3), np.float32)
        call("gs_batch_cell_avg_velocity", self._h, _ptr(out))
        return out

    def __del__(self):
        if getattr(self, "_h", None) and _lib._lib is not None:
            _lib._lib.gs_batch_destroy(self._h)
            self._h = None


def pinned_state(n: int) -> AgentState:
    """An AgentState whose arrays live in page-locked host memory
    (gs_host_alloc), freed with the state.  Host copies from it overlap with
    device work and can be captured in graphs; its arrays are laid out in the
    library's three blocks (position, direction, steering | side, up | speed,
    maxSpeed, maxForce, radius, mass, applied), so each block moves in one
    pitched copy."""
    import weakref

    blocks = [(("position", "direction", "steering"), 4), (("side", "up"), 3),
              (("speed", "max_speed", "max_force", "radius", "mass", "applied"), 1)]
    arrays, ptrs = {}, []
    lib = _lib.load()
    for names, width in blocks:
        count = max(1, len(names) * n * width)
        p = C.c_void_p()
        call("gs_host_alloc", count * 4, C.byref(p))
        ptrs.append(p)
        for j, k in enumerate(names):
            ctype = C.c_uint if k == "applied" else C.c_float
            buf = (ctype * (n * width)).from_address(p.value + 4 * j * n * width)
            a = np.ctypeslib.as_array(buf) if n else np.zeros(0, np.float32)
            arrays[k] = a.reshape((n, width)) if width > 1 else a
    st = AgentState(**arrays)
    weakref.finalize(st, lambda ps=ptrs: [lib.gs_host_free(q) for q in ps])
    return st


def batches_step_host(parts, params: StepParams, steps: int, state_in: AgentState,
                      state_out: AgentState) -> None:
    """gs_batches_step_host: host state in, `steps` steps, host state out for
    several Batch objects (the parts of one workload) with their copies and
    steps overlapped across the parts' streams.  The states hold the parts'
    agents one part after another."""
    total = sum(b.n for b in parts)
    if state_in.n != total or state_out.n != total:
        raise ValueError("host states must hold every part's agents")
    p = step_params_c(params)
    hs = (C.c_void_p * len(parts))(*[b.handle for b in parts])
    a_in, a_out = host_arrays(state_in), host_arrays(state_out)
    call("gs_batches_step_host", hs, len(parts), C.byref(p), int(steps), C.byref(a_in),
         C.byref(a_out))


class Rollout:
    """Checkpointed differentiable rollout of a plain flock (gs_rollout_*):
    `steps` fused steps from the group's state, then the adjoint backwards
    with KNN lists and memberships frozen.  Device arrays are passed as raw
    pointers (float4 per agent, agent order)."""

    def __init__(self, group: AgentGroup, bins: KNNBinData, steps: int,
                 checkpoint_every: int = 8):
        h = C.c_void_p()
        call("gs_rollout_create", group.handle, bins.handle, int(steps), int(checkpoint_every),
             C.byref(h))
        self._h = h
        self.group = group
        self.steps = steps

    def forward(self, params: StepParams) -> None:
        p = step_params_c(params)
        call("gs_rollout_forward", self._h, C.byref(p))

    def backward(self, adj_position: int | None, adj_velocity: int | None = None,
                 grad_position0: int | None = None, grad_velocity0: int | None = None):
        """Returns d loss / d (w_separation, w_alignment, w_cohesion)."""
        gw = np.zeros(3, np.float32)
        vp = lambda x: C.c_void_p(x) if x else None  # noqa: E731
        call("gs_rollout_backward", self._h, vp(adj_position), vp(adj_velocity),
             vp(grad_position0), vp(grad_velocity0), _ptr(gw))
        return gw

    def __del__(self):
        if getattr(self, "_h", None) and _lib._lib is not None:
            _lib._lib.gs_rollout_destroy(self._h)
            self._h = None


# ---- GroupSteerLibrary.cuh -----------------------------------------------------------

def wrapWorld(group: AgentGroup, world_size, mode: int = WRAP_REFERENCE) -> None:
    call("gs_wrap_world", group.handle, _f3(world_size), int(mode))


def updateKNNDatabase(group, bins: KNNBinData) -> None:
    if isinstance(group, WallGroup):
        call("gs_walls_update_knn_database", group.handle, bins.handle)
    else:
        call("gs_update_knn_database", group.handle, bins.handle)


def findKNearestNeighbors(group: AgentGroup, knn: KNNData, bins: KNNBinData, other,
                          search_radius: int = 1) -> None:
    if isinstance(other, WallGroup):
        call("gs_find_knn_walls", group.handle, knn.handle, bins.handle, other.handle,
             int(search_radius))
    else:
        call("gs_find_knn", group.handle, knn.handle, bins.handle, other.handle,
             int(search_radius))


def findKNearestNeighborsGroups(groups, bins: KNNBinData, knns) -> None:
    """findKNearestNeighbors for every group pair of a MultiGroup frame in one
    launch: knns[i][j] (None to skip) gets group i's lists against group j."""
    G = len(groups)
    hs = (C.c_void_p * G)(*[grp.handle for grp in groups])
    out = (C.c_void_p * (G * G))(*[(knns[i][j].handle if knns[i][j] is not None else None)
                                   for i in range(G) for j in range(G)])
    call("gs_find_knn_groups", hs, G, bins.handle, out)


class MultiGroupParams(C.Structure):
    """gs_multigroup_params: the values a MultiGroup frame reads."""
    _fields_ = [("world_size", C.c_float * 3), ("wrap_mode", C.c_int),
                ("min_time_to_collision", C.c_float), ("min_separation_distance", C.c_float),
                ("avoid_close", C.c_int), ("w_avoid", C.c_float), ("mask_avoid", C.c_uint),
                ("sep_min", C.c_float), ("sep_max", C.c_float), ("sep_cos", C.c_float),
                ("w_sep", C.c_float), ("mask_sep", C.c_uint),
                ("ali_min", C.c_float), ("ali_max", C.c_float), ("ali_cos", C.c_float),
                ("w_ali", C.c_float), ("mask_ali", C.c_uint),
                ("coh_min", C.c_float), ("coh_max", C.c_float), ("coh_cos", C.c_float),
                ("w_coh", C.c_float), ("mask_coh", C.c_uint),
                ("path_prediction_time", C.c_float), ("w_path", C.c_float),
                ("mask_path", C.c_uint), ("w_seek", C.c_float), ("mask_seek", C.c_uint),
                ("mask_antipen", C.c_uint), ("dt", C.c_float)]

    def __init__(self, **kw):
        super().__init__()
        for k, v in kw.items():
            if k == "world_size":
                self.world_size = (C.c_float * 3)(*v)
            else:
                setattr(self, k, v)


def multigroup_step(groups, bins: KNNBinData, knns, params: MultiGroupParams, steps: int = 1,
                    paths=None) -> None:
    """gs_multigroup_step: `steps` MultiGroup frames; knns[i][j] are group i's
    lists against group j (all pairs), paths[i] a Path or None."""
    G = len(groups)
    hs = (C.c_void_p * G)(*[grp.handle for grp in groups])
    ps = None
    if paths is not None:
        ps = (C.c_void_p * G)(*[(q.handle if q is not None else None) for q in paths])
    ks = (C.c_void_p * (G * G))(*[knns[i][j].handle for i in range(G) for j in range(G)])
    call("gs_multigroup_step", hs, G, bins.handle, ps, ks, C.byref(params), int(steps))


def findKNearestNeighborsBruteForce(group: AgentGroup, knn: KNNData, other: AgentGroup) -> None:
    call("gs_knn_bruteforce", group.handle, knn.handle, other.handle)


def bruteforce_pairs(group: AgentGroup) -> int:
    """gs_knn_bruteforce_pairs: the (query, candidate) pairs the group's last
    brute-force call ran its distance filter on."""
    out = C.c_ulonglong(0)
    call("gs_knn_bruteforce_pairs", group.handle, C.byref(out))
    return out.value


def steerForSeparation(group, knn, other, min_distance, max_distance, cos_max_angle, weight,
                       do_not_apply_with=0) -> None:
    call("gs_steer_for_separation", group.handle, knn.handle, other.handle, min_distance,
         max_distance, cos_max_angle, weight, int(do_not_apply_with))


def steerForAlignment(group, knn, other, min_distance, max_distance, cos_max_angle, weight,
                      do_not_apply_with=0) -> None:
    call("gs_steer_for_alignment", group.handle, knn.handle, other.handle, min_distance,
         max_distance, cos_max_angle, weight, int(do_not_apply_with))


def steerForCohesion(group, knn, other, min_distance, max_distance, cos_max_angle, weight,
                     do_not_apply_with=0) -> None:
    call("gs_steer_for_cohesion", group.handle, knn.handle, other.handle, min_distance,
         max_distance, cos_max_angle, weight, int(do_not_apply_with))


def steerForSeek(group, target, weight, do_not_apply_with=0) -> None:
    call("gs_steer_for_seek", group.handle, _f3(target), weight, int(do_not_apply_with))


def steerToAvoidNeighbors(group, knn, other, min_time_to_collision, min_separation_distance,
                          avoid_close_neighbors, weight, do_not_apply_with=0) -> None:
    call("gs_steer_to_avoid_neighbors", group.handle, knn.handle, other.handle,
         min_time_to_collision, min_separation_distance, int(bool(avoid_close_neighbors)),
         weight, int(do_not_apply_with))


def steerToAvoidWalls(group, knw, walls, min_time_to_collision, weight,
                      do_not_apply_with=0) -> None:
    call("gs_steer_to_avoid_walls", group.handle, knw.handle, walls.handle,
         min_time_to_collision, weight, int(do_not_apply_with))


def updateGroup(group, elapsed_time) -> None:
    call("gs_update_group", group.handle, elapsed_time)


def antiPenetrationAgents(group, knn, other, do_not_apply_with=0) -> None:
    call("gs_anti_penetration_agents", group.handle, knn.handle, other.handle,
         int(do_not_apply_with))


def updateGroupWithAntiPenetration(group, knw, walls, elapsed_time) -> None:
    """updateGroupWithAntiPenetration (UpdateCUDAKernelNew.cu:95-268); reads
    the wall list row-major, as the reference kernel does."""
    call("gs_update_group_with_antipenetration", group.handle, knw.handle, walls.handle,
         elapsed_time)


def antiPenetrationWall(group, knw, walls, elapsed_time, do_not_apply_with=0) -> None:
    """antiPenetrationWall (AntiPenetrationWallCUDAKernel.cu:52-134); reads the
    wall list row-major and ignores do_not_apply_with, as the reference does."""
    call("gs_anti_penetration_wall", group.handle, knw.handle, walls.handle, elapsed_time,
         int(do_not_apply_with))


def cell_density(group: AgentGroup, bins: KNNBinData) -> np.ndarray:
    """ComputeCellDensity (ProcessData.cu:74-101): agents per cell of the
    group's database (updateKNNDatabase first)."""
    n = C.c_uint()
    call("gs_bins_num_cells", bins.handle, C.byref(n))
    out = np.zeros(n.value, np.uint32)
    call("gs_cell_density", group.handle, bins.handle, _ptr(out, C.c_uint))
    return out


def cell_avg_velocity(group: AgentGroup, bins: KNNBinData) -> np.ndarray:
    """ComputeAvgCellVelocity (ProcessData.cu:103-134): mean velocity per cell."""
    n = C.c_uint()
    call("gs_bins_num_cells", bins.handle, C.byref(n))
    out = np.zeros((n.value, 3), np.float32)
    call("gs_cell_avg_velocity", group.handle, bins.handle, _ptr(out))
    return out


def steerToFollowPath(group, path: Path, prediction_time, weight, do_not_apply_with=0) -> None:
    call("gs_steer_to_follow_path", group.handle, path.handle, prediction_time, weight,
         int(do_not_apply_with))


def step(group: AgentGroup, bins: KNNBinData, walls: WallGroup | None, params: StepParams,
         steps: int = 1, path: Path | None = None) -> None:
    """The fused whole step, `steps` times (path: for GS_B_FOLLOW_PATH)."""
    p = step_params_c(params, path)
    call("gs_step", group.handle, bins.handle, walls.handle if walls else None, C.byref(p),
         int(steps))


def step_host(group: AgentGroup, bins: KNNBinData, walls, params: StepParams, steps: int,
              state_in: AgentState, state_out: AgentState, path: Path | None = None) -> None:
    """Upload from host arrays, `steps` fused steps, download into state_out."""
    p = step_params_c(params, path)
    a_in, a_out = host_arrays(state_in), host_arrays(state_out)
    call("gs_step_host", group.handle, bins.handle, walls.handle if walls else None, C.byref(p),
         int(steps), C.byref(a_in), state_in.n, C.byref(a_out))
