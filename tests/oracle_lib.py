"""ctypes bindings for the CPU oracle (oracle/) and, when it has been built,
the reference harness (oracle/_ref/libgsref.so).  Test infrastructure: only
tests, __graft_entry__.smoke() and bench.py's CPU legs import this module."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from gpusteer_gb300.scenario import StepParams
from gpusteer_gb300.state import AgentState

REPO = Path(__file__).resolve().parents[1]
ORACLE_SO = REPO / "oracle" / "_build" / "liboracle.so"
REF_SO = REPO / "oracle" / "_ref" / "libgsref.so"


def reference_root() -> Path:
    """The reference source tree: $GPUSTEER_REFERENCE, else the default of the
    recipe that compiles it (oracle/ref/Makefile).  It may not exist."""
    env = os.environ.get("GPUSTEER_REFERENCE")
    if env:
        return Path(env)
    out = subprocess.run(["make", "-s", "--no-print-directory", "-C",
                          str(REPO / "oracle" / "ref"), "print-ref"],
                         capture_output=True, text=True)
    return Path(out.stdout.strip() or "/nonexistent")

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_up = C.POINTER(C.c_uint)


def ptr(a: np.ndarray, t=C.c_float):
    assert a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(t))


class OrcGroup(C.Structure):
    _fields_ = [(k, _fp) for k in ("position", "direction", "steering", "side", "up", "speed",
                                   "max_speed", "max_force", "radius", "mass")] + [
        ("applied", _up), ("n", C.c_uint)]


class OrcGroupD(C.Structure):
    _fields_ = [(k, _dp) for k in ("position", "direction", "steering", "side", "up", "speed",
                                   "max_speed", "max_force", "radius", "mass")] + [
        ("applied", _up), ("n", C.c_uint)]


class OrcWalls(C.Structure):
    _fields_ = [("start", _fp), ("mid", _fp), ("end", _fp), ("normal", _fp), ("n", C.c_uint)]


class OrcStepParams(C.Structure):
    _fields_ = [
        ("world_size", C.c_float * 3), ("world_cells", C.c_uint * 3), ("search_radius", C.c_uint),
        ("wrap_mode", C.c_int), ("knn_mode", C.c_int), ("k", C.c_uint), ("clear_applied", C.c_int),
        ("knw", C.c_uint), ("min_time_to_wall", C.c_float), ("w_walls", C.c_float),
        ("mask_walls", C.c_uint),
        ("min_time_to_collision", C.c_float), ("min_separation_distance", C.c_float),
        ("avoid_close", C.c_int), ("w_avoid", C.c_float), ("mask_avoid", C.c_uint),
        ("sep_min", C.c_float), ("sep_max", C.c_float), ("sep_cos", C.c_float),
        ("w_sep", C.c_float), ("mask_sep", C.c_uint),
        ("ali_min", C.c_float), ("ali_max", C.c_float), ("ali_cos", C.c_float),
        ("w_ali", C.c_float), ("mask_ali", C.c_uint),
        ("coh_min", C.c_float), ("coh_max", C.c_float), ("coh_cos", C.c_float),
        ("w_coh", C.c_float), ("mask_coh", C.c_uint),
        ("seek_target", C.c_float * 3), ("w_seek", C.c_float), ("mask_seek", C.c_uint),
        ("order", C.c_uint * 8), ("n_order", C.c_uint), ("dt", C.c_float),
        ("path", C.c_void_p), ("path_prediction_time", C.c_float), ("w_path", C.c_float),
        ("mask_path", C.c_uint),
    ]


class OrcPath(C.Structure):
    _fields_ = [("points", _fp), ("lengths", _fp), ("normals", _fp), ("n", C.c_uint),
                ("radius", C.c_float), ("cyclic", C.c_int), ("total_length", C.c_float)]


def path_init(points, radius, cyclic):
    """PolylinePathwayCUDA::Initialize through the oracle: an OrcPath (with its
    arrays kept alive on it) for float32 points (m, 3)."""
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    m = pts.shape[0]
    po = np.zeros((m + 1, 3), np.float32)
    ln = np.zeros(m + 1, np.float32)
    nm = np.zeros((m + 1, 3), np.float32)
    tot = C.c_float()
    n = oracle().orc_path_init(ptr(pts), m, int(bool(cyclic)), ptr(po), ptr(ln), ptr(nm),
                               C.byref(tot))
    P = OrcPath()
    P.points, P.lengths, P.normals = ptr(po), ptr(ln), ptr(nm)
    P.n, P.radius, P.cyclic, P.total_length = n, float(radius), int(bool(cyclic)), tot.value
    P._keep = (po, ln, nm)
    P.arrays = (po[:n], ln[:n], nm[:n], tot.value)
    return P


def step_params_struct(p: StepParams, path=None) -> OrcStepParams:
    s = OrcStepParams()
    for name, _ in OrcStepParams._fields_:
        if name in ("order", "n_order", "path"):
            continue
        v = getattr(p, name)
        if isinstance(v, (tuple, list)):
            arr = getattr(s, name)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(s, name, v)
    for i, b in enumerate(p.order):
        s.order[i] = b
    s.n_order = len(p.order)
    if path is not None:
        s.path = C.cast(C.pointer(path), C.c_void_p)
        s._keep_path = path
    return s


def build_oracle() -> None:
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle")], check=True)


_oracle = None


def oracle():
    global _oracle
    if _oracle is None:
        build_oracle()
        lib = C.CDLL(str(ORACLE_SO))
        lib.orc_knn_binned.restype = C.c_int
        lib.orc_knn_bruteforce.restype = C.c_int
        lib.orc_run.restype = C.c_int
        lib.orc_run_d.restype = C.c_int
        lib.orc_walls_load.restype = C.c_int
        lib.orc_walls_split.restype = C.c_int
        lib.orc_max_threads.restype = C.c_int
        _oracle = lib
    return _oracle


def ref_harness():
    """The reference's own kernels on the CPU, or None when not built here."""
    if not REF_SO.exists():
        return None
    return C.CDLL(str(REF_SO))


def group_struct(s: AgentState) -> OrcGroup:
    g = OrcGroup()
    for k in AgentState.float_names():
        a = getattr(s, k)
        assert a.dtype == np.float32 and a.flags.c_contiguous, k
        setattr(g, k, ptr(a))
    g.applied = ptr(s.applied, C.c_uint)
    g.n = s.n
    g._keep = s
    return g


def group_struct_d(s: AgentState) -> OrcGroupD:
    g = OrcGroupD()
    for k in AgentState.float_names():
        a = getattr(s, k)
        assert a.dtype == np.float64 and a.flags.c_contiguous, k
        setattr(g, k, ptr(a, C.c_double))
    g.applied = ptr(s.applied, C.c_uint)
    g.n = s.n
    g._keep = s
    return g


def walls_struct(start, mid, end, normal) -> OrcWalls:
    w = OrcWalls()
    w.start, w.mid, w.end, w.normal = ptr(start), ptr(mid), ptr(end), ptr(normal)
    w.n = start.shape[0]
    w._keep = (start, mid, end, normal)
    return w


def f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


def u3(v):
    return (C.c_uint * 3)(*[int(x) for x in v])


# ---- convenience wrappers ----------------------------------------------------------

def knn_binned(posA, posB, self_, ws, wc, r, k, threads=0):
    nA, nB = posA.shape[0], posB.shape[0]
    idx = np.empty(k * nA, np.uint32)
    dist = np.empty(k * nA, np.float32)
    rc = oracle().orc_knn_binned(ptr(posA), nA, ptr(posB), nB, int(self_), f3(ws), u3(wc), r, k,
                                 ptr(idx, C.c_uint), ptr(dist), threads)
    assert rc == 0
    return idx, dist


def cell_index(pos, ws, wc):
    out = np.empty(pos.shape[0], np.uint32)
    oracle().orc_cell_index(ptr(pos), pos.shape[0], f3(ws), u3(wc), ptr(out, C.c_uint))
    return out


def cell_density(pos, ws, wc):
    out = np.empty(int(np.prod(wc)), np.uint32)
    oracle().orc_cell_density(ptr(pos), pos.shape[0], f3(ws), u3(wc), ptr(out, C.c_uint))
    return out


def cell_avg_velocity(pos, direction, speed, ws, wc):
    out = np.empty((int(np.prod(wc)), 3), np.float32)
    oracle().orc_cell_avg_velocity(ptr(pos), ptr(direction), ptr(speed), pos.shape[0], f3(ws),
                                   u3(wc), ptr(out))
    return out


def knn_brute(posA, posB, self_, k, threads=0):
    nA, nB = posA.shape[0], posB.shape[0]
    idx = np.empty(k * nA, np.uint32)
    dist = np.empty(k * nA, np.float32)
    rc = oracle().orc_knn_bruteforce(ptr(posA), nA, ptr(posB), nB, int(self_), k,
                                     ptr(idx, C.c_uint), ptr(dist), threads)
    assert rc == 0
    return idx, dist


def run(state: AgentState, p: StepParams, steps: int, walls=None, threads=0, want_knn=False,
        path=None):
    """Advance `state` in place by `steps` oracle steps (path: an OrcPath)."""
    g = group_struct(state)
    w = walls_struct(*walls) if walls is not None else None
    idx = np.empty(p.k * state.n, np.uint32) if want_knn else None
    dist = np.empty(p.k * state.n, np.float32) if want_knn else None
    rc = oracle().orc_run(C.byref(g), C.byref(w) if w is not None else None,
                          C.byref(step_params_struct(p, path)), steps,
                          ptr(idx, C.c_uint) if want_knn else None,
                          ptr(dist) if want_knn else None, threads)
    assert rc == 0, rc
    return (idx, dist) if want_knn else None


def run_d(state64: AgentState, p: StepParams, steps: int, walls=None, threads=0, path=None):
    g = group_struct_d(state64)
    w = walls_struct(*walls) if walls is not None else None
    rc = oracle().orc_run_d(C.byref(g), C.byref(w) if w is not None else None,
                            C.byref(step_params_struct(p, path)), steps, threads)
    assert rc == 0, rc


def split_walls(start, mid, end, normal, ws, wc, cap=1 << 16):
    outs = [np.zeros((cap, 4), np.float32) for _ in range(4)]
    n = oracle().orc_walls_split(ptr(start), ptr(mid), ptr(end), ptr(normal), start.shape[0],
                                 f3(ws), u3(wc), *[ptr(o) for o in outs], cap)
    assert n >= 0
    return tuple(np.ascontiguousarray(o[:n]) for o in outs)


def threads_available() -> int:
    return int(oracle().orc_max_threads())


os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")
