"""Test and fitting harness for differentiable rollouts.

* GpuRollout: a torch.autograd.Function around gs_rollout_* (forward: the
  fused steps on the GPU; backward: the hand-written adjoint kernel).
* frozen_structure / rollout64: an FP64 restatement on the CPU of the same
  rollout with the KNN lists and neighbourhood memberships frozen (taken from
  the FP32 oracle, which is bit-identical to the GPU forward pass), written
  with torch float64 so that autograd gives a reference gradient and plain
  evaluation gives finite differences.

The flock is the reference's (SteerForSeparation/Alignment/CohesionCUDAKernel.cu,
UpdateCUDAKernel.cu:78-123), with velocity = heading * speed.
"""
from __future__ import annotations

import numpy as np
import torch

import gpusteer_gb300 as gs
import oracle_lib as ol
from gpusteer_gb300 import scenario as sc
from gpusteer_gb300.state import AgentState

UINT_MAX = 0xFFFFFFFF


# ---- frozen structure from the FP32 oracle ---------------------------------------------

def memberships32(pre: AgentState, nb: np.ndarray, p: sc.StepParams):
    """inBoidNeighborhood (FlockingCommon.cuh:4-30) of every listed neighbour
    for separation, alignment, cohesion, with the kernels' FP32 operations in
    their order (no contraction)."""
    f32 = np.float32
    P = pre.position[:, :3].astype(f32)
    D = pre.direction[:, :3].astype(f32)
    valid = nb >= 0
    j = np.where(valid, nb, 0)
    O = (P[j] - P[:, None, :]).astype(f32)
    dsq = O[..., 0] * O[..., 0] + O[..., 1] * O[..., 1] + O[..., 2] * O[..., 2]
    d = np.sqrt(dsq)
    with np.errstate(divide="ignore", invalid="ignore"):
        U = O / d[..., None]
        fwd = D[:, None, 0] * U[..., 0] + D[:, None, 1] * U[..., 1] + D[:, None, 2] * U[..., 2]

    def member(mn, mx, cs):
        mn, mx, cs = f32(mn), f32(mx), f32(cs)
        near = d < mn
        ang = ~near & ~(d > mx)
        with np.errstate(invalid="ignore"):
            return valid & (near | (ang & (fwd > cs)))

    return (member(p.sep_min, p.sep_max, p.sep_cos), member(p.ali_min, p.ali_max, p.ali_cos),
            member(p.coh_min, p.coh_max, p.coh_cos))


def frozen_structure(state: AgentState, p: sc.StepParams, steps: int, states_out=None):
    """Per step: (neighbour indices (n, k) with -1 after the last, and the
    separation / alignment / cohesion membership masks), from the FP32
    oracle run of `steps` steps from `state`; also returns the final state.
    states_out (a list) receives each step's FP32 input (position, velocity)
    as float64 arrays."""
    if p.mask_sep or p.mask_ali or p.mask_coh:
        raise ValueError("the frozen rollout assumes zero behaviour masks")
    s = state.copy()
    s.steering[:] = 0
    s.applied[:] = 0
    half = np.float32(0.5) * np.asarray(p.world_size, np.float32)
    out = []
    for _ in range(steps):
        if np.any(np.abs(s.position[:, :3]) >= half):
            raise ValueError("an agent reached the world's edge: the wrap would move it")
        pre = s.copy()
        if states_out is not None:
            states_out.append((pre.position[:, :3].astype(np.float64),
                               (pre.direction[:, :3] * pre.speed[:, None]).astype(np.float64)))
        idx, _ = ol.run(s, p, 1, want_knn=True)
        nb = idx.reshape(p.k, s.n).T.astype(np.int64)
        nb[nb == UINT_MAX] = -1
        out.append((nb,) + memberships32(pre, nb, p))
    return out, s


def to_torch(structure):
    res = []
    for nb, ms, ma, mc in structure:
        res.append((torch.from_numpy(np.where(nb >= 0, nb, 0)), torch.from_numpy(ms),
                    torch.from_numpy(ma), torch.from_numpy(mc)))
    return res


# ---- FP64 frozen rollout -----------------------------------------------------------------

def _norm(x):
    return torch.sqrt((x * x).sum(-1, keepdim=True))


def _normalize(q):
    n = _norm(q)
    return q / torch.where(n > 0, n, torch.ones_like(n)), (n > 0)


def _trunc(x, limit):
    n2 = (x * x).sum(-1, keepdim=True)
    l2 = limit * limit
    scale = torch.where(n2 > l2, limit / torch.sqrt(torch.where(n2 > 0, n2, torch.ones_like(n2))),
                        torch.ones_like(n2))
    return x * scale


def rollout64(P0, V0, consts, structure_t, w, p: sc.StepParams, forced=None):
    """Final positions and velocities after len(structure_t) frozen steps.
    P0, V0: (n, 3) float64 tensors; consts: dict of (n, 1) float64 tensors
    max_speed, max_force, mass; w: (3,) float64 tensor (separation,
    alignment, cohesion).  forced (optional): each step's (position,
    velocity) input values, substituted for the computed ones while the
    derivative still flows through (the linearisation along that
    trajectory: the FP32 trajectory the GPU's adjoint linearises about)."""
    P, V = P0, V0
    dt = float(p.dt)
    order = [b for b in p.order[:len(p.order)]]
    for t, (nb, ms, ma, mc) in enumerate(structure_t):
        if forced is not None:
            Pf, Vf = forced[t]
            P = torch.from_numpy(Pf) + (P - P.detach())
            V = torch.from_numpy(Vf) + (V - V.detach())
        S = _norm(V)
        D = V / torch.where(S > 0, S, torch.ones_like(S))
        Pj = P[nb]
        O = Pj - P[:, None, :]
        F = {}
        # separation: mean of -o / |o|^2
        oo = (O * O).sum(-1)
        T = -O / torch.where(ms, oo, torch.ones_like(oo))[..., None]
        ns = ms.sum(1, keepdim=True)
        mean = torch.where(ms[..., None], T, torch.zeros_like(T)).sum(1) / ns.clamp(min=1)
        F[sc.B_SEPARATION] = torch.where(ns > 0, _normalize(mean)[0], torch.zeros_like(mean))
        # alignment: mean heading minus own heading
        Dj = D[nb]
        na = ma.sum(1, keepdim=True)
        mean = torch.where(ma[..., None], Dj, torch.zeros_like(Dj)).sum(1) / na.clamp(min=1)
        F[sc.B_ALIGNMENT] = torch.where(na > 0, _normalize(mean - D)[0], torch.zeros_like(mean))
        # cohesion: mean position minus own position
        nc = mc.sum(1, keepdim=True)
        mean = torch.where(mc[..., None], Pj, torch.zeros_like(Pj)).sum(1) / nc.clamp(min=1)
        F[sc.B_COHESION] = torch.where(nc > 0, _normalize(mean - P)[0], torch.zeros_like(mean))
        wb = {sc.B_SEPARATION: w[0], sc.B_ALIGNMENT: w[1], sc.B_COHESION: w[2]}
        steer = torch.zeros_like(P)
        for b in order:
            steer = steer + wb[b] * F[b]
        acc = _trunc(steer, consts["max_force"]) / consts["mass"]
        V = _trunc(V + acc * dt, consts["max_speed"])
        P = P + V * dt
    return P, V


def initial64(state: AgentState):
    P0 = torch.from_numpy(state.position[:, :3].astype(np.float64))
    V0 = torch.from_numpy((state.direction[:, :3] * state.speed[:, None]).astype(np.float64))
    consts = {k: torch.from_numpy(getattr(state, k).astype(np.float64)[:, None])
              for k in ("max_speed", "max_force", "mass")}
    return P0, V0, consts


def weights_of(p: sc.StepParams):
    return np.array([p.w_sep, p.w_ali, p.w_coh], np.float64)


def with_weights(p: sc.StepParams, w) -> sc.StepParams:
    return p.replace(w_sep=float(w[0]), w_ali=float(w[1]), w_coh=float(w[2]))


def with_velocity(state: AgentState, v: np.ndarray) -> AgentState:
    """state with heading v / |v| and speed |v| (float32)."""
    s = state.copy()
    v = v.astype(np.float32)
    speed = np.sqrt((v * v).sum(1)).astype(np.float32)
    s.direction[:, :3] = v / np.where(speed > 0, speed, np.float32(1))[:, None]
    s.speed[:] = speed
    return s


# ---- GPU rollout as an autograd function ---------------------------------------------------

class Runner:
    """A group, bins and rollout for one base state and parameter set."""

    def __init__(self, state: AgentState, p: sc.StepParams, steps: int, every: int = 8):
        self.base = state.copy()
        self.p = p
        self.bins = gs.KNNBinData(p.world_cells, p.world_size, p.search_radius)
        self.group = gs.AgentGroup(p.k, state.n)
        self.rollout = gs.Rollout(self.group, self.bins, steps, every)
        self.n = state.n

    def forward(self, v0: np.ndarray | None, w) -> np.ndarray:
        s = self.base if v0 is None else with_velocity(self.base, v0)
        self.group.upload(s)
        self.rollout.forward(with_weights(self.p, w))
        return self.group.download().position[:, :3].copy()

    def backward(self, g_final: torch.Tensor, want_p0: bool = False):
        """g_final: (n, 3) d loss / d final position.  Returns (d loss / d v0,
        d loss / d p0 or None, d loss / d w) as float32 CPU tensors."""
        dev = torch.device("cuda")
        seed = torch.zeros(self.n, 4, dtype=torch.float32, device=dev)
        seed[:, :3] = g_final.to(dev, torch.float32)
        gv = torch.zeros(self.n, 4, dtype=torch.float32, device=dev)
        gp = torch.zeros(self.n, 4, dtype=torch.float32, device=dev) if want_p0 else None
        torch.cuda.synchronize()
        gw = self.rollout.backward(seed.data_ptr(), None, gp.data_ptr() if want_p0 else None,
                                   gv.data_ptr())
        return (gv[:, :3].cpu(), gp[:, :3].cpu() if want_p0 else None, torch.from_numpy(gw))


class GpuRollout(torch.autograd.Function):
    """final positions = rollout(initial velocities v0, weights w) on the GPU."""

    @staticmethod
    def forward(ctx, v0: torch.Tensor, w: torch.Tensor, runner: Runner):
        ctx.runner = runner
        ctx.v_like = (v0.device, v0.dtype)
        ctx.w_like = (w.device, w.dtype)
        final = runner.forward(v0.detach().cpu().numpy(), w.detach().cpu().numpy())
        return torch.from_numpy(final).to(v0.device, v0.dtype)

    @staticmethod
    def backward(ctx, g_final):
        gv, _, gw = ctx.runner.backward(g_final)
        return gv.to(*ctx.v_like), gw.to(*ctx.w_like), None
