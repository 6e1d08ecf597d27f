"""The hand-written adjoint of the fused flocking step (gs_rollout_*,
gs_flock_adjoint_step) against the FP64 frozen-structure rollout on the CPU:
its autograd gradient (reference gradient) and central finite differences
(h = 1e-3).  Tolerance: 1e-3 relative."""
import numpy as np
import pytest
import torch

import adjoint_harness as ah
import gpusteer_gb300 as gs
from gpusteer_gb300 import scenario as sc

pytestmark = pytest.mark.gpu

W_TRUE = np.array([5.0, 8.0, 4.0])   # separation, alignment, cohesion
W_EVAL = np.array([4.5, 7.5, 4.5])


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def case(n, size, world, steps, seed):
    s = sc.boids_cube(n, size=size, seed=seed)
    p = sc.boids_params(k=16, world=world, cell=4.0)
    return s, p


def gpu_loss_grads(s, p, steps, every, target, want_p0=False):
    r = ah.Runner(s, p, steps, every)
    final = r.forward(None, W_EVAL)
    n = s.n
    g_final = torch.from_numpy(2.0 * (final - target) / (3 * n))
    gv, gp, gw = r.backward(g_final, want_p0=want_p0)
    loss = float(((final.astype(np.float64) - target) ** 2).mean())
    return loss, gv.numpy(), (gp.numpy() if gp is not None else None), gw.numpy(), final


def target_positions(s, p, steps):
    r = ah.Runner(s, p, steps, 8)
    return r.forward(None, W_TRUE).astype(np.float64)


def test_rollout_forward_equals_plain_fused_steps():
    s, p = case(4096, 60.0, 128.0, 24, seed=2)
    r = ah.Runner(s, p, 24, 8)
    r.forward(None, ah.weights_of(p))
    got = r.group.download()
    bins = gs.KNNBinData(p.world_cells, p.world_size, 1)
    g = gs.AgentGroup(p.k, s.n)
    s0 = s.copy()
    s0.steering[:] = 0
    s0.applied[:] = 0
    g.upload(s0)
    gs.step(g, bins, None, p, 24)
    want = g.download()
    for k in ("position", "direction", "speed", "side", "up"):
        np.testing.assert_array_equal(getattr(got, k), getattr(want, k), err_msg=k)


def reference_gradients(s, p, steps, target, forced: bool):
    """FP64 autograd through the frozen rollout: along the FP32 trajectory
    (forced) or free-running."""
    pe = ah.with_weights(p, W_EVAL)
    states = [] if forced else None
    structure, final32 = ah.frozen_structure(s, pe, steps, states_out=states)
    st = ah.to_torch(structure)
    P0, V0, consts = ah.initial64(s)
    P0 = P0.clone().requires_grad_(True)
    V0 = V0.clone().requires_grad_(True)
    w = torch.tensor(W_EVAL, requires_grad=True)
    P, _ = ah.rollout64(P0, V0, consts, st, w, pe, forced=states)
    # seed: d loss / d final position at the FP32 final positions (as on the GPU)
    fin = final32.position[:, :3].astype(np.float64)
    g = torch.from_numpy(2.0 * (fin - target) / (3 * s.n))
    (P * g).sum().backward()
    return w.grad.numpy(), V0.grad.numpy(), P0.grad.numpy()


def test_adjoint_matches_fp64_reference_gradient():
    """4,096 boids, 24 steps, checkpoints every 8: the GPU adjoint against
    FP64 autograd through the same frozen rollout, linearised along the same
    (FP32) trajectory, for the weights, initial velocities and positions."""
    steps = 24
    s, p = case(4096, 60.0, 128.0, steps, seed=2)
    target = target_positions(s, p, steps)
    _, gv, gp, gw, _ = gpu_loss_grads(s, p, steps, 8, target, want_p0=True)
    rw, rv, rp = reference_gradients(s, p, steps, target, forced=True)
    assert rel_err(gw, rw) < 1e-3, (gw, rw)
    assert rel_err(gv, rv) < 1e-3
    assert rel_err(gp, rp) < 1e-3
    # the free-running FP64 rollout stays close on this horizon
    fw, _, _ = reference_gradients(s, p, steps, target, forced=False)
    assert rel_err(gw, fw) < 1e-3, (gw, fw)


def test_adjoint_65536_boids_64_steps_matches_linearisation():
    """The fitting configuration: 65,536 boids, k = 16, 64 steps,
    checkpoints every 8.  Over 64 steps this flock is chaotic (headings of
    agents whose speed passes near zero, and of well-aligned agents, are
    near-singular), so the derivative is taken along the FP32 trajectory the
    GPU ran and compared with FP64 autograd along that same trajectory."""
    steps = 64
    s, p = case(65536, 200.0, 256.0, steps, seed=0)
    target = target_positions(s, p, steps)
    _, gv, _, gw, _ = gpu_loss_grads(s, p, steps, 8, target)
    rw, rv, _ = reference_gradients(s, p, steps, target, forced=True)
    assert rel_err(gw, rw) < 1e-3, (gw, rw)
    assert rel_err(gv, rv) < 1e-3


def test_adjoint_matches_finite_differences_65536_boids():
    """65,536 boids, k = 16, checkpoints every 8, over the 32-step horizon on
    which this flock (initial speeds in [4.5, 9]) is well conditioned:
    central differences with h = 1e-3 of the FP64 frozen rollout for the
    three weights and for the initial velocities along a random direction."""
    steps = 32
    s, p = case(65536, 200.0, 256.0, steps, seed=0)
    s.speed[:] = np.float32(4.5) + s.speed * np.float32(0.5)
    target = target_positions(s, p, steps)
    _, gv, _, gw, _ = gpu_loss_grads(s, p, steps, 8, target)
    pe = ah.with_weights(p, W_EVAL)
    structure, _ = ah.frozen_structure(s, pe, steps)
    st = ah.to_torch(structure)
    P0, V0, consts = ah.initial64(s)
    tgt = torch.from_numpy(target)

    def loss(w, V):
        with torch.no_grad():
            P, _ = ah.rollout64(P0, V, consts, st, torch.tensor(w), pe)
            return float(((P - tgt) ** 2).mean())

    h = 1e-3
    fd = np.zeros(3)
    for b in range(3):
        e = np.zeros(3)
        e[b] = h
        fd[b] = (loss(W_EVAL + e, V0) - loss(W_EVAL - e, V0)) / (2 * h)
    for b in range(3):
        assert gw[b] == pytest.approx(fd[b], rel=1e-3), (b, gw, fd)
    rng = np.random.default_rng(0)
    dirn = torch.from_numpy(rng.standard_normal((s.n, 3)))
    dirn /= torch.linalg.norm(dirn)
    fd_v = (loss(W_EVAL, V0 + h * dirn) - loss(W_EVAL, V0 - h * dirn)) / (2 * h)
    ad_v = float((torch.from_numpy(gv.astype(np.float64)) * dirn).sum())
    assert ad_v == pytest.approx(fd_v, rel=1e-3), (ad_v, fd_v)


def test_checkpoint_interval_does_not_change_gradients():
    """The recomputed segments equal the forward pass bit for bit and the
    adjoint sums in a fixed order, so every checkpoint interval gives the same
    gradients exactly."""
    steps = 16
    s, p = case(4096, 60.0, 128.0, steps, seed=5)
    target = target_positions(s, p, steps)
    base = None
    for every in (1, 5, 8, 16):
        _, gv, _, gw, _ = gpu_loss_grads(s, p, steps, every, target)
        if base is None:
            base = (gv, gw)
            continue
        np.testing.assert_array_equal(gw, base[1])
        np.testing.assert_array_equal(gv, base[0])


def test_backward_passes_are_bit_identical():
    """No float atomics in the adjoint: the neighbour terms of each agent are
    gathered through the reverse-KNN index and added in ascending edge order,
    so two backward passes of one rollout (65,536 boids, k = 16, 24 steps,
    checkpoints every 8) give the same gradients bit for bit."""
    steps = 24
    s = sc.boids_cube(65536, size=200.0, seed=0)
    p = sc.boids_params(k=16, world=256.0, cell=4.0)
    r = ah.Runner(s, p, steps, 8)
    final = r.forward(None, W_EVAL)
    g_final = torch.from_numpy(2.0 * (final - 0.5 * final) / (3 * s.n))
    first = [None if t is None else t.numpy().copy() for t in r.backward(g_final, want_p0=True)]
    second = [None if t is None else t.numpy().copy() for t in r.backward(g_final, want_p0=True)]
    for a, b in zip(first, second):
        np.testing.assert_array_equal(a, b)


def test_adjoint_step_entry_point_matches_rollout():
    """gs_flock_adjoint_step over one recorded step equals a 1-step rollout."""
    s, p = case(3000, 50.0, 128.0, 1, seed=7)
    target = target_positions(s, p, 1)
    _, gv_r, gp_r, gw_r, _ = gpu_loss_grads(s, p, 1, 1, target, want_p0=True)
    # record the step's inputs on the CPU: the (wrap-free) initial state and
    # the oracle's KNN lists, which equal the GPU's
    pe = ah.with_weights(p, W_EVAL)
    structure, _ = ah.frozen_structure(s, pe, 1)
    nb = structure[0][0]
    knn = np.where(nb >= 0, nb, 0xFFFFFFFF).astype(np.uint32)
    dev = torch.device("cuda")
    n = s.n
    ps = np.zeros((n, 4), np.float32)
    ps[:, :3] = s.position[:, :3]
    ps[:, 3] = s.speed
    hd = np.zeros((n, 4), np.float32)
    hd[:, :3] = s.direction[:, :3]
    final = ah.Runner(s, p, 1, 1).forward(None, W_EVAL).astype(np.float64)
    seed = np.zeros((n, 4), np.float32)
    seed[:, :3] = 2.0 * (final - target) / (3 * n)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    t_ps, t_hd, t_knn = T(ps), T(hd), T(knn.view(np.int32))
    t_ms, t_mf, t_m = T(s.max_speed), T(s.max_force), T(s.mass)
    lp_out, lv_out = T(seed), torch.zeros(n, 4, device=dev)
    lp_in, lv_in = torch.zeros(n, 4, device=dev), torch.zeros(n, 4, device=dev)
    nb_blocks = (n + 255) // 256
    wpart = torch.zeros(nb_blocks * 4, device=dev)
    torch.cuda.synchronize()
    from gpusteer_gb300._lib import call
    from gpusteer_gb300.groups import step_params_c
    import ctypes as C
    cp = step_params_c(pe)
    vp = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    call("gs_flock_adjoint_step", vp(t_ps), vp(t_hd), vp(t_knn), n, p.k, vp(t_ms), vp(t_mf),
         vp(t_m), C.byref(cp), vp(lp_out), vp(lv_out), vp(lp_in), vp(lv_in), vp(wpart),
         nb_blocks * 4, None)
    torch.cuda.synchronize()
    gw = wpart.view(-1, 4)[:, :3].double().sum(0).cpu().numpy()
    assert rel_err(gw, gw_r) < 1e-5
    # the same kernels on the same inputs, summed in the same fixed order
    np.testing.assert_array_equal(lv_in[:, :3].cpu().numpy(), gv_r)
    np.testing.assert_array_equal(lp_in[:, :3].cpu().numpy(), gp_r)
    assert float(lp_out.abs().max()) == 0.0


def test_fit_recovers_steering_weights():
    """Fits (w_sep, w_ali, w_coh) to a trajectory the method generated at
    (5, 8, 4), starting from (4, 7, 3), through the autograd function."""
    steps = 32
    s, p = case(16384, 120.0, 256.0, steps, seed=3)
    target = torch.from_numpy(target_positions(s, p, steps)).float()
    r = ah.Runner(s, p, steps, 8)
    v0 = torch.from_numpy((s.direction[:, :3] * s.speed[:, None]).astype(np.float32))
    w = torch.tensor([4.0, 7.0, 3.0], dtype=torch.float32, requires_grad=True)
    opt = torch.optim.Adam([w], lr=0.1)
    sched = torch.optim.lr_scheduler.ExponentialLR(opt, gamma=0.95)
    first = None
    for it in range(80):
        opt.zero_grad()
        final = ah.GpuRollout.apply(v0, w, r)
        loss = ((final - target) ** 2).mean()
        loss.backward()
        opt.step()
        sched.step()
        if first is None:
            first = float(loss.detach())
    final = ah.GpuRollout.apply(v0, w.detach(), r)
    last = float(((final - target) ** 2).mean())
    assert last < 1e-2 * first, (first, last, w)
    assert np.abs(w.detach().numpy() - W_TRUE).max() < 0.1, w
