"""CPU checks of the FP64 frozen-structure rollout that the adjoint's GPU
tests use as their reference: its forward pass follows the FP32 oracle's
trajectory, and its autograd gradient agrees with its own finite
differences."""
import numpy as np
import pytest
import torch

import adjoint_harness as ah
from gpusteer_gb300 import scenario as sc


def small_case(steps=24):
    s = sc.boids_cube(2000, size=50.0, seed=4)
    p = sc.boids_params(k=16, world=128.0, cell=4.0)
    structure, final32 = ah.frozen_structure(s, p, steps)
    return s, p, ah.to_torch(structure), final32


def test_frozen_rollout_follows_the_fp32_oracle():
    s, p, st, final32 = small_case()
    P0, V0, consts = ah.initial64(s)
    w = torch.tensor(ah.weights_of(p))
    P, _ = ah.rollout64(P0, V0, consts, st, w, p)
    err = np.abs(P.numpy() - final32.position[:, :3].astype(np.float64)).max()
    assert err < 1e-3, err


def test_frozen_rollout_autograd_matches_its_finite_differences():
    s, p, st, _ = small_case(steps=12)
    P0, V0, consts = ah.initial64(s)
    target = P0 + 0.1
    w = torch.tensor(ah.weights_of(p) * np.array([0.9, 0.95, 1.1]), requires_grad=True)

    def loss(wt):
        P, _ = ah.rollout64(P0, V0, consts, st, wt, p)
        return ((P - target) ** 2).mean()

    loss(w).backward()
    h = 1e-5
    for b in range(3):
        e = torch.zeros(3, dtype=torch.float64)
        e[b] = h
        with torch.no_grad():
            fd = (loss(w.detach() + e) - loss(w.detach() - e)) / (2 * h)
        assert float(w.grad[b]) == pytest.approx(float(fd), rel=1e-6, abs=1e-12)


def test_frozen_structure_refuses_agents_at_the_edge():
    s = sc.boids_cube(500, size=200.0, seed=1)
    p = sc.boids_params(k=8, world=200.0, cell=4.0)
    s.position[0, 0] = 100.0
    with pytest.raises(ValueError):
        ah.frozen_structure(s, p, 1)
