"""Host-side agent state in the reference's structure-of-arrays layout.

Mirrors ``agent_group_data`` (include/OpenSteer/AgentGroupData.cuh:19-60): float4
position, direction and steering (w = 0), float3 side and up, and per-agent
speed, maxSpeed, maxForce, radius, mass and the appliedKernels bit mask.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

FIELDS_F4 = ("position", "direction", "steering")
FIELDS_F3 = ("side", "up")
FIELDS_F1 = ("speed", "max_speed", "max_force", "radius", "mass")

# Kernel bit masks, include/OpenSteer/CUDA/CUDAKernelGlobals.cuh:12-31.
KERNEL_PURSUE_BIT = 1 << 0
KERNEL_EVADE_BIT = 1 << 1
KERNEL_SEEK_BIT = 1 << 2
KERNEL_FLEE_BIT = 1 << 3
KERNEL_SEPARATION_BIT = 1 << 4
KERNEL_ALIGNMENT_BIT = 1 << 5
KERNEL_COHESION_BIT = 1 << 6
KERNEL_AVOID_OBSTACLES_BIT = 1 << 7
KERNEL_AVOID_WALLS_BIT = 1 << 8
KERNEL_AVOID_NEIGHBORS_BIT = 1 << 9
KERNEL_AVOID_CLOSE_NEIGHBORS_BIT = 1 << 10
KERNEL_FOLLOW_PATH_BIT = 1 << 11
KERNEL_ANTI_PENETRATION_WALL = 1 << 12
KERNEL_ANTI_PENETRATION_AGENT = 1 << 13


@dataclass
class AgentState:
    """One group's agents; every array is C-contiguous and owned."""

    position: np.ndarray
    direction: np.ndarray
    steering: np.ndarray
    side: np.ndarray
    up: np.ndarray
    speed: np.ndarray
    max_speed: np.ndarray
    max_force: np.ndarray
    radius: np.ndarray
    mass: np.ndarray
    applied: np.ndarray
    extra: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.speed.shape[0])

    @classmethod
    def zeros(cls, n: int, dtype=np.float32) -> "AgentState":
        return cls(
            position=np.zeros((n, 4), dtype),
            direction=np.zeros((n, 4), dtype),
            steering=np.zeros((n, 4), dtype),
            side=np.zeros((n, 3), dtype),
            up=np.zeros((n, 3), dtype),
            speed=np.zeros(n, dtype),
            max_speed=np.zeros(n, dtype),
            max_force=np.zeros(n, dtype),
            radius=np.zeros(n, dtype),
            mass=np.zeros(n, dtype),
            applied=np.zeros(n, np.uint32),
        )

    def copy(self) -> "AgentState":
        return AgentState(**{k: np.array(getattr(self, k), copy=True) for k in self.names()})

    def astype(self, dtype) -> "AgentState":
        out = {k: np.ascontiguousarray(getattr(self, k), dtype=dtype) for k in self.float_names()}
        out["applied"] = self.applied.copy()
        return AgentState(**out)

    @staticmethod
    def float_names():
        return FIELDS_F4 + FIELDS_F3 + FIELDS_F1

    @classmethod
    def names(cls):
        return cls.float_names() + ("applied",)

    def arrays(self) -> dict:
        return {k: getattr(self, k) for k in self.names()}

    def subset(self, idx) -> "AgentState":
        return AgentState(**{k: np.ascontiguousarray(getattr(self, k)[idx]) for k in self.names()})

    @classmethod
    def concat(cls, states) -> "AgentState":
        return cls(**{k: np.ascontiguousarray(np.concatenate([getattr(s, k) for s in states]))
                      for k in cls.names()})
