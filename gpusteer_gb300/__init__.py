"""GB300-native (sm_103a) implementation of GPUSteer's per-step agent update.

The compute runs in libgpusteer.so (CUDA kernels behind the C ABI declared in
include/gpusteer.h); this package is the host-side mirror of the reference's
group API (AgentGroup, KNNData, KNNBinData, WallGroup and the
GroupSteerLibrary free functions), seeded scenarios and the build step.
"""
from ._lib import GpuSteerError, load  # noqa: F401
from .groups import (  # noqa: F401
    AgentGroup, Batch, KNNBinData, KNNData, Path, Rollout, WallGroup, antiPenetrationAgents,
    batches_step_host, bruteforce_pairs, pinned_state, MultiGroupParams, multigroup_step,
    antiPenetrationWall, updateGroupWithAntiPenetration,
    findKNearestNeighbors, findKNearestNeighborsBruteForce, findKNearestNeighborsGroups,
    set_barrier_limit, set_block, set_graphs, set_persistent,
    knn_capacity, set_knn_capacity, step, step_host, step_launches, steerForAlignment,
    steerForCohesion,
    steerForSeek, steerForSeparation, steerToAvoidNeighbors, steerToAvoidWalls, steerToFollowPath,
    updateGroup,
    updateKNNDatabase, wrapWorld)
from .scenario import StepParams  # noqa: F401
from .state import AgentState  # noqa: F401
