/*
 * gpusteer.h - C ABI of the GB300 (sm_103a) GPUSteer group library.
 *
 * This is the drop-in boundary for PsychoLogicAu/GPUSteer's group steering
 * path.  The reference exposes it as C++ objects and `static` free functions
 * (include/OpenSteer/CUDA/GroupSteerLibrary.cuh:43-223) over AgentGroup,
 * KNNData, KNNBinData and WallGroup; every entry point below names the
 * reference interface it replaces.  Plain pointers and sizes only.
 *
 * Conventions
 *  - Every function returns gs_status; GS_OK is 0.  gs_last_error() gives a
 *    per-thread message for the last failure.  Nothing aborts the process
 *    (the reference's CUDA_SAFE_CALL / cutilCheckMsg do).
 *  - Host arrays use the reference layouts (AgentGroupData.cuh:30-46):
 *    float4 position/direction/steering (w = 0), float3 side/up, float
 *    speed/maxSpeed/maxForce/radius/mass, uint appliedKernels.  KNN results
 *    are column-major idx[a + i*n] (KNNBinningV2Kernel.cu:524-525).
 *  - Each group owns a CUDA stream (or uses the one passed in); calls on a
 *    group are asynchronous on that stream unless they return host data.
 *    Calls on one handle must not be made concurrently from several threads.
 *  - Arithmetic is IEEE binary32 without FMA contraction; KNN ties break by
 *    the lower agent index.
 */
#ifndef GPUSTEER_H
#define GPUSTEER_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int gs_status;
#define GS_OK 0
#define GS_ERR_INVALID_ARG 1
#define GS_ERR_OOM 2
#define GS_ERR_CUDA 3
#define GS_ERR_TIMEOUT 4
#define GS_ERR_NONFINITE 5
#define GS_ERR_STATE 6
#define GS_ERR_UNSUPPORTED 7

typedef struct gs_bins_s* gs_bins;     /* KNNBinDataV2 (KNNBinDataV2.cuh:18-63)        */
typedef struct gs_group_s* gs_group;   /* AgentGroup + KNNDatabase (AgentGroup.h:12-56) */
typedef struct gs_knn_s* gs_knn;       /* KNNData (KNNData.cuh:10-55)                   */
typedef struct gs_walls_s* gs_walls;   /* WallGroup (WallGroup.h:12-37)                 */
typedef struct gs_path_s* gs_path;     /* PolylinePathwayCUDA (PolylinePathwayCUDA.cuh)  */

/* Pointers to one group's arrays (host or device, per the call). */
typedef struct gs_agent_arrays {
    float* position;  /* float4[n] */
    float* direction; /* float4[n] */
    float* steering;  /* float4[n] */
    float* side;      /* float3[n] */
    float* up;        /* float3[n] */
    float* speed;
    float* max_speed;
    float* max_force;
    float* radius;
    float* mass;
    unsigned* applied;
} gs_agent_arrays;

/* Wrap modes of gs_wrap_world and gs_step_params.wrap_mode. */
#define GS_WRAP_REFERENCE 0 /* WrapWorldCUDAKernel.cu:27-43 (z < 0 -> halfZ + 100) */
#define GS_WRAP_SYMMETRIC 1 /* z wrapped like x and y                              */
#define GS_WRAP_NONE 2

/* Behaviour codes of gs_step_params.order. */
#define GS_B_AVOID_WALLS 1
#define GS_B_AVOID_NEIGHBORS 2
#define GS_B_SEPARATION 3
#define GS_B_ALIGNMENT 4
#define GS_B_COHESION 5
#define GS_B_SEEK 6
#define GS_B_FOLLOW_PATH 7 /* needs gs_step_params.path */

#define GS_KNN_BINNED 0
#define GS_KNN_BRUTEFORCE 1

/* One whole step (a plugin's XxxGroup::update, e.g. plugins/BoidsGroup.cpp:606-637,
 * plugins/ChokePointNew.cpp:586-630): wrap, rebuild the bins, KNN (and wall
 * KNN), the behaviours in `order`, then UpdateCUDAKernel. */
typedef struct gs_step_params {
    float world_size[3];
    unsigned world_cells[3];
    unsigned search_radius;
    int wrap_mode;
    int knn_mode;
    unsigned k;
    int clear_applied; /* zero appliedKernels at step start (ChokePointNew.cpp:595) */
    unsigned knw;
    float min_time_to_wall, w_walls;
    unsigned mask_walls;
    float min_time_to_collision, min_separation_distance;
    int avoid_close;
    float w_avoid;
    unsigned mask_avoid;
    float sep_min, sep_max, sep_cos, w_sep;
    unsigned mask_sep;
    float ali_min, ali_max, ali_cos, w_ali;
    unsigned mask_ali;
    float coh_min, coh_max, coh_cos, w_coh;
    unsigned mask_coh;
    float seek_target[3], w_seek;
    unsigned mask_seek;
    unsigned order[8];
    unsigned n_order;
    float dt;
    /* path following (ChokePointNew.cpp:620: pathPredictionTime, weightFollowPath,
     * maskFollowPath); path may be NULL when GS_B_FOLLOW_PATH is not in order */
    gs_path path;
    float path_prediction_time, w_path;
    unsigned mask_path;
} gs_step_params;

/* ---- library -------------------------------------------------------------- */
const char* gs_status_string(gs_status s);
const char* gs_last_error(void);
int gs_version(void);
/* Largest k the KNN kernels accept. */
unsigned gs_max_k(void);
/* Selects the CUDA device for the calling thread (cudaSetDevice); handles are
 * bound to the device that was current when they were created.  The
 * reference picks its device in the plugins (plugins/ChokePointNew.cpp:654-680). */
gs_status gs_set_device(int device);
/* Page-locked host buffers for the per-frame host copies (the reference's
 * SyncDevice / SyncHost use pageable std::vector storage). */
gs_status gs_host_alloc(size_t bytes, void** out);
gs_status gs_host_free(void* p);

/* ---- KNNBinData: KNNBinDataV2::KNNBinDataV2(worldCells, worldSize, searchRadius),
 *      KNNBinDataV2.cu:30-42.  No device neighbour table is built: the
 *      (2r+1)^d neighbour cells are computed arithmetically. */
gs_status gs_bins_create(const unsigned world_cells[3], const float world_size[3],
                         unsigned search_radius, gs_bins* out);
gs_status gs_bins_destroy(gs_bins bins);
gs_status gs_bins_num_cells(gs_bins bins, unsigned* out);
/* KNNBinDataV2::hvCells(): float3 min bound, max bound and centre per cell in
 * bin_cell order (KNNBinDataV2.cu:103-135). */
gs_status gs_bins_get_cells(gs_bins bins, float* min3, float* max3, float* centre3, unsigned cap);

/* ---- AgentGroup ------------------------------------------------------------- */
/* AgentGroup(worldCells, knn) (src/AgentGroup.cpp:8-11).  `k` is the
 * KNNDatabase's k; `capacity` bounds the agent count.  `stream` may be NULL
 * (the group creates its own non-blocking stream). */
gs_status gs_group_create(unsigned k, unsigned capacity, void* stream, gs_group* out);
gs_status gs_group_destroy(gs_group g);
/* Clear + AddAgent* + SyncDevice (src/AgentGroup.cpp:34-55,97-108,128-133):
 * replaces the group's agents with n agents copied from host arrays. */
gs_status gs_group_upload(gs_group g, const gs_agent_arrays* host, unsigned n);
/* SyncHost (AgentGroupData.cuh:177-225): copies the device state to host arrays
 * (any member may be NULL to skip it) and waits for the copy. */
gs_status gs_group_download(gs_group g, const gs_agent_arrays* host);
gs_status gs_group_size(gs_group g, unsigned* n);
/* pdPosition()/pdDirection()/... accessors (AgentGroup.h:51-54,
 * AgentGroupData.cuh:62-110): device pointers in the reference layout. */
gs_status gs_group_device_arrays(gs_group g, gs_agent_arrays* dev);
gs_status gs_group_stream(gs_group g, void** stream);
gs_status gs_group_synchronize(gs_group g);
/* Phase timing of the fused step with CUDA events on the group's stream (the
 * reference's optional TIMING instrumentation, KNNBinningV2.cu:106-161).
 * While enabled, every phase launch is bracketed by events; the totals are
 * read with gs_group_phase_times: ms[i] and launches[i] for phase i =
 * 0 scan, 1 permute, 2 fused step (or its wall half), 3 second half after
 * walls.  Enabling clears the totals. */
#define GS_PHASES 4
gs_status gs_group_set_profiling(gs_group g, int enable);
/* Agents of the last fused step whose neighbour order the fast 32-bit KNN
 * scan could not vouch for (exact distance ties, crowded boxes) and that the
 * exact path redid; waits for the group's stream. */
gs_status gs_group_exact_redos(gs_group g, unsigned* count);
/* One persistent launch per fused step (no counterpart in the reference,
 * which launches one kernel per behaviour): the scan, permute, wall phase,
 * exact lists and rest phase of a step with avoid-walls first,
 * 9 <= k <= 16, a flat world (one cell high) and the streaming KNN scan
 * (capacity 128 or 256) run in one cooperative launch with grid-wide
 * barriers between the phases; the results equal the separate launches bit
 * for bit.  Other steps keep the separate launches.  Off by default. */
gs_status gs_group_set_persistent(gs_group g, int enable);
/* Polls a barrier wait of the persistent step makes before it gives up (0:
 * the default, about a second).  A step whose wait ran out is void: the
 * group must be uploaded again, and gs_group_synchronize (or the next call
 * that returns host data) reports GS_ERR_TIMEOUT. */
gs_status gs_group_set_barrier_limit(gs_group g, unsigned polls);
gs_status gs_group_phase_times(gs_group g, float* ms, unsigned* launches, unsigned cap);

/* ---- KNNData: KNNData(nSize, nK) (KNNData.cu) ---------------------------------- */
gs_status gs_knn_create(unsigned n, unsigned k, gs_knn* out);
gs_status gs_knn_destroy(gs_knn knn);
/* KNNData::syncHost + hvKNNIndices/hvKNNDistances (column-major, k*n). */
gs_status gs_knn_download(gs_knn knn, gs_group g, unsigned* idx, float* dist);
gs_status gs_knn_device_arrays(gs_knn knn, unsigned** idx, float** dist);
/* Writes the lists from the host (column-major, k*n; either array may be
 * NULL): what a caller of the reference does through pdKNNIndices() /
 * pdKNNDistances() (KNNData.cuh:37-38) with a cudaMemcpy. */
gs_status gs_knn_upload(gs_knn knn, gs_group g, const unsigned* idx, const float* dist);

/* ---- WallGroup: WallGroup::LoadFromFile + SplitWalls + SyncDevice
 *      (WallGroupData.cu:73-206, plugins/ChokePointNew.cpp:107-119) ------------- */
/* Segments from host float4 arrays (start, end, normal; mid = (start+end)/2).
 * When `bins` is given the walls are split at its cell boundaries.  `knw` is
 * the wall database's k. */
gs_status gs_walls_create(const float* start4, const float* end4, const float* normal4,
                          unsigned n, gs_bins bins, unsigned knw, gs_walls* out);
/* Reads a .map file: 9 floats per segment. */
gs_status gs_walls_load(const char* path, gs_bins bins, unsigned knw, gs_walls* out);
gs_status gs_walls_destroy(gs_walls w);
gs_status gs_walls_size(gs_walls w, unsigned* n);
gs_status gs_walls_download(gs_walls w, float* start4, float* mid4, float* end4, float* normal4,
                            unsigned cap);

/* ---- GroupSteerLibrary.cuh free functions ----------------------------------------- */
/* wrapWorld (GroupSteerLibrary.cuh:43-50). */
gs_status gs_wrap_world(gs_group g, const float world_size[3], int mode);
/* updateKNNDatabase (GroupSteerLibrary.cuh:129-136): counting-sort rebuild. */
gs_status gs_update_knn_database(gs_group g, gs_bins bins);
gs_status gs_walls_update_knn_database(gs_walls w, gs_bins bins);
/* findKNearestNeighbors (GroupSteerLibrary.cuh:138-157), binned.  `other` may
 * equal `g` (self KNN).  k is the KNNData's k.  Both databases must be
 * current (gs_update_knn_database). */
gs_status gs_find_knn(gs_group g, gs_knn out, gs_bins bins, gs_group other,
                      unsigned search_radius);
/* findKNearestNeighbors against a WallGroup (plugins/ChokePointNew.cpp:600). */
/* findKNearestNeighbors for every group pair of a MultiGroup frame
 * (plugins/MultiGroup.cpp:560-564 calls it once per pair) in one launch:
 * out[i * n_groups + j] (NULL to skip a pair) receives group i's lists against
 * group j.  Every pair reads only the databases of gs_update_knn_database, so
 * the lists equal the per-pair calls' bit for bit, also when the groups are
 * stepped in turn between the calls as MultiGroup does.  At most 7 groups. */
gs_status gs_find_knn_groups(const gs_group* groups, unsigned n_groups, gs_bins bins,
                             gs_knn* out);

/* The values a MultiGroup frame reads from its SimulationParams
 * (plugins/MultiGroup.cpp:545-610; data/MultiGroup*.params). */
typedef struct gs_multigroup_params {
    float    world_size[3];
    int      wrap_mode;                      /* GS_WRAP_*                               */
    float    min_time_to_collision, min_separation_distance;
    int      avoid_close;
    float    w_avoid;
    unsigned mask_avoid;
    float    sep_min, sep_max, sep_cos, w_sep;  /* minSeparationDistance, maxSeparation... */
    unsigned mask_sep;
    float    ali_min, ali_max, ali_cos, w_ali;  /* minFlockingDistance, maxFlocking...     */
    unsigned mask_ali;
    float    coh_min, coh_max, coh_cos, w_coh;
    unsigned mask_coh;
    float    path_prediction_time, w_path;
    unsigned mask_path;
    float    w_seek;
    unsigned mask_seek;
    unsigned mask_antipen;                   /* maskAntiPenetrationAgents               */
    float    dt;
} gs_multigroup_params;

/* `steps` frames of a MultiGroup simulation (MultiGroupSimulation::update):
 * Group::preUpdate for every group (wrap, updateKNNDatabase, applied bits
 * cleared), every group pair's KNN in one launch into knn[i * n_groups + j]
 * (all n_groups^2 lists, owned by the caller), then Group::update of each
 * group in turn: avoid the other groups' neighbours, separation from every
 * group, alignment and cohesion with itself, path following and seek of the
 * path's second point when paths[i] is set (paths may be NULL), update, and
 * anti-penetration against every group.  One steering launch per group
 * replaces its per-call launches; results equal the per-function sequence
 * bit for bit.  At most 7 groups. */
gs_status gs_multigroup_step(const gs_group* groups, unsigned n_groups, gs_bins bins,
                             const gs_path* paths, gs_knn* knn, const gs_multigroup_params* p,
                             unsigned steps);
gs_status gs_find_knn_walls(gs_group g, gs_knn out, gs_bins bins, gs_walls walls,
                            unsigned search_radius);
/* KNNBruteForceCUDAV2 (KNNBruteForceCUDA.cu:163-187).  The lists are the
 * reference's for every pair of groups; with 4,096 queries or more the
 * scan skips candidates that cannot enter a list (a seeded bound and
 * bucketed chunks), so a call evaluates far fewer than n * m pairs. */
gs_status gs_knn_bruteforce(gs_group g, gs_knn out, gs_group other);
/* The (query, candidate) pairs the last gs_knn_bruteforce call of g ran its
 * distance filter on (n * m without the skipping scan).  Synchronises the
 * group's stream.  Not part of the reference. */
gs_status gs_knn_bruteforce_pairs(gs_group g, unsigned long long* pairs);
/* steerForSeparation / steerForAlignment / steerForCohesion
 * (GroupSteerLibrary.cuh:161-186). */
gs_status gs_steer_for_separation(gs_group g, gs_knn knn, gs_group other, float min_distance,
                                  float max_distance, float cos_max_angle, float weight,
                                  unsigned do_not_apply_with);
gs_status gs_steer_for_alignment(gs_group g, gs_knn knn, gs_group other, float min_distance,
                                 float max_distance, float cos_max_angle, float weight,
                                 unsigned do_not_apply_with);
gs_status gs_steer_for_cohesion(gs_group g, gs_knn knn, gs_group other, float min_distance,
                                float max_distance, float cos_max_angle, float weight,
                                unsigned do_not_apply_with);
/* steerForSeek (GroupSteerLibrary.cuh:52-59). */
/* ---- ExtractData diagnostics: ComputeCellDensity / ComputeAvgCellVelocity
 *      (ProcessData.cu:74-237, used by src/ExtractData.cpp).  Agents per cell of
 *      the group's KNN database, and each cell's mean velocity (direction * speed
 *      of its agents now, summed in ascending agent index, divided by the count;
 *      zero when empty).  The database is the one gs_update_knn_database built
 *      with these bins when it is current; otherwise, after gs_step and before
 *      anything else changes the group, the last step's own buckets, which are
 *      the database the reference's plugin built at the start of that frame
 *      (ChokePointNew.cpp:592, extracted after the frame at :422-426): no
 *      rebuild.  Host outputs: one unsigned / one float3 per cell.
 *      Synchronous. */
gs_status gs_cell_density(gs_group g, gs_bins bins, unsigned* counts);
gs_status gs_cell_avg_velocity(gs_group g, gs_bins bins, float* avg3);

/* ---- PolylinePathwayCUDA (PolylinePathwayCUDA.cu:7-56): n float3 points, tube
 * radius, cyclic closes the loop.  Segment lengths, unit directions and the
 * total length are computed on the host in binary32, as the reference does. */
gs_status gs_path_create(const float* points3, unsigned n, float radius, int cyclic,
                         gs_path* out);
gs_status gs_path_destroy(gs_path path);
/* The path's arrays (n + cyclic points; lengths[0] and normals[0] unused). */
gs_status gs_path_get(gs_path path, float* points3, float* lengths, float* normals3,
                      unsigned cap, unsigned* n, float* total_length);
/* steerToFollowPath (GroupSteerLibrary.cuh:88, SteerToFollowPathCUDAKernel.cu:183-287). */
gs_status gs_steer_to_follow_path(gs_group g, gs_path path, float prediction_time, float weight,
                                  unsigned do_not_apply_with);
gs_status gs_steer_for_seek(gs_group g, const float target[3], float weight,
                            unsigned do_not_apply_with);
/* steerToAvoidNeighbors (GroupSteerLibrary.cuh:111-118). */
gs_status gs_steer_to_avoid_neighbors(gs_group g, gs_knn knn, gs_group other,
                                      float min_time_to_collision, float min_separation_distance,
                                      int avoid_close_neighbors, float weight,
                                      unsigned do_not_apply_with);
/* steerToAvoidWalls (GroupSteerLibrary.cuh:120-127). */
gs_status gs_steer_to_avoid_walls(gs_group g, gs_knn knw, gs_walls walls,
                                  float min_time_to_collision, float weight,
                                  unsigned do_not_apply_with);
/* updateGroup (GroupSteerLibrary.cuh:189-196). */
gs_status gs_update_group(gs_group g, float elapsed_time);
/* antiPenetrationAgents (GroupSteerLibrary.cuh:216-223). */
gs_status gs_anti_penetration_agents(gs_group g, gs_knn knn, gs_group other,
                                     unsigned do_not_apply_with);
/* updateGroupWithAntiPenetration (GroupSteerLibrary.cuh:198-205,
 * UpdateCUDAKernelNew.cu:95-268): updateGroup that also pushes an agent out of
 * a wall it overlaps and removes the velocity component that would carry it
 * across a wall this step.  As the reference kernel: `knw` is read row-major
 * (entry i*k + s for agent i), the overlap test uses each segment's end point,
 * and appliedKernels is not cleared (bit KERNEL_ANTI_PENETRATION_WALL is
 * added). */
gs_status gs_update_group_with_antipenetration(gs_group g, gs_knn knw, gs_walls walls,
                                               float elapsed_time);
/* antiPenetrationWall (GroupSteerLibrary.cuh:207-214,
 * AntiPenetrationWallCUDAKernel.cu:52-134): an agent whose next move crosses a
 * listed wall turns its heading parallel to the nearest such wall.  `knw` is
 * read row-major as in the reference kernel; do_not_apply_with is accepted and,
 * as in the reference, not used. */
gs_status gs_anti_penetration_wall(gs_group g, gs_knn knw, gs_walls walls, float elapsed_time,
                                   unsigned do_not_apply_with);

/* ---- fused step -------------------------------------------------------------- */
/* Runs `steps` whole steps; the result equals the per-function sequence
 * wrap -> rebuild -> KNN (+ wall KNN) -> behaviours in p->order -> update.
 * Requires knn_mode GS_KNN_BINNED, and avoid-walls (if present) first in order.
 * `walls` may be NULL when the order has no GS_B_AVOID_WALLS. */
gs_status gs_step(gs_group g, gs_bins bins, gs_walls walls, const gs_step_params* p,
                  unsigned steps);
/* As gs_step but the state comes from and goes back to host arrays, each copy
 * on the group's stream (the reference's per-frame SyncDevice / SyncHost).
 * When `out` shares `in`'s maxSpeed, maxForce, radius and mass arrays, those
 * constants (which no step changes) are not copied back. */
gs_status gs_step_host(gs_group g, gs_bins bins, gs_walls walls, const gs_step_params* p,
                       unsigned steps, const gs_agent_arrays* in, unsigned n,
                       const gs_agent_arrays* out);
/* Replays one captured CUDA graph per fused step while the launch
 * configuration stays the same (default on).  The first step after an
 * upload of a scene of 131,072 agents or more runs eagerly: its permute
 * gathers, in one more launch.  Not part of the reference. */
gs_status gs_group_set_graphs(gs_group g, int enable);
/* Threads per block of the fused-step launches: 64, 128 or 256 (default).
 * Results do not depend on it; the autotuner picks it. */
gs_status gs_group_set_block(gs_group g, unsigned threads);
/* Candidate capacity of the fused step's KNN scan: 32 or 64 (collecting
 * scan, for sparse crowds), 128 or 256 (streaming scan, for crowded cells),
 * or 0 (default: chosen from the crowd's density, the agents in an agent's
 * cell averaged over the agents, measured at the first step after an upload
 * that changes the agent count, or after a grid change).  Results do not
 * depend on it: agents with more candidates are redone by the exact scan.
 * Not part of the reference. */
gs_status gs_group_set_knn_capacity(gs_group g, unsigned capacity);
/* The capacity the fused step uses: the fixed one, else the one measured at
 * the last step (0 before the first).  With 128 or 256 a step makes more
 * launches: the exact lists of the agents the fast scan hands to the redo,
 * found by one warp per agent (with avoid-walls they go straight into the
 * neighbour lists; without, a redo launch then steps those agents). */
gs_status gs_group_knn_capacity(gs_group g, unsigned* capacity);

/* ---- batched scenes -------------------------------------------------------------
 * Many independent worlds (e.g. one ChokePoint plugin instance each) advanced
 * together: every step of every scene is one CUDA graph launch, and each
 * scene's result is bit-identical to stepping it alone with gs_step (scene-
 * local agent and wall indices, scene-local cells).  All scenes share one
 * grid; agents are uploaded concatenated in scene order.  No reference
 * counterpart: the reference runs one group per plugin (plugins/ChokePointNew.cpp). */
typedef struct gs_batch_s* gs_batch;
gs_status gs_batch_create(unsigned n_scenes, const unsigned* agents_per_scene, unsigned k,
                          const unsigned world_cells[3], const float world_size[3],
                          unsigned search_radius, void* stream, gs_batch* out);
gs_status gs_batch_destroy(gs_batch b);
/* A scene's walls (split at the batch grid like gs_walls_create). */
gs_status gs_batch_set_walls(gs_batch b, unsigned scene, const float* start4, const float* end4,
                             const float* normal4, unsigned n);
gs_status gs_batch_upload(gs_batch b, const gs_agent_arrays* host);
gs_status gs_batch_download(gs_batch b, const gs_agent_arrays* host);
/* The batch's underlying group (stream, profiling, graphs, block size). */
gs_status gs_batch_group(gs_batch b, gs_group* g);
gs_status gs_batch_step(gs_batch b, const gs_step_params* p, unsigned steps);
/* Host state in, `steps` steps, host state out for several batches at once,
 * e.g. consecutive ranges of one workload's scenes: each part's upload, steps
 * and download are queued on its own stream, part after part, so that the
 * copies of one part run while another part steps (host<->device copies in
 * both directions and the steps overlap).  `in` and `out` hold the parts'
 * agents one part after another, each in its scene order; they may be the same
 * arrays (then maxSpeed, maxForce, radius and mass, which no step changes, are
 * not copied back), and page-locked host memory (gs_host_alloc) lets the
 * copies overlap.
 * Returns once every part's state is in `out`.  Each scene's result equals
 * gs_batch_step's.  A fixed KNN capacity (gs_group_set_knn_capacity on each
 * part's group) keeps the parts from waiting on the host for the automatic
 * capacity measurement that follows an upload. */
gs_status gs_batches_step_host(const gs_batch* parts, unsigned n_parts, const gs_step_params* p,
                               unsigned steps, const gs_agent_arrays* in,
                               const gs_agent_arrays* out);
/* ExtractData (gs_cell_density / gs_cell_avg_velocity) for every scene after
 * gs_batch_step, from that step's own buckets on the batch grid: cells scene
 * after scene (scene s at s * cells). */
gs_status gs_batch_cell_density(gs_batch b, unsigned* counts);
gs_status gs_batch_cell_avg_velocity(gs_batch b, float* avg3);

/* ---- differentiable rollouts --------------------------------------------------------
 * No counterpart in the reference.  A rollout runs `steps` fused steps of a
 * plain flock (separation, alignment, cohesion; no walls, seek or neighbour
 * avoidance) from the group's current state, keeping the time-varying state
 * every `checkpoint_every` steps, and then runs the hand-written adjoint of
 * the fused steering-plus-integrate step backwards through it: each segment
 * between checkpoints is re-run once with its steps' inputs and KNN lists
 * recorded, so memory grows with steps / checkpoint_every + checkpoint_every
 * states.  KNN lists and neighbourhood memberships are frozen at the
 * forward pass's values (piecewise constant); the derivative of the world
 * wrap is the identity.  Velocities are heading * speed. */
typedef struct gs_rollout_s* gs_rollout;
gs_status gs_rollout_create(gs_group g, gs_bins bins, unsigned steps, unsigned checkpoint_every,
                            gs_rollout* out);
gs_status gs_rollout_destroy(gs_rollout r);
/* Runs the rollout with parameters p (steering and applied bits start at zero);
 * the group is left at the final state. */
gs_status gs_rollout_forward(gs_rollout r, const gs_step_params* p);
/* Given device arrays (float4 per agent, agent order, .w ignored) of
 * d loss / d final position and velocity (either may be null: zero), writes
 * d loss / d initial position and velocity (device, float4 per agent; either
 * may be null) and d loss / d (w_separation, w_alignment, w_cohesion) to the
 * host array grad_weights.  Synchronous; the group is left at the final state. */
gs_status gs_rollout_backward(gs_rollout r, const float* adj_position, const float* adj_velocity,
                              float* grad_position0, float* grad_velocity0,
                              float grad_weights[3]);
/* The adjoint kernel of one step on caller-provided device arrays: the step's
 * recorded inputs (position | speed and heading as float4 per agent, KNN as
 * n x k row-major agent indices, UINT_MAX after the last), the constant
 * per-agent limits, and the adjoints of its outputs (adj_*_out, float4 per
 * agent; zeroed on return).  Adds the adjoints of its inputs to adj_*_in
 * (float4 per agent) and per-block sums of d loss / d weights to
 * weight_partials (4 floats per block of 256 agents: separation, alignment,
 * cohesion, unused).  Deterministic: no float atomics; each agent's terms
 * are summed in a fixed order.  Its scratch is allocated and freed on
 * `stream` (stream-ordered).  Asynchronous on `stream`. */
gs_status gs_flock_adjoint_step(const float* position_speed, const float* heading,
                                const unsigned* knn, unsigned n, unsigned k,
                                const float* max_speed, const float* max_force, const float* mass,
                                const gs_step_params* p, float* adj_position_out,
                                float* adj_velocity_out, float* adj_position_in,
                                float* adj_velocity_in, float* weight_partials,
                                unsigned partials_cap, void* stream);

/* ---- KNN without device allocation ------------------------------------------------
 * No counterpart in the reference: an addition for callers that cannot let a
 * library allocate device memory (pre-sized memory pools, real-time loops
 * that must not allocate, external allocation accounting).
 * Binned self-KNN of n device positions (float4) into caller-provided device
 * arrays idx_out / dist_out (k * n, column-major), with the same results as
 * gs_update_knn_database + gs_find_knn on the same grid and radius.  Its work
 * memory is a fixed 32 MiB array inside the library (reserved on every GPU
 * that loads it, until exit): problems needing more than
 * 8 * (cells + 1) + 4 * ceil(cells / 4096) + 28 * n bytes (plus alignment) of
 * it return GS_ERR_INVALID_ARG.  Calls share that array: calls that overlap
 * on the GPU race and must be serialised by the caller.  The first call in a
 * CUDA context looks up the array's address (cudaGetSymbolAddress) with that
 * context's device current and keeps it for that context: the first call on
 * each device, and the first after a cudaDeviceReset (which reloads the
 * library's module, possibly at another address), do the look-up; make them
 * before any stream capture.  Asynchronous on `stream`. */
gs_status gs_knn_binned_noalloc(const float* positions4, unsigned n,
                                const unsigned world_cells[3], const float world_size[3],
                                unsigned search_radius, unsigned k, unsigned* idx_out,
                                float* dist_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif
