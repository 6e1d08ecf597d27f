// Host-side launch wrappers shared by the C ABI implementation.
#pragma once

#include "gs_behaviours.cuh"
#include "gs_internal.cuh"

namespace gs {

// ---- counting-sort binning ---------------------------------------------------
// Exclusive scan of count[0..C) into start[0..C]; zeroes count.
gs_status scan_counts(unsigned* count, unsigned* start, unsigned C, unsigned* tile,
                      cudaStream_t st);
unsigned scan_tile_count(unsigned C);
// The fused engine's scan in one launch: tile[] holds exact tile totals
// (added by the counting atomics), and only tiles within `reach` tiles of an
// occupied one get starts (live[t] = 1) and zeroed counts.
gs_status scan_counts_sparse(unsigned* count, unsigned* start, unsigned C, const unsigned* tile,
                             unsigned* live, unsigned reach, cudaStream_t st);
// tile[t] = the total of count[] over scan tile t (after a whole recount,
// whose agents come in no spatial order: per-agent tile atomics would all
// contend on a few hundred words).
gs_status scan_tile_totals(const unsigned* count, unsigned C, unsigned* tile, cudaStream_t st);
// Tiles (of the scan) between a cell and the farthest start its box of
// radius r reads, on a grid of wc cells.
unsigned scan_reach_tiles(const unsigned wc[3], unsigned r);
// Allocates db for C cells and n agents (keeps existing buffers when large enough).
gs_status db_reserve(Database& db, unsigned n, unsigned C);
void db_release(Database& db);
// updateKNNDatabase: bucket n positions (float4, reference layout) by cell.
gs_status db_build(Database& db, const float4* pos, unsigned n, const Grid& grid,
                   cudaStream_t st);

// ---- per-function (drop-in) kernels -----------------------------------------
gs_status launch_knn_binned(const Database& A, unsigned nA, const Database& B, bool self,
                            unsigned r, unsigned k, unsigned* idx, float* dist, cudaStream_t st);
// Batched binned KNN over (A, B) database pairs of one grid (every group pair
// of a MultiGroup frame): one launch, results as launch_knn_binned per pair.
// 49 pairs (seven groups, every pair) keep the parameter block under 4 KiB.
constexpr unsigned kMaxKnnPairs = 49;
struct KnnPair {
    const unsigned* a_sorted;
    const float4* a_pos_id;
    const unsigned* b_start;
    const float4* b_pos_id;
    unsigned* idx;
    float* dist;
    unsigned nA, k, block_begin;
    bool self;
};
struct KnnPairs {
    KnnPair pair[kMaxKnnPairs];
    Grid grid;
    unsigned r, n_pairs;
};
gs_status launch_knn_binned_pairs(KnnPairs& P, cudaStream_t st);
// seed (may be null): per query of A an upper bound of its k-th distance.
gs_status launch_knn_brute(const float4* posA, unsigned nA, const float4* posB, unsigned nB,
                           bool self, unsigned k, const float* seed, unsigned* idx, float* dist,
                           cudaStream_t st);
// Per query of A (by agent index) an upper bound of its k-th distance to B's
// agents: the k-th among the candidates of a box of cells (1 <= k <= 64).
gs_status launch_brute_seed(const Database& A, unsigned nA, const Database& B, bool self,
                            unsigned k, float* seed, cudaStream_t st);
// The same lists over bucketed queries and candidates (the seed databases'
// pos_id arrays), skipping chunks of 64 candidates beyond every bound of a
// warp's queries; k <= 64 and a seed.  boxes: 2 * (ceil(nB / 64) +
// ceil(nB / 2048)) float4 of scratch (chunk, then stage boxes); evaluated
// (may be null) adds the pairs the filter ran on.
gs_status launch_knn_brute_bucketed(const float4* qpos, unsigned nA, const float4* cpos,
                                    unsigned nB, float4* boxes, bool self, unsigned k,
                                    const float* seed, unsigned long long* evaluated,
                                    unsigned* idx, float* dist, cudaStream_t st);
// Largest |coordinate| per axis of n positions (synchronises st); d_tmp3: 3 words.
gs_status abs_extent(const float4* pos, unsigned n, unsigned* d_tmp3, float out[3],
                     cudaStream_t st);
gs_status launch_wrap(float4* pos, unsigned n, const float ws[3], int mode, cudaStream_t st);
gs_status launch_cell_density(const Database& db, unsigned* out, cudaStream_t st);
gs_status launch_cell_avg_velocity(const Database& db, const float4* dir, const float* speed,
                                   float3* out, cudaStream_t st);
// The same diagnostics over a fused step's frame (start-of-step buckets, new
// state in A; live: the tiles whose starts the step's scan wrote).
gs_status launch_frame_cell_density(const unsigned* start, const unsigned* live, unsigned C,
                                    unsigned* out, cudaStream_t st);
gs_status launch_frame_cell_avg_velocity(const unsigned* start, const unsigned* live,
                                         unsigned C, const float4* f0, const float4* f1,
                                         float3* out, cudaStream_t st);

struct GroupView {
    float4 *position, *direction, *steering;
    float3 *side, *up;
    float *speed, *max_speed, *max_force, *radius, *mass;
    unsigned* applied;
    unsigned n;
};
struct OtherView {
    const float4 *position, *direction;
    const float *speed, *radius;
    const unsigned* applied;
    unsigned n;
};
// kind: 0 separation, 1 alignment, 2 cohesion
gs_status launch_flock(int kind, GroupView g, const unsigned* knn, unsigned k, OtherView o,
                       float min_d, float max_d, float cos_max, float w, unsigned mask,
                       cudaStream_t st);
gs_status launch_seek(GroupView g, const float target[3], float w, unsigned mask,
                      cudaStream_t st);
gs_status launch_avoid_neighbors(GroupView g, const unsigned* knn, const float* knn_dist,
                                 unsigned k, OtherView o, float min_time, float min_sep,
                                 bool avoid_close, float w, unsigned mask, cudaStream_t st);
gs_status launch_avoid_walls(GroupView g, const unsigned* knw, unsigned kw, const float4* start,
                             const float4* end, const float4* normal, unsigned n_lines,
                             float min_time, float w, unsigned mask, cudaStream_t st);
gs_status launch_update(GroupView g, float dt, cudaStream_t st);
// MultiGroup (plugins/MultiGroup.cpp:558-601): one group's behaviour calls of
// a frame in one pass, reading every group's current state and this group's
// KNN lists against each of them.
constexpr unsigned kMaxGroups = 7;
struct MultiSteer {
    GroupView g;
    OtherView o[kMaxGroups];
    const unsigned* idx[kMaxGroups];
    const float* dist[kMaxGroups];
    unsigned k[kMaxGroups];
    unsigned n_groups, self;
    float min_time, min_sep, w_avoid;
    unsigned mask_avoid;
    int avoid_close;
    FlockParams sep, ali, coh;
    int has_path;
    PathDev path;
    float path_time, w_path, w_seek;
    unsigned mask_path, mask_seek;
    float seek_target[3];
};
gs_status launch_multigroup_steer(const MultiSteer& M, cudaStream_t st);
gs_status launch_update_antipen_wall(GroupView g, const unsigned* knl, unsigned k,
                                     const float4* start, const float4* end,
                                     const float4* normal, unsigned n_lines, float dt,
                                     cudaStream_t st);
gs_status launch_antipen_wall(GroupView g, const unsigned* knl, unsigned k, const float4* start,
                              const float4* end, const float4* normal, unsigned n_lines,
                              float dt, cudaStream_t st);
gs_status launch_follow_path(GroupView g, const PathDev& path, float prediction_time, float w,
                             unsigned mask, cudaStream_t st);
gs_status launch_antipenetration(GroupView g, const unsigned* knn, const float* knn_dist,
                                 unsigned k, OtherView o, const unsigned* applied_snapshot,
                                 float4* pos_out, unsigned mask, cudaStream_t st);

// ---- fused step ------------------------------------------------------------------
struct StepDev {
    unsigned k, knw, r;
    int wrap_mode, clear_applied, dirty;
    float sep[5], ali[5], coh[5];  // min, max, cos, weight, mask bits
    // exact squared-distance forms of each flocking test's d < min and
    // d > max: (lt, gt) with d < min <=> dsq < lt and d > max <=> dsq > gt
    float sep_dsq[2], ali_dsq[2], coh_dsq[2];
    float seek_target[3], w_seek;
    unsigned mask_seek;
    float min_time_wall, w_walls;
    unsigned mask_walls;
    float min_time_col, min_sep;
    int avoid_close;
    float w_avoid;
    unsigned mask_avoid;
    unsigned order[8];
    unsigned order_packed;  // order[o] in bits 3o .. 3o+2 (codes 1..7)
    unsigned n_order;
    float dt;
    unsigned need;      // NEED_* bits
    unsigned enum_cap;  // candidate capacity of the fast KNN scan (32, 64: collecting; 128, 256: streaming)
    unsigned block;     // threads per block of the fused launches (0: 256)
    unsigned flat;      // the grid is one cell high (y): boxes hold 3 rows of cells
    unsigned scan_reach;  // scan_reach_tiles of the step's grid and radius
    unsigned persistent;  // run a supported step as one persistent launch
    unsigned bar_limit;   // its barrier poll limit
    unsigned fresh;       // A is in agent order (first step after an upload)
    PathDev path;       // path following (GS_B_FOLLOW_PATH)
    float path_time, w_path;
    unsigned mask_path;
};
constexpr unsigned NEED_SEP = 1, NEED_ALI = 2, NEED_COH = 4, NEED_AVOID = 8, NEED_CLOSE = 16,
                   NEED_WALLS = 32;
// Bits of the fused step's device error word.
constexpr unsigned kErrCounts = 1u;          // inconsistent cell counts
constexpr unsigned kErrBarrierTimeout = 2u;  // a persistent step's barrier wait ran out

// The persistent step's extra arguments: the scan's writable starts and tile
// totals, the barrier words (zeroed before each launch) and the poll limit.
struct PersistLaunch {
    unsigned* start;
    unsigned* tile;
    unsigned* live;
    unsigned C, T;
    unsigned* bar;  // 2 words
    unsigned limit;
};
constexpr unsigned kBarrierPollsDefault = 1u << 23;  // about a second of 100 ns polls

// The exact redo's precomputed neighbour lists: kRetryListK slots per entry
// (the largest KMAX), for up to kRetryListCap entries per step.
constexpr unsigned kRetryListK = 32;
constexpr unsigned kRetryListCap = 16384;
constexpr unsigned kRetryNotListed = 0xfffffffeu;

struct FusedLaunch {
    Fused A, B;
    uint2* cellrank;
    unsigned* count;
    // [tiles] exact totals of count per scan tile: zeroed by the permute,
    // added by the counting atomics
    unsigned* tile;
    unsigned tiles;
    const unsigned* start;
    const Scene* scenes;
    unsigned n;
    // walls (may be null)
    const float4 *w_start, *w_end, *w_normal, *w_pos_id;
    const unsigned* w_cell_start;
    float4 *w0, *w1, *w2;
    unsigned* knn_slot;
    float* knn_dist;
    unsigned* err;  // device flag: bit 0 = a bucketed slot fell outside [0, n)
    unsigned* retry;        // [n] slots the fast KNN handed to the exact redo
    unsigned* retry_count;  // zeroed by the permute launch of each step
    unsigned* agent_at;     // [n] the fresh permute's slot -> agent map (scratch)
    // [retry_cap * kRetryListK] the exact neighbour slots of the first
    // retry_cap redo entries, written by the warp-per-agent exact search
    // (entry 0 = kRetryNotListed when that search left the entry to the
    // redo's own thread)
    unsigned* retry_knn;
    unsigned retry_cap;
    // optional record of the step's inputs by agent index (rollouts for the
    // adjoint; walls-free steps only): null when not recording
    float4* rec_pos;    // [n] position | speed before the step (after the wrap)
    float4* rec_dir;    // [n] heading | 0
    unsigned* rec_knn;  // [n * k] neighbour indices, row-major, UINT_MAX after the last
};

// Both count each agent's cell into count[] (zeroed beforehand); the scan
// tile totals follow from scan_tile_totals.
gs_status fused_from_reference(GroupView g, const unsigned* agent_scene, const Scene* scenes,
                               Fused A, uint2* cellrank, unsigned* count, int wrap_mode,
                               bool dirty, cudaStream_t st);
gs_status fused_recount(Fused A, unsigned n, const Scene* scenes, uint2* cellrank,
                        unsigned* count, int wrap_mode, cudaStream_t st);
// fresh: A is in agent order (the first step after an upload), permuted by a
// gather through L.agent_at (two launches instead of one).
gs_status fused_permute(const FusedLaunch& L, int wrap_mode, bool dirty, bool fresh,
                        cudaStream_t st);
// `phase` (may be null) brackets each launch: phase(i, true) before and
// phase(i, false) after the launch of phase i.
struct PhaseHook {
    virtual void mark(int phase, bool begin) = 0;
};
// The wall/rest step as one cooperative persistent launch (see gs_step.cu);
// persistent_supported tells which steps have that build.
bool persistent_supported(const StepDev& p);
gs_status fused_step_persistent(const FusedLaunch& L, const StepDev& p, const PersistLaunch& P,
                                cudaStream_t st);
gs_status fused_step(const FusedLaunch& L, const StepDev& p, cudaStream_t st,
                     PhaseHook* hook = nullptr);
// slot_of: capacity words of scratch (each agent's slot, then the gather).
gs_status fused_to_reference(Fused A, unsigned n, const Scene* scenes, unsigned* slot_of,
                             GroupView g, cudaStream_t st);
// ---- adjoint of the fused flocking step -------------------------------------------
// Inputs recorded by a forward step (FusedLaunch::rec_*), the agents' constant
// limits, and the adjoints of the step's outputs; accumulates the adjoints of
// its inputs and the steering weights.
struct AdjointLaunch {
    const float4* pos;   // [n] recorded position | speed
    const float4* dir;   // [n] recorded heading
    const unsigned* knn; // [n * k] recorded neighbour indices
    const float *max_speed, *max_force, *mass;
    float4 *lp_in, *lv_in;    // d loss / d (position, velocity) after the step; zeroed
    float4 *lp_out, *lv_out;  // d loss / d (position, velocity) before the step; +=
    float* wpart;             // [blocks * 4] per-block sums: separation, alignment, cohesion
    unsigned n, k;
    // scratch (adjoint_scratch_bind): per-edge and own terms; per target agent
    // its fill count (fill[n]: overflow count) and kBucket edge slots; the
    // overflow list of (target, edge) pairs
    float4 *edge_p, *edge_v, *own_p, *own_v;
    unsigned *fill, *bucket, *ovf;
};
constexpr unsigned kBucket = 48;
unsigned adjoint_blocks(unsigned n);
size_t adjoint_scratch_bytes(unsigned n, unsigned k);
void adjoint_scratch_bind(AdjointLaunch& A, void* base, unsigned n, unsigned k);
gs_status launch_flock_adjoint(const AdjointLaunch& A, const StepDev& p, cudaStream_t st);

// Number of non-zero entries of count[0..C) and the sum of their squares,
// read back to the host (syncs st); d_tmp: 4 words of device scratch.
gs_status count_occupied(const unsigned* count, unsigned C, unsigned* d_tmp, unsigned* h_out,
                         unsigned long long* h_sumsq, cudaStream_t st);

}  // namespace gs
