// Internal structures of libgpusteer: handle layouts, launch helpers, error
// reporting.  Not part of the ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "../../include/gpusteer.h"
#include "gs_math.cuh"

namespace gs {

constexpr unsigned kMaxK = 64;
constexpr int kBlock = 256;

// ---- errors -------------------------------------------------------------------
void set_error(const std::string& msg);
gs_status fail(gs_status s, const std::string& msg);
gs_status cuda_fail(cudaError_t e, const char* what);

#define GS_CUDA(call)                                             \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return ::gs::cuda_fail(e_, #call); \
    } while (0)
#define GS_LAUNCHED(what)                                         \
    do {                                                          \
        cudaError_t e_ = cudaGetLastError();                      \
        if (e_ != cudaSuccess) return ::gs::cuda_fail(e_, what);  \
    } while (0)
#define GS_TRY(call)                       \
    do {                                   \
        gs_status s_ = (call);             \
        if (s_ != GS_OK) return s_;        \
    } while (0)

inline unsigned blocks_for(unsigned n, unsigned b = kBlock) { return (n + b - 1) / b; }

template <class T> gs_status dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) return GS_OK;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(GS_ERR_OOM, "device allocation failed");
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    return GS_OK;
}
template <class T> void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// ---- scenes -------------------------------------------------------------------
// One independent world.  A single group is one scene; the batched engine
// concatenates many.  Cell labels of scene s occupy
// [cell_offset, cell_offset + cells); its walls' cell table starts at
// wall_cell_offset and its wall segments at wall_offset.
struct Scene {
    Grid grid;
    unsigned cell_offset;
    unsigned agent_offset;
    unsigned n_agents;
    unsigned wall_offset;
    unsigned n_walls;
    unsigned wall_cell_offset;
};
inline bool operator==(const Scene& a, const Scene& b) {
    return std::memcmp(&a, &b, sizeof(Scene)) == 0;
}

// Bucketed ("fused") state: six float4 streams per agent.
//   f0 = position.xyz, agent index (bits)    f1 = direction.xyz, speed
//   f2 = side.xyz, radius                    f3 = up.xyz, mass
//   f4 = maxSpeed, maxForce, applied (bits), scene (bits)
//   f5 = steering.xyz, 0  (read only while the steering may be non-zero)
struct Fused {
    float4* f[6];
};

// Wall segment (WallGroupData: start, mid, end, normal).
struct Segment {
    V3 s, m, e, n;
};

// Raw copies of a launch's parameter blocks (compared byte-wise to decide
// whether a captured graph still applies).
struct FusedLaunchBytes {
    unsigned char b[384];
};
struct StepDevBytes {
    unsigned char b[384];
};

// A group's bucketed binning database (KNNDatabase.cuh:30-38): cell of every
// agent, the sorted agent indices and positions, and cell_start[C + 1]
// (cell c holds slots cell_start[c] .. cell_start[c + 1]).
struct Database {
    unsigned cells = 0;         // C allocated for
    unsigned* cell = nullptr;   // [n] cell label
    unsigned* rank = nullptr;   // [n] rank within the cell (atomic order)
    unsigned* sorted = nullptr; // [n] agent index of slot
    float4* pos_id = nullptr;   // [n] (position.xyz, agent index bits) of slot
    unsigned* start = nullptr;  // [C + 1]
    unsigned* count = nullptr;  // [C] zero between uses
    unsigned* tile = nullptr;   // scan scratch; the fused engine's exact tile totals
    unsigned* live = nullptr;   // [T] tiles the fused engine's last scan wrote
    unsigned agent_cap = 0;     // agents the per-agent arrays hold, where tracked
    bool valid = false;
    Grid grid{};
};

}  // namespace gs

struct gs_bins_s {
    gs::Grid grid;
    unsigned radius;
    unsigned cells;
};

struct gs_knn_s {
    unsigned n, k;
    unsigned* idx;
    float* dist;
};

struct gs_walls_s {
    unsigned n, knw;
    std::vector<float> h_start, h_mid, h_end, h_normal;  // float4 each
    float4 *start = nullptr, *mid = nullptr, *end = nullptr, *normal = nullptr;
    gs::Database db;  // agents vs wall midpoints
    cudaStream_t stream = nullptr;
};

struct gs_group_s {
    unsigned k, capacity, n;
    cudaStream_t stream;
    bool own_stream;
    // reference-layout arrays
    float4 *position, *direction, *steering;
    float3 *side, *up;
    float *speed, *max_speed, *max_force, *radius, *mass;
    unsigned* applied;
    // binning database for the per-function API
    gs::Database db;
    // fused-step state
    gs::Fused A, B;
    uint2* cellrank;       // next cell and rank per slot of A
    float4 *w0, *w1, *w2;  // wall-phase outputs: corrected position | radius,
                           // direction | speed, steering | applied
    unsigned* knn_slot;    // [k * n] neighbour slots (wall phase)
    float* knn_dist;       // [k * n]
    gs::Database fdb;      // counts / starts of the fused step
    // brute-force KNN's seed search: databases of the queries and of the
    // other group on an automatic grid; scratch (words 0-2: the extent,
    // words 4-5: the pairs the filter ran on); the candidates' chunk boxes
    gs::Database bf_a, bf_b;
    unsigned* bf_tmp;
    float4* bf_boxes;
    size_t bf_boxes_cap;         // boxes bf_boxes holds
    bool bf_counted;             // the last call counted its pairs in bf_tmp
    unsigned long long bf_pairs; // else the pairs it ran on (n * m)
    gs::Scene* d_scene;    // scene table (one entry for a plain group)
    unsigned scene_alloc;
    std::vector<gs::Scene>* h_scenes;  // host copy of the table on the device
    unsigned* d_err;       // device error flags (see FusedLaunch::err)
    unsigned* retry;       // [capacity] exact-redo list and its counter
    unsigned* slot_of;     // [capacity] each agent's slot (conversion to the reference layout)
    unsigned* retry_count;
    unsigned* retry_knn;   // [min(capacity, kRetryListCap) * kRetryListK] exact-redo lists
    unsigned* d_stat;      // four words of scratch for device-side statistics
    // candidate capacity of the fused KNN scan: knn_cap fixed by the caller
    // (gs_group_set_knn_capacity), else auto_cap, measured from the crowd's
    // density when the state is uploaded or the grid changes
    unsigned knn_cap, auto_cap, auto_cap_r;
    bool auto_cap_valid;
    gs::Grid auto_cap_grid;
    bool fused_current;    // true: A holds the state, reference arrays stale
    // cells of the last completed fused step's database while the state is still
    // that step's result (0 once anything changes it): fdb.start then holds the
    // step's start-of-step buckets and A the agents' new state per slot
    unsigned frame_cells;
    void* diag;            // scratch of the cell diagnostics, grown on demand
    size_t diag_bytes;
    void* ap;              // scratch of anti-penetration (new positions, bit snapshot)
    cudaEvent_t read_ev;   // marks this group's reads of another group (read_done)
    size_t ap_bytes;
    bool accum_dirty;      // steering / applied may be non-zero
    int pending_wrap;      // wrap mode the pending cell counts were taken with
    unsigned fused_k_alloc;
    bool persistent;       // run supported steps as one persistent launch
    unsigned bar_limit;    // its barrier poll limit (0: default)
    unsigned* d_bar;       // its grid barrier (2 words)
    // phase profiling (gs_group_set_profiling)
    bool profiling;
    std::vector<cudaEvent_t>* prof_events;  // pairs of (start, stop) per recorded phase
    std::vector<int>* prof_phase;
    float prof_ms[4];
    unsigned prof_launches[4];
    // CUDA graph of one fused step, replayed while the launch configuration
    // (buffers, parameters, grid) stays the same
    bool use_graph;
    unsigned block;
    cudaGraphExec_t graph_exec;
    gs::FusedLaunchBytes graph_L;
    gs::StepDevBytes graph_d;
    unsigned graph_C;
};

// PolylinePathwayCUDA: host arrays (binary32, PolylinePathwayCUDA.cu:17-56)
// and their device copies.
struct gs_path_s {
    std::vector<float> h_points, h_lengths, h_normals;  // float3[n], [n], float3[n]
    float3* d_points = nullptr;
    float* d_lengths = nullptr;
    float3* d_normals = nullptr;
    unsigned n = 0;
    float radius = 0.f, total = 0.f;
    int cyclic = 0;
};

struct gs_batch_s {
    gs_group g = nullptr;  // all scenes' agents, concatenated
    gs::Grid grid{};
    unsigned cells = 0, radius = 1, total = 0;
    std::vector<unsigned> counts;
    std::vector<gs::Scene> scenes;
    std::vector<std::vector<gs::Segment>> walls;  // per scene, split on the grid
    bool walls_dirty = false;
    unsigned n_walls = 0;
    unsigned* agent_scene = nullptr;
    float4 *w_start = nullptr, *w_end = nullptr, *w_normal = nullptr, *w_pos_id = nullptr;
    unsigned* w_cell_start = nullptr;
    // gs_batches_step_host: this batch's upload, steps and download captured
    // as one graph, replayed while its key (host arrays, buffers, parameters)
    // stays the same
    cudaGraphExec_t io_exec = nullptr;
    std::vector<unsigned char> io_key;
};
