/*
 * CPU oracle for the GPUSteer per-step agent update.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C++ restatement of the reference
 * CUDA kernels (PsychoLogicAu/GPUSteer, include/OpenSteer/CUDA/ kernel sources), used as
 * the checker for the sm_103a kernels in gpusteer_gb300/csrc.  Only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline leg (and bench.py
 * --impl reference) may load it.  The product library never links it and has
 * no CPU fallback.
 *
 * Parity pinning: the restatement is checked against golden vectors produced
 * by the reference's own kernel sources compiled for the CPU (oracle/ref,
 * fixtures in tests/golden/).  See each function for the reference lines it
 * follows.
 *
 * Arithmetic contract (shared with the CUDA kernels): IEEE binary32, no FMA
 * contraction (-ffp-contract=off here, -fmad=false in nvcc), IEEE division and
 * square root, operations evaluated in the reference's source order.
 *
 * Layouts follow include/OpenSteer/AgentGroupData.cuh:30-46: float4 position,
 * direction, steering (w unused); float3 side, up; float speed, maxSpeed,
 * maxForce, radius, mass; uint appliedKernels.  KNN output is column-major
 * idx[a + i*nA] (include/OpenSteer/CUDA/KNNBinningV2Kernel.cu:524-525).
 */
#ifndef GPUSTEER_ORACLE_H
#define GPUSTEER_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Structure-of-arrays view of one agent group (binary32). */
typedef struct orc_group {
    float*    position;   /* float4[n] */
    float*    direction;  /* float4[n] */
    float*    steering;   /* float4[n] */
    float*    side;       /* float3[n] */
    float*    up;         /* float3[n] */
    float*    speed;      /* [n] */
    float*    max_speed;  /* [n] */
    float*    max_force;  /* [n] */
    float*    radius;     /* [n] */
    float*    mass;       /* [n] */
    unsigned* applied;    /* [n] appliedKernels bit mask */
    unsigned  n;
} orc_group;

/* Same view in binary64, for the FP64 trajectory rerun. */
typedef struct orc_group_d {
    double*   position;   /* double4[n] */
    double*   direction;  /* double4[n] */
    double*   steering;   /* double4[n] */
    double*   side;       /* double3[n] */
    double*   up;         /* double3[n] */
    double*   speed;
    double*   max_speed;
    double*   max_force;
    double*   radius;
    double*   mass;
    unsigned* applied;
    unsigned  n;
} orc_group_d;

/* Wall segments (WallGroupData: float4 start/mid/end/normal, w = 0). */
typedef struct orc_walls {
    const float* start;   /* float4[n] */
    const float* mid;     /* float4[n] */
    const float* end;     /* float4[n] */
    const float* normal;  /* float4[n] */
    unsigned     n;
} orc_walls;

/* Behaviour codes for orc_step_params.order. */
enum {
    ORC_B_AVOID_WALLS     = 1,
    ORC_B_AVOID_NEIGHBORS = 2,
    ORC_B_SEPARATION      = 3,
    ORC_B_ALIGNMENT       = 4,
    ORC_B_COHESION        = 5,
    ORC_B_SEEK            = 6,
    ORC_B_FOLLOW_PATH     = 7
};

/* A polyline pathway as PolylinePathwayCUDA holds it (PolylinePathwayCUDA.cu:17-56):
 * n points (a cyclic path repeats the first point at the end), lengths[i] and
 * unit normals[i] of the segment from point i-1 to point i (index 0 unused). */
typedef struct orc_path {
    const float* points;   /* float3[n] */
    const float* lengths;  /* [n] */
    const float* normals;  /* float3[n] */
    unsigned     n;
    float        radius;
    int          cyclic;
    float        total_length;
} orc_path;

/* Wrap modes. */
enum {
    ORC_WRAP_REFERENCE = 0, /* WrapWorldCUDAKernel.cu:27-43, z<0 -> halfZ+100 */
    ORC_WRAP_SYMMETRIC = 1, /* x, y and z all wrapped like x and y            */
    ORC_WRAP_NONE      = 2
};

/* KNN modes. */
enum { ORC_KNN_BINNED = 0, ORC_KNN_BRUTEFORCE = 1 };

typedef struct orc_step_params {
    float    world_size[3];
    unsigned world_cells[3];
    unsigned search_radius;
    int      wrap_mode;
    int      knn_mode;
    unsigned k;
    int      clear_applied;          /* ChokePointNew.cpp:595 memset       */
    /* walls */
    unsigned knw;
    float    min_time_to_wall, w_walls;
    unsigned mask_walls;
    /* neighbour avoidance */
    float    min_time_to_collision, min_separation_distance;
    int      avoid_close;
    float    w_avoid;
    unsigned mask_avoid;
    /* flocking */
    float    sep_min, sep_max, sep_cos, w_sep;
    unsigned mask_sep;
    float    ali_min, ali_max, ali_cos, w_ali;
    unsigned mask_ali;
    float    coh_min, coh_max, coh_cos, w_coh;
    unsigned mask_coh;
    /* seek */
    float    seek_target[3], w_seek;
    unsigned mask_seek;
    /* order of behaviours (ORC_B_*) */
    unsigned order[8];
    unsigned n_order;
    float    dt;
    /* path following (ChokePointNew.cpp:620) */
    const orc_path* path;
    float    path_prediction_time, w_path;
    unsigned mask_path;
} orc_step_params;

/* ---- cells and KNN --------------------------------------------------- */
void orc_cell_index(const float* pos4, unsigned n, const float world_size[3],
                    const unsigned world_cells[3], unsigned* cell_out);

int orc_knn_binned(const float* posA4, unsigned nA, const float* posB4, unsigned nB,
                   int group_with_self, const float world_size[3],
                   const unsigned world_cells[3], unsigned search_radius, unsigned k,
                   unsigned* idx_out, float* dist_out, int threads);

int orc_knn_bruteforce(const float* posA4, unsigned nA, const float* posB4, unsigned nB,
                       int group_with_self, unsigned k, unsigned* idx_out,
                       float* dist_out, int threads);

/* ---- ExtractData diagnostics (ProcessData.cu:132-237) ----------------- */
/* Agents per cell of the binned database (cellEnd - cellStart, 0 when empty). */
void orc_cell_density(const float* pos4, unsigned n, const float world_size[3],
                      const unsigned world_cells[3], unsigned* counts_out);
/* Each cell's mean velocity: direction * speed of its agents summed in the
 * stable sort's order (ascending agent index), divided by the count; zero
 * for an empty cell.  avg3_out holds a float3 per cell. */
void orc_cell_avg_velocity(const float* pos4, const float* dir4, const float* speed, unsigned n,
                           const float world_size[3], const unsigned world_cells[3],
                           float* avg3_out);

/* ---- behaviours (one reference kernel each) -------------------------- */
void orc_wrap_world(orc_group* g, const float world_size[3], int mode);

void orc_steer_separation(orc_group* g, const unsigned* knn_idx, unsigned k,
                          const float* posB4, unsigned nB, float min_d, float max_d,
                          float cos_max, float w, unsigned mask);
void orc_steer_alignment(orc_group* g, const unsigned* knn_idx, unsigned k,
                         const float* posB4, const float* dirB4, unsigned nB, float min_d,
                         float max_d, float cos_max, float w, unsigned mask);
void orc_steer_cohesion(orc_group* g, const unsigned* knn_idx, unsigned k,
                        const float* posB4, unsigned nB, float min_d, float max_d,
                        float cos_max, float w, unsigned mask);
void orc_steer_seek(orc_group* g, const float target[3], float w, unsigned mask);
void orc_steer_avoid_neighbors(orc_group* g, const unsigned* knn_idx,
                               const float* knn_dist, unsigned k, const float* posB4,
                               const float* dirB4, const float* speedB,
                               const float* radiusB, unsigned nB, float min_time,
                               float min_sep, int avoid_close, float w, unsigned mask);
void orc_steer_avoid_walls(orc_group* g, const unsigned* knw_idx, unsigned knw,
                           const orc_walls* walls, float min_time, float w,
                           unsigned mask);
void orc_update(orc_group* g, float dt);
/* updateGroupWithAntiPenetration (UpdateCUDAKernelNew.cu:95-268) and
 * antiPenetrationWall (AntiPenetrationWallCUDAKernel.cu:52-134).  knl is the
 * walls' KNN array (k * n), read row-major as the reference kernels read it. */
void orc_update_with_antipenetration(orc_group* g, const unsigned* knl, unsigned k,
                                     const orc_walls* walls, float dt);
void orc_antipenetration_wall(orc_group* g, const unsigned* knl, unsigned k,
                              const orc_walls* walls, float dt);
/* antiPenetrationAgents (AntiPenetrationAgentsCUDAKernel.cu:57-109): posB4,
 * radiusB and appliedB are the other group's positions, radii and bits before
 * the pass (for a group with itself: copies taken before the call). */
void orc_antipenetration_agents(orc_group* g, const unsigned* knn_idx, const float* knn_dist,
                                const float* posB4, const float* radiusB,
                                const unsigned* appliedB, unsigned nB, unsigned mask);

/* PolylinePathwayCUDA::Initialize: from n_in float3 points, writes the path's
 * points, lengths and normals (n_in + cyclic entries, caller capacity n_in + 1)
 * and its total length; returns the number of points. */
int orc_path_init(const float* points3, unsigned n_in, int cyclic, float* points_out3,
                  float* lengths_out, float* normals_out3, float* total_out);
/* FollowPathCUDAKernel (SteerToFollowPathCUDAKernel.cu:183-287). */
void orc_steer_follow_path(orc_group* g, const orc_path* path, float prediction_time, float w,
                           unsigned mask);

/* ---- walls (WallGroupData.cu:73-206) ---------------------------------- */
/* Parse a .map file: 9 floats per segment (start, end, normal).
 * Returns the number of segments written (<= cap), or -1 on open failure. */
int orc_walls_load(const char* path, float* start4, float* mid4, float* end4,
                   float* normal4, unsigned cap);
/* Split walls at cell boundaries.  in/out arrays are float4.  Returns the
 * number of output segments, or -1 if cap is too small. */
int orc_walls_split(const float* start4, const float* mid4, const float* end4,
                    const float* normal4, unsigned n, const float world_size[3],
                    const unsigned world_cells[3], float* out_start4, float* out_mid4,
                    float* out_end4, float* out_normal4, unsigned cap);

/* ---- whole steps ----------------------------------------------------- */
/* Runs `steps` steps.  knn_idx/knn_dist (k*n each, may be NULL) receive the
 * self KNN of the last step.  threads <= 0 means all OpenMP threads. */
int orc_run(orc_group* g, const orc_walls* walls, const orc_step_params* p,
            unsigned steps, unsigned* knn_idx, float* knn_dist, int threads);
int orc_run_d(orc_group_d* g, const orc_walls* walls, const orc_step_params* p,
              unsigned steps, int threads);

int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
