// Reference harness: runs PsychoLogicAu/GPUSteer's own CUDA kernel sources on
// the CPU (through cpu_simt.h) to produce golden vectors for the oracle.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/ref/Makefile from the sources
// where they lie in the reference tree; output goes to oracle/_ref/ (git
// ignored).  Each kernel file is compiled unmodified inside its own
// namespace so that the texture globals every file defines do not collide.
// The host-side set-up below follows the reference's host wrappers
// (file:line cited per function); kernels are launched one emulated CUDA
// block at a time, threads as fibers with a real __syncthreads() barrier.
#include "cpu_simt.h"

#include <ucontext.h>

#include <algorithm>
#include <functional>
#include <numeric>
#include <vector>

// ---- fiber SIMT emulation -----------------------------------------------------
uint3 gsref_threadIdx, gsref_blockIdx;
dim3 gsref_blockDim, gsref_gridDim;

namespace {
enum { RUNNABLE = 0, AT_BARRIER = 1, DONE = 2 };
struct Fiber {
    ucontext_t ctx;
    int state;
};
constexpr size_t kStack = 128 * 1024;
ucontext_t g_sched;
std::vector<Fiber> g_fibers;
std::vector<char> g_stacks;
const std::function<void()>* g_body = nullptr;
unsigned g_cur = 0;

void trampoline() {
    (*g_body)();
    g_fibers[g_cur].state = DONE;
    swapcontext(&g_fibers[g_cur].ctx, &g_sched);
}

void launch(unsigned grid, unsigned block, const std::function<void()>& body) {
    if (g_fibers.size() < block) {
        g_fibers.resize(block);
        g_stacks.resize(block * kStack);
    }
    g_body = &body;
    gsref_gridDim = dim3(grid, 1, 1);
    gsref_blockDim = dim3(block, 1, 1);
    for (unsigned b = 0; b < grid; ++b) {
        gsref_blockIdx = make_uint3(b, 0, 0);
        for (unsigned t = 0; t < block; ++t) {
            Fiber& f = g_fibers[t];
            getcontext(&f.ctx);
            f.ctx.uc_stack.ss_sp = &g_stacks[t * kStack];
            f.ctx.uc_stack.ss_size = kStack;
            f.ctx.uc_link = nullptr;
            makecontext(&f.ctx, trampoline, 0);
            f.state = RUNNABLE;
        }
        for (;;) {
            for (unsigned t = 0; t < block; ++t) {
                if (g_fibers[t].state != RUNNABLE) continue;
                g_cur = t;
                gsref_threadIdx = make_uint3(t, 0, 0);
                swapcontext(&g_sched, &g_fibers[t].ctx);
            }
            unsigned done = 0;
            for (unsigned t = 0; t < block; ++t) done += g_fibers[t].state == DONE;
            if (done == block) break;
            // Every live thread is at the barrier: release them together.
            for (unsigned t = 0; t < block; ++t)
                if (g_fibers[t].state == AT_BARRIER) g_fibers[t].state = RUNNABLE;
        }
    }
}
unsigned blocks(unsigned n, unsigned b) { return (n + b - 1) / b; }
}  // namespace

void gsref_syncthreads() {
    g_fibers[g_cur].state = AT_BARRIER;
    swapcontext(&g_fibers[g_cur].ctx, &g_sched);
    gsref_threadIdx = make_uint3(g_cur, 0, 0);
}

// ---- the reference kernel sources, each in its own namespace -----------------
namespace ref_knn { GSREF_DYNAMIC_SHARED
#include "KNNBinningV2Kernel.cu"
}
namespace ref_brute { GSREF_DYNAMIC_SHARED
#include "KNNBruteForceCudaKernel.cu"
}
namespace ref_sep { GSREF_DYNAMIC_SHARED
#include "SteerForSeparationCUDAKernel.cu"
}
namespace ref_coh { GSREF_DYNAMIC_SHARED
#include "SteerForCohesionCUDAKernel.cu"
}
namespace ref_ali { GSREF_DYNAMIC_SHARED
#include "SteerForAlignmentCUDAKernel.cu"
}
namespace ref_seek { GSREF_DYNAMIC_SHARED
#include "SteerForSeekCUDAKernel.cu"
}
namespace ref_avoid { GSREF_DYNAMIC_SHARED
#include "SteerToAvoidNeighborsCUDAKernel.cu"
}
namespace ref_walls { GSREF_DYNAMIC_SHARED
#include "AvoidWallsCUDAKernel.cu"
}
namespace ref_update { GSREF_DYNAMIC_SHARED
#include "UpdateCUDAKernel.cu"
}
namespace ref_wrap { GSREF_DYNAMIC_SHARED
#include "WrapWorldCUDAKernel.cu"
}
namespace ref_antipen { GSREF_DYNAMIC_SHARED
#include "AntiPenetrationAgentsCUDAKernel.cu"
}
namespace ref_path { GSREF_DYNAMIC_SHARED
#include "SteerToFollowPathCUDAKernel.cu"
}
namespace ref_update_ap { GSREF_DYNAMIC_SHARED
#include "UpdateCUDAKernelNew.cu"
}
namespace ref_antipen_wall { GSREF_DYNAMIC_SHARED
#include "AntiPenetrationWallCUDAKernel.cu"
}
// ProcessData.cu's kernel section (ComputeCellDensityKernel, the texture
// bindings and ComputeAvgCellVelocityKernel, ProcessData.cu:131-237), cut
// unmodified out of the file by the recipe: the file's host functions use
// <<<>>> launches and the AgentGroup class, which this harness does not build.
namespace ref_diag { GSREF_DYNAMIC_SHARED
#include "ProcessDataKernels.inc"
}

namespace {
constexpr unsigned TPB = THREADSPERBLOCK;  // AbstractCUDAKernel.cuh:46-54

const float4* f4(const float* p) { return reinterpret_cast<const float4*>(p); }
float4* f4(float* p) { return reinterpret_cast<float4*>(p); }
const float3* f3(const float* p) { return reinterpret_cast<const float3*>(p); }
float3* f3(float* p) { return reinterpret_cast<float3*>(p); }

// One group's binned database (KNNDatabase.cuh:30-38).
struct BinDB {
    std::vector<size_t> agentIdx, cellIdx;  // BuildDB writes size_t (KNNBinningV2Kernel.cu:269-272)
    std::vector<uint> agentSorted, cellSorted, cellStart, cellEnd;
    std::vector<float4> posSorted;
};

// KNNBinningV2UpdateDBCUDA::run, KNNBinningV2.cu:87-142.
void update_db(BinDB& db, const float* pos4, unsigned n, unsigned numCells) {
    db.agentIdx.assign(n, 0);
    db.cellIdx.assign(n, 0);
    launch(blocks(n, TPB), TPB, [&] {
        ref_knn::KNNBinningV2BuildDB(f4(pos4), db.agentIdx.data(), db.cellIdx.data(), n);
    });
    // thrust::sort_by_key (KNNBinningV2.cu:127-129) is a stable radix sort.
    std::vector<uint> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(),
                     [&](uint a, uint b) { return db.cellIdx[a] < db.cellIdx[b]; });
    db.agentSorted.resize(n);
    db.cellSorted.resize(n);
    for (unsigned i = 0; i < n; ++i) {
        db.agentSorted[i] = uint(db.agentIdx[order[i]]);
        db.cellSorted[i] = uint(db.cellIdx[order[i]]);
    }
    db.cellStart.assign(numCells, 0xffffffffu);  // KNNBinningV2.cu:132
    db.cellEnd.assign(numCells, 0u);
    db.posSorted.assign(n, make_float4(0, 0, 0, 0));
    ref_knn::KNNBinningV2ReorderDBBindTextures(f4(pos4), n);
    launch(blocks(n, TPB), TPB, [&] {
        ref_knn::KNNBinningV2ReorderDB(db.agentSorted.data(), db.cellSorted.data(),
                                       db.posSorted.data(), db.cellStart.data(),
                                       db.cellEnd.data(), n);
    });
    ref_knn::KNNBinningV2ReorderDBUnbindTextures();
}

// KNNBinDataV2 construction (KNNBinDataV2.cu:30-168): the cells, the
// constants and the 3D cell lookup array.  The lookup array is laid out so
// that texel (x, y, z) holds the bin_cell label x + z*X + y*X*Z, the
// labelling the neighbour table is indexed by.
struct BinGrid {
    std::vector<OpenSteer::bin_cell> cells;
    std::vector<unsigned> lookup;
    gsref_array3d arr;
};

void bin_grid(BinGrid& G, const float ws[3], const unsigned wc[3]) {
    using namespace ref_knn;
    const unsigned X = wc[0], Y = wc[1], Z = wc[2], C = X * Y * Z;
    const float3 worldSize = make_float3(ws[0], ws[1], ws[2]);
    const float3 step = make_float3(ws[0] / X, ws[1] / Y, ws[2] / Z);
    const float3 stepN = make_float3(step.x / ws[0], step.y / ws[1], step.z / ws[2]);
    std::vector<OpenSteer::bin_cell>& cells = G.cells;
    cells.resize(C);
    unsigned index = 0;
    for (size_t iH = 0; iH < Y; iH++)
        for (size_t iD = 0; iD < Z; iD++)
            for (size_t iW = 0; iW < X; iW++) {
                OpenSteer::bin_cell bc;
                bc.index = iW + (iD * X) + (iH * Z * X);
                bc.minBound.x = iW * step.x - 0.5f * ws[0];
                bc.minBound.y = iH * step.y - 0.5f * ws[1];
                bc.minBound.z = iD * step.z - 0.5f * ws[2];
                bc.position.x = bc.minBound.x + 0.5f * step.x;
                bc.position.y = bc.minBound.y + 0.5f * step.y;
                bc.position.z = bc.minBound.z + 0.5f * step.z;
                bc.maxBound.x = bc.minBound.x + step.x;
                bc.maxBound.y = bc.minBound.y + step.y;
                bc.maxBound.z = bc.minBound.z + step.z;
                cells[index++] = bc;
            }
    G.lookup.resize(C);
    for (unsigned z = 0; z < Z; ++z)
        for (unsigned y = 0; y < Y; ++y)
            for (unsigned x = 0; x < X; ++x) G.lookup[x + y * X + z * X * Y] = x + z * X + y * X * Z;
    G.arr = gsref_array3d{G.lookup.data(), X, Y, Z};
    constWorldSizeV2 = worldSize;
    constWorldStepV2 = step;
    constWorldStepNormalizedV2 = stepN;
    constWorldCellsV2 = make_uint3(X, Y, Z);
}
}  // namespace

extern "C" {

// KNNBinDataV2 construction + KNNBinningV2UpdateDBCUDA for both groups +
// KNNBinningV2CUDA::run (KNNBinningV2.cu:192-271).
int gsref_knn_binned(const float* posA4, unsigned nA, const float* posB4, unsigned nB,
                     int self, const float ws[3], const unsigned wc[3], unsigned radius,
                     unsigned k, unsigned* idx_out, float* dist_out) {
    using namespace ref_knn;
    const unsigned X = wc[0], Y = wc[1], Z = wc[2], C = X * Y * Z;
    (void)X;
    (void)Z;
    BinGrid G;
    bin_grid(G, ws, wc);
    std::vector<OpenSteer::bin_cell>& cells = G.cells;
    gsref_array3d& arr = G.arr;

    const bool b3D = Y > 1;
    const unsigned npc = ipow(radius * 2 + 1, b3D ? 3 : 2);
    if (KNN_THREADSPERBLOCK * npc > (1u << 14)) return -1;
    std::vector<uint> neighbors(size_t(C) * npc);
    KNNBinningV2BindTexture(reinterpret_cast<cudaArray*>(&arr));
    launch(blocks(C, KNN_THREADSPERBLOCK), KNN_THREADSPERBLOCK, [&] {
        if (b3D)
            KNNBinningV2ComputeCellNeighbors3D(cells.data(), neighbors.data(), npc, radius, C);
        else
            KNNBinningV2ComputeCellNeighbors2D(cells.data(), neighbors.data(), npc, radius, C);
    });

    BinDB dbA, dbB;
    update_db(dbB, posB4, nB, C);
    BinDB* pA = &dbB;
    if (!self) {
        update_db(dbA, posA4, nA, C);
        pA = &dbA;
    }
    KNNBinningV2UnbindTexture();
    if (2u * TPB * k > (1u << 15)) return -2;
    KNNBinningV2KernelBindTextures(dbB.cellStart.data(), dbB.cellEnd.data(),
                                   dbB.agentSorted.data(), dbB.posSorted.data(), neighbors.data(),
                                   C, nB, npc);
    launch(blocks(nA, TPB), TPB, [&] {
        KNNBinningV2Kernel(pA->posSorted.data(), pA->agentSorted.data(), pA->cellSorted.data(),
                           npc, radius, idx_out, dist_out, k, nA, nB, self != 0);
    });
    KNNBinningV2KernelUnbindTextures();
    return 0;
}

// ExtractData's diagnostics: ComputeCellDensity and ComputeAvgCellVelocity
// (ProcessData.cu:51-128) on the group's database as KNNBinningV2UpdateDBCUDA
// builds it (KNNBinningV2.cu:87-142): cellStart of an empty cell is
// 0xffffffff, pdAgentIndicesSorted is the stable sort's agent order.
// density_out: one count per cell; avg_velocity_out: float3 per cell.
int gsref_cell_diagnostics(const float* pos4, const float* dir4, const float* speed, unsigned n,
                           const float ws[3], const unsigned wc[3], unsigned* density_out,
                           float* avg_velocity_out) {
    const unsigned C = wc[0] * wc[1] * wc[2];
    BinGrid G;
    bin_grid(G, ws, wc);
    BinDB db;
    ref_knn::KNNBinningV2BindTexture(reinterpret_cast<cudaArray*>(&G.arr));
    update_db(db, pos4, n, C);
    ref_knn::KNNBinningV2UnbindTexture();
    launch(blocks(C, TPB), TPB, [&] {
        ref_diag::ComputeCellDensityKernel(db.cellStart.data(), db.cellEnd.data(), density_out, C);
    });
    ref_diag::ComputeAvgCellVelocityBindTextures(f4(dir4), speed, db.agentSorted.data(), n);
    launch(blocks(C, TPB), TPB, [&] {
        ref_diag::ComputeAvgCellVelocityKernel(db.cellStart.data(), db.cellEnd.data(),
                                               f3(avg_velocity_out), n, C);
    });
    ref_diag::ComputeAvgCellVelocityUnbindTextures();
    return 0;
}

// KNNBruteForceCUDAV2::run, KNNBruteForceCUDA.cu:163-187.
int gsref_knn_brute(const float* posA4, unsigned nA, const float* posB4, unsigned nB, int self,
                    unsigned k, unsigned* idx_out, float* dist_out) {
    if (2u * TPB * k > (1u << 15)) return -2;
    launch(blocks(nA, TPB), TPB, [&] {
        ref_brute::KNNBruteForceCUDAKernelV2(f4(posA4), idx_out, dist_out, k, nA, f4(posB4), nB,
                                             self != 0);
    });
    return 0;
}

// SteerForSeparationCUDA::run (SteerForSeparationCUDA.cu:48-97) and the
// cohesion / alignment wrappers built the same way.
void gsref_separation(float* pos4, float* dir4, float* steer4, unsigned* applied, unsigned nA,
                      const unsigned* knn, unsigned k, const float* posB4, unsigned nB,
                      float min_d, float max_d, float cos_max, float w, unsigned mask) {
    ref_sep::SteerForSeparationKernelBindTextures(f4(posB4), nB);
    launch(blocks(nA, TPB), TPB, [&] {
        ref_sep::SteerForSeparationKernel(f4(pos4), f4(dir4), f4(steer4), nA, knn, k, nB, min_d,
                                          max_d, cos_max, w, applied, mask);
    });
    ref_sep::SteerForSeparationKernelUnindTextures();
}
void gsref_cohesion(float* pos4, float* dir4, float* steer4, unsigned* applied, unsigned nA,
                    const unsigned* knn, unsigned k, const float* posB4, unsigned nB, float min_d,
                    float max_d, float cos_max, float w, unsigned mask) {
    ref_coh::SteerForCohesionKernelBindTextures(f4(posB4), nB);
    launch(blocks(nA, TPB), TPB, [&] {
        ref_coh::SteerForCohesionCUDAKernel(f4(pos4), f4(dir4), f4(steer4), nA, knn, k, nB, min_d,
                                            max_d, cos_max, w, applied, mask);
    });
    ref_coh::SteerForCohesionKernelUnindTextures();
}
void gsref_alignment(float* pos4, float* dir4, float* steer4, unsigned* applied, unsigned nA,
                     const unsigned* knn, unsigned k, const float* posB4, const float* dirB4,
                     unsigned nB, float min_d, float max_d, float cos_max, float w,
                     unsigned mask) {
    ref_ali::SteerForAlignmentKernelBindTextures(f4(posB4), f4(dirB4), nB);
    launch(blocks(nA, TPB), TPB, [&] {
        ref_ali::SteerForAlignmentCUDAKernel(f4(pos4), f4(dir4), f4(steer4), nA, knn, k, nB,
                                             min_d, max_d, cos_max, w, applied, mask);
    });
    ref_ali::SteerForAlignmentKernelUnindTextures();
}

// SteerForSeekCUDA::run.
void gsref_seek(float* pos4, float* dir4, float* steer4, unsigned* applied, unsigned n,
                const float target[3], float w, unsigned mask) {
    const float3 t = make_float3(target[0], target[1], target[2]);
    launch(blocks(n, TPB), TPB, [&] {
        ref_seek::SteerForSeekCUDAKernel(f4(steer4), f4(pos4), f4(dir4), t, n, w, applied, mask);
    });
}

// SteerToFollowPathCUDA::run, SteerToFollowPathCUDA.cu:45-81.  The path
// arrays are the PolylinePathwayCUDA members (points/normals float3[n],
// lengths[n]).
void gsref_follow_path(float* pos4, float* dir4, float* speed, float* steer4, unsigned* applied,
                       unsigned n, const float* points3, const float* lengths,
                       const float* normals3, unsigned n_points, float radius, int cyclic,
                       float total_length, float prediction_time, float w, unsigned mask) {
    launch(blocks(n, TPB), TPB, [&] {
        ref_path::FollowPathCUDAKernel(f4(pos4), f4(dir4), speed, f4(steer4), f3(points3), lengths,
                                       f3(normals3), n_points, radius, cyclic != 0, total_length,
                                       prediction_time, n, w, applied, mask);
    });
}

// SteerToAvoidNeighborsCUDA::run, SteerToAvoidNeighborsCUDA.cu:84-166.
void gsref_avoid_neighbors(float* pos4, float* dir4, float* side3, float* speed, float* radius,
                           float* steer4, unsigned* applied, unsigned nA, const unsigned* knn,
                           const float* knn_dist, unsigned k, const float* posB4,
                           const float* dirB4, const float* speedB, const float* radiusB,
                           unsigned nB, float min_time, float min_sep, int avoid_close, float w,
                           unsigned mask) {
    using namespace ref_avoid;
    SteerToAvoidNeighborsKernelBindTextures(f4(posB4), f4(dirB4), speedB, radiusB, nB);
    if (avoid_close) {
        launch(blocks(nA, TPB), TPB, [&] {
            SteerToAvoidCloseNeighborsCUDAKernel(knn, knn_dist, k, f4(pos4), f4(dir4), radius,
                                                 f4(steer4), nA, nB, min_sep, w, applied, mask);
        });
    }
    launch(blocks(nA, TPB), TPB, [&] {
        SteerToAvoidNeighborsCUDAKernel(knn, k, f4(pos4), f4(dir4), f3(side3), radius, speed,
                                        f4(steer4), nA, nB, min_time, w, applied,
                                        mask | KERNEL_AVOID_CLOSE_NEIGHBORS_BIT);
    });
    SteerToAvoidNeighborsKernelUnbindTextures();
}

// AvoidWallsCUDA::run, AvoidWallsCUDA.cu:52-105.
void gsref_avoid_walls(float* pos4, float* dir4, float* side3, float* speed, float* radius,
                       float* steer4, unsigned* applied, unsigned n, const unsigned* knl,
                       unsigned k, const float* start4, const float* end4, const float* normal4,
                       unsigned nLines, float min_time, float w, unsigned mask) {
    using namespace ref_walls;
    SteerToAvoidWallsKernelBindTextures(f4(start4), f4(end4), f4(normal4), nLines);
    launch(blocks(n, TPB), TPB, [&] {
        SteerToAvoidWallsCUDAKernel(f4(pos4), f4(dir4), f3(side3), speed, radius, knl, k, min_time,
                                    f4(steer4), n, nLines, w, applied, mask);
    });
    SteerToAvoidWallsKernelUnbindTextures();
}

// UpdateCUDA::run, UpdateCUDA.cu:75-99.
void gsref_update(float* side3, float* up3, float* dir4, float* pos4, float* steer4, float* speed,
                  const float* maxForce, const float* maxSpeed, const float* mass, float dt,
                  unsigned n, unsigned* applied) {
    launch(blocks(n, TPB), TPB, [&] {
        ref_update::UpdateCUDAKernel(f3(side3), f3(up3), f4(dir4), f4(pos4), f4(steer4), speed,
                                     maxForce, maxSpeed, mass, dt, n, applied);
    });
}

// WrapWorldCUDA::run.
void gsref_wrap(float* pos4, const float ws[3], unsigned n) {
    const float3 w = make_float3(ws[0], ws[1], ws[2]);
    launch(blocks(n, TPB), TPB, [&] { ref_wrap::WrapWorldKernel(f4(pos4), w, n); });
}

// AntiPenetrationAgentsCUDA::run, AntiPenetrationAgentsCUDA.cu:50-100: the
// positions are copied to a second buffer, the kernel writes that buffer and
// it is copied back.
void gsref_antipenetration_agents(float* pos4, const float* radius, unsigned nA,
                                  const unsigned* knn, const float* knn_dist, unsigned k,
                                  const float* posB4, const float* radiusB,
                                  const unsigned* appliedB, unsigned nB, unsigned* applied,
                                  unsigned mask) {
    using namespace ref_antipen;
    std::vector<float4> out(f4(pos4), f4(pos4) + nA);
    AntiPenetrationAgentsKernelBindTextures(f4(posB4), radiusB, appliedB, nB);
    launch(blocks(nA, TPB), TPB, [&] {
        AntiPenetrationAgentsCUDAKernel(f4(pos4), radius, nA, knn, knn_dist, k, nB, out.data(),
                                        applied, mask);
    });
    AntiPenetrationAgentsKernelUnbindTextures();
    std::copy(out.begin(), out.end(), f4(pos4));
}

// UpdateWithAntiPenetrationCUDA::run, UpdateCUDA.cu:125-190 (dynamic shared
// memory k * THREADSPERBLOCK words for the wall list).
int gsref_update_antipen_wall(float* side3, float* up3, float* dir4, float* pos4, float* steer4,
                              float* speed, const float* maxForce, const float* maxSpeed,
                              const float* mass, const float* radius, const unsigned* knl,
                              unsigned k, const float* start4, const float* end4,
                              const float* normal4, unsigned nLines, float dt, unsigned n,
                              unsigned* applied) {
    using namespace ref_update_ap;
    if (TPB * k > (1u << 14)) return -1;
    UpdateCUDAKernelBindTextures(f4(start4), f4(end4), f4(normal4), nLines);
    launch(blocks(n, TPB), TPB, [&] {
        UpdateCUDAKernelNew(f3(side3), f3(up3), f4(dir4), f4(pos4), f4(steer4), speed, maxForce,
                            maxSpeed, mass, radius, knl, k, nLines, dt, n, applied);
    });
    UpdateCUDAKernelUnbindTextures();
    return 0;
}

// AntiPenetrationWALLCUDA::run, AntiPenetrationWallCUDA.cu:45-87.
int gsref_antipenetration_wall(const float* pos4, float* dir4, const float* speed,
                               const unsigned* knl, unsigned k, const float* start4,
                               const float* end4, const float* normal4, unsigned nLines,
                               float dt, unsigned n, unsigned* applied) {
    using namespace ref_antipen_wall;
    if (TPB * k > (1u << 14)) return -1;
    AntiPenetrationWallKernelBindTextures(f4(start4), f4(end4), f4(normal4), nLines);
    launch(blocks(n, TPB), TPB, [&] {
        AntiPenetrationWallKernel(f4(pos4), f4(dir4), speed, knl, k, dt, n, nLines, applied);
    });
    AntiPenetrationWallKernelUnbindTextures();
    return 0;
}

}  // extern "C"
