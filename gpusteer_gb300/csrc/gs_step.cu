// The fused per-step engine.
//
// State lives in bucketed order in two ping-pong sets of six float4 streams
// (Fused A and B, layout in gs_internal.cuh).  One step is
//   scan      exclusive scan of the per-cell counts gathered by the previous
//             step (or by fused_from_reference), zeroing the counts, over the
//             cells near agents (the counting also keeps per-tile totals);
//   permute   A -> B into bucketed order, applying the world wrap
//             (WrapWorldCUDAKernel) on the way;
//   fused     one thread per agent of B: binned KNN over B's own bucketed
//             positions into a register k-list, one pass over the k
//             neighbours feeding every enabled behaviour's accumulator, the
//             behaviours finalised in the scenario's order with the
//             reference's masks, UpdateCUDAKernel's integration, the new state
//             written to A, and the next step's cell counted with an atomic.
// With wall avoidance the fused kernel splits in two at the wall behaviour,
// because avoid-walls moves agents (AvoidWallsCUDAKernel.cu:215-224) before
// later behaviours read their neighbours: the first half writes the corrected
// position/direction of every agent, the second half reads neighbours from
// those.
//
// This replaces, per step, the reference's wrap, BuildDB, host sync, thrust
// sort, memset, ReorderDB, KNN and one launch per behaviour plus update
// (plugins/BoidsGroup.cpp:606-637, plugins/ChokePointNew.cpp:586-630).
#include "gs_behaviours.cuh"
#include "gs_knn.cuh"
#include "gs_scan.cuh"
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>

#include "gs_launch.h"

namespace gs {

__device__ __forceinline__ unsigned u(float x) { return __float_as_uint(x); }
__device__ __forceinline__ float fb(unsigned x) { return __uint_as_float(x); }

// Adds 1 to the scan tile total of `cell`, once per group of active lanes in
// the same tile (a warp's agents are mostly in one).
__device__ __forceinline__ void add_to_tile(unsigned* tile, unsigned cell) {
    const unsigned t = cell / kScanTile;
    const unsigned peers = __match_any_sync(__activemask(), t);
    if ((threadIdx.x & 31u) == unsigned(__ffs(int(peers)) - 1))
        atomicAdd(tile + t, unsigned(__popc(int(peers))));
}

// The agent's cell for the next step's counting sort: counted (the old count
// is its rank in the cell) and, given tile totals (tile not null), added to
// its tile's total.
__device__ __forceinline__ unsigned count_next(const Scene& sc, V3 pos, int wrap_mode,
                                               unsigned* count, unsigned* tile, unsigned& cell) {
    const V3 wp = wrap_world(pos, sc.grid.ws, wrap_mode);
    cell = sc.cell_offset + cell_of(sc.grid, wp);
    if (tile) add_to_tile(tile, cell);
    return atomicAdd(count + cell, 1u);
}

// Reference layout -> A (identity order), counting the first step's cells.
__global__ void k_from_reference(GroupView g, const unsigned* __restrict__ agent_scene,
                                 const Scene* __restrict__ scenes, Fused A,
                                 uint2* __restrict__ cellrank, unsigned* __restrict__ count,
                                 int wrap_mode, int dirty) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    const unsigned si = agent_scene ? agent_scene[i] : 0u;
    const Scene sc = scenes[si];
    const unsigned id = i - sc.agent_offset;
    const float4 p = g.position[i], d = g.direction[i];
    const float3 sd = g.side[i], up = g.up[i];
    A.f[0][i] = make_float4(p.x, p.y, p.z, fb(id));
    A.f[1][i] = make_float4(d.x, d.y, d.z, g.speed[i]);
    A.f[2][i] = make_float4(sd.x, sd.y, sd.z, g.radius[i]);
    A.f[3][i] = make_float4(up.x, up.y, up.z, g.mass[i]);
    A.f[4][i] = make_float4(g.max_speed[i], g.max_force[i], fb(g.applied[i]), fb(si));
    if (dirty) A.f[5][i] = g.steering[i];
    unsigned cell;
    const unsigned rank = count_next(sc, v3(p), wrap_mode, count, nullptr, cell);
    cellrank[i] = make_uint2(cell, rank);
}

gs_status fused_from_reference(GroupView g, const unsigned* agent_scene, const Scene* scenes,
                               Fused A, uint2* cellrank, unsigned* count, int wrap_mode,
                               bool dirty, cudaStream_t st) {
    if (g.n == 0) return GS_OK;
    k_from_reference<<<blocks_for(g.n), kBlock, 0, st>>>(g, agent_scene, scenes, A, cellrank,
                                                         count, wrap_mode, dirty ? 1 : 0);
    GS_LAUNCHED("fused_from_reference");
    return GS_OK;
}

__global__ void k_recount(Fused A, unsigned n, const Scene* __restrict__ scenes,
                          uint2* __restrict__ cellrank, unsigned* __restrict__ count,
                          int wrap_mode) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Scene sc = scenes[u(A.f[4][i].w)];
    unsigned cell;
    const unsigned rank = count_next(sc, v3(A.f[0][i]), wrap_mode, count, nullptr, cell);
    cellrank[i] = make_uint2(cell, rank);
}

gs_status fused_recount(Fused A, unsigned n, const Scene* scenes, uint2* cellrank,
                        unsigned* count, int wrap_mode, cudaStream_t st) {
    if (n == 0) return GS_OK;
    k_recount<<<blocks_for(n), kBlock, 0, st>>>(A, n, scenes, cellrank, count, wrap_mode);
    GS_LAUNCHED("fused_recount");
    return GS_OK;
}

// A (slot i) -> B (slot dst), wrapping the position.
__device__ __forceinline__ void move_agent(const Fused& A, const Fused& B,
                                           const Scene* __restrict__ scenes, int wrap_mode,
                                           int dirty, unsigned i, unsigned dst) {
    const float4 f0 = A.f[0][i];
    const float4 f4v = A.f[4][i];
    const Scene sc = scenes[u(f4v.w)];
    const V3 wp = wrap_world(v3(f0), sc.grid.ws, wrap_mode);
    B.f[0][dst] = make_float4(wp.x, wp.y, wp.z, f0.w);
    B.f[1][dst] = A.f[1][i];
    B.f[2][dst] = A.f[2][i];
    B.f[3][dst] = A.f[3][i];
    B.f[4][dst] = f4v;
    if (dirty) B.f[5][dst] = A.f[5][i];
}

// A (slot i) -> B (slot start[cell] + rank), wrapping the position.
__device__ __forceinline__ void permute_agent(const Fused& A, const Fused& B, unsigned n,
                                              const uint2* __restrict__ cellrank,
                                              const unsigned* __restrict__ start,
                                              const Scene* __restrict__ scenes, int wrap_mode,
                                              int dirty, unsigned* __restrict__ err, unsigned i) {
    const uint2 cr = cellrank[i];
    const unsigned dst = start[cr.x] + cr.y;
    if (dst >= n) {  // inconsistent counts: record and write nothing
        atomicOr(err, kErrCounts);
        return;
    }
    move_agent(A, B, scenes, wrap_mode, dirty, i, dst);
}

__global__ void __launch_bounds__(kBlock) k_permute(Fused A, Fused B, unsigned n,
                                                    const uint2* __restrict__ cellrank,
                                                    const unsigned* __restrict__ start,
                                                    const Scene* __restrict__ scenes,
                                                    int wrap_mode, int dirty,
                                                    unsigned* __restrict__ err,
                                                    unsigned* __restrict__ retry_count,
                                                    unsigned* __restrict__ tile, unsigned tiles) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *retry_count = 0u;  // the fused launch that follows refills it
    // the scan has read the tile totals; the step's counting adds them anew
    for (unsigned t = i; t < tiles; t += gridDim.x * blockDim.x) tile[t] = 0u;
    if (i >= n) return;
    permute_agent(A, B, n, cellrank, start, scenes, wrap_mode, dirty, err, i);
}

// The first step after an upload finds A in agent order, which
// is a shuffle of the bucket order: there the scatter above stores each
// agent's five float4 to scattered slots (partial-sector writes, about five
// times the steady step's permute).  Instead, one scattered 4-byte store per
// agent records which agent each slot takes, and the permute gathers:
// scattered 16-byte reads, coalesced writes.
__global__ void k_agent_at(unsigned n, const uint2* __restrict__ cellrank,
                           const unsigned* __restrict__ start, unsigned* __restrict__ err,
                           unsigned* __restrict__ agent_at) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint2 cr = cellrank[i];
    const unsigned dst = start[cr.x] + cr.y;
    if (dst >= n) {  // inconsistent counts: record and write nothing
        atomicOr(err, kErrCounts);
        return;
    }
    agent_at[dst] = i;
}

__global__ void __launch_bounds__(kBlock) k_permute_gather(Fused A, Fused B, unsigned n,
                                                           const unsigned* __restrict__ agent_at,
                                                           const Scene* __restrict__ scenes,
                                                           int wrap_mode, int dirty,
                                                           unsigned* __restrict__ err,
                                                           unsigned* __restrict__ retry_count,
                                                           unsigned* __restrict__ tile,
                                                           unsigned tiles) {
    const unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) *retry_count = 0u;
    for (unsigned t = s; t < tiles; t += gridDim.x * blockDim.x) tile[t] = 0u;
    if (s >= n) return;
    // with consistent counts every slot below n was written just before;
    // a slot left over from inconsistent ones (the error bit is set) may hold
    // any word, so the index is checked before the reads
    const unsigned i = agent_at[s];
    if (i >= n) {
        atomicOr(err, kErrCounts);
        return;
    }
    move_agent(A, B, scenes, wrap_mode, dirty, i, s);
}

gs_status fused_permute(const FusedLaunch& L, int wrap_mode, bool dirty, bool fresh,
                        cudaStream_t st) {
    if (L.n == 0) return GS_OK;
    if (fresh) {
        k_agent_at<<<blocks_for(L.n), kBlock, 0, st>>>(L.n, L.cellrank, L.start, L.err,
                                                        L.agent_at);
        k_permute_gather<<<blocks_for(L.n), kBlock, 0, st>>>(L.A, L.B, L.n, L.agent_at, L.scenes,
                                                             wrap_mode, dirty ? 1 : 0, L.err,
                                                             L.retry_count, L.tile, L.tiles);
        GS_LAUNCHED("fused_permute");
        return GS_OK;
    }
    k_permute<<<blocks_for(L.n), kBlock, 0, st>>>(L.A, L.B, L.n, L.cellrank, L.start, L.scenes,
                                                  wrap_mode, dirty ? 1 : 0, L.err, L.retry_count,
                                                  L.tile, L.tiles);
    GS_LAUNCHED("fused_permute");
    return GS_OK;
}

// Neighbour accumulators of every behaviour that reads the KNN list.
struct Accs {
    FlockAcc sep, ali, coh;
    AvoidLite avoid;
    CloseAcc close;
};

// `need` is p.need, or a compile-time mask equal to it in a kernel
// specialised for one configuration (the unused accumulators then vanish).
// gs, ga, gc: the agent's angle gates of the three flocking behaviours.
// offset = bpos - me.pos and dsq = dot(offset, offset), computed by the caller.
__device__ __forceinline__ void accumulate_at(Accs& a, const StepDev& p, unsigned need,
                                              const FlockParams& fs, const FlockParams& fa,
                                              const FlockParams& fc, AngleGate gs_, AngleGate ga,
                                              AngleGate gc, const Self& me, unsigned rank,
                                              float knn_d, V3 offset, float dsq, V3 bpos,
                                              V3 bdir, float bspeed, float bradius) {
    if (need & (NEED_SEP | NEED_ALI | NEED_COH)) {
        // inBoidNeighborhood (FlockingCommon.cuh:4-30) for the three flocking
        // behaviours, without its square root and divisions where they cannot
        // change the outcome: d < min and d > max are compared as squared
        // distances against exact thresholds, and the angle test is decided
        // from dot(dir, offset) unless it lies within the gate's margin (then
        // the reference's unit offset and dot decide, computed once for all
        // three, as they are the same operands).
        const bool lt_s = (need & NEED_SEP) && dsq < fs.lt;
        const bool lt_a = (need & NEED_ALI) && dsq < fa.lt;
        const bool lt_c = (need & NEED_COH) && dsq < fc.lt;
        const bool ang_s = (need & NEED_SEP) && !lt_s && !(dsq > fs.gt);
        const bool ang_a = (need & NEED_ALI) && !lt_a && !(dsq > fa.gt);
        const bool ang_c = (need & NEED_COH) && !lt_c && !(dsq > fc.gt);
        bool in_s = lt_s, in_a = lt_a, in_c = lt_c;
        if (ang_s || ang_a || ang_c) {
            const float g = dot(me.dir, offset), de = d_estimate(dsq);
            const int ds = ang_s ? angle_decide(g, de, fs.cos_max, gs_) : 0;
            const int da = ang_a ? angle_decide(g, de, fa.cos_max, ga) : 0;
            const int dc = ang_c ? angle_decide(g, de, fc.cos_max, gc) : 0;
            if ((ds | da | dc) < 0) {
                const float fwd = forward_component(me.dir, offset, dsq);
                in_s = in_s || (ds < 0 ? fwd > fs.cos_max : ds > 0);
                in_a = in_a || (da < 0 ? fwd > fa.cos_max : da > 0);
                in_c = in_c || (dc < 0 ? fwd > fc.cos_max : dc > 0);
            } else {
                in_s = in_s || ds > 0;
                in_a = in_a || da > 0;
                in_c = in_c || dc > 0;
            }
        }
        if (need & NEED_SEP) {
            if (in_s) {
                a.sep.sum = add(a.sep.sum, dvd(offset, -dsq));
                a.sep.n++;
            }
        }
        if (need & NEED_ALI) {
            if (in_a) {
                a.ali.sum = add(a.ali.sum, bdir);
                a.ali.n++;
            }
        }
        if (need & NEED_COH) {
            if (in_c) {
                a.coh.sum = add(a.coh.sum, bpos);
                a.coh.n++;
            }
        }
    }
    if (need & NEED_AVOID) avoid_lite_add(a.avoid, me, rank, bpos, bdir, bspeed, bradius);
    // the KNN distance equals d unless the neighbour moved after the KNN
    // (avoid-walls); the caller passes it then, else -1
    if (need & NEED_CLOSE)
        close_add(a.close, me, p.min_sep, knn_d < 0.f ? sqrtf(dsq) : knn_d, bpos, bradius);
}

__device__ __forceinline__ void accumulate(Accs& a, const StepDev& p, unsigned need,
                                           const FlockParams& fs, const FlockParams& fa,
                                           const FlockParams& fc, AngleGate gs_, AngleGate ga,
                                           AngleGate gc, const Self& me, unsigned rank,
                                           float knn_d, V3 bpos, V3 bdir, float bspeed,
                                           float bradius) {
    const V3 offset = sub(bpos, me.pos);
    accumulate_at(a, p, need, fs, fa, fc, gs_, ga, gc, me, rank, knn_d, offset,
                  dot(offset, offset), bpos, bdir, bspeed, bradius);
}

// The rest phase's per-neighbour arithmetic with the x and y components in
// packed f32x2 subtracts and multiplies (elementwise, rounded to nearest, not
// contracted: the same operations in the same order, so the same bits).
struct PackedSelf {
    unsigned long long pos_xy, vel_xy;  // me.pos.xy, me.dir.xy * me.speed
    float vel_z;
};
__device__ __forceinline__ PackedSelf packed_self(const Self& me) {
    PackedSelf q;
    q.pos_xy = pack_xy(me.pos.x, me.pos.y);
    q.vel_xy = packed_mul(pack_xy(me.dir.x, me.dir.y), pack_xy(me.speed, me.speed));
    q.vel_z = me.dir.z * me.speed;
    return q;
}
// offset = bpos - me.pos (x and y also packed, in o_xy) and dot(offset, offset)
__device__ __forceinline__ float packed_offset(const PackedSelf& q, const Self& me, float4 b0,
                                               V3& off, unsigned long long& o_xy) {
    o_xy = packed_sub(pack_xy(b0.x, b0.y), q.pos_xy);
    unpack_xy(o_xy, off.x, off.y);
    off.z = b0.z - me.pos.z;
    float sx, sy;
    unpack_xy(packed_mul(o_xy, o_xy), sx, sy);
    return (sx + sy) + off.z * off.z;
}
// The avoidance pre-test (avoid_time_window_test) for rp = me.pos - bpos =
// -offset: h = dot(rv, rp) is -dot(rv, offset) and S the same sum of
// magnitudes (negation is exact; only the sign of a zero h can differ, which
// the comparisons do not see).
__device__ __forceinline__ bool packed_avoid_time_may_fall_in(const PackedSelf& q,
                                                              unsigned long long o_xy,
                                                              float off_z, float min_t,
                                                              float4 b1) {
    const unsigned long long rv_xy =
        packed_sub(packed_mul(pack_xy(b1.x, b1.y), pack_xy(b1.w, b1.w)), q.vel_xy);
    const float rv_z = b1.z * b1.w - q.vel_z;
    float sx, sy, hx, hy;
    unpack_xy(packed_mul(rv_xy, rv_xy), sx, sy);
    unpack_xy(packed_mul(rv_xy, o_xy), hx, hy);
    const float hz = rv_z * off_z;
    const float ss = (sx + sy) + rv_z * rv_z;
    const float h = -((hx + hy) + hz);
    const float S = (fabsf(hx) + fabsf(hy)) + fabsf(hz);
    return avoid_time_window_test(ss, h, S, min_t);
}

// Behaviours order[first..] in order, then nothing else.  fetch(rank, pos,
// dir, speed) reads neighbour list entry `rank` again (neighbour avoidance).
// A runtime loop over the packed order (3 bits per entry), so each
// behaviour's code appears once in the kernel rather than once per order
// slot; `need` drops the code of behaviours a specialised kernel never runs.
template <class Fetch>
__device__ __forceinline__ void finish_all(const Accs& a, const StepDev& p, unsigned need,
                                           unsigned first, const FlockParams& fs,
                                           const FlockParams& fa, const FlockParams& fc,
                                           const Self& me, unsigned& applied, V3& steer,
                                           Fetch&& fetch) {
#pragma unroll 1
    for (unsigned o = first; o < p.n_order; ++o) {
        switch ((p.order_packed >> (3u * o)) & 7u) {
            case GS_B_SEPARATION:
                if (need & NEED_SEP) flock_finish(0, a.sep, fs, me, applied, steer);
                break;
            case GS_B_ALIGNMENT:
                if (need & NEED_ALI) flock_finish(1, a.ali, fa, me, applied, steer);
                break;
            case GS_B_COHESION:
                if (need & NEED_COH) flock_finish(2, a.coh, fc, me, applied, steer);
                break;
            case GS_B_SEEK:
                seek_finish(v3(p.seek_target[0], p.seek_target[1], p.seek_target[2]), p.w_seek,
                            p.mask_seek, me, applied, steer);
                break;
            case GS_B_AVOID_NEIGHBORS:
                if (need & NEED_AVOID) {
                    if (p.avoid_close)
                        close_finish(a.close, p.w_avoid, p.mask_avoid, applied, steer);
                    avoid_finish(avoid_lite_full(a.avoid, fetch), p.w_avoid, p.mask_avoid, me,
                                 applied, steer);
                }
                break;
            case GS_B_FOLLOW_PATH:
                follow_path_finish(p.path, p.path_time, p.w_path, p.mask_path, me, applied, steer);
                break;
            default: break;
        }
    }
}

__device__ __forceinline__ void init_accs(Accs& a, const StepDev& p) {
    flock_init(a.sep);
    flock_init(a.ali);
    flock_init(a.coh);
    avoid_lite_init(a.avoid, p.min_time_col);
    close_init(a.close);
}

__device__ __forceinline__ void store_next(const FusedLaunch& L, unsigned s, const Self& me,
                                           unsigned id, unsigned scene, const Scene& sc,
                                           int wrap_mode) {
    // the cell count's atomic first: its round trip overlaps the state stores
    unsigned cell;
    const unsigned rank = count_next(sc, me.pos, wrap_mode, L.count, L.tile, cell);
    L.A.f[0][s] = make_float4(me.pos.x, me.pos.y, me.pos.z, fb(id));
    L.A.f[1][s] = make_float4(me.dir.x, me.dir.y, me.dir.z, me.speed);
    L.A.f[2][s] = make_float4(me.side.x, me.side.y, me.side.z, me.radius);
    L.A.f[3][s] = make_float4(me.up.x, me.up.y, me.up.z, me.mass);
    L.A.f[4][s] = make_float4(me.max_speed, me.max_force, fb(0u), fb(scene));
    L.cellrank[s] = make_uint2(cell, rank);
}

// The scene number alone (f4.w): the KNN needs position, index and scene;
// the rest of the state is loaded after it, so it is not held in registers
// through the scan.
__device__ __forceinline__ unsigned load_scene(const Fused& B, unsigned s) {
    return __float_as_uint(reinterpret_cast<const float*>(B.f[4] + s)[3]);
}

// Everything but position and index, after the KNN.
__device__ __forceinline__ Self load_rest(const Fused& B, unsigned s, V3 pos, float4& f4v) {
    const float4 f1 = B.f[1][s], f2 = B.f[2][s], f3 = B.f[3][s];
    f4v = B.f[4][s];
    Self me;
    me.pos = pos;
    me.dir = v3(f1);
    me.speed = f1.w;
    me.side = v3(f2);
    me.radius = f2.w;
    me.up = v3(f3);
    me.mass = f3.w;
    me.max_speed = f4v.x;
    me.max_force = f4v.y;
    return me;
}

// ---- KNN of one agent (fast path, or exact redo) ----------------------------------
// The exact (distance, index) list of one agent out of line: the collecting
// scan's kernels call it for the rare agents whose fast scan could not vouch
// for its order (or overflowed the tables), so its 64-bit list takes neither
// registers nor instruction cache from the common path.
template <int KMAX>
static __device__ __noinline__ void knn_exact_out_of_line(int k, V3 p, unsigned self_id,
                                                          const Grid& g, Box b,
                                                          unsigned cell_offset,
                                                          const unsigned* __restrict__ start,
                                                          const float4* __restrict__ pos_id,
                                                          unsigned* col, unsigned stride) {
    knn_neighbours_exact<KMAX>(k, p, self_id, g, b, cell_offset, start, pos_id, col, stride);
}

// Writes the agent's neighbour slots in (distance, index) order to its shared
// column: at col[(ENUM + r) * bd] on the collecting scan's fast path,
// col[r * bd] otherwise; returns the column offset of entry 0.  After the
// collecting scan (sparse boxes: a few agents per step give up, mostly
// distance ties) the agent is redone inline; after the streaming scan it is
// appended to the retry list for the warp-per-agent search and the redo
// launch, and UINT_MAX is returned.
template <int KMAX, unsigned ENUM, bool EXACT, bool FLAT>
__device__ __forceinline__ unsigned agent_knn(const FusedLaunch& L, const StepDev& p, unsigned s,
                                              unsigned it, V3 pos, unsigned id, const Scene& sc,
                                              const Box& box, unsigned* col, unsigned bd) {
    if (EXACT) {
        // redo entry `it`: the list the warp-per-agent search stored, else a
        // search by this thread
        if (it < L.retry_cap) {
            const unsigned* pre = L.retry_knn + size_t(it) * kRetryListK;
            if (pre[0] != kRetryNotListed) {
                for (unsigned r = 0; r < p.k; ++r) col[r * bd] = pre[r];
                return 0;
            }
        }
        knn_neighbours_exact<KMAX>(int(p.k), pos, id, sc.grid, box, sc.cell_offset, L.start,
                                   L.B.f[0], col, bd);
        return 0;
    }
    if constexpr (ENUM > 64) {
        // crowded boxes: streaming scan, result at col[r * bd]
        constexpr unsigned EBITS = ENUM >= 256 ? 8u : 7u;
        if (knn_neighbours_stream<KMAX, EBITS, FLAT>(int(p.k), pos, id, sc.grid, box, sc.cell_offset,
                                               L.start, L.B.f[0], col, bd))
            return 0;
    } else {
        if (knn_neighbours_fast<KMAX, ENUM>(int(p.k), pos, id, sc.grid, box, sc.cell_offset,
                                            L.start, L.B.f[0], col, col + ENUM * bd, bd))
            return ENUM;
        knn_exact_out_of_line<KMAX>(int(p.k), pos, id, sc.grid, box, sc.cell_offset, L.start,
                                    L.B.f[0], col, bd);
        atomicAdd(L.retry_count, 1u);  // counted (gs_group_exact_redos), not listed
        return 0;
    }
    L.retry[atomicAdd(L.retry_count, 1u)] = s;
    return UINT_MAX;
}

// Agents handled by one thread: slot `it` of the launch (fast path), or the
// it-th entry of the retry list (exact path, grid-stride).
// The exact launch numbers its threads block-fastest (thread t of block b is
// it = t * gridDim.x + b), so the few hundred agents of a typical retry list
// land one or two per block across every SM instead of filling the first
// blocks: the redo then takes one agent's latency, not a queue of them.
template <bool EXACT>
__device__ __forceinline__ unsigned first_agent() {
    return EXACT ? threadIdx.x * gridDim.x + blockIdx.x : blockIdx.x * blockDim.x + threadIdx.x;
}

template <bool EXACT>
__device__ __forceinline__ bool next_agent(const FusedLaunch& L, unsigned& it, unsigned& s) {
    if (!EXACT) {
        s = it;
        return it < L.n;
    }
    if (it >= *L.retry_count) return false;
    s = L.retry[it];
    return true;
}

// ---- exact redo: one warp per agent ------------------------------------------------
// The exact (distance, index) list of each redo entry, found by a whole warp:
// the lanes compute the 64-bit keys of the box's candidates side by side
// (row by row, 32 candidates at a time) into a per-warp shared table, then
// k rounds of a warp arg-min take the smallest key left and retire it.  The
// list equals knn_neighbours_exact's: the keys are unique (distinct agent
// indices), a candidate is listed only below KEY_EMPTY, the agent itself is
// skipped, and empty ranks hold UINT_MAX.  A redo entry costs a few
// arg-min rounds of latency instead of one thread's serial pass over every
// candidate.  Launched after the streaming scan only (crowded boxes, where
// the serial pass is long).
constexpr unsigned kRetryWarpKeys = 256;

// The warp's entries e = first, first + stride, ...; keys / slots: the
// warp's kRetryWarpKeys-entry shared tables.  TO_SLOTS: the step with
// avoid-walls, whose wall phase finished every agent but the redo agents'
// lists (avoid-walls does not read the agent's own neighbours): each list
// goes straight to knn_slot (and its KNN distances to knn_dist when
// avoid-close-neighbours reads them), and lane 0 searches an entry of more
// than kRetryWarpKeys candidates itself, so no redo launch follows.
// Otherwise the first retry_cap entries' lists go to retry_knn for the redo
// launch.
template <int KMAX, bool TO_SLOTS>
__device__ __forceinline__ void retry_lists(const FusedLaunch& L, const StepDev& p, unsigned first,
                                            unsigned stride, unsigned long long* keys,
                                            unsigned* slots) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned count = TO_SLOTS ? *L.retry_count : min(*L.retry_count, L.retry_cap);
    for (unsigned e = first; e < count; e += stride) {
        const unsigned s = L.retry[e];
        const float4 f0 = L.B.f[0][s];
        const V3 pos = v3(f0);
        const unsigned id = u(f0.w);
        const Scene sc = L.scenes[load_scene(L.B, s)];
        unsigned ix, iy, iz;
        cell_coords(sc.grid, pos, ix, iy, iz);
        const Box b = cell_box(sc.grid, ix, iy, iz, p.r);
        unsigned total = 0;
        for (unsigned cy = b.y0; cy <= b.y1; ++cy) {
            for (unsigned cz = b.z0; cz <= b.z1; ++cz) {
                const unsigned c0 = sc.cell_offset + cell_label(sc.grid, b.x0, cy, cz);
                const unsigned c1 = sc.cell_offset + cell_label(sc.grid, b.x1, cy, cz) + 1;
                const unsigned s0 = L.start[c0], len = L.start[c1] - s0;
                for (unsigned t = lane; t < len; t += 32) {
                    const unsigned j = total + t;
                    if (j < kRetryWarpKeys) {
                        const float4 q = L.B.f[0][s0 + t];
                        const unsigned qid = u(q.w);
                        keys[j] = qid == id ? ~0ull : knn_key(distance(pos, v3(q)), qid);
                        slots[j] = s0 + t;
                    }
                }
                total += len;
            }
        }
        __syncwarp();
        unsigned* out = TO_SLOTS ? nullptr : L.retry_knn + size_t(e) * kRetryListK;
        const bool dists = TO_SLOTS && (p.need & NEED_CLOSE);
        if (total > kRetryWarpKeys) {
            if (lane == 0) {
                if (TO_SLOTS) {
                    // the exact list into the warp's slot table, then out
                    knn_neighbours_exact<KMAX>(int(p.k), pos, id, sc.grid, b, sc.cell_offset,
                                               L.start, L.B.f[0], slots, 1u);
                    for (unsigned r = 0; r < p.k; ++r) {
                        const unsigned bs = slots[r];
                        L.knn_slot[size_t(r) * L.n + s] = bs;
                        if (dists)
                            L.knn_dist[size_t(r) * L.n + s] =
                                bs == UINT_MAX ? FLT_MAX : distance(pos, v3(L.B.f[0][bs]));
                    }
                } else {
                    out[0] = kRetryNotListed;
                }
            }
            __syncwarp();
            continue;
        }
        for (unsigned r = 0; r < p.k; ++r) {
            unsigned long long best = ~0ull;
            unsigned bj = 0;
            for (unsigned j = lane; j < total; j += 32) {
                const unsigned long long kk = keys[j];
                if (kk < best) {
                    best = kk;
                    bj = j;
                }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, off);
                const unsigned oj = __shfl_xor_sync(0xffffffffu, bj, off);
                if (ob < best) {
                    best = ob;
                    bj = oj;
                }
            }
            // every lane holds the same (best, bj): the keys are unique
            const bool listed = best < KEY_EMPTY;
            if (lane == 0) {
                const unsigned bs = listed ? slots[bj] : UINT_MAX;
                if (TO_SLOTS) {
                    L.knn_slot[size_t(r) * L.n + s] = bs;
                    if (dists) L.knn_dist[size_t(r) * L.n + s] = listed ? key_dist(best) : FLT_MAX;
                } else {
                    out[r] = bs;
                }
                if (listed) keys[bj] = ~0ull;
            }
            __syncwarp();
        }
    }
}

template <int KMAX, bool TO_SLOTS>
__global__ void __launch_bounds__(kBlock) k_knn_retry(FusedLaunch L, StepDev p) {
    __shared__ unsigned long long sk[kBlock / 32][kRetryWarpKeys];
    __shared__ unsigned ss[kBlock / 32][kRetryWarpKeys];
    const unsigned w = threadIdx.x >> 5;
    // warp w of block b takes entries w * gridDim.x + b, + nw, ...: a few
    // hundred entries land one per block across every SM
    retry_lists<KMAX, TO_SLOTS>(L, p, w * gridDim.x + blockIdx.x,
                                gridDim.x * (blockDim.x >> 5), sk[w], ss[w]);
}

// ---- whole step without walls -------------------------------------------------------
constexpr unsigned kNbrChunk = 1;  // measured best for the flock (2: +2.5 %, 4: +9 %)
constexpr unsigned kRestChunk = 2;  // the rest phase's (1: +7 %, 3: +6 %, 4: +12 %; spills)

// NEEDC: the behaviours that read the neighbour list, fixed at compile time
// (kNeedRuntime: taken from p.need).
constexpr unsigned kNeedRuntime = ~0u;
constexpr unsigned kNeedList = NEED_SEP | NEED_ALI | NEED_COH | NEED_AVOID | NEED_CLOSE;
template <int KMAX, unsigned ENUM, bool EXACT, unsigned NEEDC = kNeedRuntime, bool FLAT = false>
__global__ void __launch_bounds__(kBlock, 3) k_fused(FusedLaunch L, StepDev p) {
    const unsigned need = NEEDC == kNeedRuntime ? p.need : NEEDC;
    extern __shared__ unsigned sh_col[];
    const unsigned bd = blockDim.x;
    unsigned* col = sh_col + threadIdx.x;
    const unsigned step = EXACT ? gridDim.x * blockDim.x : 0u;
    for (unsigned it = first_agent<EXACT>();; it += step) {
        unsigned s;
        if (!next_agent<EXACT>(L, it, s)) return;
        const float4 f0 = L.B.f[0][s];
        const V3 pos = v3(f0);
        const unsigned id = u(f0.w), scene = load_scene(L.B, s);
        const Scene sc = L.scenes[scene];
        unsigned ix, iy, iz;
        cell_coords(sc.grid, pos, ix, iy, iz);
        const Box box = cell_box(sc.grid, ix, iy, iz, p.r);
        const unsigned base = agent_knn<KMAX, ENUM, EXACT, FLAT>(L, p, s, it, pos, id, sc, box, col, bd);
        if (base == UINT_MAX) return;
        const bool need_dir = need & (NEED_ALI | NEED_AVOID);
        const bool need_rad = need & (NEED_AVOID | NEED_CLOSE);
        // the neighbour pass reads position, heading, speed and radius; the
        // rest of the state is loaded after it, so it is not held through it
        Self me;
        me.pos = pos;
        {
            const float4 f1 = L.B.f[1][s];
            me.dir = v3(f1);
            me.speed = f1.w;
            me.radius = need_rad ? reinterpret_cast<const float*>(L.B.f[2] + s)[3] : 0.f;
        }
        const FlockParams fs = flock_params(p.sep, p.sep_dsq), fa = flock_params(p.ali, p.ali_dsq),
                          fc = flock_params(p.coh, p.coh_dsq);
        const AngleGate gs_ = angle_gate(me.dir, fs.cos_max), ga = angle_gate(me.dir, fa.cos_max),
                        gc = angle_gate(me.dir, fc.cos_max);
        Accs a;
        init_accs(a, p);
        unsigned* rec_knn = L.rec_knn ? L.rec_knn + size_t(id) * p.k : nullptr;
        unsigned r = 0;
        // Neighbours kNbrChunk at a time: their loads are issued together, so
        // the pass waits on a chunk's gathers once instead of on every
        // neighbour's.  The list is filled from rank 0, so the first empty
        // entry ends it; accumulation stays in list order.
        for (bool more = true; more && r < p.k;) {
            unsigned bs[kNbrChunk];
            float4 b0[kNbrChunk], b1[kNbrChunk];
            float br[kNbrChunk];
#pragma unroll
            for (unsigned j = 0; j < kNbrChunk; ++j)
                bs[j] = r + j < p.k ? col[(base + r + j) * bd] : UINT_MAX;
#pragma unroll
            for (unsigned j = 0; j < kNbrChunk; ++j) {
                const bool ok = bs[j] != UINT_MAX;
                b0[j] = ok ? L.B.f[0][bs[j]] : make_float4(0.f, 0.f, 0.f, 0.f);
                b1[j] = ok && need_dir ? L.B.f[1][bs[j]] : make_float4(0.f, 0.f, 0.f, 0.f);
                br[j] = ok && need_rad ? reinterpret_cast<const float*>(L.B.f[2] + bs[j])[3] : 0.f;
            }
#pragma unroll
            for (unsigned j = 0; j < kNbrChunk; ++j) {
                if (bs[j] == UINT_MAX) {
                    more = false;
                    break;
                }
                if (rec_knn) rec_knn[r] = u(b0[j].w);
                accumulate(a, p, need, fs, fa, fc, gs_, ga, gc, me, r, -1.f, v3(b0[j]), v3(b1[j]),
                           b1[j].w, br[j]);
                ++r;
            }
        }
        if (rec_knn) {
            for (; r < p.k; ++r) rec_knn[r] = UINT_MAX;
            L.rec_pos[id] = make_float4(me.pos.x, me.pos.y, me.pos.z, me.speed);
            L.rec_dir[id] = make_float4(me.dir.x, me.dir.y, me.dir.z, 0.f);
        }
        float4 f4v;
        {
            const float4 f2 = L.B.f[2][s], f3 = L.B.f[3][s];
            f4v = L.B.f[4][s];
            me.side = v3(f2);
            me.radius = f2.w;
            me.up = v3(f3);
            me.mass = f3.w;
            me.max_speed = f4v.x;
            me.max_force = f4v.y;
        }
        unsigned applied = p.clear_applied ? 0u : u(f4v.z);
        V3 steer = p.dirty ? v3(L.B.f[5][s]) : v3(0.f, 0.f, 0.f);
        finish_all(a, p, need, 0, fs, fa, fc, me, applied, steer,
                   [&](unsigned rank, V3& bp, V3& bh, float& bsp) {
                       const unsigned bs = col[(base + rank) * bd];
                       const float4 b0 = L.B.f[0][bs], b1 = L.B.f[1][bs];
                       bp = v3(b0);
                       bh = v3(b1);
                       bsp = b1.w;
                   });
        integrate(me, steer, p.dt);
        store_next(L, s, me, id, scene, sc, p.wrap_mode);
        if (!EXACT) return;
    }
}

// ---- wall phase: KNN, wall KNN and avoid-walls ---------------------------------------
// Agent in slot s (entry `it` of the retry list on the exact path); col: the
// thread's shared column (stride bd).
template <int KMAX, int KW, unsigned ENUM, bool EXACT, bool FLAT>
__device__ __forceinline__ void walls_agent(const FusedLaunch& L, const StepDev& p, unsigned s,
                                            unsigned it, unsigned* col, unsigned bd) {
    {
        const float4 f0 = L.B.f[0][s];
        const V3 pos = v3(f0);
        const unsigned id = u(f0.w), scene = load_scene(L.B, s);
        const Scene sc = L.scenes[scene];
        unsigned ix, iy, iz;
        cell_coords(sc.grid, pos, ix, iy, iz);
        const Box box = cell_box(sc.grid, ix, iy, iz, p.r);
        // a redo agent (base UINT_MAX: on the retry list) still gets its wall
        // behaviour here, which does not read its own neighbours; the
        // warp-per-agent search writes its list
        const unsigned base = agent_knn<KMAX, ENUM, EXACT, FLAT>(L, p, s, it, pos, id, sc, box, col, bd);
        float4 f4v;
        Self me = load_rest(L.B, s, pos, f4v);
        unsigned applied = p.clear_applied ? 0u : u(f4v.z);
        V3 steer = p.dirty ? v3(L.B.f[5][s]) : v3(0.f, 0.f, 0.f);
        for (unsigned r = 0; r < p.k && base != UINT_MAX; ++r) {
            const unsigned bs = col[(base + r) * bd];
            L.knn_slot[size_t(r) * L.n + s] = bs;
            // the KNN distance (before any wall correction moves agents),
            // read by avoid-close-neighbours only
            if (p.need & NEED_CLOSE)
                L.knn_dist[size_t(r) * L.n + s] =
                    bs == UINT_MAX ? FLT_MAX : distance(me.pos, v3(L.B.f[0][bs]));
        }
        if (sc.n_walls > 0 && L.w_pos_id != nullptr) {
            // wall lines staged in this thread's (now free) shared column
            {
                KList<KW> wl;
                wl.init(int(p.knw));
                knn_scan_box<KW>(wl, me.pos, UINT_MAX, sc.grid, box, sc.wall_cell_offset,
                                 L.w_cell_start, L.w_pos_id);
                wl.for_each(int(p.knw), [&](int r, unsigned long long key, unsigned) {
                    col[r * bd] = key_id(key);
                });
            }
            WallAcc wa;
            walls_init(wa, me, p.min_time_wall);
            for (unsigned r = 0; r < p.knw; ++r) {
                const unsigned line = col[r * bd];
                if (line >= sc.n_walls) break;
                const unsigned g = sc.wall_offset + line;
                walls_add(wa, me, line, v3(L.w_start[g]), v3(L.w_end[g]), v3(L.w_normal[g]));
            }
            walls_finish(wa, p.w_walls, p.mask_walls, me, applied, steer);
        } else if (!(applied & p.mask_walls)) {
            steer = add(mul(v3(0.f, 0.f, 0.f), p.w_walls), steer);
        }
        // the radius rides with the position: a neighbour costs the rest
        // phase two gathers (w0, w1) instead of three
        L.w0[s] = make_float4(me.pos.x, me.pos.y, me.pos.z, me.radius);
        L.w1[s] = make_float4(me.dir.x, me.dir.y, me.dir.z, me.speed);
        L.w2[s] = make_float4(steer.x, steer.y, steer.z, fb(applied));
    }
}

template <int KMAX, int KW, unsigned ENUM, bool EXACT, bool FLAT = false>
__global__ void __launch_bounds__(kBlock, 4) k_fused_walls(FusedLaunch L, StepDev p) {
    extern __shared__ unsigned sh_col[];
    const unsigned bd = blockDim.x;
    unsigned* col = sh_col + threadIdx.x;
    const unsigned step = EXACT ? gridDim.x * blockDim.x : 0u;
    for (unsigned it = first_agent<EXACT>();; it += step) {
        unsigned s;
        if (!next_agent<EXACT>(L, it, s)) return;
        walls_agent<KMAX, KW, ENUM, EXACT, FLAT>(L, p, s, it, col, bd);
        if (!EXACT) return;
    }
}

// ---- rest of the step after the wall phase --------------------------------------------
// Five blocks per SM (48 registers): the rest phase waits on neighbour
// gathers, and the extra resident warps hide more of that than the spills
// cost (0.604 -> 0.585 ms per 256-scene step against four blocks).
template <int KMAX, unsigned NEEDC>
__device__ __forceinline__ void rest_agent(const FusedLaunch& L, const StepDev& p, unsigned s) {
    const unsigned need = NEEDC == kNeedRuntime ? p.need : NEEDC;
    // the neighbour pass reads position, radius, heading and speed only; the
    // rest of the state is loaded after it, so it is not held through the pass
    const float4 w0 = L.w0[s], w1 = L.w1[s];
    Self me;
    me.pos = v3(w0);
    me.radius = w0.w;
    me.dir = v3(w1);
    me.speed = w1.w;
    const FlockParams fs = flock_params(p.sep, p.sep_dsq), fa = flock_params(p.ali, p.ali_dsq),
                      fc = flock_params(p.coh, p.coh_dsq);
    const AngleGate gs_ = angle_gate(me.dir, fs.cos_max), ga = angle_gate(me.dir, fa.cos_max),
                    gc = angle_gate(me.dir, fc.cos_max);
    Accs a;
    init_accs(a, p);
    const bool need_dir = need & (NEED_ALI | NEED_AVOID);
    // Neighbour avoidance runs as a second pass over the neighbours whose
    // approach time may fall in its window (about a fifth in a crowd); the
    // others leave its accumulator unchanged, so the result is the same.  A
    // warp then runs the exact test as often as its busiest lane needs it,
    // not once per list entry.
    // Neighbours kRestChunk at a time: their slots, then their gathers, are
    // issued together.
    unsigned exact_avoid = 0;
    const PackedSelf pq = packed_self(me);
    for (unsigned i0 = 0; i0 < p.k; i0 += kRestChunk) {
        unsigned bs[kRestChunk];
        float4 b0[kRestChunk], b1[kRestChunk];
#pragma unroll
        for (unsigned j = 0; j < kRestChunk; ++j)
            bs[j] = i0 + j < p.k ? L.knn_slot[size_t(i0 + j) * L.n + s] : UINT_MAX;
#pragma unroll
        for (unsigned j = 0; j < kRestChunk; ++j) {
            const bool ok = bs[j] != UINT_MAX;
            b0[j] = ok ? L.w0[bs[j]] : make_float4(0.f, 0.f, 0.f, 0.f);
            b1[j] = ok && need_dir ? L.w1[bs[j]] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (unsigned j = 0; j < kRestChunk; ++j) {
            if (bs[j] == UINT_MAX) break;
            const unsigned i = i0 + j;
            const float kd = (need & NEED_CLOSE) ? L.knn_dist[size_t(i) * L.n + s] : -1.f;
            V3 off;
            unsigned long long o_xy;
            const float dsq = packed_offset(pq, me, b0[j], off, o_xy);
            accumulate_at(a, p, need & ~NEED_AVOID, fs, fa, fc, gs_, ga, gc, me, i, kd, off, dsq,
                          v3(b0[j]), v3(b1[j]), b1[j].w, b0[j].w);
            if ((need & NEED_AVOID) &&
                packed_avoid_time_may_fall_in(pq, o_xy, off.z, p.min_time_col, b1[j]))
                exact_avoid |= 1u << i;
        }
        if (bs[kRestChunk - 1] == UINT_MAX) break;
    }
    while (exact_avoid) {
        const unsigned i = unsigned(__ffs(int(exact_avoid)) - 1);
        exact_avoid &= exact_avoid - 1;
        const unsigned bs = L.knn_slot[size_t(i) * L.n + s];
        const float4 b0 = L.w0[bs], b1 = L.w1[bs];
        avoid_lite_add(a.avoid, me, i, v3(b0), v3(b1), b1.w, b0.w);
    }
    const float4 w2 = L.w2[s];
    const float4 f2 = L.B.f[2][s], f3 = L.B.f[3][s], f4v = L.B.f[4][s];
    me.side = v3(f2);
    me.up = v3(f3);
    me.mass = f3.w;
    me.max_speed = f4v.x;
    me.max_force = f4v.y;
    const unsigned id = u(reinterpret_cast<const float*>(L.B.f[0] + s)[3]), scene = u(f4v.w);
    unsigned applied = u(w2.w);
    V3 steer = v3(w2);
    finish_all(a, p, need, 1, fs, fa, fc, me, applied, steer,
               [&](unsigned rank, V3& bp, V3& bh, float& bsp) {
                   const unsigned bs = L.knn_slot[size_t(rank) * L.n + s];
                   const float4 b0 = L.w0[bs], b1 = L.w1[bs];
                   bp = v3(b0);
                   bh = v3(b1);
                   bsp = b1.w;
               });
    integrate(me, steer, p.dt);
    const Scene sc = L.scenes[scene];
    store_next(L, s, me, id, scene, sc, p.wrap_mode);
}

template <int KMAX, unsigned NEEDC>
__global__ void __launch_bounds__(kBlock, 5) k_fused_rest(FusedLaunch L, StepDev p) {
    const unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < L.n) rest_agent<KMAX, NEEDC>(L, p, s);
}

// Opts a kernel into more than 48 KiB of dynamic shared memory, once per
// kernel (outside any stream capture: the first launch of a kernel is never
// captured, see gs_capi.cu).
template <class K>
static gs_status allow_smem(K kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<const void*, size_t> done;
    if (bytes <= 48 * 1024) return GS_OK;
    std::lock_guard<std::mutex> lock(mu);
    const void* key = reinterpret_cast<const void*>(kernel);
    auto it = done.find(key);
    if (it != done.end() && it->second >= bytes) return GS_OK;
    GS_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
    done[key] = bytes;
    return GS_OK;
}

// Redo launches over the retry list: a grid of up to four blocks per SM that
// strides over however many agents the fast launch appended (read on the
// device); agents that all overflowed still spread over the whole GPU.
constexpr unsigned kRetryBlocksMax = 4 * 152;

template <int KMAX, unsigned ENUM>
static gs_status launch_fused_k(const FusedLaunch& L, const StepDev& p, cudaStream_t st,
                                PhaseHook* hook) {
    const unsigned bs = p.block ? p.block : kBlock;
    const unsigned nb = blocks_for(L.n, bs);
    const unsigned nb_retry = std::min(blocks_for(L.n, kBlock), kRetryBlocksMax);
    // collecting scan: slot and key tables of ENUM words per thread;
    // streaming scan: the k result slots only
    const size_t smem = ENUM > 64 ? size_t(KMAX > 8 ? KMAX : 8) * bs * sizeof(unsigned)
                                  : size_t(2 * ENUM) * bs * sizeof(unsigned);
    const size_t smem_x = size_t(KMAX > 8 ? KMAX : 8) * kBlock * sizeof(unsigned);
    // The warp-per-agent exact lists (and, without walls, the redo launch)
    // serve the streaming scan (crowded boxes, 40-250 candidates); the
    // collecting scan's kernels redo their few agents inline (sparse boxes,
    // mostly distance ties among a dozen candidates), which costs less than a
    // launch of one agent's latency.
    if (p.need & NEED_WALLS) {
        if (hook) hook->mark(2, true);
        // flat grids (one cell high) have a 3-row build of the streaming scan
        bool launched = false;
        if constexpr (ENUM > 64) {
            if (p.flat) {
                GS_TRY(allow_smem(k_fused_walls<KMAX, 8, ENUM, false, true>, smem));
                k_fused_walls<KMAX, 8, ENUM, false, true><<<nb, bs, smem, st>>>(L, p);
                launched = true;
            }
        }
        if (!launched) {
            GS_TRY(allow_smem(k_fused_walls<KMAX, 8, ENUM, false>, smem));
            k_fused_walls<KMAX, 8, ENUM, false><<<nb, bs, smem, st>>>(L, p);
        }
        // the redo agents' exact lists, straight into the neighbour lists
        if (ENUM > 64) k_knn_retry<KMAX, true><<<nb_retry, kBlock, 0, st>>>(L, p);
        if (hook) hook->mark(2, false);
        if (hook) hook->mark(3, true);
        // the choke-point step (separation and neighbour avoidance) has its own build
        if ((p.need & kNeedList) == (NEED_SEP | NEED_AVOID))
            k_fused_rest<KMAX, NEED_SEP | NEED_AVOID><<<nb, bs, 0, st>>>(L, p);
        else
            k_fused_rest<KMAX, kNeedRuntime><<<nb, bs, 0, st>>>(L, p);
        if (hook) hook->mark(3, false);
    } else {
        GS_TRY(allow_smem(k_fused<KMAX, ENUM, false>, smem));
        if (hook) hook->mark(2, true);
        // the flock (separation, alignment, cohesion) on the collecting scan has
        // its own build
        bool done = false;
        if constexpr (ENUM == 32) {
            if ((p.need & kNeedList) == (NEED_SEP | NEED_ALI | NEED_COH)) {
                GS_TRY(allow_smem(k_fused<KMAX, 32, false, NEED_SEP | NEED_ALI | NEED_COH>, smem));
                k_fused<KMAX, 32, false, NEED_SEP | NEED_ALI | NEED_COH><<<nb, bs, smem, st>>>(L, p);
                done = true;
            }
        }
        if constexpr (ENUM > 64) {
            if (p.flat) {
                GS_TRY(allow_smem(k_fused<KMAX, ENUM, false, kNeedRuntime, true>, smem));
                k_fused<KMAX, ENUM, false, kNeedRuntime, true><<<nb, bs, smem, st>>>(L, p);
                done = true;
            }
        }
        if (!done) k_fused<KMAX, ENUM, false><<<nb, bs, smem, st>>>(L, p);
        if (ENUM > 64) {
            k_knn_retry<KMAX, false><<<nb_retry, kBlock, 0, st>>>(L, p);
            k_fused<KMAX, 32, true><<<nb_retry, kBlock, smem_x, st>>>(L, p);
        }
        if (hook) hook->mark(2, false);
    }
    GS_LAUNCHED("fused_step");
    return GS_OK;
}

template <int KMAX>
static gs_status launch_fused(const FusedLaunch& L, const StepDev& p, cudaStream_t st,
                              PhaseHook* hook) {
    if (p.enum_cap <= 32) return launch_fused_k<KMAX, 32>(L, p, st, hook);
    if (p.enum_cap <= 64) return launch_fused_k<KMAX, 64>(L, p, st, hook);
    if (p.enum_cap <= 128) return launch_fused_k<KMAX, 128>(L, p, st, hook);
    return launch_fused_k<KMAX, 256>(L, p, st, hook);
}

// ---- the wall/rest step in one persistent launch ----------------------------------
// One cooperative launch runs every phase of the step - the scan's starts, the
// permute, the wall phase, the warp-per-agent exact lists and the rest phase -
// over a grid of co-resident blocks.  Each
// phase is a grid-stride loop over the same device functions the separate
// kernels run, so the results are the same bit for bit; a grid-wide barrier
// separates the phases.  Every barrier wait is bounded: a block that polls
// more than P.limit times, or sees that another block gave up, sets
// kErrBarrierTimeout and returns.  A block passes a barrier only once every
// block has arrived there, i.e. finished the phase before it, so a step that
// gives up never feeds a phase half-written input; the step is void and the
// host reports GS_ERR_TIMEOUT.
struct GridBarrier {
    unsigned count, gen;
};

__device__ __forceinline__ unsigned ld_volatile(const unsigned* a) {
    return *reinterpret_cast<const volatile unsigned*>(a);
}

__device__ bool grid_sync(GridBarrier* bar, unsigned limit, unsigned* err) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        const unsigned gen = ld_volatile(&bar->gen);
        __threadfence();
        if (atomicAdd(&bar->count, 1u) == gridDim.x - 1) {
            atomicExch(&bar->count, 0u);
            __threadfence();
            atomicAdd(&bar->gen, 1u);
        } else {
            unsigned polls = 0;
            while (ld_volatile(&bar->gen) == gen) {
                if (++polls > limit || (ld_volatile(err) & kErrBarrierTimeout)) {
                    atomicOr(err, kErrBarrierTimeout);
                    ok = 0;
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

template <int KMAX>
constexpr size_t persistent_smem() {
    constexpr size_t scan = (kScanTile + kScanTile / 32 + kBlock / 32) * sizeof(unsigned);
    constexpr size_t cols = size_t(KMAX) * kBlock * sizeof(unsigned);
    constexpr size_t retry = (kBlock / 32) * kRetryWarpKeys * (sizeof(unsigned long long) + 4);
    return scan > cols ? (scan > retry ? scan : retry) : (cols > retry ? cols : retry);
}

template <int KMAX, unsigned ENUM, unsigned NEEDC>
__global__ void __launch_bounds__(kBlock, 4) k_step_persistent(FusedLaunch L, StepDev p,
                                                               PersistLaunch P) {
    extern __shared__ __align__(16) unsigned char sm[];
    GridBarrier* bar = reinterpret_cast<GridBarrier*>(P.bar);
    const unsigned nthreads = gridDim.x * blockDim.x;
    const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
    // scan: starts of the tiles near agents (zeroing their counts), from the
    // tile totals the counting atomics added
    unsigned* sh = reinterpret_cast<unsigned*>(sm);
    unsigned* ws = sh + kScanTile + kScanTile / 32;
    for (unsigned t = blockIdx.x; t < P.T; t += gridDim.x)
        scan_apply_sparse_tile(L.count, P.C, P.tile, P.start, P.T, t, p.scan_reach, P.live, sh,
                               ws);
    if (!grid_sync(bar, P.limit, L.err)) return;
    // permute A -> B; the tile totals start again for the step's counting
    if (gtid == 0) *L.retry_count = 0u;
    for (unsigned t = gtid; t < P.T; t += nthreads) P.tile[t] = 0u;
    for (unsigned i = gtid; i < L.n; i += nthreads)
        permute_agent(L.A, L.B, L.n, L.cellrank, P.start, L.scenes, p.wrap_mode, p.dirty, L.err, i);
    if (!grid_sync(bar, P.limit, L.err)) return;
    // wall phase
    unsigned* col = reinterpret_cast<unsigned*>(sm) + threadIdx.x;
    for (unsigned s = gtid; s < L.n; s += nthreads)
        walls_agent<KMAX, 8, ENUM, false, true>(L, p, s, s, col, kBlock);
    if (!grid_sync(bar, P.limit, L.err)) return;
    // exact lists of the redo entries, one warp per entry
    {
        const unsigned w = threadIdx.x >> 5;
        unsigned long long* keys = reinterpret_cast<unsigned long long*>(sm) + w * kRetryWarpKeys;
        unsigned* slots = reinterpret_cast<unsigned*>(reinterpret_cast<unsigned long long*>(sm) +
                                                      (kBlock / 32) * kRetryWarpKeys) +
                          w * kRetryWarpKeys;
        retry_lists<KMAX, true>(L, p, w * gridDim.x + blockIdx.x, gridDim.x * (kBlock / 32),
                                keys, slots);
    }
    if (!grid_sync(bar, P.limit, L.err)) return;
    // rest phase
    for (unsigned s = gtid; s < L.n; s += nthreads) rest_agent<KMAX, NEEDC>(L, p, s);
}

bool persistent_supported(const StepDev& p) {
    return (p.need & NEED_WALLS) && p.enum_cap > 64 && p.k > 8 && p.k <= 16 && p.flat &&
           p.knw <= 8;
}

template <unsigned ENUM, unsigned NEEDC>
static gs_status launch_persistent_k(const FusedLaunch& L, const StepDev& p,
                                     const PersistLaunch& P, cudaStream_t st) {
    auto kern = k_step_persistent<16, ENUM, NEEDC>;
    constexpr size_t smem = persistent_smem<16>();
    GS_TRY(allow_smem(kern, smem));
    int dev = 0, sms = 0, per_sm = 0;
    GS_CUDA(cudaGetDevice(&dev));
    GS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, smem));
    if (per_sm < 1) return fail(GS_ERR_UNSUPPORTED, "the persistent step does not fit on an SM");
    const unsigned grid = unsigned(per_sm) * unsigned(sms);
    // the barrier starts from zero on every launch, also after a step that gave up
    GS_CUDA(cudaMemsetAsync(P.bar, 0, sizeof(GridBarrier), st));
    FusedLaunch l = L;
    StepDev q = p;
    PersistLaunch pp = P;
    void* args[] = {&l, &q, &pp};
    GS_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(kern), dim3(grid),
                                        dim3(kBlock), args, smem, st));
    return GS_OK;
}

gs_status fused_step_persistent(const FusedLaunch& L, const StepDev& p, const PersistLaunch& P,
                                cudaStream_t st) {
    if (L.n == 0) return GS_OK;
    if (!persistent_supported(p)) return fail(GS_ERR_UNSUPPORTED, "no persistent build for this step");
    const bool sep_avoid = (p.need & kNeedList) == (NEED_SEP | NEED_AVOID);
    if (p.enum_cap <= 128)
        return sep_avoid ? launch_persistent_k<128, NEED_SEP | NEED_AVOID>(L, p, P, st)
                         : launch_persistent_k<128, kNeedRuntime>(L, p, P, st);
    return sep_avoid ? launch_persistent_k<256, NEED_SEP | NEED_AVOID>(L, p, P, st)
                     : launch_persistent_k<256, kNeedRuntime>(L, p, P, st);
}

gs_status fused_step(const FusedLaunch& L, const StepDev& p, cudaStream_t st, PhaseHook* hook) {
    if (L.n == 0) return GS_OK;
    if ((p.need & NEED_WALLS) && p.knw > 8)
        return fail(GS_ERR_UNSUPPORTED, "knw > 8 in the fused step");
    if (p.k <= 8) return launch_fused<8>(L, p, st, hook);
    if (p.k <= 16) return launch_fused<16>(L, p, st, hook);
    return launch_fused<32>(L, p, st, hook);
}

// A -> reference layout.  Slot order is bucket order, a shuffle of the agent
// order, so the conversion first records each agent's slot (one scattered
// 4-byte store per agent), then writes the reference arrays in agent order,
// coalesced, reading each agent's five float4 from its slot.
__global__ void k_slot_of(Fused A, unsigned n, const Scene* __restrict__ scenes,
                          unsigned* __restrict__ slot_of) {
    const unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const unsigned id = u(A.f[0][s].w), scene = u(A.f[4][s].w);
    slot_of[scenes[scene].agent_offset + id] = s;
}

__global__ void k_to_reference(Fused A, unsigned n, const unsigned* __restrict__ slot_of,
                               GroupView g) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned s = slot_of[i];
    const float4 f0 = A.f[0][s], f1 = A.f[1][s], f2 = A.f[2][s], f3 = A.f[3][s], f4v = A.f[4][s];
    g.position[i] = make_float4(f0.x, f0.y, f0.z, 0.f);
    g.direction[i] = make_float4(f1.x, f1.y, f1.z, 0.f);
    g.speed[i] = f1.w;
    g.side[i] = make_float3(f2.x, f2.y, f2.z);
    g.radius[i] = f2.w;
    g.up[i] = make_float3(f3.x, f3.y, f3.z);
    g.mass[i] = f3.w;
    g.max_speed[i] = f4v.x;
    g.max_force[i] = f4v.y;
    g.applied[i] = u(f4v.z);
    g.steering[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

gs_status fused_to_reference(Fused A, unsigned n, const Scene* scenes, unsigned* slot_of,
                             GroupView g, cudaStream_t st) {
    if (n == 0) return GS_OK;
    k_slot_of<<<blocks_for(n), kBlock, 0, st>>>(A, n, scenes, slot_of);
    k_to_reference<<<blocks_for(n), kBlock, 0, st>>>(A, n, slot_of, g);
    GS_LAUNCHED("fused_to_reference");
    return GS_OK;
}

}  // namespace gs

namespace gs {

// Occupied cells and the sum of squared cell counts (out[0], and the 64-bit
// word at out + 2).
__global__ void k_count_occupied(const unsigned* __restrict__ count, unsigned C,
                                 unsigned* __restrict__ out) {
    unsigned local = 0;
    unsigned long long sq = 0;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < C; i += gridDim.x * blockDim.x) {
        const unsigned c = count[i];
        local += c != 0u;
        sq += (unsigned long long)c * c;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        local += __shfl_down_sync(0xffffffffu, local, o);
        sq += __shfl_down_sync(0xffffffffu, sq, o);
    }
    if ((threadIdx.x & 31) == 0 && local) {
        atomicAdd(out, local);
        atomicAdd(reinterpret_cast<unsigned long long*>(out + 2), sq);
    }
}

gs_status count_occupied(const unsigned* count, unsigned C, unsigned* d_tmp, unsigned* h_out,
                         unsigned long long* h_sumsq, cudaStream_t st) {
    *h_out = 0;
    *h_sumsq = 0;
    if (C == 0) return GS_OK;
    GS_CUDA(cudaMemsetAsync(d_tmp, 0, 4 * sizeof(unsigned), st));
    const unsigned nb = std::min(blocks_for(C, kBlock), 8u * 152u);
    k_count_occupied<<<nb, kBlock, 0, st>>>(count, C, d_tmp);
    GS_LAUNCHED("count_occupied");
    unsigned h[4];
    GS_CUDA(cudaMemcpyAsync(h, d_tmp, sizeof(h), cudaMemcpyDeviceToHost, st));
    GS_CUDA(cudaStreamSynchronize(st));
    *h_out = h[0];
    std::memcpy(h_sumsq, h + 2, sizeof(*h_sumsq));
    return GS_OK;
}

}  // namespace gs
