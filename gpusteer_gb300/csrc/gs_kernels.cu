// Counting-sort binning and the per-function (drop-in) kernels.
//
// The bin rebuild replaces KNNBinningV2UpdateDBCUDA::run (KNNBinningV2.cu:87-162:
// BuildDB, a host synchronisation, thrust::sort_by_key, a memset of every cell
// and ReorderDB) with three passes that never leave the device: an atomic
// count per cell (which also hands each agent its rank inside the cell), an
// exclusive scan of the counts, and a scatter of (position, index) into
// bucketed order.  The order inside a cell follows the atomics and is not
// deterministic; nothing downstream depends on it because every KNN uses the
// total order (distance, agent index).
#include <algorithm>
#include <cstring>

#include "gs_behaviours.cuh"
#include "gs_knn.cuh"
#include "gs_scan.cuh"

#include "gs_launch.h"

namespace gs {

// ---- exclusive scan (device code in gs_scan.cuh) ----------------------------------
unsigned scan_tile_count(unsigned C) { return (C + kScanTile - 1) / kScanTile; }

__global__ void __launch_bounds__(kBlock) k_scan_reduce(const unsigned* __restrict__ count,
                                                        unsigned C, unsigned* __restrict__ tile) {
    __shared__ unsigned sh[kScanTile + kScanTile / 32];
    __shared__ unsigned ws[kBlock / 32];
    scan_reduce_tile(count, C, blockIdx.x, sh, ws, tile);
}

// One block scans the tile totals in place (exclusive) and writes start[C].
__global__ void __launch_bounds__(1024) k_scan_tiles(unsigned* tile, unsigned T,
                                                     unsigned* __restrict__ start, unsigned C) {
    __shared__ unsigned ws[32];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (unsigned base = 0; base < T; base += 1024) {
        const unsigned i = base + threadIdx.x;
        const unsigned v = i < T ? tile[i] : 0u;
        const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        unsigned x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= unsigned(o)) x += y;
        }
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        if (warp == 0) {
            unsigned w = ws[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= unsigned(o)) w += y;
            }
            ws[lane] = w;
        }
        __syncthreads();
        const unsigned before = (warp ? ws[warp - 1] : 0u) + carry;
        if (i < T) tile[i] = before + x - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = before + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) start[C] = carry;
}

__global__ void __launch_bounds__(kBlock) k_scan_apply(unsigned* __restrict__ count, unsigned C,
                                                       const unsigned* __restrict__ tile,
                                                       unsigned* __restrict__ start) {
    __shared__ unsigned sh[kScanTile + kScanTile / 32];
    __shared__ unsigned ws[kBlock / 32];
    unsigned items[kScanItems];
    load_tile(count, C, blockIdx.x, sh, items);
    unsigned s = 0;
#pragma unroll
    for (unsigned j = 0; j < kScanItems; ++j) s += items[j];
    unsigned total;
    unsigned run = block_exclusive_sum(s, ws, total) + tile[blockIdx.x];
#pragma unroll
    for (unsigned j = 0; j < kScanItems; ++j) {
        const unsigned i = threadIdx.x * kScanItems + j;
        sh[i + i / 32] = run;
        run += items[j];
    }
    __syncthreads();
    const unsigned base = blockIdx.x * kScanTile;
#pragma unroll
    for (unsigned j = 0; j < kScanItems; ++j) {
        const unsigned i = j * kBlock + threadIdx.x;
        if (base + i < C) {
            start[base + i] = sh[i + i / 32];
            count[base + i] = 0u;
        }
    }
}

gs_status scan_counts(unsigned* count, unsigned* start, unsigned C, unsigned* tile,
                      cudaStream_t st) {
    const unsigned T = scan_tile_count(C);
    k_scan_reduce<<<T, kBlock, 0, st>>>(count, C, tile);
    k_scan_tiles<<<1, 1024, 0, st>>>(tile, T, start, C);
    k_scan_apply<<<T, kBlock, 0, st>>>(count, C, tile, start);
    GS_LAUNCHED("scan");
    return GS_OK;
}

// ---- the fused engine's counting-sort scan: one launch, tiles near agents ---------
// The step's counting atomics add each tile's total as they go, so no reduce
// pass reads the counts (only a whole recount, from the reference layout or
// on a new grid, takes one); every block sums the totals of the tiles before its own (a
// few thousand words from L2) and writes its tile's starts, and no block
// waits on another (scan_apply_sparse_tile).
__global__ void __launch_bounds__(kBlock) k_scan_apply_sparse(unsigned* __restrict__ count,
                                                              unsigned C,
                                                              const unsigned* __restrict__ tile,
                                                              unsigned* __restrict__ start,
                                                              unsigned T, unsigned reach,
                                                              unsigned* __restrict__ live) {
    __shared__ unsigned sh[kScanTile + kScanTile / 32];
    __shared__ unsigned ws[kBlock / 32];
    scan_apply_sparse_tile(count, C, tile, start, T, blockIdx.x, reach, live, sh, ws);
}

gs_status scan_tile_totals(const unsigned* count, unsigned C, unsigned* tile, cudaStream_t st) {
    const unsigned T = scan_tile_count(C);
    if (T == 0) return GS_OK;
    k_scan_reduce<<<T, kBlock, 0, st>>>(count, C, tile);
    GS_LAUNCHED("scan_tile_totals");
    return GS_OK;
}

gs_status scan_counts_sparse(unsigned* count, unsigned* start, unsigned C, const unsigned* tile,
                             unsigned* live, unsigned reach, cudaStream_t st) {
    const unsigned T = scan_tile_count(C);
    if (T == 0) return GS_OK;
    k_scan_apply_sparse<<<T, kBlock, 0, st>>>(count, C, tile, start, T, reach, live);
    GS_LAUNCHED("scan_sparse");
    return GS_OK;
}

unsigned scan_reach_tiles(const unsigned wc[3], unsigned r) {
    // labels are x + z wc0 + y wc0 wc2: a box of radius r reads starts at
    // most rx + rz wc0 + ry wc0 wc2 + 1 labels from its centre cell (the +1:
    // the start after a row's last cell)
    auto reach = [&](unsigned n) { return std::min<unsigned long long>(r, n ? n - 1 : 0); };
    const unsigned long long d = reach(wc[0]) + reach(wc[2]) * wc[0] +
                                 reach(wc[1]) * (unsigned long long)wc[0] * wc[2] + 1;
    const unsigned long long t = (d + kScanTile - 1) / kScanTile;
    return t > 0xffffffffull ? 0xffffffffu : unsigned(t);
}

// ---- database -----------------------------------------------------------------------
gs_status db_reserve(Database& db, unsigned n, unsigned C) {
    if (db.cells != C) {
        dfree(db.start);
        dfree(db.count);
        dfree(db.tile);
        dfree(db.live);
        GS_TRY(dalloc(&db.start, size_t(C) + 1));
        GS_TRY(dalloc(&db.count, C));
        GS_TRY(dalloc(&db.tile, scan_tile_count(C) + 1));
        GS_TRY(dalloc(&db.live, scan_tile_count(C) + 1));
        GS_CUDA(cudaMemset(db.count, 0, size_t(C) * sizeof(unsigned)));
        GS_CUDA(cudaMemset(db.tile, 0, (size_t(scan_tile_count(C)) + 1) * sizeof(unsigned)));
        GS_CUDA(cudaMemset(db.live, 0, (size_t(scan_tile_count(C)) + 1) * sizeof(unsigned)));
        // the counts are used next on a non-blocking stream
        GS_CUDA(cudaDeviceSynchronize());
        db.cells = C;
    }
    if (n > 0 && db.cell == nullptr) {
        GS_TRY(dalloc(&db.cell, n));
        GS_TRY(dalloc(&db.rank, n));
        GS_TRY(dalloc(&db.sorted, n));
        GS_TRY(dalloc(&db.pos_id, n));
    }
    db.valid = false;
    return GS_OK;
}

void db_release(Database& db) {
    dfree(db.cell);
    dfree(db.rank);
    dfree(db.sorted);
    dfree(db.pos_id);
    dfree(db.start);
    dfree(db.count);
    dfree(db.tile);
    dfree(db.live);
    db.cells = 0;
    db.agent_cap = 0;
    db.valid = false;
}

__global__ void k_db_count(const float4* __restrict__ pos, unsigned n, Grid g,
                           unsigned* __restrict__ cell, unsigned* __restrict__ rank,
                           unsigned* __restrict__ count) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned c = cell_of(g, v3(pos[i]));
    cell[i] = c;
    rank[i] = atomicAdd(count + c, 1u);
}

__global__ void k_db_scatter(const float4* __restrict__ pos, unsigned n,
                             const unsigned* __restrict__ cell, const unsigned* __restrict__ rank,
                             const unsigned* __restrict__ start, unsigned* __restrict__ sorted,
                             float4* __restrict__ pos_id) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned dst = start[cell[i]] + rank[i];
    if (dst >= n) return;
    const float4 p = pos[i];
    sorted[dst] = i;
    pos_id[dst] = make_float4(p.x, p.y, p.z, __uint_as_float(i));
}

gs_status db_build(Database& db, const float4* pos, unsigned n, const Grid& grid,
                   cudaStream_t st) {
    const unsigned C = grid.wc[0] * grid.wc[1] * grid.wc[2];
    if (db.cells != C || (n > 0 && db.cell == nullptr))
        return fail(GS_ERR_STATE, "database not reserved for this grid");
    if (n > 0) k_db_count<<<blocks_for(n), kBlock, 0, st>>>(pos, n, grid, db.cell, db.rank, db.count);
    GS_TRY(scan_counts(db.count, db.start, C, db.tile, st));
    if (n > 0)
        k_db_scatter<<<blocks_for(n), kBlock, 0, st>>>(pos, n, db.cell, db.rank, db.start,
                                                       db.sorted, db.pos_id);
    GS_LAUNCHED("db_build");
    db.grid = grid;
    db.valid = true;
    return GS_OK;
}

// ---- binned KNN, reference output layout (KNNBinningV2Kernel.cu:417-528) ----------
// One thread per agent of A in bucketed order (neighbouring threads scan the
// same cells); results go to idx/dist[a + i * nA].
template <int KMAX>
__global__ void __launch_bounds__(kBlock) k_knn_binned(
    const unsigned* __restrict__ a_sorted, const float4* __restrict__ a_pos_id, unsigned nA,
    const unsigned* __restrict__ b_start, const float4* __restrict__ b_pos_id, Grid g,
    unsigned r, unsigned k, bool self, unsigned* __restrict__ idx, float* __restrict__ dist) {
    const unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nA) return;
    const unsigned a = a_sorted[s];
    const V3 p = v3(a_pos_id[s]);
    unsigned ix, iy, iz;
    cell_coords(g, p, ix, iy, iz);
    const Box box = cell_box(g, ix, iy, iz, r);
    extern __shared__ unsigned sh_col[];
    unsigned* col = sh_col + threadIdx.x;
    const unsigned bd = blockDim.x;
    knn_neighbours<KMAX, 64>(int(k), p, self ? a : UINT_MAX, g, box, 0u, b_start, b_pos_id, col,
                             bd);
    for (unsigned r = 0; r < k; ++r) {
        const unsigned bs = col[r * bd];
        const float4 q = bs == UINT_MAX ? make_float4(0.f, 0.f, 0.f, 0.f) : b_pos_id[bs];
        idx[a + size_t(r) * nA] = bs == UINT_MAX ? UINT_MAX : __float_as_uint(q.w);
        dist[a + size_t(r) * nA] = bs == UINT_MAX ? FLT_MAX : distance(p, v3(q));
    }
}

template <int KMAX>
static gs_status knn_binned_k(const Database& A, unsigned nA, const Database& B, bool self,
                              unsigned r, unsigned k, unsigned* idx, float* dist,
                              cudaStream_t st) {
    const size_t smem = size_t(2 * 64) * kBlock * sizeof(unsigned);
    if (smem > 48 * 1024)
        GS_CUDA(cudaFuncSetAttribute(k_knn_binned<KMAX>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    k_knn_binned<KMAX><<<blocks_for(nA), kBlock, smem, st>>>(A.sorted, A.pos_id, nA, B.start,
                                                             B.pos_id, B.grid, r, k, self, idx,
                                                             dist);
    GS_LAUNCHED("knn_binned");
    return GS_OK;
}

// ---- batched binned KNN over group pairs --------------------------------------
// The k_knn_binned search for several (A, B) database pairs in one launch: the
// pair table rides in the kernel parameters, each pair owns a contiguous run
// of blocks, and a block finds its pair by a scan of the (few) block offsets.
template <int KMAX>
__global__ void __launch_bounds__(kBlock) k_knn_binned_pairs(KnnPairs P) {
    unsigned q = 0;
    while (q + 1 < P.n_pairs && blockIdx.x >= P.pair[q + 1].block_begin) ++q;
    const KnnPair& pr = P.pair[q];
    const unsigned s = (blockIdx.x - pr.block_begin) * blockDim.x + threadIdx.x;
    if (s >= pr.nA) return;
    const unsigned a = pr.a_sorted[s];
    const V3 p = v3(pr.a_pos_id[s]);
    unsigned ix, iy, iz;
    cell_coords(P.grid, p, ix, iy, iz);
    const Box box = cell_box(P.grid, ix, iy, iz, P.r);
    extern __shared__ unsigned sh_col[];
    unsigned* col = sh_col + threadIdx.x;
    const unsigned bd = blockDim.x;
    knn_neighbours<KMAX, 64>(int(pr.k), p, pr.self ? a : UINT_MAX, P.grid, box, 0u, pr.b_start,
                             pr.b_pos_id, col, bd);
    for (unsigned r = 0; r < pr.k; ++r) {
        const unsigned bs = col[r * bd];
        const float4 v = bs == UINT_MAX ? make_float4(0.f, 0.f, 0.f, 0.f) : pr.b_pos_id[bs];
        pr.idx[a + size_t(r) * pr.nA] = bs == UINT_MAX ? UINT_MAX : __float_as_uint(v.w);
        pr.dist[a + size_t(r) * pr.nA] = bs == UINT_MAX ? FLT_MAX : distance(p, v3(v));
    }
}

template <int KMAX>
static gs_status knn_pairs_k(const KnnPairs& P, unsigned blocks, cudaStream_t st) {
    const size_t smem = size_t(2 * 64) * kBlock * sizeof(unsigned);
    if (smem > 48 * 1024)
        GS_CUDA(cudaFuncSetAttribute(k_knn_binned_pairs<KMAX>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    k_knn_binned_pairs<KMAX><<<blocks, kBlock, smem, st>>>(P);
    GS_LAUNCHED("knn_binned_pairs");
    return GS_OK;
}
static_assert(sizeof(KnnPairs) <= 4096, "batched KNN parameters exceed 4 KiB");

gs_status launch_knn_binned_pairs(KnnPairs& P, cudaStream_t st) {
    if (P.n_pairs == 0 || P.n_pairs > kMaxKnnPairs)
        return fail(GS_ERR_INVALID_ARG, "between 1 and 49 group pairs per batched KNN");
    unsigned blocks = 0, kmax = 0;
    for (unsigned q = 0; q < P.n_pairs; ++q) {
        P.pair[q].block_begin = blocks;
        blocks += blocks_for(P.pair[q].nA);
        kmax = std::max(kmax, P.pair[q].k);
    }
    if (blocks == 0) return GS_OK;
    if (kmax <= 8) return knn_pairs_k<8>(P, blocks, st);
    if (kmax <= 16) return knn_pairs_k<16>(P, blocks, st);
    if (kmax <= 32) return knn_pairs_k<32>(P, blocks, st);
    return knn_pairs_k<64>(P, blocks, st);
}

gs_status launch_knn_binned(const Database& A, unsigned nA, const Database& B, bool self,
                            unsigned r, unsigned k, unsigned* idx, float* dist, cudaStream_t st) {
    if (nA == 0) return GS_OK;
    if (k <= 8) return knn_binned_k<8>(A, nA, B, self, r, k, idx, dist, st);
    if (k <= 16) return knn_binned_k<16>(A, nA, B, self, r, k, idx, dist, st);
    if (k <= 32) return knn_binned_k<32>(A, nA, B, self, r, k, idx, dist, st);
    return knn_binned_k<64>(A, nA, B, self, r, k, idx, dist, st);
}

// ---- brute-force KNN (KNNBruteForceCudaKernel.cu:207-283) ---------------------------
// A candidate needs its square root only when its squared distance is within
// a rounded-up bound of the current k-th distance squared: a larger squared
// distance has a correctly rounded square root strictly above the k-th
// distance, so it can be skipped without changing the result.
__device__ __forceinline__ float prefilter_bound(unsigned long long thr) {
    const float td = key_dist(thr);
    return __fmul_ru(__fmul_ru(td, td), 1.000004f);
}

// ---- brute force, FP32-pipe form (k <= 64) ----------------------------------------------
// One warp serves kBruteQW queries and keeps each query's exact (distance,
// index) top-k list spread over its lanes: lane r holds entry r (and entry
// 32 + r for k > 32), so the list is sorted across the warp and its k-th key
// is one shuffle away.  The
// block stages kBruteTile candidates in shared memory as x / y / z arrays;
// each lane takes two neighbouring candidates per step and computes their
// squared distances to every query of its warp with packed f32x2 subtract,
// multiply and fused multiply-add.  Those squared distances only filter:
// the warp votes on "within the rounded-up bound of a list's k-th distance"
// and, when any lane says yes, every lane recomputes the candidate's distance
// with the reference's unfused binary32 operations (KNNBruteForceCudaKernel.cu
// :245-271) and the list takes it with one shuffle-and-select insertion.  The
// packed d^2 differs from the unfused one by a few units in the last place,
// far inside the bound's 4e-6 relative margin, so no candidate that belongs
// in a list is filtered out; insertion is by the exact key, so the lists are
// the reference's (distance, lower index) order.  After the first few
// hundred candidates almost no step has a vote, so the warp runs the packed
// arithmetic without divergence.
constexpr unsigned kBruteWarps = 8;
constexpr unsigned kBruteQW = 4;      // queries per warp
constexpr unsigned kBruteTile = 2048; // candidates staged per block step

__device__ __forceinline__ unsigned long long pack2(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void unpack2(unsigned long long v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ unsigned long long sub2(unsigned long long a, unsigned long long b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long mul2(unsigned long long a, unsigned long long b) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b,
                                                   unsigned long long c) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// A query's exact (distance, index) top-k list spread over the warp: lane r
// holds rank r in e[0] and, with L = 2 (32 < k <= 64), rank 32 + r in e[1].
// Ranks at or past k hold the empty key.
template <int L>
struct WarpList {
    unsigned long long e[L];
    __device__ __forceinline__ void init() {
#pragma unroll
        for (int h = 0; h < L; ++h) e[h] = KEY_EMPTY;
    }
    // the k-th key, on every lane (k is warp-uniform)
    __device__ __forceinline__ unsigned long long kth(unsigned k) const {
        if (L == 1 || k <= 32) return __shfl_sync(0xffffffffu, e[0], int(k) - 1);
        return __shfl_sync(0xffffffffu, e[L - 1], int(k) - 33);
    }
};

// Inserts candidate (x, y, z, id) into the lane-distributed list if its
// exact key is below the k-th: each rank below k whose key is larger takes
// the larger of the candidate and the rank before it (all from the old
// list); updates the filter bound.  Every lane runs it with the same
// candidate.
template <int L>
__device__ __forceinline__ void warp_list_insert(WarpList<L>& w, float& bound, float seed_bound,
                                                 V3 q, float x, float y, float z, unsigned id,
                                                 unsigned k, unsigned lane) {
    const unsigned long long key = knn_key(distance(q, v3(x, y, z)), id);
    if (!(key < w.kth(k))) return;  // warp-uniform
    const unsigned long long left0 = __shfl_up_sync(0xffffffffu, w.e[0], 1);
    if (L == 2) {
        unsigned long long left1 = __shfl_up_sync(0xffffffffu, w.e[L - 1], 1);
        const unsigned long long last0 = __shfl_sync(0xffffffffu, w.e[0], 31);
        if (lane == 0) left1 = last0;  // rank 32 follows rank 31
        if (32 + lane < k && key < w.e[L - 1]) w.e[L - 1] = key > left1 ? key : left1;
    }
    if (lane < k && key < w.e[0]) w.e[0] = (lane == 0 || key > left0) ? key : left0;
    bound = fminf(seed_bound, prefilter_bound(w.kth(k)));
}

// Writes a warp list to idx / dist[a + rank * nA], ranks below k.
template <int L>
__device__ __forceinline__ void warp_list_store(const WarpList<L>& w, unsigned a, unsigned nA,
                                                unsigned k, unsigned lane,
                                                unsigned* __restrict__ idx,
                                                float* __restrict__ dist) {
#pragma unroll
    for (int h = 0; h < L; ++h) {
        const unsigned rank = 32u * h + lane;
        if (rank < k) {
            idx[a + size_t(rank) * nA] = key_id(w.e[h]);
            dist[a + size_t(rank) * nA] = key_dist(w.e[h]);
        }
    }
}

// Rounded-up filter bound for a known upper bound d of the k-th distance.
__device__ __forceinline__ float seed_prefilter(float d) {
    return __fmul_ru(__fmul_ru(d, d), 1.000004f);
}

// The warp's step over the staged candidates t0 .. t0 + 63 (each lane the
// pair t0 + 2 lane, t0 + 2 lane + 1): the packed filter against every query
// of the warp, then the exact insertion of the candidates that passed.  sid:
// the staged candidates' indices (null: base + their position in the stage).
template <int L>
__device__ __forceinline__ void brute_chunk(
    const float* sx, const float* sy, const float* sz, const unsigned* sid, unsigned base,
    unsigned t0, unsigned cnt, unsigned lane, bool self, unsigned k, const V3 (&q)[kBruteQW],
    const unsigned (&qid)[kBruteQW], const unsigned long long (&px)[kBruteQW],
    const unsigned long long (&py)[kBruteQW], const unsigned long long (&pz)[kBruteQW],
    WarpList<L> (&entry)[kBruteQW], float (&bound)[kBruteQW],
    const float (&seed_bound)[kBruteQW]) {
    const unsigned t = t0 + 2 * lane;
    const unsigned long long x2 = *reinterpret_cast<const unsigned long long*>(sx + t);
    const unsigned long long y2 = *reinterpret_cast<const unsigned long long*>(sy + t);
    const unsigned long long z2 = *reinterpret_cast<const unsigned long long*>(sz + t);
    bool hit0[kBruteQW], hit1[kBruteQW];
    bool any = false;
#pragma unroll
    for (unsigned j = 0; j < kBruteQW; ++j) {
        const unsigned long long dx = sub2(px[j], x2), dy = sub2(py[j], y2), dz = sub2(pz[j], z2);
        float e0, e1;
        unpack2(fma2(dz, dz, fma2(dy, dy, mul2(dx, dx))), e0, e1);
        hit0[j] = e0 <= bound[j];
        hit1[j] = e1 <= bound[j];
        any |= hit0[j] | hit1[j];
    }
    if (!__any_sync(0xffffffffu, any)) return;
    // only the candidates that passed: the lane's first (h = 0) and second
    // (h = 1) candidate have separate votes
#pragma unroll
    for (unsigned j = 0; j < kBruteQW; ++j) {
#pragma unroll
        for (unsigned h = 0; h < 2; ++h) {
            unsigned m = __ballot_sync(0xffffffffu, h ? hit1[j] : hit0[j]);
            while (m) {
                const unsigned src = unsigned(__ffs(m)) - 1u;
                m &= m - 1u;
                const unsigned c = t0 + 2 * src + h;
                if (c >= cnt) continue;
                const unsigned id = sid ? sid[c] : base + c;
                if (self && id == qid[j]) continue;
                warp_list_insert(entry[j], bound[j], seed_bound[j], q[j], sx[c], sy[c], sz[c],
                                 id, k, lane);
            }
        }
    }
}

// seed (may be null): per query an upper bound of its k-th distance (the
// k-th distance among any subset of the candidates is one); the filter then
// starts at that bound instead of infinity, so a query's list takes little
// more than its k final entries.
template <int L>
__global__ void __launch_bounds__(kBruteWarps * 32) k_knn_brute3(
    const float4* __restrict__ posA, unsigned nA, const float4* __restrict__ posB, unsigned nB,
    bool self, unsigned k, const float* __restrict__ seed, unsigned* __restrict__ idx,
    float* __restrict__ dist) {
    __shared__ __align__(16) float sx[kBruteTile], sy[kBruteTile], sz[kBruteTile];
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned q0 = (blockIdx.x * kBruteWarps + warp) * kBruteQW;
    V3 q[kBruteQW];
    unsigned qid[kBruteQW];
    unsigned long long px[kBruteQW], py[kBruteQW], pz[kBruteQW];
    WarpList<L> entry[kBruteQW];
    float bound[kBruteQW], seed_bound[kBruteQW];
#pragma unroll
    for (unsigned j = 0; j < kBruteQW; ++j) {
        const bool act = q0 + j < nA;
        qid[j] = q0 + j;
        q[j] = act ? v3(posA[q0 + j]) : v3(0.f, 0.f, 0.f);
        px[j] = pack2(q[j].x, q[j].x);
        py[j] = pack2(q[j].y, q[j].y);
        pz[j] = pack2(q[j].z, q[j].z);
        entry[j].init();
        seed_bound[j] = (act && seed) ? seed_prefilter(seed[q0 + j]) : prefilter_bound(KEY_EMPTY);
        bound[j] = act ? seed_bound[j] : -1.f;
    }
    const float inf = __int_as_float(0x7f800000);
    for (unsigned base = 0; base < nB; base += kBruteTile) {
        __syncthreads();
        for (unsigned c = threadIdx.x; c < kBruteTile; c += blockDim.x) {
            const float4 v = base + c < nB ? posB[base + c] : make_float4(inf, inf, inf, 0.f);
            sx[c] = v.x;
            sy[c] = v.y;
            sz[c] = v.z;
        }
        __syncthreads();
        const unsigned cnt = min(kBruteTile, nB - base);
        for (unsigned t0 = 0; t0 < cnt; t0 += 64)
            brute_chunk(sx, sy, sz, nullptr, base, t0, cnt, lane, self, k, q, qid, px, py, pz,
                        entry, bound, seed_bound);
    }
#pragma unroll
    for (unsigned j = 0; j < kBruteQW; ++j)
        if (q0 + j < nA) warp_list_store(entry[j], q0 + j, nA, k, lane, idx, dist);
}

// ---- brute force over bucketed candidates: chunks beyond every bound skipped ---------
// With the seed's databases, queries and candidates are taken in bucket
// order (the cell-sorted pos_id arrays: position and agent index), so a
// warp's queries are neighbours and 64 consecutive candidates (a chunk) sit
// in a few neighbouring cells.  Before each stage a lane tests one of the
// stage's 32 chunks: the squared distance from each query of its warp to the
// chunk's bounding box, in the reference's unfused operations.  Per axis the
// gap to the box is fl(lo - q) or fl(q - hi), at most |fl(q - c)| for every
// candidate c of the chunk (rounding is monotone), and squares and sums are
// monotone too, so the box's squared distance is at most every candidate's
// exact one: a chunk whose box lies beyond the filter bound of every query of
// the warp holds no candidate the filter would pass, and the warp skips it
// without changing a list.  The block stages only the chunks some warp needs.

// Bounding box of each chunk of 64 consecutive slots: boxes[2c] = lower
// corner, boxes[2c + 1] = upper corner (NaN coordinates ignored: such a
// candidate's distance is NaN and never passes the filter).  With `merge`,
// pos_id holds n such boxes and each output box covers 32 of them (a stage
// of kBruteTile candidates).  One warp per output box.
__global__ void k_chunk_boxes(const float4* __restrict__ pos_id, unsigned n, bool merge,
                              float4* __restrict__ boxes) {
    const unsigned c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const unsigned per = merge ? 32u : 64u;
    if (c >= (n + per - 1) / per) return;  // warp-uniform
    const float inf = __int_as_float(0x7f800000);
    float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
    if (merge) {
        const unsigned b = c * 32 + lane;
        if (b < n) {
            const float4 l = pos_id[2 * b], h = pos_id[2 * b + 1];
            lo[0] = l.x;
            lo[1] = l.y;
            lo[2] = l.z;
            hi[0] = h.x;
            hi[1] = h.y;
            hi[2] = h.z;
        }
    } else {
#pragma unroll
        for (unsigned h = 0; h < 2; ++h) {
            const unsigned sl = c * 64 + 2 * lane + h;
            if (sl < n) {
                const float4 v = pos_id[sl];
                lo[0] = fminf(lo[0], v.x);
                lo[1] = fminf(lo[1], v.y);
                lo[2] = fminf(lo[2], v.z);
                hi[0] = fmaxf(hi[0], v.x);
                hi[1] = fmaxf(hi[1], v.y);
                hi[2] = fmaxf(hi[2], v.z);
            }
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    }
    if (lane == 0) {
        boxes[2 * c] = make_float4(lo[0], lo[1], lo[2], 0.f);
        boxes[2 * c + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
    }
}

// The scan's seed: per query (one thread each, in bucket order, so that
// neighbouring threads read the same cells) the k-th smallest distance among
// the other group's candidates in its 3 x 3 x 3 cells; in its 5 x 5 x 5, then
// 9 x 9 x 9 cells when the smaller box holds fewer than k (grid corners and
// edges); FLT_MAX when even that box does.  The k-th distance among a subset
// of the candidates is at least the k-th among all of them, and an upper
// bound is all the filter needs, so no list is kept: the k smallest squared
// distances (the reference's unfused sum) stay in registers and one square
// root is taken at the end (correctly rounded square roots keep their
// order).  Candidates at an infinite or NaN distance never enter a list and
// are not counted.  seed[a] by agent index.
template <int KMAX>
__global__ void __launch_bounds__(kBlock) k_brute_seed(const float4* __restrict__ a_pos_id,
                                                       unsigned nA,
                                                       const unsigned* __restrict__ b_start,
                                                       const float4* __restrict__ b_pos_id,
                                                       Grid g, unsigned k, bool self,
                                                       float* __restrict__ seed) {
    const unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nA) return;
    const float4 v = a_pos_id[s];
    const unsigned a = __float_as_uint(v.w);
    if (a >= nA) return;
    const V3 p = v3(v);
    unsigned ix, iy, iz;
    cell_coords(g, p, ix, iy, iz);
    const float inf = __int_as_float(0x7f800000);
    float kth = FLT_MAX;
    for (unsigned r = 1; r <= 4; r *= 2) {
        // the k smallest in top[KMAX - k .. KMAX - 1], ascending; the slots
        // below hold -1 (below every distance) and never change
        float top[KMAX];
#pragma unroll
        for (int i = 0; i < KMAX; ++i) top[i] = i < KMAX - int(k) ? -1.f : inf;
        unsigned found = 0;
        const Box b = cell_box(g, ix, iy, iz, r);
        for (unsigned cy = b.y0; cy <= b.y1; ++cy) {
            for (unsigned cz = b.z0; cz <= b.z1; ++cz) {
                const unsigned s0 = __ldg(b_start + cell_label(g, b.x0, cy, cz));
                const unsigned s1 = __ldg(b_start + cell_label(g, b.x1, cy, cz) + 1);
                for (unsigned t = s0; t < s1; ++t) {
                    const float4 q = __ldg(b_pos_id + t);
                    if (self && __float_as_uint(q.w) == a) continue;
                    const V3 o = sub(p, v3(q));
                    const float d2 = dot(o, o);
                    if (!(d2 < inf)) continue;
                    ++found;
                    if (d2 < top[KMAX - 1]) {
#pragma unroll
                        for (int i = KMAX - 1; i > 0; --i)
                            top[i] = fminf(top[i], fmaxf(top[i - 1], d2));
                        top[0] = fminf(top[0], d2);
                    }
                }
            }
        }
        if (found >= k) {
            kth = sqrtf(top[KMAX - 1]);
            break;
        }
    }
    seed[a] = kth;
}

gs_status launch_brute_seed(const Database& A, unsigned nA, const Database& B, bool self,
                            unsigned k, float* seed, cudaStream_t st) {
    if (nA == 0) return GS_OK;
    if (k == 0 || k > 64)
        return fail(GS_ERR_UNSUPPORTED, "the brute-force seed needs 1 <= k <= 64");
    if (k <= 8)
        k_brute_seed<8><<<blocks_for(nA), kBlock, 0, st>>>(A.pos_id, nA, B.start, B.pos_id, B.grid,
                                                           k, self, seed);
    else if (k <= 16)
        k_brute_seed<16><<<blocks_for(nA), kBlock, 0, st>>>(A.pos_id, nA, B.start, B.pos_id,
                                                            B.grid, k, self, seed);
    else if (k <= 32)
        k_brute_seed<32><<<blocks_for(nA), kBlock, 0, st>>>(A.pos_id, nA, B.start, B.pos_id,
                                                            B.grid, k, self, seed);
    else
        k_brute_seed<64><<<blocks_for(nA), kBlock, 0, st>>>(A.pos_id, nA, B.start, B.pos_id,
                                                            B.grid, k, self, seed);
    GS_LAUNCHED("brute_seed");
    return GS_OK;
}

// Squared distance from q to the box [lo, hi], as a lower bound of every
// inside candidate's exact squared distance (same operation order as dot).
__device__ __forceinline__ float box_dist_sq(V3 q, float4 lo, float4 hi) {
    const V3 gap = v3(fmaxf(fmaxf(lo.x - q.x, q.x - hi.x), 0.f),
                      fmaxf(fmaxf(lo.y - q.y, q.y - hi.y), 0.f),
                      fmaxf(fmaxf(lo.z - q.z, q.z - hi.z), 0.f));
    return dot(gap, gap);
}

// qpos / cpos: the queries' and candidates' bucketed (position, agent index)
// arrays; seed: per agent index an upper bound of its k-th distance; the
// lists go to idx / dist by agent index.  evaluated (may be null): adds the
// (query, candidate) pairs the packed filter ran on.
// sboxes: the boxes of the stages (32 chunks each), tested first, 32 stages
// at a time, so that a block visits only the stages some query may need.
template <int L>
__global__ void __launch_bounds__(kBruteWarps * 32) k_knn_brute3_bucketed(
    const float4* __restrict__ qpos, unsigned nA, const float4* __restrict__ cpos, unsigned nB,
    const float4* __restrict__ boxes, const float4* __restrict__ sboxes, bool self, unsigned k,
    const float* __restrict__ seed, unsigned long long* __restrict__ evaluated,
    unsigned* __restrict__ idx, float* __restrict__ dist) {
    __shared__ __align__(16) float sx[kBruteTile], sy[kBruteTile], sz[kBruteTile];
    __shared__ unsigned sid[kBruteTile];
    __shared__ unsigned wmask[kBruteWarps], smask[kBruteWarps];
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned s0 = (blockIdx.x * kBruteWarps + warp) * kBruteQW;
    V3 q[kBruteQW];
    unsigned qid[kBruteQW];
    unsigned long long px[kBruteQW], py[kBruteQW], pz[kBruteQW];
    WarpList<L> entry[kBruteQW];
    float bound[kBruteQW], seed_bound[kBruteQW];
    unsigned active = 0;
#pragma unroll
    for (unsigned j = 0; j < kBruteQW; ++j) {
        const float4 v = s0 + j < nA ? qpos[s0 + j] : make_float4(0.f, 0.f, 0.f, 0.f);
        qid[j] = s0 + j < nA ? __float_as_uint(v.w) : UINT_MAX;
        const bool act = qid[j] < nA;  // a slot holds an agent index below nA
        active += act;
        q[j] = v3(v);
        px[j] = pack2(q[j].x, q[j].x);
        py[j] = pack2(q[j].y, q[j].y);
        pz[j] = pack2(q[j].z, q[j].z);
        entry[j].init();
        seed_bound[j] = act ? seed_prefilter(seed[qid[j]]) : prefilter_bound(KEY_EMPTY);
        bound[j] = act ? seed_bound[j] : -1.f;
    }
    const float inf = __int_as_float(0x7f800000);
    const unsigned chunks = (nB + 63) / 64, stages = (nB + kBruteTile - 1) / kBruteTile;
    for (unsigned sg = 0; sg < stages; sg += 32) {
        // lane l: may stage sg + l hold a candidate some query of the warp
        // would pass?  (bounds only fall, so the answer stays safe)
        bool swant = false;
        if (sg + lane < stages) {
            const float4 lo = sboxes[2 * (sg + lane)], hi = sboxes[2 * (sg + lane) + 1];
#pragma unroll
            for (unsigned j = 0; j < kBruteQW; ++j) swant |= box_dist_sq(q[j], lo, hi) <= bound[j];
        }
        const unsigned sm = __ballot_sync(0xffffffffu, swant);
        __syncthreads();  // the previous group's reads of smask are done
        if (lane == 0) smask[warp] = sm;
        __syncthreads();
        unsigned visit = 0;
#pragma unroll
        for (unsigned w = 0; w < kBruteWarps; ++w) visit |= smask[w];
        for (; visit; visit &= visit - 1u) {
            const unsigned base = (sg + unsigned(__ffs(visit)) - 1u) * kBruteTile;
            // lane l: may chunk base / 64 + l hold a candidate some query of the
            // warp would pass?  (bounds only fall within the stage)
            const unsigned ch = base / 64 + lane;
            bool want = false;
            if (ch < chunks) {
                const float4 lo = boxes[2 * ch], hi = boxes[2 * ch + 1];
#pragma unroll
                for (unsigned j = 0; j < kBruteQW; ++j)
                    want |= box_dist_sq(q[j], lo, hi) <= bound[j];
            }
            const unsigned mask = __ballot_sync(0xffffffffu, want);
            __syncthreads();  // the previous stage's reads of the staged chunks are done
            if (lane == 0) wmask[warp] = mask;
            __syncthreads();
            unsigned need = 0;
#pragma unroll
            for (unsigned w = 0; w < kBruteWarps; ++w) need |= wmask[w];
            if (need == 0) continue;  // block-uniform
            for (unsigned c = threadIdx.x; c < kBruteTile; c += blockDim.x) {
                if (!((need >> (c / 64)) & 1u)) continue;
                const float4 v =
                    base + c < nB ? cpos[base + c] : make_float4(inf, inf, inf, 0.f);
                sx[c] = v.x;
                sy[c] = v.y;
                sz[c] = v.z;
                sid[c] = __float_as_uint(v.w);
            }
            __syncthreads();
            if (evaluated && lane == 0 && mask)
                atomicAdd(evaluated, (unsigned long long)__popc(mask) * 64u * active);
            const unsigned cnt = min(kBruteTile, nB - base);
            for (unsigned m = mask; m; m &= m - 1u)
                brute_chunk(sx, sy, sz, sid, base, 64u * (unsigned(__ffs(m)) - 1u), cnt, lane,
                            self, k, q, qid, px, py, pz, entry, bound, seed_bound);
        }
    }
#pragma unroll
    for (unsigned j = 0; j < kBruteQW; ++j)
        if (qid[j] < nA) warp_list_store(entry[j], qid[j], nA, k, lane, idx, dist);
}

gs_status launch_knn_brute_bucketed(const float4* qpos, unsigned nA, const float4* cpos,
                                    unsigned nB, float4* boxes, bool self, unsigned k,
                                    const float* seed, unsigned long long* evaluated,
                                    unsigned* idx, float* dist, cudaStream_t st) {
    if (nA == 0) return GS_OK;
    if (k == 0 || k > 64 || seed == nullptr)
        return fail(GS_ERR_UNSUPPORTED, "the bucketed brute force needs 1 <= k <= 64 and a seed");
    const unsigned chunks = (nB + 63) / 64, stages = (chunks + 31) / 32;
    float4* sboxes = boxes + 2 * size_t(chunks);
    if (chunks) {
        k_chunk_boxes<<<(chunks * 32 + kBlock - 1) / kBlock, kBlock, 0, st>>>(cpos, nB, false,
                                                                               boxes);
        k_chunk_boxes<<<(stages * 32 + kBlock - 1) / kBlock, kBlock, 0, st>>>(boxes, chunks, true,
                                                                               sboxes);
    }
    const unsigned per_block = kBruteWarps * kBruteQW, blocks = (nA + per_block - 1) / per_block;
    if (k <= 32)
        k_knn_brute3_bucketed<1><<<blocks, kBruteWarps * 32, 0, st>>>(
            qpos, nA, cpos, nB, boxes, sboxes, self, k, seed, evaluated, idx, dist);
    else
        k_knn_brute3_bucketed<2><<<blocks, kBruteWarps * 32, 0, st>>>(
            qpos, nA, cpos, nB, boxes, sboxes, self, k, seed, evaluated, idx, dist);
    GS_LAUNCHED("knn_brute_bucketed");
    return GS_OK;
}

// Largest |coordinate| per axis of n positions, as float bits (non-negative
// floats order like their bits), into out[0..2] (zeroed by the caller).
__global__ void k_abs_extent(const float4* __restrict__ pos, unsigned n, unsigned* out) {
    unsigned m[3] = {0u, 0u, 0u};
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = pos[i];
        m[0] = max(m[0], __float_as_uint(fabsf(p.x)));
        m[1] = max(m[1], __float_as_uint(fabsf(p.y)));
        m[2] = max(m[2], __float_as_uint(fabsf(p.z)));
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m[a] = max(m[a], __shfl_down_sync(0xffffffffu, m[a], o));
        if ((threadIdx.x & 31) == 0) atomicMax(out + a, m[a]);
    }
}

gs_status abs_extent(const float4* pos, unsigned n, unsigned* d_tmp3, float out[3],
                     cudaStream_t st) {
    unsigned h[3] = {0u, 0u, 0u};
    GS_CUDA(cudaMemsetAsync(d_tmp3, 0, 3 * sizeof(unsigned), st));
    if (n > 0) {
        k_abs_extent<<<std::min(blocks_for(n), 4u * 152u), kBlock, 0, st>>>(pos, n, d_tmp3);
        GS_LAUNCHED("abs_extent");
    }
    GS_CUDA(cudaMemcpyAsync(h, d_tmp3, sizeof(h), cudaMemcpyDeviceToHost, st));
    GS_CUDA(cudaStreamSynchronize(st));
    for (int a = 0; a < 3; ++a) std::memcpy(&out[a], &h[a], 4);
    return GS_OK;
}

gs_status launch_knn_brute(const float4* posA, unsigned nA, const float4* posB, unsigned nB,
                           bool self, unsigned k, const float* seed, unsigned* idx, float* dist,
                           cudaStream_t st) {
    if (nA == 0) return GS_OK;
    if (k == 0 || k > 64) return fail(GS_ERR_UNSUPPORTED, "brute force needs 1 <= k <= 64");
    const unsigned per_block = kBruteWarps * kBruteQW, blocks = (nA + per_block - 1) / per_block;
    if (k <= 32)
        k_knn_brute3<1><<<blocks, kBruteWarps * 32, 0, st>>>(posA, nA, posB, nB, self, k, seed,
                                                             idx, dist);
    else
        k_knn_brute3<2><<<blocks, kBruteWarps * 32, 0, st>>>(posA, nA, posB, nB, self, k, seed,
                                                             idx, dist);
    GS_LAUNCHED("knn_brute");
    return GS_OK;
}

// ---- ExtractData diagnostics (ProcessData.cu:132-237) -------------------------------------
// live (the fused engine's frame, may be null): tiles whose starts the last
// scan wrote; a cell of another tile is empty.
__device__ __forceinline__ bool frame_cell_live(const unsigned* live, unsigned c) {
    return live == nullptr || live[c / kScanTile] != 0u;
}

__global__ void k_cell_density(const unsigned* __restrict__ start, unsigned C,
                               const unsigned* __restrict__ live, unsigned* __restrict__ out) {
    const unsigned c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < C) out[c] = frame_cell_live(live, c) ? start[c + 1] - start[c] : 0u;
}

// A cell's agents are added in ascending index, the order the reference's
// stable sort leaves them in; this database's counting sort orders a cell's
// slots arbitrarily, so the cell's thread picks its agents by increasing
// index (quadratic in the cell's count: a diagnostic, not a step kernel).
__global__ void k_cell_avg_velocity(const unsigned* __restrict__ start,
                                    const unsigned* __restrict__ sorted, unsigned C,
                                    const float4* __restrict__ dir,
                                    const float* __restrict__ speed, float3* __restrict__ out) {
    const unsigned c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const unsigned s0 = start[c], s1 = start[c + 1];
    V3 sum = v3(0.f, 0.f, 0.f);
    unsigned last = 0;
    for (unsigned t = 0; t < s1 - s0; ++t) {
        unsigned next = UINT_MAX;
        for (unsigned s = s0; s < s1; ++s) {
            const unsigned id = sorted[s];
            if ((t == 0 || id > last) && id < next) next = id;
        }
        last = next;
        sum = add(sum, mul(v3(dir[next]), speed[next]));
    }
    const V3 avg = s1 > s0 ? dvd(sum, float(s1 - s0)) : v3(0.f, 0.f, 0.f);
    out[c] = make_float3(avg.x, avg.y, avg.z);
}

// The same average over the fused step's frame: slot s of the start-of-step
// buckets holds the agent whose new state the step wrote to A[s] (its index
// in f0.w, heading and speed in f1).  A cell's agents belong to one scene, so
// ascending index is the reference's order here too.
__global__ void k_cell_avg_velocity_frame(const unsigned* __restrict__ start, unsigned C,
                                          const unsigned* __restrict__ live,
                                          const float4* __restrict__ f0,
                                          const float4* __restrict__ f1,
                                          float3* __restrict__ out) {
    const unsigned c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const bool on = frame_cell_live(live, c);
    const unsigned s0 = on ? start[c] : 0u, s1 = on ? start[c + 1] : 0u;
    V3 sum = v3(0.f, 0.f, 0.f);
    unsigned last = 0;
    for (unsigned t = 0; t < s1 - s0; ++t) {
        unsigned next = UINT_MAX, at = s0;
        for (unsigned s = s0; s < s1; ++s) {
            const unsigned id = __float_as_uint(f0[s].w);
            if ((t == 0 || id > last) && id < next) {
                next = id;
                at = s;
            }
        }
        last = next;
        const float4 h = f1[at];
        sum = add(sum, mul(v3(h), h.w));
    }
    const V3 avg = s1 > s0 ? dvd(sum, float(s1 - s0)) : v3(0.f, 0.f, 0.f);
    out[c] = make_float3(avg.x, avg.y, avg.z);
}

gs_status launch_frame_cell_density(const unsigned* start, const unsigned* live, unsigned C,
                                    unsigned* out, cudaStream_t st) {
    if (C == 0) return GS_OK;
    k_cell_density<<<blocks_for(C), kBlock, 0, st>>>(start, C, live, out);
    GS_LAUNCHED("cell_density");
    return GS_OK;
}

gs_status launch_frame_cell_avg_velocity(const unsigned* start, const unsigned* live,
                                         unsigned C, const float4* f0, const float4* f1,
                                         float3* out, cudaStream_t st) {
    if (C == 0) return GS_OK;
    k_cell_avg_velocity_frame<<<blocks_for(C), kBlock, 0, st>>>(start, C, live, f0, f1, out);
    GS_LAUNCHED("cell_avg_velocity");
    return GS_OK;
}

gs_status launch_cell_density(const Database& db, unsigned* out, cudaStream_t st) {
    if (db.cells == 0) return GS_OK;
    k_cell_density<<<blocks_for(db.cells), kBlock, 0, st>>>(db.start, db.cells, nullptr, out);
    GS_LAUNCHED("cell_density");
    return GS_OK;
}

gs_status launch_cell_avg_velocity(const Database& db, const float4* dir, const float* speed,
                                   float3* out, cudaStream_t st) {
    if (db.cells == 0) return GS_OK;
    k_cell_avg_velocity<<<blocks_for(db.cells), kBlock, 0, st>>>(db.start, db.sorted, db.cells,
                                                                  dir, speed, out);
    GS_LAUNCHED("cell_avg_velocity");
    return GS_OK;
}

// ---- WrapWorldCUDAKernel.cu:11-48 ---------------------------------------------------
__global__ void k_wrap(float4* pos, unsigned n, float wx, float wy, float wz, int mode) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float ws[3] = {wx, wy, wz};
    pos[i] = f4(wrap_world(v3(pos[i]), ws, mode), 0.f);
}

gs_status launch_wrap(float4* pos, unsigned n, const float ws[3], int mode, cudaStream_t st) {
    if (n == 0) return GS_OK;
    k_wrap<<<blocks_for(n), kBlock, 0, st>>>(pos, n, ws[0], ws[1], ws[2], mode);
    GS_LAUNCHED("wrap_world");
    return GS_OK;
}

// ---- one behaviour per launch ----------------------------------------------------------
__device__ __forceinline__ Self load_self(const GroupView& g, unsigned i) {
    Self s;
    s.pos = v3(g.position[i]);
    s.dir = v3(g.direction[i]);
    const float3 sd = g.side[i], u = g.up[i];
    s.side = v3(sd.x, sd.y, sd.z);
    s.up = v3(u.x, u.y, u.z);
    s.speed = g.speed[i];
    s.radius = g.radius[i];
    s.max_speed = g.max_speed[i];
    s.max_force = g.max_force[i];
    s.mass = g.mass[i];
    return s;
}

__global__ void k_flock(int kind, GroupView g, const unsigned* __restrict__ knn, unsigned k,
                        OtherView o, FlockParams fp) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    unsigned applied = g.applied[i];
    if (applied & fp.mask) return;
    const V3 pos = v3(g.position[i]), dir = v3(g.direction[i]);
    FlockAcc acc;
    flock_init(acc);
    for (unsigned s = 0; s < k; ++s) {
        const unsigned b = knn[i + size_t(s) * g.n];
        if (b >= o.n) break;
        const V3 bp = v3(o.position[b]);
        const V3 offset = sub(bp, pos);
        const float dsq = dot(offset, offset);
        const float d = sqrtf(dsq);
        if (kind == 0) separation_add(acc, fp, dir, offset, dsq, d);
        else if (kind == 1) alignment_add(acc, fp, dir, offset, d, v3(o.direction[b]));
        else cohesion_add(acc, fp, dir, offset, d, bp);
    }
    Self me;
    me.pos = pos;
    me.dir = dir;
    V3 steer = v3(g.steering[i]);
    flock_finish(kind, acc, fp, me, applied, steer);
    g.steering[i] = f4(steer, 0.f);
    g.applied[i] = applied;
}

gs_status launch_flock(int kind, GroupView g, const unsigned* knn, unsigned k, OtherView o,
                       float min_d, float max_d, float cos_max, float w, unsigned mask,
                       cudaStream_t st) {
    if (g.n == 0) return GS_OK;
    const FlockParams fp{min_d, max_d, cos_max, w, mask};
    k_flock<<<blocks_for(g.n), kBlock, 0, st>>>(kind, g, knn, k, o, fp);
    GS_LAUNCHED("steer_flock");
    return GS_OK;
}

__global__ void k_seek(GroupView g, float tx, float ty, float tz, float w, unsigned mask) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    unsigned applied = g.applied[i];
    if (applied & mask) return;
    Self me;
    me.pos = v3(g.position[i]);
    me.dir = v3(g.direction[i]);
    V3 steer = v3(g.steering[i]);
    seek_finish(v3(tx, ty, tz), w, mask, me, applied, steer);
    g.steering[i] = f4(steer, 0.f);
    g.applied[i] = applied;
}

gs_status launch_seek(GroupView g, const float target[3], float w, unsigned mask,
                      cudaStream_t st) {
    if (g.n == 0) return GS_OK;
    k_seek<<<blocks_for(g.n), kBlock, 0, st>>>(g, target[0], target[1], target[2], w, mask);
    GS_LAUNCHED("steer_seek");
    return GS_OK;
}

__global__ void k_follow_path(GroupView g, PathDev path, float prediction_time, float w,
                              unsigned mask) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    unsigned applied = g.applied[i];
    if (applied & mask) return;
    Self me;
    me.pos = v3(g.position[i]);
    me.dir = v3(g.direction[i]);
    me.speed = g.speed[i];
    V3 steer = v3(g.steering[i]);
    follow_path_finish(path, prediction_time, w, mask, me, applied, steer);
    g.steering[i] = f4(steer, 0.f);
    g.applied[i] = applied;
}

gs_status launch_follow_path(GroupView g, const PathDev& path, float prediction_time, float w,
                             unsigned mask, cudaStream_t st) {
    if (g.n == 0) return GS_OK;
    k_follow_path<<<blocks_for(g.n), kBlock, 0, st>>>(g, path, prediction_time, w, mask);
    GS_LAUNCHED("steer_follow_path");
    return GS_OK;
}

__global__ void k_avoid_close(GroupView g, const unsigned* __restrict__ knn,
                              const float* __restrict__ knn_dist, unsigned k, OtherView o,
                              float min_sep, float w, unsigned mask) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    unsigned applied = g.applied[i];
    if (applied & mask) return;
    const Self me = load_self(g, i);
    CloseAcc acc;
    close_init(acc);
    for (unsigned s = 0; s < k; ++s) {
        const unsigned b = knn[i + size_t(s) * g.n];
        if (b >= o.n) break;
        close_add(acc, me, min_sep, knn_dist[i + size_t(s) * g.n], v3(o.position[b]),
                  o.radius[b]);
        if (acc.found) break;
    }
    V3 steer = v3(g.steering[i]);
    close_finish(acc, w, mask, applied, steer);
    g.steering[i] = f4(steer, 0.f);
    g.applied[i] = applied;
}

__global__ void k_avoid(GroupView g, const unsigned* __restrict__ knn, unsigned k, OtherView o,
                        float min_time, float w, unsigned mask) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    unsigned applied = g.applied[i];
    if (applied & (mask | AVOID_CLOSE_NEIGHBORS_BIT)) return;
    const Self me = load_self(g, i);
    AvoidAcc acc;
    avoid_init(acc, min_time);
    for (unsigned s = 0; s < k; ++s) {
        const unsigned b = knn[i + size_t(s) * g.n];
        if (b >= o.n) break;
        avoid_add(acc, me, b, v3(o.position[b]), v3(o.direction[b]), o.speed[b], o.radius[b]);
    }
    if (acc.threat == UINT_MAX) return;
    V3 steer = v3(g.steering[i]);
    avoid_finish(acc, w, mask, me, applied, steer);
    g.steering[i] = f4(steer, 0.f);
    g.applied[i] = applied;
}

gs_status launch_avoid_neighbors(GroupView g, const unsigned* knn, const float* knn_dist,
                                 unsigned k, OtherView o, float min_time, float min_sep,
                                 bool avoid_close, float w, unsigned mask, cudaStream_t st) {
    if (g.n == 0) return GS_OK;
    if (avoid_close)
        k_avoid_close<<<blocks_for(g.n), kBlock, 0, st>>>(g, knn, knn_dist, k, o, min_sep, w,
                                                          mask);
    k_avoid<<<blocks_for(g.n), kBlock, 0, st>>>(g, knn, k, o, min_time, w, mask);
    GS_LAUNCHED("steer_avoid_neighbors");
    return GS_OK;
}

__global__ void k_avoid_walls(GroupView g, const unsigned* __restrict__ knw, unsigned kw,
                              const float4* __restrict__ ls, const float4* __restrict__ le,
                              const float4* __restrict__ ln, unsigned n_lines, float min_time,
                              float w, unsigned mask) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    unsigned applied = g.applied[i];
    if (applied & mask) return;
    Self me = load_self(g, i);
    WallAcc acc;
    walls_init(acc, me, min_time);
    for (unsigned s = 0; s < kw; ++s) {
        const unsigned line = knw[i + size_t(s) * g.n];
        if (line >= n_lines) break;
        walls_add(acc, me, line, v3(ls[line]), v3(le[line]), v3(ln[line]));
    }
    V3 steer = v3(g.steering[i]);
    walls_finish(acc, w, mask, me, applied, steer);
    g.steering[i] = f4(steer, 0.f);
    g.position[i] = f4(me.pos, 0.f);
    g.direction[i] = f4(me.dir, 0.f);
    g.applied[i] = applied;
}

gs_status launch_avoid_walls(GroupView g, const unsigned* knw, unsigned kw, const float4* start,
                             const float4* end, const float4* normal, unsigned n_lines,
                             float min_time, float w, unsigned mask, cudaStream_t st) {
    if (g.n == 0) return GS_OK;
    k_avoid_walls<<<blocks_for(g.n), kBlock, 0, st>>>(g, knw, kw, start, end, normal, n_lines,
                                                      min_time, w, mask);
    GS_LAUNCHED("steer_avoid_walls");
    return GS_OK;
}

__global__ void k_update(GroupView g, float dt) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    Self me = load_self(g, i);
    integrate(me, v3(g.steering[i]), dt);
    g.side[i] = make_float3(me.side.x, me.side.y, me.side.z);
    g.up[i] = make_float3(me.up.x, me.up.y, me.up.z);
    g.direction[i] = f4(me.dir, 0.f);
    g.position[i] = f4(me.pos, 0.f);
    g.steering[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    g.speed[i] = me.speed;
    g.applied[i] = 0u;
}

gs_status launch_update(GroupView g, float dt, cudaStream_t st) {
    if (g.n == 0) return GS_OK;
    k_update<<<blocks_for(g.n), kBlock, 0, st>>>(g, dt);
    GS_LAUNCHED("update_group");
    return GS_OK;
}

// updateGroupWithAntiPenetration (UpdateCUDAKernelNew.cu:95-268): the update
// with the walls' anti-penetration.  Behaviour kept from the reference kernel:
// the wall list is read row-major, knl[i*k + s] (:149-150), although
// findKNearestNeighbors writes it column-major; the overlap test measures the
// distance to lineStart + (lineEnd - lineStart), the segment's end, because
// ClosestPointOnLine's clamp(0.f, 1.f, t) returns 1 (:67-80); the last listed
// line within the radius pushes the agent out (:215-229); the nearest crossing
// of the move turns the velocity parallel to that wall (:201-237); applied
// bits are kept.  An agent whose new speed is 0 keeps its side vector.
__global__ void k_update_antipen_wall(GroupView g, const unsigned* __restrict__ knl, unsigned k,
                                      const float4* __restrict__ start,
                                      const float4* __restrict__ end,
                                      const float4* __restrict__ normal, unsigned n_lines,
                                      float dt) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    Self me = load_self(g, i);
    const V3 steer = truncate_length(v3(g.steering[i]), me.max_force);
    const V3 acc = dvd(steer, me.mass);
    V3 vel = add(mul(me.dir, me.speed), mul(acc, dt));
    vel = truncate_length(vel, me.max_speed);
    const V3 future = add(me.pos, mul(vel, dt));
    const float r = me.radius;
    float line_d = FLT_MAX, hit_d = FLT_MAX;
    unsigned line = UINT_MAX, hit = UINT_MAX;
    V3 line_n = v3(0.f, 0.f, 0.f), hit_n = v3(0.f, 0.f, 0.f);
    for (unsigned s = 0; s < k; ++s) {
        const unsigned li = knl[size_t(i) * k + s];
        if (li >= n_lines) break;
        const V3 ls = v3(start[li]), le = v3(end[li]), ln = v3(normal[li]);
        V3 ip;
        if (lines_intersect(me.pos, future, ls, le, ip)) {
            const float d = distance(me.pos, ip);
            if (d < hit_d) {
                hit_d = d;
                hit = li;
                hit_n = ln;
            }
        }
        const V3 o = sub(add(ls, sub(le, ls)), me.pos);
        const float dsq = dot(o, o);
        if (dsq < r * r) {
            line_d = sqrtf(dsq);
            line = li;
            line_n = ln;
        }
    }
    unsigned applied = g.applied[i];
    if (line != UINT_MAX) {
        me.pos = add(me.pos, mul(neg(line_n), line_d - r));
        applied |= ANTI_PENETRATION_WALL;
    }
    if (hit != UINT_MAX) {
        vel = perpendicular_component(vel, hit_n);
        applied |= ANTI_PENETRATION_WALL;
    }
    me.speed = length(vel);
    if (me.speed > 0.f) {
        me.dir = dvd(vel, me.speed);
        me.side = normalize(cross(me.dir, me.up));
        me.up = cross(me.side, me.dir);
    }
    me.pos = add(me.pos, mul(vel, dt));
    g.side[i] = make_float3(me.side.x, me.side.y, me.side.z);
    g.up[i] = make_float3(me.up.x, me.up.y, me.up.z);
    g.direction[i] = f4(me.dir, 0.f);
    g.position[i] = f4(me.pos, 0.f);
    g.steering[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    g.speed[i] = me.speed;
    g.applied[i] = applied;
}

gs_status launch_update_antipen_wall(GroupView g, const unsigned* knl, unsigned k,
                                     const float4* start, const float4* end,
                                     const float4* normal, unsigned n_lines, float dt,
                                     cudaStream_t st) {
    if (g.n == 0) return GS_OK;
    k_update_antipen_wall<<<blocks_for(g.n), kBlock, 0, st>>>(g, knl, k, start, end, normal,
                                                              n_lines, dt);
    GS_LAUNCHED("update_group_with_antipenetration");
    return GS_OK;
}

// antiPenetrationWall (AntiPenetrationWallCUDAKernel.cu:52-134): an agent
// whose move velocity * dt crosses a listed wall turns its heading parallel
// to the nearest crossed wall.  As the reference kernel: every agent is
// tested (its early-out `! applied & KERNEL_AVOID_WALLS_BIT`, :73, is never
// true), the wall list is read row-major (:88-91), every direction is
// rewritten with w = 0 (:133).
__global__ void k_antipen_wall(GroupView g, const unsigned* __restrict__ knl, unsigned k,
                               const float4* __restrict__ start, const float4* __restrict__ end,
                               const float4* __restrict__ normal, unsigned n_lines, float dt) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    const V3 pos = v3(g.position[i]);
    V3 dir = v3(g.direction[i]);
    const V3 future = add(pos, mul(mul(dir, g.speed[i]), dt));
    float hit_d = FLT_MAX;
    unsigned hit = UINT_MAX;
    for (unsigned s = 0; s < k; ++s) {
        const unsigned li = knl[size_t(i) * k + s];
        if (li >= n_lines) break;
        V3 ip;
        if (lines_intersect(pos, future, v3(start[li]), v3(end[li]), ip)) {
            const float d = distance(pos, ip);
            if (d < hit_d) {
                hit_d = d;
                hit = li;
            }
        }
    }
    if (hit != UINT_MAX) {
        dir = normalize(perpendicular_component(dir, v3(normal[hit])));
        g.applied[i] |= ANTI_PENETRATION_WALL;
    }
    g.direction[i] = f4(dir, 0.f);
}

gs_status launch_antipen_wall(GroupView g, const unsigned* knl, unsigned k, const float4* start,
                              const float4* end, const float4* normal, unsigned n_lines,
                              float dt, cudaStream_t st) {
    if (g.n == 0) return GS_OK;
    k_antipen_wall<<<blocks_for(g.n), kBlock, 0, st>>>(g, knl, k, start, end, normal, n_lines,
                                                       dt);
    GS_LAUNCHED("anti_penetration_wall");
    return GS_OK;
}

// One group's behaviour calls of a MultiGroup frame (Group::update,
// plugins/MultiGroup.cpp:558-601), per agent in the calls' order: avoid the
// neighbours of every other group (close pass, then main pass, per group,
// :573-580), separation from every group (:583-588), alignment and cohesion
// with this group (:590-591), then path following and seek of the path's
// second point when the group has a path (:593-597).  Each call keeps its own
// mask test and normalisation, and the applied bits accumulate from call to
// call, as the per-call kernels do.  Only steering and applied bits are
// written (positions move in the update that follows), so every read of a
// group's state sees the state the per-call kernels see.
__global__ void k_multigroup_steer(MultiSteer M) {
    const unsigned a = blockIdx.x * blockDim.x + threadIdx.x;
    const GroupView& g = M.g;
    if (a >= g.n) return;
    const unsigned n = g.n;
    unsigned applied = g.applied[a];
    V3 steer = v3(g.steering[a]);
    const Self me = load_self(g, a);
    for (unsigned j = 0; j < M.n_groups; ++j) {
        if (j == M.self) continue;
        const OtherView& o = M.o[j];
        const unsigned* idx = M.idx[j];
        if (M.avoid_close && !(applied & M.mask_avoid)) {
            CloseAcc acc;
            close_init(acc);
            for (unsigned s = 0; s < M.k[j]; ++s) {
                const unsigned b = idx[a + size_t(s) * n];
                if (b >= o.n) break;
                close_add(acc, me, M.min_sep, M.dist[j][a + size_t(s) * n], v3(o.position[b]),
                          o.radius[b]);
                if (acc.found) break;
            }
            close_finish(acc, M.w_avoid, M.mask_avoid, applied, steer);
        }
        if (!(applied & (M.mask_avoid | AVOID_CLOSE_NEIGHBORS_BIT))) {
            AvoidAcc acc;
            avoid_init(acc, M.min_time);
            for (unsigned s = 0; s < M.k[j]; ++s) {
                const unsigned b = idx[a + size_t(s) * n];
                if (b >= o.n) break;
                avoid_add(acc, me, b, v3(o.position[b]), v3(o.direction[b]), o.speed[b],
                          o.radius[b]);
            }
            if (acc.threat != UINT_MAX) avoid_finish(acc, M.w_avoid, M.mask_avoid, me, applied, steer);
        }
    }
    for (unsigned j = 0; j < M.n_groups; ++j) {
        if (applied & M.sep.mask) continue;
        const OtherView& o = M.o[j];
        FlockAcc acc;
        flock_init(acc);
        for (unsigned s = 0; s < M.k[j]; ++s) {
            const unsigned b = M.idx[j][a + size_t(s) * n];
            if (b >= o.n) break;
            const V3 offset = sub(v3(o.position[b]), me.pos);
            const float dsq = dot(offset, offset);
            separation_add(acc, M.sep, me.dir, offset, dsq, sqrtf(dsq));
        }
        flock_finish(0, acc, M.sep, me, applied, steer);
    }
    for (int kind = 1; kind <= 2; ++kind) {
        const FlockParams& fp = kind == 1 ? M.ali : M.coh;
        if (applied & fp.mask) continue;
        const OtherView& o = M.o[M.self];
        FlockAcc acc;
        flock_init(acc);
        for (unsigned s = 0; s < M.k[M.self]; ++s) {
            const unsigned b = M.idx[M.self][a + size_t(s) * n];
            if (b >= o.n) break;
            const V3 bp = v3(o.position[b]);
            const V3 offset = sub(bp, me.pos);
            const float d = sqrtf(dot(offset, offset));
            if (kind == 1) alignment_add(acc, fp, me.dir, offset, d, v3(o.direction[b]));
            else cohesion_add(acc, fp, me.dir, offset, d, bp);
        }
        flock_finish(kind, acc, fp, me, applied, steer);
    }
    if (M.has_path) {
        if (!(applied & M.mask_path))
            follow_path_finish(M.path, M.path_time, M.w_path, M.mask_path, me, applied, steer);
        if (!(applied & M.mask_seek))
            seek_finish(v3(M.seek_target[0], M.seek_target[1], M.seek_target[2]), M.w_seek,
                        M.mask_seek, me, applied, steer);
    }
    g.steering[a] = f4(steer, 0.f);
    g.applied[a] = applied;
}

gs_status launch_multigroup_steer(const MultiSteer& M, cudaStream_t st) {
    if (M.g.n == 0) return GS_OK;
    k_multigroup_steer<<<blocks_for(M.g.n), kBlock, 0, st>>>(M);
    GS_LAUNCHED("multigroup_steer");
    return GS_OK;
}

// AntiPenetrationAgentsCUDAKernel.cu:72-108.  Positions are read from the
// group and written to pos_out (the reference's m_pdPositionNew); the other
// group's applied bits are read from a snapshot taken before the launch (the
// reference reads them while this kernel sets bit 13 on the same array).
__global__ void k_antipen(GroupView g, const unsigned* __restrict__ knn,
                          const float* __restrict__ knn_dist, OtherView o,
                          const unsigned* __restrict__ applied_b, float4* __restrict__ out,
                          unsigned mask) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    const float4 p4 = g.position[i];
    out[i] = p4;
    unsigned applied = g.applied[i];
    if (applied & mask) return;
    const unsigned b = knn[i];
    if (b >= o.n) return;
    const float sum_radii = g.radius[i] + o.radius[b];
    const float overlap = sum_radii - knn_dist[i];
    if (overlap < 0.f) return;
    const V3 pos = v3(p4);
    const V3 offset = sub(pos, v3(o.position[b]));
    const V3 unit = normalize(offset);
    const float move = (applied_b[b] & mask) ? overlap : 0.5f * overlap;
    out[i] = f4(add(pos, mul(unit, move)), 0.f);
    g.applied[i] = applied | ANTI_PENETRATION_AGENT;
}

gs_status launch_antipenetration(GroupView g, const unsigned* knn, const float* knn_dist,
                                 unsigned k, OtherView o, const unsigned* applied_snapshot,
                                 float4* pos_out, unsigned mask, cudaStream_t st) {
    (void)k;
    if (g.n == 0) return GS_OK;
    k_antipen<<<blocks_for(g.n), kBlock, 0, st>>>(g, knn, knn_dist, o, applied_snapshot,
                                                  pos_out, mask);
    GS_LAUNCHED("anti_penetration_agents");
    GS_CUDA(cudaMemcpyAsync(g.position, pos_out, size_t(g.n) * sizeof(float4),
                            cudaMemcpyDeviceToDevice, st));
    return GS_OK;
}

}  // namespace gs
