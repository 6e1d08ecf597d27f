// Device code of the counting sort's exclusive scan over per-cell counts,
// shared by the scan kernels and the persistent step: a tile is kScanTile
// counts, scanned by one block of kBlock threads.
#pragma once

#include "gs_launch.h"

namespace gs {

constexpr unsigned kScanItems = 16;
constexpr unsigned kScanTile = kBlock * kScanItems;

__device__ __forceinline__ unsigned block_exclusive_sum(unsigned v, unsigned* warp_sums,
                                                        unsigned& total) {
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= unsigned(o)) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned w = lane < kBlock / 32 ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= unsigned(o)) w += y;
        }
        if (lane < kBlock / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    total = warp_sums[kBlock / 32 - 1];
    const unsigned before = warp ? warp_sums[warp - 1] : 0u;
    __syncthreads();
    return before + x - v;
}

// Loads tile t of count[] into shared memory (coalesced), returns this
// thread's run of kScanItems consecutive items through `items`.
__device__ __forceinline__ void load_tile(const unsigned* count, unsigned C, unsigned t,
                                          unsigned* sh, unsigned items[kScanItems]) {
    const unsigned base = t * kScanTile;
#pragma unroll
    for (unsigned j = 0; j < kScanItems; ++j) {
        const unsigned i = j * kBlock + threadIdx.x;
        sh[i + i / 32] = (base + i < C) ? count[base + i] : 0u;
    }
    __syncthreads();
#pragma unroll
    for (unsigned j = 0; j < kScanItems; ++j) {
        const unsigned i = threadIdx.x * kScanItems + j;
        items[j] = sh[i + i / 32];
    }
    __syncthreads();
}

// Tile t's total into tile[t] (sh: kScanTile + kScanTile / 32 words, ws:
// kBlock / 32 words of shared memory).
__device__ __forceinline__ void scan_reduce_tile(const unsigned* __restrict__ count, unsigned C,
                                                 unsigned t, unsigned* sh, unsigned* ws,
                                                 unsigned* __restrict__ tile) {
    unsigned items[kScanItems];
    load_tile(count, C, t, sh, items);
    unsigned s = 0;
#pragma unroll
    for (unsigned j = 0; j < kScanItems; ++j) s += items[j];
    unsigned total;
    block_exclusive_sum(s, ws, total);
    if (threadIdx.x == 0) tile[t] = total;
    __syncthreads();
}

// Tile t's starts (its prefix summed from the totals of the tiles before it),
// zeroing its counts; the last tile also writes start[C].
__device__ __forceinline__ void scan_apply_tile(unsigned* __restrict__ count, unsigned C,
                                                const unsigned* __restrict__ tile,
                                                unsigned* __restrict__ start, unsigned T,
                                                unsigned t, unsigned* sh, unsigned* ws) {
    unsigned before = 0;
    for (unsigned u = threadIdx.x; u < t; u += blockDim.x) before += tile[u];
    unsigned prefix_total;
    block_exclusive_sum(before, ws, prefix_total);
    unsigned items[kScanItems];
    load_tile(count, C, t, sh, items);
    unsigned sum = 0;
#pragma unroll
    for (unsigned j = 0; j < kScanItems; ++j) sum += items[j];
    unsigned total;
    unsigned run = block_exclusive_sum(sum, ws, total) + prefix_total;
#pragma unroll
    for (unsigned j = 0; j < kScanItems; ++j) {
        const unsigned i = threadIdx.x * kScanItems + j;
        sh[i + i / 32] = run;
        run += items[j];
    }
    __syncthreads();
    const unsigned base = t * kScanTile;
#pragma unroll
    for (unsigned j = 0; j < kScanItems; ++j) {
        const unsigned i = j * kBlock + threadIdx.x;
        if (base + i < C) {
            start[base + i] = sh[i + i / 32];
            count[base + i] = 0u;
        }
    }
    if (t == T - 1 && threadIdx.x == 0) start[C] = prefix_total + total;
    __syncthreads();
}

// The fused engine's scan, over tiles near agents only.  tile[] holds each
// tile's exact total, added by the step's counting atomics themselves (after
// a whole recount, whose agents come in no spatial order, by a reduce pass);
// the step reads the starts of cells at most `reach` tiles from an
// agent's own tile (its box's rows, scan_reach_tiles).  So tile t's starts
// are written, and its counts zeroed, only when a tile within `reach` of it
// holds agents; live[t] records which.  The other tiles' counts are already
// zero and their starts, stale, are not read.  reach >= kBlock / 2: every
// tile is written.
__device__ __forceinline__ void scan_apply_sparse_tile(unsigned* __restrict__ count, unsigned C,
                                                       const unsigned* __restrict__ tile,
                                                       unsigned* __restrict__ start, unsigned T,
                                                       unsigned t, unsigned reach,
                                                       unsigned* __restrict__ live, unsigned* sh,
                                                       unsigned* ws) {
    unsigned v = reach >= kBlock / 2 ? 1u : 0u;
    if (!v && threadIdx.x <= 2 * reach) {
        const long long u = (long long)t - (long long)reach + (long long)threadIdx.x;
        if (u >= 0 && u < (long long)T) v = tile[u];
    }
    const int need = __syncthreads_or(v != 0u);
    if (threadIdx.x == 0) live[t] = need ? 1u : 0u;
    if (!need) return;
    scan_apply_tile(count, C, tile, start, T, t, sh, ws);
}

}  // namespace gs
