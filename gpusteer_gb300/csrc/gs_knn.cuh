// Register-resident k-nearest-neighbour list and the binned candidate scan.
//
// Semantics (KNNBinningV2Kernel.cu:470-515, KNNBruteForceCudaKernel.cu:245-271):
// the k smallest (distance, agent index) pairs among the candidates, in
// ascending order; unused slots hold (FLT_MAX, UINT_MAX).  Distances are
// non-negative binary32, so the bit pattern of the distance followed by the
// index is a 64-bit key whose unsigned order is exactly that total order.
#pragma once

#include "gs_math.cuh"

namespace gs {

__device__ __forceinline__ unsigned long long knn_key(float d, unsigned id) {
    return (static_cast<unsigned long long>(__float_as_uint(d)) << 32) | id;
}
__device__ __forceinline__ float key_dist(unsigned long long key) { return __uint_as_float(unsigned(key >> 32)); }
__device__ __forceinline__ unsigned key_id(unsigned long long key) { return unsigned(key); }
constexpr unsigned long long KEY_EMPTY = (0x7f7fffffull << 32) | 0xffffffffull;  // (FLT_MAX, UINT_MAX)

// KMAX slots in registers.  For k < KMAX the first KMAX - k slots hold a
// sentinel key 0 that no candidate can get below, so the k real entries sit
// in slots KMAX-k .. KMAX-1 (ascending) and the admission threshold is always
// the last slot: every register index is a compile-time constant.  Each entry
// carries a payload (the neighbour's slot in the bucketed arrays).
template <int KMAX>
struct KList {
    unsigned long long key[KMAX];
    unsigned slot[KMAX];

    __device__ __forceinline__ void init(int k) {
#pragma unroll
        for (int i = 0; i < KMAX; ++i) {
            key[i] = (i < KMAX - k) ? 0ull : KEY_EMPTY;
            slot[i] = UINT_MAX;
        }
    }

    __device__ __forceinline__ void insert(unsigned long long c, unsigned s) {
        if (!(c < key[KMAX - 1])) return;
        // Branch-free shift-insert: slot i takes slot i-1 when c is below it,
        // c itself when c falls between i-1 and i, else keeps its value.
        bool lt_prev = c < key[0];
        unsigned long long prev_key = key[0];
        unsigned prev_slot = slot[0];
        if (lt_prev) {
            key[0] = c;
            slot[0] = s;
        }
#pragma unroll
        for (int i = 1; i < KMAX; ++i) {
            const unsigned long long cur_key = key[i];
            const unsigned cur_slot = slot[i];
            const bool lt_cur = c < cur_key;
            key[i] = lt_prev ? prev_key : (lt_cur ? c : cur_key);
            slot[i] = lt_prev ? prev_slot : (lt_cur ? s : cur_slot);
            prev_key = cur_key;
            prev_slot = cur_slot;
            lt_prev = lt_cur;
        }
    }

    // Calls f(rank, key, slot) for the k entries in ascending order.
    template <class F>
    __device__ __forceinline__ void for_each(int k, F&& f) const {
#pragma unroll
        for (int i = 0; i < KMAX; ++i)
            if (i >= KMAX - k) f(i - (KMAX - k), key[i], slot[i]);
    }
};

// Candidate ranges of the clamped (2r+1)^d box of cells around (ix, iy, iz):
// one contiguous run of sorted slots per (y, z) row of cells, because labels
// are x-fastest.  The set equals the reference's de-duplicated neighbour-cell
// table (KNNBinningV2Kernel.cu:102-248).
struct Box {
    unsigned x0, x1, y0, y1, z0, z1;
};
GS_HD Box cell_box(const Grid& g, unsigned ix, unsigned iy, unsigned iz, unsigned r) {
    Box b;
    b.x0 = ix >= r ? ix - r : 0u;
    b.x1 = min(ix + r, g.wc[0] - 1);
    b.y0 = iy >= r ? iy - r : 0u;
    b.y1 = min(iy + r, g.wc[1] - 1);
    b.z0 = iz >= r ? iz - r : 0u;
    b.z1 = min(iz + r, g.wc[2] - 1);
    return b;
}

// Scans every candidate of `box` in the bucketed arrays of group B:
// pos_id[slot] = (x, y, z, index bits), cell_start[cell_offset + c] .. [+1].
// Skips the candidate whose index equals self_id (pass UINT_MAX for none).
template <int KMAX>
__device__ __forceinline__ void knn_scan_box(KList<KMAX>& L, V3 p, unsigned self_id,
                                             const Grid& g, const Box& b, unsigned cell_offset,
                                             const unsigned* __restrict__ cell_start,
                                             const float4* __restrict__ pos_id) {
    for (unsigned cy = b.y0; cy <= b.y1; ++cy) {
        for (unsigned cz = b.z0; cz <= b.z1; ++cz) {
            const unsigned c0 = cell_offset + cell_label(g, b.x0, cy, cz);
            const unsigned c1 = cell_offset + cell_label(g, b.x1, cy, cz) + 1;
            const unsigned s0 = __ldg(cell_start + c0), s1 = __ldg(cell_start + c1);
            for (unsigned s = s0; s < s1; ++s) {
                const float4 q = __ldg(pos_id + s);
                const unsigned id = __float_as_uint(q.w);
                if (id == self_id) continue;
                const float d = distance(p, v3(q));
                L.insert(knn_key(d, id), s);
            }
        }
    }
}

}  // namespace gs
