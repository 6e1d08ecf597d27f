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

// ---- fast scan: 32-bit keys of squared distances --------------------------------
// key = bits of the SQUARED distance (no square root per candidate) with the
// low EBITS = log2(ENUM) mantissa bits replaced by the candidate's enumeration
// index e.  T = key >> EBITS is the squared distance truncated to units of
// 2^EBITS ulps.  Square root rounded to nearest is monotone, so smaller keys
// never have larger distances, and two candidates whose T differ by two units
// or more have DIFFERENT distances: their squared distances differ by more
// than 2^EBITS ulps, a relative step of at least 2^(EBITS - 24), which leaves
// at least 2^(EBITS - 2) ulps between the roots before rounding.  So the k
// smallest keys are the k nearest candidates in (distance, index) order,
// except where entries' T are within one unit of each other:
//   - adjacent list entries that close are compared exactly ((distance,
//     index) from their positions: near_pairs_ordered), and the agent is
//     redone if they are out of order;
//   - a candidate left out of a full list with T within one unit of the k-th
//     entry's, or more than ENUM candidates, sends the agent to the exact
//     64-bit list (knn_scan_box).
constexpr unsigned KEY32_EMPTY = 0xffffffffu;

template <unsigned N>
struct Log2 {
    static constexpr unsigned value = 1 + Log2<N / 2>::value;
};
template <>
struct Log2<1> {
    static constexpr unsigned value = 0;
};

// True when the candidate left out of a full list (smallest left-out key
// out_min) may belong in it: its T is within one unit of the k-th entry's.
template <unsigned EBITS>
__device__ __forceinline__ bool boundary_unsure(unsigned last, unsigned out_min) {
    return last != KEY32_EMPTY && (out_min >> EBITS) < (last >> EBITS) + 2u;
}

// The listed slots out[r * stride] (r < k, in key order, UINT_MAX after the
// last neighbour) against the exact (distance, index) order, for the adjacent
// entries whose T are within one unit (the others are ordered by their keys).
// The exact comparisons of the near pairs (bit i: entries i - 1 and i of the
// register list, first listed entry at register `first`), out of line: few
// agents have any.
static __device__ __noinline__ bool near_pairs_check(unsigned near, int first, V3 p,
                                                     const float4* __restrict__ pos_id,
                                                     const unsigned* out, unsigned stride) {
    while (near) {
        const int i = __ffs(int(near)) - 1;
        near &= near - 1;
        const unsigned r = unsigned(i - first);
        const float4 qa = __ldg(pos_id + out[(r - 1) * stride]);
        const float4 qb = __ldg(pos_id + out[r * stride]);
        if (!knn_less(distance(p, v3(qa)), __float_as_uint(qa.w), distance(p, v3(qb)),
                      __float_as_uint(qb.w)))
            return false;
    }
    return true;
}

template <int KMAX, unsigned EBITS>
__device__ __forceinline__ bool near_pairs_ordered(const unsigned (&key)[KMAX], int k, V3 p,
                                                   const float4* __restrict__ pos_id,
                                                   const unsigned* out, unsigned stride) {
    unsigned near = 0;
#pragma unroll
    for (int i = 1; i < KMAX; ++i)
        if (i > KMAX - k && key[i] != KEY32_EMPTY && (key[i] >> EBITS) < (key[i - 1] >> EBITS) + 2u)
            near |= 1u << i;
    return near == 0 || near_pairs_check(near, KMAX - k, p, pos_id, out, stride);
}

template <int KMAX>
struct KList32 {
    unsigned key[KMAX];
    // Inserts c; returns the largest key, which leaves the list.  In a sorted
    // list the entry at i after the insertion is min(key[i], max(key[i-1], c)):
    // key[i-1] when c goes below it, c when it falls between, else key[i].
    // Every entry comes from the old list and c alone, so the KMAX
    // min/max pairs are independent (dependency depth 2) instead of one
    // chain through c of 2 * KMAX steps.
    __device__ __forceinline__ unsigned insert(unsigned c) {
        const unsigned out = max(key[KMAX - 1], c);
#pragma unroll
        for (int i = KMAX - 1; i > 0; --i) key[i] = min(key[i], max(key[i - 1], c));
        key[0] = min(key[0], c);
        return out;
    }
    // Merges the 4 keys c into the list, keeping the KMAX smallest, and
    // returns the smallest key that does not stay.  The chunk is sorted (5
    // compare-exchanges) and laid reversed against the list's last 4
    // entries: the elementwise minimum of an ascending and a descending
    // sequence is bitonic and holds the KMAX smallest keys of both, and the
    // elementwise maxima are the keys that leave.  log2(KMAX) half-cleaner
    // stages then sort the bitonic list.  Equal to inserting the 4 keys one
    // after another, at about two thirds of the min/max work per key.
    __device__ __forceinline__ unsigned merge4(unsigned (&c)[4]) {
        static_assert(KMAX >= 4, "chunk merge needs KMAX >= 4");
        cmpx(c[0], c[1]);
        cmpx(c[2], c[3]);
        cmpx(c[0], c[2]);
        cmpx(c[1], c[3]);
        cmpx(c[1], c[2]);
        unsigned out = KEY32_EMPTY;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const unsigned a = key[KMAX - 4 + j], b = c[3 - j];
            key[KMAX - 4 + j] = min(a, b);
            out = min(out, max(a, b));
        }
#pragma unroll
        for (int stride = KMAX / 2; stride > 0; stride >>= 1) {
#pragma unroll
            for (int i = 0; i < KMAX; ++i)
                if ((i ^ stride) > i) cmpx(key[i], key[i ^ stride]);
        }
        return out;
    }
    __device__ __forceinline__ static void cmpx(unsigned& a, unsigned& b) {
        const unsigned lo = min(a, b);
        b = max(a, b);
        a = lo;
    }
    // Ascending bitonic sort (compare-exchange = min + max).
    __device__ __forceinline__ void sort() {
#pragma unroll
        for (int size = 2; size <= KMAX; size <<= 1) {
#pragma unroll
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
#pragma unroll
                for (int i = 0; i < KMAX; ++i) {
                    const int j = i ^ stride;
                    if (j > i) {
                        const unsigned a = key[i], b = key[j];
                        const bool up = (i & size) == 0;
                        key[i] = up ? min(a, b) : max(a, b);
                        key[j] = up ? max(a, b) : min(a, b);
                    }
                }
            }
        }
    }
};

// dist_sq(p, q) with the x and y differences and squares in one packed f32x2
// subtract and one packed multiply (elementwise, round to nearest, not
// contracted): the same operations in the same order as dist_sq, so the same
// bits.  pxy: p.x and p.y packed (pack_xy), once per agent.  The streaming
// scan uses it (wall phase 0.405 -> 0.401 ms per 256-scene step); in the
// collecting scan it measured slower (flock kernel 0.255 -> 0.257 ms).
__device__ __forceinline__ unsigned long long pack_xy(float x, float y) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
    return r;
}
__device__ __forceinline__ void unpack_xy(unsigned long long v, float& x, float& y) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(v));
}
__device__ __forceinline__ unsigned long long packed_sub(unsigned long long a,
                                                         unsigned long long b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long packed_mul(unsigned long long a,
                                                         unsigned long long b) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ float dist_sq_xy2(unsigned long long pxy, float pz, float4 q) {
    const unsigned long long qxy = pack_xy(q.x, q.y);
    unsigned long long o, sq;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(o) : "l"(pxy), "l"(qxy));
    asm("mul.rn.f32x2 %0, %1, %1;" : "=l"(sq) : "l"(o));
    float sx, sy;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(sx), "=f"(sy) : "l"(sq));
    const float oz = __fsub_rn(pz, q.z);
    return __fadd_rn(__fadd_rn(sx, sy), __fmul_rn(oz, oz));
}

// Appends candidate slot s to the tables (self and non-finite squared
// distances skip).  e counts past ENUM without storing; the caller checks it.
// No early exits: the warp's lanes reconverge after every candidate.
template <unsigned ENUM>
__device__ __forceinline__ void collect_one(unsigned s, V3 p, unsigned self_id,
                                            const float4* __restrict__ pos_id, unsigned& e,
                                            unsigned* slot_tab, unsigned* key_tab,
                                            unsigned stride) {
    const float4 q = __ldg(pos_id + s);
    const unsigned bits = __float_as_uint(dist_sq(p, v3(q)));
    // inf or NaN (the distance is then inf or NaN: never below FLT_MAX, never
    // listed); a finite square gives a finite root, which is
    if (__float_as_uint(q.w) != self_id && bits <= 0x7f7fffffu) {
        if (e < ENUM) {
            slot_tab[e * stride] = s;
            key_tab[e * stride] = (bits & ~(ENUM - 1)) | e;
        }
        ++e;
    }
}

constexpr unsigned kCollectChunk = 4;

// Collects every candidate of `box` into the tables; returns the count (which
// exceeds ENUM when the tables overflowed).
template <unsigned ENUM>
__device__ __forceinline__ unsigned collect_box(V3 p, unsigned self_id, const Grid& g,
                                                const Box& b, unsigned cell_offset,
                                                const unsigned* __restrict__ cell_start,
                                                const float4* __restrict__ pos_id,
                                                unsigned* slot_tab, unsigned* key_tab,
                                                unsigned stride) {
    unsigned e = 0;
    const unsigned span = b.x1 - b.x0 + 1;
    if (b.y1 - b.y0 <= 2 && b.z1 - b.z0 <= 2) {
        // At most 3 x 3 rows.  The rows' slots are first laid end to end in
        // slot_tab (a short store loop per row), then one loop walks all of
        // them: a warp runs as many iterations as its busiest lane has
        // candidates, not the sum over rows of each row's busiest lane.
        unsigned rs[9], rn[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const unsigned cy = b.y0 + unsigned(i / 3), cz = b.z0 + unsigned(i % 3);
            const bool ok = cy <= b.y1 && cz <= b.z1;
            const unsigned c0 = cell_offset + cell_label(g, b.x0, ok ? cy : b.y0, ok ? cz : b.z0);
            const unsigned s0 = ok ? __ldg(cell_start + c0) : 0u;
            const unsigned s1 = ok ? __ldg(cell_start + c0 + span) : 0u;
            rs[i] = s0;
            rn[i] = s1 - s0;
        }
        unsigned total = 0;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            for (unsigned t = 0; t < rn[i]; ++t)
                if (total + t < ENUM) slot_tab[(total + t) * stride] = rs[i] + t;
            total += rn[i];
        }
        if (total > ENUM) return total;  // overflow: the exact path redoes the agent
        // compacted in place (self and non-finite candidates dropped): entry
        // e is written only after entries up to e were read.  kCollectChunk
        // at a time: the slots, then the positions, are loaded before any key
        // is formed, so their loads overlap.
        for (unsigned j0 = 0; j0 < total; j0 += kCollectChunk) {
            unsigned sl[kCollectChunk];
            float4 q[kCollectChunk];
#pragma unroll
            for (unsigned u = 0; u < kCollectChunk; ++u)
                sl[u] = j0 + u < total ? slot_tab[(j0 + u) * stride] : 0u;
#pragma unroll
            for (unsigned u = 0; u < kCollectChunk; ++u)
                q[u] = j0 + u < total ? __ldg(pos_id + sl[u]) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (unsigned u = 0; u < kCollectChunk; ++u) {
                if (j0 + u >= total) break;
                const unsigned bits = __float_as_uint(dist_sq(p, v3(q[u])));
                if (__float_as_uint(q[u].w) != self_id && bits <= 0x7f7fffffu) {
                    slot_tab[e * stride] = sl[u];
                    key_tab[e * stride] = (bits & ~(ENUM - 1)) | e;
                    ++e;
                }
            }
        }
        return e;
    }
    for (unsigned cy = b.y0; cy <= b.y1; ++cy)
        for (unsigned cz = b.z0; cz <= b.z1; ++cz) {
            const unsigned c0 = cell_offset + cell_label(g, b.x0, cy, cz);
            const unsigned s0 = __ldg(cell_start + c0), s1 = __ldg(cell_start + c0 + span);
            for (unsigned s = s0; s < s1; ++s)
                collect_one<ENUM>(s, p, self_id, pos_id, e, slot_tab, key_tab, stride);
        }
    return e;
}

// Fast path: the k nearest of `box` as slots in (distance, index) order at
// key_tab[r * stride], UINT_MAX after the last neighbour.  Returns false when
// the exact path must redo this agent.
template <int KMAX, unsigned ENUM>
__device__ __forceinline__ bool knn_neighbours_fast(int k, V3 p, unsigned self_id, const Grid& g,
                                                    const Box& b, unsigned cell_offset,
                                                    const unsigned* __restrict__ cell_start,
                                                    const float4* __restrict__ pos_id,
                                                    unsigned* slot_tab, unsigned* key_tab,
                                                    unsigned stride) {
    constexpr unsigned mask = ENUM - 1, EBITS = Log2<ENUM>::value;
    const unsigned n = collect_box<ENUM>(p, self_id, g, b, cell_offset, cell_start, pos_id,
                                         slot_tab, key_tab, stride);
    if (n > ENUM) return false;
    // The first min(n, k) keys, KMAX - k sentinel zeros (sorted to the front)
    // and empty keys: after sorting, entries KMAX-k .. KMAX-1 are the list.
    KList32<KMAX> L;
    const unsigned m = n < unsigned(k) ? n : unsigned(k);
#pragma unroll
    for (int i = 0; i < KMAX; ++i)
        L.key[i] = unsigned(i) < m ? key_tab[i * stride] : (i < k ? KEY32_EMPTY : 0u);
    L.sort();
    unsigned out_min = KEY32_EMPTY;  // smallest key not (or no longer) in the list
    for (unsigned e = m; e < n; ++e) {
        const unsigned c = key_tab[e * stride];
        out_min = min(out_min, c < L.key[KMAX - 1] ? L.insert(c) : c);
    }
    if (boundary_unsure<EBITS>(L.key[KMAX - 1], out_min)) return false;
#pragma unroll
    for (int i = 0; i < KMAX; ++i)
        if (i >= KMAX - k)
            key_tab[(i - (KMAX - k)) * stride] =
                L.key[i] != KEY32_EMPTY ? slot_tab[(L.key[i] & mask) * stride] : UINT_MAX;
    return near_pairs_ordered<KMAX, EBITS>(L.key, k, p, pos_id, key_tab, stride);
}

// The order the streaming scan visits the nine rows of a 3 x 3 x 3 (or
// 3 x 3) box in (kRowOrderFlat: the three rows of a flat box): the middle
// row first, then the rows beside it, then the corners, so the list fills with near candidates early and later candidates
// insert less (1.5 % of a 256-scene choke-point step).  The result does not
// depend on it: the list ends as the k smallest keys, whose enumeration
// indices do not change, and ties of truncated distance send the agent to the
// exact path.
__device__ constexpr int kRowOrder[9] = {4, 1, 3, 5, 7, 0, 2, 6, 8};
__device__ constexpr int kRowOrderFlat[3] = {1, 0, 2};

// Streaming fast path for crowded boxes: the same 32-bit keys, but the
// candidates go straight into the register list, four at a time (no
// per-candidate shared memory), so the enumeration capacity is 2^EBITS
// whatever the block size.
// e numbers every candidate of the box in row order, the agent itself
// included, so a listed key's e is decoded back to its slot from the nine
// row starts and the running row offsets alone.  Boxes of more than 3 x 3
// rows (search radius above 1) are left to the exact path.  Writes the k
// slots to out[r * stride]; returns false when the exact path must redo the
// agent, on the same conditions as the collecting scan.  FLAT: the grid is
// one cell high in y (the 2D worlds on the x-z plane), so a box has at most 3
// rows; that build keeps 3 row starts instead of 9 (no register spills at
// 64 registers) and drops the 6 empty row loops.  The rows and their
// enumeration are those of the 9-row build (rows 3-8 are empty there).
template <int KMAX, unsigned EBITS, bool FLAT = false>
__device__ __forceinline__ bool knn_neighbours_stream(int k, V3 p, unsigned self_id,
                                                      const Grid& g, const Box& b,
                                                      unsigned cell_offset,
                                                      const unsigned* __restrict__ cell_start,
                                                      const float4* __restrict__ pos_id,
                                                      unsigned* out, unsigned stride) {
    constexpr unsigned ENUM = 1u << EBITS, mask = ENUM - 1;
    constexpr int R = FLAT ? 3 : 9;
    if ((FLAT ? b.y1 != b.y0 : b.y1 - b.y0 > 2) || b.z1 - b.z0 > 2) return false;
    const unsigned span = b.x1 - b.x0 + 1;
    unsigned rs[R], pre[R + 1];
    pre[0] = 0;
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const unsigned cy = b.y0 + unsigned(FLAT ? 0 : i / 3), cz = b.z0 + unsigned(i % 3);
        const bool ok = cy <= b.y1 && cz <= b.z1;
        const unsigned c0 = cell_offset + cell_label(g, b.x0, ok ? cy : b.y0, ok ? cz : b.z0);
        const unsigned s0 = ok ? __ldg(cell_start + c0) : 0u;
        const unsigned s1 = ok ? __ldg(cell_start + c0 + span) : 0u;
        rs[i] = s0;
        pre[i + 1] = pre[i] + (s1 - s0);
    }
    if (pre[R] > ENUM) return false;
    KList32<KMAX> L;
#pragma unroll
    for (int i = 0; i < KMAX; ++i) L.key[i] = i < KMAX - k ? 0u : KEY32_EMPTY;
    unsigned out_min = KEY32_EMPTY;  // smallest key not (or no longer) in the list
    const unsigned long long pxy = pack_xy(p.x, p.y);
#pragma unroll
    for (int ii = 0; ii < R; ++ii) {
        const int i = FLAT ? kRowOrderFlat[ii] : kRowOrder[ii];
        const unsigned n_row = pre[i + 1] - pre[i];
        // four candidates at a time: their loads and distances overlap, and
        // one chunk merge costs less than four insertions
        for (unsigned t0 = 0; t0 < n_row; t0 += 4) {
            unsigned c[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const unsigned t = t0 + unsigned(j);
                c[j] = KEY32_EMPTY;
                if (t < n_row) {
                    const float4 q = __ldg(pos_id + rs[i] + t);
                    const unsigned bits = __float_as_uint(dist_sq_xy2(pxy, p.z, q));
                    if (__float_as_uint(q.w) != self_id && bits <= 0x7f7fffffu)
                        c[j] = (bits & ~mask) | (pre[i] + t);
                }
            }
            out_min = min(out_min, L.merge4(c));
        }
    }
    if (boundary_unsure<EBITS>(L.key[KMAX - 1], out_min)) return false;
#pragma unroll
    for (int i = 0; i < KMAX; ++i) {
        if (i < KMAX - k) continue;
        const unsigned key = L.key[i];
        unsigned slot = UINT_MAX;
        if (key != KEY32_EMPTY) {
            const unsigned e = key & mask;
            slot = rs[0] + e;
#pragma unroll
            for (int j = 1; j < R; ++j)
                if (e >= pre[j]) slot = rs[j] + (e - pre[j]);
        }
        out[(i - (KMAX - k)) * stride] = slot;
    }
    return near_pairs_ordered<KMAX, EBITS>(L.key, k, p, pos_id, out, stride);
}

// Exact path: the ordered slots go to col[r * stride].
template <int KMAX>
__device__ __forceinline__ void knn_neighbours_exact(int k, V3 p, unsigned self_id, const Grid& g,
                                                     const Box& b, unsigned cell_offset,
                                                     const unsigned* __restrict__ cell_start,
                                                     const float4* __restrict__ pos_id,
                                                     unsigned* col, unsigned stride) {
    KList<KMAX> L;
    L.init(k);
    knn_scan_box<KMAX>(L, p, self_id, g, b, cell_offset, cell_start, pos_id);
    L.for_each(k, [&](int r, unsigned long long key, unsigned slot) {
        col[r * stride] = key_id(key) == UINT_MAX ? UINT_MAX : slot;
    });
}

// The k nearest of `box` as slots in (distance, index) order at
// col[r * stride] (UINT_MAX after the last neighbour): the fast scan, or the
// exact list when the fast scan cannot vouch for its order.  col needs
// ENUM + KMAX entries.
template <int KMAX, unsigned ENUM>
__device__ __forceinline__ void knn_neighbours(int k, V3 p, unsigned self_id, const Grid& g,
                                               const Box& b, unsigned cell_offset,
                                               const unsigned* __restrict__ cell_start,
                                               const float4* __restrict__ pos_id,
                                               unsigned* col, unsigned stride) {
    // col holds the slot table (ENUM entries) then the key table / result
    if (knn_neighbours_fast<KMAX, ENUM>(k, p, self_id, g, b, cell_offset, cell_start, pos_id, col,
                                        col + ENUM * stride, stride)) {
        for (int r = 0; r < k; ++r) col[r * stride] = col[(ENUM + r) * stride];
        return;
    }
    knn_neighbours_exact<KMAX>(k, p, self_id, g, b, cell_offset, cell_start, pos_id, col, stride);
}

}  // namespace gs
