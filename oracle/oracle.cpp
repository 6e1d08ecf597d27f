// CPU oracle: a line-by-line C++ restatement of the GPUSteer group kernels.
//
// TEST INFRASTRUCTURE ONLY (the checker, never the product).  Each function
// cites the reference file:line it follows; paths are relative to the
// PsychoLogicAu/GPUSteer tree.  Built with -ffp-contract=off so that every
// binary32 expression is evaluated exactly as written (no FMA), which is the
// same contract the CUDA kernels use (-fmad=false).
//
// Documented decisions where the reference is ambiguous or undefined:
//  (i)   KNN order is the total order (distance, agent index).  This is the
//        reference's brute-force order (KNNBruteForceCudaKernel.cu:253-269);
//        the binned kernel breaks exact ties by cell visit order instead
//        (KNNBinningV2Kernel.cu:491-512).
//  (ii)  distance = sqrt((dx*dx + dy*dy) + dz*dz), binary32, no FMA
//        (VectorUtils.cuh:85-108,147-150).
//  (iii) cell coordinate = clamp(floor(((p + 0.5*W)/W) * n), 0, n-1), the
//        point-sampled, clamped normalised texture lookup of
//        KNNBinningV2Kernel.cu:287-292 with the texture's documented
//        nearest-point formula.  Cells are labelled x + z*X + y*X*Z, the
//        bin_cell order of KNNBinDataV2.cu:103-116.
//  (iv)  avoid-neighbours, "parallel" branch: the threat position is the
//        threat's current position (the reference reads an uninitialised
//        variable, SteerToAvoidNeighborsCUDAKernel.cu:301,372).
//  (v)   UpdateCUDAKernel with speed == 0 keeps the old side vector (the
//        reference writes back uninitialised shared memory,
//        UpdateCUDAKernel.cu:75,114).
#include "oracle.h"

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <fstream>
#include <limits>
#include <list>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <class T> struct V3 { T x, y, z; };

// ---- VectorUtils.cuh:35-189 -------------------------------------------------
template <class T> inline V3<T> add(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> sub(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> neg(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline V3<T> mul(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> dvd(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline T dot(V3<T> a, V3<T> b) { return ((a.x * b.x) + (a.y * b.y)) + (a.z * b.z); }
template <class T> inline T length(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> inline V3<T> normalize(V3<T> v) {
    const T len = length(v);
    return (len > 0) ? dvd(v, len) : v;
}
template <class T> inline V3<T> cross(V3<T> a, V3<T> b) {
    return {(a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x)};
}
template <class T> inline bool is_zero(V3<T> a) { return a.x == 0 && a.y == 0 && a.z == 0; }
template <class T> inline T distance(V3<T> a, V3<T> b) { return length(sub(a, b)); }
template <class T> inline V3<T> parallel_component(V3<T> v, V3<T> u) { return mul(u, dot(v, u)); }
template <class T> inline V3<T> perpendicular_component(V3<T> v, V3<T> u) {
    return sub(v, parallel_component(v, u));
}
template <class T> inline V3<T> truncate_length(V3<T> v, T max_len) {
    const T max_sq = max_len * max_len;
    const T len_sq = dot(v, v);
    if (len_sq <= max_sq) return v;
    return mul(v, max_len / std::sqrt(len_sq));
}

template <class T, class S> inline V3<T> ld4(const S* p, size_t i) {
    return {T(p[4 * i]), T(p[4 * i + 1]), T(p[4 * i + 2])};
}
template <class T, class S> inline V3<T> ld3(const S* p, size_t i) {
    return {T(p[3 * i]), T(p[3 * i + 1]), T(p[3 * i + 2])};
}
template <class T> inline void st4(T* p, size_t i, V3<T> v) {
    p[4 * i] = v.x; p[4 * i + 1] = v.y; p[4 * i + 2] = v.z; p[4 * i + 3] = 0;
}
template <class T> inline void st3(T* p, size_t i, V3<T> v) {
    p[3 * i] = v.x; p[3 * i + 1] = v.y; p[3 * i + 2] = v.z;
}

// Kernel bit masks, CUDAKernelGlobals.cuh:12-29.
constexpr unsigned SEEK_BIT = 1u << 2;
constexpr unsigned SEPARATION_BIT = 1u << 4;
constexpr unsigned ALIGNMENT_BIT = 1u << 5;
constexpr unsigned COHESION_BIT = 1u << 6;
constexpr unsigned AVOID_WALLS_BIT = 1u << 8;
constexpr unsigned AVOID_NEIGHBORS_BIT = 1u << 9;
constexpr unsigned AVOID_CLOSE_NEIGHBORS_BIT = 1u << 10;
constexpr unsigned ANTI_PENETRATION_WALL = 1u << 12;
constexpr unsigned ANTI_PENETRATION_AGENT = 1u << 13;
constexpr unsigned FOLLOW_PATH_BIT = 1u << 11;

inline int nthreads(int t) {
#ifdef _OPENMP
    return t > 0 ? t : omp_get_max_threads();
#else
    (void)t;
    return 1;
#endif
}

template <class T> struct Group {
    T* position; T* direction; T* steering; T* side; T* up;
    T* speed; T* max_speed; T* max_force; T* radius; T* mass;
    unsigned* applied; unsigned n;
};
template <class T, class G> Group<T> view(G* g) {
    return {g->position, g->direction, g->steering, g->side, g->up, g->speed, g->max_speed,
            g->max_force, g->radius, g->mass, g->applied, g->n};
}

// ---- cell index: KNNBinningV2Kernel.cu:269-296 + KNNBinDataV2.cu:103-116 ----
template <class T> inline unsigned cell_coord(T p, T w, unsigned n) {
    const T u = (p + T(0.5) * w) / w;
    const T f = std::floor(u * T(n));
    if (!(f >= T(0))) return 0u;
    if (f >= T(n)) return n - 1;
    return unsigned(f);
}
template <class T> inline void cell_coords(V3<T> p, const float ws[3], const unsigned wc[3],
                                           unsigned& ix, unsigned& iy, unsigned& iz) {
    ix = cell_coord(p.x, T(ws[0]), wc[0]);
    iy = cell_coord(p.y, T(ws[1]), wc[1]);
    iz = cell_coord(p.z, T(ws[2]), wc[2]);
}
inline unsigned cell_label(unsigned ix, unsigned iy, unsigned iz, const unsigned wc[3]) {
    return ix + iz * wc[0] + iy * wc[0] * wc[2];
}

// Total order (distance, index) used by every KNN here.
template <class T> inline bool knn_less(T d1, unsigned i1, T d2, unsigned i2) {
    return d1 < d2 || (d1 == d2 && i1 < i2);
}
template <class T> inline void knn_insert(T* D, unsigned* I, unsigned k, T d, unsigned j) {
    if (!knn_less(d, j, D[k - 1], I[k - 1])) return;
    D[k - 1] = d; I[k - 1] = j;
    for (unsigned s = k - 1; s > 0 && knn_less(D[s], I[s], D[s - 1], I[s - 1]); --s) {
        std::swap(D[s], D[s - 1]);
        std::swap(I[s], I[s - 1]);
    }
}
template <class T> constexpr T knn_empty() { return T(FLT_MAX); }

// ---- binned KNN: KNNBinningV2.cu:87-162 (rebuild) + KNNBinningV2Kernel.cu:417-528
template <class T, class S>
void knn_binned(const S* posA, unsigned nA, const S* posB, unsigned nB, bool self,
                const float ws[3], const unsigned wc[3], unsigned r, unsigned k,
                unsigned* idx, T* dist, int threads) {
    const unsigned C = wc[0] * wc[1] * wc[2];
    // Rebuild: cell of every B agent, then a stable sort by cell (the
    // reference uses thrust::sort_by_key, a stable radix sort).
    std::vector<unsigned> cellB(nB), start(size_t(C) + 1, 0u), sorted(nB);
    for (unsigned b = 0; b < nB; ++b) {
        unsigned ix, iy, iz;
        cell_coords(ld4<T>(posB, b), ws, wc, ix, iy, iz);
        cellB[b] = cell_label(ix, iy, iz, wc);
        start[cellB[b] + 1]++;
    }
    for (unsigned c = 0; c < C; ++c) start[c + 1] += start[c];
    {
        std::vector<unsigned> fill(start.begin(), start.end() - 1);
        for (unsigned b = 0; b < nB; ++b) sorted[fill[cellB[b]]++] = b;
    }
    // Query: the neighbour cells of KNNBinningV2ComputeCellNeighbors{3D,2D}
    // (KNNBinningV2Kernel.cu:102-248) are every cell within r in each axis,
    // clamped to the grid, duplicates removed: the clamped box below.
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads(threads))
    for (long long aa = 0; aa < (long long)nA; ++aa) {
        const unsigned a = unsigned(aa);
        std::vector<T> D(k, knn_empty<T>());
        std::vector<unsigned> I(k, UINT_MAX);
        const V3<T> pa = ld4<T>(posA, a);
        unsigned ix, iy, iz;
        cell_coords(pa, ws, wc, ix, iy, iz);
        const unsigned x0 = ix >= r ? ix - r : 0, x1 = std::min(ix + r, wc[0] - 1);
        const unsigned y0 = iy >= r ? iy - r : 0, y1 = std::min(iy + r, wc[1] - 1);
        const unsigned z0 = iz >= r ? iz - r : 0, z1 = std::min(iz + r, wc[2] - 1);
        for (unsigned cy = y0; cy <= y1; ++cy)
            for (unsigned cz = z0; cz <= z1; ++cz)
                for (unsigned cx = x0; cx <= x1; ++cx) {
                    const unsigned c = cell_label(cx, cy, cz, wc);
                    for (unsigned s = start[c]; s < start[c + 1]; ++s) {
                        const unsigned b = sorted[s];
                        if (self && a == b) continue;
                        const T d = distance(pa, ld4<T>(posB, b));
                        knn_insert(D.data(), I.data(), k, d, b);
                    }
                }
        for (unsigned i = 0; i < k; ++i) {
            idx[a + size_t(i) * nA] = I[i];
            dist[a + size_t(i) * nA] = D[i];
        }
    }
}

// ---- brute-force KNN: KNNBruteForceCudaKernel.cu:207-283 ----------------------
template <class T, class S>
void knn_brute(const S* posA, unsigned nA, const S* posB, unsigned nB, bool self,
               unsigned k, unsigned* idx, T* dist, int threads) {
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (long long aa = 0; aa < (long long)nA; ++aa) {
        const unsigned a = unsigned(aa);
        std::vector<T> D(k, knn_empty<T>());
        std::vector<unsigned> I(k, UINT_MAX);
        const V3<T> pa = ld4<T>(posA, a);
        for (unsigned b = 0; b < nB; ++b) {
            if (self && a == b) continue;
            knn_insert(D.data(), I.data(), k, distance(pa, ld4<T>(posB, b)), b);
        }
        for (unsigned i = 0; i < k; ++i) {
            idx[a + size_t(i) * nA] = I[i];
            dist[a + size_t(i) * nA] = D[i];
        }
    }
}

// ---- WrapWorldCUDAKernel.cu:11-48 ------------------------------------------
template <class T> void wrap_world(Group<T> g, const float ws[3], int mode, int threads) {
    if (mode == ORC_WRAP_NONE) return;
    const V3<T> half = mul(V3<T>{T(ws[0]), T(ws[1]), T(ws[2])}, T(0.5));
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (long long ii = 0; ii < (long long)g.n; ++ii) {
        V3<T> p = ld4<T>(g.position, ii);
        if (p.x < -half.x) p.x = half.x;
        if (p.x > half.x) p.x = -half.x;
        if (p.y < -half.y) p.y = half.y;
        if (p.y > half.y) p.y = -half.y;
        if (mode == ORC_WRAP_REFERENCE) {
            if (p.z < 0) p.z = half.z + T(100);
        } else {
            if (p.z < -half.z) p.z = half.z;
            if (p.z > half.z) p.z = -half.z;
        }
        st4(g.position, ii, p);
    }
}

// ---- FlockingCommon.cuh:4-30 -----------------------------------------------
template <class T> inline bool in_boid_neighborhood(V3<T> pos, V3<T> dir, V3<T> other, T min_d,
                                                    T max_d, T cos_max) {
    const V3<T> offset = sub(other, pos);
    const T d = length(offset);
    if (d < min_d) return true;
    if (d > max_d) return false;
    const V3<T> unit = dvd(offset, d);
    return dot(dir, unit) > cos_max;
}

inline void add_steering(float* s, size_t i, V3<float> v) {
    st4(s, i, add(v, ld4<float>(s, i)));
}
inline void add_steering(double* s, size_t i, V3<double> v) {
    st4(s, i, add(v, ld4<double>(s, i)));
}

// Flocking behaviours.  kind: 0 separation (SteerForSeparationCUDAKernel.cu:69-134),
// 1 alignment (SteerForAlignmentCUDAKernel.cu:65-140), 2 cohesion
// (SteerForCohesionCUDAKernel.cu:60-134).
template <class T, class S>
void flock(Group<T> g, int kind, const unsigned* knn, unsigned k, const S* posB,
           const S* dirB, unsigned nB, T min_d, T max_d, T cos_max, T w, unsigned mask,
           int threads) {
    const unsigned bit = kind == 0 ? SEPARATION_BIT : kind == 1 ? ALIGNMENT_BIT : COHESION_BIT;
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (long long ii = 0; ii < (long long)g.n; ++ii) {
        const size_t i = size_t(ii);
        if (g.applied[i] & mask) continue;
        const V3<T> pos = ld4<T>(g.position, i), dir = ld4<T>(g.direction, i);
        V3<T> steering{0, 0, 0};
        unsigned neighbors = 0;
        for (unsigned s = 0; s < k; ++s) {
            const unsigned b = knn[i + size_t(s) * g.n];
            if (b >= nB) break;
            const V3<T> bp = ld4<T>(posB, b);
            if (!in_boid_neighborhood(pos, dir, bp, min_d, max_d, cos_max)) continue;
            if (kind == 0) {
                const V3<T> offset = sub(bp, pos);
                const T dsq = dot(offset, offset);
                steering = add(steering, dvd(offset, -dsq));
            } else if (kind == 1) {
                steering = add(steering, ld4<T>(dirB, b));
            } else {
                steering = add(steering, bp);
            }
            neighbors++;
        }
        if (neighbors > 0) {
            const V3<T> mean = dvd(steering, T(neighbors));
            if (kind == 0) steering = normalize(mean);
            else if (kind == 1) steering = normalize(sub(mean, dir));
            else steering = normalize(sub(mean, pos));
        }
        steering = mul(steering, w);
        if (!is_zero(steering)) g.applied[i] |= bit;
        add_steering(g.steering, i, steering);
    }
}

// ---- SteerForSeekCUDAKernel.cu:35-72 ---------------------------------------
template <class T> void seek(Group<T> g, V3<T> target, T w, unsigned mask, int threads) {
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (long long ii = 0; ii < (long long)g.n; ++ii) {
        const size_t i = size_t(ii);
        if (g.applied[i] & mask) continue;
        const V3<T> desired = sub(target, ld4<T>(g.position, i));
        V3<T> steering = sub(desired, ld4<T>(g.direction, i));
        steering = mul(normalize(steering), w);
        if (!is_zero(steering)) g.applied[i] |= SEEK_BIT;
        add_steering(g.steering, i, steering);
    }
}

// ---- path following: SteerToFollowPathCUDAKernel.cu:35-287 ------------------
template <class T> struct PathView {
    const float* points;   // float3[n]
    const float* lengths;  // [n]
    const float* normals;  // float3[n]
    unsigned n;
    T radius;
    bool cyclic;
    T total;
};
// pointToSegmentDistance (:35-70): distance to the segment ep0-ep1, its
// projection and the nearest point
template <class T>
inline T point_to_segment(V3<T> point, V3<T> ep0, V3<T> ep1, V3<T> normal, T seg_len, T& proj,
                          V3<T>& chosen) {
    const V3<T> local = sub(point, ep0);
    proj = dot(normal, local);
    if (proj < T(0)) {
        chosen = ep0;
        proj = 0;
        return distance(point, ep0);
    }
    if (proj > seg_len) {
        chosen = ep1;
        proj = seg_len;
        return distance(point, ep1);
    }
    chosen = add(ep0, mul(normal, proj));
    return distance(point, chosen);
}
// mapPointToPathDistance (:72-100)
template <class T> inline T map_point_to_path_distance(V3<T> point, const PathView<T>& P) {
    T min_d = std::numeric_limits<T>::max(), total = 0, path_d = 0;
    V3<T> chosen{0, 0, 0};
    for (unsigned i = 1; i < P.n; ++i) {
        const T seg_len = T(P.lengths[i]);
        T proj;
        const T d = point_to_segment(point, ld3<T>(P.points, i - 1), ld3<T>(P.points, i),
                                     ld3<T>(P.normals, i), seg_len, proj, chosen);
        if (d < min_d) {
            min_d = d;
            path_d = total + proj;
        }
        total += seg_len;
    }
    return path_d;
}
// mapPointToPath (:102-141): nearest point on the path, its segment's
// direction, and how far outside the tube the point is
template <class T>
inline V3<T> map_point_to_path(V3<T> point, const PathView<T>& P, V3<T>& tangent, T& outside) {
    T min_d = std::numeric_limits<T>::max();
    V3<T> on_path{0, 0, 0}, chosen{0, 0, 0};
    for (unsigned i = 1; i < P.n; ++i) {
        T proj;
        const T d = point_to_segment(point, ld3<T>(P.points, i - 1), ld3<T>(P.points, i),
                                     ld3<T>(P.normals, i), T(P.lengths[i]), proj, chosen);
        if (d < min_d) {
            min_d = d;
            on_path = chosen;
            tangent = ld3<T>(P.normals, i);
        }
    }
    outside = distance(on_path, point) - P.radius;
    return on_path;
}
// mapPathDistanceToPoint (:143-181).  Decision (viii): when the segment walk
// runs past the last segment (rounding), the path's last point is returned;
// the reference returns an uninitialised value there.
template <class T> inline V3<T> map_path_distance_to_point(T path_d, const PathView<T>& P) {
    T remaining = path_d;
    if (P.cyclic) {
        remaining = std::fmod(path_d, P.total);
    } else {
        if (path_d < T(0)) return ld3<T>(P.points, 0);
        if (path_d >= P.total) return ld3<T>(P.points, P.n - 1);
    }
    for (unsigned i = 1; i < P.n; ++i) {
        const T seg_len = T(P.lengths[i]);
        if (seg_len < remaining) {
            remaining -= seg_len;
        } else {
            const T ratio = remaining / seg_len;
            const V3<T> a = ld3<T>(P.points, i - 1), b = ld3<T>(P.points, i);
            return add(a, mul(sub(b, a), ratio));  // interpolate (VectorUtils.cuh:292-295)
        }
    }
    return ld3<T>(P.points, P.n - 1);
}
template <class T> PathView<T> path_view(const orc_path* p) {
    return PathView<T>{p->points, p->lengths, p->normals, p->n, T(p->radius), p->cyclic != 0,
                       T(p->total_length)};
}

// FollowPathCUDAKernel (:183-287)
template <class T>
void follow_path(Group<T> g, const PathView<T>& P, T prediction_time, T w, unsigned mask,
                 int threads) {
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (long long ii = 0; ii < (long long)g.n; ++ii) {
        const size_t i = size_t(ii);
        if (g.applied[i] & mask) continue;
        const V3<T> pos = ld4<T>(g.position, i), dir = ld4<T>(g.direction, i);
        const T speed = g.speed[i];
        const T offset = prediction_time * speed;
        const V3<T> future = add(pos, mul(mul(dir, speed), prediction_time));
        const T now_d = map_point_to_path_distance(pos, P);
        const T future_d = map_point_to_path_distance(future, P);
        const bool rightway = (offset > T(0)) ? (now_d < future_d) : (now_d > future_d);
        V3<T> tangent{0, 0, 0};
        T outside;
        map_point_to_path(future, P, tangent, outside);
        V3<T> steering{0, 0, 0};
        if (!((outside < T(0)) && rightway)) {
            const V3<T> target = map_path_distance_to_point(now_d + offset, P);
            steering = sub(sub(target, pos), dir);
        }
        steering = mul(normalize(steering), w);
        if (!is_zero(steering)) g.applied[i] |= FOLLOW_PATH_BIT;
        add_steering(g.steering, i, steering);
    }
}

// ---- SteerToAvoidNeighborsCUDAKernel.cu:192-233 ----------------------------
template <class T> inline T nearest_approach_time(V3<T> pos, V3<T> dir, T speed, V3<T> opos,
                                                  V3<T> odir, T ospeed) {
    const V3<T> my_vel = mul(dir, speed);
    const V3<T> other_vel = mul(odir, ospeed);
    const V3<T> rel_vel = sub(other_vel, my_vel);
    const T rel_speed = length(rel_vel);
    if (rel_speed == T(0)) return T(0);
    const V3<T> rel_tangent = dvd(rel_vel, rel_speed);
    const V3<T> rel_pos = sub(pos, opos);
    const T projection = dot(rel_tangent, rel_pos);
    return projection / rel_speed;
}
template <class T> inline T nearest_approach_positions(V3<T> pos, V3<T> dir, T speed, V3<T> opos,
                                                       V3<T> odir, T ospeed, T time,
                                                       V3<T>& threat_at, V3<T>& my_at) {
    const V3<T> my_travel = mul(dir, speed * time);
    const V3<T> other_travel = mul(odir, ospeed * time);
    my_at = add(pos, my_travel);
    threat_at = add(opos, other_travel);
    return distance(my_at, threat_at);
}

// SteerToAvoidCloseNeighborsCUDAKernel (SteerToAvoidNeighborsCUDAKernel.cu:93-187)
// followed by SteerToAvoidNeighborsCUDAKernel (:235-402), launched as in
// SteerToAvoidNeighborsCUDA.cu:116-160.  branch_out (optional) records the
// branch taken: 0 none, 1 anti-parallel, 2 parallel, 3 perpendicular.
template <class T, class S>
void avoid_neighbors(Group<T> g, const unsigned* knn, const S* knn_dist, unsigned k,
                     const S* posB, const S* dirB, const S* speedB, const S* radiusB,
                     unsigned nB, T min_time, T min_sep, bool avoid_close, T w, unsigned mask,
                     unsigned* branch_out, int threads) {
    if (avoid_close) {
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
        for (long long ii = 0; ii < (long long)g.n; ++ii) {
            const size_t i = size_t(ii);
            if (g.applied[i] & mask) continue;
            const V3<T> pos = ld4<T>(g.position, i), dir = ld4<T>(g.direction, i);
            V3<T> steering{0, 0, 0};
            for (unsigned s = 0; s < k; ++s) {
                const unsigned t = knn[i + size_t(s) * g.n];
                if (t >= nB) break;
                const T tdist = T(knn_dist[i + size_t(s) * g.n]);
                const T sum_radii = g.radius[i] + T(radiusB[t]);
                const T min_c2c = min_sep + sum_radii;
                if (tdist < min_c2c) {
                    const V3<T> offset = sub(ld4<T>(posB, t), pos);
                    steering = perpendicular_component(neg(offset), dir);
                    break;
                }
            }
            steering = mul(normalize(steering), w);
            if (!is_zero(steering)) g.applied[i] |= AVOID_CLOSE_NEIGHBORS_BIT;
            add_steering(g.steering, i, steering);
        }
    }
    const unsigned main_mask = mask | AVOID_CLOSE_NEIGHBORS_BIT;
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (long long ii = 0; ii < (long long)g.n; ++ii) {
        const size_t i = size_t(ii);
        if (branch_out) branch_out[i] = 0;
        if (g.applied[i] & main_mask) continue;
        const V3<T> pos = ld4<T>(g.position, i), dir = ld4<T>(g.direction, i);
        const V3<T> side = ld3<T>(g.side, i);
        const T speed = g.speed[i], radius = g.radius[i];
        T min_t = min_time;
        V3<T> threat_at{0, 0, 0}, my_at{0, 0, 0};
        unsigned threat = UINT_MAX;
        V3<T> threat_dir{0, 0, 0}, threat_pos{0, 0, 0};
        T threat_speed = 0;
        for (unsigned s = 0; s < k; ++s) {
            const unsigned b = knn[i + size_t(s) * g.n];
            if (b >= nB) break;
            const T br = T(radiusB[b]), bs = T(speedB[b]);
            const V3<T> bp = ld4<T>(posB, b), bd = ld4<T>(dirB, b);
            const T danger = radius + br;
            const T time = nearest_approach_time(pos, dir, speed, bp, bd, bs);
            if (time >= 0 && time < min_t) {
                if (nearest_approach_positions(pos, dir, speed, bp, bd, bs, time, threat_at,
                                               my_at) < danger) {
                    min_t = time;
                    threat = b;
                    threat_dir = bd;
                    threat_speed = bs;
                    threat_pos = bp;  // decision (iv)
                }
            }
        }
        if (threat == UINT_MAX) continue;
        const T parallelness = dot(dir, threat_dir);
        const T angle = T(0.707f);
        T steer = 0;
        unsigned br = 0;
        if (parallelness < -angle) {
            const V3<T> offset = sub(threat_at, pos);
            const T side_dot = dot(offset, side);
            steer = (side_dot > 0) ? T(-1) : T(1);
            br = 1;
        } else if (parallelness > angle) {
            const V3<T> offset = sub(threat_pos, pos);
            const T side_dot = dot(offset, side);
            steer = (side_dot > 0) ? T(-1) : T(1);
            br = 2;
        } else {
            br = 3;
            if (speed <= threat_speed) {
                const T side_dot = dot(side, mul(threat_dir, threat_speed));
                steer = (side_dot > 0) ? T(-1) : T(1);
            }
        }
        if (branch_out) branch_out[i] = br;
        V3<T> steering = mul(side, steer);
        steering = mul(normalize(steering), w);
        if (!is_zero(steering)) g.applied[i] |= AVOID_NEIGHBORS_BIT;
        add_steering(g.steering, i, steering);
    }
}

// ---- VectorUtils.cuh:390-428 -----------------------------------------------
template <class T> inline bool lines_intersect(V3<T> sa, V3<T> ea, V3<T> sb, V3<T> eb, V3<T>& ip) {
    const T eps = T(0.001f);
    const T denom = ((eb.z - sb.z) * (ea.x - sa.x)) - ((eb.x - sb.x) * (ea.z - sa.z));
    const T numera = ((eb.x - sb.x) * (sa.z - sb.z)) - ((eb.z - sb.z) * (sa.x - sb.x));
    const T numerb = ((ea.x - sa.x) * (sa.z - sb.z)) - ((ea.z - sa.z) * (sa.x - sb.x));
    if (std::fabs(denom) < eps) {
        if (std::fabs(numera) < eps && std::fabs(numerb) < eps) {
            ip = sa;
            return true;
        }
        return false;
    }
    const T ua = numera / denom;
    const T ub = numerb / denom;
    if (ua >= T(0) && ua <= T(1) && ub >= T(0) && ub <= T(1)) {
        ip.x = sa.x + ua * (ea.x - sa.x);
        ip.y = T(0);
        ip.z = sa.z + ua * (ea.z - sa.z);
        return true;
    }
    return false;
}

// ---- AvoidWallsCUDAKernel.cu:67-245 ----------------------------------------
template <class T>
void avoid_walls(Group<T> g, const unsigned* knw, unsigned kw, const orc_walls* walls,
                 T min_time, T w, unsigned mask, int threads) {
    const T feeler = T(4);  // FEELER_LENGTH, AvoidWallsCUDAKernel.cu:41
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (long long ii = 0; ii < (long long)g.n; ++ii) {
        const size_t i = size_t(ii);
        if (g.applied[i] & mask) continue;
        V3<T> pos = ld4<T>(g.position, i), dir = ld4<T>(g.direction, i);
        const V3<T> side = ld3<T>(g.side, i);
        const T speed = g.speed[i], r = g.radius[i];
        V3<T> steering{0, 0, 0};
        const V3<T> vel = mul(dir, speed);
        const V3<T> feelers[3] = {
            add(pos, mul(vel, min_time)),
            add(pos, add(mul(side, feeler * r), mul(dir, feeler * r))),
            add(pos, add(mul(neg(side), feeler * r), mul(dir, feeler * r)))};
        unsigned feeler_index = 0;
        T nearest_d = T(FLT_MAX);
        unsigned nearest_line = UINT_MAX;
        V3<T> nearest_ip{0, 0, 0}, nearest_normal{0, 0, 0};
        bool touching = false;
        for (unsigned s = 0; s < kw; ++s) {
            const unsigned li = knw[i + size_t(s) * g.n];
            if (li >= walls->n) break;
            V3<T> ip{0, 0, 0};
            const V3<T> ln = ld4<T>(walls->normal, li);
            const V3<T> ls = ld4<T>(walls->start, li);
            const V3<T> le = ld4<T>(walls->end, li);
            const V3<T> closest = add(pos, mul(neg(ln), r));
            if (lines_intersect(pos, closest, ls, le, ip)) {
                touching = true;
                nearest_normal = ln;
                nearest_d = distance(pos, ip);
            }
            for (unsigned f = 0; f < 3; ++f) {
                if (lines_intersect(pos, feelers[f], ls, le, ip)) {
                    const T d = distance(pos, ip);
                    if (d < nearest_d) {
                        nearest_d = d;
                        nearest_line = li;
                        nearest_ip = ip;
                        feeler_index = f;
                        nearest_normal = ln;
                    }
                }
            }
        }
        if (touching) {
            const T pen = r - nearest_d;
            pos = add(pos, mul(nearest_normal, pen));
            dir = normalize(perpendicular_component(dir, nearest_normal));
            g.applied[i] |= ANTI_PENETRATION_WALL;
        } else if (nearest_line != UINT_MAX) {
            const T pen = length(sub(feelers[feeler_index], nearest_ip));
            steering = mul(nearest_normal, pen);
            g.applied[i] |= AVOID_WALLS_BIT;
        }
        steering = mul(steering, w);
        add_steering(g.steering, i, steering);
        st4(g.position, i, pos);
        st4(g.direction, i, dir);
    }
}

// ---- UpdateCUDAKernel.cu:47-123 --------------------------------------------
template <class T> void update(Group<T> g, T dt, int threads) {
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (long long ii = 0; ii < (long long)g.n; ++ii) {
        const size_t i = size_t(ii);
        V3<T> dir = ld4<T>(g.direction, i), pos = ld4<T>(g.position, i);
        V3<T> steer = ld4<T>(g.steering, i);
        V3<T> side = ld3<T>(g.side, i), up = ld3<T>(g.up, i);
        T speed = g.speed[i];
        steer = truncate_length(steer, g.max_force[i]);
        const V3<T> acc = dvd(steer, g.mass[i]);
        V3<T> vel = add(mul(dir, speed), mul(acc, dt));
        vel = truncate_length(vel, g.max_speed[i]);
        speed = length(vel);
        if (speed > 0) {
            dir = dvd(vel, speed);
            side = normalize(cross(dir, up));
            up = cross(side, dir);
        }
        pos = add(pos, mul(vel, dt));
        st3(g.side, i, side);
        st3(g.up, i, up);
        st4(g.direction, i, dir);
        st4(g.position, i, pos);
        st4(g.steering, i, V3<T>{0, 0, 0});
        g.speed[i] = speed;
        g.applied[i] = 0;
    }
}

// ---- UpdateCUDAKernelNew.cu:95-268 (updateGroupWithAntiPenetration) ----------
// The update with the walls' anti-penetration, as the reference kernel
// behaves:
//  * the wall list is read row-major, knl[i*k + s] (:149-150), whereas
//    findKNearestNeighbors writes it column-major, so an agent reads the
//    entries the column-major array holds at those positions;
//  * ClosestPointOnLine (:73-80) calls clamp(0.f, 1.f, t), whose argument
//    order (:67-71) returns 1: the point tested is lineStart + (lineEnd -
//    lineStart), the segment's end;
//  * the overlap test keeps the last listed line within the radius (:215-221),
//    the crossing test the nearest crossing (strict <, :205);
//  * appliedKernels is not cleared (:152-153);
//  * an agent whose new speed is 0 keeps its side vector (the reference then
//    writes a shared-memory side it never loaded, :155 and :261).
template <class T>
void update_antipen_wall(Group<T> g, const unsigned* knl, unsigned k, const orc_walls* walls,
                         T dt, int threads) {
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (long long ii = 0; ii < (long long)g.n; ++ii) {
        const size_t i = size_t(ii);
        V3<T> dir = ld4<T>(g.direction, i), pos = ld4<T>(g.position, i);
        V3<T> side = ld3<T>(g.side, i), up = ld3<T>(g.up, i);
        T speed = g.speed[i];
        const T r = g.radius[i];
        const V3<T> steer = truncate_length(ld4<T>(g.steering, i), T(g.max_force[i]));
        const V3<T> acc = dvd(steer, T(g.mass[i]));
        V3<T> vel = add(mul(dir, speed), mul(acc, dt));
        vel = truncate_length(vel, T(g.max_speed[i]));
        const V3<T> future = add(pos, mul(vel, dt));
        T line_d = T(FLT_MAX), hit_d = T(FLT_MAX);
        unsigned line = UINT_MAX, hit = UINT_MAX;
        V3<T> line_n{0, 0, 0}, hit_n{0, 0, 0};
        for (unsigned s = 0; s < k; ++s) {
            const unsigned li = knl[i * k + s];
            if (li >= walls->n) break;
            const V3<T> ls = ld4<T>(walls->start, li), le = ld4<T>(walls->end, li);
            const V3<T> ln = ld4<T>(walls->normal, li);
            V3<T> ip{0, 0, 0};
            if (lines_intersect(pos, future, ls, le, ip)) {
                const T d = distance(pos, ip);
                if (d < hit_d) {
                    hit_d = d;
                    hit = li;
                    hit_n = ln;
                }
            }
            const V3<T> end_pt = add(ls, mul(sub(le, ls), T(1)));
            const V3<T> o = sub(end_pt, pos);
            const T dsq = dot(o, o);
            if (dsq < r * r) {
                line_d = std::sqrt(dsq);
                line = li;
                line_n = ln;
            }
        }
        if (line != UINT_MAX) {
            pos = add(pos, mul(neg(line_n), line_d - r));
            g.applied[i] |= ANTI_PENETRATION_WALL;
        }
        if (hit != UINT_MAX) {
            vel = perpendicular_component(vel, hit_n);
            g.applied[i] |= ANTI_PENETRATION_WALL;
        }
        speed = length(vel);
        if (speed > 0) {
            dir = dvd(vel, speed);
            side = normalize(cross(dir, up));
            up = cross(side, dir);
        }
        pos = add(pos, mul(vel, dt));
        st3(g.side, i, side);
        st3(g.up, i, up);
        st4(g.direction, i, dir);
        st4(g.position, i, pos);
        st4(g.steering, i, V3<T>{0, 0, 0});
        g.speed[i] = speed;
    }
}

// ---- AntiPenetrationWallKernel (AntiPenetrationWallCUDAKernel.cu:52-134) ------
// Turns the heading of an agent whose next move (velocity * dt) crosses one
// of its listed walls parallel to the nearest such wall.  As the reference:
// the early-out test `! applied & KERNEL_AVOID_WALLS_BIT` (:73) is always
// false, so every agent is tested; the wall list is read row-major,
// knl[i*k + s] (:88-91); every agent's direction is rewritten with w = 0
// (:133); the doNotApplyWith mask is not used.
template <class T>
void antipen_wall(Group<T> g, const unsigned* knl, unsigned k, const orc_walls* walls, T dt,
                  int threads) {
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (long long ii = 0; ii < (long long)g.n; ++ii) {
        const size_t i = size_t(ii);
        const V3<T> pos = ld4<T>(g.position, i);
        V3<T> dir = ld4<T>(g.direction, i);
        const V3<T> future = add(pos, mul(mul(dir, T(g.speed[i])), dt));
        T hit_d = T(FLT_MAX);
        unsigned hit = UINT_MAX;
        for (unsigned s = 0; s < k; ++s) {
            const unsigned li = knl[i * k + s];
            if (li >= walls->n) break;
            V3<T> ip{0, 0, 0};
            if (lines_intersect(pos, future, ld4<T>(walls->start, li), ld4<T>(walls->end, li), ip)) {
                const T d = distance(pos, ip);
                if (d < hit_d) {
                    hit_d = d;
                    hit = li;
                }
            }
        }
        if (hit != UINT_MAX) {
            dir = normalize(perpendicular_component(dir, ld4<T>(walls->normal, hit)));
            g.applied[i] |= ANTI_PENETRATION_WALL;
        }
        st4(g.direction, i, dir);
    }
}

// ---- AntiPenetrationAgentsCUDAKernel.cu:57-109 with AntiPenetrationAgentsCUDA::run
// (AntiPenetrationAgentsCUDA.cu:62-98) ------------------------------------------
// Each agent not masked by its own bits moves away from its nearest neighbour
// (the first KNN entry) when their radii overlap: by the whole overlap when
// the neighbour's bits hit the mask, else by half.  The new positions go to a
// copy of the positions (w = 0 where moved) that replaces them afterwards;
// the neighbour's position and bits are the ones before this pass (posB4 and
// appliedB are read only).
template <class T>
void antipen_agents(Group<T> g, const unsigned* knn_idx, const T* knn_dist, const T* posB4,
                    const T* radiusB, const unsigned* appliedB, unsigned nB, unsigned mask,
                    int threads) {
    std::vector<T> out(g.position, g.position + size_t(4) * g.n);
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (long long ii = 0; ii < (long long)g.n; ++ii) {
        const size_t i = size_t(ii);
        if (g.applied[i] & mask) continue;
        const unsigned b = knn_idx[i];
        if (b >= nB) continue;
        const T sum_radii = g.radius[i] + radiusB[b];
        const T overlap = sum_radii - knn_dist[i];
        if (overlap < T(0)) continue;
        const V3<T> pos = ld4<T>(g.position, i);
        const V3<T> unit = normalize(sub(pos, ld4<T>(posB4, b)));
        const T move = (appliedB[b] & mask) ? overlap : T(0.5f) * overlap;
        st4(out.data(), i, add(pos, mul(unit, move)));
        g.applied[i] |= ANTI_PENETRATION_AGENT;
    }
    std::copy(out.begin(), out.end(), g.position);
}

// ---- one whole step (plugins/ChokePointNew.cpp:586-630, BoidsGroup.cpp:606-637)
template <class T>
int run_steps(Group<T> g, const orc_walls* walls, const orc_step_params* p, unsigned steps,
              unsigned* knn_idx_out, float* knn_dist_out, int threads) {
    const unsigned n = g.n, k = p->k;
    if (k == 0 || n == 0) return -1;
    std::vector<unsigned> idx(size_t(k) * n);
    std::vector<T> dist(size_t(k) * n);
    const bool has_walls = walls && walls->n > 0 && p->knw > 0;
    std::vector<unsigned> widx(has_walls ? size_t(p->knw) * n : 0);
    std::vector<T> wdist(has_walls ? size_t(p->knw) * n : 0);
    std::vector<T> ws_mid;
    if (has_walls) {
        ws_mid.resize(size_t(walls->n) * 4);
        for (size_t j = 0; j < ws_mid.size(); ++j) ws_mid[j] = T(walls->mid[j]);
    }
    for (unsigned step = 0; step < steps; ++step) {
        wrap_world(g, p->world_size, p->wrap_mode, threads);
        if (p->clear_applied)
            for (unsigned i = 0; i < n; ++i) g.applied[i] = 0;
        if (p->knn_mode == ORC_KNN_BRUTEFORCE)
            knn_brute<T>(g.position, n, g.position, n, true, k, idx.data(), dist.data(), threads);
        else
            knn_binned<T>(g.position, n, g.position, n, true, p->world_size, p->world_cells,
                          p->search_radius, k, idx.data(), dist.data(), threads);
        if (has_walls)
            knn_binned<T>(g.position, n, ws_mid.data(), walls->n, false, p->world_size,
                          p->world_cells, p->search_radius, p->knw, widx.data(), wdist.data(),
                          threads);
        for (unsigned o = 0; o < p->n_order; ++o) {
            switch (p->order[o]) {
                case ORC_B_AVOID_WALLS:
                    if (has_walls)
                        avoid_walls(g, widx.data(), p->knw, walls, T(p->min_time_to_wall),
                                    T(p->w_walls), p->mask_walls, threads);
                    break;
                case ORC_B_AVOID_NEIGHBORS:
                    avoid_neighbors<T, T>(g, idx.data(), dist.data(), k, g.position, g.direction,
                                          g.speed, g.radius, n, T(p->min_time_to_collision),
                                          T(p->min_separation_distance), p->avoid_close != 0,
                                          T(p->w_avoid), p->mask_avoid, nullptr, threads);
                    break;
                case ORC_B_SEPARATION:
                    flock<T, T>(g, 0, idx.data(), k, g.position, g.direction, n, T(p->sep_min),
                                T(p->sep_max), T(p->sep_cos), T(p->w_sep), p->mask_sep, threads);
                    break;
                case ORC_B_ALIGNMENT:
                    flock<T, T>(g, 1, idx.data(), k, g.position, g.direction, n, T(p->ali_min),
                                T(p->ali_max), T(p->ali_cos), T(p->w_ali), p->mask_ali, threads);
                    break;
                case ORC_B_COHESION:
                    flock<T, T>(g, 2, idx.data(), k, g.position, g.direction, n, T(p->coh_min),
                                T(p->coh_max), T(p->coh_cos), T(p->w_coh), p->mask_coh, threads);
                    break;
                case ORC_B_FOLLOW_PATH:
                    if (!p->path || p->path->n < 2) return -3;
                    follow_path(g, path_view<T>(p->path), T(p->path_prediction_time),
                                T(p->w_path), p->mask_path, threads);
                    break;
                case ORC_B_SEEK:
                    seek(g, V3<T>{T(p->seek_target[0]), T(p->seek_target[1]), T(p->seek_target[2])},
                         T(p->w_seek), p->mask_seek, threads);
                    break;
                default:
                    return -2;
            }
        }
        update(g, T(p->dt), threads);
    }
    if (knn_idx_out) std::memcpy(knn_idx_out, idx.data(), idx.size() * sizeof(unsigned));
    if (knn_dist_out)
        for (size_t j = 0; j < dist.size(); ++j) knn_dist_out[j] = float(dist[j]);
    return 0;
}

// ---- WallGroupData.cu:28-71 -------------------------------------------------
inline bool segment_enters_box(V3<float> start, V3<float> end, V3<float> bmin_, V3<float> bmax_,
                               V3<float>& ip) {
    float st, et, fst = 0, fet = 1;
    const float bmin[3] = {bmin_.x, bmin_.y, bmin_.z}, bmax[3] = {bmax_.x, bmax_.y, bmax_.z};
    const float si[3] = {start.x, start.y, start.z}, ei[3] = {end.x, end.y, end.z};
    for (int a = 0; a < 3; ++a) {
        if (si[a] < ei[a]) {
            if (si[a] > bmax[a] || ei[a] < bmin[a]) return false;
            const float di = ei[a] - si[a];
            st = (si[a] < bmin[a]) ? (bmin[a] - si[a]) / di : 0;
            et = (ei[a] > bmax[a]) ? (bmax[a] - si[a]) / di : 1;
        } else {
            if (ei[a] > bmax[a] || si[a] < bmin[a]) return false;
            const float di = ei[a] - si[a];
            st = (si[a] > bmax[a]) ? (bmax[a] - si[a]) / di : 0;
            et = (ei[a] < bmin[a]) ? (bmin[a] - si[a]) / di : 1;
        }
        if (st > fst) fst = st;
        if (et < fet) fet = et;
        if (fet < fst) return false;
    }
    ip = add(start, mul(sub(end, start), fst));
    return true;
}

struct Seg { V3<float> s, m, e, n; };

}  // namespace

extern "C" {

int orc_max_threads(void) { return nthreads(0); }

void orc_cell_index(const float* pos4, unsigned n, const float ws[3], const unsigned wc[3],
                    unsigned* cell_out) {
    for (unsigned i = 0; i < n; ++i) {
        unsigned ix, iy, iz;
        cell_coords(ld4<float>(pos4, i), ws, wc, ix, iy, iz);
        cell_out[i] = cell_label(ix, iy, iz, wc);
    }
}

// ComputeCellDensityKernel (ProcessData.cu:132-160).
void orc_cell_density(const float* pos4, unsigned n, const float ws[3], const unsigned wc[3],
                      unsigned* counts_out) {
    const size_t C = size_t(wc[0]) * wc[1] * wc[2];
    std::fill(counts_out, counts_out + C, 0u);
    for (unsigned i = 0; i < n; ++i) {
        unsigned ix, iy, iz;
        cell_coords(ld4<float>(pos4, i), ws, wc, ix, iy, iz);
        counts_out[cell_label(ix, iy, iz, wc)]++;
    }
}

// ComputeAvgCellVelocityKernel (ProcessData.cu:194-237): the database holds
// each cell's agents in the stable sort's order, i.e. ascending index, so
// visiting agents in index order and adding into their cell is that order.
void orc_cell_avg_velocity(const float* pos4, const float* dir4, const float* speed, unsigned n,
                           const float ws[3], const unsigned wc[3], float* avg3_out) {
    const size_t C = size_t(wc[0]) * wc[1] * wc[2];
    std::vector<V3<float>> sum(C, V3<float>{0.f, 0.f, 0.f});
    std::vector<unsigned> cnt(C, 0u);
    for (unsigned i = 0; i < n; ++i) {
        unsigned ix, iy, iz;
        cell_coords(ld4<float>(pos4, i), ws, wc, ix, iy, iz);
        const unsigned c = cell_label(ix, iy, iz, wc);
        sum[c] = add(sum[c], mul(ld4<float>(dir4, i), speed[i]));
        cnt[c]++;
    }
    for (size_t c = 0; c < C; ++c)
        st3(avg3_out, c, cnt[c] ? dvd(sum[c], float(cnt[c])) : V3<float>{0.f, 0.f, 0.f});
}

int orc_knn_binned(const float* posA4, unsigned nA, const float* posB4, unsigned nB,
                   int group_with_self, const float ws[3], const unsigned wc[3],
                   unsigned search_radius, unsigned k, unsigned* idx_out, float* dist_out,
                   int threads) {
    if (k == 0 || wc[0] == 0 || wc[1] == 0 || wc[2] == 0) return -1;
    knn_binned<float>(posA4, nA, posB4, nB, group_with_self != 0, ws, wc, search_radius, k,
                      idx_out, dist_out, threads);
    return 0;
}

int orc_knn_bruteforce(const float* posA4, unsigned nA, const float* posB4, unsigned nB,
                       int group_with_self, unsigned k, unsigned* idx_out, float* dist_out,
                       int threads) {
    if (k == 0) return -1;
    knn_brute<float>(posA4, nA, posB4, nB, group_with_self != 0, k, idx_out, dist_out, threads);
    return 0;
}

void orc_wrap_world(orc_group* g, const float ws[3], int mode) {
    wrap_world(view<float>(g), ws, mode, 0);
}

void orc_steer_separation(orc_group* g, const unsigned* knn_idx, unsigned k, const float* posB4,
                          unsigned nB, float min_d, float max_d, float cos_max, float w,
                          unsigned mask) {
    flock<float, float>(view<float>(g), 0, knn_idx, k, posB4, nullptr, nB, min_d, max_d, cos_max,
                        w, mask, 0);
}

void orc_steer_alignment(orc_group* g, const unsigned* knn_idx, unsigned k, const float* posB4,
                         const float* dirB4, unsigned nB, float min_d, float max_d,
                         float cos_max, float w, unsigned mask) {
    flock<float, float>(view<float>(g), 1, knn_idx, k, posB4, dirB4, nB, min_d, max_d, cos_max, w,
                        mask, 0);
}

void orc_steer_cohesion(orc_group* g, const unsigned* knn_idx, unsigned k, const float* posB4,
                        unsigned nB, float min_d, float max_d, float cos_max, float w,
                        unsigned mask) {
    flock<float, float>(view<float>(g), 2, knn_idx, k, posB4, nullptr, nB, min_d, max_d, cos_max,
                        w, mask, 0);
}

void orc_steer_seek(orc_group* g, const float target[3], float w, unsigned mask) {
    seek(view<float>(g), V3<float>{target[0], target[1], target[2]}, w, mask, 0);
}

void orc_steer_avoid_neighbors(orc_group* g, const unsigned* knn_idx, const float* knn_dist,
                               unsigned k, const float* posB4, const float* dirB4,
                               const float* speedB, const float* radiusB, unsigned nB,
                               float min_time, float min_sep, int avoid_close, float w,
                               unsigned mask) {
    avoid_neighbors<float, float>(view<float>(g), knn_idx, knn_dist, k, posB4, dirB4, speedB,
                                  radiusB, nB, min_time, min_sep, avoid_close != 0, w, mask,
                                  nullptr, 0);
}

/* As orc_steer_avoid_neighbors, recording the branch taken per agent. */
void orc_steer_avoid_neighbors_dbg(orc_group* g, const unsigned* knn_idx, const float* knn_dist,
                                   unsigned k, const float* posB4, const float* dirB4,
                                   const float* speedB, const float* radiusB, unsigned nB,
                                   float min_time, float min_sep, int avoid_close, float w,
                                   unsigned mask, unsigned* branch_out) {
    avoid_neighbors<float, float>(view<float>(g), knn_idx, knn_dist, k, posB4, dirB4, speedB,
                                  radiusB, nB, min_time, min_sep, avoid_close != 0, w, mask,
                                  branch_out, 0);
}

void orc_steer_avoid_walls(orc_group* g, const unsigned* knw_idx, unsigned knw,
                           const orc_walls* walls, float min_time, float w, unsigned mask) {
    avoid_walls(view<float>(g), knw_idx, knw, walls, min_time, w, mask, 0);
}

void orc_update(orc_group* g, float dt) { update(view<float>(g), dt, 0); }

void orc_update_with_antipenetration(orc_group* g, const unsigned* knl, unsigned k,
                                     const orc_walls* walls, float dt) {
    update_antipen_wall(view<float>(g), knl, k, walls, dt, 0);
}

void orc_antipenetration_wall(orc_group* g, const unsigned* knl, unsigned k,
                              const orc_walls* walls, float dt) {
    antipen_wall(view<float>(g), knl, k, walls, dt, 0);
}

void orc_antipenetration_agents(orc_group* g, const unsigned* knn_idx, const float* knn_dist,
                                const float* posB4, const float* radiusB,
                                const unsigned* appliedB, unsigned nB, unsigned mask) {
    antipen_agents(view<float>(g), knn_idx, knn_dist, posB4, radiusB, appliedB, nB, mask, 0);
}

// PolylinePathwayCUDA::Initialize (PolylinePathwayCUDA.cu:17-56): binary32
// host arithmetic, in the reference's order.
int orc_path_init(const float* points3, unsigned n_in, int cyclic, float* points_out3,
                  float* lengths_out, float* normals_out3, float* total_out) {
    const unsigned n = n_in + (cyclic ? 1u : 0u);
    float total = 0.f;
    for (unsigned i = 0; i < n; ++i) {
        const bool close_cycle = cyclic && i == n - 1;
        const unsigned j = close_cycle ? 0 : i;
        st3(points_out3, i, ld3<float>(points3, j));
        if (i > 0) {
            const V3<float> seg = sub(ld3<float>(points_out3, i), ld3<float>(points_out3, i - 1));
            lengths_out[i] = length(seg);
            st3(normals_out3, i, normalize(seg));
            total += lengths_out[i];
        } else {
            lengths_out[0] = 0.f;
            st3(normals_out3, 0, V3<float>{0.f, 0.f, 0.f});
        }
    }
    *total_out = total;
    return int(n);
}

void orc_steer_follow_path(orc_group* g, const orc_path* path, float prediction_time, float w,
                           unsigned mask) {
    follow_path(view<float>(g), path_view<float>(path), prediction_time, w, mask, 0);
}

// WallGroupData::LoadFromFile, WallGroupData.cu:73-106.
int orc_walls_load(const char* path, float* start4, float* mid4, float* end4, float* normal4,
                   unsigned cap) {
    std::ifstream in(path);
    if (!in.is_open()) return -1;
    unsigned n = 0;
    while (!in.eof()) {
        float s[3], e[3], nn[3];
        in >> s[0] >> s[1] >> s[2];
        in >> e[0] >> e[1] >> e[2];
        in >> nn[0] >> nn[1] >> nn[2];
        if (!in.good()) break;
        if (n >= cap) return -2;
        for (int a = 0; a < 3; ++a) {
            start4[4 * n + a] = s[a];
            end4[4 * n + a] = e[a];
            normal4[4 * n + a] = nn[a];
            mid4[4 * n + a] = 0.5f * (s[a] + e[a]);
        }
        start4[4 * n + 3] = end4[4 * n + 3] = normal4[4 * n + 3] = mid4[4 * n + 3] = 0.f;
        ++n;
    }
    return int(n);
}

// WallGroupData::SplitWalls, WallGroupData.cu:108-206, over the bin_cell list
// of KNNBinDataV2::CreateCells (KNNBinDataV2.cu:73-138).  The cell scan is
// restricted to the segment's bounding box (plus one cell); cells outside it
// cannot intersect, so the first intersecting cell in bin_cell order is the
// same as in a scan over all cells.
int orc_walls_split(const float* start4, const float* mid4, const float* end4,
                    const float* normal4, unsigned n, const float ws[3], const unsigned wc[3],
                    float* out_start4, float* out_mid4, float* out_end4, float* out_normal4,
                    unsigned cap) {
    const V3<float> step{ws[0] / float(wc[0]), ws[1] / float(wc[1]), ws[2] / float(wc[2])};
    auto cell_min = [&](unsigned ix, unsigned iy, unsigned iz) {
        return V3<float>{float(ix) * step.x - 0.5f * ws[0], float(iy) * step.y - 0.5f * ws[1],
                         float(iz) * step.z - 0.5f * ws[2]};
    };
    auto range = [&](float lo, float hi, int axis, unsigned& i0, unsigned& i1) {
        const float w = ws[axis], st = (axis == 0 ? step.x : axis == 1 ? step.y : step.z);
        const double a = std::floor((double(lo) + 0.5 * w) / st) - 1.0;
        const double b = std::floor((double(hi) + 0.5 * w) / st) + 1.0;
        const double top = double(wc[axis]) - 1.0;
        if (b < 0.0 || a > top) return false;
        i0 = unsigned(std::max(a, 0.0));
        i1 = unsigned(std::min(b, top));
        return true;
    };
    std::list<Seg> segs;
    for (unsigned i = 0; i < n; ++i)
        segs.push_back(Seg{ld4<float>(start4, i), ld4<float>(mid4, i), ld4<float>(end4, i),
                           ld4<float>(normal4, i)});
    const float eps = 0.001f;
    for (auto it = segs.begin(); it != segs.end();) {
        bool split = false;
        unsigned x0, x1, y0, y1, z0, z1;
        const V3<float> s = it->s, e = it->e;
        if (range(std::min(s.x, e.x), std::max(s.x, e.x), 0, x0, x1) &&
            range(std::min(s.y, e.y), std::max(s.y, e.y), 1, y0, y1) &&
            range(std::min(s.z, e.z), std::max(s.z, e.z), 2, z0, z1)) {
            for (unsigned iy = y0; iy <= y1 && !split; ++iy)
                for (unsigned iz = z0; iz <= z1 && !split; ++iz)
                    for (unsigned ix = x0; ix <= x1 && !split; ++ix) {
                        const V3<float> bmin = cell_min(ix, iy, iz);
                        const V3<float> bmax = add(bmin, step);
                        V3<float> ip;
                        if (!segment_enters_box(s, e, bmin, bmax, ip)) continue;
                        if (distance(s, ip) > eps && distance(ip, e) > eps) {
                            const V3<float> m1 = add(s, mul(sub(ip, s), 0.5f));
                            segs.push_back(Seg{s, m1, ip, it->n});
                            const V3<float> m2 = add(ip, mul(sub(e, ip), 0.5f));
                            segs.push_back(Seg{ip, m2, e, it->n});
                            split = true;
                        }
                    }
        }
        if (split) it = segs.erase(it);
        else ++it;
    }
    if (segs.size() > cap) return -1;
    unsigned o = 0;
    for (const Seg& sg : segs) {
        st4(out_start4, o, sg.s);
        st4(out_mid4, o, sg.m);
        st4(out_end4, o, sg.e);
        st4(out_normal4, o, sg.n);
        ++o;
    }
    return int(o);
}

int orc_run(orc_group* g, const orc_walls* walls, const orc_step_params* p, unsigned steps,
            unsigned* knn_idx, float* knn_dist, int threads) {
    return run_steps<float>(view<float>(g), walls, p, steps, knn_idx, knn_dist, threads);
}

int orc_run_d(orc_group_d* g, const orc_walls* walls, const orc_step_params* p, unsigned steps,
              int threads) {
    return run_steps<double>(view<double>(g), walls, p, steps, nullptr, nullptr, threads);
}

}  // extern "C"
