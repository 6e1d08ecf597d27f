// Binary32 vector math of the GPUSteer group path.
//
// Every function restates include/OpenSteer/VectorUtils.cuh:35-189 (and
// FlockingCommon.cuh, the nearest-approach helpers of
// SteerToAvoidNeighborsCUDAKernel.cu:192-233 and LinesIntersect,
// VectorUtils.cuh:390-428) with the same operation order.  The library is
// compiled with -fmad=false and IEEE division / square root, so each
// expression rounds exactly as written; results are bit-identical to the
// reference kernels evaluated without FMA contraction.
#pragma once

#include <cfloat>
#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

#define GS_HD __host__ __device__ __forceinline__

namespace gs {

struct V3 {
    float x, y, z;
};

GS_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
GS_HD V3 v3(float4 a) { return V3{a.x, a.y, a.z}; }
GS_HD float4 f4(V3 a, float w) { return make_float4(a.x, a.y, a.z, w); }
GS_HD V3 add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
GS_HD V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
GS_HD V3 neg(V3 a) { return V3{-a.x, -a.y, -a.z}; }
GS_HD V3 mul(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
GS_HD V3 dvd(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
GS_HD float dot(V3 a, V3 b) { return ((a.x * b.x) + (a.y * b.y)) + (a.z * b.z); }
GS_HD float length(V3 a) { return sqrtf(dot(a, a)); }
GS_HD V3 normalize(V3 v) {
    const float len = length(v);
    return (len > 0.f) ? dvd(v, len) : v;
}
GS_HD V3 cross(V3 a, V3 b) {
    return V3{(a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x)};
}
GS_HD bool is_zero(V3 a) { return a.x == 0.f && a.y == 0.f && a.z == 0.f; }
GS_HD float distance(V3 a, V3 b) { return length(sub(a, b)); }
// The squared distance under distance()'s square root: distance(a, b) is
// sqrtf(dist_sq(a, b)) bit for bit.
GS_HD float dist_sq(V3 a, V3 b) {
    const V3 o = sub(a, b);
    return dot(o, o);
}
GS_HD V3 perpendicular_component(V3 v, V3 u) { return sub(v, mul(u, dot(v, u))); }
GS_HD V3 truncate_length(V3 v, float max_len) {
    const float max_sq = max_len * max_len;
    const float len_sq = dot(v, v);
    if (len_sq <= max_sq) return v;
    return mul(v, max_len / sqrtf(len_sq));
}

// Kernel bit masks (CUDAKernelGlobals.cuh:12-29).
constexpr unsigned SEEK_BIT = 1u << 2;
constexpr unsigned SEPARATION_BIT = 1u << 4;
constexpr unsigned ALIGNMENT_BIT = 1u << 5;
constexpr unsigned COHESION_BIT = 1u << 6;
constexpr unsigned AVOID_WALLS_BIT = 1u << 8;
constexpr unsigned AVOID_NEIGHBORS_BIT = 1u << 9;
constexpr unsigned AVOID_CLOSE_NEIGHBORS_BIT = 1u << 10;
constexpr unsigned FOLLOW_PATH_BIT = 1u << 11;
constexpr unsigned ANTI_PENETRATION_WALL = 1u << 12;
constexpr unsigned ANTI_PENETRATION_AGENT = 1u << 13;

// ---- cells (KNNBinningV2Kernel.cu:269-296, KNNBinDataV2.cu:103-116) --------
// Normalised coordinate u = (p + W/2) / W point-sampled with clamping:
// i = clamp(floor(u * n), 0, n - 1).  Labels run x + z*X + y*X*Z.
GS_HD unsigned cell_coord(float p, float w, unsigned n) {
    const float u = (p + 0.5f * w) / w;
    const float f = floorf(u * float(n));
    if (!(f >= 0.f)) return 0u;
    if (f >= float(n)) return n - 1;
    return unsigned(f);
}

struct Grid {
    float ws[3];
    unsigned wc[3];
};

GS_HD void cell_coords(const Grid& g, V3 p, unsigned& ix, unsigned& iy, unsigned& iz) {
    ix = cell_coord(p.x, g.ws[0], g.wc[0]);
    iy = cell_coord(p.y, g.ws[1], g.wc[1]);
    iz = cell_coord(p.z, g.ws[2], g.wc[2]);
}
GS_HD unsigned cell_label(const Grid& g, unsigned ix, unsigned iy, unsigned iz) {
    return ix + iz * g.wc[0] + iy * g.wc[0] * g.wc[2];
}
GS_HD unsigned cell_of(const Grid& g, V3 p) {
    unsigned ix, iy, iz;
    cell_coords(g, p, ix, iy, iz);
    return cell_label(g, ix, iy, iz);
}

// ---- WrapWorldCUDAKernel.cu:21-47 ----------------------------------------------
enum WrapMode : int { WRAP_REFERENCE = 0, WRAP_SYMMETRIC = 1, WRAP_NONE = 2 };

GS_HD V3 wrap_world(V3 p, const float ws[3], int mode) {
    if (mode == WRAP_NONE) return p;
    const V3 half = mul(v3(ws[0], ws[1], ws[2]), 0.5f);
    if (p.x < -half.x) p.x = half.x;
    if (p.x > half.x) p.x = -half.x;
    if (p.y < -half.y) p.y = half.y;
    if (p.y > half.y) p.y = -half.y;
    if (mode == WRAP_REFERENCE) {
        if (p.z < 0.f) p.z = half.z + 100.f;
    } else {
        if (p.z < -half.z) p.z = half.z;
        if (p.z > half.z) p.z = -half.z;
    }
    return p;
}

// ---- total order of every KNN here: (distance, agent index) -------------------
GS_HD bool knn_less(float d1, unsigned i1, float d2, unsigned i2) {
    return d1 < d2 || (d1 == d2 && i1 < i2);
}

// ---- FlockingCommon.cuh:4-30 -----------------------------------------------------
// `d` is length(offset), computed once by the caller for all behaviours.
GS_HD bool in_boid_neighborhood(V3 dir, V3 offset, float d, float min_d, float max_d,
                                float cos_max) {
    if (d < min_d) return true;
    if (d > max_d) return false;
    const V3 unit = dvd(offset, d);
    return dot(dir, unit) > cos_max;
}

// ---- SteerToAvoidNeighborsCUDAKernel.cu:192-233 -----------------------------------
GS_HD float nearest_approach_time(V3 pos, V3 dir, float speed, V3 opos, V3 odir, float ospeed) {
    const V3 my_vel = mul(dir, speed);
    const V3 other_vel = mul(odir, ospeed);
    const V3 rel_vel = sub(other_vel, my_vel);
    const float rel_speed = length(rel_vel);
    if (rel_speed == 0.f) return 0.f;
    const V3 rel_tangent = dvd(rel_vel, rel_speed);
    const V3 rel_pos = sub(pos, opos);
    const float projection = dot(rel_tangent, rel_pos);
    return projection / rel_speed;
}
GS_HD float nearest_approach_positions(V3 pos, V3 dir, float speed, V3 opos, V3 odir,
                                       float ospeed, float time, V3& threat_at) {
    const V3 my_travel = mul(dir, speed * time);
    const V3 other_travel = mul(odir, ospeed * time);
    const V3 my_at = add(pos, my_travel);
    threat_at = add(opos, other_travel);
    return distance(my_at, threat_at);
}

// ---- VectorUtils.cuh:390-428 (x/z plane) ------------------------------------------
GS_HD bool lines_intersect(V3 sa, V3 ea, V3 sb, V3 eb, V3& ip) {
    const float eps = 0.001f;
    const float denom = ((eb.z - sb.z) * (ea.x - sa.x)) - ((eb.x - sb.x) * (ea.z - sa.z));
    const float numera = ((eb.x - sb.x) * (sa.z - sb.z)) - ((eb.z - sb.z) * (sa.x - sb.x));
    const float numerb = ((ea.x - sa.x) * (sa.z - sb.z)) - ((ea.z - sa.z) * (sa.x - sb.x));
    if (fabsf(denom) < eps) {
        if (fabsf(numera) < eps && fabsf(numerb) < eps) {
            ip = sa;
            return true;
        }
        return false;
    }
    const float ua = numera / denom;
    const float ub = numerb / denom;
    if (ua >= 0.f && ua <= 1.f && ub >= 0.f && ub <= 1.f) {
        ip.x = sa.x + ua * (ea.x - sa.x);
        ip.y = 0.f;
        ip.z = sa.z + ua * (ea.z - sa.z);
        return true;
    }
    return false;
}

}  // namespace gs
