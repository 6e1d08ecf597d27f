// Per-agent steering behaviours and integration, shared by the per-behaviour
// (drop-in) kernels and the fused step kernels.
//
// A behaviour is split into an accumulation over the agent's KNN list (one
// call per neighbour, in list order) and a finalisation that applies the
// weight, the applied-kernel bit and the add into the steering vector, exactly
// as the reference kernel does for that agent.  The fused kernels run all
// accumulations in a single pass over the neighbours and then finalise the
// behaviours in the scenario's order; each accumulator sees the same operands
// in the same order as the reference's separate kernel, so the results are
// identical.
#pragma once

#include "gs_math.cuh"

namespace gs {

struct Self {
    V3 pos, dir, side, up;
    float speed, radius, max_speed, max_force, mass;
};

// ---- flocking: SteerFor{Separation,Alignment,Cohesion}CUDAKernel.cu -------------
struct FlockAcc {
    V3 sum;
    unsigned n;
};
struct FlockParams {
    float min_d, max_d, cos_max, w;
    unsigned mask;
    // squared-distance thresholds: d < min_d <=> dsq < lt, d > max_d <=> dsq > gt
    float lt, gt;
};

// Packed (min, max, cos, weight, mask bits) as the fused step's parameters
// hold them, with the squared-distance thresholds (lt, gt).
__device__ __forceinline__ FlockParams flock_params(const float v[5], const float dsq[2]) {
    return FlockParams{v[0], v[1], v[2], v[3], __float_as_uint(v[4]), dsq[0], dsq[1]};
}

// ---- the angle test of inBoidNeighborhood without its divisions ----------------
// FlockingCommon.cuh:24-27 tests f > c with f = dot(dir, offset / d), the unit
// offset rounded componentwise (three IEEE divisions).  With g = dot(dir,
// offset) (same operation order) and real arithmetic, d (F - c) = (a.o) - c d
// for F the exact value of f; the rounding errors of f, of g and of c d are
// bounded by standard floating-point error analysis:
//   |f - F| <= gamma_4 S / d,  |g - a.o| <= gamma_3 S,  |fl(c d) - c d| <= u |c| d,
// u = 2^-24, gamma_n = n u / (1 - n u), S = sum |dir_i offset_i| <= A d (1 + 3u)
// with A = |dir_x| + |dir_y| + |dir_z|.  So when
//   |g - c d| > (gamma_3 + gamma_4) A d (1 + 3u) + u |c| d + (error of d's estimate) |c|
// the sign of g - c d is the sign of f - c, and f != c.  The margin used is
// 2^-14 (A + |c|) d: over 100 times the A term (about 2^-21 A d) and, with d
// estimated by sqrt.approx to better than 2^-20 relative, over 50 times the
// c term; it holds for any estimate better than 2^-15.  The estimate is only
// trusted for squared distances in [2^-60, 2^60] and A + |c| in [2^-60, 2^30]
// (no underflow or overflow in any term).  Everywhere else, and inside the
// margin, the reference's expression decides.  The result is the reference's
// bit for bit; only the cost differs.
struct AngleGate {
    float k;  // 2^-14 (A + |c|), or +inf where the estimate is not trusted
};

__device__ __forceinline__ AngleGate angle_gate(V3 dir, float c) {
    const float s = (fabsf(dir.x) + fabsf(dir.y) + fabsf(dir.z)) + fabsf(c);
    return AngleGate{(s >= 0x1p-60f && s <= 0x1p30f) ? 0x1p-14f * s : __int_as_float(0x7f800000)};
}

// sqrt.approx of a squared distance in [2^-60, 2^60], NaN elsewhere (so that
// no margin test passes and the exact expression decides).
__device__ __forceinline__ float d_estimate(float dsq) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(dsq));
    return (dsq >= 0x1p-60f && dsq <= 0x1p60f) ? r : __int_as_float(0x7fffffff);
}

// The reference's f = dot(dir, offset / d), d = sqrtf(dsq), out of line: the
// gate decides almost every test, so this stays out of the unrolled loops.
static __device__ __noinline__ float forward_component(V3 dir, V3 offset, float dsq) {
    return dot(dir, dvd(offset, sqrtf(dsq)));
}

// 1: f > c; 0: f <= c; -1: undecided (the caller evaluates the reference's
// expression).  g = dot(dir, offset), de = d_estimate(dsq).
__device__ __forceinline__ int angle_decide(float g, float de, float c, AngleGate gate) {
    const float diff = g - c * de;
    if (!(fabsf(diff) > gate.k * de)) return -1;
    return diff > 0.f ? 1 : 0;
}

GS_HD void flock_init(FlockAcc& a) {
    a.sum = v3(0.f, 0.f, 0.f);
    a.n = 0;
}
// SteerForSeparationCUDAKernel.cu:109-116
GS_HD void separation_add(FlockAcc& a, const FlockParams& p, V3 dir, V3 offset, float dsq,
                          float d) {
    if (in_boid_neighborhood(dir, offset, d, p.min_d, p.max_d, p.cos_max)) {
        a.sum = add(a.sum, dvd(offset, -dsq));
        a.n++;
    }
}
// SteerForCohesionCUDAKernel.cu:109-117
GS_HD void cohesion_add(FlockAcc& a, const FlockParams& p, V3 dir, V3 offset, float d, V3 bpos) {
    if (in_boid_neighborhood(dir, offset, d, p.min_d, p.max_d, p.cos_max)) {
        a.sum = add(a.sum, bpos);
        a.n++;
    }
}
// SteerForAlignmentCUDAKernel.cu:110-118
GS_HD void alignment_add(FlockAcc& a, const FlockParams& p, V3 dir, V3 offset, float d, V3 bdir) {
    if (in_boid_neighborhood(dir, offset, d, p.min_d, p.max_d, p.cos_max)) {
        a.sum = add(a.sum, bdir);
        a.n++;
    }
}
// kind 0 separation, 1 alignment, 2 cohesion (…CUDAKernel.cu:119-134 of each).
GS_HD void flock_finish(int kind, const FlockAcc& a, const FlockParams& p, const Self& s,
                        unsigned& applied, V3& steer) {
    if (applied & p.mask) return;
    V3 r = a.sum;
    if (a.n > 0) {
        const V3 mean = dvd(a.sum, float(a.n));
        if (kind == 0) r = normalize(mean);
        else if (kind == 1) r = normalize(sub(mean, s.dir));
        else r = normalize(sub(mean, s.pos));
    }
    r = mul(r, p.w);
    const unsigned bit = kind == 0 ? SEPARATION_BIT : kind == 1 ? ALIGNMENT_BIT : COHESION_BIT;
    if (!is_zero(r)) applied |= bit;
    steer = add(r, steer);
}

// ---- SteerForSeekCUDAKernel.cu:41-71 ------------------------------------------------
GS_HD void seek_finish(V3 target, float w, unsigned mask, const Self& s, unsigned& applied,
                       V3& steer) {
    if (applied & mask) return;
    const V3 desired = sub(target, s.pos);
    V3 r = sub(desired, s.dir);
    r = mul(normalize(r), w);
    if (!is_zero(r)) applied |= SEEK_BIT;
    steer = add(r, steer);
}

// ---- FollowPathCUDAKernel (SteerToFollowPathCUDAKernel.cu:35-287) -------------------
// A polyline pathway on the device: points, segment lengths and unit segment
// directions (index i describes the segment from point i-1 to point i).
struct PathDev {
    const float3* points;
    const float* lengths;
    const float3* normals;
    unsigned n;
    float radius;
    int cyclic;
    float total;
};

GS_HD V3 path_point(const PathDev& P, unsigned i) {
    const float3 v = P.points[i];
    return v3(v.x, v.y, v.z);
}
GS_HD V3 path_normal(const PathDev& P, unsigned i) {
    const float3 v = P.normals[i];
    return v3(v.x, v.y, v.z);
}
// Distance from `point` to segment i (1 <= i < n), its clamped projection
// along the segment and the nearest point (:35-70).
GS_HD float segment_distance(const PathDev& P, unsigned i, V3 point, float& proj, V3& nearest) {
    const V3 a = path_point(P, i - 1), nrm = path_normal(P, i);
    const float len = P.lengths[i];
    proj = dot(nrm, sub(point, a));
    if (proj < 0.f) {
        proj = 0.f;
        nearest = a;
    } else if (proj > len) {
        proj = len;
        nearest = path_point(P, i);
    } else {
        nearest = add(a, mul(nrm, proj));
    }
    return distance(point, nearest);
}
// Path distance of the point's nearest path point, first nearest segment (:72-100).
GS_HD float path_distance_of(const PathDev& P, V3 point) {
    float best = FLT_MAX, walked = 0.f, along = 0.f;
    for (unsigned i = 1; i < P.n; ++i) {
        float proj;
        V3 nearest;
        const float d = segment_distance(P, i, point, proj, nearest);
        if (d < best) {
            best = d;
            along = walked + proj;
        }
        walked += P.lengths[i];
    }
    return along;
}
// Nearest path point and how far `point` is outside the tube (:102-141).
GS_HD V3 nearest_on_path(const PathDev& P, V3 point, float& outside) {
    float best = FLT_MAX;
    V3 on = v3(0.f, 0.f, 0.f);
    for (unsigned i = 1; i < P.n; ++i) {
        float proj;
        V3 nearest;
        const float d = segment_distance(P, i, point, proj, nearest);
        if (d < best) {
            best = d;
            on = nearest;
        }
    }
    outside = distance(on, point) - P.radius;
    return on;
}
// The point at a path distance (:143-181); past the last segment (only by
// rounding) it is the last point, where the reference leaves a value unset.
GS_HD V3 point_at_path_distance(const PathDev& P, float along) {
    float rest = along;
    if (P.cyclic) {
        rest = fmodf(along, P.total);
    } else {
        if (along < 0.f) return path_point(P, 0);
        if (along >= P.total) return path_point(P, P.n - 1);
    }
    for (unsigned i = 1; i < P.n; ++i) {
        const float len = P.lengths[i];
        if (len < rest) {
            rest -= len;
            continue;
        }
        const V3 a = path_point(P, i - 1), b = path_point(P, i);
        return add(a, mul(sub(b, a), rest / len));
    }
    return path_point(P, P.n - 1);
}
// The behaviour for one agent (:183-287): seek a point `prediction_time *
// speed` further along the path unless the predicted position is inside the
// tube and moving the right way.
GS_HD void follow_path_finish(const PathDev& P, float prediction_time, float w, unsigned mask,
                              const Self& s, unsigned& applied, V3& steer) {
    if (applied & mask) return;
    const float ahead = prediction_time * s.speed;
    const V3 future = add(s.pos, mul(mul(s.dir, s.speed), prediction_time));
    const float now_d = path_distance_of(P, s.pos);
    const float future_d = path_distance_of(P, future);
    const bool rightway = (ahead > 0.f) ? (now_d < future_d) : (now_d > future_d);
    float outside;
    nearest_on_path(P, future, outside);
    V3 r = v3(0.f, 0.f, 0.f);
    if (!((outside < 0.f) && rightway))
        r = sub(sub(point_at_path_distance(P, now_d + ahead), s.pos), s.dir);
    r = mul(normalize(r), w);
    if (!is_zero(r)) applied |= FOLLOW_PATH_BIT;
    steer = add(r, steer);
}

// ---- SteerToAvoidCloseNeighborsCUDAKernel (SteerToAvoidNeighborsCUDAKernel.cu:93-187)
struct CloseAcc {
    bool found;
    V3 steer;
};
GS_HD void close_init(CloseAcc& a) {
    a.found = false;
    a.steer = v3(0.f, 0.f, 0.f);
}
// knn_dist is the KNN distance of this list entry, not a recomputed one.
GS_HD void close_add(CloseAcc& a, const Self& s, float min_sep, float knn_dist, V3 bpos,
                     float bradius) {
    if (a.found) return;
    const float sum_radii = s.radius + bradius;
    const float min_c2c = min_sep + sum_radii;
    if (knn_dist < min_c2c) {
        const V3 offset = sub(bpos, s.pos);
        a.steer = perpendicular_component(neg(offset), s.dir);
        a.found = true;
    }
}
GS_HD void close_finish(const CloseAcc& a, float w, unsigned mask, unsigned& applied, V3& steer) {
    if (applied & mask) return;
    const V3 r = mul(normalize(a.steer), w);
    if (!is_zero(r)) applied |= AVOID_CLOSE_NEIGHBORS_BIT;
    steer = add(r, steer);
}

// ---- SteerToAvoidNeighborsCUDAKernel (SteerToAvoidNeighborsCUDAKernel.cu:259-401) ---
struct AvoidAcc {
    float min_t;
    unsigned threat;
    V3 threat_at, threat_dir, threat_pos;
    float threat_speed;
};
GS_HD void avoid_init(AvoidAcc& a, float min_time) {
    a.min_t = min_time;
    a.threat = UINT_MAX;
    a.threat_at = a.threat_dir = a.threat_pos = v3(0.f, 0.f, 0.f);
    a.threat_speed = 0.f;
}
// `threat_at` keeps the nearest-approach position of the last candidate that
// passed the time test, as in the reference (:330-340).
GS_HD void avoid_add(AvoidAcc& a, const Self& s, unsigned bid, V3 bpos, V3 bdir, float bspeed,
                     float bradius) {
    const float danger = s.radius + bradius;
    const float time = nearest_approach_time(s.pos, s.dir, s.speed, bpos, bdir, bspeed);
    if (time >= 0.f && time < a.min_t) {
        if (nearest_approach_positions(s.pos, s.dir, s.speed, bpos, bdir, bspeed, time,
                                       a.threat_at) < danger) {
            a.min_t = time;
            a.threat = bid;
            a.threat_dir = bdir;
            a.threat_speed = bspeed;
            a.threat_pos = bpos;  // the reference reads an uninitialised variable here
        }
    }
}
GS_HD void avoid_finish(const AvoidAcc& a, float w, unsigned mask, const Self& s,
                        unsigned& applied, V3& steer) {
    if (applied & (mask | AVOID_CLOSE_NEIGHBORS_BIT)) return;  // SteerToAvoidNeighborsCUDA.cu:159
    if (a.threat == UINT_MAX) return;
    const float parallelness = dot(s.dir, a.threat_dir);
    const float angle = 0.707f;
    float st = 0.f;
    if (parallelness < -angle) {
        const V3 offset = sub(a.threat_at, s.pos);
        st = (dot(offset, s.side) > 0.f) ? -1.f : 1.f;
    } else if (parallelness > angle) {
        const V3 offset = sub(a.threat_pos, s.pos);
        st = (dot(offset, s.side) > 0.f) ? -1.f : 1.f;
    } else if (s.speed <= a.threat_speed) {
        const float side_dot = dot(s.side, mul(a.threat_dir, a.threat_speed));
        st = (side_dot > 0.f) ? -1.f : 1.f;
    }
    V3 r = mul(s.side, st);
    r = mul(normalize(r), w);
    if (!is_zero(r)) applied |= AVOID_NEIGHBORS_BIT;
    steer = add(r, steer);
}

// The same behaviour with a four-word accumulator, for kernels that can
// read their neighbours again after the pass: the smallest accepted time,
// the threat's list rank, and the rank and time of the last neighbour that
// passed the time test (whose nearest-approach position the reference keeps
// in threat_at).  avoid_lite_full rebuilds AvoidAcc from those two
// neighbours with the expressions avoid_add evaluates, so the result is the
// same bit for bit; the pass itself holds 4 words instead of 12.
struct AvoidLite {
    float min_t, last_t;
    unsigned threat, last;  // list ranks, UINT_MAX for none
};
GS_HD void avoid_lite_init(AvoidLite& a, float min_time) {
    a.min_t = min_time;
    a.last_t = 0.f;
    a.threat = a.last = UINT_MAX;
}
GS_HD void avoid_lite_add(AvoidLite& a, const Self& s, unsigned rank, V3 bpos, V3 bdir,
                          float bspeed, float bradius) {
    const float danger = s.radius + bradius;
    const float time = nearest_approach_time(s.pos, s.dir, s.speed, bpos, bdir, bspeed);
    if (time >= 0.f && time < a.min_t) {
        V3 at;
        a.last = rank;
        a.last_t = time;
        if (nearest_approach_positions(s.pos, s.dir, s.speed, bpos, bdir, bspeed, time, at) <
            danger) {
            a.min_t = time;
            a.threat = rank;
        }
    }
}
// Neighbour avoidance's pre-test: false only when the nearest-approach time
// of a neighbour is provably outside [0, min_t), so that avoid_lite_add
// would leave the accumulator as it is (its window only narrows during the
// pass).  From the relative velocity rv = bdir * bspeed - dir * speed and
// rp = pos - bpos: ss = dot(rv, rv), h = dot(rv, rp) and S = sum |rv_i rp_i|.
// The reference's time (nearest_approach_time, SteerToAvoidNeighborsCUDA
// Kernel.cu:192-233) is t = fl(fl(dot(fl(rv / rs), rp)) / rs) with
// rs = sqrtf(dot(rv, rv)); standard error analysis gives
// |t - h / rs^2| <= gamma_6 S / rs^2 and rs^2 = |rv|^2 (1 + eta), |eta| <= 5u
// (u = 2^-24).  So h < -2^-14 S proves t < 0 (nonzero: S >= 2^-60 and
// |rv|^2 <= 2^60 keep |t| above 2^-134), and h - min_t |rv|^2 >
// 2^-14 (S + min_t |rv|^2) proves t > min_t, each margin hundreds of times
// the rounding bound.  Outside the guarded ranges (tiny or huge magnitudes,
// rs = 0, NaN) it answers true and the exact test runs.  (The sign of a zero
// h does not matter: no comparison here sees it.)
GS_HD bool avoid_time_window_test(float ss, float h, float S, float min_t) {
    if (!(ss >= 0x1p-60f && ss <= 0x1p60f && S >= 0x1p-60f && S <= 0x1p60f && min_t > 0.f &&
          min_t <= 0x1p30f))
        return true;
    if (h < -0x1p-14f * S) return false;
    const float msq = min_t * ss;
    return !(h - msq > 0x1p-14f * (S + msq));
}

// fetch(rank, pos, dir, speed) reads list entry `rank` as the pass saw it.
template <class Fetch>
GS_HD AvoidAcc avoid_lite_full(const AvoidLite& a, Fetch&& fetch) {
    AvoidAcc f;
    avoid_init(f, a.min_t);
    f.threat = a.threat;
    V3 pos, dir;
    float speed;
    if (a.last != UINT_MAX) {
        fetch(a.last, pos, dir, speed);
        f.threat_at = add(pos, mul(dir, speed * a.last_t));  // nearest_approach_positions
    }
    if (a.threat != UINT_MAX) {
        fetch(a.threat, pos, dir, speed);
        f.threat_pos = pos;
        f.threat_dir = dir;
        f.threat_speed = speed;
    }
    return f;
}

// ---- SteerToAvoidWallsCUDAKernel (AvoidWallsCUDAKernel.cu:89-244) -----------------
struct WallAcc {
    V3 feelers[3];
    unsigned feeler_index;
    float nearest_d;
    unsigned nearest_line;
    V3 nearest_ip, nearest_normal;
    bool touching;
};
GS_HD void walls_init(WallAcc& a, const Self& s, float min_time) {
    const float fl = 4.f * s.radius;  // FEELER_LENGTH * radius (AvoidWallsCUDAKernel.cu:41)
    const V3 vel = mul(s.dir, s.speed);
    a.feelers[0] = add(s.pos, mul(vel, min_time));
    a.feelers[1] = add(s.pos, add(mul(s.side, fl), mul(s.dir, fl)));
    a.feelers[2] = add(s.pos, add(mul(neg(s.side), fl), mul(s.dir, fl)));
    a.feeler_index = 0;
    a.nearest_d = FLT_MAX;
    a.nearest_line = UINT_MAX;
    a.nearest_ip = a.nearest_normal = v3(0.f, 0.f, 0.f);
    a.touching = false;
}
GS_HD void walls_add(WallAcc& a, const Self& s, unsigned line, V3 ls, V3 le, V3 ln) {
    V3 ip = v3(0.f, 0.f, 0.f);
    const V3 closest = add(s.pos, mul(neg(ln), s.radius));
    if (lines_intersect(s.pos, closest, ls, le, ip)) {
        a.touching = true;
        a.nearest_normal = ln;
        a.nearest_d = distance(s.pos, ip);
    }
#pragma unroll
    for (unsigned f = 0; f < 3; ++f) {
        if (lines_intersect(s.pos, a.feelers[f], ls, le, ip)) {
            const float d = distance(s.pos, ip);
            if (d < a.nearest_d) {
                a.nearest_d = d;
                a.nearest_line = line;
                a.nearest_ip = ip;
                a.feeler_index = f;
                a.nearest_normal = ln;
            }
        }
    }
}
// Applies the result: may move the agent (anti-penetration) and adds the
// weighted wall steering.  Returns false when masked (nothing changes).
GS_HD bool walls_finish(const WallAcc& a, float w, unsigned mask, Self& s, unsigned& applied,
                        V3& steer) {
    if (applied & mask) return false;
    V3 r = v3(0.f, 0.f, 0.f);
    if (a.touching) {
        const float pen = s.radius - a.nearest_d;
        s.pos = add(s.pos, mul(a.nearest_normal, pen));
        s.dir = normalize(perpendicular_component(s.dir, a.nearest_normal));
        applied |= ANTI_PENETRATION_WALL;
    } else if (a.nearest_line != UINT_MAX) {
        const V3 f = a.feeler_index == 0 ? a.feelers[0]
                     : a.feeler_index == 1 ? a.feelers[1] : a.feelers[2];
        const float pen = length(sub(f, a.nearest_ip));
        r = mul(a.nearest_normal, pen);
        applied |= AVOID_WALLS_BIT;
    }
    r = mul(r, w);
    steer = add(r, steer);
    return true;
}

// ---- UpdateCUDAKernel.cu:78-123 -----------------------------------------------------
// A new speed of 0 keeps the previous side vector (the reference writes back
// uninitialised shared memory there).
GS_HD void integrate(Self& s, V3 steer, float dt) {
    steer = truncate_length(steer, s.max_force);
    const V3 acc = dvd(steer, s.mass);
    V3 vel = add(mul(s.dir, s.speed), mul(acc, dt));
    vel = truncate_length(vel, s.max_speed);
    s.speed = length(vel);
    if (s.speed > 0.f) {
        s.dir = dvd(vel, s.speed);
        s.side = normalize(cross(s.dir, s.up));
        s.up = cross(s.side, s.dir);
    }
    s.pos = add(s.pos, mul(vel, dt));
}

}  // namespace gs
