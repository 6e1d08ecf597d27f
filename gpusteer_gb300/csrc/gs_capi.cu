// C ABI of libgpusteer (include/gpusteer.h): handle management, host <-> device
// transfers, the GroupSteerLibrary.cuh free functions and the fused step.
#include <cmath>
#include <cstdint>
#include <limits>
#include <cstring>
#include <fstream>
#include <list>
#include <new>
#include <string>

#include "gs_launch.h"

namespace gs {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

gs_status fail(gs_status s, const std::string& msg) {
    set_error(msg);
    return s;
}

gs_status cuda_fail(cudaError_t e, const char* what) {
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return GS_ERR_CUDA;
}

static GroupView view(gs_group g) {
    return GroupView{g->position, g->direction, g->steering, g->side, g->up, g->speed,
                     g->max_speed, g->max_force, g->radius, g->mass, g->applied, g->n};
}
static OtherView other_view(gs_group g) {
    return OtherView{g->position, g->direction, g->speed, g->radius, g->applied, g->n};
}

static void release_fused(gs_group g) {
    for (int j = 0; j < 6; ++j) {
        dfree(g->A.f[j]);
        dfree(g->B.f[j]);
    }
    dfree(g->cellrank);
    dfree(g->w0);
    dfree(g->w1);
    dfree(g->w2);
    dfree(g->knn_slot);
    dfree(g->knn_dist);
    dfree(g->d_scene);
    dfree(g->d_err);
    dfree(g->retry);
    dfree(g->slot_of);
    dfree(g->retry_count);
    dfree(g->retry_knn);
    dfree(g->d_stat);
    dfree(g->d_bar);
    db_release(g->fdb);
    g->fused_k_alloc = 0;
}

static void drop_graph(gs_group g) {
    if (g->graph_exec) cudaGraphExecDestroy(g->graph_exec);
    g->graph_exec = nullptr;
}

// Brings the reference-layout arrays up to date after fused steps.
static gs_status ensure_reference(gs_group g) {
    if (!g->fused_current) return GS_OK;
    GS_TRY(fused_to_reference(g->A, g->n, g->d_scene, g->slot_of, view(g), g->stream));
    g->fused_current = false;
    g->db.valid = false;
    return GS_OK;
}

// Marks the reference-layout arrays as modified by a per-function call.
static void touched(gs_group g) {
    g->fused_current = false;
    g->accum_dirty = true;
    g->frame_cells = 0;
}

// A call queued on g's stream reads `other`'s arrays (it waited for other's
// earlier work first).  Later work on other's stream must not overwrite them
// before that read: other's stream waits for g's stream up to here.
static gs_status read_done(gs_group g, gs_group other) {
    if (other == g || other->stream == g->stream) return GS_OK;
    if (!g->read_ev) GS_CUDA(cudaEventCreateWithFlags(&g->read_ev, cudaEventDisableTiming));
    GS_CUDA(cudaEventRecord(g->read_ev, g->stream));
    GS_CUDA(cudaStreamWaitEvent(other->stream, g->read_ev, 0));
    return GS_OK;
}

static bool finite3(const float* v) {
    return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]);
}

static gs_status check_grid(const unsigned wc[3], const float ws[3], Grid& g, unsigned& cells) {
    unsigned long long c = 1;
    for (int a = 0; a < 3; ++a) {
        if (wc[a] == 0) return fail(GS_ERR_INVALID_ARG, "world cells must be positive");
        if (!(ws[a] > 0.f) || !std::isfinite(ws[a]))
            return fail(GS_ERR_INVALID_ARG, "world size must be positive and finite");
        // checked after every factor: the running product stays below 2^62
        c *= wc[a];
        if (c > (1ull << 30)) return fail(GS_ERR_INVALID_ARG, "too many cells");
        g.wc[a] = wc[a];
        g.ws[a] = ws[a];
    }
    cells = unsigned(c);
    return GS_OK;
}

// ---- walls: WallGroupData::LoadFromFile / SplitWalls --------------------------------
// WallGroupData::intersects (WallGroupData.cu:28-71): entry point of a
// segment into an axis-aligned box, or false.
static bool enters_box(V3 start, V3 end, V3 lo, V3 hi, V3& ip) {
    const float si[3] = {start.x, start.y, start.z}, ei[3] = {end.x, end.y, end.z};
    const float bmin[3] = {lo.x, lo.y, lo.z}, bmax[3] = {hi.x, hi.y, hi.z};
    float fst = 0.f, fet = 1.f;
    for (int a = 0; a < 3; ++a) {
        float st, et;
        const float di = ei[a] - si[a];
        if (si[a] < ei[a]) {
            if (si[a] > bmax[a] || ei[a] < bmin[a]) return false;
            st = (si[a] < bmin[a]) ? (bmin[a] - si[a]) / di : 0.f;
            et = (ei[a] > bmax[a]) ? (bmax[a] - si[a]) / di : 1.f;
        } else {
            if (ei[a] > bmax[a] || si[a] < bmin[a]) return false;
            st = (si[a] > bmax[a]) ? (bmax[a] - si[a]) / di : 0.f;
            et = (ei[a] < bmin[a]) ? (bmin[a] - si[a]) / di : 1.f;
        }
        fst = st > fst ? st : fst;
        fet = et < fet ? et : fet;
        if (fet < fst) return false;
    }
    ip = add(start, mul(sub(end, start), fst));
    return true;
}

// WallGroupData::SplitWalls (WallGroupData.cu:108-206): every segment that
// enters a cell (in bin_cell order) at a point more than EPSILON from both
// ends is replaced by its two halves, appended to the list and split in turn.
// Cells that cannot intersect (outside the segment's bounding box grown by one
// cell) are skipped; the first intersecting cell in bin_cell order is
// unchanged by that.
static std::vector<Segment> split_walls(const std::vector<Segment>& in, const Grid& g) {
    const V3 step = v3(g.ws[0] / float(g.wc[0]), g.ws[1] / float(g.wc[1]), g.ws[2] / float(g.wc[2]));
    const float steps[3] = {step.x, step.y, step.z};
    auto cell_lo = [&](unsigned ix, unsigned iy, unsigned iz) {
        return v3(float(ix) * step.x - 0.5f * g.ws[0], float(iy) * step.y - 0.5f * g.ws[1],
                  float(iz) * step.z - 0.5f * g.ws[2]);
    };
    auto axis_range = [&](float a, float b, int axis, unsigned& i0, unsigned& i1) {
        const double lo = std::min(a, b), hi = std::max(a, b);
        const double half = 0.5 * double(g.ws[axis]);
        const double first = std::floor((lo + half) / steps[axis]) - 1.0;
        const double last = std::floor((hi + half) / steps[axis]) + 1.0;
        const double top = double(g.wc[axis]) - 1.0;
        if (last < 0.0 || first > top) return false;
        i0 = unsigned(first < 0.0 ? 0.0 : first);
        i1 = unsigned(last > top ? top : last);
        return true;
    };
    std::list<Segment> segs(in.begin(), in.end());
    const float eps = 0.001f;
    for (auto it = segs.begin(); it != segs.end();) {
        const V3 s = it->s, e = it->e;
        bool split = false;
        unsigned x0, x1, y0, y1, z0, z1;
        if (axis_range(s.x, e.x, 0, x0, x1) && axis_range(s.y, e.y, 1, y0, y1) &&
            axis_range(s.z, e.z, 2, z0, z1)) {
            for (unsigned iy = y0; iy <= y1 && !split; ++iy)
                for (unsigned iz = z0; iz <= z1 && !split; ++iz)
                    for (unsigned ix = x0; ix <= x1 && !split; ++ix) {
                        const V3 lo = cell_lo(ix, iy, iz);
                        V3 ip;
                        if (!enters_box(s, e, lo, add(lo, step), ip)) continue;
                        if (distance(s, ip) > eps && distance(ip, e) > eps) {
                            segs.push_back(Segment{s, add(s, mul(sub(ip, s), 0.5f)), ip, it->n});
                            segs.push_back(Segment{ip, add(ip, mul(sub(e, ip), 0.5f)), e, it->n});
                            split = true;
                        }
                    }
        }
        if (split) it = segs.erase(it);
        else ++it;
    }
    return std::vector<Segment>(segs.begin(), segs.end());
}

static gs_status make_walls(const std::vector<Segment>& raw, gs_bins bins, unsigned knw,
                            gs_walls* out) {
    if (!out) return fail(GS_ERR_INVALID_ARG, "null output handle");
    if (knw == 0 || knw > 8) return fail(GS_ERR_INVALID_ARG, "knw must be in 1..8");
    std::vector<Segment> segs = bins ? split_walls(raw, bins->grid) : raw;
    gs_walls w = new (std::nothrow) gs_walls_s();
    if (!w) return fail(GS_ERR_OOM, "host allocation failed");
    w->n = unsigned(segs.size());
    w->knw = knw;
    auto put = [](std::vector<float>& v, V3 a) {
        v.push_back(a.x);
        v.push_back(a.y);
        v.push_back(a.z);
        v.push_back(0.f);
    };
    for (const Segment& s : segs) {
        put(w->h_start, s.s);
        put(w->h_mid, s.m);
        put(w->h_end, s.e);
        put(w->h_normal, s.n);
    }
    gs_status st = GS_OK;
    if (w->n > 0) {
        st = dalloc(&w->start, w->n);
        if (st == GS_OK) st = dalloc(&w->mid, w->n);
        if (st == GS_OK) st = dalloc(&w->end, w->n);
        if (st == GS_OK) st = dalloc(&w->normal, w->n);
        if (st == GS_OK) {
            const size_t bytes = size_t(w->n) * sizeof(float4);
            cudaError_t e = cudaMemcpy(w->start, w->h_start.data(), bytes, cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMemcpy(w->mid, w->h_mid.data(), bytes, cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMemcpy(w->end, w->h_end.data(), bytes, cudaMemcpyHostToDevice);
            if (e == cudaSuccess)
                e = cudaMemcpy(w->normal, w->h_normal.data(), bytes, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) st = cuda_fail(e, "wall upload");
        }
    }
    if (st != GS_OK) {
        gs_walls_destroy(w);
        return st;
    }
    *out = w;
    return GS_OK;
}

static gs_status walls_db(gs_walls w, const Grid& grid, unsigned C, cudaStream_t stream) {
    const bool same = w->db.valid && w->db.cells == C &&
                      std::memcmp(&w->db.grid, &grid, sizeof(Grid)) == 0;
    if (same) return GS_OK;
    GS_TRY(db_reserve(w->db, w->n, C));
    GS_TRY(db_build(w->db, w->mid, w->n, grid, stream));
    // later users may run on other streams
    GS_CUDA(cudaStreamSynchronize(stream));
    return GS_OK;
}

// Candidate capacity of the fused KNN scan from the crowd's density.  The
// other agents in an agent's own cell, averaged over the agents, are
// lambda = sum c (c - 1) / n over the cell counts c (for a Poisson scatter of
// lambda agents per cell this is lambda itself; averaged over agents, not
// cells, so the dense scenes of a batch count by their agents), and an agent
// sees m = lambda * (2r+1)^d candidates on average.  32 (collecting scan)
// when m is at least four standard deviations below 32, else the streaming
// scan with 128 or 256 candidates.  Agents beyond the capacity take the
// exact redo path, so this only affects speed (a batch whose densest scenes
// passed 128 candidates per box ran 3.7 times slower on 128 than on 256).
static unsigned knn_capacity(unsigned n, unsigned long long sumsq, const Grid& g, unsigned r) {
    double box = 1.0;
    for (int a = 0; a < 3; ++a) box *= double(std::min<unsigned>(2 * r + 1, g.wc[a]));
    const double lambda = n ? (double(sumsq) - double(n)) / double(n) : 0.0;
    const double m = std::max(lambda, 0.0) * box;
    const double top = m + 4.0 * std::sqrt(m) + 1.0;
    if (top <= 32.0) return 32u;
    return top <= 128.0 ? 128u : 256u;
}

// Exact squared-distance forms of the flocking tests' d < m and d > m, for
// d = sqrtf(dsq) as the kernels round it (the host's float sqrt is the same
// IEEE operation): d < m <=> dsq < lt and d > m <=> dsq > gt.  The square
// root is monotone on the non-negative floats, so bisection over their bit
// patterns (0 .. +inf, in value order) finds the smallest dsq whose root
// reaches m and the largest whose root stays at or below m.  Squared
// distances are never negative; NaN compares false on both sides, as its
// root does.
static float sqrt_reaches(float m) {  // lt: smallest x >= 0 with sqrt(x) >= m
    if (!(m > 0.f)) return 0.f;        // m <= 0 or NaN: d < m never holds
    uint32_t lo = 0, hi = 0x7f800000u;  // sqrt(+inf) = +inf >= m
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        float x;
        std::memcpy(&x, &mid, 4);
        if (std::sqrt(x) >= m) hi = mid;
        else lo = mid + 1;
    }
    float r;
    std::memcpy(&r, &lo, 4);
    return r;
}
static float sqrt_stays(float m) {  // gt: largest x >= 0 with sqrt(x) <= m
    if (std::isnan(m)) return std::numeric_limits<float>::infinity();  // d > NaN never holds
    if (m < 0.f) return -1.f;  // every d >= 0 is above m
    uint32_t lo = 0, hi = 0x7f800000u;  // sqrt(0) = 0 <= m
    while (lo < hi) {
        const uint32_t mid = hi - (hi - lo) / 2;
        float x;
        std::memcpy(&x, &mid, 4);
        if (std::sqrt(x) <= m) lo = mid;
        else hi = mid - 1;
    }
    float r;
    std::memcpy(&r, &lo, 4);
    return r;
}

static gs_status validate_step(const gs_step_params* p, gs_walls walls, StepDev& d) {
    if (!p) return fail(GS_ERR_INVALID_ARG, "null step parameters");
    if (p->knn_mode != GS_KNN_BINNED)
        return fail(GS_ERR_UNSUPPORTED, "the fused step uses binned KNN");
    if (p->k == 0 || p->k > 32) return fail(GS_ERR_INVALID_ARG, "fused step needs 1 <= k <= 32");
    if (p->wrap_mode < 0 || p->wrap_mode > 2) return fail(GS_ERR_INVALID_ARG, "bad wrap mode");
    if (p->n_order > 8) return fail(GS_ERR_INVALID_ARG, "at most 8 behaviours");
    if (!std::isfinite(p->dt)) return fail(GS_ERR_NONFINITE, "dt is not finite");
    std::memset(&d, 0, sizeof(d));
    d.k = p->k;
    d.flat = p->world_cells[1] == 1 ? 1u : 0u;
    d.scan_reach = scan_reach_tiles(p->world_cells, p->search_radius);
    d.knw = p->knw;
    d.r = p->search_radius;
    d.wrap_mode = p->wrap_mode;
    d.clear_applied = p->clear_applied;
    auto fl = [](float* out, float a, float b, float c, float w, unsigned m) {
        out[0] = a;
        out[1] = b;
        out[2] = c;
        out[3] = w;
        std::memcpy(&out[4], &m, 4);
    };
    fl(d.sep, p->sep_min, p->sep_max, p->sep_cos, p->w_sep, p->mask_sep);
    fl(d.ali, p->ali_min, p->ali_max, p->ali_cos, p->w_ali, p->mask_ali);
    fl(d.coh, p->coh_min, p->coh_max, p->coh_cos, p->w_coh, p->mask_coh);
    d.sep_dsq[0] = sqrt_reaches(p->sep_min);
    d.sep_dsq[1] = sqrt_stays(p->sep_max);
    d.ali_dsq[0] = sqrt_reaches(p->ali_min);
    d.ali_dsq[1] = sqrt_stays(p->ali_max);
    d.coh_dsq[0] = sqrt_reaches(p->coh_min);
    d.coh_dsq[1] = sqrt_stays(p->coh_max);
    std::memcpy(d.seek_target, p->seek_target, sizeof(d.seek_target));
    d.w_seek = p->w_seek;
    d.mask_seek = p->mask_seek;
    d.min_time_wall = p->min_time_to_wall;
    d.w_walls = p->w_walls;
    d.mask_walls = p->mask_walls;
    d.min_time_col = p->min_time_to_collision;
    d.min_sep = p->min_separation_distance;
    d.avoid_close = p->avoid_close;
    d.w_avoid = p->w_avoid;
    d.mask_avoid = p->mask_avoid;
    d.n_order = p->n_order;
    d.dt = p->dt;
    for (unsigned o = 0; o < p->n_order; ++o) {
        const unsigned b = p->order[o];
        d.order[o] = b;
        d.order_packed |= (b & 7u) << (3u * o);
        switch (b) {
            case GS_B_AVOID_WALLS:
                if (o != 0)
                    return fail(GS_ERR_UNSUPPORTED, "the fused step needs avoid-walls first");
                d.need |= NEED_WALLS;
                break;
            case GS_B_AVOID_NEIGHBORS:
                d.need |= NEED_AVOID | (p->avoid_close ? NEED_CLOSE : 0u);
                break;
            case GS_B_SEPARATION: d.need |= NEED_SEP; break;
            case GS_B_ALIGNMENT: d.need |= NEED_ALI; break;
            case GS_B_COHESION: d.need |= NEED_COH; break;
            case GS_B_SEEK: break;
            case GS_B_FOLLOW_PATH: {
                const gs_path P = p->path;
                if (!P || P->n < 2)
                    return fail(GS_ERR_INVALID_ARG, "follow-path needs a path of 2+ points");
                d.path = PathDev{P->d_points, P->d_lengths, P->d_normals, P->n, P->radius,
                                 P->cyclic, P->total};
                d.path_time = p->path_prediction_time;
                d.w_path = p->w_path;
                d.mask_path = p->mask_path;
                break;
            }
            default: return fail(GS_ERR_INVALID_ARG, "unknown behaviour code");
        }
    }
    if ((d.need & NEED_WALLS) && (p->knw == 0 || p->knw > 8))
        return fail(GS_ERR_INVALID_ARG, "knw must be in 1..8");
    (void)walls;
    return GS_OK;
}

// Records a (start, stop) event pair per phase launch on the group's stream
// and folds finished pairs into the group's totals.
struct Profiler final : PhaseHook {
    gs_group g;
    explicit Profiler(gs_group grp) : g(grp) {}
    void mark(int phase, bool begin) override {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return;
        cudaEventRecord(e, g->stream);
        g->prof_events->push_back(e);
        if (begin) g->prof_phase->push_back(phase);
    }
};

static void prof_collect(gs_group g) {
    if (!g->prof_events) return;
    auto& ev = *g->prof_events;
    auto& ph = *g->prof_phase;
    if (!ev.empty()) cudaEventSynchronize(ev.back());
    for (size_t i = 0; i + 1 < ev.size() && i / 2 < ph.size(); i += 2) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, ev[i], ev[i + 1]) == cudaSuccess) {
            g->prof_ms[ph[i / 2]] += ms;
            g->prof_launches[ph[i / 2]] += 1;
        }
    }
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    ev.clear();
    ph.clear();
}

}  // namespace gs

using namespace gs;

extern "C" {

const char* gs_status_string(gs_status s) {
    switch (s) {
        case GS_OK: return "ok";
        case GS_ERR_INVALID_ARG: return "invalid argument";
        case GS_ERR_OOM: return "out of memory";
        case GS_ERR_CUDA: return "CUDA error";
        case GS_ERR_TIMEOUT: return "timeout";
        case GS_ERR_NONFINITE: return "non-finite value";
        case GS_ERR_STATE: return "invalid state";
        case GS_ERR_UNSUPPORTED: return "unsupported";
        default: return "unknown status";
    }
}

const char* gs_last_error(void) { return g_last_error.c_str(); }

gs_status gs_set_device(int device) {
    GS_CUDA(cudaSetDevice(device));
    return GS_OK;
}

gs_status gs_host_alloc(size_t bytes, void** out) {
    if (!out) return fail(GS_ERR_INVALID_ARG, "null output");
    *out = nullptr;
    if (bytes == 0) return GS_OK;
    cudaError_t e = cudaMallocHost(out, bytes);
    if (e == cudaErrorMemoryAllocation) return fail(GS_ERR_OOM, "pinned allocation failed");
    GS_CUDA(e);
    return GS_OK;
}

gs_status gs_host_free(void* p) {
    if (p) GS_CUDA(cudaFreeHost(p));
    return GS_OK;
}

gs_status gs_group_set_profiling(gs_group g, int enable) {
    if (!g) return fail(GS_ERR_INVALID_ARG, "null group");
    if (!g->prof_events) {
        g->prof_events = new std::vector<cudaEvent_t>();
        g->prof_phase = new std::vector<int>();
    }
    prof_collect(g);
    g->profiling = enable != 0;
    for (int i = 0; i < 4; ++i) {
        g->prof_ms[i] = 0.f;
        g->prof_launches[i] = 0;
    }
    return GS_OK;
}

gs_status gs_group_exact_redos(gs_group g, unsigned* count) {
    if (!g || !count) return fail(GS_ERR_INVALID_ARG, "null argument");
    *count = 0;
    if (!g->retry_count) return GS_OK;
    GS_CUDA(cudaMemcpyAsync(count, g->retry_count, sizeof(unsigned), cudaMemcpyDeviceToHost,
                            g->stream));
    GS_CUDA(cudaStreamSynchronize(g->stream));
    return GS_OK;
}

gs_status gs_group_phase_times(gs_group g, float* ms, unsigned* launches, unsigned cap) {
    if (!g) return fail(GS_ERR_INVALID_ARG, "null group");
    prof_collect(g);
    for (unsigned i = 0; i < cap && i < 4; ++i) {
        if (ms) ms[i] = g->prof_ms[i];
        if (launches) launches[i] = g->prof_launches[i];
    }
    return GS_OK;
}
int gs_version(void) { return 1; }
unsigned gs_max_k(void) { return kMaxK; }

// ---- bins -----------------------------------------------------------------------
gs_status gs_bins_create(const unsigned world_cells[3], const float world_size[3],
                         unsigned search_radius, gs_bins* out) {
    if (!out || !world_cells || !world_size) return fail(GS_ERR_INVALID_ARG, "null argument");
    Grid g;
    unsigned cells;
    GS_TRY(check_grid(world_cells, world_size, g, cells));
    gs_bins b = new (std::nothrow) gs_bins_s();
    if (!b) return fail(GS_ERR_OOM, "host allocation failed");
    b->grid = g;
    b->radius = search_radius;
    b->cells = cells;
    *out = b;
    return GS_OK;
}

gs_status gs_bins_destroy(gs_bins bins) {
    delete bins;
    return GS_OK;
}

gs_status gs_bins_num_cells(gs_bins bins, unsigned* out) {
    if (!bins || !out) return fail(GS_ERR_INVALID_ARG, "null argument");
    *out = bins->cells;
    return GS_OK;
}

gs_status gs_bins_get_cells(gs_bins bins, float* min3, float* max3, float* centre3, unsigned cap) {
    if (!bins) return fail(GS_ERR_INVALID_ARG, "null bins");
    if (cap < bins->cells) return fail(GS_ERR_INVALID_ARG, "output too small");
    const Grid& g = bins->grid;
    const float sx = g.ws[0] / float(g.wc[0]), sy = g.ws[1] / float(g.wc[1]),
                sz = g.ws[2] / float(g.wc[2]);
    unsigned i = 0;
    for (unsigned iy = 0; iy < g.wc[1]; ++iy)
        for (unsigned iz = 0; iz < g.wc[2]; ++iz)
            for (unsigned ix = 0; ix < g.wc[0]; ++ix, ++i) {
                const float lo[3] = {float(ix) * sx - 0.5f * g.ws[0], float(iy) * sy - 0.5f * g.ws[1],
                                     float(iz) * sz - 0.5f * g.ws[2]};
                const float st[3] = {sx, sy, sz};
                for (int a = 0; a < 3; ++a) {
                    if (min3) min3[3 * i + a] = lo[a];
                    if (max3) max3[3 * i + a] = lo[a] + st[a];
                    if (centre3) centre3[3 * i + a] = lo[a] + 0.5f * st[a];
                }
            }
    return GS_OK;
}

// ---- groups -----------------------------------------------------------------------
gs_status gs_group_destroy(gs_group g) {
    if (!g) return GS_OK;
    if (g->stream) cudaStreamSynchronize(g->stream);
    // the reference-layout arrays live in three blocks (see gs_group_create)
    dfree(g->position);
    dfree(g->side);
    dfree(g->speed);
    db_release(g->db);
    db_release(g->bf_a);
    db_release(g->bf_b);
    dfree(g->bf_tmp);
    dfree(g->bf_boxes);
    if (g->diag) cudaFree(g->diag);
    if (g->ap) cudaFree(g->ap);
    if (g->read_ev) cudaEventDestroy(g->read_ev);
    release_fused(g);
    if (g->prof_events) {
        prof_collect(g);
        delete g->prof_events;
        delete g->prof_phase;
    }
    drop_graph(g);
    delete g->h_scenes;
    if (g->own_stream && g->stream) cudaStreamDestroy(g->stream);
    delete g;
    return GS_OK;
}

gs_status gs_group_create(unsigned k, unsigned capacity, void* stream, gs_group* out) {
    if (!out) return fail(GS_ERR_INVALID_ARG, "null output handle");
    if (k == 0 || k > kMaxK) return fail(GS_ERR_INVALID_ARG, "k must be in 1..64");
    if (capacity == 0 || capacity > (1u << 30)) return fail(GS_ERR_INVALID_ARG, "bad capacity");
    gs_group g = new (std::nothrow) gs_group_s();
    if (!g) return fail(GS_ERR_OOM, "host allocation failed");
    std::memset(static_cast<void*>(g), 0, sizeof(*g));
    new (&g->db) Database();
    new (&g->fdb) Database();
    g->use_graph = true;
    g->block = kBlock;
    g->k = k;
    g->capacity = capacity;
    gs_status s = GS_OK;
    if (stream) {
        g->stream = static_cast<cudaStream_t>(stream);
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) s = cuda_fail(e, "cudaStreamCreate");
        g->own_stream = true;
    }
    // The reference-layout arrays, one block per element size: position,
    // direction, steering (float4); side, up (float3); speed, maxSpeed,
    // maxForce, radius, mass, applied (4 bytes).  Arrays of one block sit at a
    // fixed stride, so a host state laid out the same way moves in one pitched
    // copy per block (copy_arrays).
    const size_t n = capacity;
    if (s == GS_OK) s = dalloc(&g->position, 3 * n);
    if (s == GS_OK) s = dalloc(&g->side, 2 * n);
    if (s == GS_OK) s = dalloc(&g->speed, 6 * n);
    if (s == GS_OK) {
        g->direction = g->position + n;
        g->steering = g->position + 2 * n;
        g->up = g->side + n;
        g->max_speed = g->speed + n;
        g->max_force = g->speed + 2 * n;
        g->radius = g->speed + 3 * n;
        g->mass = g->speed + 4 * n;
        g->applied = reinterpret_cast<unsigned*>(g->speed + 5 * n);
    }
    if (s != GS_OK) {
        const std::string msg = g_last_error;
        gs_group_destroy(g);
        set_error(msg);
        return s;
    }
    *out = g;
    return GS_OK;
}

// Copies n elements of `count` arrays (elem bytes each) from src[i] to dst[i]:
// one pitched copy when both sides hold the arrays at one fixed, increasing
// stride (then the copy engine pays its fixed cost once, not per array), else
// one copy per array.
static cudaError_t copy_arrays(void* const* dst, const void* const* src, int count, size_t elem,
                               unsigned n, cudaMemcpyKind kind, cudaStream_t st) {
    const size_t width = size_t(n) * elem;
    if (width == 0) return cudaSuccess;
    static int max_pitch = -1;
    if (max_pitch < 0) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&v, cudaDevAttrMaxPitch, dev) != cudaSuccess) {
            cudaGetLastError();
            v = 0;
        }
        max_pitch = v;
    }
    if (count > 1) {
        auto gap = [](const void* a, const void* b) {
            return static_cast<const char*>(b) - static_cast<const char*>(a);
        };
        const ptrdiff_t dp = gap(dst[0], dst[1]), sp = gap(src[0], src[1]);
        bool ok = dp >= ptrdiff_t(width) && sp >= ptrdiff_t(width) && dp <= max_pitch &&
                  sp <= max_pitch;
        for (int i = 2; i < count && ok; ++i)
            ok = gap(dst[i - 1], dst[i]) == dp && gap(src[i - 1], src[i]) == sp;
        if (ok)
            return cudaMemcpy2DAsync(dst[0], size_t(dp), src[0], size_t(sp), width, size_t(count),
                                     kind, st);
    }
    for (int i = 0; i < count; ++i) {
        const cudaError_t e = cudaMemcpyAsync(dst[i], src[i], width, kind, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

static gs_status upload_enqueue(gs_group g, const gs_agent_arrays* h, unsigned n);

gs_status gs_group_upload(gs_group g, const gs_agent_arrays* h, unsigned n) {
    if (!g || !h) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (n > g->capacity) return fail(GS_ERR_INVALID_ARG, "more agents than the group's capacity");
    if (!h->position || !h->direction || !h->steering || !h->side || !h->up || !h->speed ||
        !h->max_speed || !h->max_force || !h->radius || !h->mass || !h->applied)
        return fail(GS_ERR_INVALID_ARG, "upload needs every array");
    GS_TRY(upload_enqueue(g, h, n));
    // the automatic KNN capacity is measured again (a synchronising read)
    // only when the agent count changes: stepping host state in a loop keeps
    // its choice, which never changes results
    if (n != g->n) g->auto_cap_valid = false;
    g->n = n;
    g->db.valid = false;
    touched(g);
    return GS_OK;
}

// Queues the copies of gs_group_upload on the group's stream.
static gs_status upload_enqueue(gs_group g, const gs_agent_arrays* h, unsigned n) {
    cudaStream_t st = g->stream;
    void* d4[] = {g->position, g->direction, g->steering};
    const void* h4[] = {h->position, h->direction, h->steering};
    void* d3[] = {g->side, g->up};
    const void* h3[] = {h->side, h->up};
    void* d1[] = {g->speed, g->max_speed, g->max_force, g->radius, g->mass, g->applied};
    const void* h1[] = {h->speed, h->max_speed, h->max_force, h->radius, h->mass, h->applied};
    cudaError_t e = copy_arrays(d4, h4, 3, 16, n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = copy_arrays(d3, h3, 2, 12, n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = copy_arrays(d1, h1, 6, 4, n, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "upload");
    return GS_OK;
}

static gs_status check_device_flags(gs_group g);

// Queues the copies of gs_group_download on the group's stream.  With
// skip_constants the per-agent constants (maxSpeed, maxForce, radius, mass),
// which no step changes, are not copied.
static gs_status download_copies(gs_group g, const gs_agent_arrays* h, bool skip_constants);
static gs_status download_enqueue(gs_group g, const gs_agent_arrays* h,
                                  bool skip_constants = false) {
    GS_TRY(ensure_reference(g));
    return download_copies(g, h, skip_constants);
}

// The device-to-host copies of the reference-layout arrays (a NULL host
// array is left out).
static gs_status download_copies(gs_group g, const gs_agent_arrays* h, bool skip_constants) {
    cudaStream_t st = g->stream;
    const unsigned n = g->n;
    const bool all4 = h->position && h->direction && h->steering, all3 = h->side && h->up;
    const bool all1 = h->speed && h->max_speed && h->max_force && h->radius && h->mass && h->applied;
    cudaError_t e = cudaSuccess;
    auto cp = [&](void* dst, const void* src, size_t elem) {
        if (e == cudaSuccess && dst && n)
            e = cudaMemcpyAsync(dst, src, size_t(n) * elem, cudaMemcpyDeviceToHost, st);
    };
    if (all4) {
        void* h4[] = {h->position, h->direction, h->steering};
        const void* d4[] = {g->position, g->direction, g->steering};
        e = copy_arrays(h4, d4, 3, 16, n, cudaMemcpyDeviceToHost, st);
    } else {
        cp(h->position, g->position, 16);
        cp(h->direction, g->direction, 16);
        cp(h->steering, g->steering, 16);
    }
    if (all3) {
        void* h3[] = {h->side, h->up};
        const void* d3[] = {g->side, g->up};
        if (e == cudaSuccess) e = copy_arrays(h3, d3, 2, 12, n, cudaMemcpyDeviceToHost, st);
    } else {
        cp(h->side, g->side, 12);
        cp(h->up, g->up, 12);
    }
    if (all1 && !skip_constants) {
        void* h1[] = {h->speed, h->max_speed, h->max_force, h->radius, h->mass, h->applied};
        const void* d1[] = {g->speed, g->max_speed, g->max_force, g->radius, g->mass, g->applied};
        if (e == cudaSuccess) e = copy_arrays(h1, d1, 6, 4, n, cudaMemcpyDeviceToHost, st);
    } else {
        cp(h->speed, g->speed, 4);
        if (!skip_constants) {
            cp(h->max_speed, g->max_speed, 4);
            cp(h->max_force, g->max_force, 4);
            cp(h->radius, g->radius, 4);
            cp(h->mass, g->mass, 4);
        }
        cp(h->applied, g->applied, 4);
    }
    if (e != cudaSuccess) return cuda_fail(e, "download");
    return GS_OK;
}

gs_status gs_group_download(gs_group g, const gs_agent_arrays* h) {
    if (!g || !h) return fail(GS_ERR_INVALID_ARG, "null argument");
    GS_TRY(download_enqueue(g, h));
    GS_CUDA(cudaStreamSynchronize(g->stream));
    return check_device_flags(g);
}

gs_status gs_group_size(gs_group g, unsigned* n) {
    if (!g || !n) return fail(GS_ERR_INVALID_ARG, "null argument");
    *n = g->n;
    return GS_OK;
}

gs_status gs_group_device_arrays(gs_group g, gs_agent_arrays* d) {
    if (!g || !d) return fail(GS_ERR_INVALID_ARG, "null argument");
    GS_TRY(ensure_reference(g));
    d->position = reinterpret_cast<float*>(g->position);
    d->direction = reinterpret_cast<float*>(g->direction);
    d->steering = reinterpret_cast<float*>(g->steering);
    d->side = reinterpret_cast<float*>(g->side);
    d->up = reinterpret_cast<float*>(g->up);
    d->speed = g->speed;
    d->max_speed = g->max_speed;
    d->max_force = g->max_force;
    d->radius = g->radius;
    d->mass = g->mass;
    d->applied = g->applied;
    // The caller may write through these pointers.  The KNN database keeps
    // the positions of its last update (the binned search reads only its own
    // sorted copies), as the reference's does: a plugin may fetch the
    // pointers between updateKNNDatabase and findKNearestNeighbors.
    touched(g);
    return GS_OK;
}

gs_status gs_group_stream(gs_group g, void** stream) {
    if (!g || !stream) return fail(GS_ERR_INVALID_ARG, "null argument");
    *stream = g->stream;
    return GS_OK;
}

// Reads and clears the device error flags of the fused step.
static gs_status check_device_flags(gs_group g) {
    if (!g->d_err) return GS_OK;
    unsigned flags = 0;
    GS_CUDA(cudaMemcpyAsync(&flags, g->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost,
                            g->stream));
    GS_CUDA(cudaStreamSynchronize(g->stream));
    if (flags) {
        GS_CUDA(cudaMemsetAsync(g->d_err, 0, sizeof(unsigned), g->stream));
        if (flags & kErrBarrierTimeout)
            return fail(GS_ERR_TIMEOUT,
                        "persistent step: a grid barrier wait ran out (state void; upload again)");
        return fail(GS_ERR_STATE, "fused step: inconsistent cell counts (state not updated)");
    }
    return GS_OK;
}

gs_status gs_group_synchronize(gs_group g) {
    if (!g) return fail(GS_ERR_INVALID_ARG, "null group");
    GS_CUDA(cudaStreamSynchronize(g->stream));
    return check_device_flags(g);
}

// ---- KNN data -----------------------------------------------------------------------
gs_status gs_knn_create(unsigned n, unsigned k, gs_knn* out) {
    if (!out) return fail(GS_ERR_INVALID_ARG, "null output handle");
    if (k == 0 || k > kMaxK) return fail(GS_ERR_INVALID_ARG, "k must be in 1..64");
    gs_knn kd = new (std::nothrow) gs_knn_s();
    if (!kd) return fail(GS_ERR_OOM, "host allocation failed");
    kd->n = n;
    kd->k = k;
    kd->idx = nullptr;
    kd->dist = nullptr;
    gs_status s = dalloc(&kd->idx, size_t(n) * k);
    if (s == GS_OK) s = dalloc(&kd->dist, size_t(n) * k);
    if (s != GS_OK) {
        gs_knn_destroy(kd);
        return s;
    }
    *out = kd;
    return GS_OK;
}

gs_status gs_knn_destroy(gs_knn kd) {
    if (!kd) return GS_OK;
    dfree(kd->idx);
    dfree(kd->dist);
    delete kd;
    return GS_OK;
}

gs_status gs_knn_download(gs_knn kd, gs_group g, unsigned* idx, float* dist) {
    if (!kd) return fail(GS_ERR_INVALID_ARG, "null knn");
    cudaStream_t st = g ? g->stream : nullptr;
    const size_t cnt = size_t(kd->n) * kd->k;
    if (idx) GS_CUDA(cudaMemcpyAsync(idx, kd->idx, cnt * 4, cudaMemcpyDeviceToHost, st));
    if (dist) GS_CUDA(cudaMemcpyAsync(dist, kd->dist, cnt * 4, cudaMemcpyDeviceToHost, st));
    GS_CUDA(cudaStreamSynchronize(st));
    return GS_OK;
}

gs_status gs_knn_upload(gs_knn kd, gs_group g, const unsigned* idx, const float* dist) {
    if (!kd) return fail(GS_ERR_INVALID_ARG, "null knn");
    cudaStream_t st = g ? g->stream : nullptr;
    const size_t cnt = size_t(kd->n) * kd->k;
    if (idx) GS_CUDA(cudaMemcpyAsync(kd->idx, idx, cnt * 4, cudaMemcpyHostToDevice, st));
    if (dist) GS_CUDA(cudaMemcpyAsync(kd->dist, dist, cnt * 4, cudaMemcpyHostToDevice, st));
    GS_CUDA(cudaStreamSynchronize(st));
    return GS_OK;
}

gs_status gs_knn_device_arrays(gs_knn kd, unsigned** idx, float** dist) {
    if (!kd) return fail(GS_ERR_INVALID_ARG, "null knn");
    if (idx) *idx = kd->idx;
    if (dist) *dist = kd->dist;
    return GS_OK;
}

// ---- walls -----------------------------------------------------------------------
gs_status gs_walls_create(const float* start4, const float* end4, const float* normal4,
                          unsigned n, gs_bins bins, unsigned knw, gs_walls* out) {
    if (n > 0 && (!start4 || !end4 || !normal4)) return fail(GS_ERR_INVALID_ARG, "null arrays");
    std::vector<Segment> raw(n);
    for (unsigned i = 0; i < n; ++i) {
        raw[i].s = v3(start4[4 * i], start4[4 * i + 1], start4[4 * i + 2]);
        raw[i].e = v3(end4[4 * i], end4[4 * i + 1], end4[4 * i + 2]);
        raw[i].n = v3(normal4[4 * i], normal4[4 * i + 1], normal4[4 * i + 2]);
        // WallGroupData.cu:87-89
        raw[i].m = v3(0.5f * (raw[i].s.x + raw[i].e.x), 0.5f * (raw[i].s.y + raw[i].e.y),
                      0.5f * (raw[i].s.z + raw[i].e.z));
    }
    return make_walls(raw, bins, knw, out);
}

gs_status gs_walls_load(const char* path, gs_bins bins, unsigned knw, gs_walls* out) {
    if (!path) return fail(GS_ERR_INVALID_ARG, "null path");
    std::ifstream in(path);
    if (!in.is_open()) return fail(GS_ERR_INVALID_ARG, std::string("cannot open ") + path);
    std::vector<float> s4, e4, n4;
    for (;;) {
        float v[9];
        for (float& x : v) in >> x;
        if (!in.good()) break;
        s4.insert(s4.end(), {v[0], v[1], v[2], 0.f});
        e4.insert(e4.end(), {v[3], v[4], v[5], 0.f});
        n4.insert(n4.end(), {v[6], v[7], v[8], 0.f});
    }
    return gs_walls_create(s4.data(), e4.data(), n4.data(), unsigned(s4.size() / 4), bins, knw,
                           out);
}

gs_status gs_walls_destroy(gs_walls w) {
    if (!w) return GS_OK;
    dfree(w->start);
    dfree(w->mid);
    dfree(w->end);
    dfree(w->normal);
    db_release(w->db);
    delete w;
    return GS_OK;
}

gs_status gs_walls_size(gs_walls w, unsigned* n) {
    if (!w || !n) return fail(GS_ERR_INVALID_ARG, "null argument");
    *n = w->n;
    return GS_OK;
}

gs_status gs_walls_download(gs_walls w, float* start4, float* mid4, float* end4, float* normal4,
                            unsigned cap) {
    if (!w) return fail(GS_ERR_INVALID_ARG, "null walls");
    if (cap < w->n) return fail(GS_ERR_INVALID_ARG, "output too small");
    const size_t bytes = size_t(w->n) * 4 * sizeof(float);
    if (start4) std::memcpy(start4, w->h_start.data(), bytes);
    if (mid4) std::memcpy(mid4, w->h_mid.data(), bytes);
    if (end4) std::memcpy(end4, w->h_end.data(), bytes);
    if (normal4) std::memcpy(normal4, w->h_normal.data(), bytes);
    return GS_OK;
}

// ---- GroupSteerLibrary ------------------------------------------------------------
gs_status gs_wrap_world(gs_group g, const float world_size[3], int mode) {
    if (!g || !world_size) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (mode < 0 || mode > 2) return fail(GS_ERR_INVALID_ARG, "bad wrap mode");
    GS_TRY(ensure_reference(g));
    GS_TRY(launch_wrap(g->position, g->n, world_size, mode, g->stream));
    touched(g);
    return GS_OK;
}

gs_status gs_update_knn_database(gs_group g, gs_bins bins) {
    if (!g || !bins) return fail(GS_ERR_INVALID_ARG, "null argument");
    GS_TRY(ensure_reference(g));
    GS_TRY(db_reserve(g->db, g->capacity, bins->cells));
    GS_TRY(db_build(g->db, g->position, g->n, bins->grid, g->stream));
    return GS_OK;
}

gs_status gs_walls_update_knn_database(gs_walls w, gs_bins bins) {
    if (!w || !bins) return fail(GS_ERR_INVALID_ARG, "null argument");
    return walls_db(w, bins->grid, bins->cells, nullptr);
}

gs_status gs_find_knn(gs_group g, gs_knn out, gs_bins bins, gs_group other,
                      unsigned search_radius) {
    (void)search_radius;  // the bins' radius applies, as in KNNBinningV2.cu:210-243
    if (!g || !out || !bins || !other) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (out->n != g->n) return fail(GS_ERR_INVALID_ARG, "KNNData size differs from the group");
    if (!g->db.valid || !other->db.valid || g->db.cells != bins->cells ||
        other->db.cells != bins->cells)
        return fail(GS_ERR_STATE, "call gs_update_knn_database on both groups first");
    if (other != g) GS_CUDA(cudaStreamSynchronize(other->stream));
    GS_TRY(launch_knn_binned(g->db, g->n, other->db, other == g, bins->radius, out->k, out->idx,
                             out->dist, g->stream));
    return read_done(g, other);
}

// The pair table of a batched KNN over groups (out[i * n + j], NULL skips).
static gs_status knn_pairs(const gs_group* groups, unsigned n_groups, gs_bins bins,
                           gs_knn* out, KnnPairs& P) {
    std::memset(&P, 0, sizeof(P));
    P.grid = bins->grid;
    P.r = bins->radius;
    for (unsigned i = 0; i < n_groups; ++i)
        for (unsigned j = 0; j < n_groups; ++j) {
            gs_knn o = out[size_t(i) * n_groups + j];
            if (!o) continue;
            gs_group a = groups[i], b = groups[j];
            if (o->n != a->n) return fail(GS_ERR_INVALID_ARG, "KNNData size differs from its group");
            KnnPair& q = P.pair[P.n_pairs++];
            q.a_sorted = a->db.sorted;
            q.a_pos_id = a->db.pos_id;
            q.b_start = b->db.start;
            q.b_pos_id = b->db.pos_id;
            q.idx = o->idx;
            q.dist = o->dist;
            q.nA = a->n;
            q.k = o->k;
            q.self = a == b;
        }
    return GS_OK;
}

gs_status gs_find_knn_groups(const gs_group* groups, unsigned n_groups, gs_bins bins,
                             gs_knn* out) {
    if (!groups || !bins || !out || n_groups == 0) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (size_t(n_groups) * n_groups > kMaxKnnPairs)
        return fail(GS_ERR_INVALID_ARG, "at most 7 groups (49 pairs) per batched KNN");
    for (unsigned i = 0; i < n_groups; ++i) {
        gs_group g = groups[i];
        if (!g) return fail(GS_ERR_INVALID_ARG, "null group");
        if (!g->db.valid || g->db.cells != bins->cells)
            return fail(GS_ERR_STATE, "call gs_update_knn_database on every group first");
    }
    KnnPairs P;
    GS_TRY(knn_pairs(groups, n_groups, bins, out, P));
    if (P.n_pairs == 0) return GS_OK;
    // One launch on the first group's stream, after every group's database
    // build; every group's stream then waits for it.
    cudaStream_t st = groups[0]->stream;
    for (unsigned i = 1; i < n_groups; ++i)
        if (groups[i]->stream != st) GS_CUDA(cudaStreamSynchronize(groups[i]->stream));
    GS_TRY(launch_knn_binned_pairs(P, st));
    cudaEvent_t done = nullptr;
    for (unsigned i = 1; i < n_groups; ++i) {
        if (groups[i]->stream == st) continue;
        if (!done) {
            GS_CUDA(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
            const cudaError_t e = cudaEventRecord(done, st);
            if (e != cudaSuccess) {
                cudaEventDestroy(done);
                return cuda_fail(e, "cudaEventRecord");
            }
        }
        const cudaError_t e = cudaStreamWaitEvent(groups[i]->stream, done, 0);
        if (e != cudaSuccess) {
            cudaEventDestroy(done);
            return cuda_fail(e, "cudaStreamWaitEvent");
        }
    }
    if (done) cudaEventDestroy(done);
    return GS_OK;
}

static gs_status antipen_enqueue(gs_group g, gs_knn knn, gs_group other, unsigned mask,
                                 cudaStream_t st);

gs_status gs_multigroup_step(const gs_group* groups, unsigned n_groups, gs_bins bins,
                             const gs_path* paths, gs_knn* knn, const gs_multigroup_params* p,
                             unsigned steps) {
    if (!groups || !bins || !knn || !p || n_groups == 0)
        return fail(GS_ERR_INVALID_ARG, "null argument");
    if (n_groups > kMaxGroups) return fail(GS_ERR_INVALID_ARG, "at most 7 groups");
    if (p->wrap_mode < 0 || p->wrap_mode > 2) return fail(GS_ERR_INVALID_ARG, "bad wrap mode");
    if (!finite3(p->world_size) || !std::isfinite(p->dt))
        return fail(GS_ERR_NONFINITE, "non-finite parameter");
    const unsigned G = n_groups;
    for (unsigned i = 0; i < G; ++i) {
        if (!groups[i]) return fail(GS_ERR_INVALID_ARG, "null group");
        for (unsigned j = 0; j < i; ++j)
            if (groups[j] == groups[i]) return fail(GS_ERR_INVALID_ARG, "a group appears twice");
        for (unsigned j = 0; j < G; ++j) {
            gs_knn o = knn[size_t(i) * G + j];
            if (!o) return fail(GS_ERR_INVALID_ARG, "every group pair needs its KNNData");
            if (o->n != groups[i]->n)
                return fail(GS_ERR_INVALID_ARG, "KNNData size differs from its group");
        }
        if (paths && paths[i] && paths[i]->n < 2)
            return fail(GS_ERR_INVALID_ARG, "follow-path needs a path of 2+ points");
    }
    // Everything runs on the first group's stream, after the other groups'
    // pending work; their streams wait for it at the end.
    cudaStream_t st = groups[0]->stream;
    for (unsigned i = 0; i < G; ++i) {
        GS_TRY(ensure_reference(groups[i]));
        if (groups[i]->stream != st) GS_CUDA(cudaStreamSynchronize(groups[i]->stream));
        GS_TRY(db_reserve(groups[i]->db, groups[i]->capacity, bins->cells));
    }
    for (unsigned step = 0; step < steps; ++step) {
        // Group::preUpdate for every group (MultiGroup.cpp:545-556)
        for (unsigned i = 0; i < G; ++i) {
            gs_group g = groups[i];
            GS_TRY(launch_wrap(g->position, g->n, p->world_size, p->wrap_mode, st));
            GS_TRY(db_build(g->db, g->position, g->n, bins->grid, st));
            if (g->n) GS_CUDA(cudaMemsetAsync(g->applied, 0, size_t(g->n) * 4, st));
        }
        // every pair's KNN reads only those databases: one launch (:561-564)
        KnnPairs P;
        GS_TRY(knn_pairs(groups, G, bins, knn, P));
        if (P.n_pairs) GS_TRY(launch_knn_binned_pairs(P, st));
        // Group::update of each group in turn (:558-610)
        for (unsigned i = 0; i < G; ++i) {
            gs_group g = groups[i];
            MultiSteer M;
            std::memset(static_cast<void*>(&M), 0, sizeof(M));
            M.g = view(g);
            for (unsigned j = 0; j < G; ++j) {
                M.o[j] = other_view(groups[j]);
                gs_knn o = knn[size_t(i) * G + j];
                M.idx[j] = o->idx;
                M.dist[j] = o->dist;
                M.k[j] = o->k;
            }
            M.n_groups = G;
            M.self = i;
            M.min_time = p->min_time_to_collision;
            M.min_sep = p->min_separation_distance;
            M.w_avoid = p->w_avoid;
            M.mask_avoid = p->mask_avoid;
            M.avoid_close = p->avoid_close;
            M.sep = FlockParams{p->sep_min, p->sep_max, p->sep_cos, p->w_sep, p->mask_sep};
            M.ali = FlockParams{p->ali_min, p->ali_max, p->ali_cos, p->w_ali, p->mask_ali};
            M.coh = FlockParams{p->coh_min, p->coh_max, p->coh_cos, p->w_coh, p->mask_coh};
            const gs_path P_i = paths ? paths[i] : nullptr;
            if (P_i) {
                M.has_path = 1;
                M.path = PathDev{P_i->d_points, P_i->d_lengths, P_i->d_normals, P_i->n,
                                 P_i->radius, P_i->cyclic, P_i->total};
                M.path_time = p->path_prediction_time;
                M.w_path = p->w_path;
                M.mask_path = p->mask_path;
                M.w_seek = p->w_seek;
                M.mask_seek = p->mask_seek;
                for (int c = 0; c < 3; ++c) M.seek_target[c] = P_i->h_points[3 + c];
            }
            GS_TRY(launch_multigroup_steer(M, st));
            GS_TRY(launch_update(view(g), p->dt, st));
            for (unsigned j = 0; j < G; ++j)
                GS_TRY(antipen_enqueue(g, knn[size_t(i) * G + j], groups[j], p->mask_antipen, st));
        }
    }
    for (unsigned i = 0; i < G; ++i) {
        touched(groups[i]);
        groups[i]->db.valid = true;  // built this frame, as the reference's stays
    }
    cudaEvent_t done = nullptr;
    for (unsigned i = 1; i < G; ++i) {
        if (groups[i]->stream == st) continue;
        if (!done) {
            GS_CUDA(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
            const cudaError_t e = cudaEventRecord(done, st);
            if (e != cudaSuccess) {
                cudaEventDestroy(done);
                return cuda_fail(e, "cudaEventRecord");
            }
        }
        const cudaError_t e = cudaStreamWaitEvent(groups[i]->stream, done, 0);
        if (e != cudaSuccess) {
            cudaEventDestroy(done);
            return cuda_fail(e, "cudaStreamWaitEvent");
        }
    }
    if (done) cudaEventDestroy(done);
    return GS_OK;
}

gs_status gs_find_knn_walls(gs_group g, gs_knn out, gs_bins bins, gs_walls walls,
                            unsigned search_radius) {
    (void)search_radius;
    if (!g || !out || !bins || !walls) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (out->n != g->n) return fail(GS_ERR_INVALID_ARG, "KNNData size differs from the group");
    if (!g->db.valid || g->db.cells != bins->cells)
        return fail(GS_ERR_STATE, "call gs_update_knn_database first");
    GS_TRY(walls_db(walls, bins->grid, bins->cells, g->stream));
    GS_TRY(launch_knn_binned(g->db, g->n, walls->db, false, bins->radius, out->k, out->idx,
                             out->dist, g->stream));
    return GS_OK;
}

// A grid centred on the origin that covers every position of the other
// group (largest |coordinate| per axis).  Its cell count per axis with extent
// depends on n alone (about two agents per cell for an even spread), so a
// moving crowd keeps the same database; only the cell size follows the
// extent.  False when the extent is not finite.
static bool brute_seed_grid(const float ext[3], unsigned n, Grid& grid, unsigned& C) {
    double w[3], wmax = 0.0;
    for (int a = 0; a < 3; ++a) {
        if (!std::isfinite(ext[a])) return false;
        w[a] = 2.0 * double(ext[a]) * 1.001 + 1e-6;
        wmax = std::max(wmax, w[a]);
    }
    bool active[3];
    int dims = 0;
    for (int a = 0; a < 3; ++a) {
        active[a] = w[a] > 1e-3 * wmax;
        dims += active[a];
    }
    const double per_axis =
        std::floor(std::pow(std::max(1.0, double(n) / 2.0), 1.0 / std::max(1, dims)));
    unsigned long long cells = 1;
    for (int a = 0; a < 3; ++a) {
        grid.wc[a] = active[a] ? unsigned(std::min(std::max(per_axis, 1.0), 1024.0)) : 1u;
        grid.ws[a] = float(w[a]);
        cells *= grid.wc[a];
    }
    if (cells > (1ull << 22)) return false;
    C = unsigned(cells);
    return true;
}

gs_status gs_knn_bruteforce(gs_group g, gs_knn out, gs_group other) {
    if (!g || !out || !other) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (out->n != g->n) return fail(GS_ERR_INVALID_ARG, "KNNData size differs from the group");
    GS_TRY(ensure_reference(g));
    if (other != g) {
        GS_TRY(ensure_reference(other));
        GS_CUDA(cudaStreamSynchronize(other->stream));
    }
    cudaStream_t st = g->stream;
    const float* seed = nullptr;
    g->bf_counted = false;
    g->bf_pairs = (unsigned long long)g->n * other->n;
    // Seed every query's filter with the k-th distance among the candidates
    // of its 3 x 3 x 3 cells on an automatic grid: the k-th distance among a
    // subset of the candidates bounds the true one from above, so the full
    // scan still sees every pair it needs and gives the same lists.  The
    // scan then runs over the seed databases' bucketed arrays and skips
    // chunks of candidates beyond every bound of a warp's queries.
    if (g->n >= 4096 && other->n > out->k) {
        if (!g->bf_tmp) GS_TRY(dalloc(&g->bf_tmp, 6));
        float ext[3];
        GS_TRY(abs_extent(other->position, other->n, g->bf_tmp, ext, st));
        Grid grid;
        unsigned C = 0;
        if (brute_seed_grid(ext, other->n, grid, C)) {
            Database& A = g->bf_a;
            Database& B = other == g ? g->bf_a : g->bf_b;
            GS_TRY(db_reserve(A, g->capacity, C));
            GS_TRY(db_build(A, g->position, g->n, grid, st));
            if (other != g) {
                // sized for the other group's capacity (it may differ per call)
                if (B.cell != nullptr && B.agent_cap < other->capacity) db_release(B);
                GS_TRY(db_reserve(B, other->capacity, C));
                B.agent_cap = other->capacity;
                GS_TRY(db_build(B, other->position, other->n, grid, st));
            }
            // the seed goes to the k-th distance column, which the scan
            // overwrites; a query whose box holds fewer than k candidates at
            // every size tried starts unbounded (its block then takes the
            // longest: it inserts most candidates of the first stages)
            float* seed_col = out->dist + size_t(out->k - 1) * g->n;
            GS_TRY(launch_brute_seed(A, g->n, B, other == g, out->k, seed_col, st));
            seed = seed_col;
            // chunk boxes of 64 candidates, then stage boxes of 32 chunks
            const size_t chunks = (size_t(other->capacity) + 63) / 64;
            const size_t boxes = chunks + (chunks + 31) / 32;
            if (g->bf_boxes_cap < boxes) {
                dfree(g->bf_boxes);
                g->bf_boxes_cap = 0;
                GS_TRY(dalloc(&g->bf_boxes, 2 * boxes));
                g->bf_boxes_cap = boxes;
            }
            auto* evaluated = reinterpret_cast<unsigned long long*>(g->bf_tmp + 4);
            GS_CUDA(cudaMemsetAsync(evaluated, 0, sizeof(unsigned long long), st));
            GS_TRY(launch_knn_brute_bucketed(A.pos_id, g->n, B.pos_id, other->n, g->bf_boxes,
                                             other == g, out->k, seed, evaluated, out->idx,
                                             out->dist, st));
            g->bf_counted = true;
            return read_done(g, other);
        }
    }
    GS_TRY(launch_knn_brute(g->position, g->n, other->position, other->n, other == g, out->k,
                            seed, out->idx, out->dist, st));
    return read_done(g, other);
}

gs_status gs_knn_bruteforce_pairs(gs_group g, unsigned long long* pairs) {
    if (!g || !pairs) return fail(GS_ERR_INVALID_ARG, "null argument");
    *pairs = g->bf_pairs;
    if (!g->bf_counted) return GS_OK;
    GS_CUDA(cudaMemcpyAsync(pairs, g->bf_tmp + 4, sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, g->stream));
    GS_CUDA(cudaStreamSynchronize(g->stream));
    return GS_OK;
}

static gs_status flock_call(int kind, gs_group g, gs_knn knn, gs_group other, float a, float b,
                            float c, float w, unsigned mask) {
    if (!g || !knn || !other) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (knn->n != g->n) return fail(GS_ERR_INVALID_ARG, "KNNData size differs from the group");
    GS_TRY(ensure_reference(g));
    if (other != g) {
        GS_TRY(ensure_reference(other));
        GS_CUDA(cudaStreamSynchronize(other->stream));
    }
    GS_TRY(launch_flock(kind, view(g), knn->idx, knn->k, other_view(other), a, b, c, w, mask,
                        g->stream));
    touched(g);
    return read_done(g, other);
}

gs_status gs_steer_for_separation(gs_group g, gs_knn knn, gs_group other, float min_distance,
                                  float max_distance, float cos_max_angle, float weight,
                                  unsigned mask) {
    return flock_call(0, g, knn, other, min_distance, max_distance, cos_max_angle, weight, mask);
}
gs_status gs_steer_for_alignment(gs_group g, gs_knn knn, gs_group other, float min_distance,
                                 float max_distance, float cos_max_angle, float weight,
                                 unsigned mask) {
    return flock_call(1, g, knn, other, min_distance, max_distance, cos_max_angle, weight, mask);
}
gs_status gs_steer_for_cohesion(gs_group g, gs_knn knn, gs_group other, float min_distance,
                                float max_distance, float cos_max_angle, float weight,
                                unsigned mask) {
    return flock_call(2, g, knn, other, min_distance, max_distance, cos_max_angle, weight, mask);
}

// ---- ExtractData diagnostics ----------------------------------------------------------
// The database the diagnostics read: the per-function one when it is current
// on this grid (gs_update_knn_database since the last change), else the fused
// step's own when the state is still that step's result (the reference reads
// the database its plugin built at the start of the frame, ChokePointNew.cpp:
// 592 and :422-426, which is the fused step's start-of-step buckets).
enum DiagSource { DIAG_NONE, DIAG_DB, DIAG_FRAME };
static DiagSource diag_source(gs_group g, gs_bins bins) {
    if (g->db.valid && g->db.cells == bins->cells &&
        std::memcmp(&g->db.grid, &bins->grid, sizeof(Grid)) == 0)
        return DIAG_DB;
    if (g->frame_cells != 0 && g->frame_cells == bins->cells &&
        std::memcmp(&g->fdb.grid, &bins->grid, sizeof(Grid)) == 0)
        return DIAG_FRAME;
    return DIAG_NONE;
}

// Scratch of the diagnostics, kept with the group (no allocation per call).
static gs_status diag_scratch(gs_group g, size_t bytes, void** p) {
    if (g->diag_bytes < bytes) {
        if (g->diag) cudaFree(g->diag);
        g->diag = nullptr;
        g->diag_bytes = 0;
        GS_CUDA(cudaMalloc(&g->diag, bytes));
        g->diag_bytes = bytes;
    }
    *p = g->diag;
    return GS_OK;
}

static gs_status diag_copy_out(gs_group g, void* host, const void* dev, size_t bytes,
                               gs_status s) {
    if (s == GS_OK && cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, g->stream) !=
                          cudaSuccess)
        s = fail(GS_ERR_CUDA, "cell diagnostics copy");
    if (cudaStreamSynchronize(g->stream) != cudaSuccess && s == GS_OK)
        s = fail(GS_ERR_CUDA, "cell diagnostics");
    return s;
}

gs_status gs_cell_density(gs_group g, gs_bins bins, unsigned* counts) {
    if (!g || !bins) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (!counts) return fail(GS_ERR_INVALID_ARG, "null output");
    const DiagSource src = diag_source(g, bins);
    if (src == DIAG_NONE)
        return fail(GS_ERR_STATE, "call gs_update_knn_database on this grid, or gs_step, first");
    const unsigned C = bins->cells;
    void* d = nullptr;
    GS_TRY(diag_scratch(g, size_t(C) * 4, &d));
    const gs_status s = src == DIAG_DB
                            ? launch_cell_density(g->db, static_cast<unsigned*>(d), g->stream)
                            : launch_frame_cell_density(g->fdb.start, g->fdb.live, C,
                                                        static_cast<unsigned*>(d), g->stream);
    return diag_copy_out(g, counts, d, size_t(C) * 4, s);
}

gs_status gs_cell_avg_velocity(gs_group g, gs_bins bins, float* avg3) {
    if (!g || !bins) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (!avg3) return fail(GS_ERR_INVALID_ARG, "null output");
    const DiagSource src = diag_source(g, bins);
    if (src == DIAG_NONE)
        return fail(GS_ERR_STATE, "call gs_update_knn_database on this grid, or gs_step, first");
    const unsigned C = bins->cells;
    void* d = nullptr;
    GS_TRY(diag_scratch(g, size_t(C) * 12, &d));
    float3* out = static_cast<float3*>(d);
    gs_status s;
    if (src == DIAG_DB) {
        s = launch_cell_avg_velocity(g->db, g->direction, g->speed, out, g->stream);
    } else {
        s = launch_frame_cell_avg_velocity(g->fdb.start, g->fdb.live, C, g->A.f[0], g->A.f[1],
                                           out, g->stream);
    }
    return diag_copy_out(g, avg3, d, size_t(C) * 12, s);
}

// ---- PolylinePathwayCUDA ------------------------------------------------------------
gs_status gs_path_create(const float* points3, unsigned n_in, float radius, int cyclic,
                         gs_path* out) {
    if (!out) return fail(GS_ERR_INVALID_ARG, "null output handle");
    *out = nullptr;
    if (!points3 || n_in == 0) return fail(GS_ERR_INVALID_ARG, "a path needs points");
    if (!std::isfinite(radius)) return fail(GS_ERR_NONFINITE, "radius is not finite");
    for (unsigned i = 0; i < 3 * n_in; ++i)
        if (!std::isfinite(points3[i])) return fail(GS_ERR_NONFINITE, "path point not finite");
    gs_path P = new (std::nothrow) gs_path_s();
    if (!P) return fail(GS_ERR_OOM, "host allocation failed");
    // PolylinePathwayCUDA::Initialize: binary32, the reference's operation order
    const unsigned n = n_in + (cyclic ? 1u : 0u);
    P->n = n;
    P->radius = radius;
    P->cyclic = cyclic ? 1 : 0;
    P->h_points.assign(3 * size_t(n), 0.f);
    P->h_lengths.assign(n, 0.f);
    P->h_normals.assign(3 * size_t(n), 0.f);
    float total = 0.f;
    for (unsigned i = 0; i < n; ++i) {
        const unsigned j = (cyclic && i == n - 1) ? 0u : i;
        for (int c = 0; c < 3; ++c) P->h_points[3 * i + c] = points3[3 * j + c];
        if (i == 0) continue;
        const float sx = P->h_points[3 * i] - P->h_points[3 * i - 3];
        const float sy = P->h_points[3 * i + 1] - P->h_points[3 * i - 2];
        const float sz = P->h_points[3 * i + 2] - P->h_points[3 * i - 1];
        const float len = std::sqrt(((sx * sx) + (sy * sy)) + (sz * sz));
        P->h_lengths[i] = len;
        const bool nz = len > 0.f;
        P->h_normals[3 * i] = nz ? sx / len : sx;
        P->h_normals[3 * i + 1] = nz ? sy / len : sy;
        P->h_normals[3 * i + 2] = nz ? sz / len : sz;
        total += len;
    }
    P->total = total;
    gs_status s = dalloc(&P->d_points, n);
    if (s == GS_OK) s = dalloc(&P->d_lengths, n);
    if (s == GS_OK) s = dalloc(&P->d_normals, n);
    if (s == GS_OK &&
        (cudaMemcpy(P->d_points, P->h_points.data(), size_t(n) * 12, cudaMemcpyHostToDevice) !=
             cudaSuccess ||
         cudaMemcpy(P->d_lengths, P->h_lengths.data(), size_t(n) * 4, cudaMemcpyHostToDevice) !=
             cudaSuccess ||
         cudaMemcpy(P->d_normals, P->h_normals.data(), size_t(n) * 12, cudaMemcpyHostToDevice) !=
             cudaSuccess))
        s = fail(GS_ERR_CUDA, "path upload");
    if (s != GS_OK) {
        gs_path_destroy(P);
        return s;
    }
    *out = P;
    return GS_OK;
}

gs_status gs_path_destroy(gs_path P) {
    if (!P) return GS_OK;
    dfree(P->d_points);
    dfree(P->d_lengths);
    dfree(P->d_normals);
    delete P;
    return GS_OK;
}

gs_status gs_path_get(gs_path P, float* points3, float* lengths, float* normals3, unsigned cap,
                      unsigned* n, float* total_length) {
    if (!P) return fail(GS_ERR_INVALID_ARG, "null path");
    if (n) *n = P->n;
    if (total_length) *total_length = P->total;
    if ((points3 || lengths || normals3) && cap < P->n)
        return fail(GS_ERR_INVALID_ARG, "path arrays too small");
    if (points3) std::memcpy(points3, P->h_points.data(), size_t(P->n) * 12);
    if (lengths) std::memcpy(lengths, P->h_lengths.data(), size_t(P->n) * 4);
    if (normals3) std::memcpy(normals3, P->h_normals.data(), size_t(P->n) * 12);
    return GS_OK;
}

gs_status gs_steer_to_follow_path(gs_group g, gs_path P, float prediction_time, float weight,
                                  unsigned mask) {
    if (!g || !P) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (P->n < 2) return fail(GS_ERR_INVALID_ARG, "follow-path needs a path of 2+ points");
    if (!std::isfinite(prediction_time) || !std::isfinite(weight))
        return fail(GS_ERR_NONFINITE, "non-finite parameter");
    GS_TRY(ensure_reference(g));
    GS_TRY(launch_follow_path(view(g),
                              PathDev{P->d_points, P->d_lengths, P->d_normals, P->n, P->radius,
                                      P->cyclic, P->total},
                              prediction_time, weight, mask, g->stream));
    touched(g);
    return GS_OK;
}

gs_status gs_steer_for_seek(gs_group g, const float target[3], float weight, unsigned mask) {
    if (!g || !target) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (!finite3(target)) return fail(GS_ERR_NONFINITE, "seek target is not finite");
    GS_TRY(ensure_reference(g));
    GS_TRY(launch_seek(view(g), target, weight, mask, g->stream));
    touched(g);
    return GS_OK;
}

gs_status gs_steer_to_avoid_neighbors(gs_group g, gs_knn knn, gs_group other,
                                      float min_time_to_collision, float min_separation_distance,
                                      int avoid_close, float weight, unsigned mask) {
    if (!g || !knn || !other) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (knn->n != g->n) return fail(GS_ERR_INVALID_ARG, "KNNData size differs from the group");
    GS_TRY(ensure_reference(g));
    if (other != g) {
        GS_TRY(ensure_reference(other));
        GS_CUDA(cudaStreamSynchronize(other->stream));
    }
    GS_TRY(launch_avoid_neighbors(view(g), knn->idx, knn->dist, knn->k, other_view(other),
                                  min_time_to_collision, min_separation_distance,
                                  avoid_close != 0, weight, mask, g->stream));
    touched(g);
    return read_done(g, other);
}

gs_status gs_steer_to_avoid_walls(gs_group g, gs_knn knw, gs_walls walls, float min_time,
                                  float weight, unsigned mask) {
    if (!g || !knw || !walls) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (knw->n != g->n) return fail(GS_ERR_INVALID_ARG, "KNNData size differs from the group");
    GS_TRY(ensure_reference(g));
    GS_TRY(launch_avoid_walls(view(g), knw->idx, knw->k, walls->start, walls->end, walls->normal,
                              walls->n, min_time, weight, mask, g->stream));
    touched(g);
    return GS_OK;
}

gs_status gs_update_group(gs_group g, float elapsed_time) {
    if (!g) return fail(GS_ERR_INVALID_ARG, "null group");
    if (!std::isfinite(elapsed_time)) return fail(GS_ERR_NONFINITE, "elapsed time is not finite");
    GS_TRY(ensure_reference(g));
    GS_TRY(launch_update(view(g), elapsed_time, g->stream));
    g->fused_current = false;
    g->frame_cells = 0;
    g->accum_dirty = false;
    return GS_OK;
}

gs_status gs_update_group_with_antipenetration(gs_group g, gs_knn knw, gs_walls walls,
                                               float elapsed_time) {
    if (!g || !knw || !walls) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (knw->n != g->n) return fail(GS_ERR_INVALID_ARG, "KNNData size differs from the group");
    if (!std::isfinite(elapsed_time)) return fail(GS_ERR_NONFINITE, "elapsed time is not finite");
    GS_TRY(ensure_reference(g));
    GS_TRY(launch_update_antipen_wall(view(g), knw->idx, knw->k, walls->start, walls->end,
                                      walls->normal, walls->n, elapsed_time, g->stream));
    g->fused_current = false;
    g->frame_cells = 0;
    g->accum_dirty = false;
    return GS_OK;
}

gs_status gs_anti_penetration_wall(gs_group g, gs_knn knw, gs_walls walls, float elapsed_time,
                                   unsigned /*do_not_apply_with: unused, as in the reference*/) {
    if (!g || !knw || !walls) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (knw->n != g->n) return fail(GS_ERR_INVALID_ARG, "KNNData size differs from the group");
    if (!std::isfinite(elapsed_time)) return fail(GS_ERR_NONFINITE, "elapsed time is not finite");
    GS_TRY(ensure_reference(g));
    GS_TRY(launch_antipen_wall(view(g), knw->idx, knw->k, walls->start, walls->end,
                               walls->normal, walls->n, elapsed_time, g->stream));
    touched(g);
    return GS_OK;
}

// antiPenetrationAgents on g's stream, with the scratch kept with the group
// (grown on demand, not allocated per call as the reference's
// AntiPenetrationAgentsCUDA does): the new positions, then a snapshot of the
// other group's bits.  Queued on st; the groups' earlier work must be complete
// or on st.
static gs_status antipen_enqueue(gs_group g, gs_knn knn, gs_group other, unsigned mask,
                                 cudaStream_t st) {
    if (g->n == 0) return GS_OK;
    const size_t pos_bytes = size_t(g->n) * 16, snap_bytes = size_t(other->n ? other->n : 1) * 4;
    if (g->ap_bytes < pos_bytes + snap_bytes) {
        GS_CUDA(cudaStreamSynchronize(st));
        if (g->ap) cudaFree(g->ap);
        g->ap = nullptr;
        g->ap_bytes = 0;
        GS_CUDA(cudaMalloc(&g->ap, pos_bytes + snap_bytes));
        g->ap_bytes = pos_bytes + snap_bytes;
    }
    float4* pos_out = static_cast<float4*>(g->ap);
    unsigned* snap = reinterpret_cast<unsigned*>(static_cast<char*>(g->ap) + pos_bytes);
    if (other->n)
        GS_CUDA(cudaMemcpyAsync(snap, other->applied, size_t(other->n) * 4,
                                cudaMemcpyDeviceToDevice, st));
    return launch_antipenetration(view(g), knn->idx, knn->dist, knn->k, other_view(other), snap,
                                  pos_out, mask, st);
}

gs_status gs_anti_penetration_agents(gs_group g, gs_knn knn, gs_group other, unsigned mask) {
    if (!g || !knn || !other) return fail(GS_ERR_INVALID_ARG, "null argument");
    if (knn->n != g->n) return fail(GS_ERR_INVALID_ARG, "KNNData size differs from the group");
    GS_TRY(ensure_reference(g));
    if (other != g) {
        GS_TRY(ensure_reference(other));
        GS_CUDA(cudaStreamSynchronize(other->stream));
    }
    GS_TRY(antipen_enqueue(g, knn, other, mask, g->stream));
    touched(g);
    return read_done(g, other);
}

// ---- fused step ------------------------------------------------------------------
static gs_status reserve_fused(gs_group g, unsigned C, bool walls, unsigned k, unsigned n_scenes) {
    if (!g->cellrank) {
        const size_t n = g->capacity;
        for (int j = 0; j < 6; ++j) {
            GS_TRY(dalloc(&g->A.f[j], n));
            GS_TRY(dalloc(&g->B.f[j], n));
        }
        GS_TRY(dalloc(&g->cellrank, n));
        GS_TRY(dalloc(&g->d_err, 1));
        GS_TRY(dalloc(&g->retry, n));
        GS_TRY(dalloc(&g->slot_of, n));
        GS_TRY(dalloc(&g->retry_count, 1));
        GS_TRY(dalloc(&g->retry_knn, size_t(std::min<size_t>(n, kRetryListCap)) * kRetryListK));
        GS_TRY(dalloc(&g->d_stat, 4));
        GS_TRY(dalloc(&g->d_bar, 2));
        GS_CUDA(cudaMemset(g->d_bar, 0, 2 * sizeof(unsigned)));
        GS_CUDA(cudaMemset(g->d_err, 0, sizeof(unsigned)));
        GS_CUDA(cudaMemset(g->retry_count, 0, sizeof(unsigned)));
        GS_CUDA(cudaDeviceSynchronize());
    }
    if (g->scene_alloc < n_scenes) {
        dfree(g->d_scene);
        GS_TRY(dalloc(&g->d_scene, n_scenes));
        g->scene_alloc = n_scenes;
    }
    if (g->fdb.cells != C) GS_TRY(db_reserve(g->fdb, 0, C));
    if (walls && (!g->w0 || g->fused_k_alloc < k)) {
        const size_t n = g->capacity;
        dfree(g->w0);
        dfree(g->w1);
        dfree(g->w2);
        dfree(g->knn_slot);
        dfree(g->knn_dist);
        GS_TRY(dalloc(&g->w0, n));
        GS_TRY(dalloc(&g->w1, n));
        GS_TRY(dalloc(&g->w2, n));
        GS_TRY(dalloc(&g->knn_slot, n * k));
        GS_TRY(dalloc(&g->knn_dist, n * k));
        g->fused_k_alloc = k;
    }
    return GS_OK;
}

static_assert(sizeof(FusedLaunch) <= sizeof(FusedLaunchBytes), "graph key size");
static_assert(sizeof(StepDev) <= sizeof(StepDevBytes), "graph key size");

// Uploads the scene table when it differs from the one on the device.
static gs_status put_scenes(gs_group g, const std::vector<Scene>& scenes) {
    if (g->h_scenes && *g->h_scenes == scenes) return GS_OK;
    if (!g->h_scenes) g->h_scenes = new std::vector<Scene>();
    *g->h_scenes = scenes;
    GS_CUDA(cudaMemcpyAsync(g->d_scene, g->h_scenes->data(), scenes.size() * sizeof(Scene),
                            cudaMemcpyHostToDevice, g->stream));
    return GS_OK;
}

struct WallsDev {
    const float4 *start = nullptr, *end = nullptr, *normal = nullptr, *pos_id = nullptr;
    const unsigned* cell_start = nullptr;
};

// Zeroes the fused engine's counts before a recount.
static gs_status clear_counts(gs_group g, unsigned C, cudaStream_t st) {
    GS_CUDA(cudaMemsetAsync(g->fdb.count, 0, size_t(C) * 4, st));
    return GS_OK;
}

// One step's launches: scan, permute, fused (+ exact redo); or, for a
// supported step with the persistent form on, one launch for all of them.
static gs_status step_body(gs_group g, const FusedLaunch& L, const StepDev& d, unsigned C,
                           PhaseHook* hook) {
    cudaStream_t st = g->stream;
    if (d.persistent && persistent_supported(d)) {
        PersistLaunch P;
        P.start = g->fdb.start;
        P.tile = g->fdb.tile;
        P.live = g->fdb.live;
        P.C = C;
        P.T = scan_tile_count(C);
        P.bar = g->d_bar;
        P.limit = d.bar_limit;
        if (hook) hook->mark(2, true);
        GS_TRY(fused_step_persistent(L, d, P, st));
        if (hook) hook->mark(2, false);
        return GS_OK;
    }
    if (hook) hook->mark(0, true);
    GS_TRY(scan_counts_sparse(g->fdb.count, g->fdb.start, C, g->fdb.tile, g->fdb.live,
                              d.scan_reach, st));
    if (hook) hook->mark(0, false);
    if (hook) hook->mark(1, true);
    GS_TRY(fused_permute(L, d.wrap_mode, d.dirty != 0, d.fresh != 0, st));
    if (hook) hook->mark(1, false);
    GS_TRY(fused_step(L, d, st, hook));
    return GS_OK;
}

static void fill_launch(gs_group g, const StepDev& d, const WallsDev& w, FusedLaunch& L);

// Whether the first step after an upload permutes by a gather.  A scene's
// agents in agent order scatter within the scene's slot range: a scene of a
// few thousand agents (a few hundred KB) scatters into lines that stay in L2
// until they are whole, and there the gather's extra pass only adds time.
// Measured end to end: a 10,000-agent scene, and batched scenes of up to
// 20,000, are as fast either way (within 1-2 %); a 1,048,576-agent flock
// gains 5 % with the gather.
constexpr unsigned kGatherPermuteMinAgents = 1u << 17;  // 12 MB of state per scene
static bool gather_first_permute(gs_group g) {
    unsigned most = 0;
    if (g->h_scenes)
        for (const Scene& sc : *g->h_scenes) most = std::max(most, sc.n_agents);
    return most >= kGatherPermuteMinAgents;
}

// Brings the fused engine's bucketed state and pending cell counts up to
// date for steps on `grid` and fills the launch block L; picks the KNN
// capacity into d.  dirty: the first step must add the steering and applied
// bits left by per-function calls.  fresh: the bucketed state was just
// rebuilt in agent order, from scenes large enough that the first step's
// permute gathers.
static gs_status fused_setup(gs_group g, StepDev& d, const Grid& grid, unsigned C,
                             const unsigned* agent_scene, const WallsDev& w, FusedLaunch& L,
                             bool& dirty, bool& fresh) {
    cudaStream_t st = g->stream;
    dirty = false;
    fresh = false;
    if (!g->fused_current) {
        dirty = g->accum_dirty;
        fresh = gather_first_permute(g);
        // counts left pending by an earlier fused step no longer apply
        GS_TRY(clear_counts(g, C, st));
        GS_TRY(fused_from_reference(view(g), agent_scene, g->d_scene, g->A, g->cellrank,
                                    g->fdb.count, d.wrap_mode, dirty, st));
        GS_TRY(scan_tile_totals(g->fdb.count, C, g->fdb.tile, st));
        g->fused_current = true;
    } else if (std::memcmp(&g->fdb.grid, &grid, sizeof(Grid)) != 0 || !g->fdb.valid ||
               g->pending_wrap != d.wrap_mode) {
        GS_TRY(clear_counts(g, C, st));
        GS_TRY(fused_recount(g->A, g->n, g->d_scene, g->cellrank, g->fdb.count, d.wrap_mode,
                             st));
        GS_TRY(scan_tile_totals(g->fdb.count, C, g->fdb.tile, st));
    }
    g->fdb.grid = grid;
    g->fdb.valid = true;
    g->pending_wrap = d.wrap_mode;
    if (g->knn_cap) {
        d.enum_cap = g->knn_cap;
    } else {
        if (!g->auto_cap_valid || g->auto_cap_r != d.r ||
            std::memcmp(&g->auto_cap_grid, &grid, sizeof(Grid)) != 0) {
            // one synchronising read per upload or grid change
            unsigned occupied = 0;
            unsigned long long sumsq = 0;
            GS_TRY(count_occupied(g->fdb.count, C, g->d_stat, &occupied, &sumsq, st));
            g->auto_cap = knn_capacity(g->n, sumsq, grid, d.r);
            g->auto_cap_grid = grid;
            g->auto_cap_r = d.r;
            g->auto_cap_valid = true;
        }
        d.enum_cap = g->auto_cap;
    }

    fill_launch(g, d, w, L);
    return GS_OK;
}

// The launch block of the fused kernels for the group's current buffers.
static void fill_launch(gs_group g, const StepDev& d, const WallsDev& w, FusedLaunch& L) {
    std::memset(static_cast<void*>(&L), 0, sizeof(L));  // byte-compared as a graph key
    L.A = g->A;
    L.B = g->B;
    L.cellrank = g->cellrank;
    L.count = g->fdb.count;
    L.tile = g->fdb.tile;
    L.tiles = scan_tile_count(g->fdb.cells);
    L.start = g->fdb.start;
    L.scenes = g->d_scene;
    L.n = g->n;
    L.err = g->d_err;
    L.retry = g->retry;
    L.retry_count = g->retry_count;
    L.agent_at = g->slot_of;  // free during a step: fused_to_reference refills it
    L.retry_knn = g->retry_knn;
    L.retry_cap = unsigned(std::min<size_t>(g->capacity, kRetryListCap));
    if (d.need & NEED_WALLS) {
        L.w_start = w.start;
        L.w_end = w.end;
        L.w_normal = w.normal;
        L.w_pos_id = w.pos_id;
        L.w_cell_start = w.cell_start;
        L.w0 = g->w0;
        L.w1 = g->w1;
        L.w2 = g->w2;
        L.knn_slot = g->knn_slot;
        L.knn_dist = g->knn_dist;
    }
}

// The fused engine for a group whose scene table is in g->h_scenes / d_scene
// (one scene for a plain group, many for a batch).
static gs_status fused_run(gs_group g, StepDev d, const Grid& grid, unsigned C,
                           const unsigned* agent_scene, const WallsDev& w, unsigned steps) {
    cudaStream_t st = g->stream;
    FusedLaunch L;
    bool dirty = false, fresh = false;
    g->frame_cells = 0;
    // part of the graph key: a changed form or limit captures again
    d.persistent = g->persistent ? 1u : 0u;
    d.bar_limit = g->bar_limit ? g->bar_limit : kBarrierPollsDefault;
    GS_TRY(fused_setup(g, d, grid, C, agent_scene, w, L, dirty, fresh));
    Profiler prof(g);
    PhaseHook* hook = g->profiling ? &prof : nullptr;
    unsigned step = 0;
    // A step with steering carried in from per-function calls, or the first
    // after an upload (its permute gathers), runs eagerly; so do all steps
    // while profiling, and the first step of a new launch configuration
    // (which also performs one-time kernel set-up).
    const bool cfg_same = g->graph_exec && std::memcmp(&g->graph_L, &L, sizeof(L)) == 0 &&
                          std::memcmp(&g->graph_d, &d, sizeof(d)) == 0 && g->graph_C == C;
    // The legacy default stream cannot be captured: a group on it runs eagerly.
    const bool graphs = g->use_graph && st != cudaStreamLegacy && st != nullptr;
    if (dirty || fresh || hook || !graphs || !cfg_same) {
        const unsigned eager = (hook || !graphs) ? steps : 1u;
        for (; step < eager && step < steps; ++step) {
            d.dirty = dirty ? 1 : 0;
            d.fresh = fresh ? 1 : 0;
            GS_TRY(step_body(g, L, d, C, hook));
            dirty = false;
            fresh = false;
        }
    }
    d.dirty = 0;
    d.fresh = 0;
    if (step < steps) {
        if (!(g->graph_exec && std::memcmp(&g->graph_L, &L, sizeof(L)) == 0 &&
              std::memcmp(&g->graph_d, &d, sizeof(d)) == 0 && g->graph_C == C)) {
            drop_graph(g);
            cudaGraph_t graph = nullptr;
            GS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            const gs_status s = step_body(g, L, d, C, nullptr);
            const cudaError_t e = cudaStreamEndCapture(st, &graph);
            if (s != GS_OK) {
                if (graph) cudaGraphDestroy(graph);
                return s;
            }
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
            const cudaError_t ei = cudaGraphInstantiate(&g->graph_exec, graph, 0);
            cudaGraphDestroy(graph);
            if (ei != cudaSuccess) {
                g->graph_exec = nullptr;
                return cuda_fail(ei, "cudaGraphInstantiate");
            }
            std::memcpy(&g->graph_L, &L, sizeof(L));
            std::memcpy(&g->graph_d, &d, sizeof(d));
            g->graph_C = C;
        }
        for (; step < steps; ++step) GS_CUDA(cudaGraphLaunch(g->graph_exec, st));
    }
    g->accum_dirty = false;
    g->db.valid = false;
    g->frame_cells = C;
    return GS_OK;
}

gs_status gs_step(gs_group g, gs_bins bins, gs_walls walls, const gs_step_params* p,
                  unsigned steps) {
    if (!g || !bins) return fail(GS_ERR_INVALID_ARG, "null argument");
    StepDev d;
    GS_TRY(validate_step(p, walls, d));
    Grid grid;
    unsigned C;
    GS_TRY(check_grid(p->world_cells, p->world_size, grid, C));
    if (C != bins->cells || std::memcmp(&grid, &bins->grid, sizeof(Grid)) != 0)
        return fail(GS_ERR_INVALID_ARG, "step grid differs from the bins");
    const bool has_walls = d.need & NEED_WALLS;
    if (has_walls && !walls) return fail(GS_ERR_INVALID_ARG, "avoid-walls needs a wall group");
    if (steps == 0 || g->n == 0) return GS_OK;
    GS_TRY(reserve_fused(g, C, has_walls, d.k, 1));
    if (has_walls) GS_TRY(walls_db(walls, grid, C, g->stream));
    Scene sc{};
    sc.grid = grid;
    sc.n_agents = g->n;
    sc.n_walls = has_walls ? walls->n : 0;
    GS_TRY(put_scenes(g, std::vector<Scene>{sc}));
    d.block = g->block;
    WallsDev w;
    if (has_walls) {
        w.start = walls->start;
        w.end = walls->end;
        w.normal = walls->normal;
        w.pos_id = walls->db.pos_id;
        w.cell_start = walls->db.start;
    }
    return fused_run(g, d, grid, C, nullptr, w, steps);
}

gs_status gs_step_host(gs_group g, gs_bins bins, gs_walls walls, const gs_step_params* p,
                       unsigned steps, const gs_agent_arrays* in, unsigned n,
                       const gs_agent_arrays* out) {
    if (!g || !in || !out) return fail(GS_ERR_INVALID_ARG, "null argument");
    GS_TRY(gs_group_upload(g, in, n));
    GS_TRY(gs_step(g, bins, walls, p, steps));
    // in place, the per-agent constants no step changes (maxSpeed, maxForce,
    // radius, mass) are already on the host and are not copied back
    const bool in_place = out->max_speed == in->max_speed && out->max_force == in->max_force &&
                          out->radius == in->radius && out->mass == in->mass;
    GS_TRY(download_enqueue(g, out, in_place));
    GS_CUDA(cudaStreamSynchronize(g->stream));
    return check_device_flags(g);
}

gs_status gs_group_set_persistent(gs_group g, int enable) {
    if (!g) return fail(GS_ERR_INVALID_ARG, "null group");
    g->persistent = enable != 0;
    return GS_OK;
}

gs_status gs_group_set_barrier_limit(gs_group g, unsigned polls) {
    if (!g) return fail(GS_ERR_INVALID_ARG, "null group");
    g->bar_limit = polls;
    return GS_OK;
}

gs_status gs_group_set_graphs(gs_group g, int enable) {
    if (!g) return fail(GS_ERR_INVALID_ARG, "null group");
    g->use_graph = enable != 0;
    if (!g->use_graph) drop_graph(g);
    return GS_OK;
}

gs_status gs_group_set_knn_capacity(gs_group g, unsigned capacity) {
    if (!g) return fail(GS_ERR_INVALID_ARG, "null group");
    if (capacity != 0 && capacity != 32 && capacity != 64 && capacity != 128 && capacity != 256)
        return fail(GS_ERR_INVALID_ARG, "KNN capacity must be 0 (auto), 32, 64, 128 or 256");
    g->knn_cap = capacity;
    return GS_OK;
}

gs_status gs_group_knn_capacity(gs_group g, unsigned* capacity) {
    if (!g || !capacity) return fail(GS_ERR_INVALID_ARG, "null argument");
    *capacity = g->knn_cap ? g->knn_cap : (g->auto_cap_valid ? g->auto_cap : 0u);
    return GS_OK;
}

gs_status gs_group_set_block(gs_group g, unsigned threads) {
    if (!g) return fail(GS_ERR_INVALID_ARG, "null group");
    if (threads != 64 && threads != 128 && threads != 256)
        return fail(GS_ERR_INVALID_ARG, "threads per block must be 64, 128 or 256");
    g->block = threads;
    return GS_OK;
}

// ---- batched scenes ---------------------------------------------------------------
gs_status gs_batch_destroy(gs_batch b) {
    if (!b) return GS_OK;
    if (b->io_exec) cudaGraphExecDestroy(b->io_exec);
    gs_group_destroy(b->g);
    dfree(b->agent_scene);
    dfree(b->w_start);
    dfree(b->w_end);
    dfree(b->w_normal);
    dfree(b->w_pos_id);
    dfree(b->w_cell_start);
    delete b;
    return GS_OK;
}

gs_status gs_batch_create(unsigned n_scenes, const unsigned* agents_per_scene, unsigned k,
                          const unsigned world_cells[3], const float world_size[3],
                          unsigned search_radius, void* stream, gs_batch* out) {
    if (!out || !agents_per_scene || !world_cells || !world_size)
        return fail(GS_ERR_INVALID_ARG, "null argument");
    if (n_scenes == 0) return fail(GS_ERR_INVALID_ARG, "no scenes");
    Grid grid;
    unsigned cells;
    GS_TRY(check_grid(world_cells, world_size, grid, cells));
    unsigned long long total = 0;
    for (unsigned s = 0; s < n_scenes; ++s) total += agents_per_scene[s];
    if (total == 0 || total > (1ull << 30)) return fail(GS_ERR_INVALID_ARG, "bad agent count");
    if (static_cast<unsigned long long>(cells) * n_scenes > (1ull << 31))
        return fail(GS_ERR_INVALID_ARG, "too many cells over all scenes");
    gs_batch b = new (std::nothrow) gs_batch_s();
    if (!b) return fail(GS_ERR_OOM, "host allocation failed");
    b->grid = grid;
    b->cells = cells;
    b->radius = search_radius;
    b->counts.assign(agents_per_scene, agents_per_scene + n_scenes);
    b->walls.resize(n_scenes);
    b->total = unsigned(total);
    gs_status st = gs_group_create(k, b->total, stream, &b->g);
    std::vector<unsigned> scene_of(b->total);
    unsigned off = 0;
    for (unsigned s = 0; s < n_scenes; ++s) {
        Scene sc{};
        sc.grid = grid;
        sc.cell_offset = s * cells;
        sc.agent_offset = off;
        sc.n_agents = agents_per_scene[s];
        sc.wall_cell_offset = s * cells;
        b->scenes.push_back(sc);
        for (unsigned i = 0; i < agents_per_scene[s]; ++i) scene_of[off + i] = s;
        off += agents_per_scene[s];
    }
    if (st == GS_OK) st = dalloc(&b->agent_scene, b->total);
    if (st == GS_OK &&
        cudaMemcpy(b->agent_scene, scene_of.data(), size_t(b->total) * 4, cudaMemcpyHostToDevice) !=
            cudaSuccess)
        st = fail(GS_ERR_CUDA, "scene map upload");
    if (st != GS_OK) {
        const std::string msg = g_last_error;
        gs_batch_destroy(b);
        set_error(msg);
        return st;
    }
    *out = b;
    return GS_OK;
}

gs_status gs_batch_set_walls(gs_batch b, unsigned scene, const float* start4, const float* end4,
                             const float* normal4, unsigned n) {
    if (!b) return fail(GS_ERR_INVALID_ARG, "null batch");
    if (scene >= b->scenes.size()) return fail(GS_ERR_INVALID_ARG, "scene out of range");
    if (n > 0 && (!start4 || !end4 || !normal4)) return fail(GS_ERR_INVALID_ARG, "null arrays");
    std::vector<Segment> raw(n);
    for (unsigned i = 0; i < n; ++i) {
        raw[i].s = v3(start4[4 * i], start4[4 * i + 1], start4[4 * i + 2]);
        raw[i].e = v3(end4[4 * i], end4[4 * i + 1], end4[4 * i + 2]);
        raw[i].n = v3(normal4[4 * i], normal4[4 * i + 1], normal4[4 * i + 2]);
        raw[i].m = v3(0.5f * (raw[i].s.x + raw[i].e.x), 0.5f * (raw[i].s.y + raw[i].e.y),
                      0.5f * (raw[i].s.z + raw[i].e.z));
    }
    b->walls[scene] = split_walls(raw, b->grid);
    b->walls_dirty = true;
    return GS_OK;
}

// Concatenated wall arrays and the walls' bucketed database over all scenes'
// cells (wall index = the scene-local index, as a per-scene run sees it).
static gs_status batch_walls(gs_batch b) {
    if (!b->walls_dirty) return GS_OK;
    const unsigned S = unsigned(b->scenes.size());
    const unsigned Ct = b->cells * S;
    std::vector<float4> st, en, nm, mid;
    std::vector<unsigned> label;
    for (unsigned s = 0; s < S; ++s) {
        b->scenes[s].wall_offset = unsigned(st.size());
        b->scenes[s].n_walls = unsigned(b->walls[s].size());
        for (unsigned j = 0; j < b->walls[s].size(); ++j) {
            const Segment& w = b->walls[s][j];
            st.push_back(f4(w.s, 0.f));
            en.push_back(f4(w.e, 0.f));
            nm.push_back(f4(w.n, 0.f));
            float idbits;
            std::memcpy(&idbits, &j, sizeof(float));
            mid.push_back(f4(w.m, idbits));
            label.push_back(b->scenes[s].cell_offset + cell_of(b->grid, w.m));
        }
    }
    const unsigned W = unsigned(st.size());
    std::vector<unsigned> start(size_t(Ct) + 1, 0u);
    for (unsigned i = 0; i < W; ++i) start[label[i] + 1]++;
    for (unsigned c = 0; c < Ct; ++c) start[c + 1] += start[c];
    std::vector<float4> pos_id(W);
    {
        std::vector<unsigned> fill(start.begin(), start.end() - 1);
        for (unsigned i = 0; i < W; ++i) pos_id[fill[label[i]]++] = mid[i];
    }
    dfree(b->w_start);
    dfree(b->w_end);
    dfree(b->w_normal);
    dfree(b->w_pos_id);
    dfree(b->w_cell_start);
    GS_TRY(dalloc(&b->w_start, W));
    GS_TRY(dalloc(&b->w_end, W));
    GS_TRY(dalloc(&b->w_normal, W));
    GS_TRY(dalloc(&b->w_pos_id, W));
    GS_TRY(dalloc(&b->w_cell_start, size_t(Ct) + 1));
    if (W) {
        GS_CUDA(cudaMemcpy(b->w_start, st.data(), W * sizeof(float4), cudaMemcpyHostToDevice));
        GS_CUDA(cudaMemcpy(b->w_end, en.data(), W * sizeof(float4), cudaMemcpyHostToDevice));
        GS_CUDA(cudaMemcpy(b->w_normal, nm.data(), W * sizeof(float4), cudaMemcpyHostToDevice));
        GS_CUDA(cudaMemcpy(b->w_pos_id, pos_id.data(), W * sizeof(float4), cudaMemcpyHostToDevice));
    }
    GS_CUDA(cudaMemcpy(b->w_cell_start, start.data(), (size_t(Ct) + 1) * 4,
                       cudaMemcpyHostToDevice));
    b->n_walls = W;
    b->walls_dirty = false;
    drop_graph(b->g);
    return GS_OK;
}

gs_status gs_batch_upload(gs_batch b, const gs_agent_arrays* host) {
    if (!b) return fail(GS_ERR_INVALID_ARG, "null batch");
    return gs_group_upload(b->g, host, b->total);
}

gs_status gs_batch_download(gs_batch b, const gs_agent_arrays* host) {
    if (!b) return fail(GS_ERR_INVALID_ARG, "null batch");
    return gs_group_download(b->g, host);
}

gs_status gs_batch_group(gs_batch b, gs_group* g) {
    if (!b || !g) return fail(GS_ERR_INVALID_ARG, "null argument");
    *g = b->g;
    return GS_OK;
}

// Host arrays of agents [off, ...) of `h`.
static gs_agent_arrays host_at(const gs_agent_arrays& h, size_t off) {
    gs_agent_arrays v = h;
    v.position = h.position + 4 * off;
    v.direction = h.direction + 4 * off;
    v.steering = h.steering + 4 * off;
    v.side = h.side + 3 * off;
    v.up = h.up + 3 * off;
    v.speed = h.speed + off;
    v.max_speed = h.max_speed + off;
    v.max_force = h.max_force + off;
    v.radius = h.radius + off;
    v.mass = h.mass + off;
    v.applied = h.applied + off;
    return v;
}

static gs_status batch_prepare(gs_batch b, const gs_step_params* p, StepDev& d, Grid& grid,
                               unsigned& Ct, WallsDev& w);

// True when every array of h is page-locked host memory (copies from it can
// be captured in a graph and overlap with other work).
static bool host_pinned(const gs_agent_arrays& h) {
    const void* ptrs[] = {h.position, h.direction, h.steering, h.side, h.up, h.speed,
                          h.max_speed, h.max_force, h.radius, h.mass, h.applied};
    for (const void* q : ptrs) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
            cudaGetLastError();  // clear the query's error
            return false;
        }
        if (a.type != cudaMemoryTypeHost) return false;
    }
    return true;
}


// One part's plan for gs_batches_step_host: its launch set-up and host views.
struct IoPart {
    gs_batch b;
    StepDev d;
    Grid grid;
    unsigned Ct;
    WallsDev w;
    FusedLaunch L;
    gs_agent_arrays hi, ho;
};

// One part's upload, then its steps, conversion back and download, queued on
// its stream: the eager sequence (the upload marks steering and applied bits
// as carried in, so the first step adds them), as a graph captures it.
static gs_status io_upload(IoPart& q) { return upload_enqueue(q.b->g, &q.hi, q.b->g->n); }

static gs_status io_compute_and_download(IoPart& q, unsigned steps, bool in_place) {
    gs_group g = q.b->g;
    cudaStream_t st = g->stream;
    GS_TRY(clear_counts(g, q.Ct, st));
    GS_TRY(fused_from_reference(view(g), q.b->agent_scene, g->d_scene, g->A, g->cellrank,
                                g->fdb.count, q.d.wrap_mode, true, st));
    GS_TRY(scan_tile_totals(g->fdb.count, q.Ct, g->fdb.tile, st));
    for (unsigned i = 0; i < steps; ++i) {
        StepDev di = q.d;
        di.dirty = i == 0 ? 1 : 0;
        di.fresh = i == 0 && gather_first_permute(g) ? 1 : 0;
        GS_TRY(step_body(g, q.L, di, q.Ct, nullptr));
    }
    GS_TRY(fused_to_reference(g->A, g->n, g->d_scene, g->slot_of, view(g), st));
    return download_copies(g, &q.ho, in_place);
}

// The parts of gs_batches_step_host as one graph over the parts' streams:
// part i's uploads follow part i-1's (so the first part's data arrive first
// and its steps start early), its steps follow its uploads, its download its
// steps.  One launch per call, kept while the key (parts, host arrays,
// buffers, parameters) holds; cached on the first part.
static gs_status io_graph(std::vector<IoPart>& parts, unsigned steps, bool in_place) {
    gs_batch b0 = parts[0].b;
    cudaStream_t st0 = b0->g->stream;
    std::vector<unsigned char> key;
    auto put = [&](const void* v, size_t bytes) {
        const unsigned char* c = static_cast<const unsigned char*>(v);
        key.insert(key.end(), c, c + bytes);
    };
    for (const IoPart& q : parts) {
        put(&q.b, sizeof(q.b));
        put(&q.hi, sizeof(q.hi));
        put(&q.ho, sizeof(q.ho));
        put(&q.L, sizeof(q.L));
        put(&q.d, sizeof(q.d));
        const unsigned extra[2] = {q.b->g->n, q.Ct};
        put(extra, sizeof(extra));
    }
    const unsigned call[2] = {steps, in_place ? 1u : 0u};
    put(call, sizeof(call));
    if (!b0->io_exec || key != b0->io_key) {
        if (b0->io_exec) cudaGraphExecDestroy(b0->io_exec);
        b0->io_exec = nullptr;
        b0->io_key.clear();
        const size_t P = parts.size();
        std::vector<cudaEvent_t> ev(2 * P, nullptr);  // uploaded_i, done_i
        gs_status s = GS_OK;
        for (cudaEvent_t& e : ev)
            if (s == GS_OK && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
                s = fail(GS_ERR_CUDA, "cudaEventCreate");
        cudaGraph_t graph_h = nullptr;
        if (s == GS_OK && cudaStreamBeginCapture(st0, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
            s = fail(GS_ERR_CUDA, "cudaStreamBeginCapture");
        const bool capturing = s == GS_OK;
        for (size_t i = 0; i < P && s == GS_OK; ++i) {
            cudaStream_t st = parts[i].b->g->stream;
            if (i > 0 && cudaStreamWaitEvent(st, ev[i - 1], 0) != cudaSuccess)
                s = fail(GS_ERR_CUDA, "cudaStreamWaitEvent");
            if (s == GS_OK) s = io_upload(parts[i]);
            if (s == GS_OK && cudaEventRecord(ev[i], st) != cudaSuccess)
                s = fail(GS_ERR_CUDA, "cudaEventRecord");
            if (s == GS_OK) s = io_compute_and_download(parts[i], steps, in_place);
            if (s == GS_OK && i > 0 && cudaEventRecord(ev[P + i], st) != cudaSuccess)
                s = fail(GS_ERR_CUDA, "cudaEventRecord");
        }
        for (size_t i = 1; i < P && s == GS_OK; ++i)
            if (cudaStreamWaitEvent(st0, ev[P + i], 0) != cudaSuccess)
                s = fail(GS_ERR_CUDA, "cudaStreamWaitEvent");
        if (capturing) {
            const cudaError_t e = cudaStreamEndCapture(st0, &graph_h);
            if (s == GS_OK && e != cudaSuccess) s = cuda_fail(e, "cudaStreamEndCapture");
        }
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        if (s == GS_OK) {
            const cudaError_t ei = cudaGraphInstantiate(&b0->io_exec, graph_h, 0);
            if (ei != cudaSuccess) {
                b0->io_exec = nullptr;
                s = cuda_fail(ei, "cudaGraphInstantiate");
            }
        }
        if (graph_h) cudaGraphDestroy(graph_h);
        if (s != GS_OK) return s;
        b0->io_key = key;
    }
    GS_CUDA(cudaGraphLaunch(b0->io_exec, st0));
    return GS_OK;
}

gs_status gs_batches_step_host(const gs_batch* parts, unsigned n_parts, const gs_step_params* p,
                               unsigned steps, const gs_agent_arrays* in,
                               const gs_agent_arrays* out) {
    if (!parts || !p || !in || !out || n_parts == 0)
        return fail(GS_ERR_INVALID_ARG, "null argument");
    for (unsigned i = 0; i < n_parts; ++i) {
        if (!parts[i]) return fail(GS_ERR_INVALID_ARG, "null batch");
        for (unsigned j = 0; j < i; ++j)
            if (parts[j] == parts[i] || parts[j]->g->stream == parts[i]->g->stream)
                return fail(GS_ERR_INVALID_ARG, "every part needs a batch and a stream of its own");
    }
    // When out is in, the constants no step changes are already in place on
    // the host and are not copied back.
    const bool in_place = out->max_speed == in->max_speed && out->max_force == in->max_force &&
                          out->radius == in->radius && out->mass == in->mass;
    const bool pinned = host_pinned(*in) && host_pinned(*out);
    std::vector<IoPart> plan(n_parts);
    bool graph = pinned && steps > 0;
    size_t off = 0;
    for (unsigned i = 0; i < n_parts; ++i) {
        IoPart& q = plan[i];
        q.b = parts[i];
        q.hi = host_at(*in, off);
        q.ho = host_at(*out, off);
        off += q.b->total;
        GS_TRY(batch_prepare(q.b, p, q.d, q.grid, q.Ct, q.w));
        gs_group g = q.b->g;
        graph = graph && g->knn_cap != 0 && !g->profiling && g->use_graph &&
                g->stream != cudaStreamLegacy && g->stream != nullptr;
    }
    if (graph) {
        for (IoPart& q : plan) {
            gs_group g = q.b->g;
            g->n = q.b->total;
            q.d.enum_cap = g->knn_cap;
            fill_launch(g, q.d, q.w, q.L);
        }
        GS_TRY(io_graph(plan, steps, in_place));
        // the result is in the reference arrays and, with the step's buckets, in A
        for (IoPart& q : plan) {
            gs_group g = q.b->g;
            g->fused_current = false;
            g->accum_dirty = false;
            g->db.valid = false;
            g->auto_cap_valid = false;
            g->fdb.grid = q.grid;
            g->fdb.valid = true;
            g->pending_wrap = q.d.wrap_mode;
            g->frame_cells = q.Ct;
        }
    } else {
        // call by call: each part's upload, steps and download on its stream
        for (IoPart& q : plan) {
            GS_TRY(gs_group_upload(q.b->g, &q.hi, q.b->total));
            if (steps) GS_TRY(fused_run(q.b->g, q.d, q.grid, q.Ct, q.b->agent_scene, q.w, steps));
            GS_TRY(download_enqueue(q.b->g, &q.ho, in_place));
        }
    }
    gs_status s = GS_OK;
    for (unsigned i = 0; i < n_parts; ++i) {
        const cudaError_t e = cudaStreamSynchronize(parts[i]->g->stream);
        if (e != cudaSuccess && s == GS_OK) s = cuda_fail(e, "batches step");
    }
    for (unsigned i = 0; i < n_parts && s == GS_OK; ++i) s = check_device_flags(parts[i]->g);
    return s;
}

// ExtractData of the last gs_batch_step's frame for every scene, from the
// step's own buckets: cells scene after scene (scene s at s * cells).
static gs_status batch_frame(gs_batch b, unsigned& Ct) {
    if (!b) return fail(GS_ERR_INVALID_ARG, "null batch");
    Ct = b->cells * unsigned(b->scenes.size());
    if (b->g->frame_cells == 0 || b->g->frame_cells != Ct)
        return fail(GS_ERR_STATE, "run gs_batch_step first");
    return GS_OK;
}

gs_status gs_batch_cell_density(gs_batch b, unsigned* counts) {
    unsigned Ct = 0;
    GS_TRY(batch_frame(b, Ct));
    if (!counts) return fail(GS_ERR_INVALID_ARG, "null output");
    gs_group g = b->g;
    void* d = nullptr;
    GS_TRY(diag_scratch(g, size_t(Ct) * 4, &d));
    const gs_status s =
        launch_frame_cell_density(g->fdb.start, g->fdb.live, Ct, static_cast<unsigned*>(d),
                                  g->stream);
    return diag_copy_out(g, counts, d, size_t(Ct) * 4, s);
}

gs_status gs_batch_cell_avg_velocity(gs_batch b, float* avg3) {
    unsigned Ct = 0;
    GS_TRY(batch_frame(b, Ct));
    if (!avg3) return fail(GS_ERR_INVALID_ARG, "null output");
    gs_group g = b->g;
    void* d = nullptr;
    GS_TRY(diag_scratch(g, size_t(Ct) * 12, &d));
    const gs_status s =
        launch_frame_cell_avg_velocity(g->fdb.start, g->fdb.live, Ct, g->A.f[0], g->A.f[1],
                                       static_cast<float3*>(d), g->stream);
    return diag_copy_out(g, avg3, d, size_t(Ct) * 12, s);
}

// gs_batch_step's checks and set-up (buffers, walls, scene table), without
// launching: the step parameters d, grid, cells over all scenes and walls.
static gs_status batch_prepare(gs_batch b, const gs_step_params* p, StepDev& d, Grid& grid,
                               unsigned& Ct, WallsDev& w) {
    GS_TRY(validate_step(p, nullptr, d));
    unsigned C;
    GS_TRY(check_grid(p->world_cells, p->world_size, grid, C));
    if (std::memcmp(&grid, &b->grid, sizeof(Grid)) != 0)
        return fail(GS_ERR_INVALID_ARG, "step grid differs from the batch grid");
    if (d.r != b->radius) return fail(GS_ERR_INVALID_ARG, "search radius differs from the batch");
    gs_group g = b->g;
    const unsigned S = unsigned(b->scenes.size());
    Ct = b->cells * S;
    const bool has_walls = d.need & NEED_WALLS;
    GS_TRY(reserve_fused(g, Ct, has_walls, d.k, S));
    if (has_walls) GS_TRY(batch_walls(b));
    std::vector<Scene> scenes = b->scenes;
    if (!has_walls)
        for (Scene& sc : scenes) sc.n_walls = 0;
    GS_TRY(put_scenes(g, scenes));
    d.block = g->block;
    w = WallsDev();
    if (has_walls) {
        w.start = b->w_start;
        w.end = b->w_end;
        w.normal = b->w_normal;
        w.pos_id = b->w_pos_id;
        w.cell_start = b->w_cell_start;
    }
    return GS_OK;
}

gs_status gs_batch_step(gs_batch b, const gs_step_params* p, unsigned steps) {
    if (!b) return fail(GS_ERR_INVALID_ARG, "null batch");
    StepDev d;
    Grid grid;
    unsigned Ct = 0;
    WallsDev w;
    GS_TRY(batch_prepare(b, p, d, grid, Ct, w));
    if (steps == 0) return GS_OK;
    return fused_run(b->g, d, grid, Ct, b->agent_scene, w, steps);
}

}  // extern "C"

// ---- differentiable rollouts: checkpointed forward, adjoint backward ----------------
struct gs_rollout_s {
    gs_group g = nullptr;
    gs_bins bins = nullptr;
    unsigned steps = 0, every = 0, n_seg = 0, cap = 0, k = 0;
    unsigned n = 0;           // agents at the last forward pass
    bool have_forward = false;
    gs_step_params params{};  // of the last forward pass
    // checkpoints [n_seg + 1][cap]: the state at the start of each segment, then the final state
    float4 *ck_pos = nullptr, *ck_dir = nullptr;
    float* ck_speed = nullptr;
    float3 *ck_side = nullptr, *ck_up = nullptr;
    // one segment's step records: [every][cap] and [every][cap * k]
    float4 *rec_pos = nullptr, *rec_dir = nullptr;
    unsigned* rec_knn = nullptr;
    // adjoint state, ping-pong: d loss / d (position, velocity)
    float4 *lp[2] = {nullptr, nullptr}, *lv[2] = {nullptr, nullptr};
    float* wpart = nullptr;  // [adjoint_blocks(cap) * 4]
    unsigned char* adj_scratch = nullptr;  // adjoint_scratch_bytes(cap, k)
};

static void rollout_release(gs_rollout r) {
    dfree(r->ck_pos);
    dfree(r->ck_dir);
    dfree(r->ck_speed);
    dfree(r->ck_side);
    dfree(r->ck_up);
    dfree(r->rec_pos);
    dfree(r->rec_dir);
    dfree(r->rec_knn);
    for (int i = 0; i < 2; ++i) {
        dfree(r->lp[i]);
        dfree(r->lv[i]);
    }
    dfree(r->wpart);
    dfree(r->adj_scratch);
}

gs_status gs_rollout_create(gs_group g, gs_bins bins, unsigned steps, unsigned checkpoint_every,
                            gs_rollout* out) {
    if (!g || !bins || !out) return fail(GS_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    if (steps == 0 || checkpoint_every == 0)
        return fail(GS_ERR_INVALID_ARG, "steps and checkpoint interval must be positive");
    if (g->k > 32) return fail(GS_ERR_INVALID_ARG, "rollouts need k <= 32");
    gs_rollout r = new (std::nothrow) gs_rollout_s();
    if (!r) return fail(GS_ERR_OOM, "host allocation failed");
    r->g = g;
    r->bins = bins;
    r->steps = steps;
    r->every = std::min(checkpoint_every, steps);
    r->n_seg = (steps + r->every - 1) / r->every;
    r->cap = g->capacity;
    r->k = g->k;
    const size_t cap = r->cap, nck = size_t(r->n_seg) + 1;
    gs_status s = dalloc(&r->ck_pos, nck * cap);
    if (s == GS_OK) s = dalloc(&r->ck_dir, nck * cap);
    if (s == GS_OK) s = dalloc(&r->ck_speed, nck * cap);
    if (s == GS_OK) s = dalloc(&r->ck_side, nck * cap);
    if (s == GS_OK) s = dalloc(&r->ck_up, nck * cap);
    if (s == GS_OK) s = dalloc(&r->rec_pos, size_t(r->every) * cap);
    if (s == GS_OK) s = dalloc(&r->rec_dir, size_t(r->every) * cap);
    if (s == GS_OK) s = dalloc(&r->rec_knn, size_t(r->every) * cap * r->k);
    for (int i = 0; i < 2 && s == GS_OK; ++i) {
        s = dalloc(&r->lp[i], cap);
        if (s == GS_OK) s = dalloc(&r->lv[i], cap);
    }
    if (s == GS_OK) s = dalloc(&r->wpart, size_t(adjoint_blocks(r->cap)) * 4);
    if (s == GS_OK) s = dalloc(&r->adj_scratch, adjoint_scratch_bytes(r->cap, r->k));
    if (s != GS_OK) {
        rollout_release(r);
        delete r;
        return s;
    }
    *out = r;
    return GS_OK;
}

gs_status gs_rollout_destroy(gs_rollout r) {
    if (!r) return GS_OK;
    if (r->g) cudaStreamSynchronize(r->g->stream);
    rollout_release(r);
    delete r;
    return GS_OK;
}

// Checks that p is a walls-free flock the adjoint covers and fills d, grid, C.
static gs_status rollout_params(gs_rollout r, const gs_step_params* p, StepDev& d, Grid& grid,
                                unsigned& C) {
    GS_TRY(validate_step(p, nullptr, d));
    if (d.need & ~(NEED_SEP | NEED_ALI | NEED_COH))
        return fail(GS_ERR_UNSUPPORTED,
                    "differentiable rollouts cover separation, alignment and cohesion");
    for (unsigned o = 0; o < p->n_order; ++o)
        if (p->order[o] == GS_B_SEEK)
            return fail(GS_ERR_UNSUPPORTED,
                        "differentiable rollouts cover separation, alignment and cohesion");
    if (p->k != r->k) return fail(GS_ERR_INVALID_ARG, "k differs from the group's");
    GS_TRY(check_grid(p->world_cells, p->world_size, grid, C));
    if (C != r->bins->cells || std::memcmp(&grid, &r->bins->grid, sizeof(Grid)) != 0)
        return fail(GS_ERR_INVALID_ARG, "step grid differs from the bins");
    return GS_OK;
}

// Copies the group's time-varying state (reference layout) to checkpoint c.
static gs_status rollout_save(gs_rollout r, unsigned c) {
    gs_group g = r->g;
    const size_t n = r->n, off = size_t(c) * r->cap;
    cudaStream_t st = g->stream;
    GS_TRY(ensure_reference(g));
    GS_CUDA(cudaMemcpyAsync(r->ck_pos + off, g->position, n * 16, cudaMemcpyDeviceToDevice, st));
    GS_CUDA(cudaMemcpyAsync(r->ck_dir + off, g->direction, n * 16, cudaMemcpyDeviceToDevice, st));
    GS_CUDA(cudaMemcpyAsync(r->ck_speed + off, g->speed, n * 4, cudaMemcpyDeviceToDevice, st));
    GS_CUDA(cudaMemcpyAsync(r->ck_side + off, g->side, n * 12, cudaMemcpyDeviceToDevice, st));
    GS_CUDA(cudaMemcpyAsync(r->ck_up + off, g->up, n * 12, cudaMemcpyDeviceToDevice, st));
    return GS_OK;
}

// Puts checkpoint c back into the group, with steering and applied bits cleared.
static gs_status rollout_restore(gs_rollout r, unsigned c) {
    gs_group g = r->g;
    const size_t n = r->n, off = size_t(c) * r->cap;
    cudaStream_t st = g->stream;
    GS_CUDA(cudaMemcpyAsync(g->position, r->ck_pos + off, n * 16, cudaMemcpyDeviceToDevice, st));
    GS_CUDA(cudaMemcpyAsync(g->direction, r->ck_dir + off, n * 16, cudaMemcpyDeviceToDevice, st));
    GS_CUDA(cudaMemcpyAsync(g->speed, r->ck_speed + off, n * 4, cudaMemcpyDeviceToDevice, st));
    GS_CUDA(cudaMemcpyAsync(g->side, r->ck_side + off, n * 12, cudaMemcpyDeviceToDevice, st));
    GS_CUDA(cudaMemcpyAsync(g->up, r->ck_up + off, n * 12, cudaMemcpyDeviceToDevice, st));
    GS_CUDA(cudaMemsetAsync(g->steering, 0, n * 16, st));
    GS_CUDA(cudaMemsetAsync(g->applied, 0, n * 4, st));
    g->fused_current = false;
    g->frame_cells = 0;
    g->accum_dirty = false;
    g->db.valid = false;
    return GS_OK;
}

gs_status gs_rollout_forward(gs_rollout r, const gs_step_params* p) {
    if (!r) return fail(GS_ERR_INVALID_ARG, "null rollout");
    gs_group g = r->g;
    StepDev d;
    Grid grid;
    unsigned C;
    GS_TRY(rollout_params(r, p, d, grid, C));
    r->have_forward = false;
    r->n = g->n;
    r->params = *p;
    if (g->n == 0) {
        r->have_forward = true;
        return GS_OK;
    }
    // the rollout starts from zero steering and applied bits
    GS_TRY(ensure_reference(g));
    GS_CUDA(cudaMemsetAsync(g->steering, 0, size_t(g->n) * 16, g->stream));
    GS_CUDA(cudaMemsetAsync(g->applied, 0, size_t(g->n) * 4, g->stream));
    g->fused_current = false;
    g->frame_cells = 0;
    g->accum_dirty = false;
    GS_TRY(rollout_save(r, 0));
    for (unsigned c = 0; c < r->n_seg; ++c) {
        const unsigned len = std::min(r->every, r->steps - c * r->every);
        GS_TRY(gs_step(g, r->bins, nullptr, p, len));
        GS_TRY(rollout_save(r, c + 1));
    }
    r->have_forward = true;
    return GS_OK;
}

// Re-runs segment c from its checkpoint, recording every step's inputs.
static gs_status rollout_record(gs_rollout r, unsigned c, StepDev d, const Grid& grid,
                                unsigned C, unsigned len) {
    gs_group g = r->g;
    GS_TRY(rollout_restore(r, c));
    GS_TRY(reserve_fused(g, C, false, d.k, 1));
    Scene sc{};
    sc.grid = grid;
    sc.n_agents = g->n;
    GS_TRY(put_scenes(g, std::vector<Scene>{sc}));
    d.block = g->block;
    FusedLaunch L;
    bool dirty = false, fresh = false;
    GS_TRY(fused_setup(g, d, grid, C, nullptr, WallsDev{}, L, dirty, fresh));
    d.dirty = 0;
    for (unsigned j = 0; j < len; ++j) {
        d.fresh = fresh && j == 0 ? 1u : 0u;
        FusedLaunch Lj = L;
        Lj.rec_pos = r->rec_pos + size_t(j) * r->cap;
        Lj.rec_dir = r->rec_dir + size_t(j) * r->cap;
        Lj.rec_knn = r->rec_knn + size_t(j) * r->cap * r->k;
        GS_TRY(step_body(g, Lj, d, C, nullptr));
    }
    g->db.valid = false;
    return GS_OK;
}

gs_status gs_rollout_backward(gs_rollout r, const float* adj_position, const float* adj_velocity,
                              float* grad_position0, float* grad_velocity0,
                              float grad_weights[3]) {
    if (!r) return fail(GS_ERR_INVALID_ARG, "null rollout");
    if (!r->have_forward) return fail(GS_ERR_INVALID_ARG, "backward needs a forward pass first");
    gs_group g = r->g;
    if (g->n != r->n) return fail(GS_ERR_INVALID_ARG, "the group changed size since forward");
    StepDev d;
    Grid grid;
    unsigned C;
    GS_TRY(rollout_params(r, &r->params, d, grid, C));
    cudaStream_t st = g->stream;
    const size_t n = r->n;
    const unsigned nb = adjoint_blocks(r->cap);
    if (n == 0) {
        if (grad_weights) grad_weights[0] = grad_weights[1] = grad_weights[2] = 0.f;
        return GS_OK;
    }
    if (adj_position)
        GS_CUDA(cudaMemcpyAsync(r->lp[0], adj_position, n * 16, cudaMemcpyDeviceToDevice, st));
    else
        GS_CUDA(cudaMemsetAsync(r->lp[0], 0, n * 16, st));
    if (adj_velocity)
        GS_CUDA(cudaMemcpyAsync(r->lv[0], adj_velocity, n * 16, cudaMemcpyDeviceToDevice, st));
    else
        GS_CUDA(cudaMemsetAsync(r->lv[0], 0, n * 16, st));
    GS_CUDA(cudaMemsetAsync(r->lp[1], 0, n * 16, st));
    GS_CUDA(cudaMemsetAsync(r->lv[1], 0, n * 16, st));
    GS_CUDA(cudaMemsetAsync(r->wpart, 0, size_t(nb) * 16, st));
    int cur = 0;
    for (unsigned c = r->n_seg; c-- > 0;) {
        const unsigned len = std::min(r->every, r->steps - c * r->every);
        GS_TRY(rollout_record(r, c, d, grid, C, len));
        for (unsigned j = len; j-- > 0;) {
            AdjointLaunch A;
            A.pos = r->rec_pos + size_t(j) * r->cap;
            A.dir = r->rec_dir + size_t(j) * r->cap;
            A.knn = r->rec_knn + size_t(j) * r->cap * r->k;
            A.max_speed = g->max_speed;
            A.max_force = g->max_force;
            A.mass = g->mass;
            A.lp_in = r->lp[cur];
            A.lv_in = r->lv[cur];
            A.lp_out = r->lp[1 - cur];
            A.lv_out = r->lv[1 - cur];
            A.wpart = r->wpart;
            A.n = r->n;
            A.k = r->k;
            adjoint_scratch_bind(A, r->adj_scratch, r->n, r->k);
            GS_TRY(launch_flock_adjoint(A, d, st));
            cur = 1 - cur;
        }
    }
    if (grad_position0)
        GS_CUDA(cudaMemcpyAsync(grad_position0, r->lp[cur], n * 16, cudaMemcpyDeviceToDevice, st));
    if (grad_velocity0)
        GS_CUDA(cudaMemcpyAsync(grad_velocity0, r->lv[cur], n * 16, cudaMemcpyDeviceToDevice, st));
    std::vector<float> part(size_t(nb) * 4);
    GS_CUDA(cudaMemcpyAsync(part.data(), r->wpart, part.size() * 4, cudaMemcpyDeviceToHost, st));
    // leave the group at the rollout's final state
    GS_TRY(rollout_restore(r, r->n_seg));
    GS_CUDA(cudaStreamSynchronize(st));
    GS_TRY(check_device_flags(g));
    if (grad_weights) {
        for (int b = 0; b < 3; ++b) {
            double sum = 0.0;  // host-side sum of the per-block partials
            for (unsigned i = 0; i < nb; ++i) sum += part[size_t(i) * 4 + b];
            grad_weights[b] = float(sum);
        }
    }
    return GS_OK;
}

gs_status gs_flock_adjoint_step(const float* position_speed, const float* heading,
                                const unsigned* knn, unsigned n, unsigned k,
                                const float* max_speed, const float* max_force, const float* mass,
                                const gs_step_params* p, float* adj_position_out,
                                float* adj_velocity_out, float* adj_position_in,
                                float* adj_velocity_in, float* weight_partials,
                                unsigned partials_cap, void* stream) {
    StepDev d;
    GS_TRY(validate_step(p, nullptr, d));
    if (d.need & ~(NEED_SEP | NEED_ALI | NEED_COH))
        return fail(GS_ERR_UNSUPPORTED, "the adjoint covers separation, alignment and cohesion");
    if (k != p->k) return fail(GS_ERR_INVALID_ARG, "k differs from the parameters'");
    if (n == 0) return GS_OK;
    if (!position_speed || !heading || !knn || !max_speed || !max_force || !mass ||
        !adj_position_out || !adj_velocity_out || !adj_position_in || !adj_velocity_in ||
        !weight_partials)
        return fail(GS_ERR_INVALID_ARG, "null device array");
    if (partials_cap < adjoint_blocks(n) * 4)
        return fail(GS_ERR_INVALID_ARG, "weight partials need 4 * ceil(n / 256) floats");
    AdjointLaunch A;
    A.pos = reinterpret_cast<const float4*>(position_speed);
    A.dir = reinterpret_cast<const float4*>(heading);
    A.knn = knn;
    A.max_speed = max_speed;
    A.max_force = max_force;
    A.mass = mass;
    A.lp_in = reinterpret_cast<float4*>(adj_position_out);
    A.lv_in = reinterpret_cast<float4*>(adj_velocity_out);
    A.lp_out = reinterpret_cast<float4*>(adj_position_in);
    A.lv_out = reinterpret_cast<float4*>(adj_velocity_in);
    A.wpart = weight_partials;
    A.n = n;
    A.k = k;
    // the step's scratch is stream-ordered: allocated and freed on `stream`,
    // so calls on different streams never share it
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    void* scratch = nullptr;
    GS_CUDA(cudaMallocAsync(&scratch, adjoint_scratch_bytes(n, k), st));
    adjoint_scratch_bind(A, scratch, n, k);
    const gs_status s = launch_flock_adjoint(A, d, st);
    const cudaError_t e = cudaFreeAsync(scratch, st);
    if (s != GS_OK) return s;
    if (e != cudaSuccess) return cuda_fail(e, "cudaFreeAsync(adjoint scratch)");
    return GS_OK;
}
