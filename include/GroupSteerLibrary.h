/* GroupSteerLibrary.h - C++ drop-in for the reference's group objects and the
 * free functions of include/OpenSteer/CUDA/GroupSteerLibrary.cuh:43-223,
 * implemented over the C ABI in gpusteer.h (libgpusteer.so, sm_103a).
 *
 * A plugin that includes this header instead of the reference's keeps its
 * calls: the same class names and member functions it uses (AgentGroup,
 * AgentData, KNNData, KNNBinData, WallGroup, BaseGroup, bin_cell), the same
 * free-function signatures, the same KERNEL_*_BIT mask constants, all in
 * namespace OpenSteer.  Differences:
 *   - errors throw OpenSteer::GpuSteerError (the reference aborts through
 *     CUDA_SAFE_CALL);
 *   - the behaviours outside the GB300 path (flee, pursuit, evade, stay-on-
 *     path, obstacles) are not declared, so a plugin that calls them fails to
 *     compile rather than at run time;
 *   - WallGroup::SplitWalls takes the cell list of a KNNBinData made by this
 *     header (the split runs in the library, on that grid).
 * Every AgentGroup made here runs its work on the legacy default stream, as
 * the reference's kernels do, so a plugin's own CUDA calls on the pd*()
 * device pointers (a cudaMemset of the applied bits, a kernel of its own)
 * are ordered with the library's launches as they are in the reference.
 * Results are bit-identical to the reference kernels' restatement (oracle/). */
#ifndef GPUSTEER_GROUP_STEER_LIBRARY_H
#define GPUSTEER_GROUP_STEER_LIBRARY_H

#include <vector_types.h> /* float3, float4, uint3 (CUDA toolkit) */
#include <driver_types.h> /* cudaStreamLegacy */

#include <climits>
#include <cstddef>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "gpusteer.h"

namespace OpenSteer {

typedef unsigned int uint;
typedef unsigned int id_type;

/* Kernel bit masks (CUDAKernelGlobals.cuh:11-31). */
static uint const KERNEL_PURSUE_BIT = 1;
static uint const KERNEL_EVADE_BIT = 1 << 1;
static uint const KERNEL_SEEK_BIT = 1 << 2;
static uint const KERNEL_FLEE_BIT = 1 << 3;
static uint const KERNEL_SEPARATION_BIT = 1 << 4;
static uint const KERNEL_ALIGNMENT_BIT = 1 << 5;
static uint const KERNEL_COHESION_BIT = 1 << 6;
static uint const KERNEL_AVOID_OBSTACLES_BIT = 1 << 7;
static uint const KERNEL_AVOID_WALLS_BIT = 1 << 8;
static uint const KERNEL_AVOID_NEIGHBORS_BIT = 1 << 9;
static uint const KERNEL_AVOID_CLOSE_NEIGHBORS_BIT = 1 << 10;
static uint const KERNEL_FOLLOW_PATH_BIT = 1 << 11;
static uint const KERNEL_ANTI_PENETRATION_WALL = 1 << 12;
static uint const KERNEL_ANTI_PENETRATION_AGENT = 1 << 13;
static uint const KERNEL_ALL_BIT = UINT_MAX;

class GpuSteerError : public std::runtime_error {
public:
    GpuSteerError(gs_status s, std::string const& what)
        : std::runtime_error(what), status(s) {}
    gs_status status;
};

inline void gsCheck(gs_status s) {
    if (s != GS_OK) {
        char const* m = gs_last_error();
        throw GpuSteerError(s, std::string(gs_status_string(s)) + ": " + (m ? m : ""));
    }
}

/* One agent (AgentData.h: agent_data). */
struct AgentData {
    id_type id;
    float3 side;
    float3 up;
    float4 direction;
    float4 position;
    float4 steering;
    float speed;
    float maxSpeed;
    float maxForce;
    float radius;
    float mass;
    uint appliedKernels;
};

/* One spatial cell (KNNBinDataGlobals.cuh: bin_cell). */
struct bin_cell {
    size_t index;
    float3 position;
    float3 minBound;
    float3 maxBound;
};

/* ---- KNNBinData (KNNBinDataV2.cuh:18-63) -------------------------------------------- */
class KNNBinData {
public:
    KNNBinData(uint3 const& worldCells, float3 const& worldSize, uint const searchRadius)
        : m_worldCells(worldCells), m_worldSize(worldSize), m_radius(searchRadius) {
        unsigned const wc[3] = {worldCells.x, worldCells.y, worldCells.z};
        float const ws[3] = {worldSize.x, worldSize.y, worldSize.z};
        gsCheck(gs_bins_create(wc, ws, searchRadius, &m_bins));
        gsCheck(gs_bins_num_cells(m_bins, &m_nCells));
    }
    ~KNNBinData() {
        unregisterCells();
        gs_bins_destroy(m_bins);
    }
    KNNBinData(KNNBinData const&) = delete;
    KNNBinData& operator=(KNNBinData const&) = delete;

    uint radius() const { return m_radius; }
    uint3 const& WorldCells() const { return m_worldCells; }
    float3 const& WorldSize() const { return m_worldSize; }
    uint getNumCells() const { return m_nCells; }
    bool is3D() const { return m_worldCells.y > 1; }

    /* The cells' bounds and centres, read from the library once. */
    std::vector<bin_cell> const& hvCells() const {
        if (m_cells.empty() && m_nCells) {
            std::vector<float> mn(size_t(m_nCells) * 3), mx(mn.size()), ct(mn.size());
            gsCheck(gs_bins_get_cells(m_bins, mn.data(), mx.data(), ct.data(), m_nCells));
            m_cells.resize(m_nCells);
            for (size_t i = 0; i < m_cells.size(); ++i) {
                m_cells[i].index = i;
                m_cells[i].position = make3(&ct[3 * i]);
                m_cells[i].minBound = make3(&mn[3 * i]);
                m_cells[i].maxBound = make3(&mx[3 * i]);
            }
            std::lock_guard<std::mutex> lock(registryMutex());
            registry()[&m_cells] = m_bins;
        }
        return m_cells;
    }

    gs_bins handle() const { return m_bins; }

    /* The bins whose hvCells() returned `cells` (for WallGroup::SplitWalls). */
    static gs_bins binsOfCells(std::vector<bin_cell> const& cells) {
        std::lock_guard<std::mutex> lock(registryMutex());
        auto it = registry().find(&cells);
        return it == registry().end() ? nullptr : it->second;
    }

private:
    static float3 make3(float const* v) {
        float3 r;
        r.x = v[0];
        r.y = v[1];
        r.z = v[2];
        return r;
    }
    static std::map<void const*, gs_bins>& registry() {
        static std::map<void const*, gs_bins> r;
        return r;
    }
    static std::mutex& registryMutex() {
        static std::mutex m;
        return m;
    }
    void unregisterCells() {
        std::lock_guard<std::mutex> lock(registryMutex());
        registry().erase(&m_cells);
    }

    uint3 m_worldCells;
    float3 m_worldSize;
    uint m_radius;
    uint m_nCells = 0;
    gs_bins m_bins = nullptr;
    mutable std::vector<bin_cell> m_cells;
};
typedef KNNBinData KNNBinDataV2;

/* ---- KNNData (KNNData.cuh:10-55) ---------------------------------------------------- */
class KNNData {
public:
    KNNData(uint const nSize, uint const nK) : m_nSize(nSize), m_nK(nK) {
        gsCheck(gs_knn_create(nSize, nK, &m_knn));
    }
    ~KNNData() { gs_knn_destroy(m_knn); }
    KNNData(KNNData const&) = delete;
    KNNData& operator=(KNNData const&) = delete;

    uint* pdKNNIndices() {
        unsigned* idx = nullptr;
        float* dist = nullptr;
        gsCheck(gs_knn_device_arrays(m_knn, &idx, &dist));
        return idx;
    }
    float* pdKNNDistances() {
        unsigned* idx = nullptr;
        float* dist = nullptr;
        gsCheck(gs_knn_device_arrays(m_knn, &idx, &dist));
        return dist;
    }
    /* Column-major idx[a + i * size()], as the reference stores them. */
    std::vector<uint> const& hvKNNIndices() const {
        syncHost();
        return m_hvIdx;
    }
    std::vector<float> const& hvKNNDistances() const {
        syncHost();
        return m_hvDist;
    }
    uint k() const { return m_nK; }
    uint size() const { return m_nSize; }
    void setSyncHost() { m_bSyncHost = true; }
    /* Marks the lists as written on `g`'s stream (host copy stale). */
    void setSyncHost(gs_group g) {
        m_writer = g;
        m_bSyncHost = true;
    }
    gs_knn handle() const { return m_knn; }

private:
    void syncHost() const {
        if (!m_bSyncHost) return;
        m_hvIdx.resize(size_t(m_nSize) * m_nK);
        m_hvDist.resize(m_hvIdx.size());
        gsCheck(gs_knn_download(m_knn, m_writer, m_hvIdx.data(), m_hvDist.data()));
        m_bSyncHost = false;
    }

    uint m_nSize, m_nK;
    gs_knn m_knn = nullptr;
    gs_group m_writer = nullptr;
    mutable bool m_bSyncHost = true;
    mutable std::vector<uint> m_hvIdx;
    mutable std::vector<float> m_hvDist;
};

/* ---- BaseGroup (BaseGroup.h:8-33) --------------------------------------------------- */
class BaseGroup {
public:
    virtual ~BaseGroup() {}
    virtual uint const& Size() const = 0;
    virtual float4* pdPosition() = 0;
    virtual float4* pdDirection() = 0;
    virtual float* pdSpeed() = 0;
    virtual float* pdRadius() = 0;
    virtual void SetSyncHost() = 0;
    /* The library handles behind the group (one of them is null). */
    virtual gs_group gsGroup() { return nullptr; }
    virtual gs_walls gsWalls() { return nullptr; }
};

/* ---- AgentGroupData / AgentGroup (AgentGroupData.cuh:19-297, AgentGroup.h:12-56) --- */
class AgentGroup;

/* Device pointers of a group's arrays in the reference layout.  Writing
 * through them is allowed (the library then treats the arrays as modified). */
class AgentGroupData {
public:
    explicit AgentGroupData(AgentGroup* g) : m_group(g) {}
    float4* pdPosition() { return reinterpret_cast<float4*>(arrays().position); }
    float4* pdDirection() { return reinterpret_cast<float4*>(arrays().direction); }
    float4* pdSteering() { return reinterpret_cast<float4*>(arrays().steering); }
    float3* pdSide() { return reinterpret_cast<float3*>(arrays().side); }
    float3* pdUp() { return reinterpret_cast<float3*>(arrays().up); }
    float* pdSpeed() { return arrays().speed; }
    float* pdMaxSpeed() { return arrays().max_speed; }
    float* pdMaxForce() { return arrays().max_force; }
    float* pdRadius() { return arrays().radius; }
    float* pdMass() { return arrays().mass; }
    uint* pdAppliedKernels() { return arrays().applied; }
    uint size() const;

private:
    gs_agent_arrays arrays();
    AgentGroup* m_group;
};

class AgentGroup : public BaseGroup {
public:
    AgentGroup(uint3 const& worldCells, uint const knn)
        : m_worldCells(worldCells), m_k(knn), m_data(this) {}
    virtual ~AgentGroup() {
        if (m_group) gs_group_destroy(m_group);
    }
    AgentGroup(AgentGroup const&) = delete;
    AgentGroup& operator=(AgentGroup const&) = delete;

    /* Appends an agent on the host (SyncDevice sends it); false if the id exists. */
    bool AddAgent(AgentData const& ad) {
        SyncHost();
        if (m_index.count(ad.id)) return false;
        m_index[ad.id] = m_nCount;
        m_hv.push_back(ad);
        ++m_nCount;
        m_bSyncDevice = true;
        return true;
    }
    void RemoveAgent(id_type const id) {
        SyncHost();
        auto it = m_index.find(id);
        if (it == m_index.end()) return;
        m_hv.erase(m_hv.begin() + it->second);
        RebuildIDToIndexMap();
        m_bSyncDevice = true;
    }
    void Clear() {
        m_hv.clear();
        m_index.clear();
        m_nCount = 0;
        m_bSyncHost = false;
        m_bSyncDevice = true;
    }
    bool GetDataForAgent(id_type const id, AgentData& ad) {
        SyncHost();
        auto it = m_index.find(id);
        if (it == m_index.end()) return false;
        ad = m_hv[it->second];
        return true;
    }
    int GetAgentIndex(id_type const id) const {
        auto it = m_index.find(id);
        return it == m_index.end() ? -1 : int(it->second);
    }

    /* Host -> device (AgentGroupData.cuh:227-250). */
    void SyncDevice() {
        if (!m_bSyncDevice) return;
        const size_t n = m_hv.size();
        if (!m_group || n > m_capacity) {
            size_t cap = m_capacity ? m_capacity : 1024;
            while (cap < n) cap *= 2;
            if (m_group) gs_group_destroy(m_group);
            m_group = nullptr;
            gsCheck(gs_group_create(m_k, unsigned(cap), cudaStreamLegacy, &m_group));
            m_capacity = cap;
        }
        std::vector<float> pos(4 * n), dir(4 * n), steer(4 * n), side(3 * n), up(3 * n);
        std::vector<float> speed(n), maxs(n), maxf(n), rad(n), mass(n);
        std::vector<unsigned> applied(n);
        for (size_t i = 0; i < n; ++i) {
            AgentData const& a = m_hv[i];
            put4(&pos[4 * i], a.position);
            put4(&dir[4 * i], a.direction);
            put4(&steer[4 * i], a.steering);
            put3(&side[3 * i], a.side);
            put3(&up[3 * i], a.up);
            speed[i] = a.speed;
            maxs[i] = a.maxSpeed;
            maxf[i] = a.maxForce;
            rad[i] = a.radius;
            mass[i] = a.mass;
            applied[i] = a.appliedKernels;
        }
        gs_agent_arrays h = {pos.data(), dir.data(), steer.data(), side.data(), up.data(),
                             speed.data(), maxs.data(), maxf.data(), rad.data(), mass.data(),
                             applied.data()};
        gsCheck(gs_group_upload(m_group, &h, unsigned(n)));
        gsCheck(gs_group_synchronize(m_group));
        m_bSyncDevice = false;
    }
    /* Device -> host (AgentGroupData.cuh:177-225), when the device copy is newer. */
    void SyncHost() {
        if (!m_bSyncHost || !m_group) return;
        const size_t n = m_hv.size();
        std::vector<float> pos(4 * n), dir(4 * n), steer(4 * n), side(3 * n), up(3 * n);
        std::vector<float> speed(n), maxs(n), maxf(n), rad(n), mass(n);
        std::vector<unsigned> applied(n);
        gs_agent_arrays h = {pos.data(), dir.data(), steer.data(), side.data(), up.data(),
                             speed.data(), maxs.data(), maxf.data(), rad.data(), mass.data(),
                             applied.data()};
        gsCheck(gs_group_download(m_group, &h));
        for (size_t i = 0; i < n; ++i) {
            AgentData& a = m_hv[i];
            a.position = get4(&pos[4 * i]);
            a.direction = get4(&dir[4 * i]);
            a.steering = get4(&steer[4 * i]);
            a.side = get3(&side[3 * i]);
            a.up = get3(&up[3 * i]);
            a.speed = speed[i];
            a.maxSpeed = maxs[i];
            a.maxForce = maxf[i];
            a.radius = rad[i];
            a.mass = mass[i];
            a.appliedKernels = applied[i];
        }
        m_bSyncHost = false;
    }

    virtual void SetSyncHost() { m_bSyncHost = true; }
    virtual uint const& Size() const { return m_nCount; }
    AgentGroupData& GetAgentGroupData() { return m_data; }
    virtual float4* pdPosition() { return m_data.pdPosition(); }
    virtual float4* pdDirection() { return m_data.pdDirection(); }
    virtual float* pdSpeed() { return m_data.pdSpeed(); }
    virtual float* pdRadius() { return m_data.pdRadius(); }
    uint3 const& WorldCells() const { return m_worldCells; }

    /* The device group, brought up to date with the host first. */
    virtual gs_group gsGroup() {
        SyncDevice();
        return m_group;
    }

private:
    friend class AgentGroupData;
    void RebuildIDToIndexMap() {
        m_index.clear();
        for (uint i = 0; i < m_hv.size(); ++i) m_index[m_hv[i].id] = i;
        m_nCount = uint(m_hv.size());
    }
    static void put4(float* d, float4 const& v) {
        d[0] = v.x;
        d[1] = v.y;
        d[2] = v.z;
        d[3] = v.w;
    }
    static void put3(float* d, float3 const& v) {
        d[0] = v.x;
        d[1] = v.y;
        d[2] = v.z;
    }
    static float4 get4(float const* s) {
        float4 v;
        v.x = s[0];
        v.y = s[1];
        v.z = s[2];
        v.w = s[3];
        return v;
    }
    static float3 get3(float const* s) {
        float3 v;
        v.x = s[0];
        v.y = s[1];
        v.z = s[2];
        return v;
    }

    uint3 m_worldCells;
    uint m_k;
    uint m_nCount = 0;
    size_t m_capacity = 0;
    gs_group m_group = nullptr;
    bool m_bSyncHost = false, m_bSyncDevice = true;
    std::vector<AgentData> m_hv;
    std::map<id_type, uint> m_index;
    AgentGroupData m_data;
};

inline gs_agent_arrays AgentGroupData::arrays() {
    gs_agent_arrays d;
    std::memset(&d, 0, sizeof(d));
    gsCheck(gs_group_device_arrays(m_group->gsGroup(), &d));
    m_group->SetSyncHost();  /* the caller may write through the pointers */
    return d;
}
inline uint AgentGroupData::size() const { return m_group->Size(); }

/* ---- WallGroup (WallGroup.h:12-37, WallGroupData.cu:73-206) ------------------------- */
class WallGroup : public BaseGroup {
public:
    WallGroup(uint3 const& worldCells, uint const knw) : m_worldCells(worldCells), m_knw(knw) {}
    ~WallGroup() {
        if (m_walls) gs_walls_destroy(m_walls);
    }
    WallGroup(WallGroup const&) = delete;
    WallGroup& operator=(WallGroup const&) = delete;

    /* .map file: start, end, normal (9 floats) per segment. */
    bool LoadFromFile(char const* szFilename) {
        std::ifstream in(szFilename);
        if (!in) return false;
        m_start.clear();
        m_end.clear();
        m_normal.clear();
        float v[9];
        while (true) {
            int i = 0;
            for (; i < 9 && (in >> v[i]); ++i) {
            }
            if (i < 9) break;
            m_start.insert(m_start.end(), {v[0], v[1], v[2], 0.f});
            m_end.insert(m_end.end(), {v[3], v[4], v[5], 0.f});
            m_normal.insert(m_normal.end(), {v[6], v[7], v[8], 0.f});
        }
        return !m_start.empty();
    }
    /* Split at the cells of a KNNBinData from this header (its hvCells()). */
    void SplitWalls(std::vector<bin_cell> const& cells) {
        m_bins = KNNBinData::binsOfCells(cells);
        if (!m_bins) throw GpuSteerError(GS_ERR_INVALID_ARG, "SplitWalls: unknown cell list");
    }
    /* Splits (on the SplitWalls grid) and uploads. */
    void SyncDevice() {
        if (!m_bins) throw GpuSteerError(GS_ERR_STATE, "SyncDevice before SplitWalls");
        if (m_walls) gs_walls_destroy(m_walls);
        m_walls = nullptr;
        gsCheck(gs_walls_create(m_start.data(), m_end.data(), m_normal.data(),
                                unsigned(m_start.size() / 4), m_bins, m_knw, &m_walls));
        gsCheck(gs_walls_size(m_walls, &m_nCount));
    }
    virtual uint const& Size() const { return m_nCount; }
    virtual float4* pdPosition() { return nullptr; }
    virtual float4* pdDirection() { return nullptr; }
    virtual float* pdSpeed() { return nullptr; }
    virtual float* pdRadius() { return nullptr; }
    virtual void SetSyncHost() {}
    virtual gs_walls gsWalls() { return m_walls; }
    uint knw() const { return m_knw; }

private:
    uint3 m_worldCells;
    uint m_knw;
    uint m_nCount = 0;
    gs_bins m_bins = nullptr;
    gs_walls m_walls = nullptr;
    std::vector<float> m_start, m_end, m_normal;
};

/* ---- PolylinePathwayCUDA (PolylinePathwayCUDA.cuh) ---------------------------------- */
class PolylinePathwayCUDA {
public:
    PolylinePathwayCUDA(std::vector<float3> const& points, float const radius, bool const cyclic)
        : m_points(points), m_radius(radius), m_cyclic(cyclic) {
        std::vector<float> p3(points.size() * 3);
        for (size_t i = 0; i < points.size(); ++i) {
            p3[3 * i] = points[i].x;
            p3[3 * i + 1] = points[i].y;
            p3[3 * i + 2] = points[i].z;
        }
        gsCheck(gs_path_create(p3.data(), unsigned(points.size()), radius, cyclic ? 1 : 0,
                               &m_path));
    }
    ~PolylinePathwayCUDA() { gs_path_destroy(m_path); }
    PolylinePathwayCUDA(PolylinePathwayCUDA const&) = delete;
    PolylinePathwayCUDA& operator=(PolylinePathwayCUDA const&) = delete;

    /* The points as given (a cyclic path's closing point is not repeated). */
    std::vector<float3> const& hvPoints() const { return m_points; }
    float radius() const { return m_radius; }
    bool cyclic() const { return m_cyclic; }
    gs_path handle() const { return m_path; }

private:
    std::vector<float3> m_points;
    float m_radius;
    bool m_cyclic;
    gs_path m_path = nullptr;
};

/* ---- the free functions (GroupSteerLibrary.cuh:43-223) ------------------------------ */
namespace detail {
inline gs_group group(AgentGroup* g) {
    gs_group h = g->gsGroup();
    g->SetSyncHost();
    return h;
}
inline void f3(float3 const& v, float out[3]) {
    out[0] = v.x;
    out[1] = v.y;
    out[2] = v.z;
}
}  // namespace detail

/* GroupSteerLibrary.cuh:43 */
inline void wrapWorld(AgentGroup* pAgentGroup, float3 const& worldSize) {
    float ws[3];
    detail::f3(worldSize, ws);
    gsCheck(gs_wrap_world(detail::group(pAgentGroup), ws, GS_WRAP_REFERENCE));
}
/* :52 */
inline void steerForSeek(AgentGroup* pAgentGroup, float3 const& target, float const fWeight,
                         uint const doNotApplyWith) {
    float t[3];
    detail::f3(target, t);
    gsCheck(gs_steer_for_seek(detail::group(pAgentGroup), t, fWeight, doNotApplyWith));
}
/* :88 */
inline void steerToFollowPath(AgentGroup* pAgentGroup, PolylinePathwayCUDA* pPath,
                              float const predictionTime, float const fWeight,
                              uint const doNotApplyWith) {
    gsCheck(gs_steer_to_follow_path(detail::group(pAgentGroup), pPath->handle(), predictionTime,
                                    fWeight, doNotApplyWith));
}
/* :111 */
inline void steerToAvoidNeighbors(AgentGroup* pAgentGroup, KNNData* pKNNData,
                                  AgentGroup* pOtherGroup, const float fMinTimeToCollision,
                                  float const fMinSeparationDistance,
                                  bool const bAvoidCloseNeighbors, float const fWeight,
                                  uint const doNotApplyWith) {
    gsCheck(gs_steer_to_avoid_neighbors(detail::group(pAgentGroup), pKNNData->handle(),
                                        pOtherGroup->gsGroup(), fMinTimeToCollision,
                                        fMinSeparationDistance, bAvoidCloseNeighbors ? 1 : 0,
                                        fWeight, doNotApplyWith));
}
/* :120 */
inline void steerToAvoidWalls(AgentGroup* pAgentGroup, KNNData* pKNNData, WallGroup* pWallGroup,
                              float const fMinTimeToCollision, float const fWeight,
                              uint const doNotApplyWith) {
    gsCheck(gs_steer_to_avoid_walls(detail::group(pAgentGroup), pKNNData->handle(),
                                    pWallGroup->gsWalls(), fMinTimeToCollision, fWeight,
                                    doNotApplyWith));
}
/* :129 */
inline void updateKNNDatabase(BaseGroup* pGroup, KNNBinData* pKNNBinData) {
    if (gs_walls w = pGroup->gsWalls())
        gsCheck(gs_walls_update_knn_database(w, pKNNBinData->handle()));
    else
        gsCheck(gs_update_knn_database(pGroup->gsGroup(), pKNNBinData->handle()));
}
/* :138 */
inline void findKNearestNeighbors(AgentGroup* pAgentGroup, KNNData* pKNNData,
                                  KNNBinData* pKNNBinData, BaseGroup* pOtherGroup,
                                  uint const searchRadius) {
    gs_group g = detail::group(pAgentGroup);
    if (gs_walls w = pOtherGroup->gsWalls())
        gsCheck(gs_find_knn_walls(g, pKNNData->handle(), pKNNBinData->handle(), w, searchRadius));
    else
        gsCheck(gs_find_knn(g, pKNNData->handle(), pKNNBinData->handle(), pOtherGroup->gsGroup(),
                            searchRadius));
    pKNNData->setSyncHost(g);
}
/* KNNBruteForceCUDA.cu:163 (KNNBruteForceCUDAV2) */
inline void findKNearestNeighborsBruteForce(AgentGroup* pAgentGroup, KNNData* pKNNData,
                                            AgentGroup* pOtherGroup) {
    gs_group g = detail::group(pAgentGroup);
    gsCheck(gs_knn_bruteforce(g, pKNNData->handle(), pOtherGroup->gsGroup()));
    pKNNData->setSyncHost(g);
}
/* :161 */
inline void steerForSeparation(AgentGroup* pAgentGroup, KNNData* pKNNData, AgentGroup* pOtherGroup,
                               float const minDistance, float const maxDistance,
                               float const cosMaxAngle, float const fWeight,
                               uint const doNotApplyWith) {
    gsCheck(gs_steer_for_separation(detail::group(pAgentGroup), pKNNData->handle(),
                                    pOtherGroup->gsGroup(), minDistance, maxDistance, cosMaxAngle,
                                    fWeight, doNotApplyWith));
}
/* :170 */
inline void steerForAlignment(AgentGroup* pAgentGroup, KNNData* pKNNData, AgentGroup* pOtherGroup,
                              float const minDistance, float const maxDistance,
                              float const cosMaxAngle, float const fWeight,
                              uint const doNotApplyWith) {
    gsCheck(gs_steer_for_alignment(detail::group(pAgentGroup), pKNNData->handle(),
                                   pOtherGroup->gsGroup(), minDistance, maxDistance, cosMaxAngle,
                                   fWeight, doNotApplyWith));
}
/* :179 */
inline void steerForCohesion(AgentGroup* pAgentGroup, KNNData* pKNNData, AgentGroup* pOtherGroup,
                             float const minDistance, float const maxDistance,
                             float const cosMaxAngle, float const fWeight,
                             uint const doNotApplyWith) {
    gsCheck(gs_steer_for_cohesion(detail::group(pAgentGroup), pKNNData->handle(),
                                  pOtherGroup->gsGroup(), minDistance, maxDistance, cosMaxAngle,
                                  fWeight, doNotApplyWith));
}
/* :189 */
inline void updateGroup(AgentGroup* pAgentGroup, const float elapsedTime) {
    gsCheck(gs_update_group(detail::group(pAgentGroup), elapsedTime));
}
/* :198 (UpdateCUDAKernelNew.cu:95-268; the wall list is read row-major, as
 * that kernel reads it) */
inline void updateGroupWithAntiPenetration(AgentGroup* pAgentGroup, KNNData* pKNNData,
                                           WallGroup* pWallGroup, const float elapsedTime) {
    gsCheck(gs_update_group_with_antipenetration(detail::group(pAgentGroup), pKNNData->handle(),
                                                 pWallGroup->gsWalls(), elapsedTime));
}
/* :207 (AntiPenetrationWallCUDAKernel.cu:52-134; doNotApplyWith is not used,
 * as in the reference) */
inline void antiPenetrationWall(AgentGroup* pAgentGroup, KNNData* pKNNData, WallGroup* pWallGroup,
                                float const elapsedTime, uint const doNotApplyWith) {
    gsCheck(gs_anti_penetration_wall(detail::group(pAgentGroup), pKNNData->handle(),
                                     pWallGroup->gsWalls(), elapsedTime, doNotApplyWith));
}
/* No counterpart in the reference: findKNearestNeighbors for every group
 * pair of a MultiGroup frame (MultiGroup.cpp:560-564) in one launch;
 * ppKNNData[i * nGroups + j] (null to skip) receives group i against group j,
 * equal to the per-pair calls. */
inline void findKNearestNeighborsGroups(AgentGroup* const* ppGroups, uint const nGroups,
                                        KNNBinData* pKNNBinData, KNNData* const* ppKNNData) {
    std::vector<gs_group> g(nGroups);
    for (uint i = 0; i < nGroups; ++i) g[i] = ppGroups[i]->gsGroup();
    std::vector<gs_knn> out(size_t(nGroups) * nGroups, nullptr);
    for (size_t q = 0; q < out.size(); ++q)
        if (ppKNNData[q]) out[q] = ppKNNData[q]->handle();
    gsCheck(gs_find_knn_groups(g.data(), nGroups, pKNNBinData->handle(), out.data()));
    for (size_t q = 0; q < out.size(); ++q)
        if (ppKNNData[q]) ppKNNData[q]->setSyncHost(g[q / nGroups]);
}
/* :216 */
inline void antiPenetrationAgents(AgentGroup* pAgentGroup, KNNData* pKNNData,
                                  AgentGroup* pOtherGroup, uint const doNotApplyWith) {
    gsCheck(gs_anti_penetration_agents(detail::group(pAgentGroup), pKNNData->handle(),
                                       pOtherGroup->gsGroup(), doNotApplyWith));
}

}  // namespace OpenSteer

#endif
