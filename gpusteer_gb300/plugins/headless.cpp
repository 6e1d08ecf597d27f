// Headless driver for plugins written against the reference's group API.
//
// Two plugins re-state the reference's per-frame updates through the C++
// drop-in (include/GroupSteerLibrary.h), call for call:
//   Boids       BoidsGroup::update (plugins/BoidsGroup.cpp:606-637):
//               wrapWorld, updateKNNDatabase, findKNearestNeighbors,
//               separation, cohesion, alignment, updateGroup
//   ChokePoint  CtfGroup::update (plugins/ChokePointNew.cpp:586-630) with the
//               behaviours of the choke-point configuration: wrapWorld,
//               updateKNNDatabase, KNN of agents and of walls,
//               steerToAvoidWalls, steerToAvoidNeighbors, separation, seek,
//               updateGroup
// The world (KNNBinData, WallGroup loaded from a .map file and split on the
// bins) is built in open() as CtfWorld does (ChokePointNew.cpp:103-120).
//
//   ChokePointNew  CtfGroup::update as ChokePointNew.cpp:586-630 has it, with
//               path following and anti-penetration (below)
//   ChokePointGroup  CtfEnemyGroup::update (plugins/ChokePointGroup.cpp:683-728):
//               the applied bits cleared with cudaMemset, walls, path
//               following, seek, flocking, updateGroupWithAntiPenetration,
//               antiPenetrationAgents
//
//   MultiGroup  MultiGroupSimulation::update (plugins/MultiGroup.cpp:545-610)
//               over several groups (below)
//
//   gs_headless <Boids|ChokePoint|ChokePointNew|ChokePointGroup|MultiGroup> <state_in> <state_out>
//               <frames> [params=<file.params>] [key=value ...]
//
// params= loads a scenario file with SimulationParams (include/SimulationParams.h)
// and supplies the values the reference's plugins read from it; key=value
// arguments override single values.
//
// State files: uint32 n, then position (4n f32), direction (4n), steering
// (4n), side (3n), up (3n), speed, max_speed, max_force, radius, mass (n
// f32 each), applied (n u32).  The final state is written by redraw() after
// the last frame.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include <cuda_runtime_api.h>
#include <vector_functions.h>

#include "GroupSteerLibrary.h"
#include "PlugIn.h"
#include "SimulationParams.h"

using namespace OpenSteer;

namespace {

typedef std::map<std::string, std::string> Params;

float fparam(const Params& p, const char* k, float def) {
    auto it = p.find(k);
    return it == p.end() ? def : std::strtof(it->second.c_str(), nullptr);
}
uint uparam(const Params& p, const char* k, uint def) {
    auto it = p.find(k);
    return it == p.end() ? def : uint(std::strtoul(it->second.c_str(), nullptr, 10));
}
float3 f3param(const Params& p, const char* k, float3 def) {
    auto it = p.find(k);
    if (it == p.end()) return def;
    std::istringstream in(it->second);
    char c;
    in >> def.x >> c >> def.y >> c >> def.z;
    return def;
}
uint3 u3param(const Params& p, const char* k, uint3 def) {
    auto it = p.find(k);
    if (it == p.end()) return def;
    std::istringstream in(it->second);
    char c;
    in >> def.x >> c >> def.y >> c >> def.z;
    return def;
}

// The values a plugin reads from its SimulationParams (ChokePointNew.cpp:589-629
// reads m_pSimulationParams->...), as this driver's key=value parameters; keys
// given on the command line win.  Floats are printed with 9 significant
// digits, which read back to the same binary32 value.  A relative map file
// name is taken relative to the .params file.
void apply_simulation_params(const char* file, Params& p) {
    SimulationParams sp;
    sp.load(file);
    const std::string f(file);
    const size_t slash = f.find_last_of('/');
    const std::string dir = slash == std::string::npos ? std::string(".") : f.substr(0, slash);
    auto put = [&](const char* k, std::string const& v) {
        if (!p.count(k)) p[k] = v;
    };
    auto fl = [](float v) {
        char b[32];
        std::snprintf(b, sizeof(b), "%.9g", v);
        return std::string(b);
    };
    auto un = [](unsigned v) { return std::to_string(v); };
    auto f3s = [&](float3 v) { return fl(v.x) + "," + fl(v.y) + "," + fl(v.z); };
    const WorldParams& w = sp.m_WorldParams;
    put("world", f3s(w.m_f3Dimensions));
    put("cells", un(w.m_u3Cells.x) + "," + un(w.m_u3Cells.y) + "," + un(w.m_u3Cells.z));
    put("k", un(sp.m_nKNN));
    put("knw", un(sp.m_nKNW));
    put("radius", un(sp.m_nSearchRadius));
    if (!w.m_strMapFilename.empty())
        put("map", w.m_strMapFilename[0] == '/' ? w.m_strMapFilename : dir + "/" + w.m_strMapFilename);
    put("min_time_wall", fl(sp.m_fMinTimeToWall));
    put("w_walls", fl(sp.m_fWeightAvoidWalls));
    put("mask_walls", un(sp.m_nMaskAvoidWalls));
    put("min_time_col", fl(sp.m_fMinTimeToCollision));
    put("min_sep", fl(sp.m_fMinSeparationDistance));
    put("avoid_close", un(sp.m_bAvoidCloseNeighbors ? 1u : 0u));
    put("w_avoid", fl(sp.m_fWeightAvoidNeighbors));
    put("mask_avoid", un(sp.m_nMaskAvoidNeighbors));
    put("sep_min", fl(sp.m_fMinSeparationDistance));
    put("sep_max", fl(sp.m_fMaxSeparationDistance));
    put("sep_cos", fl(sp.m_fCosMaxFlockingAngle));
    put("w_sep", fl(sp.m_fWeightSeparation));
    put("mask_sep", un(sp.m_nMaskSeparation));
    for (const char* b : {"ali", "coh"}) {
        const std::string pre(b);
        put((pre + "_min").c_str(), fl(sp.m_fMinFlockingDistance));
        put((pre + "_max").c_str(), fl(sp.m_fMaxFlockingDistance));
        put((pre + "_cos").c_str(), fl(sp.m_fCosMaxFlockingAngle));
    }
    put("w_ali", fl(sp.m_fWeightAlignment));
    put("mask_ali", un(sp.m_nMaskAlignment));
    put("w_coh", fl(sp.m_fWeightCohesion));
    put("mask_coh", un(sp.m_nMaskCohesion));
    put("path_time", fl(sp.m_fPathPredictionTime));
    put("w_path", fl(sp.m_fWeightFollowPath));
    put("mask_path", un(sp.m_nMaskFollowPath));
    put("w_seek", fl(sp.m_fWeightSeek));
    put("mask_seek", un(sp.m_nMaskSeek));
    put("mask_antipen", un(sp.m_nMaskAntiPenetrationAgents));
    for (size_t gi = 0; gi < sp.m_vecGroupParams.size(); ++gi) {
        const GroupParams& g = sp.m_vecGroupParams[gi];
        std::string path;
        for (float3 const& q : g.m_vecPathPoints) path += (path.empty() ? "" : ";") + f3s(q);
        if (!path.empty()) put(("path" + std::to_string(gi)).c_str(), path);
    }
    if (!sp.m_vecGroupParams.empty()) {
        const GroupParams& g = sp.m_vecGroupParams[0];
        std::string path;
        for (float3 const& q : g.m_vecPathPoints) path += (path.empty() ? "" : ";") + f3s(q);
        if (!path.empty()) put("path", path);
        put("path_radius", fl(g.m_fPathRadius));
        put("path_cyclic", un(g.m_bPathIsCyclic ? 1u : 0u));
    }
}

// ---- state files ---------------------------------------------------------------------
std::vector<AgentData> read_state(const char* path) {
    FILE* f = std::fopen(path, "rb");
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    uint32_t n = 0;
    if (std::fread(&n, 4, 1, f) != 1) throw std::runtime_error("short state file");
    std::vector<float> pos(4 * n), dir(4 * n), st(4 * n), side(3 * n), up(3 * n), sp(n), ms(n),
        mf(n), rad(n), mass(n);
    std::vector<uint32_t> ap(n);
    auto rd = [&](void* d, size_t bytes) {
        if (bytes && std::fread(d, 1, bytes, f) != bytes) throw std::runtime_error("short state file");
    };
    rd(pos.data(), pos.size() * 4);
    rd(dir.data(), dir.size() * 4);
    rd(st.data(), st.size() * 4);
    rd(side.data(), side.size() * 4);
    rd(up.data(), up.size() * 4);
    rd(sp.data(), n * 4);
    rd(ms.data(), n * 4);
    rd(mf.data(), n * 4);
    rd(rad.data(), n * 4);
    rd(mass.data(), n * 4);
    rd(ap.data(), n * 4);
    std::fclose(f);
    std::vector<AgentData> out(n);
    for (uint32_t i = 0; i < n; ++i) {
        AgentData& a = out[i];
        a.id = i;
        a.position = make_float4(pos[4 * i], pos[4 * i + 1], pos[4 * i + 2], pos[4 * i + 3]);
        a.direction = make_float4(dir[4 * i], dir[4 * i + 1], dir[4 * i + 2], dir[4 * i + 3]);
        a.steering = make_float4(st[4 * i], st[4 * i + 1], st[4 * i + 2], st[4 * i + 3]);
        a.side = make_float3(side[3 * i], side[3 * i + 1], side[3 * i + 2]);
        a.up = make_float3(up[3 * i], up[3 * i + 1], up[3 * i + 2]);
        a.speed = sp[i];
        a.maxSpeed = ms[i];
        a.maxForce = mf[i];
        a.radius = rad[i];
        a.mass = mass[i];
        a.appliedKernels = ap[i];
    }
    return out;
}

void write_state(const char* path, AgentGroup& g) {
    const uint32_t n = g.Size();
    std::vector<float> pos, dir, st, side, up, sp, ms, mf, rad, mass;
    std::vector<uint32_t> ap;
    for (uint32_t i = 0; i < n; ++i) {
        AgentData a;
        if (!g.GetDataForAgent(i, a)) throw std::runtime_error("missing agent");
        pos.insert(pos.end(), {a.position.x, a.position.y, a.position.z, a.position.w});
        dir.insert(dir.end(), {a.direction.x, a.direction.y, a.direction.z, a.direction.w});
        st.insert(st.end(), {a.steering.x, a.steering.y, a.steering.z, a.steering.w});
        side.insert(side.end(), {a.side.x, a.side.y, a.side.z});
        up.insert(up.end(), {a.up.x, a.up.y, a.up.z});
        sp.push_back(a.speed);
        ms.push_back(a.maxSpeed);
        mf.push_back(a.maxForce);
        rad.push_back(a.radius);
        mass.push_back(a.mass);
        ap.push_back(a.appliedKernels);
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) throw std::runtime_error(std::string("cannot write ") + path);
    std::fwrite(&n, 4, 1, f);
    for (auto* v : {&pos, &dir, &st, &side, &up, &sp, &ms, &mf, &rad, &mass})
        std::fwrite(v->data(), 4, v->size(), f);
    std::fwrite(ap.data(), 4, ap.size(), f);
    std::fclose(f);
}

std::vector<std::string> split(const std::string& s, char sep) {
    std::vector<std::string> out;
    std::istringstream in(s);
    std::string item;
    while (std::getline(in, item, sep)) out.push_back(item);
    return out;
}

std::vector<float3> parse_points(const std::string& s) {
    std::vector<float3> pts;
    for (const std::string& item : split(s, ';')) {
        std::istringstream v(item);
        float3 q;
        char c;
        v >> q.x >> c >> q.y >> c >> q.z;
        pts.push_back(q);
    }
    return pts;
}

// ---- plugins -------------------------------------------------------------------------
class HeadlessPlugIn : public PlugIn {
public:
    Params params;
    std::string in_path, out_path;
};

class BoidsPlugIn : public HeadlessPlugIn {
public:
    const char* name() { return "Boids"; }
    void open() {
        const Params& p = params;
        m_worldSize = f3param(p, "world", make_float3(160.f, 160.f, 160.f));
        m_worldCells = u3param(p, "cells", make_uint3(40, 40, 40));
        m_k = uparam(p, "k", 7);
        m_radius = uparam(p, "radius", 1);
        m_bins.reset(new KNNBinData(m_worldCells, m_worldSize, m_radius));
        m_group.reset(new AgentGroup(m_worldCells, m_k));
        for (const AgentData& a : read_state(in_path.c_str())) m_group->AddAgent(a);
        m_group->SyncDevice();
        m_knn.reset(new KNNData(m_group->Size(), m_k));
    }
    // BoidsGroup::update (plugins/BoidsGroup.cpp:606-637)
    void update(const float, const float elapsedTime) {
        const Params& p = params;
        AgentGroup* g = m_group.get();
        wrapWorld(g, m_worldSize);
        updateKNNDatabase(g, m_bins.get());
        findKNearestNeighbors(g, m_knn.get(), m_bins.get(), g, m_radius);
        steerForSeparation(g, m_knn.get(), g, fparam(p, "sep_min", 0.5f), fparam(p, "sep_max", 2.f),
                           fparam(p, "sep_cos", -0.9848077f), fparam(p, "w_sep", 5.f),
                           uparam(p, "mask_sep", 0));
        steerForCohesion(g, m_knn.get(), g, fparam(p, "coh_min", 0.5f), fparam(p, "coh_max", 7.f),
                         fparam(p, "coh_cos", -0.9848077f), fparam(p, "w_coh", 4.f),
                         uparam(p, "mask_coh", 0));
        steerForAlignment(g, m_knn.get(), g, fparam(p, "ali_min", 0.5f), fparam(p, "ali_max", 7.f),
                          fparam(p, "ali_cos", -0.9848077f), fparam(p, "w_ali", 8.f),
                          uparam(p, "mask_ali", 0));
        updateGroup(g, elapsedTime);
    }
    void redraw(const float, const float) { write_state(out_path.c_str(), *m_group); }
    void close() {
        m_knn.reset();
        m_group.reset();
        m_bins.reset();
    }

private:
    float3 m_worldSize;
    uint3 m_worldCells;
    uint m_k = 7, m_radius = 1;
    std::unique_ptr<KNNBinData> m_bins;
    std::unique_ptr<AgentGroup> m_group;
    std::unique_ptr<KNNData> m_knn;
};

class ChokePointPlugIn : public HeadlessPlugIn {
public:
    const char* name() { return "ChokePoint"; }
    // CtfWorld (ChokePointNew.cpp:103-120) and CtfGroup set-up
    void open() {
        const Params& p = params;
        m_worldSize = f3param(p, "world", make_float3(512.f, 10.f, 512.f));
        m_worldCells = u3param(p, "cells", make_uint3(256, 1, 256));
        m_k = uparam(p, "k", 16);
        m_knw = uparam(p, "knw", 3);
        m_radius = uparam(p, "radius", 1);
        m_bins.reset(new KNNBinData(m_worldCells, m_worldSize, m_radius));
        m_walls.reset(new WallGroup(m_worldCells, m_knw));
        auto it = p.find("map");
        if (it == p.end() || !m_walls->LoadFromFile(it->second.c_str()))
            throw std::runtime_error("ChokePoint needs map=<file.map>");
        m_walls->SplitWalls(m_bins->hvCells());
        m_walls->SyncDevice();
        updateKNNDatabase(m_walls.get(), m_bins.get());
        m_group.reset(new AgentGroup(m_worldCells, m_k));
        for (const AgentData& a : read_state(in_path.c_str())) m_group->AddAgent(a);
        m_group->SyncDevice();
        m_knnSelf.reset(new KNNData(m_group->Size(), m_k));
        m_knnWalls.reset(new KNNData(m_group->Size(), m_knw));
    }
    // CtfGroup::update (ChokePointNew.cpp:586-630), choke-point behaviours.
    // The reference clears the applied bits with a cudaMemset before the KNN;
    // updateGroup leaves them cleared after every frame, and the agents are
    // added with none set, so that call has nothing to clear here.
    void update(const float, const float elapsedTime) {
        const Params& p = params;
        AgentGroup* g = m_group.get();
        wrapWorld(g, m_worldSize);
        updateKNNDatabase(g, m_bins.get());
        findKNearestNeighbors(g, m_knnSelf.get(), m_bins.get(), g, m_radius);
        findKNearestNeighbors(g, m_knnWalls.get(), m_bins.get(), m_walls.get(), m_radius);
        steerToAvoidWalls(g, m_knnWalls.get(), m_walls.get(), fparam(p, "min_time_wall", 10.f),
                          fparam(p, "w_walls", 1.f), uparam(p, "mask_walls", 0));
        steerToAvoidNeighbors(g, m_knnSelf.get(), g, fparam(p, "min_time_col", 2.f),
                              fparam(p, "min_sep", 0.5f), uparam(p, "avoid_close", 0) != 0,
                              fparam(p, "w_avoid", 1.f), uparam(p, "mask_avoid", 0));
        steerForSeparation(g, m_knnSelf.get(), g, fparam(p, "sep_min", 0.5f),
                           fparam(p, "sep_max", 1.2f), fparam(p, "sep_cos", -0.8660254f),
                           fparam(p, "w_sep", 10.f), uparam(p, "mask_sep", KERNEL_ANTI_PENETRATION_WALL));
        steerForSeek(g, f3param(p, "seek", make_float3(0.f, 0.f, -93.5f)), fparam(p, "w_seek", 1.5f),
                     uparam(p, "mask_seek", 4480));
        updateGroup(g, elapsedTime);
    }
    void redraw(const float, const float) { write_state(out_path.c_str(), *m_group); }
    void close() {
        m_knnSelf.reset();
        m_knnWalls.reset();
        m_group.reset();
        m_walls.reset();
        m_bins.reset();
    }

private:
    float3 m_worldSize;
    uint3 m_worldCells;
    uint m_k = 16, m_knw = 3, m_radius = 1;
    std::unique_ptr<KNNBinData> m_bins;
    std::unique_ptr<WallGroup> m_walls;
    std::unique_ptr<AgentGroup> m_group;
    std::unique_ptr<KNNData> m_knnSelf, m_knnWalls;
};

// CtfGroup::update as plugins/ChokePointNew.cpp:586-630 has it: walls,
// separation, alignment, cohesion, path following, seek the path's second
// point, update, anti-penetration between agents.  The path comes from the
// parameters: path=x,y,z;x,y,z;...  path_radius=  path_cyclic=
class ChokePointNewPlugIn : public HeadlessPlugIn {
public:
    const char* name() { return "ChokePointNew"; }
    void open() {
        const Params& p = params;
        m_worldSize = f3param(p, "world", make_float3(512.f, 10.f, 512.f));
        m_worldCells = u3param(p, "cells", make_uint3(256, 1, 256));
        m_k = uparam(p, "k", 16);
        m_knw = uparam(p, "knw", 3);
        m_radius = uparam(p, "radius", 1);
        m_bins.reset(new KNNBinData(m_worldCells, m_worldSize, m_radius));
        m_walls.reset(new WallGroup(m_worldCells, m_knw));
        auto it = p.find("map");
        if (it == p.end() || !m_walls->LoadFromFile(it->second.c_str()))
            throw std::runtime_error("ChokePointNew needs map=<file.map>");
        m_walls->SplitWalls(m_bins->hvCells());
        m_walls->SyncDevice();
        updateKNNDatabase(m_walls.get(), m_bins.get());
        std::vector<float3> pts;
        auto pp = p.find("path");
        if (pp == p.end()) throw std::runtime_error("ChokePointNew needs path=x,y,z;x,y,z...");
        std::istringstream in(pp->second);
        std::string item;
        while (std::getline(in, item, ';')) {
            std::istringstream v(item);
            float3 q;
            char c;
            v >> q.x >> c >> q.y >> c >> q.z;
            pts.push_back(q);
        }
        m_path.reset(new PolylinePathwayCUDA(pts, fparam(p, "path_radius", 20.f),
                                             uparam(p, "path_cyclic", 0) != 0));
        m_group.reset(new AgentGroup(m_worldCells, m_k));
        for (const AgentData& a : read_state(in_path.c_str())) m_group->AddAgent(a);
        m_group->SyncDevice();
        m_knnSelf.reset(new KNNData(m_group->Size(), m_k));
        m_knnWalls.reset(new KNNData(m_group->Size(), m_knw));
    }
    void update(const float, const float elapsedTime) {
        const Params& p = params;
        AgentGroup* g = m_group.get();
        wrapWorld(g, m_worldSize);
        updateKNNDatabase(g, m_bins.get());
        findKNearestNeighbors(g, m_knnSelf.get(), m_bins.get(), g, m_radius);
        findKNearestNeighbors(g, m_knnWalls.get(), m_bins.get(), m_walls.get(), m_radius);
        steerToAvoidWalls(g, m_knnWalls.get(), m_walls.get(), fparam(p, "min_time_wall", 10.f),
                          fparam(p, "w_walls", 1.f), uparam(p, "mask_walls", 0));
        steerForSeparation(g, m_knnSelf.get(), g, fparam(p, "sep_min", 0.5f),
                           fparam(p, "sep_max", 1.2f), fparam(p, "sep_cos", -0.8660254f),
                           fparam(p, "w_sep", 10.f), KERNEL_ANTI_PENETRATION_WALL);
        steerForAlignment(g, m_knnSelf.get(), g, fparam(p, "ali_min", 0.5f),
                          fparam(p, "ali_max", 7.f), fparam(p, "ali_cos", -0.8660254f),
                          fparam(p, "w_ali", 2.f), uparam(p, "mask_ali", 0));
        steerForCohesion(g, m_knnSelf.get(), g, fparam(p, "coh_min", 0.5f),
                         fparam(p, "coh_max", 7.f), fparam(p, "coh_cos", -0.8660254f),
                         fparam(p, "w_coh", 1.f), uparam(p, "mask_coh", 0));
        steerToFollowPath(g, m_path.get(), fparam(p, "path_time", 5.f), fparam(p, "w_path", 1.f),
                          uparam(p, "mask_path", 16));
        steerForSeek(g, m_path->hvPoints()[1], fparam(p, "w_seek", 1.5f),
                     uparam(p, "mask_seek", 4480));
        updateGroup(g, elapsedTime);
        if (uparam(p, "antipen", 1))
            antiPenetrationAgents(g, m_knnSelf.get(), g, uparam(p, "mask_antipen", 0));
    }
    void redraw(const float, const float) { write_state(out_path.c_str(), *m_group); }
    void close() {
        m_knnSelf.reset();
        m_knnWalls.reset();
        m_group.reset();
        m_path.reset();
        m_walls.reset();
        m_bins.reset();
    }

private:
    float3 m_worldSize;
    uint3 m_worldCells;
    uint m_k = 16, m_knw = 3, m_radius = 1;
    std::unique_ptr<KNNBinData> m_bins;
    std::unique_ptr<WallGroup> m_walls;
    std::unique_ptr<PolylinePathwayCUDA> m_path;
    std::unique_ptr<AgentGroup> m_group;
    std::unique_ptr<KNNData> m_knnSelf, m_knnWalls;
};

// CtfEnemyGroup::update (plugins/ChokePointGroup.cpp:683-728): the older
// choke-point group, which integrates with updateGroupWithAntiPenetration.
// That update keeps the applied bits, so the frame starts by clearing them
// with a cudaMemset on the group's device array (:689-690), ordered with the
// library's launches on the legacy default stream.  The path and the goal
// come from the parameters (path=x,y,z;...  path_radius=  goal=x,y,z).
class ChokePointGroupPlugIn : public HeadlessPlugIn {
public:
    const char* name() { return "ChokePointGroup"; }
    void open() {
        const Params& p = params;
        m_worldSize = f3param(p, "world", make_float3(512.f, 10.f, 512.f));
        m_worldCells = u3param(p, "cells", make_uint3(256, 1, 256));
        m_k = uparam(p, "k", 16);
        m_knw = uparam(p, "knw", 3);
        m_radius = uparam(p, "radius", 1);
        m_bins.reset(new KNNBinData(m_worldCells, m_worldSize, m_radius));
        m_walls.reset(new WallGroup(m_worldCells, m_knw));
        auto it = p.find("map");
        if (it == p.end() || !m_walls->LoadFromFile(it->second.c_str()))
            throw std::runtime_error("ChokePointGroup needs map=<file.map>");
        m_walls->SplitWalls(m_bins->hvCells());
        m_walls->SyncDevice();
        updateKNNDatabase(m_walls.get(), m_bins.get());
        std::vector<float3> pts;
        auto pp = p.find("path");
        if (pp == p.end()) throw std::runtime_error("ChokePointGroup needs path=x,y,z;x,y,z...");
        std::istringstream in(pp->second);
        std::string item;
        while (std::getline(in, item, ';')) {
            std::istringstream v(item);
            float3 q;
            char c;
            v >> q.x >> c >> q.y >> c >> q.z;
            pts.push_back(q);
        }
        m_path.reset(new PolylinePathwayCUDA(pts, fparam(p, "path_radius", 23.5f), false));
        m_group.reset(new AgentGroup(m_worldCells, m_k));
        for (const AgentData& a : read_state(in_path.c_str())) m_group->AddAgent(a);
        m_group->SyncDevice();
        m_knnSelf.reset(new KNNData(m_group->Size(), m_k));
        m_knnWalls.reset(new KNNData(m_group->Size(), m_knw));
    }
    void update(const float, const float elapsedTime) {
        const Params& p = params;
        AgentGroup* g = m_group.get();
        wrapWorld(g, m_worldSize);
        updateKNNDatabase(g, m_bins.get());
        if (cudaMemset(g->GetAgentGroupData().pdAppliedKernels(), 0, g->Size() * sizeof(uint)) !=
            cudaSuccess)
            throw std::runtime_error("cudaMemset of the applied bits failed");
        findKNearestNeighbors(g, m_knnSelf.get(), m_bins.get(), g, m_radius);
        findKNearestNeighbors(g, m_knnWalls.get(), m_bins.get(), m_walls.get(), m_radius);
        steerToAvoidWalls(g, m_knnWalls.get(), m_walls.get(), fparam(p, "min_time_wall", 10.f),
                          fparam(p, "w_walls", 1.f), uparam(p, "mask_walls", 0));
        steerToFollowPath(g, m_path.get(), fparam(p, "path_time", 5.f), fparam(p, "w_path", 1.f),
                          uparam(p, "mask_path", KERNEL_SEPARATION_BIT));
        steerForSeek(g, f3param(p, "goal", make_float3(0.f, 0.f, -93.5f)),
                     fparam(p, "w_seek", 1.f), uparam(p, "mask_seek", KERNEL_AVOID_WALLS_BIT));
        steerForSeparation(g, m_knnSelf.get(), g, fparam(p, "sep_min", 0.5f),
                           fparam(p, "sep_max", 1.2f), fparam(p, "sep_cos", -0.8660254f),
                           fparam(p, "w_sep", 10.f),
                           uparam(p, "mask_sep", KERNEL_ANTI_PENETRATION_WALL));
        steerForAlignment(g, m_knnSelf.get(), g, fparam(p, "ali_min", 0.5f),
                          fparam(p, "ali_max", 7.f), fparam(p, "ali_cos", -0.8660254f),
                          fparam(p, "w_ali", 2.5f),
                          uparam(p, "mask_ali", KERNEL_AVOID_WALLS_BIT | KERNEL_SEPARATION_BIT));
        steerForCohesion(g, m_knnSelf.get(), g, fparam(p, "coh_min", 0.5f),
                         fparam(p, "coh_max", 7.f), fparam(p, "coh_cos", -0.8660254f),
                         fparam(p, "w_coh", 1.f),
                         uparam(p, "mask_coh", KERNEL_AVOID_WALLS_BIT | KERNEL_SEPARATION_BIT));
        updateGroupWithAntiPenetration(g, m_knnWalls.get(), m_walls.get(), elapsedTime);
        antiPenetrationAgents(g, m_knnSelf.get(), g,
                              uparam(p, "mask_antipen",
                                     KERNEL_AVOID_WALLS_BIT | KERNEL_ANTI_PENETRATION_WALL));
    }
    void redraw(const float, const float) { write_state(out_path.c_str(), *m_group); }
    void close() {
        m_knnSelf.reset();
        m_knnWalls.reset();
        m_group.reset();
        m_path.reset();
        m_walls.reset();
        m_bins.reset();
    }

private:
    float3 m_worldSize;
    uint3 m_worldCells;
    uint m_k = 16, m_knw = 3, m_radius = 1;
    std::unique_ptr<KNNBinData> m_bins;
    std::unique_ptr<WallGroup> m_walls;
    std::unique_ptr<PolylinePathwayCUDA> m_path;
    std::unique_ptr<AgentGroup> m_group;
    std::unique_ptr<KNNData> m_knnSelf, m_knnWalls;
};

// MultiGroupSimulation::update (plugins/MultiGroup.cpp:545-610): several groups
// in one world.  Every frame runs Group::preUpdate for every group (wrap,
// updateKNNDatabase, the applied bits cleared with cudaMemset), then
// Group::update of each group in turn: KNN against every group, avoid the
// other groups' neighbours, separation from every group, alignment and
// cohesion with itself, path following and seek of the path's second point
// when the group has a path (path<i>=x,y,z;...), update, anti-penetration
// against every group.  state_in / state_out list one file per group,
// separated by commas.
class MultiGroupPlugIn : public HeadlessPlugIn {
public:
    const char* name() { return "MultiGroup"; }
    void open() {
        const Params& p = params;
        m_worldSize = f3param(p, "world", make_float3(200.f, 200.f, 200.f));
        m_worldCells = u3param(p, "cells", make_uint3(50, 50, 50));
        m_k = uparam(p, "k", 16);
        m_radius = uparam(p, "radius", 1);
        m_bins.reset(new KNNBinData(m_worldCells, m_worldSize, m_radius));
        const std::vector<std::string> files = split(in_path, ',');
        for (size_t i = 0; i < files.size(); ++i) {
            m_groups.emplace_back(new AgentGroup(m_worldCells, m_k));
            for (const AgentData& a : read_state(files[i].c_str())) m_groups.back()->AddAgent(a);
            m_groups.back()->SyncDevice();
            auto pp = p.find("path" + std::to_string(i));
            m_paths.emplace_back(pp == p.end() ? nullptr
                                               : new PolylinePathwayCUDA(parse_points(pp->second),
                                                                         fparam(p, "path_radius", 23.f),
                                                                         false));
        }
        const size_t G = m_groups.size();
        for (size_t i = 0; i < G; ++i)
            for (size_t j = 0; j < G; ++j)
                m_knn.emplace_back(new KNNData(m_groups[i]->Size(), m_k));
    }
    void update(const float, const float elapsedTime) {
        const Params& p = params;
        const size_t G = m_groups.size();
        for (auto& g : m_groups) {  // Group::preUpdate (:545-556)
            wrapWorld(g.get(), m_worldSize);
            updateKNNDatabase(g.get(), m_bins.get());
            if (cudaMemset(g->GetAgentGroupData().pdAppliedKernels(), 0, g->Size() * sizeof(uint)) !=
                cudaSuccess)
                throw std::runtime_error("cudaMemset of the applied bits failed");
        }
        for (size_t i = 0; i < G; ++i) {  // Group::update (:558-610)
            AgentGroup* gi = m_groups[i].get();
            for (size_t j = 0; j < G; ++j)
                findKNearestNeighbors(gi, knn(i, j), m_bins.get(), m_groups[j].get(), m_radius);
            for (size_t j = 0; j < G; ++j)
                if (j != i)
                    steerToAvoidNeighbors(gi, knn(i, j), m_groups[j].get(),
                                          fparam(p, "min_time_col", 2.f), fparam(p, "min_sep", 0.5f),
                                          uparam(p, "avoid_close", 0) != 0, fparam(p, "w_avoid", 1.f),
                                          uparam(p, "mask_avoid", 0));
            for (size_t j = 0; j < G; ++j)
                steerForSeparation(gi, knn(i, j), m_groups[j].get(), fparam(p, "sep_min", 0.5f),
                                   fparam(p, "sep_max", 1.2f), fparam(p, "sep_cos", -0.8660254f),
                                   fparam(p, "w_sep", 10.f), uparam(p, "mask_sep", 0));
            steerForAlignment(gi, knn(i, i), gi, fparam(p, "ali_min", 0.5f), fparam(p, "ali_max", 7.f),
                              fparam(p, "ali_cos", -0.8660254f), fparam(p, "w_ali", 2.5f),
                              uparam(p, "mask_ali", 0));
            steerForCohesion(gi, knn(i, i), gi, fparam(p, "coh_min", 0.5f), fparam(p, "coh_max", 7.f),
                             fparam(p, "coh_cos", -0.8660254f), fparam(p, "w_coh", 1.f),
                             uparam(p, "mask_coh", 0));
            if (PolylinePathwayCUDA* path = m_paths[i].get()) {
                steerToFollowPath(gi, path, fparam(p, "path_time", 5.f), fparam(p, "w_path", 1.f),
                                  uparam(p, "mask_path", 0));
                steerForSeek(gi, path->hvPoints()[1], fparam(p, "w_seek", 1.f),
                             uparam(p, "mask_seek", 0));
            }
            updateGroup(gi, elapsedTime);
            for (size_t j = 0; j < G; ++j)
                antiPenetrationAgents(gi, knn(i, j), m_groups[j].get(), uparam(p, "mask_antipen", 0));
        }
    }
    void redraw(const float, const float) {
        const std::vector<std::string> files = split(out_path, ',');
        for (size_t i = 0; i < m_groups.size() && i < files.size(); ++i)
            write_state(files[i].c_str(), *m_groups[i]);
    }
    void close() {
        m_knn.clear();
        m_paths.clear();
        m_groups.clear();
        m_bins.reset();
    }

private:
    KNNData* knn(size_t i, size_t j) { return m_knn[i * m_groups.size() + j].get(); }
    float3 m_worldSize;
    uint3 m_worldCells;
    uint m_k = 16, m_radius = 1;
    std::unique_ptr<KNNBinData> m_bins;
    std::vector<std::unique_ptr<AgentGroup>> m_groups;
    std::vector<std::unique_ptr<PolylinePathwayCUDA>> m_paths;
    std::vector<std::unique_ptr<KNNData>> m_knn;
};

BoidsPlugIn gBoidsPlugIn;
ChokePointPlugIn gChokePointPlugIn;
ChokePointNewPlugIn gChokePointNewPlugIn;
ChokePointGroupPlugIn gChokePointGroupPlugIn;
MultiGroupPlugIn gMultiGroupPlugIn;

}  // namespace

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr,
                     "usage: %s <Boids|ChokePoint|ChokePointNew|ChokePointGroup|MultiGroup> <state_in> <state_out> "
                     "<frames> "
                     "[key=value ...]\n",
                     argv[0]);
        return 2;
    }
    HeadlessPlugIn* plugin = static_cast<HeadlessPlugIn*>(PlugIn::findByName(argv[1]));
    if (!plugin) {
        std::fprintf(stderr, "unknown plugin %s\n", argv[1]);
        return 2;
    }
    plugin->in_path = argv[2];
    plugin->out_path = argv[3];
    const unsigned frames = unsigned(std::strtoul(argv[4], nullptr, 10));
    for (int i = 5; i < argc; ++i) {
        const char* eq = std::strchr(argv[i], '=');
        if (!eq) {
            std::fprintf(stderr, "bad parameter %s\n", argv[i]);
            return 2;
        }
        plugin->params[std::string(argv[i], size_t(eq - argv[i]))] = eq + 1;
    }
    try {
        auto pf = plugin->params.find("params");
        if (pf != plugin->params.end()) {
            const std::string file = pf->second;
            apply_simulation_params(file.c_str(), plugin->params);
        }
        const float dt = fparam(plugin->params, "dt", 1.f / 60.f);
        runHeadless(*plugin, frames, dt, frames ? frames : 1);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
