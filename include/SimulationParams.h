/* SimulationParams.h - the reference's scenario parameter files (.params) for
 * plugins written against GroupSteerLibrary.h: GroupParams, WorldParams and
 * SimulationParams with the members of include/OpenSteer/Simulation.h:14-122,
 * filled by load() from the format src/Simulation.cpp:7-250 reads.
 *
 * The format: whitespace-separated tokens; a token that starts with '#'
 * comments out the rest of its line; `key = value...` pairs at the top level,
 * inside <world> ... </world> and inside <group> ... </group>, which may hold
 * a <path> ... </path> of `point = x y z`, `cyclic = 0|1`, `radius = r`; the
 * file ends at </simulation>.
 *
 * Differences from the reference: every member starts at zero (the reference
 * leaves a key the file omits uninitialised), and an unknown key throws
 * OpenSteer::ParamsError (the reference asserts, and in a release build reads
 * on out of step). */
#ifndef GPUSTEER_SIMULATION_PARAMS_H
#define GPUSTEER_SIMULATION_PARAMS_H

#include <vector_types.h>

#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace OpenSteer {

class ParamsError : public std::runtime_error {
public:
    explicit ParamsError(std::string const& what) : std::runtime_error(what) {}
};

namespace detail {

/* The file's tokens with comments removed, read front to back. */
class ParamsTokens {
public:
    explicit ParamsTokens(std::istream& in) {
        std::string line;
        while (std::getline(in, line)) {
            std::istringstream ls(line);
            std::string t;
            while (ls >> t) {
                if (t[0] == '#') break;
                m_tok.push_back(t);
            }
        }
    }
    bool done() const { return m_pos >= m_tok.size(); }
    std::string next() {
        if (done()) throw ParamsError("unexpected end of the parameter file");
        return m_tok[m_pos++];
    }
    float f() { return std::strtof(next().c_str(), nullptr); }
    unsigned u() { return unsigned(std::strtoul(next().c_str(), nullptr, 10)); }
    float3 f3() {
        float3 v;
        v.x = f();
        v.y = f();
        v.z = f();
        return v;
    }

private:
    std::vector<std::string> m_tok;
    size_t m_pos = 0;
};

}  // namespace detail

class GroupParams {
public:
    unsigned m_nNumAgents = 0;
    float m_fMaxSpeed = 0.f;
    float m_fMaxForce = 0.f;
    float3 m_f3StartPosition = float3{0.f, 0.f, 0.f};
    float m_fMinStartRadius = 0.f;
    float m_fMaxStartRadius = 0.f;
    std::vector<float3> m_vecPathPoints;
    float m_fPathRadius = 0.f;
    bool m_bPathIsCyclic = false;
    float3 m_f3BodyColor = float3{0.f, 0.f, 0.f};

    /* From after <group> up to and including </group>. */
    void load(detail::ParamsTokens& t) {
        for (std::string key = t.next(); key != "</group>"; key = t.next()) {
            if (key == "<path>") {
                for (std::string pk = t.next(); pk != "</path>"; pk = t.next()) {
                    t.next();  // delimiter
                    if (pk == "point")
                        m_vecPathPoints.push_back(t.f3());
                    else if (pk == "cyclic")
                        m_bPathIsCyclic = t.u() != 0;
                    else if (pk == "radius")
                        m_fPathRadius = t.f();
                    else
                        throw ParamsError("unknown path key " + pk);
                }
                continue;
            }
            t.next();  // delimiter
            if (key == "numAgents")
                m_nNumAgents = t.u();
            else if (key == "startPosition")
                m_f3StartPosition = t.f3();
            else if (key == "minStartRadius")
                m_fMinStartRadius = t.f();
            else if (key == "maxStartRadius")
                m_fMaxStartRadius = t.f();
            else if (key == "maxSpeed")
                m_fMaxSpeed = t.f();
            else if (key == "maxForce")
                m_fMaxForce = t.f();
            else if (key == "bodyColor")
                m_f3BodyColor = t.f3();
            else
                throw ParamsError("unknown group key " + key);
        }
    }
};

class WorldParams {
public:
    float3 m_f3Dimensions = float3{0.f, 0.f, 0.f};
    uint3 m_u3Cells = uint3{0u, 0u, 0u};
    unsigned m_nObstacleCount = 0;
    std::string m_strMapFilename;

    /* From after <world> up to and including </world>. */
    void load(detail::ParamsTokens& t) {
        for (std::string key = t.next(); key != "</world>"; key = t.next()) {
            t.next();  // delimiter
            if (key == "dimensions") {
                m_f3Dimensions = t.f3();
            } else if (key == "cells") {
                m_u3Cells.x = t.u();
                m_u3Cells.y = t.u();
                m_u3Cells.z = t.u();
            } else if (key == "obstacleCount") {
                m_nObstacleCount = t.u();
            } else if (key == "mapFilename") {
                m_strMapFilename = t.next();
            } else {
                throw ParamsError("unknown world key " + key);
            }
        }
    }
};

class SimulationParams {
public:
    WorldParams m_WorldParams;
    std::vector<GroupParams> m_vecGroupParams;

    unsigned m_nSeed = 0, m_nKNN = 0, m_nKNO = 0, m_nKNW = 0, m_nSearchRadius = 0;
    float m_fMaxPursuitPredictionTime = 0.f, m_fMinTimeToCollision = 0.f,
          m_fMinTimeToObstacle = 0.f, m_fMinTimeToWall = 0.f, m_fPathPredictionTime = 0.f,
          m_fMinSeparationDistance = 0.f, m_fMaxSeparationDistance = 0.f,
          m_fMinFlockingDistance = 0.f, m_fMaxFlockingDistance = 0.f,
          m_fCosMaxFlockingAngle = 0.f;
    bool m_bAvoidCloseNeighbors = false;
    /* weights */
    float m_fWeightAlignment = 0.f, m_fWeightCohesion = 0.f, m_fWeightSeparation = 0.f,
          m_fWeightPursuit = 0.f, m_fWeightSeek = 0.f, m_fWeightFlee = 0.f,
          m_fWeightEvade = 0.f, m_fWeightFollowPath = 0.f, m_fWeightAvoidObstacles = 0.f,
          m_fWeightAvoidWalls = 0.f, m_fWeightAvoidNeighbors = 0.f;
    /* masks */
    unsigned m_nMaskAlignment = 0, m_nMaskAntiPenetrationAgents = 0, m_nMaskCohesion = 0,
             m_nMaskSeparation = 0, m_nMaskPursuit = 0, m_nMaskSeek = 0, m_nMaskFlee = 0,
             m_nMaskEvade = 0, m_nMaskFollowPath = 0, m_nMaskAvoidObstacles = 0,
             m_nMaskAvoidWalls = 0, m_nMaskAvoidNeighbors = 0;

    /* As SimulationParams::load (Simulation.cpp:124-250): a file that cannot be
     * opened leaves the parameters as they are. */
    void load(char const* szFilename) {
        std::ifstream fs(szFilename);
        if (!fs.is_open()) return;
        load(fs);
    }
    void load(std::istream& in) {
        detail::ParamsTokens t(in);
        while (!t.done()) {
            const std::string key = t.next();
            if (key == "</simulation>") break;
            if (key == "<simulation>") continue;
            if (key == "<world>") {
                m_WorldParams.load(t);
                continue;
            }
            if (key == "<group>") {
                GroupParams gp;
                gp.load(t);
                m_vecGroupParams.push_back(gp);
                continue;
            }
            t.next();  // delimiter
            if (!assign(key, t)) throw ParamsError("unknown key " + key);
        }
    }

private:
    bool assign(std::string const& key, detail::ParamsTokens& t) {
        struct U {
            char const* name;
            unsigned SimulationParams::*m;
        };
        struct F {
            char const* name;
            float SimulationParams::*m;
        };
        static const U us[] = {
            {"seed", &SimulationParams::m_nSeed},
            {"knn", &SimulationParams::m_nKNN},
            {"kno", &SimulationParams::m_nKNO},
            {"knw", &SimulationParams::m_nKNW},
            {"searchRadius", &SimulationParams::m_nSearchRadius},
            {"maskAlignment", &SimulationParams::m_nMaskAlignment},
            {"maskAntiPenetrationAgents", &SimulationParams::m_nMaskAntiPenetrationAgents},
            {"maskCohesion", &SimulationParams::m_nMaskCohesion},
            {"maskSeparation", &SimulationParams::m_nMaskSeparation},
            {"maskSeek", &SimulationParams::m_nMaskSeek},
            {"maskFlee", &SimulationParams::m_nMaskFlee},
            {"maskPursuit", &SimulationParams::m_nMaskPursuit},
            {"maskEvade", &SimulationParams::m_nMaskEvade},
            {"maskFollowPath", &SimulationParams::m_nMaskFollowPath},
            {"maskAvoidObstacles", &SimulationParams::m_nMaskAvoidObstacles},
            {"maskAvoidWalls", &SimulationParams::m_nMaskAvoidWalls},
            {"maskAvoidNeighbors", &SimulationParams::m_nMaskAvoidNeighbors},
        };
        static const F fs[] = {
            {"maxPursuitPredictionTime", &SimulationParams::m_fMaxPursuitPredictionTime},
            {"minTimeToCollision", &SimulationParams::m_fMinTimeToCollision},
            {"minTimeToObstacle", &SimulationParams::m_fMinTimeToObstacle},
            {"minTimeToWall", &SimulationParams::m_fMinTimeToWall},
            {"pathPredictionTime", &SimulationParams::m_fPathPredictionTime},
            {"minSeparationDistance", &SimulationParams::m_fMinSeparationDistance},
            {"maxSeparationDistance", &SimulationParams::m_fMaxSeparationDistance},
            {"minFlockingDistance", &SimulationParams::m_fMinFlockingDistance},
            {"maxFlockingDistance", &SimulationParams::m_fMaxFlockingDistance},
            {"cosMaxFlockingAngle", &SimulationParams::m_fCosMaxFlockingAngle},
            {"weightAlignment", &SimulationParams::m_fWeightAlignment},
            {"weightCohesion", &SimulationParams::m_fWeightCohesion},
            {"weightSeparation", &SimulationParams::m_fWeightSeparation},
            {"weightPursuit", &SimulationParams::m_fWeightPursuit},
            {"weightSeek", &SimulationParams::m_fWeightSeek},
            {"weightFollowPath", &SimulationParams::m_fWeightFollowPath},
            {"weightAvoidObstacles", &SimulationParams::m_fWeightAvoidObstacles},
            {"weightAvoidWalls", &SimulationParams::m_fWeightAvoidWalls},
            {"weightAvoidNeighbors", &SimulationParams::m_fWeightAvoidNeighbors},
        };
        for (U const& e : us)
            if (key == e.name) {
                this->*e.m = t.u();
                return true;
            }
        for (F const& e : fs)
            if (key == e.name) {
                this->*e.m = t.f();
                return true;
            }
        if (key == "avoidCloseNeighbors") {
            m_bAvoidCloseNeighbors = t.u() != 0;
            return true;
        }
        return false;
    }
};

}  // namespace OpenSteer

#endif
