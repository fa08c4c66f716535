// C++ host interface of the GB300 PBF step, mirroring AkuaEngine::PBFSolver
// (include/AkuaEngine/Simulation/PBFSolver.h:12-31, src/Simulation/PBFSolver.cpp:13-78) over the
// C ABI in akua_pbf.h.  Header-only; link against libakua_pbf.so.
//
//   reference                                           here
//   PBFConfig / LambdaCorrParams (PBFConfig.h:10-29)     akua::PBFConfig / akua::LambdaCorrParams
//   PBFSolver(int, const PBFConfig&, const LambdaCorrParams&)   same
//   step(const InteropResource&, float, vec3, vec3)      step(const DeviceParticles&, float, V, V)
//   setGravity(glm::vec3)                                setGravity(V)
//
// V is any type with float members x, y, z (glm::vec3 included, or akua::Vec3).  The reference's
// InteropResource maps a GL buffer and hands its device pointer to the kernels; DeviceParticles is
// that pointer (plus the record stride), so a caller with GL interop passes the mapped pointer and
// a headless caller passes its own device array.  Where the reference reports no errors, every
// call here throws akua::Error on a non-zero status.
#pragma once

#include <akua_pbf.h>

#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>

namespace akua {

struct Vec3 {
    float x, y, z;
};

// Same fields, order and defaults as AkuaEngine::PBFConfig (PBFConfig.h:19-29).
struct PBFConfig {
    float restDensity = 7600.0f;
    float particle_spacing = 0.05f;
    float smoothRadius = 0.1f;
    float spatialHashCellSize = 0.1f;
    float relaxation = 600.0f;
    float vorticityEpsilon = 0.00001f;
    float viscosity = 0.01f;
    int maxNeighbours = 128;
    int solverIterations = 4;
    Vec3 gravity = {0.0f, -9.8f, 0.0f};
};

// Same fields and defaults as AkuaEngine::LambdaCorrParams (PBFConfig.h:10-15).
struct LambdaCorrParams {
    bool enabled = true;
    float k = 0.0001f;
    float n = 4.0f;
    float delta_q = 0.03f;
};

using Particle = akua_particle;  // AkuaEngine::Particle, 108 bytes

class Error : public std::runtime_error {
public:
    Error(const char* what, int status)
        : std::runtime_error(std::string(what) + ": " + akua_pbf_status_string(status)),
          status_(status) {}
    int status() const { return status_; }

private:
    int status_;
};

inline void check(int status, const char* what) {
    if (status != AKUA_OK) throw Error(what, status);
}

// A device array of particle records: what the reference's interop mapping yields.
struct DeviceParticles {
    void* data;
    std::size_t strideBytes = sizeof(akua_particle);
};

class PBFSolver {
public:
    PBFSolver(int numParticles, const PBFConfig& config, const LambdaCorrParams& corrParams) {
        akua_pbf_config c{};
        c.restDensity = config.restDensity;
        c.particle_spacing = config.particle_spacing;
        c.smoothRadius = config.smoothRadius;
        c.spatialHashCellSize = config.spatialHashCellSize;
        c.relaxation = config.relaxation;
        c.vorticityEpsilon = config.vorticityEpsilon;
        c.viscosity = config.viscosity;
        c.maxNeighbours = config.maxNeighbours;
        c.solverIterations = config.solverIterations;
        c.gravity[0] = config.gravity.x;
        c.gravity[1] = config.gravity.y;
        c.gravity[2] = config.gravity.z;
        akua_lambda_corr_params k{};
        k.enabled = corrParams.enabled ? 1 : 0;
        k.k = corrParams.k;
        k.n = corrParams.n;
        k.delta_q = corrParams.delta_q;
        check(akua_pbf_create(numParticles, &c, &k, &h_), "akua_pbf_create");
        n_ = numParticles;
    }
    ~PBFSolver() {
        if (h_) akua_pbf_destroy(h_);
    }
    PBFSolver(const PBFSolver&) = delete;
    PBFSolver& operator=(const PBFSolver&) = delete;
    PBFSolver(PBFSolver&& o) noexcept : h_(std::exchange(o.h_, nullptr)), n_(o.n_) {}
    PBFSolver& operator=(PBFSolver&& o) noexcept {
        if (this != &o) {
            if (h_) akua_pbf_destroy(h_);
            h_ = std::exchange(o.h_, nullptr);
            n_ = o.n_;
        }
        return *this;
    }

    // PBFSolver::step (PBFSolver.cpp:22-78) over a device particle array; asynchronous on the
    // solver's stream.  The records are rewritten in place in hash-sorted order.
    template <class V>
    void step(const DeviceParticles& particles, float deltaTime, const V& boxMin, const V& boxMax) {
        const float lo[3] = {boxMin.x, boxMin.y, boxMin.z};
        const float hi[3] = {boxMax.x, boxMax.y, boxMax.z};
        check(akua_pbf_attach_particles(h_, particles.data, particles.strideBytes),
              "akua_pbf_attach_particles");
        check(akua_pbf_step(h_, deltaTime, lo, hi), "akua_pbf_step");
    }

    // The same step over records in host memory (copied in and out; synchronous).
    template <class V>
    void stepHost(Particle* particles, float deltaTime, const V& boxMin, const V& boxMax) {
        const float lo[3] = {boxMin.x, boxMin.y, boxMin.z};
        const float hi[3] = {boxMax.x, boxMax.y, boxMax.z};
        check(akua_pbf_step_host(h_, particles, sizeof(Particle), deltaTime, lo, hi),
              "akua_pbf_step_host");
    }

    // PBFSolver::setGravity (PBFSolver.h:29-31).
    template <class V>
    void setGravity(const V& gravity) {
        const float g[3] = {gravity.x, gravity.y, gravity.z};
        check(akua_pbf_set_gravity(h_, g), "akua_pbf_set_gravity");
    }

    void setStream(void* cudaStream) { check(akua_pbf_set_stream(h_, cudaStream), "akua_pbf_set_stream"); }
    void setOptions(unsigned options) { check(akua_pbf_set_options(h_, options), "akua_pbf_set_options"); }
    void synchronize() { check(akua_pbf_synchronize(h_), "akua_pbf_synchronize"); }
    akua_pbf_stats stats() {
        akua_pbf_stats s{};
        check(akua_pbf_get_stats(h_, &s), "akua_pbf_get_stats");
        return s;
    }
    int numParticles() const { return n_; }
    akua_pbf* handle() { return h_; }

private:
    akua_pbf* h_ = nullptr;
    int n_ = 0;
};

}  // namespace akua
