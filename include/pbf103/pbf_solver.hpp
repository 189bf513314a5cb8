// pbf103/pbf_solver.hpp -- header-only C++ shim with the reference solver's API.
//
// Same class name, method names, argument types and exception types as
// include/pbf/pbf_solver.hpp of DusanCojic/Fluid-Simulator (PBFSolver,
// SimulationParams, SphereCollider, BoxCollider, PlaneCollider), implemented
// over the C ABI of pbf103.h.  Code written against the reference builds
// against this header and links libpbf103.so instead of the reference's
// static library.
#ifndef PBF103_PBF_SOLVER_HPP
#define PBF103_PBF_SOLVER_HPP

#include <cuda_runtime.h>  // float3/float4 and make_float3/4, as the reference headers

#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

#include "pbf103.h"

// include/pbf/simulation_params.hpp:6-29
struct SimulationParams {
    float dt;
    float restDensity;
    float particleMass;
    float particleRadius;
    float collisionRestitution;
    float collisionFriction;
    float smoothingRadius;
    float lambdaEpsilon;
    int solverIterations;
    int substeps;
    float3 gravity;
    float scorrK;
    int scorrN;
    float scorrDeltaQ;
    float xsphViscosity;
    float vorticityStrength;
};

// include/pbf/colliders.hpp:8-24
struct Container {
    float3 min;
    float3 max;
};
struct SphereCollider {
    float3 center;
    float radius;
};
struct BoxCollider {
    float3 center;
    float3 halfExtents;
};
struct PlaneCollider {
    float3 point;
    float3 normal;
};

static_assert(sizeof(SimulationParams) == sizeof(pbf_params), "params layout");
static_assert(sizeof(SphereCollider) == sizeof(pbf_sphere), "sphere layout");
static_assert(sizeof(BoxCollider) == sizeof(pbf_box), "box layout");
static_assert(sizeof(PlaneCollider) == sizeof(pbf_plane), "plane layout");
static_assert(sizeof(float4) == sizeof(pbf_float4), "float4 layout");

namespace pbf103_detail {

// Rethrows a status as the exception type the reference throws.
inline void rethrow(pbf_status st, const char* msg) {
    const std::string m = msg ? msg : "";
    switch (st) {
        case PBF_OK: return;
        case PBF_ERR_INVALID_ARGUMENT: throw std::invalid_argument(m);
        case PBF_ERR_LOGIC: throw std::logic_error(m);
        case PBF_ERR_OUT_OF_RANGE: throw std::out_of_range(m);
        case PBF_ERR_LENGTH: throw std::length_error(m);
        case PBF_ERR_OVERFLOW: throw std::overflow_error(m);
        default: throw std::runtime_error(m);
    }
}

inline pbf_float3 f3(float3 v) { return pbf_float3{v.x, v.y, v.z}; }

}  // namespace pbf103_detail

class PBFSolver {
public:
    PBFSolver() {
        pbf103_detail::rethrow(pbf_solver_create(&h_, -1), pbf_global_last_error());
    }
    ~PBFSolver() { pbf_solver_destroy(h_); }
    PBFSolver(const PBFSolver&) = delete;
    PBFSolver& operator=(const PBFSolver&) = delete;
    PBFSolver(PBFSolver&& o) noexcept : h_(o.h_) { o.h_ = nullptr; }
    PBFSolver& operator=(PBFSolver&& o) noexcept {
        if (this != &o) {
            pbf_solver_destroy(h_);
            h_ = o.h_;
            o.h_ = nullptr;
        }
        return *this;
    }

    void initialize(size_t maxParticles, float3 minBounds, float3 maxBounds,
                    const SimulationParams& params) {
        check(pbf_initialize(h_, maxParticles, pbf103_detail::f3(minBounds),
                             pbf103_detail::f3(maxBounds),
                             reinterpret_cast<const pbf_params*>(&params)));
    }

    void setParticles(const float4* positions, const float4* velocities, size_t particleCount) {
        check(pbf_set_particles(h_, reinterpret_cast<const pbf_float4*>(positions),
                                reinterpret_cast<const pbf_float4*>(velocities),
                                particleCount));
    }

    void setSpheres(const std::vector<SphereCollider>& spheres) {
        check(pbf_set_spheres(h_, reinterpret_cast<const pbf_sphere*>(spheres.data()),
                              spheres.size()));
    }
    void setBoxes(const std::vector<BoxCollider>& boxes) {
        check(pbf_set_boxes(h_, reinterpret_cast<const pbf_box*>(boxes.data()), boxes.size()));
    }
    void setPlanes(const std::vector<PlaneCollider>& planes) {
        check(pbf_set_planes(h_, reinterpret_cast<const pbf_plane*>(planes.data()),
                             planes.size()));
    }

    void step() { check(pbf_step(h_)); }
    void run() { check(pbf_run(h_, 1)); }
    void run(std::size_t frameCount) { check(pbf_run(h_, frameCount)); }

    void copyPositionsToHost(float4* positions, size_t particleCount) const {
        check(pbf_copy_positions(h_, reinterpret_cast<pbf_float4*>(positions), particleCount));
    }
    void copyVelocitiesToHost(float4* velocities, size_t particleCount) const {
        check(pbf_copy_velocities(h_, reinterpret_cast<pbf_float4*>(velocities), particleCount));
    }

    // Not in the reference: the underlying C handle.
    pbf_solver* handle() const { return h_; }

private:
    void check(pbf_status st) const { pbf103_detail::rethrow(st, pbf_last_error(h_)); }
    pbf_solver* h_ = nullptr;
};

#endif  // PBF103_PBF_SOLVER_HPP
