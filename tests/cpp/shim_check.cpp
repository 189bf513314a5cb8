// shim_check.cpp -- builds against include/pbf103/pbf_solver.hpp exactly like
// code written for the reference's PBFSolver and checks its behaviour.
//   shim_check cpu   argument validation and exception types (no GPU needed)
//   shim_check gpu   the reference's two-particle and collider scenarios
// Prints "OK" and exits 0 on success.
#include "pbf103/pbf_solver.hpp"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <vector>

static int failures = 0;
#define CHECK(c)                                                            \
    do {                                                                    \
        if (!(c)) {                                                         \
            std::printf("FAILED %s:%d %s\n", __FILE__, __LINE__, #c);       \
            ++failures;                                                     \
        }                                                                   \
    } while (0)

template <class E, class F>
static bool throws(F&& f) {
    try {
        f();
    } catch (const E&) {
        return true;
    } catch (...) {
        return false;
    }
    return false;
}

static SimulationParams validParams() {
    const float pi = 3.14159265358979323846f;
    SimulationParams p{};
    p.dt = 0.1f;
    p.restDensity = 315.0f / (64.0f * pi);
    p.particleMass = 1.0f;
    p.particleRadius = 1.0f;
    p.collisionRestitution = 0.0f;
    p.collisionFriction = 0.03f;
    p.smoothingRadius = 1.0f;
    p.lambdaEpsilon = 0.01f;
    p.solverIterations = 1;
    p.substeps = 1;
    p.gravity = make_float3(0.0f, -9.8f, 0.0f);
    return p;
}

static void cpu_checks() {
    PBFSolver solver;
    const float4 particle = make_float4(0, 0, 0, 1);
    CHECK(throws<std::logic_error>([&] { solver.setParticles(&particle, &particle, 1); }));
    CHECK(throws<std::logic_error>([&] { solver.step(); }));
    CHECK(throws<std::logic_error>([&] { solver.run(); }));
    CHECK(throws<std::out_of_range>([&] { solver.copyPositionsToHost(nullptr, 1); }));
    CHECK(throws<std::invalid_argument>(
        [&] { solver.initialize(0, make_float3(0, 0, 0), make_float3(1, 1, 1), validParams()); }));
    CHECK(throws<std::length_error>([&] {
        solver.initialize(size_t(std::numeric_limits<int>::max()) + 1, make_float3(0, 0, 0),
                          make_float3(1, 1, 1), validParams());
    }));
    SimulationParams bad = validParams();
    bad.dt = std::numeric_limits<float>::quiet_NaN();
    CHECK(throws<std::invalid_argument>(
        [&] { solver.initialize(8, make_float3(0, 0, 0), make_float3(2, 2, 2), bad); }));
    CHECK(throws<std::invalid_argument>(
        [&] { solver.setSpheres({{make_float3(0, 0, 0), 0.0f}}); }));
}

static void gpu_checks() {
    // SeparatesTwoNeighboringParticlesSymmetrically (test/test_pbf_solver.cu:457-503).
    PBFSolver solver;
    SimulationParams p = validParams();
    const float pi = 3.14159265358979323846f;
    p.gravity = make_float3(0, 0, 0);
    p.solverIterations = 3;
    p.restDensity = 1.0f * 315.0f / (64.0f * pi * std::pow(1.0f, 3.0f));
    solver.initialize(2, make_float3(-2, -2, -2), make_float3(12, 12, 12), p);
    const std::vector<float4> pos = {make_float4(4.75f, 5, 5, 3), make_float4(5.25f, 5, 5, 4)};
    const std::vector<float4> vel = {make_float4(0, 0, 0, 7), make_float4(0, 0, 0, 8)};
    solver.setParticles(pos.data(), vel.data(), pos.size());
    solver.step();
    std::vector<float4> rp(2), rv(2);
    solver.copyPositionsToHost(rp.data(), 2);
    solver.copyVelocitiesToHost(rv.data(), 2);
    CHECK(rp[0].x < 4.75f && rp[1].x > 5.25f);
    CHECK(std::fabs(rp[0].x + rp[1].x - 10.0f) < 1e-5f);
    CHECK(rp[0].w == 3.0f && rv[1].w == 8.0f);
    CHECK(rv[0].x < 0.0f && rv[1].x > 0.0f);

    // ForwardsSphereColliderAndCanClearIt (test/test_pbf_solver.cu:744-770).
    PBFSolver s2;
    SimulationParams c = validParams();
    c.particleRadius = 0.25f;
    c.smoothingRadius = 0.5f;
    c.restDensity = 315.0f / (64.0f * pi * std::pow(0.5f, 3.0f));
    c.solverIterations = 4;
    c.gravity = make_float3(0, 0, 0);
    c.collisionFriction = 0.0f;
    s2.initialize(1, make_float3(-2, -2, -2), make_float3(12, 12, 12), c);
    s2.setSpheres({{make_float3(3, 5, 5), 0.5f}});
    const float4 p0 = make_float4(4, 5, 5, 1), v0 = make_float4(-4, 0, 0, 2);
    s2.setParticles(&p0, &v0, 1);
    s2.step();
    float4 q{}, w{};
    s2.copyPositionsToHost(&q, 1);
    s2.copyVelocitiesToHost(&w, 1);
    CHECK(std::fabs(q.x - 3.75f) < 1e-5f && std::fabs(w.x) < 1e-5f && w.w == 2.0f);
    s2.setSpheres({});
    s2.setParticles(&p0, &v0, 1);
    s2.step();
    s2.copyPositionsToHost(&q, 1);
    CHECK(std::fabs(q.x - 3.6f) < 1e-5f);

    // RejectsNeighborOverflowBeforeConstraintSolve (test/test_pbf_solver.cu:708-725).
    PBFSolver s3;
    SimulationParams o = validParams();
    o.gravity = make_float3(0, 0, 0);
    o.particleRadius = 0.01f;
    s3.initialize(258, make_float3(-2, -2, -2), make_float3(12, 12, 12), o);
    const std::vector<float4> many(258, make_float4(5, 5, 5, 1));
    const std::vector<float4> zero(258, make_float4(0, 0, 0, 0));
    s3.setParticles(many.data(), zero.data(), many.size());
    CHECK(throws<std::overflow_error>([&] { s3.step(); }));
}

int main(int argc, char** argv) {
    const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
    cpu_checks();
    if (gpu) gpu_checks();
    if (failures) return 1;
    std::printf("OK\n");
    return 0;
}
