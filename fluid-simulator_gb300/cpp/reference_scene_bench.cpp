// reference_scene_bench.cpp -- the reference's own benchmark scene driven
// through the C++ shim (include/pbf103/pbf_solver.hpp), timed the way the
// reference's driver times it (benchmark/pbf_benchmark.cu:117-212).
//
// Scene (benchmark/pbf_benchmark.cu:20-114): 262,144 particles in 128 x 64
// layers at spacing 0.06 filled down from y = 3.75 and centred in x and z in
// the container (0,0,0)-(8.2,4,4.2); one box (centre (2.4,0.675,2.1), half
// extents (0.65,0.625,0.75)) and one sphere (centre (5.7,0.8,2.1), radius
// 0.75); dt 1/60, 2 substeps, 4 iterations.
//
// Protocol: 10 warm-up frames, then 5 repetitions of 60 frames, each from the
// initial state; every PBFSolver::step() is timed on the host with
// std::chrono::steady_clock (step() returns when the frame is done on the GPU);
// the repetition with the median average is reported.
//
// Usage: reference_scene_bench            run the benchmark, print one JSON line
//        reference_scene_bench --dump F   write the initial positions (float4,
//                                         binary) to F and exit; no GPU needed
#include "pbf103/pbf_solver.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <numeric>
#include <vector>

namespace {

constexpr size_t kLayerX = 128, kLayerZ = 64;
constexpr size_t kParticles = 262144;
constexpr float kSpacing = 0.06f;
constexpr float kTop = 3.75f;
constexpr size_t kWarmup = 10, kFrames = 60, kReps = 5;

const float3 kLo = make_float3(0.0f, 0.0f, 0.0f);
const float3 kHi = make_float3(8.2f, 4.0f, 4.2f);

SimulationParams scene_params() {
    SimulationParams p{};
    p.dt = 1.0f / 60.0f;
    p.restDensity = 1000.0f;
    p.particleMass = p.restDensity * kSpacing * kSpacing * kSpacing;
    p.particleRadius = 0.025f;
    p.collisionRestitution = 0.0f;
    p.collisionFriction = 0.03f;
    p.smoothingRadius = 0.12f;
    p.lambdaEpsilon = 100.0f;
    p.solverIterations = 4;
    p.substeps = 2;
    p.gravity = make_float3(0.0f, -9.81f, 0.0f);
    p.scorrK = 0.0001f;
    p.scorrN = 4;
    p.scorrDeltaQ = 0.036f;
    p.xsphViscosity = 0.00001f;
    p.vorticityStrength = 0.00001f;
    return p;
}

// Layer by layer from the top, z rows, x fastest; single-precision products
// and sums (the build disables floating-point contraction).
std::vector<float4> scene_positions() {
    const size_t layers = kParticles / (kLayerX * kLayerZ);
    const float x0 = (kHi.x - static_cast<float>(kLayerX - 1) * kSpacing) * 0.5f;
    const float z0 = (kHi.z - static_cast<float>(kLayerZ - 1) * kSpacing) * 0.5f;
    std::vector<float4> pos;
    pos.reserve(kParticles);
    for (size_t y = 0; y < layers; ++y)
        for (size_t z = 0; z < kLayerZ; ++z)
            for (size_t x = 0; x < kLayerX; ++x)
                pos.push_back(make_float4(x0 + static_cast<float>(x) * kSpacing,
                                          kTop - static_cast<float>(y) * kSpacing,
                                          z0 + static_cast<float>(z) * kSpacing, 1.0f));
    return pos;
}

struct Run {
    std::vector<double> ms;
    double total = 0.0, mean = 0.0;
};

Run timed_run(PBFSolver& s) {
    Run r;
    r.ms.reserve(kFrames);
    for (size_t f = 0; f < kFrames; ++f) {
        const auto t0 = std::chrono::steady_clock::now();
        s.step();
        const auto t1 = std::chrono::steady_clock::now();
        r.ms.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
    }
    r.total = std::accumulate(r.ms.begin(), r.ms.end(), 0.0);
    r.mean = r.total / static_cast<double>(kFrames);
    return r;
}

double p95(std::vector<double> v) {
    std::sort(v.begin(), v.end());
    const size_t k = static_cast<size_t>(std::ceil(0.95 * static_cast<double>(v.size()))) - 1;
    return v[k];
}

int bench() {
    const SimulationParams prm = scene_params();
    const std::vector<float4> pos = scene_positions();
    const std::vector<float4> vel(kParticles, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    PBFSolver s;
    s.initialize(kParticles, kLo, kHi, prm);
    s.setBoxes({BoxCollider{make_float3(2.4f, 0.675f, 2.1f), make_float3(0.65f, 0.625f, 0.75f)}});
    s.setSpheres({SphereCollider{make_float3(5.7f, 0.8f, 2.1f), 0.75f}});
    s.setParticles(pos.data(), vel.data(), kParticles);
    s.run(kWarmup);
    std::vector<Run> runs;
    for (size_t r = 0; r < kReps; ++r) {
        s.setParticles(pos.data(), vel.data(), kParticles);
        runs.push_back(timed_run(s));
    }
    std::vector<size_t> order(kReps);
    std::iota(order.begin(), order.end(), size_t(0));
    std::sort(order.begin(), order.end(),
              [&](size_t a, size_t b) { return runs[a].mean < runs[b].mean; });
    const Run& med = runs[order[kReps / 2]];
    double avg = 0.0, var = 0.0;
    for (const Run& r : runs) avg += r.mean / static_cast<double>(kReps);
    for (const Run& r : runs) var += (r.mean - avg) * (r.mean - avg) / static_cast<double>(kReps);
    const double sec = med.total / 1000.0;
    const double pf = static_cast<double>(kParticles * kFrames) / sec;
    std::printf("{\"particles\": %zu, \"frames\": %zu, \"repetitions\": %zu, \"warmup_frames\": %zu, "
                "\"substeps\": %d, \"ms_per_frame\": %.6f, \"p95_ms\": %.6f, \"min_ms\": %.6f, "
                "\"max_ms\": %.6f, \"run_average_stddev_ms\": %.6f, "
                "\"particle_frames_per_s\": %.1f, \"particle_substeps_per_s\": %.1f, \"runs_ms\": [",
                kParticles, kFrames, kReps, kWarmup, prm.substeps, med.mean, p95(med.ms),
                *std::min_element(med.ms.begin(), med.ms.end()),
                *std::max_element(med.ms.begin(), med.ms.end()), std::sqrt(var), pf,
                pf * static_cast<double>(prm.substeps));
    for (size_t r = 0; r < kReps; ++r) std::printf("%s%.6f", r ? ", " : "", runs[r].total);
    std::printf("]}\n");
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    try {
        if (argc == 3 && std::strcmp(argv[1], "--dump") == 0) {
            const std::vector<float4> pos = scene_positions();
            std::FILE* f = std::fopen(argv[2], "wb");
            if (!f) return 2;
            const size_t w = std::fwrite(pos.data(), sizeof(float4), pos.size(), f);
            std::fclose(f);
            return w == pos.size() ? 0 : 2;
        }
        return bench();
    } catch (const std::exception& e) {
        std::fprintf(stderr, "reference_scene_bench: %s\n", e.what());
        return 1;
    }
}
