// ref_driver.cu -- runs the reference's own CUDA kernels on the GPU.
//
// TEST INFRASTRUCTURE ONLY: the comparison point "reference CUDA solver".
// The device code is the reference's (DusanCojic/Fluid-Simulator src/pbf/*.cu
// compiled by oracle/build_ref.py into oracle/_ref/*.fatbin, Release flags,
// sm_103a).  This file restates the host side of PBFSolver
// (src/pbf/pbf_solver.cu:23-379), SpatialGrid::build (src/pbf/spatial_grid.cu:139-226)
// and CollisionSystem::solve/resolveVelocities (src/pbf/collision_system.cu:133-218):
// the same buffers, launch shapes (<<<ceil(N/256), 256>>>, default stream),
// CUB radix sort over all 32 key bits, blocking memsets/copies and the host
// synchronisations after every grid build, every neighbour search and every
// collision pass.  Kernels are looked up by their mangled names and launched
// through the driver API.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cub/cub.cuh>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <utility>
#include <vector>

// Parameter and container layouts of the reference (SimulationParams,
// Container).  Kept outside the anonymous namespace: the extern "C" entry
// points take them, and a parameter type with internal linkage would give
// those functions internal linkage too.
struct RefParams {  // SimulationParams layout
    float dt, restDensity, particleMass, particleRadius, collisionRestitution, collisionFriction,
        smoothingRadius, lambdaEpsilon;
    int solverIterations, substeps;
    float3 gravity;
    float scorrK;
    int scorrN;
    float scorrDeltaQ, xsphViscosity, vorticityStrength;
};
struct RefContainer {
    float3 min, max;
};

namespace {

constexpr int kBlock = 256;
constexpr int kMaxNeighbors = 256;

enum { REF_OK = 0, REF_ERR = 1, REF_OVERFLOW = 2, REF_NOT_CONVERGED = 3 };

std::string g_err;

bool ok(cudaError_t e) {
    if (e != cudaSuccess) {
        g_err = cudaGetErrorString(e);
        return false;
    }
    return true;
}
bool okd(CUresult r) {
    if (r != CUDA_SUCCESS) {
        const char* s = nullptr;
        cuGetErrorString(r, &s);
        g_err = s ? s : "driver error";
        return false;
    }
    return true;
}

template <class T>
T* dalloc(size_t n) {
    T* p = nullptr;
    if (n && cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return nullptr;
    return p;
}

struct Kernels {
    CUmodule mods[5] = {};
    CUfunction integrate, keys, ranges, gather, search, lambda, delta, apply, update, xsph, vort,
        confine, ids, scatter, container, spheres, boxes, planes, resolve;
};

bool load_module(const std::string& path, CUmodule* m) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        g_err = "cannot open " + path;
        return false;
    }
    std::vector<char> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    return okd(cuModuleLoadData(m, bytes.data()));
}

bool get(CUmodule m, const char* name, CUfunction* f) { return okd(cuModuleGetFunction(f, m, name)); }

}  // namespace

struct RefSolver {
    int maxNbCap = kMaxNeighbors;  // kMaxNeighbors, or a raised capacity
    Kernels k;
    size_t maxParticles = 0, n = 0, stride = 0;
    RefParams prm{};
    float3 mn{}, mx{};
    int3 gridSize{};
    size_t numCells = 0;
    // PBFSolver buffers (include/pbf/pbf_solver.hpp:45-66)
    float4 *pos = nullptr, *pred = nullptr, *vel = nullptr, *xsphv = nullptr, *vin = nullptr,
           *vort = nullptr, *rpos = nullptr, *rpred = nullptr, *rvel = nullptr, *rvin = nullptr,
           *delta = nullptr;
    uint32_t *sid = nullptr, *rsid = nullptr, *nbr = nullptr;
    int *cnt = nullptr, *overflow = nullptr;
    float* lam = nullptr;
    // SpatialGrid buffers (include/pbf/spatial_grid.cuh:39-56)
    uint32_t *keys = nullptr, *idx = nullptr, *skeys = nullptr, *sidx = nullptr;
    int *cs = nullptr, *ce = nullptr;
    void* temp = nullptr;
    size_t tempBytes = 0;
    // CollisionSystem buffers
    RefContainer* cont = nullptr;
    int* flag = nullptr;
    float4* colliders = nullptr;  // spheres | boxes | planes, packed like the host structs
    size_t ns = 0, nb = 0, np = 0;
    void *dSpheres = nullptr, *dBoxes = nullptr, *dPlanes = nullptr;

    void release() {
        void* ptrs[] = {pos, pred, vel, xsphv, vin, vort, rpos, rpred, rvel, rvin, delta, sid,
                        rsid, nbr, cnt, overflow, lam, keys, idx, skeys, sidx, cs, ce, temp,
                        cont, flag, dSpheres, dBoxes, dPlanes};
        for (void* p : ptrs)
            if (p) cudaFree(p);
    }

    bool launch(CUfunction f, size_t count, void** args) {
        const unsigned grid = static_cast<unsigned>((count + kBlock - 1) / kBlock);
        if (!okd(cuLaunchKernel(f, grid, 1, 1, kBlock, 1, 1, 0, nullptr, args, nullptr)))
            return false;
        return ok(cudaGetLastError());
    }

    // SpatialGrid::build (src/pbf/spatial_grid.cu:139-226).
    bool build(const float4* p, size_t count) {
        if (count == 0) {
            return ok(cudaMemset(cs, 0xff, numCells * sizeof(int))) &&
                   ok(cudaMemset(ce, 0xff, numCells * sizeof(int))) &&
                   ok(cudaDeviceSynchronize());
        }
        float cell = prm.smoothingRadius;
        void* a1[] = {&p, &keys, &idx, &count, &mn, &cell, &gridSize};
        if (!launch(k.keys, count, a1)) return false;
        size_t bytes = tempBytes;
        if (!ok(cub::DeviceRadixSort::SortPairs(temp, bytes, keys, skeys, idx, sidx,
                                                static_cast<int>(count))))
            return false;
        if (!ok(cudaMemset(cs, 0xff, numCells * sizeof(int))) ||
            !ok(cudaMemset(ce, 0xff, numCells * sizeof(int))))
            return false;
        void* a2[] = {&skeys, &cs, &ce, &count};
        if (!launch(k.ranges, count, a2)) return false;
        return ok(cudaDeviceSynchronize());
    }

    // PBFSolver::reorderWorkingSet (src/pbf/pbf_solver.cu:154-172).
    bool reorder() {
        void* a[] = {&sidx, &pos, &pred, &vel, &vin, &sid, &rpos, &rpred, &rvel, &rvin, &rsid, &n};
        if (!launch(k.gather, n, a)) return false;
        std::swap(pos, rpos);
        std::swap(pred, rpred);
        std::swap(vel, rvel);
        std::swap(vin, rvin);
        std::swap(sid, rsid);
        return true;
    }

    int search() {
        if (!ok(cudaMemset(overflow, 0, sizeof(int)))) return REF_ERR;
        float cell = prm.smoothingRadius, h = prm.smoothingRadius;
        int maxNb = maxNbCap;
        void* a[] = {&pred, &cs, &ce, &gridSize, &mn, &cell, &n, &h, &nbr, &cnt, &maxNb, &stride,
                     &overflow};
        if (!launch(k.search, n, a)) return REF_ERR;
        int of = 0;
        if (!ok(cudaMemcpy(&of, overflow, sizeof(int), cudaMemcpyDeviceToHost))) return REF_ERR;
        return of ? REF_OVERFLOW : REF_OK;
    }

    // CollisionSystem::solve (src/pbf/collision_system.cu:133-172).
    int collide() {
        float r = prm.particleRadius;
        for (int it = 0; it < 32; ++it) {
            if (!ok(cudaMemset(flag, 0, sizeof(int)))) return REF_ERR;
            void* a0[] = {&pred, &n, &cont, &r, &flag};
            if (!launch(k.container, n, a0)) return REF_ERR;
            if (ns) {
                void* a[] = {&pred, &n, &dSpheres, &ns, &r, &flag};
                if (!launch(k.spheres, n, a)) return REF_ERR;
            }
            if (nb) {
                void* a[] = {&pred, &n, &dBoxes, &nb, &r, &flag};
                if (!launch(k.boxes, n, a)) return REF_ERR;
            }
            if (np) {
                void* a[] = {&pred, &n, &dPlanes, &np, &r, &flag};
                if (!launch(k.planes, n, a)) return REF_ERR;
            }
            int made = 0;
            if (!ok(cudaMemcpy(&made, flag, sizeof(int), cudaMemcpyDeviceToHost))) return REF_ERR;
            if (!made) return REF_OK;
        }
        return REF_NOT_CONVERGED;
    }

    // PBFSolver::step (src/pbf/pbf_solver.cu:186-328).
    int step() {
        if (n == 0) return REF_OK;
        const float sub = prm.dt / static_cast<float>(prm.substeps);
        int ni = static_cast<int>(n);
        int maxNb = maxNbCap;
        for (int s = 0; s < prm.substeps; ++s) {
            float3 g = prm.gravity;
            float dt = sub;
            void* ai[] = {&pos, &pred, &vel, &ni, &dt, &g};
            if (!launch(k.integrate, n, ai)) return REF_ERR;
            if (!ok(cudaMemcpy(vin, vel, n * sizeof(float4), cudaMemcpyDeviceToDevice)))
                return REF_ERR;
            for (int it = 0; it < prm.solverIterations; ++it) {
                if (!build(pred, n) || !reorder()) return REF_ERR;
                int st = search();
                if (st != REF_OK) return st;
                float h = prm.smoothingRadius, m = prm.particleMass, rho = prm.restDensity,
                      eps = prm.lambdaEpsilon;
                void* al[] = {&pred, &nbr, &cnt, &maxNb, &n, &h, &m, &rho, &eps, &lam, &stride};
                if (!launch(k.lambda, n, al)) return REF_ERR;
                float kk = prm.scorrK, dq = prm.scorrDeltaQ;
                int nn = prm.scorrN;
                void* ad[] = {&pred, &nbr, &cnt, &maxNb, &lam, &n, &h, &m, &rho, &kk, &nn, &dq,
                              &delta, &stride};
                if (!launch(k.delta, n, ad)) return REF_ERR;
                void* aa[] = {&pred, &delta, &n};
                if (!launch(k.apply, n, aa)) return REF_ERR;
                st = collide();
                if (st != REF_OK) return st;
            }
            if (prm.xsphViscosity != 0.0f || prm.vorticityStrength != 0.0f) {
                if (!build(pred, n) || !reorder()) return REF_ERR;
                int st = search();
                if (st != REF_OK) return st;
            }
            float inv = 1.0f / sub;
            void* au[] = {&pos, &pred, &vel, &n, &inv};
            if (!launch(k.update, n, au)) return REF_ERR;
            float h = prm.smoothingRadius;
            if (prm.xsphViscosity != 0.0f) {
                float c = prm.xsphViscosity;
                void* ax[] = {&pred, &nbr, &cnt, &maxNb, &vel, &xsphv, &n, &h, &c, &stride};
                if (!launch(k.xsph, n, ax)) return REF_ERR;
                std::swap(vel, xsphv);
            }
            if (prm.vorticityStrength != 0.0f) {
                void* av[] = {&pred, &vel, &nbr, &cnt, &maxNb, &n, &h, &vort, &stride};
                if (!launch(k.vort, n, av)) return REF_ERR;
                float e = prm.vorticityStrength;
                void* ac[] = {&pred, &nbr, &cnt, &maxNb, &vort, &vel, &xsphv, &n, &h, &dt, &e,
                              &stride};
                if (!launch(k.confine, n, ac)) return REF_ERR;
                std::swap(vel, xsphv);
            }
            float r = prm.particleRadius, e = prm.collisionRestitution, f = prm.collisionFriction;
            void* ar[] = {&pos, &vin, &vel, &n, &cont, &dSpheres, &ns, &dBoxes, &nb, &dPlanes, &np,
                          &r, &e, &f};
            if (!launch(k.resolve, n, ar)) return REF_ERR;
        }
        return ok(cudaDeviceSynchronize()) ? REF_OK : REF_ERR;
    }
};

extern "C" {

const char* ref_last_error(void) { return g_err.c_str(); }

RefSolver* ref_create(const char* fatbin_dir) {
    if (!ok(cudaFree(nullptr))) return nullptr;  // create the primary context
    RefSolver* s = new RefSolver();
    const std::string d = fatbin_dir;
    const char* units[5] = {"integration", "neighbors", "pbf_solver_kernels", "collision_kernels",
                            "spatial_grid"};
    for (int i = 0; i < 5; ++i)
        if (!load_module(d + "/" + units[i] + ".fatbin", &s->k.mods[i])) {
            delete s;
            return nullptr;
        }
    Kernels& k = s->k;
    const bool good =
        get(k.mods[0], "_Z9integratePK6float4PS_S2_if6float3", &k.integrate) &&
        get(k.mods[1], "_Z13findNeighborsPK6float4PKiS3_4int36float3fmfPjPiimS7_", &k.search) &&
        get(k.mods[2], "_Z13computeLambdaPK6float4PKjPKiimffffPfm", &k.lambda) &&
        get(k.mods[2], "_Z20computeDeltaPositionPK6float4PKjPKiiPKfmffffifPS_m", &k.delta) &&
        get(k.mods[2], "_Z18applyDeltaPositionP6float4PKS_m", &k.apply) &&
        get(k.mods[2], "_Z25updateVelocityAndPositionP6float4PKS_S0_mf", &k.update) &&
        get(k.mods[2], "_Z18applyXsphViscosityPK6float4PKjPKiiS1_PS_mffm", &k.xsph) &&
        get(k.mods[2], "_Z16computeVorticityPK6float4S1_PKjPKiimfPS_m", &k.vort) &&
        get(k.mods[2], "_Z25applyVorticityConfinementPK6float4PKjPKiiS1_S1_PS_mfffm", &k.confine) &&
        get(k.mods[2], "_Z17gatherSolverStatePKjPK6float4S3_S3_S3_S0_PS1_S4_S4_S4_Pjm", &k.gather) &&
        get(k.mods[2], "_Z27initializeStableParticleIdsPjm", &k.ids) &&
        get(k.mods[2], "_Z23scatterFloat4ByStableIdPK6float4PKjPS_m", &k.scatter) &&
        get(k.mods[3], "_Z20solveContainerKernelP6float4mPK9ContainerfPi", &k.container) &&
        get(k.mods[3], "_Z18solveSpheresKernelP6float4mPK14SphereCollidermfPi", &k.spheres) &&
        get(k.mods[3], "_Z16solveBoxesKernelP6float4mPK11BoxCollidermfPi", &k.boxes) &&
        get(k.mods[3], "_Z17solvePlanesKernelP6float4mPK13PlaneCollidermfPi", &k.planes) &&
        get(k.mods[3],
            "_Z23resolveVelocitiesKernelPK6float4S1_PS_mPK9ContainerPK14SphereCollidermPK11BoxCollidermPK13PlaneCollidermfff",
            &k.resolve) &&
        get(k.mods[4], "_Z19computeParticleKeysPK6float4PjS2_m6float3f4int3", &k.keys) &&
        get(k.mods[4], "_Z15buildCellRangesPKjPiS1_m", &k.ranges);
    if (!good) {
        delete s;
        return nullptr;
    }
    return s;
}

void ref_destroy(RefSolver* s) {
    if (!s) return;
    s->release();
    for (auto m : s->k.mods)
        if (m) cuModuleUnload(m);
    delete s;
}

// PBFSolver::initialize allocations (validation is the product's job), with
// the list capacity `cap`.
static int init_alloc(RefSolver* s, size_t maxParticles, float3 mn, float3 mx, const RefParams* p,
                      int cap) {
    s->maxNbCap = cap;
    s->release();
    s->maxParticles = maxParticles;
    s->prm = *p;
    s->mn = mn;
    s->mx = mx;
    const float cell = p->smoothingRadius;
    const float lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z};
    int d[3];
    for (int a = 0; a < 3; ++a)
        d[a] = static_cast<int>(std::ceil((double(hi[a]) - double(lo[a])) / double(cell)));
    s->gridSize = make_int3(d[0], d[1], d[2]);
    s->numCells = size_t(d[0]) * size_t(d[1]) * size_t(d[2]);
    s->stride = (maxParticles + kBlock - 1) / kBlock * kBlock;
    const size_t N = maxParticles;
    bool good = (s->pos = dalloc<float4>(N)) && (s->pred = dalloc<float4>(N)) &&
                (s->vel = dalloc<float4>(N)) && (s->xsphv = dalloc<float4>(N)) &&
                (s->vin = dalloc<float4>(N)) && (s->vort = dalloc<float4>(N)) &&
                (s->rpos = dalloc<float4>(N)) && (s->rpred = dalloc<float4>(N)) &&
                (s->rvel = dalloc<float4>(N)) && (s->rvin = dalloc<float4>(N)) &&
                (s->delta = dalloc<float4>(N)) && (s->sid = dalloc<uint32_t>(N)) &&
                (s->rsid = dalloc<uint32_t>(N)) &&
                (s->nbr = dalloc<uint32_t>(s->stride * size_t(s->maxNbCap))) &&
                (s->cnt = dalloc<int>(N)) && (s->overflow = dalloc<int>(1)) &&
                (s->lam = dalloc<float>(N)) && (s->keys = dalloc<uint32_t>(N)) &&
                (s->idx = dalloc<uint32_t>(N)) && (s->skeys = dalloc<uint32_t>(N)) &&
                (s->sidx = dalloc<uint32_t>(N)) && (s->cs = dalloc<int>(s->numCells)) &&
                (s->ce = dalloc<int>(s->numCells)) && (s->cont = dalloc<RefContainer>(1)) &&
                (s->flag = dalloc<int>(1));
    if (!good) {
        g_err = "allocation failed";
        return REF_ERR;
    }
    s->tempBytes = 0;
    if (!ok(cub::DeviceRadixSort::SortPairs(nullptr, s->tempBytes, s->keys, s->skeys, s->idx,
                                            s->sidx, static_cast<int>(N))))
        return REF_ERR;
    if (!ok(cudaMalloc(&s->temp, s->tempBytes))) return REF_ERR;
    RefContainer c{mn, mx};
    if (!ok(cudaMemcpy(s->cont, &c, sizeof(c), cudaMemcpyHostToDevice))) return REF_ERR;
    s->n = 0;
    return REF_OK;
}

// spheres: (cx, cy, cz, r) x ns; boxes: 6 floats x nb; planes: 6 floats x np.
int ref_initialize(RefSolver* s, size_t maxParticles, float3 mn, float3 mx, const RefParams* p) {
    return init_alloc(s, maxParticles, mn, mx, p, kMaxNeighbors);
}

// The same with the neighbour capacity raised from kMaxNeighbors, as a patched
// reference build would have it (src/pbf/pbf_solver.cu:12); the kernels take
// the capacity as an argument.
int ref_initialize_ex(RefSolver* s, size_t maxParticles, float3 mn, float3 mx, const RefParams* p,
                      int maxNeighbors) {
    if (maxNeighbors <= 0) {
        g_err = "maxNeighbors must be positive";
        return REF_ERR;
    }
    return init_alloc(s, maxParticles, mn, mx, p, maxNeighbors);
}

int ref_set_colliders(RefSolver* s, const float* sp, size_t ns, const float* bx, size_t nb,
                      const float* pl, size_t np) {
    for (void* p : {s->dSpheres, s->dBoxes, s->dPlanes})
        if (p) cudaFree(p);
    s->dSpheres = s->dBoxes = s->dPlanes = nullptr;
    s->ns = ns;
    s->nb = nb;
    s->np = np;
    if (ns && (!ok(cudaMalloc(&s->dSpheres, ns * 16)) ||
               !ok(cudaMemcpy(s->dSpheres, sp, ns * 16, cudaMemcpyHostToDevice))))
        return REF_ERR;
    if (nb && (!ok(cudaMalloc(&s->dBoxes, nb * 24)) ||
               !ok(cudaMemcpy(s->dBoxes, bx, nb * 24, cudaMemcpyHostToDevice))))
        return REF_ERR;
    if (np && (!ok(cudaMalloc(&s->dPlanes, np * 24)) ||
               !ok(cudaMemcpy(s->dPlanes, pl, np * 24, cudaMemcpyHostToDevice))))
        return REF_ERR;
    return REF_OK;
}

int ref_set_particles(RefSolver* s, const float4* p, const float4* v, size_t n) {
    if (n > s->maxParticles) return REF_ERR;
    s->n = n;
    if (!n) return REF_OK;
    if (!ok(cudaMemcpy(s->pos, p, n * 16, cudaMemcpyHostToDevice)) ||
        !ok(cudaMemcpy(s->vel, v, n * 16, cudaMemcpyHostToDevice)))
        return REF_ERR;
    void* a[] = {&s->sid, &n};
    if (!s->launch(s->k.ids, n, a)) return REF_ERR;
    return ok(cudaDeviceSynchronize()) ? REF_OK : REF_ERR;
}

int ref_step(RefSolver* s) { return s->step(); }

// Wall time of `frames` step() calls, steady_clock around each call
// (benchmark/pbf_benchmark.cu:121-137).
int ref_time_steps(RefSolver* s, size_t frames, double* ms) {
    double total = 0.0;
    for (size_t f = 0; f < frames; ++f) {
        const auto t0 = std::chrono::steady_clock::now();
        const int st = s->step();
        const auto t1 = std::chrono::steady_clock::now();
        if (st != REF_OK) return st;
        total += std::chrono::duration<double, std::milli>(t1 - t0).count();
    }
    *ms = total;
    return REF_OK;
}

int ref_copy(RefSolver* s, int velocities, float4* out, size_t n) {
    if (n != s->n) return REF_ERR;
    if (!n) return REF_OK;
    float4* src = velocities ? s->vel : s->pos;
    float4* dst = velocities ? s->rvel : s->rpos;
    void* a[] = {&src, &s->sid, &dst, &n};
    if (!s->launch(s->k.scatter, n, a)) return REF_ERR;
    return ok(cudaMemcpy(out, dst, n * 16, cudaMemcpyDeviceToHost)) ? REF_OK : REF_ERR;
}

// SpatialGrid::build on caller positions (current order): sorted keys,
// sorted indices, cellStart, cellEnd.
int ref_grid_build(RefSolver* s, const float4* p, size_t n, uint32_t* skeys, uint32_t* sidx,
                   int* cs, int* ce) {
    if (n > s->maxParticles) return REF_ERR;
    if (n && !ok(cudaMemcpy(s->rpred, p, n * 16, cudaMemcpyHostToDevice))) return REF_ERR;
    if (!s->build(s->rpred, n)) return REF_ERR;
    if (n && (!ok(cudaMemcpy(skeys, s->skeys, n * 4, cudaMemcpyDeviceToHost)) ||
              !ok(cudaMemcpy(sidx, s->sidx, n * 4, cudaMemcpyDeviceToHost))))
        return REF_ERR;
    return (ok(cudaMemcpy(cs, s->cs, s->numCells * 4, cudaMemcpyDeviceToHost)) &&
            ok(cudaMemcpy(ce, s->ce, s->numCells * 4, cudaMemcpyDeviceToHost)))
               ? REF_OK
               : REF_ERR;
}

// findNeighbors over sorted positions with the grid of the last
// ref_grid_build; slot-major lists with the solver's stride.
int ref_find_neighbors(RefSolver* s, const float4* sp, size_t n, uint32_t* nbr, int* cnt,
                       size_t* stride_out) {
    if (n > s->maxParticles) return REF_ERR;
    if (n && !ok(cudaMemcpy(s->pred, sp, n * 16, cudaMemcpyHostToDevice))) return REF_ERR;
    const size_t keep = s->n;
    s->n = n;
    const int st = s->search();
    s->n = keep;
    if (st == REF_ERR) return st;
    *stride_out = s->stride;
    if (n && (!ok(cudaMemcpy(nbr, s->nbr, s->stride * size_t(s->maxNbCap) * 4, cudaMemcpyDeviceToHost)) ||
              !ok(cudaMemcpy(cnt, s->cnt, n * 4, cudaMemcpyDeviceToHost))))
        return REF_ERR;
    return st;
}

size_t ref_stride(RefSolver* s) { return s->stride; }
size_t ref_num_cells(RefSolver* s) { return s->numCells; }

}  // extern "C"
