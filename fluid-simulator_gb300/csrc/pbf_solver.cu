// pbf_solver.cu -- the solver object behind the C ABI (include/pbf103.h).
//
// Host side of PBFSolver (src/pbf/pbf_solver.cu).  Differences in mechanism,
// not in results:
//   * one frame (all substeps) is captured once into a CUDA graph and
//     replayed; the reference issues ~70 launches and >= 13 host syncs per
//     substep from the host;
//   * neighbour overflow and collision non-convergence are device status
//     bits read once per step()/run() call instead of a device-to-host copy
//     per iteration and per collision pass (src/pbf/pbf_solver.cu:227-230,
//     src/pbf/collision_system.cu:150-171);
//   * within a substep only the predicted positions are physically reordered
//     each iteration; positions, incoming velocities, velocity payloads and
//     stable ids follow once through the composite permutation.  The data
//     every kernel sees is identical to the reference's gathers
//     (src/pbf/pbf_solver.cu:154-172).
#include "pbf_common.h"
#include "pbf_kernels.cuh"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

namespace pbf {

namespace detail {
std::mutex g_err_mu;
std::string g_err;
}  // namespace detail

void set_global_error(const std::string& m) {
    std::lock_guard<std::mutex> lk(detail::g_err_mu);
    detail::g_err = m;
}

}  // namespace pbf

using namespace pbf;

namespace {

constexpr int kDefaultMaxNeighbors = 256;  // kMaxNeighbors, src/pbf/pbf_solver.cu:12
constexpr int kStrideAlignment = 256;      // neighbour stride rounding, :36-39
constexpr int kF4Pool = 6;                 // float4 buffers rotated through roles

// Stages of one frame, for the event profiler (pbf_profile_frame).
enum Stage {
    kStPredict, kStSort, kStGatherRanges, kStSearchLambda, kStDeltaApply, kStSearch,
    kStFinalize, kStXsph, kStVorticity, kStConfine, kStResolve, kStageCount
};
const char* const kStageNames[kStageCount] = {
    "predict", "sort", "gather_ranges", "search_lambda", "delta_apply_collide",
    "search_final", "finalize", "xsph", "vorticity", "confine_resolve", "resolve"};

// Event marks recorded between the launches of a frame; interval i belongs to
// the stage of mark i.
struct Marks {
    std::vector<cudaEvent_t> events;
    std::vector<int> stages;
    size_t used = 0;
    void mark(int stage, cudaStream_t st) {
        if (used == events.size()) {
            cudaEvent_t e;
            cuda_check(cudaEventCreate(&e));
            events.push_back(e);
            stages.push_back(stage);
        }
        stages[used] = stage;
        // External records become event nodes of the captured graph, so the
        // events are really recorded each time the graph runs.
        cuda_check(cudaEventRecordWithFlags(events[used], st, cudaEventRecordExternal));
        ++used;
    }
    ~Marks() {
        for (auto e : events) cudaEventDestroy(e);
    }
};


}  // namespace

namespace pbf {

bool finite3(pbf_float3 v) { return std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z); }

// Parameter validation of PBFSolver::initialize (src/pbf/pbf_solver.cu:45-79).
std::vector<float4> collider_records(int kind, const void* data, size_t count) {
    std::vector<float4> next;
    if (kind == 0) {
        const pbf_sphere* s = static_cast<const pbf_sphere*>(data);
        if (count && !s) fail(PBF_ERR_INVALID_ARGUMENT, "Sphere array must not be null");
        for (size_t i = 0; i < count; ++i) {
            if (!finite3(s[i].center) || !std::isfinite(s[i].radius) || s[i].radius <= 0.0f)
                fail(PBF_ERR_INVALID_ARGUMENT, "Sphere radius must be positive");
            next.push_back(make_float4(s[i].center.x, s[i].center.y, s[i].center.z, s[i].radius));
        }
    } else if (kind == 1) {
        const pbf_box* b = static_cast<const pbf_box*>(data);
        if (count && !b) fail(PBF_ERR_INVALID_ARGUMENT, "Box array must not be null");
        for (size_t i = 0; i < count; ++i) {
            const pbf_float3 c = b[i].center, e = b[i].halfExtents;
            if (!finite3(c) || !std::isfinite(e.x) || e.x <= 0.0f || !std::isfinite(e.y) ||
                e.y <= 0.0f || !std::isfinite(e.z) || e.z <= 0.0f)
                fail(PBF_ERR_INVALID_ARGUMENT, "Box half extents must be positive");
            next.push_back(make_float4(c.x, c.y, c.z, 0.0f));
            next.push_back(make_float4(e.x, e.y, e.z, 0.0f));
        }
    } else {
        const pbf_plane* p = static_cast<const pbf_plane*>(data);
        if (count && !p) fail(PBF_ERR_INVALID_ARGUMENT, "Plane array must not be null");
        for (size_t i = 0; i < count; ++i) {
            const pbf_float3 q = p[i].point, nn = p[i].normal;
            const float l2 = nn.x * nn.x + nn.y * nn.y + nn.z * nn.z;
            if (!finite3(q) || !std::isfinite(l2) || l2 == 0.0f)
                fail(PBF_ERR_INVALID_ARGUMENT, "Plane normal must not be zero");
            next.push_back(make_float4(q.x, q.y, q.z, 0.0f));
            next.push_back(make_float4(nn.x, nn.y, nn.z, 0.0f));
        }
    }
    return next;
}

void validate_params(const pbf_params& p) {
    if (!std::isfinite(p.dt) || p.dt <= 0.0f || !std::isfinite(p.restDensity) ||
        p.restDensity <= 0.0f || !std::isfinite(p.particleMass) || p.particleMass <= 0.0f ||
        !std::isfinite(p.particleRadius) || p.particleRadius <= 0.0f ||
        !std::isfinite(p.collisionRestitution) || p.collisionRestitution < 0.0f ||
        p.collisionRestitution > 1.0f || !std::isfinite(p.collisionFriction) ||
        p.collisionFriction < 0.0f || p.collisionFriction > 1.0f ||
        !std::isfinite(p.smoothingRadius) || p.smoothingRadius <= 0.0f ||
        !std::isfinite(p.lambdaEpsilon) || p.lambdaEpsilon <= 0.0f || !std::isfinite(p.scorrK) ||
        p.scorrK < 0.0f ||
        (p.scorrK > 0.0f && (p.scorrN <= 0 || !std::isfinite(p.scorrDeltaQ) ||
                             p.scorrDeltaQ < 0.0f || p.scorrDeltaQ >= p.smoothingRadius)) ||
        !std::isfinite(p.xsphViscosity) || p.xsphViscosity < 0.0f ||
        !std::isfinite(p.vorticityStrength) || p.vorticityStrength < 0.0f ||
        !finite3(p.gravity) || p.solverIterations <= 0 || p.substeps <= 0)
        fail(PBF_ERR_INVALID_ARGUMENT, "Invalid PBF simulation parameters");
    const float sub = p.dt / static_cast<float>(p.substeps);
    if (!std::isfinite(sub) || sub <= 0.0f || !std::isfinite(1.0f / sub))
        fail(PBF_ERR_INVALID_ARGUMENT, "Substep duration is not representable");
}

// SpatialGrid::initialize validation and dims (src/pbf/spatial_grid.cu:10-64).
std::array<int, 3> grid_dims_checked(pbf_float3 mn, pbf_float3 mx, float cell) {
    if (!std::isfinite(cell) || cell <= 0.0f)
        fail(PBF_ERR_INVALID_ARGUMENT, "cellSize must be greater than zero");
    if (!finite3(mn) || !finite3(mx) || mx.x <= mn.x || mx.y <= mn.y || mx.z <= mn.z)
        fail(PBF_ERR_INVALID_ARGUMENT, "Invalid spatial grid bounds");
    const float lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z};
    std::array<int, 3> d{};
    for (int a = 0; a < 3; ++a) {
        const double c = std::ceil((double(hi[a]) - double(lo[a])) / double(cell));
        if (!std::isfinite(c) || c < 1.0 || c > double(std::numeric_limits<int>::max()))
            fail(PBF_ERR_LENGTH, "Spatial grid axis exceeds integer capacity");
        d[a] = static_cast<int>(c);
    }
    const size_t maxCells = std::numeric_limits<uint32_t>::max();
    const size_t cx = size_t(d[0]), cy = size_t(d[1]), cz = size_t(d[2]);
    if (cx > maxCells / cy || cx * cy > maxCells / cz)
        fail(PBF_ERR_LENGTH, "Spatial grid exceeds 32-bit key capacity");
    return d;
}

}  // namespace pbf

struct pbf_solver {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string last_error;

    // Configuration (valid when cap > 0).
    size_t cap = 0, n = 0, stride = 0;
    int max_nb = kDefaultMaxNeighbors;
    pbf_params prm{};
    pbf_float3 mn{}, mx{};
    std::array<int, 3> dims{};
    uint64_t cells = 0;

    // Colliders (host copy; may be set before initialize, like CollisionSystem).
    std::vector<float4> h_spheres, h_boxes, h_planes;
    DeviceBuffer d_colliders;
    bool colliders_dirty = true;

    // Batched mode (nscenes > 0): scenes occupy fixed slot ranges
    // [scene_off[s], scene_off[s + 1]); every kernel reads its scene's grid,
    // container and density terms from scene_tab through scene_id.
    int nscenes = 0;
    std::vector<size_t> scene_off;
    DeviceBuffer scene_tab, scene_id;

    // Threads per block of the tuned kernels (0 = the default 256).
    int tuned[kTunedCount] = {};
    int tuned_lanes = 0;  // lanes per particle of the walks set by pbf_set_walk_lanes; 0 = default
    int sort_tile = 0;    // keys per radix-sort tile chosen by the autotuner; 0 = by size

    // Compact neighbour lists (list_cap > 0): every rebuild counts the
    // neighbours, scans the counts into nb_off and writes each particle's
    // list contiguously into list_cap entries in all.  0: slot-major lists of
    // max_nb slots per particle.
    size_t list_cap = 0;
    DeviceBuffer nb_off, nb_scratch;

    // Device state.
    DeviceBuffer f4[kF4Pool];
    DeviceBuffer ids[2], org[2];
    DeviceBuffer keys, skeys, sidx, akeys, aidx;
    DeviceBuffer cell_first, nbr, cnt, lam, sort_scratch, status, tmp4, ftmp;
    DeviceBuffer soa;  // x, y, z components of the reordered predicted positions
    // Component array stride (see soa_stride_for).
    size_t soa_stride() const { return soa_stride_for(cap); }
    unsigned* h_status = nullptr;
    int ix = 0, iv = 1, iid = 0;  // roles: positions, velocities, ids

    // Graph cache keyed by the role assignment at frame start.
    std::map<std::tuple<int, int, int, bool>, std::pair<cudaGraphExec_t, std::tuple<int, int, int>>>
        graphs;
    int kernels_per_frame = 0;
    Marks marks;          // events of the profiling graph
    Marks* prof = nullptr;  // set while capturing the profiling graph

    ~pbf_solver() {
        clear_graphs();
        if (h_status) cudaFreeHost(h_status);
        if (own_stream) cudaStreamDestroy(own_stream);
    }

    void clear_graphs() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second.first);
        graphs.clear();
    }

    // CUDA is touched lazily, so argument validation works without a device.
    void use_device() {
        cuda_check(cudaSetDevice(device));
        if (!own_stream) {
            cuda_check(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking));
            if (!stream) stream = own_stream;
        }
        if (!h_status) cuda_check(cudaMallocHost(&h_status, sizeof(unsigned)));
    }

    // ---- constants -----------------------------------------------------------
    StepConst make_const() const {
        StepConst c{};
        const float h = prm.smoothingRadius;
        c.k = make_kernel_const(h);
        c.sc = make_scorr_const(h, prm.scorrK, prm.scorrN, prm.scorrDeltaQ);
        c.g.minx = mn.x;
        c.g.miny = mn.y;
        c.g.minz = mn.z;
        c.g.cell = h;
        c.g.gx = dims[0];
        c.g.gy = dims[1];
        c.g.gz = dims[2];
        const double r = std::ceil(double(h) / double(h));
        const int maxdim = std::max(dims[0], std::max(dims[1], dims[2]));
        c.g.radius = static_cast<int>(std::min(r, double(maxdim)));
        c.mass = prm.particleMass;
        c.rho0 = prm.restDensity;
        c.lambda_eps = prm.lambdaEpsilon;
        c.gs = prm.particleMass / prm.restDensity;
        c.gs2 = c.gs * c.gs;
        c.dt = prm.dt / static_cast<float>(prm.substeps);
        c.inv_dt = 1.0f / c.dt;
        c.gravx = prm.gravity.x;
        c.gravy = prm.gravity.y;
        c.gravz = prm.gravity.z;
        c.particle_radius = prm.particleRadius;
        c.restitution = prm.collisionRestitution;
        c.friction = prm.collisionFriction;
        c.xsph_c = prm.xsphViscosity;
        c.vort_eps = prm.vorticityStrength;
        c.max_nb = max_nb;
        c.stride = stride;
        const float4* base = d_colliders.as<float4>();
        const size_t ns = h_spheres.size(), nb = h_boxes.size() / 2, np = h_planes.size() / 2;
        c.col.spheres = base;
        c.col.boxes = base ? base + ns : nullptr;
        c.col.planes = base ? base + ns + 2 * nb : nullptr;
        c.col.ns = static_cast<int>(ns);
        c.col.nb = static_cast<int>(nb);
        c.col.np = static_cast<int>(np);
        c.col.cminx = mn.x;
        c.col.cminy = mn.y;
        c.col.cminz = mn.z;
        c.col.cmaxx = mx.x;
        c.col.cmaxy = mx.y;
        c.col.cmaxz = mx.z;
        if (nscenes > 0) {
            c.scenes = scene_tab.as<SceneConst>();
            c.sid = scene_id.as<uint16_t>();
        }
        for (int k = 0; k < kTunedCount; ++k) c.blk[k] = tuned[k];
        if (list_cap > 0) {
            c.nb_off = nb_off.as<uint32_t>();
            c.nb_cap = list_cap;
        }
        c.walk_lanes = walk_lanes();
        c.prune_cells = true;
        return c;
    }

    void upload_colliders() {
        if (!colliders_dirty) return;
        std::vector<float4> all;
        all.insert(all.end(), h_spheres.begin(), h_spheres.end());
        all.insert(all.end(), h_boxes.begin(), h_boxes.end());
        all.insert(all.end(), h_planes.begin(), h_planes.end());
        DeviceBuffer next(all.size() * sizeof(float4));
        if (!all.empty())
            cuda_check(cudaMemcpy(next.get(), all.data(), all.size() * sizeof(float4),
                                  cudaMemcpyHostToDevice));
        d_colliders = std::move(next);
        colliders_dirty = false;
        clear_graphs();
    }

    // ---- frame emission -----------------------------------------------------
    // Enqueues one frame on `st` starting from roles (ix, iv, iid) and returns
    // the roles after it.  Buffer roles are handed out lowest-free-first, so
    // the mapping from input to output roles is fixed and the captured graph
    // for a given input assignment is reusable.
    std::tuple<int, int, int> enqueue_frame(cudaStream_t st, int rx, int rv, int rid) {
        const StepConst c = make_const();
        const int N = static_cast<int>(n);
        unsigned* sp = status.as<unsigned>();
        bool used[kF4Pool] = {};
        used[rx] = used[rv] = true;
        auto take = [&]() {
            for (int i = 0; i < kF4Pool; ++i)
                if (!used[i]) {
                    used[i] = true;
                    return i;
                }
            fail(PBF_ERR_RUNTIME, "internal buffer pool exhausted");
        };
        auto give = [&](int i) { used[i] = false; };
        auto P = [&](int i) { return f4[i].as<float4>(); };
        const SortPlan plan = make_sort_plan(N, cells, sort_tile);
        const bool post = prm.xsphViscosity != 0.0f || prm.vorticityStrength != 0.0f;

        auto M = [&](int stage) {
            if (prof) prof->mark(stage, st);
        };
        for (int sub = 0; sub < prm.substeps; ++sub) {
            const int xs0 = take();
            const int vin = take();
            M(kStPredict);
            launch_predict(P(rx), P(rv), P(xs0), P(vin), keys.as<uint32_t>(), N, c, sp, st);
            int cur = xs0;
            int org_cur = -1;
            auto rebuild = [&]() {
                M(kStSort);
                launch_sort(plan, keys.as<uint32_t>(), skeys.as<uint32_t>(), sidx.as<uint32_t>(),
                            akeys.as<uint32_t>(), aidx.as<uint32_t>(), sort_scratch.get(), sp, st);
                const int nxt = take();
                const int org_next = org_cur < 0 ? 0 : 1 - org_cur;
                M(kStGatherRanges);
                launch_gather_first(sidx.as<uint32_t>(), P(cur), P(nxt),
                                    org_cur < 0 ? nullptr : org[org_cur].as<uint32_t>(),
                                    org[org_next].as<uint32_t>(), soa.as<float>(),
                                    soa.as<float>() + soa_stride(),
                                    soa.as<float>() + 2 * soa_stride(), N, skeys.as<uint32_t>(),
                                    cells, cell_first.as<int>(), sp, st);
                give(cur);
                cur = nxt;
                org_cur = org_next;
            };
            // Compact lists: neighbour counts and their scan before each walk
            // that writes lists.
            auto count_and_scan = [&](int xs) {
                if (list_cap == 0) return;
                launch_count(P(xs), soa.as<float>(), soa.as<float>() + soa_stride(),
                             soa.as<float>() + 2 * soa_stride(), cell_first.as<int>(), c, N,
                             cnt.as<int>(), sp, st);
                launch_nb_scan(cnt.as<int>(), nb_off.as<uint32_t>(), list_cap, N,
                               nb_scratch.as<uint32_t>(), sp, st);
            };
            for (int it = 0; it < prm.solverIterations; ++it) {
                rebuild();
                M(kStSearchLambda);
                count_and_scan(cur);
                launch_search(P(cur), soa.as<float>(), soa.as<float>() + soa_stride(),
                              soa.as<float>() + 2 * soa_stride(), cell_first.as<int>(), c, N,
                              nbr.as<uint32_t>(), cnt.as<int>(), lam.as<float>(), sp, true, st);
                const int nxt = take();
                M(kStDeltaApply);
                launch_delta_apply(P(cur), nbr.as<uint32_t>(), cnt.as<int>(), lam.as<float>(), c,
                                   N, P(nxt), keys.as<uint32_t>(), sp, st);
                give(cur);
                cur = nxt;
            }
            // The final rebuild, then the velocity update (it needs only the
            // composed permutation), then the final walk: with XSPH on, the
            // walk applies XSPH in a second pass over its new lists.
            if (post) rebuild();
            const int vnew = take();
            const int vinnew = take();
            const int idnew = 1 - rid;
            M(kStFinalize);
            launch_finalize(org[org_cur].as<uint32_t>(), P(rx), P(vin), P(rv),
                            ids[rid].as<uint32_t>(), P(cur), N, c, P(vnew), P(vinnew),
                            ids[idnew].as<uint32_t>(), sp, st);
            give(rx);
            give(rv);
            give(vin);
            rx = cur;
            rv = vnew;
            rid = idnew;
            const int vin2 = vinnew;
            const bool xsph = prm.xsphViscosity != 0.0f;
            const bool vort = prm.vorticityStrength != 0.0f;
            if (xsph) {
                const int t = take();
                M(kStSearch);
                count_and_scan(rx);
                launch_search_xsph(P(rx), soa.as<float>(), soa.as<float>() + soa_stride(),
                                   soa.as<float>() + 2 * soa_stride(), cell_first.as<int>(), c,
                                   N, nbr.as<uint32_t>(), cnt.as<int>(), P(rv), P(t), P(vin2),
                                   !vort, sp, st);
                give(rv);
                rv = t;
            } else if (vort) {
                M(kStSearch);
                count_and_scan(rx);
                launch_search(P(rx), soa.as<float>(), soa.as<float>() + soa_stride(),
                              soa.as<float>() + 2 * soa_stride(), cell_first.as<int>(), c, N,
                              nbr.as<uint32_t>(), cnt.as<int>(), nullptr, sp, false, st);
            }
            if (vort) {
                const int om = take();
                M(kStVorticity);
                launch_vorticity(P(rx), P(rv), nbr.as<uint32_t>(), cnt.as<int>(), c, N, P(om), true,
                                 sp, st);
                const int t = take();
                M(kStConfine);
                launch_confine(P(rx), nbr.as<uint32_t>(), cnt.as<int>(), P(om), P(rv), c, N, P(t),
                               P(vin2), true, sp, st);
                give(rv);
                give(om);
                rv = t;
            }
            if (!xsph && !vort) M(kStResolve);
            if (!xsph && !vort) launch_resolve(P(rx), P(vin2), P(rv), c, N, sp, st);
            give(vin2);
        }
        M(kStageCount);  // closing mark
        cuda_check(cudaGetLastError());
        return {rx, rv, rid};
    }

    std::pair<cudaGraphExec_t, std::tuple<int, int, int>>& graph_for(int rx, int rv, int rid,
                                                                     bool profiled = false) {
        const auto key = std::make_tuple(rx, rv, rid, profiled);
        auto it = graphs.find(key);
        if (it != graphs.end()) return it->second;
        cudaStream_t cap_stream = stream;
        cuda_check(cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal));
        std::tuple<int, int, int> out;
        if (profiled) {
            marks.used = 0;
            prof = &marks;
        }
        try {
            out = enqueue_frame(cap_stream, rx, rv, rid);
            prof = nullptr;
        } catch (...) {
            prof = nullptr;
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(cap_stream, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        cudaGraph_t g = nullptr;
        cuda_check(cudaStreamEndCapture(cap_stream, &g));
        size_t nn = 0;
        cuda_check(cudaGraphGetNodes(g, nullptr, &nn));
        std::vector<cudaGraphNode_t> nodes(nn);
        if (nn) cuda_check(cudaGraphGetNodes(g, nodes.data(), &nn));
        int kernels = 0;
        for (auto nd : nodes) {
            cudaGraphNodeType t;
            cuda_check(cudaGraphNodeGetType(nd, &t));
            if (t == cudaGraphNodeTypeKernel) ++kernels;
        }
        if (!profiled) kernels_per_frame = kernels;
        cudaGraphExec_t ex = nullptr;
        const cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        cuda_check(e);
        auto res = graphs.emplace(key, std::make_pair(ex, out));
        return res.first->second;
    }

    void require_initialized(const char* what) const {
        if (cap == 0) fail(PBF_ERR_LOGIC, what);
    }

    void enqueue_frames(size_t frames) {
        for (size_t f = 0; f < frames; ++f) {
            auto& g = graph_for(ix, iv, iid);
            cuda_check(cudaGraphLaunch(g.first, stream));
            std::tie(ix, iv, iid) = g.second;
        }
    }

    // One profiled frame: per-stage device milliseconds and launch counts.
    void profile_frame(float* ms, int* launches) {
        use_device();
        if (n == 0) fail(PBF_ERR_LOGIC, "no particles to profile");
        upload_colliders();
        cuda_check(cudaMemsetAsync(status.get(), 0, sizeof(unsigned), stream));
        auto& g = graph_for(ix, iv, iid, true);
        cuda_check(cudaGraphLaunch(g.first, stream));
        std::tie(ix, iv, iid) = g.second;
        check_status();
        for (int k = 0; k < kStageCount; ++k) {
            ms[k] = 0.0f;
            launches[k] = 0;
        }
        for (size_t i = 0; i + 1 < marks.used; ++i) {
            float t = 0.0f;
            cuda_check(cudaEventElapsedTime(&t, marks.events[i], marks.events[i + 1]));
            ms[marks.stages[i]] += t;
            launches[marks.stages[i]] += 1;
        }
    }

    // Autotuner: for each tuned kernel, time its stage in profiled frames at
    // 64, 128, 256 and 512 threads per block and keep the fastest (coordinate
    // descent, one kernel at a time; the other kernels keep their current
    // sizes); then the radix sort's tile (1,024 keys in 256-thread blocks or
    // 4,096 keys in 512-thread blocks), timed on the sort stage.  Neither
    // changes any arithmetic or the sort's result, so results stay bit for
    // bit the same.  The particle state is saved before and restored after,
    // so tuning does not advance the simulation.
    void autotune(int frames_per_trial) {
        require_initialized("PBFSolver must be initialized before tuning");
        if (n == 0) fail(PBF_ERR_LOGIC, "no particles to tune on");
        if (frames_per_trial <= 0) fail(PBF_ERR_INVALID_ARGUMENT, "frames per trial must be positive");
        use_device();
        DeviceBuffer sx(n * sizeof(float4)), sv(n * sizeof(float4));
        copy_out(false, sx.as<float4>(), n, true);
        copy_out(true, sv.as<float4>(), n, true);
        std::vector<float> ms(kStageCount);
        std::vector<int> launches(kStageCount);
        int saved[kTunedCount];
        std::copy(tuned, tuned + kTunedCount, saved);
        const int saved_tile = sort_tile;
        try {
            tune_all(frames_per_trial, ms, launches, sx.as<float4>(), sv.as<float4>());
        } catch (...) {
            std::copy(saved, saved + kTunedCount, tuned);
            sort_tile = saved_tile;
            clear_graphs();
            set_particles(sx.as<float4>(), sv.as<float4>(), n, true);
            throw;
        }
        clear_graphs();
        set_particles(sx.as<float4>(), sv.as<float4>(), n, true);
    }

    // Every trial frame starts from the saved state (x0, v0), so the sizes are
    // compared on the same work.
    // Frames of a trial before the timed ones: set_particles alternates the
    // buffers, so the first two frames capture and first launch the two
    // graphs a trial uses; they are not timed.
    void warm_trial(std::vector<float>& ms, std::vector<int>& launches, const float4* x0,
                    const float4* v0) {
        for (int f = 0; f < 2; ++f) {
            set_particles(x0, v0, n, true);
            profile_frame(ms.data(), launches.data());
        }
    }

    void tune_all(int frames_per_trial, std::vector<float>& ms, std::vector<int>& launches,
                  const float4* x0, const float4* v0) {
        static const int stage_of[kTunedCount] = {kStSearchLambda, kStDeltaApply, kStSearch,
                                                  kStXsph, kStVorticity, kStConfine};
        static const int sizes[4] = {64, 128, 256, 512};
        for (int k = 0; k < kTunedCount; ++k) {
            int best = tuned[k] > 0 ? tuned[k] : kBlock;
            float best_ms = -1.0f;
            for (int b : sizes) {
                tuned[k] = b;
                clear_graphs();
                warm_trial(ms, launches, x0, v0);
                float t = -1.0f;
                for (int f = 0; f < frames_per_trial; ++f) {
                    set_particles(x0, v0, n, true);
                    profile_frame(ms.data(), launches.data());
                    const float v = ms[stage_of[k]];
                    if (launches[stage_of[k]] == 0) break;  // stage not in this frame
                    t = t < 0.0f ? v : std::min(t, v);
                }
                if (t >= 0.0f && (best_ms < 0.0f || t < best_ms)) {
                    best_ms = t;
                    best = b;
                }
            }
            tuned[k] = best;
        }
        // The sort tile, timed on the sort stage of the same frames.
        int best_tile = sort_tile;
        float best_ms = -1.0f;
        for (int tile : {kSortMinTile, kSortMaxTile}) {
            sort_tile = tile;
            clear_graphs();
            warm_trial(ms, launches, x0, v0);
            float t = -1.0f;
            for (int f = 0; f < frames_per_trial; ++f) {
                set_particles(x0, v0, n, true);
                profile_frame(ms.data(), launches.data());
                t = t < 0.0f ? ms[kStSort] : std::min(t, ms[kStSort]);
            }
            if (t >= 0.0f && (best_ms < 0.0f || t < best_ms)) {
                best_ms = t;
                best_tile = tile;
            }
        }
        sort_tile = best_tile;
    }

    // Lanes per particle of the list-writing walks: the value set, else the
    // default for the scene size; 1 with compact lists.
    int walk_lanes() const {
        if (list_cap > 0) return 1;
        const int L = tuned_lanes > 0 ? tuned_lanes : default_walk_lanes(n, max_nb);
        return max_nb >= L && n * size_t(L) <= (size_t(1) << 30) ? L : 1;
    }

    void check_status() {
        cuda_check(cudaMemcpyAsync(h_status, status.get(), sizeof(unsigned),
                                   cudaMemcpyDeviceToHost, stream));
        cuda_check(cudaStreamSynchronize(stream));
        const unsigned s = *h_status;
        if (s & kStatusNeighborOverflow)
            fail(PBF_ERR_OVERFLOW, "Particle neighbor count exceeds solver capacity");
        if (s & kStatusNotConverged) fail(PBF_ERR_RUNTIME, "Collision constraints did not converge");
        if (s & kStatusListOverflow)
            fail(PBF_ERR_OVERFLOW, "Neighbor lists exceed the compact list capacity");
    }

    void run_frames(size_t frames, bool sync) {
        use_device();
        if (n == 0 || frames == 0) return;
        upload_colliders();
        cuda_check(cudaMemsetAsync(status.get(), 0, sizeof(unsigned), stream));
        enqueue_frames(frames);
        if (sync) check_status();
    }

    // ---- API ------------------------------------------------------------------
    // lcap > 0: compact neighbour lists of lcap entries in all.
    void initialize(size_t max_particles, pbf_float3 lo, pbf_float3 hi, const pbf_params& p,
                    int maxnb, size_t lcap = 0) {
        if (max_particles == 0)
            fail(PBF_ERR_INVALID_ARGUMENT, "maxParticles must be greater than zero");
        if (maxnb <= 0) fail(PBF_ERR_INVALID_ARGUMENT, "maxNeighbors must be greater than zero");
        if (lcap > 0xffffffffull)
            fail(PBF_ERR_LENGTH, "Compact neighbor list capacity exceeds 2^32 - 1 entries");
        if (max_particles > std::numeric_limits<size_t>::max() / size_t(maxnb))
            fail(PBF_ERR_LENGTH, "Neighbor buffer size overflows size_t");
        if (max_particles > static_cast<size_t>(std::numeric_limits<int>::max()))
            fail(PBF_ERR_LENGTH, "Particle count exceeds CUDA kernel index range");
        const size_t strd =
            (max_particles + kStrideAlignment - 1) / kStrideAlignment * kStrideAlignment;
        if (strd > std::numeric_limits<size_t>::max() / size_t(maxnb))
            fail(PBF_ERR_LENGTH, "Neighbor buffer size overflows size_t");
        validate_params(p);
        const double width = double(hi.x) - double(lo.x);
        const double depth = double(hi.z) - double(lo.z);
        const double diameter = 2.0 * double(p.particleRadius);
        if (width < diameter || depth < diameter)
            fail(PBF_ERR_INVALID_ARGUMENT, "Particle diameter exceeds closed container dimensions");
        const std::array<int, 3> d = grid_dims_checked(lo, hi, p.smoothingRadius);
        const uint64_t ncells = uint64_t(d[0]) * uint64_t(d[1]) * uint64_t(d[2]);

        use_device();
        allocate_and_commit(max_particles, strd, maxnb, ncells, DeviceBuffer(), DeviceBuffer(), {},
                            lcap);
        prm = p;
        mn = lo;
        mx = hi;
        dims = d;
    }

    // Allocates the device state for `max_particles` slots and `ncells` grid
    // cells, then makes it (and the scene table, empty for one scene) the
    // active configuration.  Nothing changes if an allocation fails.
    void allocate_and_commit(size_t max_particles, size_t strd, int maxnb, uint64_t ncells,
                             DeviceBuffer ntab, DeviceBuffer nsid, std::vector<size_t> off,
                             size_t lcap = 0) {
        const size_t f4b = max_particles * sizeof(float4);
        const size_t u4b = max_particles * sizeof(uint32_t);
        DeviceBuffer nf4[kF4Pool], nids[2], norg[2];
        for (auto& b : nf4) b.allocate(f4b);
        for (auto& b : nids) b.allocate(u4b);
        for (auto& b : norg) b.allocate(u4b);
        DeviceBuffer nkeys(u4b), nskeys(u4b), nsidx(u4b), nakeys(u4b), naidx(u4b);
        DeviceBuffer nfirst((ncells + 1) * sizeof(int));
        DeviceBuffer nsoa(3 * soa_stride_for(max_particles) * sizeof(float));
        DeviceBuffer nnbr((lcap > 0 ? lcap : strd * size_t(maxnb)) * sizeof(uint32_t));
        DeviceBuffer nnboff, nnbscr;
        if (lcap > 0) {
            nnboff.allocate((max_particles + 1) * sizeof(uint32_t));
            nnbscr.allocate(nb_scan_scratch_words(max_particles) * sizeof(uint32_t));
        }
        DeviceBuffer ncnt(u4b), nlam(u4b), nscr(sort_scratch_bytes(int(max_particles)));
        DeviceBuffer nstat(sizeof(unsigned)), ntmp(f4b), nftmp(u4b);

        clear_graphs();
        for (int i = 0; i < kF4Pool; ++i) f4[i] = std::move(nf4[i]);
        for (int i = 0; i < 2; ++i) {
            ids[i] = std::move(nids[i]);
            org[i] = std::move(norg[i]);
        }
        keys = std::move(nkeys);
        skeys = std::move(nskeys);
        sidx = std::move(nsidx);
        akeys = std::move(nakeys);
        aidx = std::move(naidx);
        cell_first = std::move(nfirst);
        soa = std::move(nsoa);
        nbr = std::move(nnbr);
        nb_off = std::move(nnboff);
        nb_scratch = std::move(nnbscr);
        list_cap = lcap;
        cnt = std::move(ncnt);
        lam = std::move(nlam);
        sort_scratch = std::move(nscr);
        status = std::move(nstat);
        tmp4 = std::move(ntmp);
        ftmp = std::move(nftmp);
        cuda_check(cudaMemsetAsync(cnt.get(), 0, u4b, stream));
        cuda_check(cudaMemsetAsync(status.get(), 0, sizeof(unsigned), stream));
        cuda_check(cudaStreamSynchronize(stream));

        cap = max_particles;
        n = 0;
        stride = strd;
        max_nb = maxnb;
        cells = ncells;
        ix = 0;
        iv = 1;
        iid = 0;
        colliders_dirty = true;
        scene_tab = std::move(ntab);
        scene_id = std::move(nsid);
        scene_off = std::move(off);
        nscenes = scene_off.empty() ? 0 : static_cast<int>(scene_off.size()) - 1;
    }

    // Batched initialisation: `count` scenes, each with its own particle
    // count, container (== grid bounds) and rest density, mass and XSPH
    // strength; every other parameter is shared.
    void initialize_batch(const pbf_scene* sc, int count, const pbf_params& common, int maxnb) {
        if (count <= 0 || sc == nullptr)
            fail(PBF_ERR_INVALID_ARGUMENT, "A batch needs at least one scene");
        if (count > 65535) fail(PBF_ERR_LENGTH, "A batch holds at most 65535 scenes");
        if (maxnb <= 0) fail(PBF_ERR_INVALID_ARGUMENT, "maxNeighbors must be greater than zero");
        validate_params(common);
        std::vector<size_t> off(1, 0);
        std::vector<SceneConst> tab(static_cast<size_t>(count));
        uint64_t total_cells = 0;
        const bool xsph_on = sc[0].xsphViscosity != 0.0f;
        for (int k = 0; k < count; ++k) {
            const pbf_scene& q = sc[k];
            if (q.count == 0) fail(PBF_ERR_INVALID_ARGUMENT, "Every scene needs particles");
            pbf_params p = common;
            p.restDensity = q.restDensity;
            p.particleMass = q.particleMass;
            p.xsphViscosity = q.xsphViscosity;
            validate_params(p);
            if ((q.xsphViscosity != 0.0f) != xsph_on)
                fail(PBF_ERR_INVALID_ARGUMENT,
                     "XSPH must be enabled in every scene of a batch or in none");
            const double width = double(q.maxBounds.x) - double(q.minBounds.x);
            const double depth = double(q.maxBounds.z) - double(q.minBounds.z);
            const double diameter = 2.0 * double(common.particleRadius);
            if (width < diameter || depth < diameter)
                fail(PBF_ERR_INVALID_ARGUMENT,
                     "Particle diameter exceeds closed container dimensions");
            const std::array<int, 3> d =
                grid_dims_checked(q.minBounds, q.maxBounds, common.smoothingRadius);
            SceneConst& t = tab[static_cast<size_t>(k)];
            t.g.minx = q.minBounds.x;
            t.g.miny = q.minBounds.y;
            t.g.minz = q.minBounds.z;
            t.g.cell = common.smoothingRadius;
            t.g.gx = d[0];
            t.g.gy = d[1];
            t.g.gz = d[2];
            t.g.radius = 1;
            t.cell_base = static_cast<uint32_t>(total_cells);
            t.cminx = q.minBounds.x;
            t.cminy = q.minBounds.y;
            t.cminz = q.minBounds.z;
            t.cmaxx = q.maxBounds.x;
            t.cmaxy = q.maxBounds.y;
            t.cmaxz = q.maxBounds.z;
            t.rho0 = q.restDensity;
            t.mass = q.particleMass;
            t.gs = q.particleMass / q.restDensity;
            t.gs2 = t.gs * t.gs;
            t.xsph_c = q.xsphViscosity;
            total_cells += uint64_t(d[0]) * uint64_t(d[1]) * uint64_t(d[2]);
            if (total_cells >= (uint64_t(1) << 32))
                fail(PBF_ERR_LENGTH, "Batch grid exceeds 32-bit key capacity");
            off.push_back(off.back() + q.count);
            if (off.back() > static_cast<size_t>(std::numeric_limits<int>::max()))
                fail(PBF_ERR_LENGTH, "Particle count exceeds CUDA kernel index range");
        }
        const size_t total = off.back();
        const size_t strd = (total + kStrideAlignment - 1) / kStrideAlignment * kStrideAlignment;
        if (strd > std::numeric_limits<size_t>::max() / size_t(maxnb))
            fail(PBF_ERR_LENGTH, "Neighbor buffer size overflows size_t");
        std::vector<uint16_t> sid(total);
        for (int k = 0; k < count; ++k)
            std::fill(sid.begin() + off[k], sid.begin() + off[k + 1], static_cast<uint16_t>(k));

        use_device();
        DeviceBuffer ntab(tab.size() * sizeof(SceneConst)), nsid(total * sizeof(uint16_t));
        cuda_check(cudaMemcpy(ntab.get(), tab.data(), tab.size() * sizeof(SceneConst),
                              cudaMemcpyHostToDevice));
        cuda_check(cudaMemcpy(nsid.get(), sid.data(), total * sizeof(uint16_t),
                              cudaMemcpyHostToDevice));
        allocate_and_commit(total, strd, maxnb, total_cells, std::move(ntab), std::move(nsid),
                            std::move(off));
        prm = common;
        prm.restDensity = sc[0].restDensity;
        prm.particleMass = sc[0].particleMass;
        prm.xsphViscosity = sc[0].xsphViscosity;
        mn = sc[0].minBounds;
        mx = sc[0].maxBounds;
        dims = {tab[0].g.gx, tab[0].g.gy, tab[0].g.gz};
    }

    void set_particles(const float4* pos, const float4* vel, size_t count, bool device_ptrs) {
        require_initialized("PBFSolver must be initialized before setting particles");
        if (count > cap) fail(PBF_ERR_OUT_OF_RANGE, "Particle count exceeds solver capacity");
        if (nscenes > 0 && count != cap)
            fail(PBF_ERR_OUT_OF_RANGE, "A batch takes exactly the particles of all its scenes");
        use_device();
        if (count == 0) {
            n = 0;
            clear_graphs();
            return;
        }
        if (pos == nullptr || vel == nullptr)
            fail(PBF_ERR_INVALID_ARGUMENT, "Particle positions and velocities must not be null");
        // Upload into two buffers that hold no live state, check finiteness on
        // the device, and only then make them the active positions and
        // velocities: a rejected upload leaves the previous particles intact
        // (src/pbf/pbf_solver.cu:131-140 validates before uploading).
        int spare[2], k = 0;
        for (int i = 0; i < kF4Pool && k < 2; ++i)
            if (i != ix && i != iv) spare[k++] = i;
        const cudaMemcpyKind kind = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        cuda_check(cudaMemcpyAsync(f4[spare[0]].get(), pos, count * sizeof(float4), kind, stream));
        cuda_check(cudaMemcpyAsync(f4[spare[1]].get(), vel, count * sizeof(float4), kind, stream));
        check_finite_device(f4[spare[0]].as<float4>(), f4[spare[1]].as<float4>(), count);
        const int nid = 1 - iid;
        launch_iota(ids[nid].as<uint32_t>(), static_cast<int>(count), stream);
        cuda_check(cudaGetLastError());
        ix = spare[0];
        iv = spare[1];
        iid = nid;
        if (n != count) clear_graphs();
        n = count;
    }

    void check_finite_device(const float4* pos, const float4* vel, size_t count);

    void copy_out(bool velocities, float4* out, size_t count, bool device_ptr) {
        if (count != n)
            fail(PBF_ERR_OUT_OF_RANGE, velocities
                                           ? "Requested velocity count does not match active particles"
                                           : "Requested position count does not match active particles");
        if (count == 0) return;
        use_device();
        launch_scatter_by_id(f4[velocities ? iv : ix].as<float4>(), ids[iid].as<uint32_t>(),
                             tmp4.as<float4>(), static_cast<int>(count), stream);
        cuda_check(cudaGetLastError());
        if (out == nullptr) fail(PBF_ERR_INVALID_ARGUMENT, "Destination cannot be null");
        cuda_check(cudaMemcpyAsync(out, tmp4.get(), count * sizeof(float4),
                                   device_ptr ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                   stream));
        cuda_check(cudaStreamSynchronize(stream));
    }

    void set_colliders(int kind, const void* data, size_t count) {
        std::vector<float4> next = collider_records(kind, data, count);
        (kind == 0 ? h_spheres : kind == 1 ? h_boxes : h_planes).swap(next);
        colliders_dirty = true;
        clear_graphs();
    }
};

namespace pbf {
namespace detail {
__global__ void k_check_finite(const float4* __restrict__ p, const float4* __restrict__ v,
                               int n, unsigned* flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = p[i], b = v[i];
    if (!isfinite(a.x) || !isfinite(a.y) || !isfinite(a.z) || !isfinite(b.x) || !isfinite(b.y) ||
        !isfinite(b.z))
        atomicOr(flag, 1u);
}
}  // namespace detail
}  // namespace pbf

void pbf_solver::check_finite_device(const float4* pos, const float4* vel, size_t count) {
    unsigned* flag = ftmp.as<unsigned>();
    cuda_check(cudaMemsetAsync(flag, 0, sizeof(unsigned), stream));
    detail::k_check_finite<<<blocks_for(count), kBlock, 0, stream>>>(pos, vel, static_cast<int>(count), flag);
    cuda_check(cudaGetLastError());
    unsigned h = 0;
    cuda_check(cudaMemcpyAsync(&h, flag, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
    cuda_check(cudaStreamSynchronize(stream));
    if (h) fail(PBF_ERR_INVALID_ARGUMENT, "Particle coordinates and velocities must be finite");
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

#define PBF_GUARD(s, ...)                                                     \
    do {                                                                      \
        if (!(s)) {                                                           \
            pbf::set_global_error("solver handle must not be null");          \
            return PBF_ERR_INVALID_ARGUMENT;                                  \
        }                                                                     \
        return pbf::guarded(&(s)->last_error, [&]() { __VA_ARGS__; });            \
    } while (0)

extern "C" {

const char* pbf_version(void) { return "pbf103 0.1.0 (sm_103a)"; }

const char* pbf_global_last_error(void) {
    static thread_local std::string copy;
    std::lock_guard<std::mutex> lk(pbf::detail::g_err_mu);
    copy = pbf::detail::g_err;
    return copy.c_str();
}

pbf_status pbf_solver_create(pbf_solver** out, int device) {
    if (!out) {
        set_global_error("output pointer must not be null");
        return PBF_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    pbf_solver* s = nullptr;
    const pbf_status st = guarded(nullptr, [&]() {
        s = new pbf_solver();
        s->device = device;
        if (device < 0) {
            int dev = 0;
            if (cudaGetDevice(&dev) == cudaSuccess) s->device = dev;
            else s->device = 0;
            cudaGetLastError();
        }
    });
    if (st != PBF_OK) {
        delete s;
        return st;
    }
    *out = s;
    return PBF_OK;
}

void pbf_solver_destroy(pbf_solver* s) {
    if (!s) return;
    if (s->own_stream) {
        cudaSetDevice(s->device);
        cudaStreamSynchronize(s->stream);
    }
    delete s;
}

const char* pbf_last_error(const pbf_solver* s) { return s ? s->last_error.c_str() : ""; }

pbf_status pbf_initialize(pbf_solver* s, size_t max_particles, pbf_float3 lo, pbf_float3 hi,
                          const pbf_params* p) {
    PBF_GUARD(s, {
        if (!p) fail(PBF_ERR_INVALID_ARGUMENT, "params must not be null");
        s->initialize(max_particles, lo, hi, *p, kDefaultMaxNeighbors);
    });
}

pbf_status pbf_initialize_ex(pbf_solver* s, size_t max_particles, pbf_float3 lo, pbf_float3 hi,
                             const pbf_params* p, int max_neighbors) {
    PBF_GUARD(s, {
        if (!p) fail(PBF_ERR_INVALID_ARGUMENT, "params must not be null");
        s->initialize(max_particles, lo, hi, *p, max_neighbors);
    });
}

pbf_status pbf_initialize_compact(pbf_solver* s, size_t max_particles, pbf_float3 lo,
                                  pbf_float3 hi, const pbf_params* p, int max_neighbors,
                                  size_t list_capacity) {
    PBF_GUARD(s, {
        if (!p) fail(PBF_ERR_INVALID_ARGUMENT, "params must not be null");
        if (list_capacity == 0)
            fail(PBF_ERR_INVALID_ARGUMENT, "compact neighbor list capacity must be positive");
        s->initialize(max_particles, lo, hi, *p, max_neighbors, list_capacity);
    });
}

pbf_status pbf_set_particles(pbf_solver* s, const pbf_float4* pos, const pbf_float4* vel,
                             size_t count) {
    PBF_GUARD(s, s->set_particles(reinterpret_cast<const float4*>(pos),
                                  reinterpret_cast<const float4*>(vel), count, false));
}

pbf_status pbf_set_particles_device(pbf_solver* s, const pbf_float4* pos, const pbf_float4* vel,
                                    size_t count) {
    PBF_GUARD(s, s->set_particles(reinterpret_cast<const float4*>(pos),
                                  reinterpret_cast<const float4*>(vel), count, true));
}

pbf_status pbf_set_spheres(pbf_solver* s, const pbf_sphere* sp, size_t count) {
    PBF_GUARD(s, s->set_colliders(0, sp, count));
}
pbf_status pbf_set_boxes(pbf_solver* s, const pbf_box* b, size_t count) {
    PBF_GUARD(s, s->set_colliders(1, b, count));
}
pbf_status pbf_set_planes(pbf_solver* s, const pbf_plane* p, size_t count) {
    PBF_GUARD(s, s->set_colliders(2, p, count));
}

pbf_status pbf_step(pbf_solver* s) {
    const NvtxRange range("pbf_step");
    PBF_GUARD(s, {
        s->require_initialized("PBFSolver must be initialized before stepping");
        s->run_frames(1, true);
    });
}

pbf_status pbf_run(pbf_solver* s, size_t frames) {
    const NvtxRange range("pbf_run");
    PBF_GUARD(s, {
        s->require_initialized("PBFSolver must be initialized before running");
        s->run_frames(frames, true);
    });
}

pbf_status pbf_run_async(pbf_solver* s, size_t frames) {
    const NvtxRange range("pbf_run_async");
    PBF_GUARD(s, {
        s->require_initialized("PBFSolver must be initialized before running");
        s->run_frames(frames, false);
    });
}

pbf_status pbf_synchronize(pbf_solver* s) {
    PBF_GUARD(s, {
        s->use_device();
        if (s->cap) s->check_status();
        else cuda_check(cudaStreamSynchronize(s->stream));
    });
}

pbf_status pbf_time_frames(pbf_solver* s, size_t frames, float* ms) {
    const NvtxRange range("pbf_time_frames");
    PBF_GUARD(s, {
        s->require_initialized("PBFSolver must be initialized before running");
        if (!ms) fail(PBF_ERR_INVALID_ARGUMENT, "milliseconds must not be null");
        s->use_device();
        cudaEvent_t a, b;
        cuda_check(cudaEventCreate(&a));
        cuda_check(cudaEventCreate(&b));
        cuda_check(cudaStreamSynchronize(s->stream));
        cuda_check(cudaEventRecord(a, s->stream));
        s->run_frames(frames, false);
        cuda_check(cudaEventRecord(b, s->stream));
        cuda_check(cudaEventSynchronize(b));
        cuda_check(cudaEventElapsedTime(ms, a, b));
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        s->check_status();
    });
}

pbf_status pbf_profile_frame(pbf_solver* s, float* ms, int* launches) {
    PBF_GUARD(s, {
        s->require_initialized("PBFSolver must be initialized before running");
        if (!ms || !launches) fail(PBF_ERR_INVALID_ARGUMENT, "outputs must not be null");
        s->profile_frame(ms, launches);
    });
}

int pbf_stage_count(void) { return kStageCount; }

const char* pbf_stage_name(int stage) {
    return (stage >= 0 && stage < kStageCount) ? kStageNames[stage] : "";
}

pbf_status pbf_kernels_per_frame(pbf_solver* s, int* k) {
    PBF_GUARD(s, {
        s->require_initialized("PBFSolver must be initialized before running");
        if (!k) fail(PBF_ERR_INVALID_ARGUMENT, "output must not be null");
        s->use_device();
        if (s->n == 0) {
            *k = 0;
            return;
        }
        s->upload_colliders();
        (void)s->graph_for(s->ix, s->iv, s->iid);
        *k = s->kernels_per_frame;
    });
}

pbf_status pbf_copy_positions(pbf_solver* s, pbf_float4* out, size_t count) {
    PBF_GUARD(s, s->copy_out(false, reinterpret_cast<float4*>(out), count, false));
}
pbf_status pbf_copy_velocities(pbf_solver* s, pbf_float4* out, size_t count) {
    PBF_GUARD(s, s->copy_out(true, reinterpret_cast<float4*>(out), count, false));
}
pbf_status pbf_copy_positions_device(pbf_solver* s, pbf_float4* out, size_t count) {
    PBF_GUARD(s, s->copy_out(false, reinterpret_cast<float4*>(out), count, true));
}
pbf_status pbf_copy_velocities_device(pbf_solver* s, pbf_float4* out, size_t count) {
    PBF_GUARD(s, s->copy_out(true, reinterpret_cast<float4*>(out), count, true));
}

size_t pbf_particle_count(const pbf_solver* s) { return s ? s->n : 0; }

pbf_status pbf_batch_initialize(pbf_solver* s, const pbf_scene* scenes, int scene_count,
                                const pbf_params* common, int max_neighbors) {
    PBF_GUARD(s, {
        if (!common) fail(PBF_ERR_INVALID_ARGUMENT, "params must not be null");
        s->initialize_batch(scenes, scene_count, *common, max_neighbors);
    });
}

int pbf_batch_scene_count(const pbf_solver* s) { return s ? s->nscenes : 0; }

pbf_status pbf_autotune(pbf_solver* s, int frames_per_trial) {
    PBF_GUARD(s, s->autotune(frames_per_trial));
}

pbf_status pbf_block_sizes(const pbf_solver* s, int* sizes, int count) {
    if (!s || !sizes) {
        pbf::set_global_error("solver handle and sizes must not be null");
        return PBF_ERR_INVALID_ARGUMENT;
    }
    for (int k = 0; k < count && k < kTunedCount; ++k)
        sizes[k] = s->tuned[k] > 0 ? s->tuned[k] : kBlock;
    return PBF_OK;
}

pbf_status pbf_sort_tile(const pbf_solver* s, int* keys_per_tile) {
    if (!s || !keys_per_tile) {
        pbf::set_global_error("solver handle and keys_per_tile must not be null");
        return PBF_ERR_INVALID_ARGUMENT;
    }
    *keys_per_tile = make_sort_plan(static_cast<int>(std::min<size_t>(s->n, 1u << 30)),
                                    uint64_t(1), s->sort_tile).tile;
    return PBF_OK;
}

pbf_status pbf_set_walk_lanes(pbf_solver* s, int lanes) {
    PBF_GUARD(s, {
        if (lanes != 0 && lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8)
            fail(PBF_ERR_INVALID_ARGUMENT, "walk lanes must be 0, 1, 2, 4 or 8");
        s->tuned_lanes = lanes;
        s->clear_graphs();
    });
}

pbf_status pbf_walk_lanes(const pbf_solver* s, int* lanes) {
    if (!s || !lanes) {
        pbf::set_global_error("solver handle and lanes must not be null");
        return PBF_ERR_INVALID_ARGUMENT;
    }
    *lanes = s->walk_lanes();
    return PBF_OK;
}

pbf_status pbf_set_stream(pbf_solver* s, void* stream) {
    PBF_GUARD(s, {
        s->use_device();
        cuda_check(cudaStreamSynchronize(s->stream));
        s->clear_graphs();
        s->stream = stream ? static_cast<cudaStream_t>(stream) : s->own_stream;
    });
}

pbf_status pbf_density_error(pbf_solver* s, double* mean, double* mxe) {
    PBF_GUARD(s, {
        s->require_initialized("PBFSolver must be initialized before querying density");
        if (!mean || !mxe) fail(PBF_ERR_INVALID_ARGUMENT, "outputs must not be null");
        *mean = 0.0;
        *mxe = 0.0;
        if (s->n == 0) return;
        s->use_device();
        const StepConst c = s->make_const();
        launch_density(s->f4[s->ix].as<float4>(), s->nbr.as<uint32_t>(), s->cnt.as<int>(), c,
                       static_cast<int>(s->n), s->lam.as<float>(), s->stream);
        cuda_check(cudaGetLastError());
        std::vector<float> err(s->n);
        cuda_check(cudaMemcpyAsync(err.data(), s->lam.get(), s->n * sizeof(float),
                                   cudaMemcpyDeviceToHost, s->stream));
        cuda_check(cudaStreamSynchronize(s->stream));
        double sum = 0.0, m = 0.0;
        for (float e : err) {
            sum += e;
            m = std::max(m, double(e));
        }
        *mean = sum / double(s->n);
        *mxe = m;
    });
}

pbf_status pbf_copy_working_state(pbf_solver* s, pbf_float4* pos, uint32_t* idsOut, int* counts,
                                  size_t count) {
    PBF_GUARD(s, {
        if (count != s->n) fail(PBF_ERR_OUT_OF_RANGE, "count does not match active particles");
        if (count == 0) return;
        s->use_device();
        if (pos)
            cuda_check(cudaMemcpyAsync(pos, s->f4[s->ix].get(), count * sizeof(float4),
                                       cudaMemcpyDeviceToHost, s->stream));
        if (idsOut)
            cuda_check(cudaMemcpyAsync(idsOut, s->ids[s->iid].get(), count * sizeof(uint32_t),
                                       cudaMemcpyDeviceToHost, s->stream));
        if (counts)
            cuda_check(cudaMemcpyAsync(counts, s->cnt.get(), count * sizeof(int),
                                       cudaMemcpyDeviceToHost, s->stream));
        cuda_check(cudaStreamSynchronize(s->stream));
    });
}

}  // extern "C"
