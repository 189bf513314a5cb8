// pbf_stages.cu -- stage entry points of the C ABI (host arrays in and out).
//
// The reference's tests drive SpatialGrid::build, findNeighbors and the
// solver kernels one at a time (test/test_spatial_grid.cu, test/test_neighbors.cu,
// test/test_pbf_solver_kernels.cu, test/test_collision_kernels.cu).  These
// entry points run the same device code the solver uses on caller-provided
// arrays so the same checks can be made against this library.
#include "pbf_common.h"
#include "pbf_kernels.cuh"

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

using namespace pbf;

namespace {

template <class T>
DeviceBuffer upload(const T* h, size_t count) {
    DeviceBuffer b(std::max<size_t>(count, 1) * sizeof(T));
    if (count) cuda_check(cudaMemcpy(b.get(), h, count * sizeof(T), cudaMemcpyHostToDevice));
    return b;
}

template <class T>
void download(T* h, const DeviceBuffer& b, size_t count) {
    if (count) cuda_check(cudaMemcpy(h, b.get(), count * sizeof(T), cudaMemcpyDeviceToHost));
}

void need(const void* p, size_t count, const char* what) {
    if (count && !p) fail(PBF_ERR_INVALID_ARGUMENT, what);
}

void check_count(size_t count) {
    if (count > static_cast<size_t>(std::numeric_limits<int>::max()))
        fail(PBF_ERR_LENGTH, "Particle count exceeds CUDA kernel index range");
}

bool finite3(pbf_float3 v) { return std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z); }

std::vector<int> dims_of(pbf_float3 mn, pbf_float3 mx, float cell) {
    if (!std::isfinite(cell) || cell <= 0.0f)
        fail(PBF_ERR_INVALID_ARGUMENT, "cellSize must be greater than zero");
    if (!finite3(mn) || !finite3(mx) || mx.x <= mn.x || mx.y <= mn.y || mx.z <= mn.z)
        fail(PBF_ERR_INVALID_ARGUMENT, "Invalid spatial grid bounds");
    const float lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z};
    std::vector<int> d(3);
    for (int a = 0; a < 3; ++a) {
        const double c = std::ceil((double(hi[a]) - double(lo[a])) / double(cell));
        if (!std::isfinite(c) || c < 1.0 || c > double(std::numeric_limits<int>::max()))
            fail(PBF_ERR_LENGTH, "Spatial grid axis exceeds integer capacity");
        d[a] = static_cast<int>(c);
    }
    const size_t maxCells = std::numeric_limits<uint32_t>::max();
    if (size_t(d[0]) > maxCells / size_t(d[1]) ||
        size_t(d[0]) * size_t(d[1]) > maxCells / size_t(d[2]))
        fail(PBF_ERR_LENGTH, "Spatial grid exceeds 32-bit key capacity");
    return d;
}

GridConst grid_const(pbf_float3 mn, float cell, const int* d, float h) {
    GridConst g{};
    g.minx = mn.x;
    g.miny = mn.y;
    g.minz = mn.z;
    g.cell = cell;
    g.gx = d[0];
    g.gy = d[1];
    g.gz = d[2];
    const double r = std::ceil(double(h) / double(cell));
    const int maxdim = std::max(d[0], std::max(d[1], d[2]));
    g.radius = static_cast<int>(std::min(std::isfinite(r) ? r : double(maxdim), double(maxdim)));
    return g;
}

StepConst kernel_const(float h, float mass, float rho0, int max_nb, size_t stride) {
    StepConst c{};
    c.k = make_kernel_const(h);
    c.mass = mass;
    c.rho0 = rho0;
    c.gs = mass / rho0;
    c.gs2 = c.gs * c.gs;
    c.max_nb = max_nb;
    c.stride = stride;
    return c;
}

struct ColliderUpload {
    DeviceBuffer buf;
    Colliders col{};
};

ColliderUpload upload_colliders(pbf_float3 cmin, pbf_float3 cmax, const pbf_sphere* s,
                                size_t ns, const pbf_box* b, size_t nb, const pbf_plane* p,
                                size_t np) {
    need(s, ns, "spheres must not be null");
    need(b, nb, "boxes must not be null");
    need(p, np, "planes must not be null");
    std::vector<float4> all;
    for (size_t i = 0; i < ns; ++i)
        all.push_back(make_float4(s[i].center.x, s[i].center.y, s[i].center.z, s[i].radius));
    for (size_t i = 0; i < nb; ++i) {
        all.push_back(make_float4(b[i].center.x, b[i].center.y, b[i].center.z, 0.0f));
        all.push_back(make_float4(b[i].halfExtents.x, b[i].halfExtents.y, b[i].halfExtents.z, 0.0f));
    }
    for (size_t i = 0; i < np; ++i) {
        all.push_back(make_float4(p[i].point.x, p[i].point.y, p[i].point.z, 0.0f));
        all.push_back(make_float4(p[i].normal.x, p[i].normal.y, p[i].normal.z, 0.0f));
    }
    ColliderUpload u;
    u.buf = upload(all.data(), all.size());
    const float4* base = u.buf.as<float4>();
    u.col.spheres = base;
    u.col.boxes = base + ns;
    u.col.planes = base + ns + 2 * nb;
    u.col.ns = static_cast<int>(ns);
    u.col.nb = static_cast<int>(nb);
    u.col.np = static_cast<int>(np);
    u.col.cminx = cmin.x;
    u.col.cminy = cmin.y;
    u.col.cminz = cmin.z;
    u.col.cmaxx = cmax.x;
    u.col.cmaxy = cmax.y;
    u.col.cmaxz = cmax.z;
    return u;
}

}  // namespace

#define STAGE(...) return pbf::guarded(nullptr, [&]() { __VA_ARGS__; })

extern "C" {

pbf_status pbf_grid_dims(pbf_float3 mn, pbf_float3 mx, float cell, int dims[3]) {
    STAGE({
        need(dims, 1, "dims must not be null");
        const auto d = dims_of(mn, mx, cell);
        dims[0] = d[0];
        dims[1] = d[1];
        dims[2] = d[2];
    });
}

pbf_status pbf_grid_build(const pbf_float4* positions, size_t count, pbf_float3 mn,
                          pbf_float3 mx, float cell, uint32_t* sorted_keys,
                          uint32_t* sorted_indices, int* cell_start, int* cell_end) {
    STAGE({
        const auto d = dims_of(mn, mx, cell);
        check_count(count);
        need(positions, count, "predictedPositions must not be null");
        const size_t cells = size_t(d[0]) * size_t(d[1]) * size_t(d[2]);
        need(cell_start, cells, "cell_start must not be null");
        need(cell_end, cells, "cell_end must not be null");
        DeviceBuffer dcs(cells * sizeof(int)), dce(cells * sizeof(int));
        cuda_check(cudaMemset(dcs.get(), 0xff, cells * sizeof(int)));
        cuda_check(cudaMemset(dce.get(), 0xff, cells * sizeof(int)));
        if (count) {
            need(sorted_keys, count, "sorted_keys must not be null");
            need(sorted_indices, count, "sorted_indices must not be null");
            const int n = static_cast<int>(count);
            DeviceBuffer dpos = upload(reinterpret_cast<const float4*>(positions), count);
            DeviceBuffer keys(count * 4), sk(count * 4), si(count * 4), ak(count * 4),
                ai(count * 4), scr(sort_scratch_bytes(n));
            const GridConst g = grid_const(mn, cell, d.data(), cell);
            launch_grid_keys(dpos.as<float4>(), keys.as<uint32_t>(), n, g, nullptr);
            const SortPlan plan = make_sort_plan(n, cells);
            launch_sort(plan, keys.as<uint32_t>(), sk.as<uint32_t>(), si.as<uint32_t>(),
                        ak.as<uint32_t>(), ai.as<uint32_t>(), scr.get(), nullptr, nullptr);
            launch_cell_ranges(sk.as<uint32_t>(), dcs.as<int>(), dce.as<int>(), n, nullptr,
                               nullptr);
            cuda_check(cudaGetLastError());
            cuda_check(cudaDeviceSynchronize());
            download(sorted_keys, sk, count);
            download(sorted_indices, si, count);
        }
        cuda_check(cudaDeviceSynchronize());
        download(cell_start, dcs, cells);
        download(cell_end, dce, cells);
    });
}

pbf_status pbf_find_neighbors(const pbf_float4* sorted_positions, size_t count,
                              const int* cell_start, const int* cell_end, const int dims[3],
                              pbf_float3 mn, float cell, float h, uint32_t* neighbors,
                              int* counts, int max_neighbors, size_t stride, int* overflow) {
    STAGE({
        check_count(count);
        need(dims, 1, "dims must not be null");
        if (max_neighbors < 0) fail(PBF_ERR_INVALID_ARGUMENT, "max_neighbors must be >= 0");
        if (stride < count) fail(PBF_ERR_INVALID_ARGUMENT, "stride must be >= count");
        if (overflow) *overflow = 0;
        if (count == 0) return;
        need(sorted_positions, count, "positions must not be null");
        need(counts, count, "counts must not be null");
        const size_t cells = size_t(dims[0]) * size_t(dims[1]) * size_t(dims[2]);
        const size_t list = stride * size_t(max_neighbors);
        need(neighbors, list, "neighbors must not be null");
        need(cell_start, cells, "cell_start must not be null");
        need(cell_end, cells, "cell_end must not be null");
        // cellStart/cellEnd -> lower bound of every key (empty cells take the
        // next occupied cell's start), the table the search kernel walks.
        std::vector<int> first(cells + 1);
        first[cells] = static_cast<int>(count);
        for (size_t k = cells; k-- > 0;) first[k] = cell_start[k] != -1 ? cell_start[k] : first[k + 1];
        DeviceBuffer dpos = upload(reinterpret_cast<const float4*>(sorted_positions), count);
        DeviceBuffer dfirst = upload(first.data(), first.size());
        DeviceBuffer dnb = upload(neighbors, list);  // untouched slots keep caller values
        DeviceBuffer dcnt(count * sizeof(int)), dstat(sizeof(unsigned));
        cuda_check(cudaMemset(dstat.get(), 0, sizeof(unsigned)));
        StepConst c = kernel_const(h, 1.0f, 1.0f, max_neighbors, stride);
        c.k.h2 = h * h;
        c.g = grid_const(mn, cell, dims, h);
        // Component arrays for the search (identity gather of the given order),
        // padded as the walk needs (soa_stride_for).
        const size_t pad = soa_stride_for(count);
        DeviceBuffer dsoa(3 * pad * sizeof(float)), dids(count * sizeof(uint32_t)),
            dcopy(count * sizeof(float4));
        launch_iota(dids.as<uint32_t>(), static_cast<int>(count), nullptr);
        float* sx = dsoa.as<float>();
        launch_gather_xs(dids.as<uint32_t>(), dpos.as<float4>(), dcopy.as<float4>(), nullptr,
                         nullptr, sx, sx + pad, sx + 2 * pad, static_cast<int>(count), nullptr,
                         nullptr);
        launch_search(dpos.as<float4>(), sx, sx + pad, sx + 2 * pad, dfirst.as<int>(), c,
                      static_cast<int>(count), dnb.as<uint32_t>(), dcnt.as<int>(), nullptr,
                      dstat.as<unsigned>(), false, nullptr);
        cuda_check(cudaGetLastError());
        cuda_check(cudaDeviceSynchronize());
        download(neighbors, dnb, list);
        download(counts, dcnt, count);
        unsigned st = 0;
        download(&st, dstat, 1);
        if (overflow) *overflow = (st & kStatusNeighborOverflow) ? 1 : 0;
    });
}

pbf_status pbf_compute_lambda(const pbf_float4* positions, const uint32_t* neighbors,
                              const int* counts, int max_neighbors, size_t count, size_t stride,
                              float h, float mass, float rho0, float eps, float* lambdas) {
    STAGE({
        check_count(count);
        if (count == 0) return;
        need(positions, count, "positions must not be null");
        need(counts, count, "counts must not be null");
        need(lambdas, count, "lambdas must not be null");
        const size_t list = stride * size_t(max_neighbors);
        DeviceBuffer dpos = upload(reinterpret_cast<const float4*>(positions), count);
        DeviceBuffer dnb = upload(neighbors, list), dcnt = upload(counts, count);
        DeviceBuffer dl(count * sizeof(float));
        StepConst c = kernel_const(h, mass, rho0, max_neighbors, stride);
        c.lambda_eps = eps;
        launch_lambda_list(dpos.as<float4>(), dnb.as<uint32_t>(), dcnt.as<int>(), c,
                           static_cast<int>(count), dl.as<float>(), nullptr);
        cuda_check(cudaGetLastError());
        cuda_check(cudaDeviceSynchronize());
        download(lambdas, dl, count);
    });
}

pbf_status pbf_compute_delta(const pbf_float4* positions, const uint32_t* neighbors,
                             const int* counts, int max_neighbors, const float* lambdas,
                             size_t count, size_t stride, float h, float mass, float rho0,
                             float k, int nexp, float dq, pbf_float4* deltas) {
    STAGE({
        check_count(count);
        if (count == 0) return;
        need(positions, count, "positions must not be null");
        need(lambdas, count, "lambdas must not be null");
        need(deltas, count, "deltas must not be null");
        const size_t list = stride * size_t(max_neighbors);
        DeviceBuffer dpos = upload(reinterpret_cast<const float4*>(positions), count);
        DeviceBuffer dnb = upload(neighbors, list), dcnt = upload(counts, count);
        DeviceBuffer dl = upload(lambdas, count), dd(count * sizeof(float4));
        StepConst c = kernel_const(h, mass, rho0, max_neighbors, stride);
        c.sc = make_scorr_const(h, k, nexp, dq);
        launch_delta_list(dpos.as<float4>(), dnb.as<uint32_t>(), dcnt.as<int>(), dl.as<float>(), c,
                          static_cast<int>(count), dd.as<float4>(), nullptr);
        cuda_check(cudaGetLastError());
        cuda_check(cudaDeviceSynchronize());
        download(reinterpret_cast<float4*>(deltas), dd, count);
    });
}

pbf_status pbf_xsph(const pbf_float4* positions, const uint32_t* neighbors, const int* counts,
                    int max_neighbors, const pbf_float4* velocities, pbf_float4* out,
                    size_t count, size_t stride, float h, float viscosity) {
    STAGE({
        check_count(count);
        if (count == 0) return;
        need(out, count, "output must not be null");
        if (viscosity == 0.0f) {  // applyXsphViscosity copies the input through
            std::copy(velocities, velocities + count, out);
            return;
        }
        const size_t list = stride * size_t(max_neighbors);
        DeviceBuffer dpos = upload(reinterpret_cast<const float4*>(positions), count);
        DeviceBuffer dv = upload(reinterpret_cast<const float4*>(velocities), count);
        DeviceBuffer dnb = upload(neighbors, list), dcnt = upload(counts, count);
        DeviceBuffer dout(count * sizeof(float4));
        StepConst c = kernel_const(h, 1.0f, 1.0f, max_neighbors, stride);
        c.xsph_c = viscosity;
        launch_xsph(dpos.as<float4>(), dv.as<float4>(), dnb.as<uint32_t>(), dcnt.as<int>(), c,
                    static_cast<int>(count), dout.as<float4>(), nullptr, false, nullptr, nullptr);
        cuda_check(cudaGetLastError());
        cuda_check(cudaDeviceSynchronize());
        download(reinterpret_cast<float4*>(out), dout, count);
    });
}

pbf_status pbf_vorticity(const pbf_float4* positions, const pbf_float4* velocities,
                         const uint32_t* neighbors, const int* counts, int max_neighbors,
                         size_t count, size_t stride, float h, pbf_float4* omega) {
    STAGE({
        check_count(count);
        if (count == 0) return;
        need(omega, count, "omega must not be null");
        const size_t list = stride * size_t(max_neighbors);
        DeviceBuffer dpos = upload(reinterpret_cast<const float4*>(positions), count);
        DeviceBuffer dv = upload(reinterpret_cast<const float4*>(velocities), count);
        DeviceBuffer dnb = upload(neighbors, list), dcnt = upload(counts, count);
        DeviceBuffer dout(count * sizeof(float4));
        const StepConst c = kernel_const(h, 1.0f, 1.0f, max_neighbors, stride);
        launch_vorticity(dpos.as<float4>(), dv.as<float4>(), dnb.as<uint32_t>(), dcnt.as<int>(), c,
                         static_cast<int>(count), dout.as<float4>(), false, nullptr, nullptr);
        cuda_check(cudaGetLastError());
        cuda_check(cudaDeviceSynchronize());
        download(reinterpret_cast<float4*>(omega), dout, count);
    });
}

pbf_status pbf_confinement(const pbf_float4* positions, const uint32_t* neighbors,
                           const int* counts, int max_neighbors, const pbf_float4* omega,
                           const pbf_float4* velocities, pbf_float4* out, size_t count,
                           size_t stride, float h, float dt, float strength) {
    STAGE({
        check_count(count);
        if (count == 0) return;
        need(out, count, "output must not be null");
        const size_t list = stride * size_t(max_neighbors);
        DeviceBuffer dpos = upload(reinterpret_cast<const float4*>(positions), count);
        DeviceBuffer dom = upload(reinterpret_cast<const float4*>(omega), count);
        DeviceBuffer dv = upload(reinterpret_cast<const float4*>(velocities), count);
        DeviceBuffer dnb = upload(neighbors, list), dcnt = upload(counts, count);
        DeviceBuffer dout(count * sizeof(float4));
        StepConst c = kernel_const(h, 1.0f, 1.0f, max_neighbors, stride);
        c.dt = dt;
        c.vort_eps = strength;
        launch_omega_norm(dom.as<float4>(), static_cast<int>(count), nullptr);
        launch_confine(dpos.as<float4>(), dnb.as<uint32_t>(), dcnt.as<int>(), dom.as<float4>(),
                       dv.as<float4>(), c, static_cast<int>(count), dout.as<float4>(), nullptr,
                       false, nullptr, nullptr);
        cuda_check(cudaGetLastError());
        cuda_check(cudaDeviceSynchronize());
        download(reinterpret_cast<float4*>(out), dout, count);
    });
}

pbf_status pbf_collision_pass(pbf_float4* positions, size_t count, int kind, pbf_float3 cmin,
                              pbf_float3 cmax, const pbf_sphere* s, size_t ns, const pbf_box* b,
                              size_t nb, const pbf_plane* p, size_t np, float r,
                              int* corrected) {
    STAGE({
        check_count(count);
        if (kind < 0 || kind > 4) fail(PBF_ERR_INVALID_ARGUMENT, "unknown collision kind");
        if (corrected) *corrected = 0;
        if (count == 0) return;
        need(positions, count, "positions must not be null");
        ColliderUpload cu = upload_colliders(cmin, cmax, s, ns, b, nb, p, np);
        DeviceBuffer dpos = upload(reinterpret_cast<const float4*>(positions), count);
        DeviceBuffer flag(sizeof(unsigned));
        cuda_check(cudaMemset(flag.get(), 0, sizeof(unsigned)));
        StepConst c{};
        c.col = cu.col;
        c.particle_radius = r;
        launch_collide(dpos.as<float4>(), static_cast<int>(count), c, kind, flag.as<unsigned>(),
                       nullptr);
        cuda_check(cudaGetLastError());
        cuda_check(cudaDeviceSynchronize());
        download(reinterpret_cast<float4*>(positions), dpos, count);
        unsigned h = 0;
        download(&h, flag, 1);
        if (corrected) *corrected = h ? 1 : 0;
    });
}

pbf_status pbf_collide(pbf_float4* positions, size_t count, pbf_float3 cmin, pbf_float3 cmax,
                       const pbf_sphere* s, size_t ns, const pbf_box* b, size_t nb,
                       const pbf_plane* p, size_t np, float r) {
    int bad = 0;
    const pbf_status st =
        pbf_collision_pass(positions, count, 4, cmin, cmax, s, ns, b, nb, p, np, r, &bad);
    if (st != PBF_OK) return st;
    if (bad) {
        set_global_error("Collision constraints did not converge");
        return PBF_ERR_RUNTIME;
    }
    return PBF_OK;
}

pbf_status pbf_resolve_velocities(const pbf_float4* positions, const pbf_float4* vin,
                                  pbf_float4* vel, size_t count, pbf_float3 cmin, pbf_float3 cmax,
                                  const pbf_sphere* s, size_t ns, const pbf_box* b, size_t nb,
                                  const pbf_plane* p, size_t np, float r, float e, float fr) {
    STAGE({
        check_count(count);
        if (count == 0) return;
        need(positions, count, "positions must not be null");
        need(vin, count, "incoming velocities must not be null");
        need(vel, count, "velocities must not be null");
        ColliderUpload cu = upload_colliders(cmin, cmax, s, ns, b, nb, p, np);
        DeviceBuffer dpos = upload(reinterpret_cast<const float4*>(positions), count);
        DeviceBuffer dvin = upload(reinterpret_cast<const float4*>(vin), count);
        DeviceBuffer dv = upload(reinterpret_cast<const float4*>(vel), count);
        StepConst c{};
        c.col = cu.col;
        c.particle_radius = r;
        c.restitution = e;
        c.friction = fr;
        launch_resolve(dpos.as<float4>(), dvin.as<float4>(), dv.as<float4>(), c,
                       static_cast<int>(count), nullptr, nullptr);
        cuda_check(cudaGetLastError());
        cuda_check(cudaDeviceSynchronize());
        download(reinterpret_cast<float4*>(vel), dv, count);
    });
}

pbf_status pbf_integrate(const pbf_float4* positions, pbf_float4* predicted, pbf_float4* vel,
                         size_t count, float dt, pbf_float3 gravity) {
    STAGE({
        check_count(count);
        if (count == 0) return;
        need(positions, count, "positions must not be null");
        need(predicted, count, "predicted must not be null");
        need(vel, count, "velocities must not be null");
        DeviceBuffer dx = upload(reinterpret_cast<const float4*>(positions), count);
        DeviceBuffer dv = upload(reinterpret_cast<const float4*>(vel), count);
        DeviceBuffer dxs(count * sizeof(float4));
        StepConst c{};
        c.dt = dt;
        c.gravx = gravity.x;
        c.gravy = gravity.y;
        c.gravz = gravity.z;
        launch_integrate(dx.as<float4>(), dxs.as<float4>(), dv.as<float4>(),
                         static_cast<int>(count), c, nullptr);
        cuda_check(cudaGetLastError());
        cuda_check(cudaDeviceSynchronize());
        download(reinterpret_cast<float4*>(predicted), dxs, count);
        download(reinterpret_cast<float4*>(vel), dv, count);
    });
}

}  // extern "C"
