// pbf_diff_oracle.cpp -- FP64 restatement of the differentiated PBF step
// with forward-mode tangents.  Test infrastructure: the checker for the
// GPU adjoint (central finite differences run it without tangents; the
// forward-mode gradient runs it with them).
//
// One step, in the reference's formulas evaluated in double
// (include/pbf/sph_helpers.cuh:13-95, src/pbf/pbf_solver_kernels.cu:26-385,
// src/pbf/collision_kernels.cu:21-82,236-276, src/pbf/pbf_solver.cu:198-325):
//   v1 = v + g dt, p = x + v1 dt
//   I times: neighbours of p (|p_i - p_j|^2 <= h^2, j != i),
//            rho_i = m (W(0) + sum W_ij), C_i = rho_i / rho0 - 1,
//            lambda_i = -C_i / (gs^2 (sum |g_ij|^2 + |sum g_ij|^2) + eps),
//            p_i <- clamp(p_i + gs sum (lambda_i + lambda_j + s_corr_ij) g_ij)
//   neighbours of p; v2 = (p - x) / dt; v3 = v2 + c sum (v2_j - v2_i) W_ij;
//   with vorticity strength eps: w_i = sum g_ij x (v3_j - v3_i),
//   eta_i = sum (|w_j| - |w_i|) g_ij, v3 <- v3 + dt eps (eta/|eta| x w_i);
//   v4 = container contacts of v3 against v1 at p; x <- p, v <- v4.
// Values are double; every quantity carries K tangents (Dual<K>), the
// derivatives along K input directions of (x0, v0, rho0, c).  Neighbour sets,
// clamps and contact decisions follow the values only.
#include "pbf_oracle.h"

#include <algorithm>
#include <cfloat>
#include <array>
#include <cmath>
#include <cstddef>
#include <vector>

#include <omp.h>

namespace {

template <int K>
struct Dual {
    double v = 0.0;
    std::array<double, K> d{};
    Dual() = default;
    Dual(double x) : v(x) {}  // NOLINT: constants promote implicitly
};
template <int K> Dual<K> operator+(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v + b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <int K> Dual<K> operator-(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v - b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <int K> Dual<K> operator-(const Dual<K>& a) {
    Dual<K> r(-a.v);
    for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
    return r;
}
template <int K> Dual<K> operator*(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v * b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
template <int K> Dual<K> operator/(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v / b.v);
    for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
    return r;
}
template <int K> Dual<K> dsqrt(const Dual<K>& a) {
    Dual<K> r(std::sqrt(a.v));
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] / (2.0 * r.v);
    return r;
}
template <int K> Dual<K> ipow(Dual<K> b, int n) {
    Dual<K> r(1.0);
    for (int i = 0; i < n; ++i) r = r * b;
    return r;
}

template <int K>
struct D3 {
    Dual<K> x, y, z;
};
template <int K> D3<K> operator+(const D3<K>& a, const D3<K>& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <int K> D3<K> operator-(const D3<K>& a, const D3<K>& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <int K> D3<K> operator*(const Dual<K>& s, const D3<K>& a) { return {s * a.x, s * a.y, s * a.z}; }
template <int K> Dual<K> dot(const D3<K>& a, const D3<K>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <int K> D3<K> cross(const D3<K>& a, const D3<K>& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// |a|, with a zero derivative at a = 0 (where the norm has none).
template <int K> Dual<K> norm3(const D3<K>& a) {
    const Dual<K> q = dot(a, a);
    return q.v > 0.0 ? dsqrt(q) : Dual<K>(0.0);
}

template <int K>
struct Diff {
    size_t n;
    orc_params p;
    orc_float3 lo, hi;
    double h, h2;
    int gx, gy, gz;
    Dual<K> rho0, xsph;
    std::vector<D3<K>> x, v;
    std::vector<std::vector<int>> nb;
    bool failed = false;  // a projection that did not converge

    void cell_of(double px, double py, double pz, int& cx, int& cy, int& cz) const {
        auto c1 = [&](double q, double m, int g) {
            double f = std::floor((q - m) / h);
            if (!(f >= 0.0)) f = 0.0;  // NaN and below
            if (f > double(g - 1)) f = double(g - 1);
            return int(f);
        };
        cx = c1(px, lo.x, gx);
        cy = c1(py, lo.y, gy);
        cz = c1(pz, lo.z, gz);
    }

    // Neighbours of every particle by the values of p (cell grid, 27 cells).
    void lists(const std::vector<D3<K>>& q) {
        const size_t cells = size_t(gx) * gy * gz;
        std::vector<std::vector<int>> bucket(cells);
        std::vector<int> cell(n);
        for (size_t i = 0; i < n; ++i) {
            int cx, cy, cz;
            cell_of(q[i].x.v, q[i].y.v, q[i].z.v, cx, cy, cz);
            cell[i] = cx + gx * (cy + gy * cz);
            bucket[cell[i]].push_back(int(i));
        }
        nb.assign(n, {});
#pragma omp parallel for schedule(dynamic, 256)
        for (long ii = 0; ii < long(n); ++ii) {
            const size_t i = size_t(ii);
            const int c = cell[i];
            const int cx = c % gx, cy = (c / gx) % gy, cz = c / (gx * gy);
            for (int z = std::max(0, cz - 1); z <= std::min(gz - 1, cz + 1); ++z)
                for (int y = std::max(0, cy - 1); y <= std::min(gy - 1, cy + 1); ++y)
                    for (int xq = std::max(0, cx - 1); xq <= std::min(gx - 1, cx + 1); ++xq)
                        for (int j : bucket[size_t(xq) + gx * (size_t(y) + gy * size_t(z))]) {
                            if (size_t(j) == i) continue;
                            const double dx = q[i].x.v - q[j].x.v, dy = q[i].y.v - q[j].y.v,
                                         dz = q[i].z.v - q[j].z.v;
                            if (dx * dx + dy * dy + dz * dz <= h2) nb[i].push_back(j);
                        }
        }
    }

    Dual<K> poly6(const Dual<K>& d2) const {
        if (d2.v >= h2) return Dual<K>(0.0);
        const double norm = 315.0 / (64.0 * M_PI) / h / h / h;
        const Dual<K> t = Dual<K>(1.0) - d2 / Dual<K>(h2);
        return Dual<K>(norm) * t * t * t;
    }
    D3<K> spiky(const D3<K>& r, const Dual<K>& d2) const {
        const Dual<K> rr = dsqrt(d2);
        if (rr.v <= 0.0 || rr.v >= h) return {Dual<K>(0.0), Dual<K>(0.0), Dual<K>(0.0)};
        const double norm = -45.0 / M_PI / h / h / h / h;
        const Dual<K> t = Dual<K>(1.0) - rr / Dual<K>(h);
        return (Dual<K>(norm) * t * t / rr) * r;
    }
    Dual<K> scorr(const Dual<K>& d2) const {
        const double dq2 = double(p.scorrDeltaQ) * p.scorrDeltaQ;
        if (p.scorrK == 0.0f || p.scorrN <= 0 || d2.v >= h2 || dq2 >= h2) return Dual<K>(0.0);
        const Dual<K> ratio = (Dual<K>(h2) - d2) / Dual<K>(h2 - dq2);
        return Dual<K>(-double(p.scorrK)) * ipow(ratio * ratio * ratio, p.scorrN);
    }

    // solveContainerKernel (collision_kernels.cu:47-82); true when moved.
    bool clamp(D3<K>& q) const {
        const double r = p.particleRadius;
        const double minX = double(lo.x) + r, maxX = double(hi.x) - r;
        const double minY = double(lo.y) + r;
        const double minZ = double(lo.z) + r, maxZ = double(hi.z) - r;
        bool mark = false;
        auto lim = [&](Dual<K>& a, double v) { a = Dual<K>(v); mark = true; };
        if (q.x.v < minX) lim(q.x, minX);
        if (q.x.v > maxX) lim(q.x, maxX);
        if (q.y.v < minY) lim(q.y, minY);
        if (q.z.v < minZ) lim(q.z, minZ);
        if (q.z.v > maxZ) lim(q.z, maxZ);
        return mark;
    }

    // Sphere, box and plane colliders (collision_kernels.cu:84-234): the
    // projections, decided on the values, carrying the tangents.
    std::vector<orc_sphere> sph;
    std::vector<orc_box> bxs;
    std::vector<orc_plane> pls;

    // projectionTolerance (collision_kernels.cu:9-14).
    static double tol(const D3<K>& q, double ox, double oy, double oz, double rad) {
        double t = std::fmax(rad, std::fmax(std::fabs(q.x.v), std::fabs(ox)));
        t = std::fmax(t, std::fmax(std::fabs(q.y.v), std::fabs(oy)));
        t = std::fmax(t, std::fmax(std::fabs(q.z.v), std::fabs(oz)));
        return double(8.0f * FLT_EPSILON) * t;
    }
    // clamp of one coordinate into [lo, hi], keeping the tangent inside.
    static Dual<K> clamp1(const Dual<K>& a, double lo_, double hi_) {
        if (a.v < lo_) return Dual<K>(lo_);
        if (a.v > hi_) return Dual<K>(hi_);
        return a;
    }
    static void plane_unit(const orc_plane& pl, double& nx, double& ny, double& nz) {
        const double nl = std::sqrt(double(pl.normal.x) * pl.normal.x +
                                    double(pl.normal.y) * pl.normal.y +
                                    double(pl.normal.z) * pl.normal.z);
        nx = pl.normal.x / nl;
        ny = pl.normal.y / nl;
        nz = pl.normal.z / nl;
    }
    bool proj_spheres(D3<K>& q) const {
        const double r = p.particleRadius;
        bool mark = false;
        for (const orc_sphere& sp : sph) {
            const double cx = sp.center.x, cy = sp.center.y, cz = sp.center.z;
            const double minD = double(sp.radius) + r;
            const D3<K> o{q.x - Dual<K>(cx), q.y - Dual<K>(cy), q.z - Dual<K>(cz)};
            const Dual<K> d2 = dot(o, o);
            if (!(d2.v < minD * minD)) continue;
            if (minD - std::sqrt(d2.v) <= tol(q, cx, cy, cz, minD)) continue;
            mark = true;
            if (d2.v == 0.0) {
                q.x = Dual<K>(cx + minD);
            } else {
                const Dual<K> scale = Dual<K>(minD) / dsqrt(d2);
                q = D3<K>{Dual<K>(cx), Dual<K>(cy), Dual<K>(cz)} + scale * o;
            }
        }
        return mark;
    }
    bool proj_boxes(D3<K>& q) const {
        const double r = p.particleRadius;
        bool mark = false;
        for (const orc_box& b : bxs) {
            const double mnx = double(b.center.x) - b.halfExtents.x;
            const double mny = double(b.center.y) - b.halfExtents.y;
            const double mnz = double(b.center.z) - b.halfExtents.z;
            const double mxx = double(b.center.x) + b.halfExtents.x;
            const double mxy = double(b.center.y) + b.halfExtents.y;
            const double mxz = double(b.center.z) + b.halfExtents.z;
            const D3<K> cl{clamp1(q.x, mnx, mxx), clamp1(q.y, mny, mxy), clamp1(q.z, mnz, mxz)};
            const D3<K> o = q - cl;
            const Dual<K> d2 = dot(o, o);
            if (d2.v > 0.0 && d2.v < r * r) {
                if (r - std::sqrt(d2.v) <= tol(q, cl.x.v, cl.y.v, cl.z.v, r)) continue;
                mark = true;
                q = cl + (Dual<K>(r) / dsqrt(d2)) * o;
            } else if (d2.v == 0.0) {
                mark = true;
                const double dX = std::fmin(q.x.v - mnx, mxx - q.x.v);
                const double dY = std::fmin(q.y.v - mny, mxy - q.y.v);
                const double dZ = std::fmin(q.z.v - mnz, mxz - q.z.v);
                if (dX <= dY && dX <= dZ)
                    q.x = Dual<K>(q.x.v - mnx < mxx - q.x.v ? mnx - r : mxx + r);
                else if (dY <= dZ)
                    q.y = Dual<K>(q.y.v - mny < mxy - q.y.v ? mny - r : mxy + r);
                else
                    q.z = Dual<K>(q.z.v - mnz < mxz - q.z.v ? mnz - r : mxz + r);
            }
        }
        return mark;
    }
    bool proj_planes(D3<K>& q) const {
        const double r = p.particleRadius;
        bool mark = false;
        for (const orc_plane& pl : pls) {
            if (pl.normal.x == 0.0f && pl.normal.y == 0.0f && pl.normal.z == 0.0f) continue;
            double nx, ny, nz;
            plane_unit(pl, nx, ny, nz);
            const D3<K> n{Dual<K>(nx), Dual<K>(ny), Dual<K>(nz)};
            const D3<K> pt{Dual<K>(pl.point.x), Dual<K>(pl.point.y), Dual<K>(pl.point.z)};
            const Dual<K> dist = dot(q - pt, n);
            if (!(dist.v < r)) continue;
            if (r - dist.v <= tol(q, pl.point.x, pl.point.y, pl.point.z, r)) continue;
            mark = true;
            q = q + (Dual<K>(r) - dist) * n;
        }
        return mark;
    }
    // CollisionSystem::solve per particle (collision_system.cu:133-172): to
    // the fixed point, at most 32 passes; false when it did not converge.
    bool project(D3<K>& q) const {
        for (int pass = 0; pass < 32; ++pass) {
            bool mark = clamp(q);
            if (!sph.empty()) mark = proj_spheres(q) || mark;
            if (!bxs.empty()) mark = proj_boxes(q) || mark;
            if (!pls.empty()) mark = proj_planes(q) || mark;
            if (!mark) return true;
        }
        return false;
    }

    // resolveContactVelocity for an axis normal (collision_kernels.cu:21-43).
    void contact(int a, double s, const D3<K>& vin, D3<K>& vv) const {
        Dual<K>* c[3] = {&vv.x, &vv.y, &vv.z};
        const Dual<K>* ci[3] = {&vin.x, &vin.y, &vin.z};
        const Dual<K> vn = Dual<K>(s) * *c[a];
        const Dual<K> vinn = Dual<K>(s) * *ci[a];
        const Dual<K> target =
            vinn.v < 0.0 ? Dual<K>(-double(p.collisionRestitution)) * vinn : Dual<K>(0.0);
        if (vn.v > target.v || (vn.v == target.v && vinn.v >= 0.0)) return;
        const Dual<K> ts(1.0 - double(p.collisionFriction));
        for (int b = 0; b < 3; ++b)
            *c[b] = b == a ? Dual<K>(s) * target : ts * *c[b];
    }
    // resolveContactVelocity against a unit normal n that may carry tangents.
    void contact_n(const D3<K>& n, const D3<K>& vin, D3<K>& vv) const {
        const Dual<K> vn = dot(vv, n), vinn = dot(vin, n);
        const Dual<K> target =
            vinn.v < 0.0 ? Dual<K>(-double(p.collisionRestitution)) * vinn : Dual<K>(0.0);
        if (vn.v > target.v || (vn.v == target.v && vinn.v >= 0.0)) return;
        const Dual<K> ts(1.0 - double(p.collisionFriction));
        vv = ts * (vv - vn * n) + target * n;
    }
    void respond(const D3<K>& pos, const D3<K>& vin, D3<K>& vv) const {
        const double r = p.particleRadius, eps = double(1e-4f);  // kContactEpsilon
        const double minX = double(lo.x) + r, maxX = double(hi.x) - r;
        const double minY = double(lo.y) + r;
        const double minZ = double(lo.z) + r, maxZ = double(hi.z) - r;
        if (pos.x.v <= minX + eps) contact(0, 1.0, vin, vv);
        else if (pos.x.v >= maxX - eps) contact(0, -1.0, vin, vv);
        if (pos.y.v <= minY + eps) contact(1, 1.0, vin, vv);
        if (pos.z.v <= minZ + eps) contact(2, 1.0, vin, vv);
        else if (pos.z.v >= maxZ - eps) contact(2, -1.0, vin, vv);
        for (const orc_sphere& sp : sph) {
            const double minD = double(sp.radius) + r;
            const D3<K> o{pos.x - Dual<K>(sp.center.x), pos.y - Dual<K>(sp.center.y),
                          pos.z - Dual<K>(sp.center.z)};
            const Dual<K> d2 = dot(o, o);
            const double cd = minD + eps;
            if (d2.v > 0.0 && d2.v <= cd * cd) contact_n((Dual<K>(1.0) / dsqrt(d2)) * o, vin, vv);
        }
        for (const orc_box& b : bxs) {
            const double mnx = double(b.center.x) - b.halfExtents.x;
            const double mny = double(b.center.y) - b.halfExtents.y;
            const double mnz = double(b.center.z) - b.halfExtents.z;
            const double mxx = double(b.center.x) + b.halfExtents.x;
            const double mxy = double(b.center.y) + b.halfExtents.y;
            const double mxz = double(b.center.z) + b.halfExtents.z;
            const D3<K> cl{clamp1(pos.x, mnx, mxx), clamp1(pos.y, mny, mxy),
                           clamp1(pos.z, mnz, mxz)};
            const D3<K> o = pos - cl;
            const Dual<K> d2 = dot(o, o);
            const double re = r + eps;
            if (d2.v > 0.0 && d2.v <= re * re) {
                contact_n((Dual<K>(1.0) / dsqrt(d2)) * o, vin, vv);
            } else if (d2.v == 0.0) {
                const double dX = std::fmin(pos.x.v - mnx, mxx - pos.x.v);
                const double dY = std::fmin(pos.y.v - mny, mxy - pos.y.v);
                const double dZ = std::fmin(pos.z.v - mnz, mxz - pos.z.v);
                double n3[3] = {0.0, 0.0, 0.0};
                if (dX <= dY && dX <= dZ) n3[0] = pos.x.v - mnx < mxx - pos.x.v ? -1.0 : 1.0;
                else if (dY <= dZ) n3[1] = pos.y.v - mny < mxy - pos.y.v ? -1.0 : 1.0;
                else n3[2] = pos.z.v - mnz < mxz - pos.z.v ? -1.0 : 1.0;
                contact_n(D3<K>{Dual<K>(n3[0]), Dual<K>(n3[1]), Dual<K>(n3[2])}, vin, vv);
            }
        }
        for (const orc_plane& pl : pls) {
            if (pl.normal.x == 0.0f && pl.normal.y == 0.0f && pl.normal.z == 0.0f) continue;
            double nx, ny, nz;
            plane_unit(pl, nx, ny, nz);
            const double dist = (pos.x.v - pl.point.x) * nx + (pos.y.v - pl.point.y) * ny +
                                (pos.z.v - pl.point.z) * nz;
            if (dist <= r + eps)
                contact_n(D3<K>{Dual<K>(nx), Dual<K>(ny), Dual<K>(nz)}, vin, vv);
        }
    }

    // One frame: `substeps` substeps of dt / substeps (rounded to float as
    // the solver forms it, src/pbf/pbf_solver.cu:193).
    void step() {
        const float sub_dt = p.dt / float(p.substeps);
        for (int k = 0; k < p.substeps; ++k) substep(double(sub_dt));
    }

    void substep(double dt_value) {
        const Dual<K> dt(dt_value), m(p.particleMass), eps(p.lambdaEpsilon);
        const Dual<K> gs = m / rho0, gs2 = gs * gs;
        const D3<K> g{Dual<K>(p.gravity.x), Dual<K>(p.gravity.y), Dual<K>(p.gravity.z)};
        std::vector<D3<K>> v1(n), q(n), nq(n);
        for (size_t i = 0; i < n; ++i) {
            v1[i] = v[i] + dt * g;
            q[i] = x[i] + dt * v1[i];
        }
        std::vector<Dual<K>> lam(n);
        const double w0 = 315.0 / (64.0 * M_PI) / h / h / h;
        for (int it = 0; it < p.solverIterations; ++it) {
            lists(q);
#pragma omp parallel for schedule(dynamic, 256)
            for (long ii = 0; ii < long(n); ++ii) {
                const size_t i = size_t(ii);
                Dual<K> wsum(w0), s2(0.0);
                D3<K> G{Dual<K>(0.0), Dual<K>(0.0), Dual<K>(0.0)};
                for (int j : nb[i]) {
                    const D3<K> r = q[i] - q[size_t(j)];
                    const Dual<K> d2 = dot(r, r);
                    wsum = wsum + poly6(d2);
                    const D3<K> gr = spiky(r, d2);
                    s2 = s2 + dot(gr, gr);
                    G = G + gr;
                }
                const Dual<K> C = m * wsum / rho0 - Dual<K>(1.0);
                lam[i] = -C / (gs2 * (s2 + dot(G, G)) + eps);
            }
#pragma omp parallel for schedule(dynamic, 256)
            for (long ii = 0; ii < long(n); ++ii) {
                const size_t i = size_t(ii);
                D3<K> acc{Dual<K>(0.0), Dual<K>(0.0), Dual<K>(0.0)};
                for (int j : nb[i]) {
                    const D3<K> r = q[i] - q[size_t(j)];
                    const Dual<K> d2 = dot(r, r);
                    acc = acc + (lam[i] + lam[size_t(j)] + scorr(d2)) * spiky(r, d2);
                }
                D3<K> np = q[i] + gs * acc;
                if (!project(np)) failed = true;
                nq[i] = np;
            }
            q.swap(nq);
        }
        lists(q);
        std::vector<D3<K>> v2(n), v3(n);
        for (size_t i = 0; i < n; ++i) v2[i] = Dual<K>(1.0) / dt * (q[i] - x[i]);
#pragma omp parallel for schedule(dynamic, 256)
        for (long ii = 0; ii < long(n); ++ii) {
            const size_t i = size_t(ii);
            D3<K> acc{Dual<K>(0.0), Dual<K>(0.0), Dual<K>(0.0)};
            for (int j : nb[i]) {
                const D3<K> r = q[i] - q[size_t(j)];
                acc = acc + poly6(dot(r, r)) * (v2[size_t(j)] - v2[i]);
            }
            v3[i] = v2[i] + xsph * acc;
        }
        if (p.vorticityStrength != 0.0f) {
            // computeVorticity / applyVorticityConfinement
            // (pbf_solver_kernels.cu:268-385): w_i = sum_j grad W_ij x (v_j - v_i),
            // eta_i = sum_j (|w_j| - |w_i|) grad W_ij, v += dt eps (eta/|eta| x w_i).
            std::vector<D3<K>> w(n);
            std::vector<Dual<K>> mw(n);
#pragma omp parallel for schedule(dynamic, 256)
            for (long ii = 0; ii < long(n); ++ii) {
                const size_t i = size_t(ii);
                D3<K> acc{Dual<K>(0.0), Dual<K>(0.0), Dual<K>(0.0)};
                for (int j : nb[i]) {
                    const D3<K> r = q[i] - q[size_t(j)];
                    acc = acc + cross(spiky(r, dot(r, r)), v3[size_t(j)] - v3[i]);
                }
                w[i] = acc;
                mw[i] = norm3(acc);
            }
            const Dual<K> eps_v(double(p.vorticityStrength));
            std::vector<D3<K>> v5(n);
#pragma omp parallel for schedule(dynamic, 256)
            for (long ii = 0; ii < long(n); ++ii) {
                const size_t i = size_t(ii);
                D3<K> eta{Dual<K>(0.0), Dual<K>(0.0), Dual<K>(0.0)};
                for (int j : nb[i]) {
                    const D3<K> r = q[i] - q[size_t(j)];
                    eta = eta + (mw[size_t(j)] - mw[i]) * spiky(r, dot(r, r));
                }
                const Dual<K> le = norm3(eta);
                D3<K> N{Dual<K>(0.0), Dual<K>(0.0), Dual<K>(0.0)};
                if (le.v > 1.0e-6) N = (Dual<K>(1.0) / le) * eta;
                v5[i] = v3[i] + (dt * eps_v) * cross(N, w[i]);
            }
            v3.swap(v5);
        }
        for (size_t i = 0; i < n; ++i) {
            D3<K> vv = v3[i];
            respond(q[i], v1[i], vv);
            v[i] = vv;
        }
        x.swap(q);
    }
};

template <int K>
int run(size_t n, const orc_float4* x0, const orc_float4* v0, const double* tx0,
        const double* tv0, const double* trho, const double* tc, int ntan, const orc_params* prm,
        orc_float3 lo, orc_float3 hi, int steps, const orc_float4* states, double* x_out,
        double* v_out, double* tx_out, double* tv_out, const double* phys,
        const orc_sphere* sp, size_t ns, const orc_box* bx, size_t nb, const orc_plane* pl,
        size_t np) {
    Diff<K> s;
    s.n = n;
    s.p = *prm;
    s.lo = lo;
    s.hi = hi;
    s.h = prm->smoothingRadius;
    s.h2 = s.h * s.h;
    int dims[3];
    if (orc_grid_dims(lo, hi, prm->smoothingRadius, dims) != ORC_OK) return ORC_ERR_INVALID;
    s.gx = dims[0];
    s.gy = dims[1];
    s.gz = dims[2];
    // phys (optional): rest density and XSPH strength in double, so central
    // differences may take steps below float32 resolution.
    if (sp) s.sph.assign(sp, sp + ns);
    if (bx) s.bxs.assign(bx, bx + nb);
    if (pl) s.pls.assign(pl, pl + np);
    s.rho0 = Dual<K>(phys ? phys[0] : double(prm->restDensity));
    s.xsph = Dual<K>(phys ? phys[1] : double(prm->xsphViscosity));
    for (int k = 0; k < ntan; ++k) {
        s.rho0.d[size_t(k)] = trho ? trho[k] : 0.0;
        s.xsph.d[size_t(k)] = tc ? tc[k] : 0.0;
    }
    s.x.resize(n);
    s.v.resize(n);
    for (size_t i = 0; i < n; ++i) {
        s.x[i] = {Dual<K>(x0[i].x), Dual<K>(x0[i].y), Dual<K>(x0[i].z)};
        s.v[i] = {Dual<K>(v0[i].x), Dual<K>(v0[i].y), Dual<K>(v0[i].z)};
        for (int k = 0; k < ntan; ++k) {
            const size_t o = (size_t(k) * n + i) * 3;
            if (tx0) {
                s.x[i].x.d[size_t(k)] = tx0[o];
                s.x[i].y.d[size_t(k)] = tx0[o + 1];
                s.x[i].z.d[size_t(k)] = tx0[o + 2];
            }
            if (tv0) {
                s.v[i].x.d[size_t(k)] = tv0[o];
                s.v[i].y.d[size_t(k)] = tv0[o + 1];
                s.v[i].z.d[size_t(k)] = tv0[o + 2];
            }
        }
    }
    for (int t = 0; t < steps; ++t) {
        if (states && t > 0) {
            // Linearise about a given trajectory: the values restart from its
            // state at the start of step t, the tangents carry on.
            const orc_float4* xs = states + size_t(t) * 2 * n;
            const orc_float4* vs = xs + n;
            for (size_t i = 0; i < n; ++i) {
                s.x[i].x.v = xs[i].x;
                s.x[i].y.v = xs[i].y;
                s.x[i].z.v = xs[i].z;
                s.v[i].x.v = vs[i].x;
                s.v[i].y.v = vs[i].y;
                s.v[i].z.v = vs[i].z;
            }
        }
        s.step();
        if (s.failed) return ORC_ERR_NOT_CONVERGED;
    }
    for (size_t i = 0; i < n; ++i) {
        const D3<K>& a = s.x[i];
        const D3<K>& b = s.v[i];
        x_out[3 * i] = a.x.v;
        x_out[3 * i + 1] = a.y.v;
        x_out[3 * i + 2] = a.z.v;
        v_out[3 * i] = b.x.v;
        v_out[3 * i + 1] = b.y.v;
        v_out[3 * i + 2] = b.z.v;
        for (int k = 0; k < ntan; ++k) {
            const size_t o = (size_t(k) * n + i) * 3;
            if (tx_out) {
                tx_out[o] = a.x.d[size_t(k)];
                tx_out[o + 1] = a.y.d[size_t(k)];
                tx_out[o + 2] = a.z.d[size_t(k)];
            }
            if (tv_out) {
                tv_out[o] = b.x.d[size_t(k)];
                tv_out[o + 1] = b.y.d[size_t(k)];
                tv_out[o + 2] = b.z.d[size_t(k)];
            }
        }
    }
    return ORC_OK;
}

}  // namespace

extern "C" int orc_diff_rollout_col(size_t n, const orc_float4* x0, const orc_float4* v0,
                                    const double* tx0, const double* tv0, const double* trho,
                                    const double* tc, int ntan, const orc_params* prm,
                                    orc_float3 lo, orc_float3 hi, int steps,
                                    const orc_float4* states, double* x_out, double* v_out,
                                    double* tx_out, double* tv_out, const double* phys,
                                    const orc_sphere* sp, size_t ns, const orc_box* bx,
                                    size_t nb, const orc_plane* pl, size_t np) {
    if (!prm || !x0 || !v0 || !x_out || !v_out || ntan < 0 || ntan > 12 || steps < 0)
        return ORC_ERR_INVALID;
    if ((ns && !sp) || (nb && !bx) || (np && !pl)) return ORC_ERR_INVALID;
    if (ntan == 0)
        return run<0>(n, x0, v0, nullptr, nullptr, nullptr, nullptr, 0, prm, lo, hi, steps,
                      states, x_out, v_out, nullptr, nullptr, phys, sp, ns, bx, nb, pl, np);
    if (ntan <= 4)
        return run<4>(n, x0, v0, tx0, tv0, trho, tc, ntan, prm, lo, hi, steps, states, x_out,
                      v_out, tx_out, tv_out, phys, sp, ns, bx, nb, pl, np);
    return run<12>(n, x0, v0, tx0, tv0, trho, tc, ntan, prm, lo, hi, steps, states, x_out, v_out,
                   tx_out, tv_out, phys, sp, ns, bx, nb, pl, np);
}

extern "C" int orc_diff_rollout_phys(size_t n, const orc_float4* x0, const orc_float4* v0,
                                     const double* tx0, const double* tv0, const double* trho,
                                     const double* tc, int ntan, const orc_params* prm,
                                     orc_float3 lo, orc_float3 hi, int steps,
                                     const orc_float4* states, double* x_out, double* v_out,
                                     double* tx_out, double* tv_out, const double* phys) {
    return orc_diff_rollout_col(n, x0, v0, tx0, tv0, trho, tc, ntan, prm, lo, hi, steps, states,
                                x_out, v_out, tx_out, tv_out, phys, nullptr, 0, nullptr, 0,
                                nullptr, 0);
}

extern "C" int orc_diff_rollout(size_t n, const orc_float4* x0, const orc_float4* v0,
                                const double* tx0, const double* tv0, const double* trho,
                                const double* tc, int ntan, const orc_params* prm,
                                orc_float3 lo, orc_float3 hi, int steps,
                                const orc_float4* states, double* x_out, double* v_out,
                                double* tx_out, double* tv_out) {
    return orc_diff_rollout_col(n, x0, v0, tx0, tv0, trho, tc, ntan, prm, lo, hi, steps, states,
                                x_out, v_out, tx_out, tv_out, nullptr, nullptr, 0, nullptr, 0,
                                nullptr, 0);
}
