// pbf_oracle.cpp -- CPU oracle for the Position Based Fluids step.
//
// TEST INFRASTRUCTURE ONLY: this file is the checker for the CUDA library in
// this repository and the timed CPU baseline.  It restates the reference
// solver (DusanCojic/Fluid-Simulator) on the host; every function names the
// reference file:line it follows.  Nothing in the product links it.
//
// Build: g++ -O2 -std=c++17 -fopenmp -ffp-contract=off -fPIC -shared.
// -ffp-contract=off is required: every fused multiply-add below is written
// out with std::fma, every other operation is one IEEE rounding, so the FP32
// mode reproduces the CUDA kernels bit for bit.

#include "pbf_oracle.h"

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr float kPiF = 3.14159265358979323846f;
constexpr double kPiD = 3.14159265358979323846;
constexpr int kMaxCollisionPasses = 32;   // src/pbf/collision_system.cu:148
constexpr float kContactEpsilon = 1e-4f;  // src/pbf/collision_kernels.cu:254
constexpr float kEtaEpsilon = 1.0e-6f;    // src/pbf/pbf_solver_kernels.cu:367

template <class T> struct V4 { T x, y, z, w; };
template <class T> struct V3 { T x, y, z; };

// Device float->int conversion saturates and maps NaN to 0; on the host the
// plain cast is undefined for out-of-range values, so saturate explicitly
// (include/pbf/spatial_grid.cuh:65-81 relies on the device behaviour).
inline int sat_int(double v) {
    if (std::isnan(v)) return 0;
    if (v >= 2147483647.0) return INT_MAX;
    if (v <= -2147483648.0) return INT_MIN;
    return static_cast<int>(v);
}

// ---------------------------------------------------------------------------
// Arithmetic policies.  F32: the operation sequence of this repository's CUDA
// kernels.  F64: the reference formulas (include/pbf/sph_helpers.cuh,
// src/pbf/pbf_solver_kernels.cu) evaluated in double.
// ---------------------------------------------------------------------------

struct F32 {
    using T = float;
    T h = 0, h2 = 0, inv_h = 0, inv_h2 = 0, c_poly6 = 0, c_spiky = 0;

    void init(float hh) {
        h = hh;
        h2 = hh * hh;
        inv_h = 1.0f / hh;
        inv_h2 = 1.0f / h2;
        c_poly6 = 315.0f / (64.0f * kPiF) / hh / hh / hh;
        c_spiky = -45.0f / kPiF / hh / hh / hh / hh;
    }
    // Squared length rounded as the reference's compiled findNeighbors rounds
    // dx*dx + dy*dy + dz*dz (src/pbf/neighbors.cu:73-74): fma(dz, dz,
    // fma(dy, dy, dx*dx)).
    static T dist2(T dx, T dy, T dz) { return std::fma(dz, dz, std::fma(dy, dy, dx * dx)); }
    static T len(T x, T y, T z) { return std::sqrt(dist2(x, y, z)); }
    // poly6FromDistanceSquared (include/pbf/sph_helpers.cuh:13-34).
    T poly6(T d2) const {
        if (d2 >= h2) return 0.0f;
        const T t = std::fma(-d2, inv_h2, 1.0f);
        const T t2 = t * t;
        const T t3 = t2 * t;
        return c_poly6 * t3;
    }
    // Reciprocal square root by Newton's method from the bit-level seed of
    // C. Lomont, "Fast Inverse Square Root" (2003), constant 0x5f375a86:
    // three steps y <- y (3/2 - (x/2) y^2) as multiply / fma, the sequence of
    // the CUDA kernels.
    static T rsqrt_nt(T x) {
        uint32_t bits;
        std::memcpy(&bits, &x, sizeof bits);
        bits = 0x5f375a86u - (bits >> 1);
        T y;
        std::memcpy(&y, &bits, sizeof y);
        const T nxh = -0.5f * x;
        for (int it = 0; it < 3; ++it) y = y * std::fma(nxh * y, y, 1.5f);
        return y;
    }
    // spikyGradientFromDistanceSquared (include/pbf/sph_helpers.cuh:48-81):
    // g = d * s, s = c_spiky (1 - r/h)^2 / r with r = d2 * rsqrt(d2); zero
    // for d2 >= h^2 and for d2 < 2^-100 (coincident within 2^-50).
    void spiky(T dx, T dy, T dz, T d2, T g[3]) const {
        if (d2 < 7.8886090522101181e-31f || d2 >= h2) { g[0] = g[1] = g[2] = 0.0f; return; }
        const T rr = rsqrt_nt(d2);
        const T r = d2 * rr;
        const T t = std::fma(-r, inv_h, 1.0f);
        const T s = (c_spiky * (t * t)) * rr;
        g[0] = dx * s;
        g[1] = dy * s;
        g[2] = dz * s;
    }
    static T fma_(T a, T b, T c) { return std::fma(a, b, c); }
    // a.y*b.z - a.z*b.y with one rounding of the product a.y*b.z.
    static T cross_x(T ay, T az, T by, T bz) { return std::fma(ay, bz, -(az * by)); }
};

struct F64 {
    using T = double;
    T h = 0, h2 = 0;
    void init(float hh) { h = hh; h2 = h * h; }
    static T dist2(T dx, T dy, T dz) { return dx * dx + dy * dy + dz * dz; }
    static T len(T x, T y, T z) { return std::sqrt(dist2(x, y, z)); }
    T poly6(T d2) const {
        if (d2 >= h2) return 0.0;
        const T norm = 315.0 / (64.0 * kPiD) / h / h / h;
        const T t = 1.0 - d2 / h2;
        return norm * t * t * t;
    }
    void spiky(T dx, T dy, T dz, T d2, T g[3]) const {
        const T r = std::sqrt(d2);
        if (r <= 0.0 || r >= h) { g[0] = g[1] = g[2] = 0.0; return; }
        const T norm = -45.0 / kPiD / h / h / h / h;
        const T t = 1.0 - r / h;
        const T mag = norm * t * t;
        g[0] = dx / r * mag;
        g[1] = dy / r * mag;
        g[2] = dz / r * mag;
    }
    static T fma_(T a, T b, T c) { return a * b + c; }
    static T cross_x(T ay, T az, T by, T bz) { return ay * bz - az * by; }
};

// Integer power by squaring, fixed sequence shared with the CUDA kernels.
inline float ipow_f(float b, int n) {
    float r = 1.0f;
    while (n > 0) {
        if (n & 1) r = r * b;
        n >>= 1;
        if (n) b = b * b;
    }
    return r;
}

// computeArtificialPressure (include/pbf/pbf_solver_kernels.cuh:24-47).
struct Scorr32 {
    float k = 0, negk = 0, h2 = 0, dq2 = 0, inv_den = 0;
    int n = 0;
    void init(float h, float kk, int nn, float dq) {
        k = kk; negk = -kk; n = nn; h2 = h * h; dq2 = dq * dq;
        inv_den = 1.0f / (h2 - dq2);
    }
    float operator()(float d2) const {
        if (k == 0.0f || n <= 0) return 0.0f;
        if (d2 >= h2 || dq2 >= h2) return 0.0f;
        const float ratio = (h2 - d2) * inv_den;
        const float r3 = (ratio * ratio) * ratio;
        return negk * ipow_f(r3, n);
    }
};
struct Scorr64 {
    double k = 0, h2 = 0, dq2 = 0;
    int n = 0;
    void init(float h, float kk, int nn, float dq) {
        k = kk; n = nn; h2 = double(h) * h; dq2 = double(dq) * dq;
    }
    double operator()(double d2) const {
        if (k == 0.0 || n <= 0) return 0.0;
        if (d2 >= h2 || dq2 >= h2) return 0.0;
        const double ratio = std::pow((h2 - d2) / (h2 - dq2), 3.0);
        return -k * std::pow(ratio, double(n));
    }
};
template <class P> struct ScorrOf;
template <> struct ScorrOf<F32> { using type = Scorr32; };
template <> struct ScorrOf<F64> { using type = Scorr64; };

// ---------------------------------------------------------------------------
// Spatial grid (src/pbf/spatial_grid.cu, include/pbf/spatial_grid.cuh:65-102)
// ---------------------------------------------------------------------------

struct Grid {
    int gx = 0, gy = 0, gz = 0;
    float minx = 0, miny = 0, minz = 0, cell = 0;
    size_t cells = 0;
};

// SpatialGrid::initialize dims (src/pbf/spatial_grid.cu:37-64).
int grid_dims(orc_float3 mn, orc_float3 mx, float cell, int d[3]) {
    if (!std::isfinite(cell) || cell <= 0.0f) return ORC_ERR_INVALID;
    if (!std::isfinite(mn.x) || !std::isfinite(mn.y) || !std::isfinite(mn.z) ||
        !std::isfinite(mx.x) || !std::isfinite(mx.y) || !std::isfinite(mx.z) ||
        mx.x <= mn.x || mx.y <= mn.y || mx.z <= mn.z)
        return ORC_ERR_INVALID;
    const float lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z};
    for (int a = 0; a < 3; ++a) {
        const double c = std::ceil((double(hi[a]) - double(lo[a])) / double(cell));
        if (!std::isfinite(c) || c < 1.0 || c > double(INT_MAX)) return ORC_ERR_LENGTH;
        d[a] = int(c);
    }
    const size_t maxCells = 0xFFFFFFFFu;
    const size_t cx = size_t(d[0]), cy = size_t(d[1]), cz = size_t(d[2]);
    if (cx > maxCells / cy || cx * cy > maxCells / cz) return ORC_ERR_LENGTH;
    return ORC_OK;
}

// positionToCell + clampCellToGrid, FP32 (spatial_grid.cuh:65-102).
inline void cell_of(const Grid& g, float px, float py, float pz, int c[3]) {
    c[0] = sat_int(std::floor((px - g.minx) / g.cell));
    c[1] = sat_int(std::floor((py - g.miny) / g.cell));
    c[2] = sat_int(std::floor((pz - g.minz) / g.cell));
    c[0] = std::max(0, std::min(c[0], g.gx - 1));
    c[1] = std::max(0, std::min(c[1], g.gy - 1));
    c[2] = std::max(0, std::min(c[2], g.gz - 1));
}
// FP64 cell: same rule evaluated on double positions.
inline void cell_of(const Grid& g, double px, double py, double pz, int c[3]) {
    c[0] = sat_int(std::floor((px - double(g.minx)) / double(g.cell)));
    c[1] = sat_int(std::floor((py - double(g.miny)) / double(g.cell)));
    c[2] = sat_int(std::floor((pz - double(g.minz)) / double(g.cell)));
    c[0] = std::max(0, std::min(c[0], g.gx - 1));
    c[1] = std::max(0, std::min(c[1], g.gy - 1));
    c[2] = std::max(0, std::min(c[2], g.gz - 1));
}
// cellToKey: u64 arithmetic truncated to u32 (spatial_grid.cuh:83-90).
inline uint32_t key_of(const Grid& g, const int c[3]) {
    return uint32_t(uint64_t(c[0]) + uint64_t(c[1]) * uint64_t(g.gx) +
                    uint64_t(c[2]) * uint64_t(g.gx) * uint64_t(g.gy));
}

// Stable counting sort of the current order by key (CUB SortPairs over all
// 32 key bits is a stable LSD sort, src/pbf/spatial_grid.cu:188-196), then
// buildCellRanges (src/pbf/spatial_grid.cu:123-137).
void stable_sort_keys(const uint32_t* keys, size_t n, size_t cells, uint32_t* sortedKeys,
                      uint32_t* sortedIdx, int* cellStart, int* cellEnd,
                      std::vector<uint32_t>& scratch) {
    scratch.assign(cells + 1, 0u);
    for (size_t i = 0; i < n; ++i) scratch[keys[i] + 1]++;
    for (size_t c = 0; c < cells; ++c) scratch[c + 1] += scratch[c];
    for (size_t i = 0; i < n; ++i) {
        const uint32_t k = keys[i];
        const uint32_t pos = scratch[k]++;
        sortedIdx[pos] = uint32_t(i);
        sortedKeys[pos] = k;
    }
    if (cellStart) {
        std::fill(cellStart, cellStart + cells, -1);
        std::fill(cellEnd, cellEnd + cells, -1);
        for (size_t i = 0; i < n; ++i) {
            const uint32_t k = sortedKeys[i];
            if (i == 0 || sortedKeys[i - 1] != k) cellStart[k] = int(i);
            if (i == n - 1 || sortedKeys[i + 1] != k) cellEnd[k] = int(i + 1);
        }
    }
}

// findNeighbors' neighbourhood radius in cells (src/pbf/neighbors.cu:39-50):
// ceil in double, then the [first, last] bounds clamped to the grid.
inline void search_bounds(const Grid& g, double radius, const int c[3], int first[3],
                          int last[3]) {
    const int dims[3] = {g.gx, g.gy, g.gz};
    for (int a = 0; a < 3; ++a) {
        first[a] = int(std::fmax(0.0, double(c[a]) - radius));
        last[a] = int(std::fmin(double(dims[a] - 1), double(c[a]) + radius));
    }
}

template <class T> inline T vsub(T a, T b) { return a - b; }

// One particle's cell walk: z -> y -> x over clamped cells, ranges in sorted
// order, self skipped, accept d2 <= h2 (src/pbf/neighbors.cu:52-86).
// Visitor receives every accepted neighbour index in list order.
template <class P, class Pos, class Visit>
int walk_neighbors(const P& m, const Grid& g, double radius, const Pos* sp, size_t i,
                   const int* cs, const int* ce, typename P::T h2, Visit&& visit) {
    using T = typename P::T;
    const Pos pi = sp[i];
    int c[3];
    cell_of(g, pi.x, pi.y, pi.z, c);
    int first[3], last[3];
    search_bounds(g, radius, c, first, last);
    int count = 0;
    for (int z = first[2]; z <= last[2]; ++z)
        for (int y = first[1]; y <= last[1]; ++y)
            for (int x = first[0]; x <= last[0]; ++x) {
                const int cc[3] = {x, y, z};
                const uint32_t key = key_of(g, cc);
                const int s = cs[key], e = ce[key];
                if (s == -1) continue;
                for (int j = s; j < e; ++j) {
                    if (size_t(j) == i) continue;
                    const T dx = T(pi.x) - T(sp[j].x);
                    const T dy = T(pi.y) - T(sp[j].y);
                    const T dz = T(pi.z) - T(sp[j].z);
                    const T d2 = m.dist2(dx, dy, dz);
                    if (d2 <= h2) {
                        visit(count, uint32_t(j));
                        ++count;
                    }
                }
            }
    (void)m;
    return count;
}

inline void set_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

// ---------------------------------------------------------------------------
// Per-particle stages on particle-major lists nb[i*cap + k].
// ---------------------------------------------------------------------------

template <class P>
struct Stages {
    using T = typename P::T;
    using Pos = V4<T>;
    P m;
    typename ScorrOf<P>::type sc;

    // computeLambda (src/pbf/pbf_solver_kernels.cu:26-105).
    T lambda_one(const Pos* x, const uint32_t* nb, int cnt, int cap, size_t i, T mass,
                 T rho0, T eps) const {
        if (cnt < 0 || cnt > cap) return T(NAN);
        const Pos pi = x[i];
        if constexpr (std::is_same<P, F32>::value) {
            const float gs = mass / rho0;
            float wsum = m.poly6(0.0f);
            float s2 = 0.0f, gx = 0.0f, gy = 0.0f, gz = 0.0f;
            for (int k = 0; k < cnt; ++k) {
                const Pos pj = x[nb[k]];
                const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                const float d2 = m.dist2(dx, dy, dz);
                wsum = wsum + m.poly6(d2);
                float g[3];
                m.spiky(dx, dy, dz, d2, g);
                s2 = std::fma(g[2], g[2], std::fma(g[1], g[1], std::fma(g[0], g[0], s2)));
                gx = gx + g[0]; gy = gy + g[1]; gz = gz + g[2];
            }
            const float rho = mass * wsum;
            const float g2 = m.dist2(gx, gy, gz);
            const float denom = std::fma(gs * gs, s2 + g2, eps);
            const float C = rho / rho0 - 1.0f;
            return -C / denom;
        } else {
            const double gs = mass / rho0;
            double rho = mass * m.poly6(0.0), sum = 0, gx = 0, gy = 0, gz = 0;
            for (int k = 0; k < cnt; ++k) {
                const Pos pj = x[nb[k]];
                const double dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                const double d2 = m.dist2(dx, dy, dz);
                rho += mass * m.poly6(d2);
                double g[3];
                m.spiky(dx, dy, dz, d2, g);
                const double jx = -gs * g[0], jy = -gs * g[1], jz = -gs * g[2];
                sum += jx * jx + jy * jy + jz * jz;
                gx -= jx; gy -= jy; gz -= jz;
            }
            sum += gx * gx + gy * gy + gz * gz;
            const double C = rho / rho0 - 1.0;
            return -C / (sum + eps);
        }
    }

    // computeDeltaPosition (src/pbf/pbf_solver_kernels.cu:108-182); the
    // caller adds the result (applyDeltaPosition, :184-193).
    void delta_one(const Pos* x, const uint32_t* nb, int cnt, int cap, const T* lam,
                   size_t i, T gs, T out[3]) const {
        if (cnt < 0 || cnt > cap) { out[0] = out[1] = out[2] = T(NAN); return; }
        const Pos pi = x[i];
        const T li = lam[i];
        T ax = 0, ay = 0, az = 0;
        for (int k = 0; k < cnt; ++k) {
            const uint32_t j = nb[k];
            const Pos pj = x[j];
            const T dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const T d2 = m.dist2(dx, dy, dz);
            T g[3];
            m.spiky(dx, dy, dz, d2, g);
            const T ls = (li + lam[j]) + sc(d2);
            ax = P::fma_(ls, g[0], ax);
            ay = P::fma_(ls, g[1], ay);
            az = P::fma_(ls, g[2], az);
        }
        out[0] = gs * ax; out[1] = gs * ay; out[2] = gs * az;
    }

    // applyXsphViscosity (src/pbf/pbf_solver_kernels.cu:213-266).
    Pos xsph_one(const Pos* x, const Pos* v, const uint32_t* nb, int cnt, int cap, size_t i,
                 T c) const {
        const Pos vi = v[i];
        if (cnt < 0 || cnt > cap) return Pos{T(NAN), T(NAN), T(NAN), vi.w};
        const Pos pi = x[i];
        T cx = 0, cy = 0, cz = 0;
        for (int k = 0; k < cnt; ++k) {
            const uint32_t j = nb[k];
            const Pos pj = x[j], vj = v[j];
            const T dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const T w = m.poly6(m.dist2(dx, dy, dz));
            cx = P::fma_(vj.x - vi.x, w, cx);
            cy = P::fma_(vj.y - vi.y, w, cy);
            cz = P::fma_(vj.z - vi.z, w, cz);
        }
        return Pos{P::fma_(c, cx, vi.x), P::fma_(c, cy, vi.y), P::fma_(c, cz, vi.z), vi.w};
    }

    // computeVorticity (src/pbf/pbf_solver_kernels.cu:268-315).
    Pos omega_one(const Pos* x, const Pos* v, const uint32_t* nb, int cnt, int cap,
                  size_t i) const {
        if (cnt < 0 || cnt > cap) return Pos{T(NAN), T(NAN), T(NAN), T(0)};
        const Pos pi = x[i], vi = v[i];
        T ox = 0, oy = 0, oz = 0;
        for (int k = 0; k < cnt; ++k) {
            const uint32_t j = nb[k];
            const Pos pj = x[j], vj = v[j];
            const T dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            T g[3];
            m.spiky(dx, dy, dz, m.dist2(dx, dy, dz), g);
            const T vx = vj.x - vi.x, vy = vj.y - vi.y, vz = vj.z - vi.z;
            ox = ox + P::cross_x(g[1], g[2], vy, vz);
            oy = oy + P::cross_x(g[2], g[0], vz, vx);
            oz = oz + P::cross_x(g[0], g[1], vx, vy);
        }
        return Pos{ox, oy, oz, T(0)};
    }

    // applyVorticityConfinement (src/pbf/pbf_solver_kernels.cu:317-385).
    Pos confine_one(const Pos* x, const uint32_t* nb, int cnt, int cap, const Pos* om,
                    const Pos* v, size_t i, T dt, T eps) const {
        const Pos vi = v[i];
        if (cnt < 0 || cnt > cap) return Pos{T(NAN), T(NAN), T(NAN), vi.w};
        const Pos pi = x[i], wi = om[i];
        const T wil = P::len(wi.x, wi.y, wi.z);
        T ex = 0, ey = 0, ez = 0;
        for (int k = 0; k < cnt; ++k) {
            const uint32_t j = nb[k];
            const Pos pj = x[j], wj = om[j];
            const T wjl = P::len(wj.x, wj.y, wj.z);
            const T dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            T g[3];
            m.spiky(dx, dy, dz, m.dist2(dx, dy, dz), g);
            const T md = wjl - wil;
            ex = P::fma_(md, g[0], ex);
            ey = P::fma_(md, g[1], ey);
            ez = P::fma_(md, g[2], ez);
        }
        const T el = P::len(ex, ey, ez);
        T nx = 0, ny = 0, nz = 0;
        if (el > T(kEtaEpsilon)) { nx = ex / el; ny = ey / el; nz = ez / el; }
        const T cx = eps * P::cross_x(ny, nz, wi.y, wi.z);
        const T cy = eps * P::cross_x(nz, nx, wi.z, wi.x);
        const T cz = eps * P::cross_x(nx, ny, wi.x, wi.y);
        return Pos{P::fma_(dt, cx, vi.x), P::fma_(dt, cy, vi.y), P::fma_(dt, cz, vi.z), vi.w};
    }
};

// ---------------------------------------------------------------------------
// Collisions (src/pbf/collision_kernels.cu), templated on precision.
// ---------------------------------------------------------------------------

template <class P>
struct Collide {
    using T = typename P::T;
    using Pos = V4<T>;

    // projectionTolerance (collision_kernels.cu:9-14).
    static T tol(const Pos& p, T ox, T oy, T oz, T rad) {
        T s = std::fmax(rad, std::fmax(std::fabs(p.x), std::fabs(ox)));
        s = std::fmax(s, std::fmax(std::fabs(p.y), std::fabs(oy)));
        s = std::fmax(s, std::fmax(std::fabs(p.z), std::fabs(oz)));
        return T(8.0f * FLT_EPSILON) * s;
    }
    // solveContainerKernel (:47-82).
    static bool container(Pos& p, const orc_container& c, T r) {
        const T minX = T(c.min.x) + r, maxX = T(c.max.x) - r;
        const T minY = T(c.min.y) + r;
        const T minZ = T(c.min.z) + r, maxZ = T(c.max.z) - r;
        const Pos o = p;
        p.x = std::fmin(std::fmax(p.x, minX), maxX);
        p.y = std::fmax(p.y, minY);
        p.z = std::fmin(std::fmax(p.z, minZ), maxZ);
        return p.x != o.x || p.y != o.y || p.z != o.z;
    }
    // solveSpheresKernel (:84-124).
    static bool spheres(Pos& p, const orc_sphere* s, size_t ns, T r) {
        bool mark = false;
        for (size_t k = 0; k < ns; ++k) {
            const T cx = s[k].center.x, cy = s[k].center.y, cz = s[k].center.z;
            const T minD = T(s[k].radius) + r;
            const T ox = p.x - cx, oy = p.y - cy, oz = p.z - cz;
            const T d2 = P::dist2(ox, oy, oz);
            if (d2 < minD * minD) {
                if (minD - std::sqrt(d2) <= tol(p, cx, cy, cz, minD)) continue;
                mark = true;
                if (d2 == T(0)) {
                    p.x = cx + minD;
                } else {
                    const T scale = minD / std::sqrt(d2);
                    p.x = P::fma_(ox, scale, cx);
                    p.y = P::fma_(oy, scale, cy);
                    p.z = P::fma_(oz, scale, cz);
                }
            }
        }
        return mark;
    }
    // solveBoxesKernel (:126-189).
    static bool boxes(Pos& p, const orc_box* b, size_t nb, T r) {
        bool mark = false;
        for (size_t k = 0; k < nb; ++k) {
            const T mnx = T(b[k].center.x) - T(b[k].halfExtents.x);
            const T mny = T(b[k].center.y) - T(b[k].halfExtents.y);
            const T mnz = T(b[k].center.z) - T(b[k].halfExtents.z);
            const T mxx = T(b[k].center.x) + T(b[k].halfExtents.x);
            const T mxy = T(b[k].center.y) + T(b[k].halfExtents.y);
            const T mxz = T(b[k].center.z) + T(b[k].halfExtents.z);
            const T clx = std::fmin(std::fmax(p.x, mnx), mxx);
            const T cly = std::fmin(std::fmax(p.y, mny), mxy);
            const T clz = std::fmin(std::fmax(p.z, mnz), mxz);
            const T ox = p.x - clx, oy = p.y - cly, oz = p.z - clz;
            const T d2 = P::dist2(ox, oy, oz);
            if (d2 > T(0) && d2 < r * r) {
                if (r - std::sqrt(d2) <= tol(p, clx, cly, clz, r)) continue;
                mark = true;
                const T scale = r / std::sqrt(d2);
                p.x = P::fma_(ox, scale, clx);
                p.y = P::fma_(oy, scale, cly);
                p.z = P::fma_(oz, scale, clz);
            } else if (d2 == T(0)) {
                mark = true;
                const T dX = std::fmin(p.x - mnx, mxx - p.x);
                const T dY = std::fmin(p.y - mny, mxy - p.y);
                const T dZ = std::fmin(p.z - mnz, mxz - p.z);
                if (dX <= dY && dX <= dZ)
                    p.x = p.x - mnx < mxx - p.x ? mnx - r : mxx + r;
                else if (dY <= dZ)
                    p.y = p.y - mny < mxy - p.y ? mny - r : mxy + r;
                else
                    p.z = p.z - mnz < mxz - p.z ? mnz - r : mxz + r;
            }
        }
        return mark;
    }
    // solvePlanesKernel (:191-234).
    static bool planes(Pos& p, const orc_plane* pl, size_t np, T r) {
        bool mark = false;
        for (size_t k = 0; k < np; ++k) {
            const T nl2 = P::dist2(pl[k].normal.x, pl[k].normal.y, pl[k].normal.z);
            if (nl2 == T(0)) continue;
            const T ns = T(1) / std::sqrt(nl2);
            const T nx = T(pl[k].normal.x) * ns, ny = T(pl[k].normal.y) * ns,
                    nz = T(pl[k].normal.z) * ns;
            const T px = pl[k].point.x, py = pl[k].point.y, pz = pl[k].point.z;
            const T dist = P::fma_(p.z - pz, nz, P::fma_(p.y - py, ny, (p.x - px) * nx));
            if (dist < r) {
                if (r - dist <= tol(p, px, py, pz, r)) continue;
                mark = true;
                const T corr = r - dist;
                p.x = P::fma_(nx, corr, p.x);
                p.y = P::fma_(ny, corr, p.y);
                p.z = P::fma_(nz, corr, p.z);
            }
        }
        return mark;
    }
    // CollisionSystem::solve (src/pbf/collision_system.cu:133-172), per
    // particle: a pass that marks nothing leaves the particle unchanged, so
    // iterating each particle to its own fixed point equals the global loop.
    static bool solve(Pos& p, const orc_container& c, const orc_sphere* s, size_t ns,
                      const orc_box* b, size_t nb, const orc_plane* pl, size_t np, T r,
                      int maxPasses) {
        for (int pass = 0; pass < maxPasses; ++pass) {
            bool mark = container(p, c, r);
            if (ns) mark = spheres(p, s, ns, r) || mark;
            if (nb) mark = boxes(p, b, nb, r) || mark;
            if (np) mark = planes(p, pl, np, r) || mark;
            if (!mark) return true;
        }
        return false;
    }

    // resolveContactVelocity (:21-43).
    static void contact(T nx, T ny, T nz, const Pos& vin, T e, T ts, Pos& v) {
        const T vn = P::fma_(v.z, nz, P::fma_(v.y, ny, v.x * nx));
        const T vinn = P::fma_(vin.z, nz, P::fma_(vin.y, ny, vin.x * nx));
        const T target = vinn < T(0) ? (-e) * vinn : T(0);
        if (vn > target || (vn == target && vinn >= T(0))) return;
        const T tx = P::fma_(-vn, nx, v.x), ty = P::fma_(-vn, ny, v.y),
                tz = P::fma_(-vn, nz, v.z);
        v.x = P::fma_(ts, tx, target * nx);
        v.y = P::fma_(ts, ty, target * ny);
        v.z = P::fma_(ts, tz, target * nz);
    }
    // resolveVelocitiesKernel (:236-371).
    static void resolve(const Pos& p, const Pos& vin, Pos& v, const orc_container& c,
                        const orc_sphere* s, size_t ns, const orc_box* b, size_t nb,
                        const orc_plane* pl, size_t np, T r, T e, T fr) {
        const T ts = T(1) - fr;
        const T eps = T(kContactEpsilon);
        const T minX = T(c.min.x) + r, maxX = T(c.max.x) - r;
        const T minY = T(c.min.y) + r;
        const T minZ = T(c.min.z) + r, maxZ = T(c.max.z) - r;
        if (p.x <= minX + eps) contact(1, 0, 0, vin, e, ts, v);
        else if (p.x >= maxX - eps) contact(-1, 0, 0, vin, e, ts, v);
        if (p.y <= minY + eps) contact(0, 1, 0, vin, e, ts, v);
        if (p.z <= minZ + eps) contact(0, 0, 1, vin, e, ts, v);
        else if (p.z >= maxZ - eps) contact(0, 0, -1, vin, e, ts, v);
        for (size_t k = 0; k < ns; ++k) {
            const T minD = T(s[k].radius) + r;
            const T ox = p.x - T(s[k].center.x), oy = p.y - T(s[k].center.y),
                    oz = p.z - T(s[k].center.z);
            const T d2 = P::dist2(ox, oy, oz);
            const T cd = minD + eps;
            if (d2 > T(0) && d2 <= cd * cd) {
                const T sc = T(1) / std::sqrt(d2);
                contact(ox * sc, oy * sc, oz * sc, vin, e, ts, v);
            }
        }
        for (size_t k = 0; k < nb; ++k) {
            const T mnx = T(b[k].center.x) - T(b[k].halfExtents.x);
            const T mny = T(b[k].center.y) - T(b[k].halfExtents.y);
            const T mnz = T(b[k].center.z) - T(b[k].halfExtents.z);
            const T mxx = T(b[k].center.x) + T(b[k].halfExtents.x);
            const T mxy = T(b[k].center.y) + T(b[k].halfExtents.y);
            const T mxz = T(b[k].center.z) + T(b[k].halfExtents.z);
            const T clx = std::fmin(std::fmax(p.x, mnx), mxx);
            const T cly = std::fmin(std::fmax(p.y, mny), mxy);
            const T clz = std::fmin(std::fmax(p.z, mnz), mxz);
            const T ox = p.x - clx, oy = p.y - cly, oz = p.z - clz;
            const T d2 = P::dist2(ox, oy, oz);
            const T re = r + eps;
            T nx, ny, nz;
            if (d2 > T(0) && d2 <= re * re) {
                const T sc = T(1) / std::sqrt(d2);
                nx = ox * sc; ny = oy * sc; nz = oz * sc;
            } else if (d2 == T(0)) {
                const T dX = std::fmin(p.x - mnx, mxx - p.x);
                const T dY = std::fmin(p.y - mny, mxy - p.y);
                const T dZ = std::fmin(p.z - mnz, mxz - p.z);
                nx = ny = nz = T(0);
                if (dX <= dY && dX <= dZ) nx = p.x - mnx < mxx - p.x ? T(-1) : T(1);
                else if (dY <= dZ) ny = p.y - mny < mxy - p.y ? T(-1) : T(1);
                else nz = p.z - mnz < mxz - p.z ? T(-1) : T(1);
            } else {
                continue;
            }
            contact(nx, ny, nz, vin, e, ts, v);
        }
        for (size_t k = 0; k < np; ++k) {
            const T nl2 = P::dist2(pl[k].normal.x, pl[k].normal.y, pl[k].normal.z);
            if (nl2 == T(0)) continue;
            const T ns_ = T(1) / std::sqrt(nl2);
            const T nx = T(pl[k].normal.x) * ns_, ny = T(pl[k].normal.y) * ns_,
                    nz = T(pl[k].normal.z) * ns_;
            const T dist = P::fma_(p.z - T(pl[k].point.z), nz,
                                   P::fma_(p.y - T(pl[k].point.y), ny,
                                           (p.x - T(pl[k].point.x)) * nx));
            if (dist <= r + eps) contact(nx, ny, nz, vin, e, ts, v);
        }
    }
};

// ---------------------------------------------------------------------------
// Whole solver.
// ---------------------------------------------------------------------------

struct SolverBase {
    virtual ~SolverBase() = default;
    virtual int initialize(size_t maxParticles, orc_float3 mn, orc_float3 mx,
                           const orc_params& p, int maxNeighbors) = 0;
    virtual int set_particles(const orc_float4* pos, const orc_float4* vel, size_t n) = 0;
    virtual void set_colliders(const orc_sphere* s, size_t ns, const orc_box* b, size_t nb,
                               const orc_plane* pl, size_t np) = 0;
    virtual int step() = 0;
    virtual int copy_positions(orc_float4* out, size_t n) const = 0;
    virtual int copy_velocities(orc_float4* out, size_t n) const = 0;
    virtual int copy_working(orc_float4* pos, uint32_t* ids, int* counts, size_t n) const = 0;
    virtual int density_error(double* mean, double* mx) const = 0;
    int threads = 0;
};

template <class P>
struct Solver final : SolverBase {
    using T = typename P::T;
    using Pos = V4<T>;

    orc_params prm{};
    Grid g;
    orc_container box{};
    std::vector<orc_sphere> spheres;
    std::vector<orc_box> boxes;
    std::vector<orc_plane> planes;
    size_t cap = 0, n = 0;
    int maxNb = 256;
    double radius = 1.0;
    T h2 = 0;
    Stages<P> st;

    // Working set in the current spatial order (PBFSolver members,
    // include/pbf/pbf_solver.hpp:45-66).
    std::vector<Pos> x, xs, v, vin, tmp, om, dp;
    std::vector<uint32_t> id, keys, skeys, sidx, nb, scratch;
    std::vector<int> cs, ce, cnt;
    std::vector<T> lam;
    std::vector<uint32_t> id2;

    int initialize(size_t maxParticles, orc_float3 mn, orc_float3 mx, const orc_params& p,
                   int maxNeighbors) override {
        int d[3];
        const int st_ = grid_dims(mn, mx, p.smoothingRadius, d);
        if (st_ != ORC_OK) return st_;
        prm = p;
        g.gx = d[0]; g.gy = d[1]; g.gz = d[2];
        g.minx = mn.x; g.miny = mn.y; g.minz = mn.z;
        g.cell = p.smoothingRadius;
        g.cells = size_t(d[0]) * size_t(d[1]) * size_t(d[2]);
        box.min = mn; box.max = mx;
        cap = maxParticles;
        maxNb = maxNeighbors;
        radius = std::ceil(double(p.smoothingRadius) / double(p.smoothingRadius));
        st.m.init(p.smoothingRadius);
        st.sc.init(p.smoothingRadius, p.scorrK, p.scorrN, p.scorrDeltaQ);
        h2 = T(p.smoothingRadius) * T(p.smoothingRadius);
        n = 0;
        return ORC_OK;
    }

    int set_particles(const orc_float4* pos, const orc_float4* vel, size_t count) override {
        if (count > cap) return ORC_ERR_INVALID;
        n = count;
        x.resize(n); v.resize(n); xs.resize(n); vin.resize(n); tmp.resize(n);
        om.resize(n); dp.resize(n); id.resize(n); id2.resize(n); keys.resize(n);
        skeys.resize(n); sidx.resize(n); lam.resize(n); cnt.assign(n, 0);
        nb.assign(n * size_t(maxNb), 0u);
        cs.assign(g.cells, -1); ce.assign(g.cells, -1);
        for (size_t i = 0; i < n; ++i) {
            x[i] = Pos{T(pos[i].x), T(pos[i].y), T(pos[i].z), T(pos[i].w)};
            v[i] = Pos{T(vel[i].x), T(vel[i].y), T(vel[i].z), T(vel[i].w)};
            id[i] = uint32_t(i);  // initializeStableParticleIds
        }
        return ORC_OK;
    }

    void set_colliders(const orc_sphere* s, size_t ns, const orc_box* b, size_t nb_,
                       const orc_plane* pl, size_t np) override {
        spheres.assign(s, s + ns);
        boxes.assign(b, b + nb_);
        planes.assign(pl, pl + np);
    }

    // SpatialGrid::build + PBFSolver::reorderWorkingSet (pbf_solver.cu:154-172).
    void build_and_reorder() {
        const long long N = (long long)n;
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < N; ++i) {
            int c[3];
            cell_of(g, xs[i].x, xs[i].y, xs[i].z, c);
            keys[i] = key_of(g, c);
        }
        stable_sort_keys(keys.data(), n, g.cells, skeys.data(), sidx.data(), cs.data(),
                         ce.data(), scratch);
        permute(x); permute(xs); permute(v); permute(vin);
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < N; ++i) id2[i] = id[sidx[i]];
        id.swap(id2);
    }
    void permute(std::vector<Pos>& a) {
        const long long N = (long long)n;
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < N; ++i) tmp[i] = a[sidx[i]];
        a.swap(tmp);
    }

    // findNeighbors over the working order; returns true on overflow.
    bool search() {
        const long long N = (long long)n;
        int overflow = 0;
#pragma omp parallel for schedule(static) reduction(| : overflow)
        for (long long i = 0; i < N; ++i) {
            uint32_t* row = nb.data() + size_t(i) * size_t(maxNb);
            const int mnb = maxNb;
            const int c = walk_neighbors(st.m, g, radius, xs.data(), size_t(i), cs.data(),
                                         ce.data(), h2, [&](int k, uint32_t j) {
                                             if (k < mnb) row[k] = j;
                                         });
            cnt[i] = c;
            if (c > maxNb) overflow = 1;
        }
        return overflow != 0;
    }

    int step() override {
        if (n == 0) return ORC_OK;
        const float subDtF = prm.dt / float(prm.substeps);
        const T dt = T(subDtF);
        const T invDt = std::is_same<T, float>::value ? T(1.0f / subDtF) : T(1) / dt;
        const T mass = prm.particleMass, rho0 = prm.restDensity;
        const T gs = mass / rho0;
        const T r = prm.particleRadius;
        const long long N = (long long)n;
        const size_t ns = spheres.size(), nbx = boxes.size(), np = planes.size();
        for (int sub = 0; sub < prm.substeps; ++sub) {
            // integrate (src/pbf/integration.cu:6-32) + v_in copy (pbf_solver.cu:205-208).
#pragma omp parallel for schedule(static)
            for (long long i = 0; i < N; ++i) {
                Pos vv = v[i];
                const Pos p = x[i];
                vv.x = P::fma_(T(prm.gravity.x), dt, vv.x);
                vv.y = P::fma_(T(prm.gravity.y), dt, vv.y);
                vv.z = P::fma_(T(prm.gravity.z), dt, vv.z);
                v[i] = vv;
                xs[i] = Pos{P::fma_(vv.x, dt, p.x), P::fma_(vv.y, dt, p.y),
                            P::fma_(vv.z, dt, p.z), p.w};
                vin[i] = vv;
            }
            for (int it = 0; it < prm.solverIterations; ++it) {
                build_and_reorder();
                if (search()) return ORC_ERR_OVERFLOW;
#pragma omp parallel for schedule(static)
                for (long long i = 0; i < N; ++i)
                    lam[i] = st.lambda_one(xs.data(), nb.data() + size_t(i) * maxNb, cnt[i],
                                           maxNb, size_t(i), mass, rho0, T(prm.lambdaEpsilon));
                int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
                for (long long i = 0; i < N; ++i) {
                    T d[3];
                    st.delta_one(xs.data(), nb.data() + size_t(i) * maxNb, cnt[i], maxNb,
                                 lam.data(), size_t(i), gs, d);
                    Pos p = xs[i];
                    p.x = p.x + d[0]; p.y = p.y + d[1]; p.z = p.z + d[2];
                    if (!Collide<P>::solve(p, box, spheres.data(), ns, boxes.data(), nbx,
                                           planes.data(), np, r, kMaxCollisionPasses))
                        bad = 1;
                    tmp[i] = p;
                }
                xs.swap(tmp);
                if (bad) return ORC_ERR_NOT_CONVERGED;
            }
            if (prm.xsphViscosity != 0.0f || prm.vorticityStrength != 0.0f) {
                build_and_reorder();
                if (search()) return ORC_ERR_OVERFLOW;
            }
            // updateVelocityAndPosition (pbf_solver_kernels.cu:195-211).
#pragma omp parallel for schedule(static)
            for (long long i = 0; i < N; ++i) {
                v[i].x = (xs[i].x - x[i].x) * invDt;
                v[i].y = (xs[i].y - x[i].y) * invDt;
                v[i].z = (xs[i].z - x[i].z) * invDt;
                x[i] = xs[i];
            }
            if (prm.xsphViscosity != 0.0f) {
#pragma omp parallel for schedule(static)
                for (long long i = 0; i < N; ++i)
                    tmp[i] = st.xsph_one(xs.data(), v.data(), nb.data() + size_t(i) * maxNb,
                                         cnt[i], maxNb, size_t(i), T(prm.xsphViscosity));
                v.swap(tmp);
            }
            if (prm.vorticityStrength != 0.0f) {
#pragma omp parallel for schedule(static)
                for (long long i = 0; i < N; ++i)
                    om[i] = st.omega_one(xs.data(), v.data(), nb.data() + size_t(i) * maxNb,
                                         cnt[i], maxNb, size_t(i));
#pragma omp parallel for schedule(static)
                for (long long i = 0; i < N; ++i)
                    tmp[i] = st.confine_one(xs.data(), nb.data() + size_t(i) * maxNb, cnt[i],
                                            maxNb, om.data(), v.data(), size_t(i), dt,
                                            T(prm.vorticityStrength));
                v.swap(tmp);
            }
            // CollisionSystem::resolveVelocities (collision_system.cu:182-218).
#pragma omp parallel for schedule(static)
            for (long long i = 0; i < N; ++i)
                Collide<P>::resolve(x[i], vin[i], v[i], box, spheres.data(), ns, boxes.data(),
                                    nbx, planes.data(), np, r, T(prm.collisionRestitution),
                                    T(prm.collisionFriction));
        }
        return ORC_OK;
    }

    // scatterFloat4ByStableId (pbf_solver_kernels.cu:418-427).
    int copy_positions(orc_float4* out, size_t count) const override {
        if (count != n) return ORC_ERR_INVALID;
        for (size_t i = 0; i < n; ++i)
            out[id[i]] = orc_float4{float(x[i].x), float(x[i].y), float(x[i].z), float(x[i].w)};
        return ORC_OK;
    }
    int copy_velocities(orc_float4* out, size_t count) const override {
        if (count != n) return ORC_ERR_INVALID;
        for (size_t i = 0; i < n; ++i)
            out[id[i]] = orc_float4{float(v[i].x), float(v[i].y), float(v[i].z), float(v[i].w)};
        return ORC_OK;
    }
    int copy_working(orc_float4* pos, uint32_t* ids, int* counts, size_t count) const override {
        if (count != n) return ORC_ERR_INVALID;
        for (size_t i = 0; i < n; ++i) {
            if (pos) pos[i] = orc_float4{float(x[i].x), float(x[i].y), float(x[i].z), float(x[i].w)};
            if (ids) ids[i] = id[i];
            if (counts) counts[i] = cnt[i];
        }
        return ORC_OK;
    }
    // Density over the current lists (the reference computes rho inside
    // computeLambda, pbf_solver_kernels.cu:50-75, and never exposes it).
    int density_error(double* mean, double* mx) const override {
        double s = 0.0, m = 0.0;
        for (size_t i = 0; i < n; ++i) {
            double rho = double(prm.particleMass) * double(st.m.poly6(T(0)));
            const uint32_t* row = nb.data() + i * size_t(maxNb);
            const int c = std::min(cnt[i], maxNb);
            for (int k = 0; k < c; ++k) {
                const Pos pj = xs[row[k]];
                const T dx = xs[i].x - pj.x, dy = xs[i].y - pj.y, dz = xs[i].z - pj.z;
                rho += double(prm.particleMass) * double(st.m.poly6(st.m.dist2(dx, dy, dz)));
            }
            const double e = std::fabs(rho / double(prm.restDensity) - 1.0);
            s += e;
            m = std::max(m, e);
        }
        *mean = n ? s / double(n) : 0.0;
        *mx = m;
        return ORC_OK;
    }
};

}  // namespace

struct orc_solver {
    SolverBase* impl;
};

extern "C" {

int orc_grid_dims(orc_float3 mn, orc_float3 mx, float cell, int dims[3]) {
    return grid_dims(mn, mx, cell, dims);
}

uint32_t orc_cell_key(orc_float4 p, orc_float3 mn, float cell, const int dims[3]) {
    Grid g;
    g.gx = dims[0]; g.gy = dims[1]; g.gz = dims[2];
    g.minx = mn.x; g.miny = mn.y; g.minz = mn.z; g.cell = cell;
    int c[3];
    cell_of(g, p.x, p.y, p.z, c);
    return key_of(g, c);
}

void orc_grid_build(const orc_float4* pos, size_t n, orc_float3 mn, float cell,
                    const int dims[3], uint32_t* sortedKeys, uint32_t* sortedIdx,
                    int* cellStart, int* cellEnd) {
    Grid g;
    g.gx = dims[0]; g.gy = dims[1]; g.gz = dims[2];
    g.minx = mn.x; g.miny = mn.y; g.minz = mn.z; g.cell = cell;
    g.cells = size_t(dims[0]) * size_t(dims[1]) * size_t(dims[2]);
    std::vector<uint32_t> keys(n), scratch;
    for (size_t i = 0; i < n; ++i) {
        int c[3];
        cell_of(g, pos[i].x, pos[i].y, pos[i].z, c);
        keys[i] = key_of(g, c);
    }
    stable_sort_keys(keys.data(), n, g.cells, sortedKeys, sortedIdx, cellStart, cellEnd,
                     scratch);
}

int orc_find_neighbors(const orc_float4* sp, size_t n, const int* cs, const int* ce,
                       const int dims[3], orc_float3 mn, float cell, float h,
                       uint32_t* neighbors, int* counts, int maxNeighbors, size_t stride) {
    Grid g;
    g.gx = dims[0]; g.gy = dims[1]; g.gz = dims[2];
    g.minx = mn.x; g.miny = mn.y; g.minz = mn.z; g.cell = cell;
    F32 m;
    m.init(h);
    const double radius = std::ceil(double(h) / double(cell));
    const float h2 = h * h;
    const V4<float>* p = reinterpret_cast<const V4<float>*>(sp);
    int overflow = 0;
    for (size_t i = 0; i < n; ++i) {
        const int c = walk_neighbors(m, g, radius, p, i, cs, ce, h2, [&](int k, uint32_t j) {
            if (k < maxNeighbors) neighbors[size_t(k) * stride + i] = j;
        });
        counts[i] = c;
        if (c > maxNeighbors) overflow = 1;
    }
    return overflow;
}

// Slot-major list -> particle-major row helper for the single-stage mirrors.
static void gather_row(const uint32_t* nbrs, size_t stride, size_t i, int cnt, int cap,
                       std::vector<uint32_t>& row) {
    row.resize(size_t(std::max(0, std::min(cnt, cap))));
    for (size_t k = 0; k < row.size(); ++k) row[k] = nbrs[k * stride + i];
}

void orc_lambda(const orc_float4* pos, const uint32_t* nbrs, const int* counts, int cap,
                size_t n, size_t stride, float h, float mass, float rho0, float eps,
                float* lambda) {
    Stages<F32> st;
    st.m.init(h);
    std::vector<uint32_t> row;
    for (size_t i = 0; i < n; ++i) {
        gather_row(nbrs, stride, i, counts[i], cap, row);
        lambda[i] = st.lambda_one(reinterpret_cast<const V4<float>*>(pos), row.data(),
                                  counts[i], cap, i, mass, rho0, eps);
    }
}

void orc_delta(const orc_float4* pos, const uint32_t* nbrs, const int* counts, int cap,
               const float* lambda, size_t n, size_t stride, float h, float mass,
               float rho0, float k, int nexp, float dq, orc_float4* delta) {
    Stages<F32> st;
    st.m.init(h);
    st.sc.init(h, k, nexp, dq);
    const float gs = mass / rho0;
    std::vector<uint32_t> row;
    for (size_t i = 0; i < n; ++i) {
        gather_row(nbrs, stride, i, counts[i], cap, row);
        float d[3];
        st.delta_one(reinterpret_cast<const V4<float>*>(pos), row.data(), counts[i], cap,
                     lambda, i, gs, d);
        delta[i] = orc_float4{d[0], d[1], d[2], 0.0f};
    }
}

float orc_scorr(float d2, float h, float k, int nexp, float dq) {
    Scorr32 s;
    s.init(h, k, nexp, dq);
    return s(d2);
}

float orc_poly6(float d2, float h) {
    F32 m;
    m.init(h);
    return m.poly6(d2);
}

void orc_spiky(float dx, float dy, float dz, float h, float out[3]) {
    F32 m;
    m.init(h);
    m.spiky(dx, dy, dz, F32::dist2(dx, dy, dz), out);
}

void orc_xsph(const orc_float4* pos, const uint32_t* nbrs, const int* counts, int cap,
              const orc_float4* vin, orc_float4* vout, size_t n, size_t stride, float h,
              float c) {
    Stages<F32> st;
    st.m.init(h);
    std::vector<uint32_t> row;
    for (size_t i = 0; i < n; ++i) {
        if (c == 0.0f) { vout[i] = vin[i]; continue; }
        gather_row(nbrs, stride, i, counts[i], cap, row);
        const V4<float> r = st.xsph_one(reinterpret_cast<const V4<float>*>(pos),
                                        reinterpret_cast<const V4<float>*>(vin), row.data(),
                                        counts[i], cap, i, c);
        vout[i] = orc_float4{r.x, r.y, r.z, r.w};
    }
}

void orc_vorticity(const orc_float4* pos, const orc_float4* vel, const uint32_t* nbrs,
                   const int* counts, int cap, size_t n, size_t stride, float h,
                   orc_float4* omega) {
    Stages<F32> st;
    st.m.init(h);
    std::vector<uint32_t> row;
    for (size_t i = 0; i < n; ++i) {
        gather_row(nbrs, stride, i, counts[i], cap, row);
        const V4<float> r = st.omega_one(reinterpret_cast<const V4<float>*>(pos),
                                         reinterpret_cast<const V4<float>*>(vel), row.data(),
                                         counts[i], cap, i);
        omega[i] = orc_float4{r.x, r.y, r.z, r.w};
    }
}

void orc_confinement(const orc_float4* pos, const uint32_t* nbrs, const int* counts, int cap,
                     const orc_float4* omega, const orc_float4* vin, orc_float4* vout,
                     size_t n, size_t stride, float h, float dt, float eps) {
    Stages<F32> st;
    st.m.init(h);
    std::vector<uint32_t> row;
    for (size_t i = 0; i < n; ++i) {
        gather_row(nbrs, stride, i, counts[i], cap, row);
        const V4<float> r = st.confine_one(reinterpret_cast<const V4<float>*>(pos), row.data(),
                                           counts[i], cap,
                                           reinterpret_cast<const V4<float>*>(omega),
                                           reinterpret_cast<const V4<float>*>(vin), i, dt, eps);
        vout[i] = orc_float4{r.x, r.y, r.z, r.w};
    }
}

int orc_solve_container(orc_float4* pos, size_t n, orc_container c, float r) {
    int mark = 0;
    for (size_t i = 0; i < n; ++i)
        mark |= Collide<F32>::container(*reinterpret_cast<V4<float>*>(&pos[i]), c, r);
    return mark;
}
int orc_solve_spheres(orc_float4* pos, size_t n, const orc_sphere* s, size_t ns, float r) {
    int mark = 0;
    for (size_t i = 0; i < n; ++i)
        mark |= Collide<F32>::spheres(*reinterpret_cast<V4<float>*>(&pos[i]), s, ns, r);
    return mark;
}
int orc_solve_boxes(orc_float4* pos, size_t n, const orc_box* b, size_t nb, float r) {
    int mark = 0;
    for (size_t i = 0; i < n; ++i)
        mark |= Collide<F32>::boxes(*reinterpret_cast<V4<float>*>(&pos[i]), b, nb, r);
    return mark;
}
int orc_solve_planes(orc_float4* pos, size_t n, const orc_plane* p, size_t np, float r) {
    int mark = 0;
    for (size_t i = 0; i < n; ++i)
        mark |= Collide<F32>::planes(*reinterpret_cast<V4<float>*>(&pos[i]), p, np, r);
    return mark;
}
int orc_collide(orc_float4* pos, size_t n, orc_container c, const orc_sphere* s, size_t ns,
                const orc_box* b, size_t nb, const orc_plane* p, size_t np, float r,
                int maxPasses) {
    int bad = 0;
    for (size_t i = 0; i < n; ++i)
        if (!Collide<F32>::solve(*reinterpret_cast<V4<float>*>(&pos[i]), c, s, ns, b, nb, p, np,
                                 r, maxPasses))
            bad = 1;
    return bad ? ORC_ERR_NOT_CONVERGED : ORC_OK;
}
void orc_resolve_velocities(const orc_float4* pos, const orc_float4* vin, orc_float4* vel,
                            size_t n, orc_container c, const orc_sphere* s, size_t ns,
                            const orc_box* b, size_t nb, const orc_plane* p, size_t np,
                            float r, float restitution, float friction) {
    for (size_t i = 0; i < n; ++i)
        Collide<F32>::resolve(*reinterpret_cast<const V4<float>*>(&pos[i]),
                              *reinterpret_cast<const V4<float>*>(&vin[i]),
                              *reinterpret_cast<V4<float>*>(&vel[i]), c, s, ns, b, nb, p, np,
                              r, restitution, friction);
}

orc_solver* orc_solver_create(int precision) {
    orc_solver* s = new (std::nothrow) orc_solver;
    if (!s) return nullptr;
    if (precision == 64) s->impl = new Solver<F64>();
    else s->impl = new Solver<F32>();
    return s;
}
void orc_solver_destroy(orc_solver* s) {
    if (!s) return;
    delete s->impl;
    delete s;
}
void orc_solver_set_threads(orc_solver* s, int t) {
    s->impl->threads = t;
    set_threads(t);
}
int orc_solver_initialize(orc_solver* s, size_t maxParticles, orc_float3 mn, orc_float3 mx,
                          const orc_params* p, int maxNeighbors) {
    return s->impl->initialize(maxParticles, mn, mx, *p, maxNeighbors);
}
int orc_solver_set_particles(orc_solver* s, const orc_float4* pos, const orc_float4* vel,
                             size_t n) {
    return s->impl->set_particles(pos, vel, n);
}
int orc_solver_set_colliders(orc_solver* s, const orc_sphere* sp, size_t ns, const orc_box* bx,
                             size_t nb, const orc_plane* pl, size_t np) {
    s->impl->set_colliders(sp, ns, bx, nb, pl, np);
    return ORC_OK;
}
int orc_solver_step(orc_solver* s) {
    set_threads(s->impl->threads);
    return s->impl->step();
}
int orc_solver_copy_positions(const orc_solver* s, orc_float4* out, size_t n) {
    return s->impl->copy_positions(out, n);
}
int orc_solver_copy_velocities(const orc_solver* s, orc_float4* out, size_t n) {
    return s->impl->copy_velocities(out, n);
}
int orc_solver_copy_working(const orc_solver* s, orc_float4* pos, uint32_t* ids, int* counts,
                            size_t n) {
    return s->impl->copy_working(pos, ids, counts, n);
}
int orc_solver_density_error(const orc_solver* s, double* mean, double* mx) {
    return s->impl->density_error(mean, mx);
}

// The density that computeLambda forms (src/pbf/pbf_solver_kernels.cu:50-75),
// in double and over all pairs within h found through cells of size h: a
// yardstick for comparing two solvers' final states, independent of either
// solver's own lists.
int orc_density_stats(const orc_float4* pos, size_t n, orc_float3 mn, orc_float3 mx, float h,
                      float mass, float rho0, double* meanErr, double* maxErr,
                      double* fracAbove10) {
    int d[3];
    const int st = grid_dims(mn, mx, h, d);
    if (st != ORC_OK) return st;
    const size_t cells = size_t(d[0]) * size_t(d[1]) * size_t(d[2]);
    std::vector<uint32_t> key(n), start(cells + 1, 0), order(n);
    const double inv = 1.0 / double(h);
    auto cell = [&](double p, float lo, int dim) {
        const double c = std::floor((p - double(lo)) * inv);
        return c < 0.0 ? 0 : (c > double(dim - 1) ? dim - 1 : int(c));
    };
    for (size_t i = 0; i < n; ++i) {
        const int cx = cell(pos[i].x, mn.x, d[0]), cy = cell(pos[i].y, mn.y, d[1]),
                  cz = cell(pos[i].z, mn.z, d[2]);
        key[i] = uint32_t(cx + size_t(d[0]) * (cy + size_t(d[1]) * cz));
        ++start[key[i] + 1];
    }
    for (size_t c = 0; c < cells; ++c) start[c + 1] += start[c];
    {
        std::vector<uint32_t> fill(start.begin(), start.end() - 1);
        for (size_t i = 0; i < n; ++i) order[fill[key[i]]++] = uint32_t(i);
    }
    const double hh = double(h), h2 = hh * hh;
    const double norm = 315.0 / (64.0 * kPiD * hh * hh * hh * hh * hh * hh * hh * hh * hh);
    double sum = 0.0, mxe = 0.0;
    long long above = 0;
#pragma omp parallel for schedule(dynamic, 4096) reduction(+ : sum, above) reduction(max : mxe)
    for (long long ii = 0; ii < (long long)n; ++ii) {
        const size_t i = size_t(ii);
        const int cx = cell(pos[i].x, mn.x, d[0]), cy = cell(pos[i].y, mn.y, d[1]),
                  cz = cell(pos[i].z, mn.z, d[2]);
        double w = 0.0;
        for (int z = std::max(0, cz - 1); z <= std::min(d[2] - 1, cz + 1); ++z)
            for (int y = std::max(0, cy - 1); y <= std::min(d[1] - 1, cy + 1); ++y)
                for (int x = std::max(0, cx - 1); x <= std::min(d[0] - 1, cx + 1); ++x) {
                    const size_t c = size_t(x) + size_t(d[0]) * (size_t(y) + size_t(d[1]) * z);
                    for (uint32_t k = start[c]; k < start[c + 1]; ++k) {
                        const orc_float4 q = pos[order[k]];
                        const double dx = double(pos[i].x) - q.x, dy = double(pos[i].y) - q.y,
                                     dz = double(pos[i].z) - q.z;
                        const double r2 = dx * dx + dy * dy + dz * dz;
                        if (r2 < h2) {
                            const double t = h2 - r2;
                            w += norm * t * t * t;
                        }
                    }
                }
        const double e = std::fabs(double(mass) * w / double(rho0) - 1.0);
        sum += e;
        mxe = std::max(mxe, e);
        above += e > 0.1 ? 1 : 0;
    }
    *meanErr = n ? sum / double(n) : 0.0;
    *maxErr = mxe;
    if (fracAbove10) *fracAbove10 = n ? double(above) / double(n) : 0.0;
    return ORC_OK;
}

}  // extern "C"
