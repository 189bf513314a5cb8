// pbf_kernels.cu -- per-particle kernels of the PBF step for sm_103a.
//
// Hot path per constraint iteration (reference: src/pbf/pbf_solver.cu:210-258):
//   k_predict        integrate + v_in copy + first cell keys      (integration.cu:6-32)
//   [sort]           stable radix sort of (key, index)            (spatial_grid.cu:188-196)
//   k_gather_first   reorder predicted positions, compose the permutation and
//                    refresh first[] (lower bound of every cell key; the row
//                    walk's form of cellStart/cellEnd, spatial_grid.cu:123-137)
//   k_search<true>   neighbour walk + lambda in one pass           (neighbors.cu:3-91,
//                                                                  pbf_solver_kernels.cu:26-105)
//   k_delta_apply    delta p + apply + collision projection + next keys
//                                                                 (pbf_solver_kernels.cu:108-193,
//                                                                  collision_system.cu:133-172)
// After the last iteration (pbf_solver.cu:260-323), after the final rebuild:
//   k_finalize       gather x, v_in, ids by the composite permutation + velocity update
//   k_search_xsph    rebuilt lists for the velocity terms + XSPH over them
//                    (k_search<false> when XSPH is off)
//   k_vorticity, k_confine   (pbf_solver_kernels.cu:268-385), collision velocity
//                    response fused into the last velocity kernel
//   k_xsph           XSPH alone (stage API)
//
// Every floating-point operation uses the explicit-rounding helpers of
// pbf_math.cuh so the host oracle reproduces the step bit for bit.
#include "pbf_kernels.cuh"

#include "pbf_common.h"

#include <math_constants.h>

#include <algorithm>

namespace pbf {

void launch_error_check(cudaError_t e) { cuda_check(e); }

// Register cap of a neighbour-loop kernel bound by the latency of its
// dependent gathers (list index, then the neighbour's data): fewer registers
// a thread, more warps in flight (k_delta_apply: 58 -> 48 registers, no
// spills, 6 % faster at 1M particles).
#define PBF_GATHER_REGS(r) __maxnreg__(r)


namespace {

__device__ __forceinline__ bool fatal(const unsigned* status) {
    return status != nullptr && (__ldcg(status) & kStatusFatalMask) != 0u;
}

// The scene of particle slot i in a batched solver.
__device__ __forceinline__ const SceneConst& scene_of(const StepConst& c, int i) {
    return c.scenes[__ldg(&c.sid[i])];
}

// First entry and entry stride of particle i's neighbour list.
__device__ __forceinline__ size_t nb_first(const StepConst& c, int i) {
    return c.nb_off ? static_cast<size_t>(__ldg(&c.nb_off[i])) : static_cast<size_t>(i);
}
__device__ __forceinline__ size_t nb_step(const StepConst& c) {
    return c.nb_off ? size_t(1) : c.stride;
}

// Grid and first global cell key of slot i: the scene's (B) or c.g.
template <bool B>
__device__ __forceinline__ void grid_of(const StepConst& c, int i, GridConst& g, uint32_t& base) {
    if constexpr (B) {
        const SceneConst& s = scene_of(c, i);
        g = s.g;
        base = s.cell_base;
    } else {
        g = c.g;
        base = 0u;
    }
}

// Colliders with the container of slot i's scene (B) or c.col.
template <bool B>
__device__ __forceinline__ Colliders colliders_of(const StepConst& c, int i) {
    Colliders col = c.col;
    if constexpr (B) {
        const SceneConst& s = scene_of(c, i);
        col.cminx = s.cminx;
        col.cminy = s.cminy;
        col.cminz = s.cminz;
        col.cmaxx = s.cmaxx;
        col.cmaxy = s.cmaxy;
        col.cmaxz = s.cmaxz;
    }
    return col;
}

// ---------------------------------------------------------------------------
// integrate + collision input velocity + keys of the first rebuild
// ---------------------------------------------------------------------------
template <bool B>
__global__ void __launch_bounds__(kBlock)
k_predict(const float4* __restrict__ x, const float4* __restrict__ v, float4* __restrict__ xs,
          float4* __restrict__ vin, uint32_t* __restrict__ keys, int n, StepConst c,
          const unsigned* __restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || fatal(status)) return;
    float4 vv = v[i];
    const float4 p = x[i];
    vv.x = ffma(c.gravx, c.dt, vv.x);
    vv.y = ffma(c.gravy, c.dt, vv.y);
    vv.z = ffma(c.gravz, c.dt, vv.z);
    float4 q;
    q.x = ffma(vv.x, c.dt, p.x);
    q.y = ffma(vv.y, c.dt, p.y);
    q.z = ffma(vv.z, c.dt, p.z);
    q.w = p.w;
    xs[i] = q;
    vin[i] = vv;
    GridConst g;
    uint32_t base;
    grid_of<B>(c, i, g, base);
    keys[i] = base + key_of(g, q);
}

__global__ void __launch_bounds__(kBlock)
k_cell_ranges(const uint32_t* __restrict__ skeys, int* __restrict__ cs, int* __restrict__ ce,
              int n, const unsigned* __restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || fatal(status)) return;
    const uint32_t key = skeys[i];
    if (i == 0 || skeys[i - 1] != key) cs[key] = i;
    if (i == n - 1 || skeys[i + 1] != key) ce[key] = i + 1;
}

// first[k] = lower_bound(sorted keys, k) for k in [0, cells]: the particles of
// cells [a, b] are exactly [first[a], first[b + 1]).  Equivalent to the
// reference's cellStart/cellEnd pair (spatial_grid.cu:123-137) with empty
// cells resolved to the next occupied one, so a run of cells along x is one
// contiguous index range.
__global__ void __launch_bounds__(kBlock)
k_gather_xs(const uint32_t* __restrict__ perm, const float4* __restrict__ xs_in,
            float4* __restrict__ xs_out, const uint32_t* __restrict__ org_in,
            uint32_t* __restrict__ org_out, float* __restrict__ sx, float* __restrict__ sy,
            float* __restrict__ sz, int n, const unsigned* __restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || fatal(status)) return;
    const uint32_t p = perm[i];
    const float4 q = xs_in[p];
    xs_out[i] = q;
    sx[i] = q.x;
    sy[i] = q.y;
    sz[i] = q.z;
    if (org_out) org_out[i] = org_in ? org_in[p] : p;
}

// Lower bound of key k in skeys[0, n), searched outward from a guess: the
// table of the previous rebuild, whose entries move little between
// iterations.  Any guess gives the same answer; a good one needs one or two
// loads instead of log2(n).
__device__ __forceinline__ int lower_bound_from(const uint32_t* __restrict__ skeys, int n,
                                                uint32_t k, int guess) {
    int g = min(max(guess, 0), n);
    int lo, hi;  // answer in [lo, hi]
    if (g > 0 && __ldg(&skeys[g - 1]) >= k) {
        // Answer < g: gallop down until skeys[lo - 1] < k (or lo == 0).
        hi = g - 1;
        int step = 1;
        lo = g - 1;
        while (lo > 0 && __ldg(&skeys[lo - 1]) >= k) {
            hi = lo - 1;
            lo = lo > step ? lo - step : 0;
            step = step < (1 << 29) ? step << 1 : step;
        }
    } else if (g < n && __ldg(&skeys[g]) < k) {
        // Answer > g: gallop up until skeys[hi] >= k (or hi == n).
        lo = g + 1;
        int step = 1;
        hi = min(n, g + 1);
        while (hi < n && __ldg(&skeys[hi]) < k) {
            lo = hi + 1;
            hi = n - hi > step ? hi + step : n;
            step = step < (1 << 29) ? step << 1 : step;
        }
    } else {
        return g;
    }
    // Invariant: skeys[lo - 1] < k (or lo == 0) and skeys[hi] >= k (or hi == n).
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&skeys[mid]) < k) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// One launch after each sort: thread i reorders particle i (as k_gather_xs)
// and refreshes first[i] for i <= cells, in place.
__global__ void __launch_bounds__(kBlock)
k_gather_first(const uint32_t* __restrict__ perm, const float4* __restrict__ xs_in,
               float4* __restrict__ xs_out, const uint32_t* __restrict__ org_in,
               uint32_t* __restrict__ org_out, float* __restrict__ sx, float* __restrict__ sy,
               float* __restrict__ sz, int n, const uint32_t* __restrict__ skeys, uint32_t cells,
               int* __restrict__ first, const unsigned* __restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (fatal(status)) return;
    if (i < n) {
        const uint32_t p = perm[i];
        const float4 q = xs_in[p];
        xs_out[i] = q;
        sx[i] = q.x;
        sy[i] = q.y;
        sz[i] = q.z;
        org_out[i] = org_in ? org_in[p] : p;
    }
    if (static_cast<uint32_t>(i) <= cells) {
        const uint32_t k = static_cast<uint32_t>(i);
        first[k] = lower_bound_from(skeys, n, k, first[k]);
    }
}

// ---------------------------------------------------------------------------
// Neighbour walk.  Order of the list = z -> y -> x over the clamped cells,
// ascending sorted index inside a cell, self skipped, accept d2 <= h2
// (src/pbf/neighbors.cu:52-86).  With LAMBDA the constraint terms of
// computeLambda are accumulated in that same list order.
// ---------------------------------------------------------------------------
struct LambdaAcc {
    float wsum, s2, gx, gy, gz;
};

__device__ __forceinline__ void lambda_add(const KernelConst& k, LambdaAcc& a, float dx, float dy,
                                           float dz, float d2) {
    a.wsum = fadd(a.wsum, poly6(k, d2));
    float gx, gy, gz;
    spiky(k, dx, dy, dz, d2, gx, gy, gz);
    a.s2 = ffma(gz, gz, ffma(gy, gy, ffma(gx, gx, a.s2)));
    a.gx = fadd(a.gx, gx);
    a.gy = fadd(a.gy, gy);
    a.gz = fadd(a.gz, gz);
}

// Two neighbours' terms, lane 0 first: the same sums as two lambda_add calls.
__device__ __forceinline__ void lambda_add2(const KernelConst& k, LambdaAcc& a, f32x2 dx, f32x2 dy,
                                            f32x2 dz, f32x2 d2) {
    const f32x2 s = spiky_scale2(k, d2);
    float w0, w1, x0, x1, y0, y1, z0, z1;
    unpack2(poly6_2(k, d2), w0, w1);
    unpack2(mul2(dx, s), x0, x1);
    unpack2(mul2(dy, s), y0, y1);
    unpack2(mul2(dz, s), z0, z1);
    a.wsum = fadd(fadd(a.wsum, w0), w1);
    a.s2 = ffma(z0, z0, ffma(y0, y0, ffma(x0, x0, a.s2)));
    a.s2 = ffma(z1, z1, ffma(y1, y1, ffma(x1, x1, a.s2)));
    a.gx = fadd(fadd(a.gx, x0), x1);
    a.gy = fadd(fadd(a.gy, y0), y1);
    a.gz = fadd(fadd(a.gz, z0), z1);
}

__device__ __forceinline__ float lambda_finish(float mass, float rho0, float gs2, float eps,
                                               const LambdaAcc& a) {
    const float rho = fmul(mass, a.wsum);
    const float g2 = dist2(a.gx, a.gy, a.gz);
    const float denom = ffma(gs2, fadd(a.s2, g2), eps);
    const float C = fsub(fdiv(rho, rho0), 1.0f);
    return fdiv(-C, denom);
}
__device__ __forceinline__ float lambda_finish(const StepConst& c, const LambdaAcc& a) {
    return lambda_finish(c.mass, c.rho0, c.gs2, c.lambda_eps, a);
}

// Squared distances from coordinate p to the slabs of the cells below and
// above cell k on one axis (cell k spans [lo + k cell, lo + (k + 1) cell);
// the clamped end cells extend to infinity, which changes neither distance),
// each first reduced by eps.  Margin arithmetic only: it decides which cells
// the walk reads, never a neighbour.
__device__ __forceinline__ void slab_dist2(float p, float lo, float cell, int k, float eps,
                                           float& below, float& above) {
    const float b0 = fmaf(static_cast<float>(k), cell, lo);
    const float b1 = fmaf(static_cast<float>(k + 1), cell, lo);
    const float d0 = fmaxf(p - b0 - eps, 0.0f);
    const float d1 = fmaxf(b1 - p - eps, 0.0f);
    below = d0 * d0;
    above = d1 * d1;
}

// The neighbour walk of particle i (position pi): writes the list slot-major
// at out[slot * stride] (at most cap entries) and returns the full count.
// STORE = false counts the hits without writing the list.
// The stencil rows of particle i, as the walks visit them: z0..z1 x y0..y1
// (clamped to the grid), and range(z, y) gives row (z, y)'s candidate index
// range [s, e): its cells x0..x1 are consecutive keys.  Keys fit in 32 bits
// (cells < 2^32 is checked at initialisation), so the reference's 64-bit key
// arithmetic truncates to the same values.
// Cell pruning (radius 1): a stencil cell whose box lies farther than h
// from the particle holds no neighbour, so range() returns false for the
// rows (y, z) that far and leaves out the end cells of a row that far.  Per
// axis, eps = 2^-14 (|p| + |min| + cell) covers the FP32 rounding of every
// cell index (floor((p - min) / cell)) and of the candidates' differences,
// and the bound h2 (1 + 2^-10) the rounding of d2: only certain misses are
// left out, so the list is entry for entry the unpruned walk's.
template <bool B>
struct StencilRows {
    GridConst g;
    uint32_t base, gx, gxy;
    int cx, cy, cz, x0, x1, y0, y1, z0, z1;
    bool prune;
    float xb2, xa2, yb2, ya2, zb2, za2, lim2;
    __device__ __forceinline__ StencilRows(const StepConst& c, int i, float4 pi) {
        grid_of<B>(c, i, g, base);
        cell_of(g, pi.x, pi.y, pi.z, cx, cy, cz);
        const int R = g.radius;
        x0 = max(0, cx - R);
        x1 = min(g.gx - 1, cx + R);
        y0 = max(0, cy - R);
        y1 = min(g.gy - 1, cy + R);
        z0 = max(0, cz - R);
        z1 = min(g.gz - 1, cz + R);
        gx = static_cast<uint32_t>(g.gx);
        gxy = gx * static_cast<uint32_t>(g.gy);
        prune = c.prune_cells && R == 1;
        xb2 = xa2 = yb2 = ya2 = zb2 = za2 = lim2 = 0.0f;
        if (prune) {
            const float eps = 6.103515625e-05f *
                              (fabsf(pi.x) + fabsf(pi.y) + fabsf(pi.z) + fabsf(g.minx) +
                               fabsf(g.miny) + fabsf(g.minz) + g.cell);
            slab_dist2(pi.x, g.minx, g.cell, cx, eps, xb2, xa2);
            slab_dist2(pi.y, g.miny, g.cell, cy, eps, yb2, ya2);
            slab_dist2(pi.z, g.minz, g.cell, cz, eps, zb2, za2);
            lim2 = c.k.h2 * 1.0009765625f;
        }
    }
    __device__ __forceinline__ bool range(const int* __restrict__ first, int z, int y, int& s,
                                          int& e) const {
        int xa = x0, xb = x1;
        if (prune) {
            const float dyz = (z < cz ? zb2 : (z > cz ? za2 : 0.0f)) +
                              (y < cy ? yb2 : (y > cy ? ya2 : 0.0f));
            if (dyz > lim2) return false;
            if (xa < cx && dyz + xb2 > lim2) xa = cx;
            if (xb > cx && dyz + xa2 > lim2) xb = cx;
        }
        const uint32_t row =
            base + static_cast<uint32_t>(y) * gx + static_cast<uint32_t>(z) * gxy;
        s = __ldg(&first[row + static_cast<uint32_t>(xa)]);
        e = __ldg(&first[row + static_cast<uint32_t>(xb) + 1u]);
        return true;
    }
};

// Bits of a 32-candidate chunk from j0 that belong to the row range [s, e),
// less the particle i itself.
__device__ __forceinline__ uint32_t chunk_valid(int j0, int s, int e, int i) {
    const int left = e - j0;
    uint32_t valid = left >= 32 ? 0xffffffffu : ((1u << left) - 1u);
    if (j0 < s) valid &= ~((1u << (s - j0)) - 1u);
    const int self = i - j0;
    if (self >= 0 && self < 32) valid &= ~(1u << self);
    return valid;
}

// The neighbour walk of particle i (position pi): writes the list slot-major
// at out[slot * stride] (at most cap entries) and returns the full count.
// STORE = false counts the hits without writing the list.
template <bool B, bool STORE = true>
__device__ __forceinline__ int walk(const StepConst& c, int i, float4 pi,
                                    const float* __restrict__ sx, const float* __restrict__ sy,
                                    const float* __restrict__ sz, const int* __restrict__ first,
                                    uint32_t* __restrict__ out, int cap) {
    const StencilRows<B> rows(c, i, pi);
    // The hit test d2 <= h2 as a sign bit: for finite d2 it holds exactly
    // when d2 - h2u < 0, h2u being the float just above h2 (the difference
    // of two distinct floats is never zero, and +inf or NaN, the canonical
    // NaN of the FP32 units, give a clear sign bit: no hit, as d2 <= h2).
    const f32x2 h2u = splat2(__uint_as_float(__float_as_uint(c.k.h2) + 1u));
    const size_t stride = nb_step(c);
    const f32x2 px = splat2(pi.x), py = splat2(pi.y), pz = splat2(pi.z);
    int count = 0;
    // 16 candidates from j (a multiple of 4): the x, y, z arrays are read
    // four floats at a time and tested two at a time with FP32x2
    // arithmetic; each test's sign bit is shifted into acc (the first
    // candidate ends up highest).
    auto test16 = [&](int j, uint32_t& acc) {
#pragma unroll
        for (int q = 0; q < 16; q += 4) {
            const float4 X = __ldg(reinterpret_cast<const float4*>(sx + j + q));
            const float4 Y = __ldg(reinterpret_cast<const float4*>(sy + j + q));
            const float4 Z = __ldg(reinterpret_cast<const float4*>(sz + j + q));
            const f32x2 da = dist2x2(sub2(px, pack2(X.x, X.y)), sub2(py, pack2(Y.x, Y.y)),
                                     sub2(pz, pack2(Z.x, Z.y)));
            const f32x2 db = dist2x2(sub2(px, pack2(X.z, X.w)), sub2(py, pack2(Y.z, Y.w)),
                                     sub2(pz, pack2(Z.z, Z.w)));
            float a0, a1, b0, b1;
            unpack2(sub2(da, h2u), a0, a1);
            unpack2(sub2(db, h2u), b0, b1);
            acc = __funnelshift_l(__float_as_uint(a0), acc, 1);
            acc = __funnelshift_l(__float_as_uint(a1), acc, 1);
            acc = __funnelshift_l(__float_as_uint(b0), acc, 1);
            acc = __funnelshift_l(__float_as_uint(b1), acc, 1);
        }
    };
    // Rows z -> y, each one index range walked in ascending order -- exactly
    // the reference's z -> y -> x cell walk (neighbors.cu:52-86).  Each range
    // is tested in 32-candidate chunks from a multiple of 4 (the second half
    // of a chunk only if the range reaches it); candidates outside [s, e) and
    // the particle itself are masked off, and the hits are then appended in
    // ascending order.  The component arrays are padded (soa_stride_for), so
    // a chunk may read past the last particle.
    for (int z = rows.z0; z <= rows.z1; ++z)
        for (int y = rows.y0; y <= rows.y1; ++y) {
            int s, e;
            if (!rows.range(first, z, y, s, e)) continue;
            for (int j0 = s & ~3; j0 < e; j0 += 32) {
                uint32_t acc = 0u;
                test16(j0, acc);
                if (e - j0 > 16) test16(j0 + 16, acc);
                else acc <<= 16;
                uint32_t mask = __brev(acc) & chunk_valid(j0, s, e, i);
                if constexpr (STORE) {
                    while (mask) {
                        const int b = __ffs(mask) - 1;
                        mask &= mask - 1u;
                        if (count < cap)
                            out[static_cast<size_t>(count) * stride] =
                                static_cast<uint32_t>(j0 + b);
                        ++count;
                    }
                } else {
                    count += __popc(mask);
                }
            }
        }
    return count;
}

// Second pass over the list just written: the constraint terms run once per
// neighbour instead of once per candidate in which any lane of the warp hit.
// Same order as the list, so the same sums.  Neighbours are taken two at a
// time with FP32x2 arithmetic; the sums stay in list order.  The next pair's
// indices are loaded before this pair is gathered.
template <bool B>
__device__ __forceinline__ float lambda_of_list(const StepConst& c, int i, float4 pi,
                                                const float4* __restrict__ xs,
                                                const uint32_t* __restrict__ out, size_t stride,
                                                int count) {
    const f32x2 px = pack2(pi.x, pi.x), py = pack2(pi.y, pi.y), pz = pack2(pi.z, pi.z);
    LambdaAcc acc{c.k.c_poly6, 0.0f, 0.0f, 0.0f, 0.0f};
    int k = 0;
    uint32_t na = 0u, nb2 = 0u;
    if (count >= 2) {
        na = out[0];
        nb2 = out[stride];
    }
    for (; k + 2 <= count; k += 2) {
        const uint32_t ja = na, jb = nb2;
        if (k + 4 <= count) {
            na = out[static_cast<size_t>(k + 2) * stride];
            nb2 = out[static_cast<size_t>(k + 3) * stride];
        }
        const float4 a = __ldg(&xs[ja]);
        const float4 b = __ldg(&xs[jb]);
        const f32x2 dx = sub2(px, pack2(a.x, b.x));
        const f32x2 dy = sub2(py, pack2(a.y, b.y));
        const f32x2 dz = sub2(pz, pack2(a.z, b.z));
        lambda_add2(c.k, acc, dx, dy, dz, dist2x2(dx, dy, dz));
    }
    if (k < count) {
        const float4 pj = __ldg(&xs[out[static_cast<size_t>(k) * stride]]);
        const float dx = fsub(pi.x, pj.x), dy = fsub(pi.y, pj.y), dz = fsub(pi.z, pj.z);
        lambda_add(c.k, acc, dx, dy, dz, dist2(dx, dy, dz));
    }
    if constexpr (B) {
        const SceneConst& sc = scene_of(c, i);
        return lambda_finish(sc.mass, sc.rho0, sc.gs2, c.lambda_eps, acc);
    } else {
        return lambda_finish(c, acc);
    }
}

// What k_search does once particle i's list (count entries) is written.
template <bool LAMBDA, bool B>
__device__ __forceinline__ void search_tail(const StepConst& c, int i, float4 pi,
                                            const float4* __restrict__ xs,
                                            const uint32_t* __restrict__ out, int count,
                                            int* __restrict__ cnt, float* __restrict__ lam,
                                            unsigned* __restrict__ status) {
    cnt[i] = count;
    if (count > c.max_nb) atomicOr(status, kStatusNeighborOverflow);
    if (LAMBDA)
        lam[i] = count > c.max_nb ? CUDART_NAN_F
                                  : lambda_of_list<B>(c, i, pi, xs, out, nb_step(c), count);
}

template <bool LAMBDA, bool B>
__global__ void __launch_bounds__(kMaxTunedBlock)
k_search(const float4* __restrict__ xs, const float* __restrict__ sx,
         const float* __restrict__ sy, const float* __restrict__ sz, const int* __restrict__ first,
         StepConst c, int n, uint32_t* __restrict__ nbr, int* __restrict__ cnt,
         float* __restrict__ lam, unsigned* __restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || fatal(status)) return;
    const float4 pi = xs[i];
    uint32_t* __restrict__ out = nbr + nb_first(c, i);
    const int count = walk<B>(c, i, pi, sx, sy, sz, first, out, c.max_nb);
    search_tail<LAMBDA, B>(c, i, pi, xs, out, count, cnt, lam, status);
}

// The walk on a group of L lanes (gmask; lane `sub`), for scenes too small
// to fill the GPU with one thread per particle.  The lanes visit the same
// rows and chunks together; lane q tests candidates [qW, (q + 1)W) of each
// 32-candidate chunk (W = 32 / L), the group ORs the hit masks, and each
// lane writes its own hits at their places in the list (the hits of lower
// lanes first).  The list is walk()'s, entry for entry; the count is
// returned on every lane.
template <bool B, int L>
__device__ __forceinline__ int walk_chunks(const StepConst& c, int i, int sub, unsigned gmask,
                                           float4 pi, const float* __restrict__ sx,
                                           const float* __restrict__ sy,
                                           const float* __restrict__ sz,
                                           const int* __restrict__ first,
                                           uint32_t* __restrict__ out) {
    constexpr int W = 32 / L;
    const StencilRows<B> rows(c, i, pi);
    const f32x2 h2u = splat2(__uint_as_float(__float_as_uint(c.k.h2) + 1u));
    const size_t stride = nb_step(c);
    const int cap = c.max_nb;
    const f32x2 px = splat2(pi.x), py = splat2(pi.y), pz = splat2(pi.z);
    const uint32_t lower = (1u << (sub * W)) - 1u;  // bits of lower lanes' candidates
    const uint32_t own = W == 32 ? 0xffffffffu : (((1u << W) - 1u) << (sub * W));
    int count = 0;
    for (int z = rows.z0; z <= rows.z1; ++z)
        for (int y = rows.y0; y <= rows.y1; ++y) {
            int s, e;
            if (!rows.range(first, z, y, s, e)) continue;
            for (int j0 = s & ~3; j0 < e; j0 += 32) {
                const int jb = j0 + sub * W;
                uint32_t acc = 0u;
                if (jb < e) {
#pragma unroll
                    for (int q = 0; q < W; q += 4) {
                        const float4 X = __ldg(reinterpret_cast<const float4*>(sx + jb + q));
                        const float4 Y = __ldg(reinterpret_cast<const float4*>(sy + jb + q));
                        const float4 Z = __ldg(reinterpret_cast<const float4*>(sz + jb + q));
                        const f32x2 da = dist2x2(sub2(px, pack2(X.x, X.y)),
                                                 sub2(py, pack2(Y.x, Y.y)),
                                                 sub2(pz, pack2(Z.x, Z.y)));
                        const f32x2 db = dist2x2(sub2(px, pack2(X.z, X.w)),
                                                 sub2(py, pack2(Y.z, Y.w)),
                                                 sub2(pz, pack2(Z.z, Z.w)));
                        float a0, a1, b0, b1;
                        unpack2(sub2(da, h2u), a0, a1);
                        unpack2(sub2(db, h2u), b0, b1);
                        acc = __funnelshift_l(__float_as_uint(a0), acc, 1);
                        acc = __funnelshift_l(__float_as_uint(a1), acc, 1);
                        acc = __funnelshift_l(__float_as_uint(b0), acc, 1);
                        acc = __funnelshift_l(__float_as_uint(b1), acc, 1);
                    }
                }
                // This lane's W hit bits at its place in the chunk's mask.
                uint32_t mask = (W == 32 ? __brev(acc) : (__brev(acc) >> (32 - W))) << (sub * W);
#pragma unroll
                for (int d = 1; d < L; d <<= 1) mask |= __shfl_xor_sync(gmask, mask, d, L);
                mask &= chunk_valid(j0, s, e, i);
                uint32_t mine = mask & own;
                int pos = count + __popc(mask & lower);
                while (mine) {
                    const int b = __ffs(mine) - 1;
                    mine &= mine - 1u;
                    if (pos < cap) out[static_cast<size_t>(pos) * stride] = static_cast<uint32_t>(j0 + b);
                    ++pos;
                }
                count += __popc(mask);
            }
        }
    __syncwarp(gmask);  // the group's stores ordered before any lane reads the list
    return count;
}


template <int L>
__device__ __forceinline__ unsigned lane_group_mask() {
    const unsigned lane = threadIdx.x & 31u;
    return ((1u << L) - 1u) << (lane & ~(L - 1u));
}

// A neighbour sum of particle i spread over its group of L lanes (gmask),
// the accumulation kept on lane 0 in list order.  In round m, lane q
// evaluates the V terms of list entry mL + q (term(k, t)), the group hands
// them to lane 0 by shuffles, and lane 0 adds them in entry order
// (add(u)).  Each term is the value one lane computes for that entry alone
// and the additions run in the same order, so the sum is the one-lane
// loop's, bit for bit; the lanes share the gathers and the term arithmetic.
template <int L, int V, class Term, class Add>
__device__ __forceinline__ void group_sum(int count, int sub, unsigned gmask, Term term, Add add) {
    for (int k0 = 0; k0 < count; k0 += L) {
        float t[V];
#pragma unroll
        for (int v = 0; v < V; ++v) t[v] = 0.0f;
        if (k0 + sub < count) term(k0 + sub, t);
#pragma unroll
        for (int q = 0; q < L; ++q) {
            float u[V];
#pragma unroll
            for (int v = 0; v < V; ++v) u[v] = __shfl_sync(gmask, t[v], q, L);
            if (sub == 0 && k0 + q < count) add(u);
        }
    }
}

// lambda_of_list on a group of L lanes (the value is lane 0's).
template <bool B, int L>
__device__ __forceinline__ float lambda_group(const StepConst& c, int i, int sub, unsigned gmask,
                                              float4 pi, const float4* __restrict__ xs,
                                              const uint32_t* __restrict__ out, size_t stride,
                                              int count) {
    LambdaAcc acc{c.k.c_poly6, 0.0f, 0.0f, 0.0f, 0.0f};
    group_sum<L, 4>(
        count, sub, gmask,
        [&](int k, float (&t)[4]) {
            const float4 pj = __ldg(&xs[out[static_cast<size_t>(k) * stride]]);
            const float dx = fsub(pi.x, pj.x), dy = fsub(pi.y, pj.y), dz = fsub(pi.z, pj.z);
            const float d2 = dist2(dx, dy, dz);
            t[0] = poly6(c.k, d2);
            spiky(c.k, dx, dy, dz, d2, t[1], t[2], t[3]);
        },
        [&](const float (&u)[4]) {
            acc.wsum = fadd(acc.wsum, u[0]);
            acc.s2 = ffma(u[3], u[3], ffma(u[2], u[2], ffma(u[1], u[1], acc.s2)));
            acc.gx = fadd(acc.gx, u[1]);
            acc.gy = fadd(acc.gy, u[2]);
            acc.gz = fadd(acc.gz, u[3]);
        });
    if constexpr (B) {
        const SceneConst& sc = scene_of(c, i);
        return lambda_finish(sc.mass, sc.rho0, sc.gs2, c.lambda_eps, acc);
    } else {
        return lambda_finish(c, acc);
    }
}

// k_search with L lanes per particle (slot-major lists only): the group
// walks the rows together (walk_chunks) and shares lambda's neighbour terms
// (lambda_group).  For scenes too small to fill the GPU with one thread per
// particle, where a walk is bound by the latency of one thread's row after
// row.
template <bool LAMBDA, bool B, int L>
__global__ void __launch_bounds__(kMaxTunedBlock)
k_search_split(const float4* __restrict__ xs, const float* __restrict__ sx,
               const float* __restrict__ sy, const float* __restrict__ sz,
               const int* __restrict__ first, StepConst c, int n, uint32_t* __restrict__ nbr,
               int* __restrict__ cnt, float* __restrict__ lam, unsigned* __restrict__ status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / L, sub = t % L;
    if (i >= n) return;  // whole groups
    const unsigned gmask = lane_group_mask<L>();
    if (__any_sync(gmask, fatal(status))) return;
    const float4 pi = xs[i];
    uint32_t* __restrict__ out = nbr + nb_first(c, i);
    const int count = walk_chunks<B, L>(c, i, sub, gmask, pi, sx, sy, sz, first, out);
    if (sub == 0) {
        cnt[i] = count;
        if (count > c.max_nb) atomicOr(status, kStatusNeighborOverflow);
    }
    if (LAMBDA) {
        const float l = count > c.max_nb
                            ? CUDART_NAN_F
                            : lambda_group<B, L>(c, i, sub, gmask, pi, xs, out, nb_step(c), count);
        if (sub == 0) lam[i] = l;
    }
}

// Compact lists, first pass: the walk's neighbour count only.
template <bool B>
__global__ void __launch_bounds__(kMaxTunedBlock)
k_count(const float4* __restrict__ xs, const float* __restrict__ sx,
        const float* __restrict__ sy, const float* __restrict__ sz,
        const int* __restrict__ first, StepConst c, int n, int* __restrict__ cnt,
        unsigned* __restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || fatal(status)) return;
    const int count = walk<B, false>(c, i, xs[i], sx, sy, sz, first, nullptr, c.max_nb);
    cnt[i] = count;
    if (count > c.max_nb) atomicOr(status, kStatusNeighborOverflow);
}

// Exclusive scan of the counts into list offsets, in three launches: tile
// scans with tile totals, a scan of the totals, and the carry-in.  64-bit
// sums; offsets are 32-bit because the list capacity is below 2^32.
constexpr int kScanThreads = 256, kScanItems = 8, kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ unsigned long long block_scan_u64(unsigned long long v,
                                                             unsigned long long* warp_tot,
                                                             unsigned long long& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x / 32;
        unsigned long long w = lane < nw ? warp_tot[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < nw) warp_tot[lane] = w;
    }
    __syncthreads();
    total = warp_tot[blockDim.x / 32 - 1];
    const unsigned long long before = warp ? warp_tot[warp - 1] : 0ull;
    __syncthreads();
    return before + incl - v;
}

__global__ void __launch_bounds__(kScanThreads)
k_nb_scan_tiles(const int* __restrict__ cnt, int n, uint32_t* __restrict__ off,
                unsigned long long* __restrict__ tile_sum, const unsigned* __restrict__ status) {
    if (fatal(status)) return;
    __shared__ unsigned long long warp_tot[kScanThreads / 32];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    unsigned long long v[kScanItems], sum = 0;
#pragma unroll
    for (int r = 0; r < kScanItems; ++r) {
        const int idx = base + r;
        v[r] = idx < n ? static_cast<unsigned long long>(max(0, cnt[idx])) : 0ull;
        sum += v[r];
    }
    unsigned long long total;
    unsigned long long run = block_scan_u64(sum, warp_tot, total);
#pragma unroll
    for (int r = 0; r < kScanItems; ++r) {
        const int idx = base + r;
        // Tile-local; a clamped value means a total of at least 2^32 entries,
        // above any capacity, which the last launch flags.
        if (idx < n) off[idx] = static_cast<uint32_t>(min(run, 0xffffffffull));
        run += v[r];
    }
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// One block: exclusive scan of the tile totals in place.
__global__ void __launch_bounds__(kScanThreads)
k_nb_scan_sums(unsigned long long* __restrict__ tile_sum, int tiles,
               const unsigned* __restrict__ status) {
    if (fatal(status)) return;
    __shared__ unsigned long long warp_tot[kScanThreads / 32];
    unsigned long long carry = 0;
    for (int t0 = 0; t0 < tiles; t0 += kScanThreads) {
        const int t = t0 + threadIdx.x;
        const unsigned long long v = t < tiles ? tile_sum[t] : 0ull;
        unsigned long long total;
        const unsigned long long ex = block_scan_u64(v, warp_tot, total);
        if (t < tiles) tile_sum[t] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) tile_sum[tiles] = carry;
}

// Carry-in, the total at off[n], and the capacity check.
__global__ void __launch_bounds__(kScanThreads)
k_nb_scan_add(int n, size_t cap, const unsigned long long* __restrict__ tile_sum, int tiles,
              uint32_t* __restrict__ off, unsigned* __restrict__ status) {
    if (fatal(status)) return;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned long long total = tile_sum[tiles];
    if (idx < n) {
        const unsigned long long o = tile_sum[idx / kScanTile] + off[idx];
        off[idx] = static_cast<uint32_t>(min(o, 0xffffffffull));
    }
    if (idx == 0) {
        off[n] = static_cast<uint32_t>(min(total, 0xffffffffull));
        if (total > cap) atomicOr(status, kStatusListOverflow);
    }
}

__device__ __forceinline__ bool count_ok(int count, int max_nb) {
    return count >= 0 && count <= max_nb;
}

// Walks a slot-major list in order, four neighbours at a time: their four
// gathers (load(j)) are issued before any term is used.  Terms are handed
// over two at a time (use2(first, second)) for FP32x2 evaluation; a last odd
// neighbour goes to use1.  List order is kept.
template <class T, class Load, class Use2, class Use1>
__device__ __forceinline__ void for_each_neighbor_pair(const uint32_t* __restrict__ row,
                                                       size_t stride, int count, Load load,
                                                       Use2 use2, Use1 use1) {
    // The indices of the next four neighbours are loaded while the current
    // four are gathered and used, so the list read (from DRAM) overlaps the
    // dependent gathers instead of preceding them.
    int k = 0;
    uint32_t jn[4];
    if (count >= 4) {
#pragma unroll
        for (int b = 0; b < 4; ++b) jn[b] = __ldg(&row[static_cast<size_t>(b) * stride]);
    }
    for (; k + 4 <= count; k += 4) {
        uint32_t j[4];
#pragma unroll
        for (int b = 0; b < 4; ++b) j[b] = jn[b];
        if (k + 8 <= count) {
#pragma unroll
            for (int b = 0; b < 4; ++b)
                jn[b] = __ldg(&row[static_cast<size_t>(k + 4 + b) * stride]);
        }
        T v[4];
#pragma unroll
        for (int b = 0; b < 4; ++b) v[b] = load(j[b]);
        use2(v[0], v[1]);
        use2(v[2], v[3]);
    }
    if (k + 2 <= count) {
        const uint32_t j0 = __ldg(&row[static_cast<size_t>(k) * stride]);
        const uint32_t j1 = __ldg(&row[static_cast<size_t>(k + 1) * stride]);
        const T a = load(j0), b = load(j1);
        use2(a, b);
        k += 2;
    }
    if (k < count) use1(load(__ldg(&row[static_cast<size_t>(k) * stride])));
}

struct PosVel {
    float4 p, v;
};
struct PosLam {
    float4 p;
    float l;
};

// Differences a - (b0, b1) of one float against a pair.
__device__ __forceinline__ f32x2 diff2(float a, float b0, float b1) {
    return sub2(splat2(a), pack2(b0, b1));
}
__device__ __forceinline__ f32x2 rdiff2(float b0, float b1, float a) {
    return sub2(pack2(b0, b1), splat2(a));
}
// crossc on pairs: a.y*b.z - a.z*b.y with one rounding of a.y*b.z.
__device__ __forceinline__ f32x2 crossc2(f32x2 ay, f32x2 az, f32x2 by, f32x2 bz) {
    return fma2(ay, bz, mul2(mul2(az, splat2(-1.0f)), by));
}

// computeDeltaPosition summed in list order (pbf_solver_kernels.cu:134-171).
// Indices, positions and lambdas of four neighbours are loaded before any of
// them is used, so the dependent gathers overlap; the sum stays in list order.
template <int N>
__device__ __forceinline__ void delta_term(const StepConst& c, float4 pi, float li, float4 pj,
                                           float lj, float& ax, float& ay, float& az) {
    const float dx = fsub(pi.x, pj.x), dy = fsub(pi.y, pj.y), dz = fsub(pi.z, pj.z);
    const float d2 = dist2(dx, dy, dz);
    float gx, gy, gz;
    spiky(c.k, dx, dy, dz, d2, gx, gy, gz);
    const float ls = fadd(fadd(li, lj), scorr<N>(c.sc, d2));
    ax = ffma(ls, gx, ax);
    ay = ffma(ls, gy, ay);
    az = ffma(ls, gz, az);
}

// Two neighbours' terms, lane 0 first: the same sums as two delta_term calls.
template <int N>
__device__ __forceinline__ void delta_term2(const StepConst& c, float4 pi, float li, float4 pa,
                                            float la, float4 pb, float lb, float& ax, float& ay,
                                            float& az) {
    const f32x2 dx = sub2(splat2(pi.x), pack2(pa.x, pb.x));
    const f32x2 dy = sub2(splat2(pi.y), pack2(pa.y, pb.y));
    const f32x2 dz = sub2(splat2(pi.z), pack2(pa.z, pb.z));
    const f32x2 d2 = dist2x2(dx, dy, dz);
    const f32x2 s = spiky_scale2(c.k, d2);
    const f32x2 ls = add2(add2(splat2(li), pack2(la, lb)), scorr2<N>(c.sc, d2));
    float l0, l1, x0, x1, y0, y1, z0, z1;
    unpack2(ls, l0, l1);
    unpack2(mul2(dx, s), x0, x1);
    unpack2(mul2(dy, s), y0, y1);
    unpack2(mul2(dz, s), z0, z1);
    ax = ffma(l1, x1, ffma(l0, x0, ax));
    ay = ffma(l1, y1, ffma(l0, y0, ay));
    az = ffma(l1, z1, ffma(l0, z0, az));
}

template <int N>
__device__ __forceinline__ void delta_sum(const StepConst& c, const float4* __restrict__ xs,
                                          const uint32_t* __restrict__ nbr,
                                          const float* __restrict__ lam, int i, int count,
                                          float4 pi, float gs, float& dpx, float& dpy,
                                          float& dpz) {
    const float li = lam[i];
    float ax = 0.0f, ay = 0.0f, az = 0.0f;
    for_each_neighbor_pair<PosLam>(
        nbr + nb_first(c, i), nb_step(c), count,
        [&](uint32_t j) { return PosLam{__ldg(&xs[j]), __ldg(&lam[j])}; },
        [&](const PosLam& a, const PosLam& b) {
            delta_term2<N>(c, pi, li, a.p, a.l, b.p, b.l, ax, ay, az);
        },
        [&](const PosLam& q) { delta_term<N>(c, pi, li, q.p, q.l, ax, ay, az); });
    dpx = fmul(gs, ax);
    dpy = fmul(gs, ay);
    dpz = fmul(gs, az);
}

// delta_sum with its terms spread over a group of L lanes (lane 0's value).
template <int N, int L>
__device__ __forceinline__ void delta_sum_group(const StepConst& c, const float4* __restrict__ xs,
                                                const uint32_t* __restrict__ nbr,
                                                const float* __restrict__ lam, int i, int sub,
                                                unsigned gmask, int count, float4 pi, float gs,
                                                float& dpx, float& dpy, float& dpz) {
    const float li = lam[i];
    const uint32_t* row = nbr + nb_first(c, i);
    const size_t st = nb_step(c);
    float ax = 0.0f, ay = 0.0f, az = 0.0f;
    group_sum<L, 4>(
        count, sub, gmask,
        [&](int k, float (&t)[4]) {
            const uint32_t j = __ldg(&row[static_cast<size_t>(k) * st]);
            const float4 pj = __ldg(&xs[j]);
            const float lj = __ldg(&lam[j]);
            const float dx = fsub(pi.x, pj.x), dy = fsub(pi.y, pj.y), dz = fsub(pi.z, pj.z);
            const float d2 = dist2(dx, dy, dz);
            spiky(c.k, dx, dy, dz, d2, t[1], t[2], t[3]);
            t[0] = fadd(fadd(li, lj), scorr<N>(c.sc, d2));
        },
        [&](const float (&u)[4]) {
            ax = ffma(u[0], u[1], ax);
            ay = ffma(u[0], u[2], ay);
            az = ffma(u[0], u[3], az);
        });
    dpx = fmul(gs, ax);
    dpy = fmul(gs, ay);
    dpz = fmul(gs, az);
}

// The thread's particle and lane in a launch of L lanes per particle; false
// for threads past the last particle (whole groups) and, group-wide, once a
// fatal status bit is set.
template <int L>
__device__ __forceinline__ bool group_thread(int n, const unsigned* status, int& i, int& sub,
                                             unsigned& gmask) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    i = t / L;
    sub = t % L;
    gmask = 0u;
    if (i >= n) return false;
    if constexpr (L == 1) {
        return !fatal(status);
    } else {
        gmask = lane_group_mask<L>();
        return !__any_sync(gmask, fatal(status));
    }
}

// delta p + applyDeltaPosition + CollisionSystem::solve + next cell keys.
// N: artificial-pressure exponent fixed at compile time (0 = read at run time).
// moved (optional): bit a set where the projection changed component a.
// pre (optional): the position before the projection.
// L lanes per particle share the neighbour terms (small scenes, with the
// split walks); lane 0 applies.
template <int N, bool B, int L>
__global__ void PBF_GATHER_REGS(48)
k_delta_apply(const float4* __restrict__ xs, const uint32_t* __restrict__ nbr,
              const int* __restrict__ cnt, const float* __restrict__ lam, StepConst c, int n,
              float4* __restrict__ xs_out, uint32_t* __restrict__ keys_out,
              uint8_t* __restrict__ moved, float4* __restrict__ pre,
              unsigned* __restrict__ status) {
    int i, sub;
    unsigned gmask;
    if (!group_thread<L>(n, status, i, sub, gmask)) return;
    const float4 pi = xs[i];
    const int count = cnt[i];
    float dpx, dpy, dpz;
    if (!count_ok(count, c.max_nb)) {
        dpx = dpy = dpz = CUDART_NAN_F;
    } else {
        const float gs = B ? scene_of(c, i).gs : c.gs;
        if constexpr (L == 1)
            delta_sum<N>(c, xs, nbr, lam, i, count, pi, gs, dpx, dpy, dpz);
        else
            delta_sum_group<N, L>(c, xs, nbr, lam, i, sub, gmask, count, pi, gs, dpx, dpy, dpz);
    }
    if (sub != 0) return;
    float px = fadd(pi.x, dpx), py = fadd(pi.y, dpy), pz = fadd(pi.z, dpz);
    const float ux = px, uy = py, uz = pz;
    if (pre) pre[i] = make_float4(ux, uy, uz, pi.w);
    if (!project_all(colliders_of<B>(c, i), c.particle_radius, px, py, pz))
        atomicOr(status, kStatusNotConverged);
    if (moved)
        moved[i] = static_cast<uint8_t>((px != ux) | ((py != uy) << 1) | ((pz != uz) << 2));
    const float4 q = make_float4(px, py, pz, pi.w);
    xs_out[i] = q;
    if (keys_out) {
        GridConst g;
        uint32_t base;
        grid_of<B>(c, i, g, base);
        keys_out[i] = base + key_of(g, q);
    }
}

// Gather x, v_in, v.w and ids through the composite permutation of the
// substep, then updateVelocityAndPosition (pbf_solver_kernels.cu:195-211).
// The new positions are the predicted ones, so xs becomes x without a copy.
__global__ void __launch_bounds__(kBlock)
k_finalize(const uint32_t* __restrict__ org, const float4* __restrict__ x_old,
           const float4* __restrict__ vin_old, const float4* __restrict__ v_old,
           const uint32_t* __restrict__ id_old, const float4* __restrict__ xs, int n,
           StepConst c, float4* __restrict__ v_new, float4* __restrict__ vin_new,
           uint32_t* __restrict__ id_new, const unsigned* __restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || fatal(status)) return;
    const uint32_t o = org[i];
    const float4 xo = x_old[o];
    const float4 q = xs[i];
    float4 vv;
    vv.x = fmul(fsub(q.x, xo.x), c.inv_dt);
    vv.y = fmul(fsub(q.y, xo.y), c.inv_dt);
    vv.z = fmul(fsub(q.z, xo.z), c.inv_dt);
    vv.w = v_old[o].w;
    v_new[i] = vv;
    vin_new[i] = vin_old[o];
    if (id_new) id_new[i] = id_old[o];
}

// applyXsphViscosity (pbf_solver_kernels.cu:213-266).
__device__ __forceinline__ float4 xsph_one(const StepConst& c, const float4* __restrict__ x,
                                           const float4* __restrict__ v,
                                           const uint32_t* __restrict__ nbr, int count, int i,
                                           float xsph_c) {
    const float4 vi = v[i];
    if (!count_ok(count, c.max_nb))
        return make_float4(CUDART_NAN_F, CUDART_NAN_F, CUDART_NAN_F, vi.w);
    const float4 pi = x[i];
    float cx = 0.0f, cy = 0.0f, cz = 0.0f;
    for_each_neighbor_pair<PosVel>(
        nbr + nb_first(c, i), nb_step(c), count,
        [&](uint32_t j) { return PosVel{__ldg(&x[j]), __ldg(&v[j])}; },
        [&](const PosVel& a, const PosVel& b) {
            float w0, w1, x0, x1, y0, y1, z0, z1;
            unpack2(poly6_2(c.k, dist2x2(diff2(pi.x, a.p.x, b.p.x), diff2(pi.y, a.p.y, b.p.y),
                                         diff2(pi.z, a.p.z, b.p.z))),
                    w0, w1);
            unpack2(rdiff2(a.v.x, b.v.x, vi.x), x0, x1);
            unpack2(rdiff2(a.v.y, b.v.y, vi.y), y0, y1);
            unpack2(rdiff2(a.v.z, b.v.z, vi.z), z0, z1);
            cx = ffma(x1, w1, ffma(x0, w0, cx));
            cy = ffma(y1, w1, ffma(y0, w0, cy));
            cz = ffma(z1, w1, ffma(z0, w0, cz));
        },
        [&](const PosVel& q) {
            const float w =
                poly6(c.k, dist2(fsub(pi.x, q.p.x), fsub(pi.y, q.p.y), fsub(pi.z, q.p.z)));
            cx = ffma(fsub(q.v.x, vi.x), w, cx);
            cy = ffma(fsub(q.v.y, vi.y), w, cy);
            cz = ffma(fsub(q.v.z, vi.z), w, cz);
        });
    return make_float4(ffma(xsph_c, cx, vi.x), ffma(xsph_c, cy, vi.y), ffma(xsph_c, cz, vi.z),
                       vi.w);
}

template <bool B>
__global__ void __launch_bounds__(kMaxTunedBlock)
k_xsph(const float4* __restrict__ x, const float4* __restrict__ v,
       const uint32_t* __restrict__ nbr, const int* __restrict__ cnt, StepConst c, int n,
       float4* __restrict__ v_out, const float4* __restrict__ vin, bool resolve,
       const unsigned* __restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || fatal(status)) return;
    float4 out = xsph_one(c, x, v, nbr, cnt[i], i, B ? scene_of(c, i).xsph_c : c.xsph_c);
    if (resolve)
        resolve_velocity(colliders_of<B>(c, i), c.particle_radius, c.restitution, c.friction,
                         x[i], vin[i], out);
    v_out[i] = out;
}

// What the final walk does once particle i's list (count entries) is written.
template <bool B>
__device__ __forceinline__ void xsph_tail(const StepConst& c, int i, float4 pi,
                                          const float4* __restrict__ xs,
                                          const uint32_t* __restrict__ nbr, int count,
                                          int* __restrict__ cnt, const float4* __restrict__ v,
                                          float4* __restrict__ v_out,
                                          const float4* __restrict__ vin, bool resolve,
                                          unsigned* __restrict__ status) {
    cnt[i] = count;
    if (count > c.max_nb) atomicOr(status, kStatusNeighborOverflow);
    float4 out = xsph_one(c, xs, v, nbr, count, i, B ? scene_of(c, i).xsph_c : c.xsph_c);
    if (resolve)
        resolve_velocity(colliders_of<B>(c, i), c.particle_radius, c.restitution, c.friction,
                         pi, vin[i], out);
    v_out[i] = out;
}

// The final rebuild's walk with XSPH fused in: the list is written, then
// applyXsphViscosity runs over it in a second pass (velocities v are the
// updated ones, computed before this walk), with the velocity response when
// no vorticity pass follows.
template <bool B>
__global__ void __launch_bounds__(kMaxTunedBlock)
k_search_xsph(const float4* __restrict__ xs, const float* __restrict__ sx,
              const float* __restrict__ sy, const float* __restrict__ sz,
              const int* __restrict__ first, StepConst c, int n, uint32_t* __restrict__ nbr,
              int* __restrict__ cnt, const float4* __restrict__ v, float4* __restrict__ v_out,
              const float4* __restrict__ vin, bool resolve, unsigned* __restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || fatal(status)) return;
    const float4 pi = xs[i];
    const int count = walk<B>(c, i, pi, sx, sy, sz, first, nbr + nb_first(c, i), c.max_nb);
    xsph_tail<B>(c, i, pi, xs, nbr, count, cnt, v, v_out, vin, resolve, status);
}

// k_search_xsph with L lanes per particle: the group walks together
// (walk_chunks) and shares the XSPH terms; lane 0 writes.
template <bool B, int L>
__global__ void __launch_bounds__(kMaxTunedBlock)
k_search_xsph_split(const float4* __restrict__ xs, const float* __restrict__ sx,
                    const float* __restrict__ sy, const float* __restrict__ sz,
                    const int* __restrict__ first, StepConst c, int n,
                    uint32_t* __restrict__ nbr, int* __restrict__ cnt,
                    const float4* __restrict__ v, float4* __restrict__ v_out,
                    const float4* __restrict__ vin, bool resolve, unsigned* __restrict__ status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / L, sub = t % L;
    if (i >= n) return;  // whole groups
    const unsigned gmask = lane_group_mask<L>();
    if (__any_sync(gmask, fatal(status))) return;
    const float4 pi = xs[i];
    const int count =
        walk_chunks<B, L>(c, i, sub, gmask, pi, sx, sy, sz, first, nbr + nb_first(c, i));
    if (sub == 0) {
        cnt[i] = count;
        if (count > c.max_nb) atomicOr(status, kStatusNeighborOverflow);
    }
    // applyXsphViscosity over the new list, its terms spread over the group.
    const float4 vi = v[i];
    float4 out;
    if (!count_ok(count, c.max_nb)) {
        out = make_float4(CUDART_NAN_F, CUDART_NAN_F, CUDART_NAN_F, vi.w);
    } else {
        const uint32_t* row = nbr + nb_first(c, i);
        const size_t st = nb_step(c);
        float cx = 0.0f, cy = 0.0f, cz = 0.0f;
        group_sum<L, 4>(
            count, sub, gmask,
            [&](int k, float (&t)[4]) {
                const uint32_t j = row[static_cast<size_t>(k) * st];  // written above
                const float4 pj = __ldg(&xs[j]), vj = __ldg(&v[j]);
                t[0] = poly6(c.k, dist2(fsub(pi.x, pj.x), fsub(pi.y, pj.y), fsub(pi.z, pj.z)));
                t[1] = fsub(vj.x, vi.x);
                t[2] = fsub(vj.y, vi.y);
                t[3] = fsub(vj.z, vi.z);
            },
            [&](const float (&u)[4]) {
                cx = ffma(u[1], u[0], cx);
                cy = ffma(u[2], u[0], cy);
                cz = ffma(u[3], u[0], cz);
            });
        const float xc = B ? scene_of(c, i).xsph_c : c.xsph_c;
        out = make_float4(ffma(xc, cx, vi.x), ffma(xc, cy, vi.y), ffma(xc, cz, vi.z), vi.w);
    }
    if (sub != 0) return;
    if (resolve)
        resolve_velocity(colliders_of<B>(c, i), c.particle_radius, c.restitution, c.friction, pi,
                         vin[i], out);
    v_out[i] = out;
}

// computeVorticity (pbf_solver_kernels.cu:268-315).
__global__ void __launch_bounds__(kMaxTunedBlock)
k_vorticity(const float4* __restrict__ x, const float4* __restrict__ v,
            const uint32_t* __restrict__ nbr, const int* __restrict__ cnt, StepConst c, int n,
            float4* __restrict__ omega, bool store_norm, const unsigned* __restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || fatal(status)) return;
    const int count = cnt[i];
    if (!count_ok(count, c.max_nb)) {
        omega[i] = make_float4(CUDART_NAN_F, CUDART_NAN_F, CUDART_NAN_F,
                               store_norm ? CUDART_NAN_F : 0.0f);
        return;
    }
    const float4 pi = x[i], vi = v[i];
    float ox = 0.0f, oy = 0.0f, oz = 0.0f;
    for_each_neighbor_pair<PosVel>(
        nbr + nb_first(c, i), nb_step(c), count,
        [&](uint32_t j) { return PosVel{__ldg(&x[j]), __ldg(&v[j])}; },
        [&](const PosVel& a, const PosVel& b) {
            const f32x2 dx = diff2(pi.x, a.p.x, b.p.x), dy = diff2(pi.y, a.p.y, b.p.y),
                        dz = diff2(pi.z, a.p.z, b.p.z);
            const f32x2 sc = spiky_scale2(c.k, dist2x2(dx, dy, dz));
            const f32x2 gx = mul2(dx, sc), gy = mul2(dy, sc), gz = mul2(dz, sc);
            const f32x2 vx = rdiff2(a.v.x, b.v.x, vi.x), vy = rdiff2(a.v.y, b.v.y, vi.y),
                        vz = rdiff2(a.v.z, b.v.z, vi.z);
            float x0, x1, y0, y1, z0, z1;
            unpack2(crossc2(gy, gz, vy, vz), x0, x1);
            unpack2(crossc2(gz, gx, vz, vx), y0, y1);
            unpack2(crossc2(gx, gy, vx, vy), z0, z1);
            ox = fadd(fadd(ox, x0), x1);
            oy = fadd(fadd(oy, y0), y1);
            oz = fadd(fadd(oz, z0), z1);
        },
        [&](const PosVel& q) {
            const float dx = fsub(pi.x, q.p.x), dy = fsub(pi.y, q.p.y), dz = fsub(pi.z, q.p.z);
            float gx, gy, gz;
            spiky(c.k, dx, dy, dz, dist2(dx, dy, dz), gx, gy, gz);
            const float vx = fsub(q.v.x, vi.x), vy = fsub(q.v.y, vi.y), vz = fsub(q.v.z, vi.z);
            ox = fadd(ox, crossc(gy, gz, vy, vz));
            oy = fadd(oy, crossc(gz, gx, vz, vx));
            oz = fadd(oz, crossc(gx, gy, vx, vy));
        });
    // With store_norm, w carries |omega| (read by the confinement for every
    // neighbour); otherwise w = 0 as computeVorticity writes it.
    omega[i] = make_float4(ox, oy, oz, store_norm ? len3(ox, oy, oz) : 0.0f);
}

// w <- |omega| for a vorticity array written with w = 0.
__global__ void __launch_bounds__(kBlock) k_omega_norm(float4* __restrict__ om, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 w = om[i];
    w.w = len3(w.x, w.y, w.z);
    om[i] = w;
}

// The confinement velocity from the summed eta = sum (|w_j| - |w_i|) grad W.
__device__ __forceinline__ float4 confine_finish(const StepConst& c, float ex, float ey, float ez,
                                                 float4 wi, float4 vi) {
    const float el = len3(ex, ey, ez);
    float nx = 0.0f, ny = 0.0f, nz = 0.0f;
    if (el > kEtaEpsilon) {
        nx = fdiv(ex, el);
        ny = fdiv(ey, el);
        nz = fdiv(ez, el);
    }
    const float cx = fmul(c.vort_eps, crossc(ny, nz, wi.y, wi.z));
    const float cy = fmul(c.vort_eps, crossc(nz, nx, wi.z, wi.x));
    const float cz = fmul(c.vort_eps, crossc(nx, ny, wi.x, wi.y));
    return make_float4(ffma(c.dt, cx, vi.x), ffma(c.dt, cy, vi.y), ffma(c.dt, cz, vi.z), vi.w);
}

// applyVorticityConfinement (pbf_solver_kernels.cu:317-385).
__device__ __forceinline__ float4 confine_one(const StepConst& c, const float4* __restrict__ x,
                                              const uint32_t* __restrict__ nbr, int count,
                                              const float4* __restrict__ om,
                                              const float4* __restrict__ v, int i) {
    const float4 vi = v[i];
    if (!count_ok(count, c.max_nb))
        return make_float4(CUDART_NAN_F, CUDART_NAN_F, CUDART_NAN_F, vi.w);
    const float4 pi = x[i], wi = om[i];
    const float wil = wi.w;  // |omega_i|, stored by k_vorticity
    float ex = 0.0f, ey = 0.0f, ez = 0.0f;
    for_each_neighbor_pair<PosVel>(
        nbr + nb_first(c, i), nb_step(c), count,
        [&](uint32_t j) { return PosVel{__ldg(&x[j]), __ldg(&om[j])}; },
        [&](const PosVel& a, const PosVel& b) {
            const f32x2 dx = diff2(pi.x, a.p.x, b.p.x), dy = diff2(pi.y, a.p.y, b.p.y),
                        dz = diff2(pi.z, a.p.z, b.p.z);
            const f32x2 sc = spiky_scale2(c.k, dist2x2(dx, dy, dz));
            float m0, m1, x0, x1, y0, y1, z0, z1;
            unpack2(rdiff2(a.v.w, b.v.w, wil), m0, m1);
            unpack2(mul2(dx, sc), x0, x1);
            unpack2(mul2(dy, sc), y0, y1);
            unpack2(mul2(dz, sc), z0, z1);
            ex = ffma(m1, x1, ffma(m0, x0, ex));
            ey = ffma(m1, y1, ffma(m0, y0, ey));
            ez = ffma(m1, z1, ffma(m0, z0, ez));
        },
        [&](const PosVel& q) {
            const float wjl = q.v.w;
            const float dx = fsub(pi.x, q.p.x), dy = fsub(pi.y, q.p.y), dz = fsub(pi.z, q.p.z);
            float gx, gy, gz;
            spiky(c.k, dx, dy, dz, dist2(dx, dy, dz), gx, gy, gz);
            const float md = fsub(wjl, wil);
            ex = ffma(md, gx, ex);
            ey = ffma(md, gy, ey);
            ez = ffma(md, gz, ez);
        });
    return confine_finish(c, ex, ey, ez, wi, vi);
}

template <bool B>
__global__ void __launch_bounds__(kMaxTunedBlock)
k_confine(const float4* __restrict__ x, const uint32_t* __restrict__ nbr,
          const int* __restrict__ cnt, const float4* __restrict__ om,
          const float4* __restrict__ v, StepConst c, int n, float4* __restrict__ v_out,
          const float4* __restrict__ vin, bool resolve, const unsigned* __restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || fatal(status)) return;
    float4 out = confine_one(c, x, nbr, cnt[i], om, v, i);
    if (resolve)
        resolve_velocity(colliders_of<B>(c, i), c.particle_radius, c.restitution, c.friction,
                         x[i], vin[i], out);
    v_out[i] = out;
}

// k_vorticity with L lanes per particle sharing the neighbour terms (small
// scenes); lane 0 writes.
template <int L>
__global__ void __launch_bounds__(kMaxTunedBlock)
k_vorticity_group(const float4* __restrict__ x, const float4* __restrict__ v,
                  const uint32_t* __restrict__ nbr, const int* __restrict__ cnt, StepConst c,
                  int n, float4* __restrict__ omega, bool store_norm,
                  const unsigned* __restrict__ status) {
    int i, sub;
    unsigned gmask;
    if (!group_thread<L>(n, status, i, sub, gmask)) return;
    const int count = cnt[i];
    if (!count_ok(count, c.max_nb)) {
        if (sub == 0)
            omega[i] = make_float4(CUDART_NAN_F, CUDART_NAN_F, CUDART_NAN_F,
                                   store_norm ? CUDART_NAN_F : 0.0f);
        return;
    }
    const float4 pi = x[i], vi = v[i];
    const uint32_t* row = nbr + nb_first(c, i);
    const size_t st = nb_step(c);
    float ox = 0.0f, oy = 0.0f, oz = 0.0f;
    group_sum<L, 3>(
        count, sub, gmask,
        [&](int k, float (&t)[3]) {
            const uint32_t j = __ldg(&row[static_cast<size_t>(k) * st]);
            const float4 pj = __ldg(&x[j]), vj = __ldg(&v[j]);
            const float dx = fsub(pi.x, pj.x), dy = fsub(pi.y, pj.y), dz = fsub(pi.z, pj.z);
            float gx, gy, gz;
            spiky(c.k, dx, dy, dz, dist2(dx, dy, dz), gx, gy, gz);
            const float vx = fsub(vj.x, vi.x), vy = fsub(vj.y, vi.y), vz = fsub(vj.z, vi.z);
            t[0] = crossc(gy, gz, vy, vz);
            t[1] = crossc(gz, gx, vz, vx);
            t[2] = crossc(gx, gy, vx, vy);
        },
        [&](const float (&u)[3]) {
            ox = fadd(ox, u[0]);
            oy = fadd(oy, u[1]);
            oz = fadd(oz, u[2]);
        });
    if (sub == 0) omega[i] = make_float4(ox, oy, oz, store_norm ? len3(ox, oy, oz) : 0.0f);
}

template <bool B>
__global__ void __launch_bounds__(kBlock)
k_resolve(const float4* __restrict__ x, const float4* __restrict__ vin, float4* __restrict__ v,
          StepConst c, int n, const unsigned* __restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || fatal(status)) return;
    float4 vv = v[i];
    resolve_velocity(colliders_of<B>(c, i), c.particle_radius, c.restitution, c.friction, x[i],
                     vin[i], vv);
    v[i] = vv;
}

// scatterFloat4ByStableId (pbf_solver_kernels.cu:418-427).
__global__ void __launch_bounds__(kBlock)
k_scatter_by_id(const float4* __restrict__ vals, const uint32_t* __restrict__ id,
                float4* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[id[i]] = vals[i];
}

__global__ void __launch_bounds__(kBlock) k_iota(uint32_t* a, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = static_cast<uint32_t>(i);
}

// |rho/rho0 - 1| per particle over the current lists.
__global__ void __launch_bounds__(kBlock)
k_density(const float4* __restrict__ x, const uint32_t* __restrict__ nbr,
          const int* __restrict__ cnt, StepConst c, int n, float* __restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 pi = x[i];
    const int count = min(cnt[i], c.max_nb);
    float wsum = c.k.c_poly6;
    const uint32_t* list = nbr + nb_first(c, i);
    const size_t step = nb_step(c);
    for (int k = 0; k < count; ++k) {
        const float4 pj = __ldg(&x[__ldg(&list[static_cast<size_t>(k) * step])]);
        wsum = fadd(wsum, poly6(c.k, dist2(fsub(pi.x, pj.x), fsub(pi.y, pj.y), fsub(pi.z, pj.z))));
    }
    const float mass = c.scenes ? scene_of(c, i).mass : c.mass;
    const float rho0 = c.scenes ? scene_of(c, i).rho0 : c.rho0;
    err[i] = fabsf(fsub(fdiv(fmul(mass, wsum), rho0), 1.0f));
}

// --- stage kernels -----------------------------------------------------------
__global__ void __launch_bounds__(kBlock)
k_grid_keys(const float4* __restrict__ pos, uint32_t* __restrict__ keys, int n, GridConst g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) keys[i] = key_of(g, pos[i]);
}

__global__ void __launch_bounds__(kBlock)
k_lambda_list(const float4* __restrict__ xs, const uint32_t* __restrict__ nbr,
              const int* __restrict__ cnt, StepConst c, int n, float* __restrict__ lam) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int count = cnt[i];
    if (!count_ok(count, c.max_nb)) {
        lam[i] = CUDART_NAN_F;
        return;
    }
    const float4 pi = xs[i];
    LambdaAcc acc{c.k.c_poly6, 0.0f, 0.0f, 0.0f, 0.0f};
    for (int k = 0; k < count; ++k) {
        const float4 pj = xs[nbr[static_cast<size_t>(k) * c.stride + i]];
        const float dx = fsub(pi.x, pj.x), dy = fsub(pi.y, pj.y), dz = fsub(pi.z, pj.z);
        lambda_add(c.k, acc, dx, dy, dz, dist2(dx, dy, dz));
    }
    lam[i] = lambda_finish(c, acc);
}

__global__ void __launch_bounds__(kBlock)
k_delta_list(const float4* __restrict__ xs, const uint32_t* __restrict__ nbr,
             const int* __restrict__ cnt, const float* __restrict__ lam, StepConst c, int n,
             float4* __restrict__ delta) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int count = cnt[i];
    if (!count_ok(count, c.max_nb)) {
        delta[i] = make_float4(CUDART_NAN_F, CUDART_NAN_F, CUDART_NAN_F, 0.0f);
        return;
    }
    float dx, dy, dz;
    delta_sum<0>(c, xs, nbr, lam, i, count, xs[i], c.gs, dx, dy, dz);
    delta[i] = make_float4(dx, dy, dz, 0.0f);
}

// kind: 0 container, 1 spheres, 2 boxes, 3 planes (one pass), 4 converge all.
__global__ void __launch_bounds__(kBlock)
k_collide(float4* __restrict__ pos, int n, StepConst c, int kind, unsigned* __restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = pos[i];
    bool mark = false;
    switch (kind) {
        case 0: mark = project_container(c.col, c.particle_radius, p.x, p.y, p.z); break;
        case 1: mark = project_spheres(c.col, c.particle_radius, p.x, p.y, p.z); break;
        case 2: mark = project_boxes(c.col, c.particle_radius, p.x, p.y, p.z); break;
        case 3: mark = project_planes(c.col, c.particle_radius, p.x, p.y, p.z); break;
        default: mark = !project_all(c.col, c.particle_radius, p.x, p.y, p.z); break;
    }
    if (mark) atomicOr(flag, 1u);
    pos[i] = p;
}

__global__ void __launch_bounds__(kBlock)
k_integrate(const float4* __restrict__ x, float4* __restrict__ xs, float4* __restrict__ v,
            int n, StepConst c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 vv = v[i];
    const float4 p = x[i];
    vv.x = ffma(c.gravx, c.dt, vv.x);
    vv.y = ffma(c.gravy, c.dt, vv.y);
    vv.z = ffma(c.gravz, c.dt, vv.z);
    v[i] = vv;
    xs[i] = make_float4(ffma(vv.x, c.dt, p.x), ffma(vv.y, c.dt, p.y), ffma(vv.z, c.dt, p.z), p.w);
}

}  // namespace

// --- launchers ---------------------------------------------------------------
void launch_predict(const float4* x, const float4* v, float4* xs, float4* vin, uint32_t* keys,
                    int n, const StepConst& c, const unsigned* status, cudaStream_t st) {
    if (c.scenes)
        launch_k(k_predict<true>, blocks_for(n), kBlock, st, x, v, xs, vin, keys, n, c, status);
    else
        launch_k(k_predict<false>, blocks_for(n), kBlock, st, x, v, xs, vin, keys, n, c, status);
}
void launch_cell_ranges(const uint32_t* skeys, int* cs, int* ce, int n, const unsigned* status,
                        cudaStream_t st) {
    k_cell_ranges<<<blocks_for(n), kBlock, 0, st>>>(skeys, cs, ce, n, status);
}
void launch_gather_xs(const uint32_t* perm, const float4* xs_in, float4* xs_out,
                      const uint32_t* org_in, uint32_t* org_out, float* sx, float* sy, float* sz,
                      int n, const unsigned* status, cudaStream_t st) {
    k_gather_xs<<<blocks_for(n), kBlock, 0, st>>>(perm, xs_in, xs_out, org_in, org_out, sx, sy, sz,
                                                  n, status);
}
void launch_gather_first(const uint32_t* perm, const float4* xs_in, float4* xs_out,
                         const uint32_t* org_in, uint32_t* org_out, float* sx, float* sy, float* sz,
                         int n, const uint32_t* skeys, uint64_t cells, int* first,
                         const unsigned* status, cudaStream_t st) {
    const uint64_t threads = std::max<uint64_t>(static_cast<uint64_t>(n), cells + 1);
    launch_k(k_gather_first, blocks_for(threads), kBlock, st, perm, xs_in, xs_out, org_in, org_out,
             sx, sy, sz, n, skeys, static_cast<uint32_t>(cells), first, status);
}
inline int tuned_block(const StepConst& c, int k) { return c.blk[k] > 0 ? c.blk[k] : kBlock; }

// Scene sizes for which a group of 8 or 4 lanes walks each particle by
// default.  Measured steps of dam breaks at 1 / 4 / 8 lanes: 0.219 / 0.206 /
// 0.174 ms at 8,192 particles, 0.270 / 0.230 / 0.215 at 16,384, 0.249 / 0.242
// / 0.237 at 20,480, 0.262 / 0.247 / 0.268 at 24,576, 0.269 / 0.255 / 0.291 at
// 28,672 and 0.274 / 0.283 / 0.334 at 32,768; 2 lanes are slower than 1 or 4
// (0.329 ms at 16,384, 0.399 at 65,536 against 0.316 for 1 lane: from there
// on the GPU is full with one lane per particle).
constexpr size_t kSplitWalk8Max = 20480;
constexpr size_t kSplitWalk4Below = size_t(1) << 15;

// Lanes per particle of a launch: c.walk_lanes where the split walk applies.
inline int split_lanes(const StepConst& c, int n) {
    const int L = c.walk_lanes;
    if ((L != 2 && L != 4 && L != 8) || c.nb_off != nullptr || c.max_nb < L ||
        static_cast<long long>(n) * L > (1LL << 30))
        return 1;
    return L;
}

int default_walk_lanes(size_t n, int max_nb) {
    int L = n <= kSplitWalk8Max ? 8 : (n < kSplitWalk4Below ? 4 : 1);
    while (L > 1 && max_nb < L) L /= 2;  // a group never has more lanes than list slots
    return L;
}

template <bool LAMBDA, bool B>
void launch_search_split(int L, int bs, const float4* xs, const float* sx, const float* sy,
                         const float* sz, const int* first, const StepConst& c, int n,
                         uint32_t* nbr, int* cnt, float* lam, unsigned* status, cudaStream_t st) {
    const unsigned g = blocks_for(static_cast<size_t>(n) * L, bs);
    if (L == 8)
        launch_k(k_search_split<LAMBDA, B, 8>, g, bs, st, xs, sx, sy, sz, first, c, n, nbr, cnt,
                 lam, status);
    else if (L == 4)
        launch_k(k_search_split<LAMBDA, B, 4>, g, bs, st, xs, sx, sy, sz, first, c, n, nbr, cnt,
                 lam, status);
    else
        launch_k(k_search_split<LAMBDA, B, 2>, g, bs, st, xs, sx, sy, sz, first, c, n, nbr, cnt,
                 lam, status);
}

void launch_search(const float4* xs, const float* sx, const float* sy, const float* sz,
                   const int* first, const StepConst& c, int n, uint32_t* nbr, int* cnt, float* lam,
                   unsigned* status, bool with_lambda, cudaStream_t st) {
    const int bs = tuned_block(c, with_lambda ? kTunedSearchLambda : kTunedSearch);
    if (const int L = split_lanes(c, n); L > 1) {
        if (with_lambda && c.scenes)
            launch_search_split<true, true>(L, bs, xs, sx, sy, sz, first, c, n, nbr, cnt, lam,
                                            status, st);
        else if (with_lambda)
            launch_search_split<true, false>(L, bs, xs, sx, sy, sz, first, c, n, nbr, cnt, lam,
                                             status, st);
        else if (c.scenes)
            launch_search_split<false, true>(L, bs, xs, sx, sy, sz, first, c, n, nbr, cnt, lam,
                                             status, st);
        else
            launch_search_split<false, false>(L, bs, xs, sx, sy, sz, first, c, n, nbr, cnt, lam,
                                              status, st);
        return;
    }
    const unsigned g = blocks_for(n, bs);
    if (with_lambda && c.scenes)
        launch_k(k_search<true, true>, g, bs, st, xs, sx, sy, sz, first, c, n, nbr, cnt, lam,
                 status);
    else if (with_lambda)
        launch_k(k_search<true, false>, g, bs, st, xs, sx, sy, sz, first, c, n, nbr, cnt, lam,
                 status);
    else if (c.scenes)
        launch_k(k_search<false, true>, g, bs, st, xs, sx, sy, sz, first, c, n, nbr, cnt, lam,
                 status);
    else
        launch_k(k_search<false, false>, g, bs, st, xs, sx, sy, sz, first, c, n, nbr, cnt, lam,
                 status);
}

template <bool B>
void launch_search_xsph_split(int L, unsigned g, int bs, const float4* xs, const float* sx,
                              const float* sy, const float* sz, const int* first,
                              const StepConst& c, int n, uint32_t* nbr, int* cnt, const float4* v,
                              float4* v_out, const float4* vin, bool resolve, unsigned* status,
                              cudaStream_t st) {
    if (L == 8)
        launch_k(k_search_xsph_split<B, 8>, g, bs, st, xs, sx, sy, sz, first, c, n, nbr, cnt, v,
                 v_out, vin, resolve, status);
    else if (L == 4)
        launch_k(k_search_xsph_split<B, 4>, g, bs, st, xs, sx, sy, sz, first, c, n, nbr, cnt, v,
                 v_out, vin, resolve, status);
    else
        launch_k(k_search_xsph_split<B, 2>, g, bs, st, xs, sx, sy, sz, first, c, n, nbr, cnt, v,
                 v_out, vin, resolve, status);
}

void launch_search_xsph(const float4* xs, const float* sx, const float* sy, const float* sz,
                        const int* first, const StepConst& c, int n, uint32_t* nbr, int* cnt,
                        const float4* v, float4* v_out, const float4* vin, bool resolve,
                        unsigned* status, cudaStream_t st) {
    const int bs = tuned_block(c, kTunedSearch);
    if (const int L = split_lanes(c, n); L > 1) {
        const unsigned g = blocks_for(static_cast<size_t>(n) * L, bs);
        if (c.scenes)
            launch_search_xsph_split<true>(L, g, bs, xs, sx, sy, sz, first, c, n, nbr, cnt, v,
                                           v_out, vin, resolve, status, st);
        else
            launch_search_xsph_split<false>(L, g, bs, xs, sx, sy, sz, first, c, n, nbr, cnt, v,
                                            v_out, vin, resolve, status, st);
        return;
    }
    const unsigned g = blocks_for(n, bs);
    if (c.scenes)
        launch_k(k_search_xsph<true>, g, bs, st, xs, sx, sy, sz, first, c, n, nbr, cnt, v, v_out,
                 vin, resolve, status);
    else
        launch_k(k_search_xsph<false>, g, bs, st, xs, sx, sy, sz, first, c, n, nbr, cnt, v, v_out,
                 vin, resolve, status);
}

void launch_count(const float4* xs, const float* sx, const float* sy, const float* sz,
                  const int* first, const StepConst& c, int n, int* cnt, unsigned* status,
                  cudaStream_t st) {
    const int bs = tuned_block(c, kTunedSearch);
    const unsigned g = blocks_for(n, bs);
    if (c.scenes)
        launch_k(k_count<true>, g, bs, st, xs, sx, sy, sz, first, c, n, cnt, status);
    else
        launch_k(k_count<false>, g, bs, st, xs, sx, sy, sz, first, c, n, cnt, status);
}

size_t nb_scan_scratch_words(size_t n) {
    const size_t tiles = (n + kScanTile - 1) / kScanTile;
    return 2 * (tiles + 1);  // 64-bit tile sums and the total
}

void launch_nb_scan(const int* cnt, uint32_t* off, size_t cap, int n, uint32_t* scratch,
                    unsigned* status, cudaStream_t st) {
    const int tiles = static_cast<int>((static_cast<size_t>(n) + kScanTile - 1) / kScanTile);
    auto* sums = reinterpret_cast<unsigned long long*>(scratch);
    launch_k(k_nb_scan_tiles, static_cast<unsigned>(std::max(tiles, 1)), kScanThreads, st, cnt,
             n, off, sums, status);
    launch_k(k_nb_scan_sums, 1u, kScanThreads, st, sums, tiles, status);
    launch_k(k_nb_scan_add, blocks_for(std::max(n, 1), kScanThreads), kScanThreads, st, n, cap,
             sums, tiles, off, status);
}

template <bool B>
void launch_delta_apply_b(const float4* xs, const uint32_t* nbr, const int* cnt, const float* lam,
                          const StepConst& c, int n, float4* xs_out, uint32_t* keys_out,
                          uint8_t* moved, float4* pre, unsigned* status, cudaStream_t st) {
    const int bs = tuned_block(c, kTunedDelta);
    const unsigned g = blocks_for(n, bs);
    const int L = split_lanes(c, n);
    const unsigned gl = blocks_for(static_cast<size_t>(n) * L, bs);
#define PBF_DELTA_CASE(N)                                                                        \
    if (L == 8)                                                                                  \
        launch_k(k_delta_apply<N, B, 8>, gl, bs, st, xs, nbr, cnt, lam, c, n, xs_out, keys_out,  \
                 moved, pre, status);                                                            \
    else if (L == 4)                                                                             \
        launch_k(k_delta_apply<N, B, 4>, gl, bs, st, xs, nbr, cnt, lam, c, n, xs_out, keys_out,  \
                 moved, pre, status);                                                            \
    else if (L == 2)                                                                             \
        launch_k(k_delta_apply<N, B, 2>, gl, bs, st, xs, nbr, cnt, lam, c, n, xs_out, keys_out,  \
                 moved, pre, status);                                                            \
    else                                                                                         \
        launch_k(k_delta_apply<N, B, 1>, g, bs, st, xs, nbr, cnt, lam, c, n, xs_out, keys_out,   \
                 moved, pre, status)
    switch (c.sc.k != 0.0f ? c.sc.n : 0) {
        case 1: PBF_DELTA_CASE(1); break;
        case 2: PBF_DELTA_CASE(2); break;
        case 3: PBF_DELTA_CASE(3); break;
        case 4: PBF_DELTA_CASE(4); break;
        default: PBF_DELTA_CASE(0); break;
    }
#undef PBF_DELTA_CASE
}
void launch_delta_apply(const float4* xs, const uint32_t* nbr, const int* cnt, const float* lam,
                        const StepConst& c, int n, float4* xs_out, uint32_t* keys_out,
                        unsigned* status, cudaStream_t st, uint8_t* moved, float4* pre) {
    if (c.scenes)
        launch_delta_apply_b<true>(xs, nbr, cnt, lam, c, n, xs_out, keys_out, moved, pre, status,
                                   st);
    else
        launch_delta_apply_b<false>(xs, nbr, cnt, lam, c, n, xs_out, keys_out, moved, pre, status,
                                    st);
}
void launch_finalize(const uint32_t* org, const float4* x_old, const float4* vin_old,
                     const float4* v_old, const uint32_t* id_old, const float4* xs, int n,
                     const StepConst& c, float4* v_new, float4* vin_new, uint32_t* id_new,
                     const unsigned* status, cudaStream_t st) {
    launch_k(k_finalize, blocks_for(n), kBlock, st, org, x_old, vin_old, v_old, id_old, xs, n, c,
             v_new, vin_new, id_new, status);
}
void launch_xsph(const float4* x, const float4* v, const uint32_t* nbr, const int* cnt,
                 const StepConst& c, int n, float4* v_out, const float4* vin, bool resolve,
                 const unsigned* status, cudaStream_t st) {
    const int bs = tuned_block(c, kTunedXsph);
    if (c.scenes)
        launch_k(k_xsph<true>, blocks_for(n, bs), bs, st, x, v, nbr, cnt, c, n, v_out, vin,
                 resolve, status);
    else
        launch_k(k_xsph<false>, blocks_for(n, bs), bs, st, x, v, nbr, cnt, c, n, v_out, vin,
                 resolve, status);
}
void launch_vorticity(const float4* x, const float4* v, const uint32_t* nbr, const int* cnt,
                      const StepConst& c, int n, float4* omega, bool store_norm,
                      const unsigned* status, cudaStream_t st) {
    const int bs = tuned_block(c, kTunedVorticity);
    const int L = split_lanes(c, n);
    const unsigned gl = blocks_for(static_cast<size_t>(n) * L, bs);
    if (L == 8)
        launch_k(k_vorticity_group<8>, gl, bs, st, x, v, nbr, cnt, c, n, omega, store_norm,
                 status);
    else if (L == 4)
        launch_k(k_vorticity_group<4>, gl, bs, st, x, v, nbr, cnt, c, n, omega, store_norm,
                 status);
    else if (L == 2)
        launch_k(k_vorticity_group<2>, gl, bs, st, x, v, nbr, cnt, c, n, omega, store_norm,
                 status);
    else
        launch_k(k_vorticity, blocks_for(n, bs), bs, st, x, v, nbr, cnt, c, n, omega, store_norm,
                 status);
}
void launch_omega_norm(float4* omega, int n, cudaStream_t st) {
    launch_k(k_omega_norm, blocks_for(n), kBlock, st, omega, n);
}
void launch_confine(const float4* x, const uint32_t* nbr, const int* cnt, const float4* omega,
                    const float4* v, const StepConst& c, int n, float4* v_out,
                    const float4* vin, bool resolve, const unsigned* status, cudaStream_t st) {
    const int bs = tuned_block(c, kTunedConfine);
    if (c.scenes)
        launch_k(k_confine<true>, blocks_for(n, bs), bs, st, x, nbr, cnt, omega, v, c, n, v_out,
                 vin, resolve, status);
    else
        launch_k(k_confine<false>, blocks_for(n, bs), bs, st, x, nbr, cnt, omega, v, c, n,
                 v_out, vin, resolve, status);
}
void launch_resolve(const float4* x, const float4* vin, float4* v, const StepConst& c, int n,
                    const unsigned* status, cudaStream_t st) {
    if (c.scenes)
        launch_k(k_resolve<true>, blocks_for(n), kBlock, st, x, vin, v, c, n, status);
    else
        launch_k(k_resolve<false>, blocks_for(n), kBlock, st, x, vin, v, c, n, status);
}
void launch_scatter_by_id(const float4* vals, const uint32_t* id, float4* out, int n,
                          cudaStream_t st) {
    k_scatter_by_id<<<blocks_for(n), kBlock, 0, st>>>(vals, id, out, n);
}
void launch_iota(uint32_t* a, int n, cudaStream_t st) {
    k_iota<<<blocks_for(n), kBlock, 0, st>>>(a, n);
}
void launch_density(const float4* x, const uint32_t* nbr, const int* cnt, const StepConst& c,
                    int n, float* err, cudaStream_t st) {
    k_density<<<blocks_for(n), kBlock, 0, st>>>(x, nbr, cnt, c, n, err);
}
void launch_grid_keys(const float4* pos, uint32_t* keys, int n, const GridConst& g,
                      cudaStream_t st) {
    k_grid_keys<<<blocks_for(n), kBlock, 0, st>>>(pos, keys, n, g);
}
void launch_lambda_list(const float4* xs, const uint32_t* nbr, const int* cnt,
                        const StepConst& c, int n, float* lam, cudaStream_t st) {
    k_lambda_list<<<blocks_for(n), kBlock, 0, st>>>(xs, nbr, cnt, c, n, lam);
}
void launch_delta_list(const float4* xs, const uint32_t* nbr, const int* cnt, const float* lam,
                       const StepConst& c, int n, float4* delta, cudaStream_t st) {
    k_delta_list<<<blocks_for(n), kBlock, 0, st>>>(xs, nbr, cnt, lam, c, n, delta);
}
void launch_collide(float4* pos, int n, const StepConst& c, int kind, unsigned* flag,
                    cudaStream_t st) {
    k_collide<<<blocks_for(n), kBlock, 0, st>>>(pos, n, c, kind, flag);
}
void launch_integrate(const float4* x, float4* xs, float4* v, int n, const StepConst& c,
                      cudaStream_t st) {
    k_integrate<<<blocks_for(n), kBlock, 0, st>>>(x, xs, v, n, c);
}

}  // namespace pbf
