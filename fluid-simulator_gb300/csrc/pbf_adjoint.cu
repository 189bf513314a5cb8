// pbf_adjoint.cu -- reverse-mode derivative of the PBF step: gradients of a
// loss on the final particle state with respect to the initial positions and
// velocities, the rest density and the XSPH strength.
//
// Differentiated step (one substep; container walls only; no vorticity
// confinement):
//   integrate   v1 = v + g dt, p0 = x + v1 dt               (integration.cu:6-32)
//   I times     lambda_i = -C_i / (gs^2 (S2_i + |G_i|^2) + eps),
//               q = p + gs sum_j (lambda_i + lambda_j + s_corr) grad W_ij,
//               p' = container clamp of q
//               (pbf_solver_kernels.cu:26-193, collision_kernels.cu:47-82)
//   velocity    v2 = (p_I - x) / dt                         (pbf_solver_kernels.cu:195-211)
//   XSPH        v3 = v2 + c sum_j (v2_j - v2_i) W_ij        (pbf_solver_kernels.cu:213-266)
//   response    v4 = wall contacts against v1 (restitution, friction)
//               (collision_kernels.cu:236-276)
// gs = m / rho0, C_i = rho_i / rho0 - 1, rho_i = m (W(0) + sum_j W_ij),
// G_i = sum_j grad W_ij, S2_i = sum_j |grad W_ij|^2.
//
// The neighbour lists of every iteration are recorded (integer data, not
// differentiated) in particle-id order, built by the solver's own grid, sort
// and search kernels; clamps and contact decisions are recorded the same way.
// A list holds j iff it holds i for j (d2 is computed bit-identically from
// both sides), and grad W is odd while its Hessian is even, so every
// transposed (scatter) term of the adjoint is evaluated as a gather over the
// particle's own list: no atomics, a deterministic result.
//
// Checkpointing: the forward keeps (x, v) every K steps; the backward
// recomputes each K-step segment from its checkpoint into a tape and runs the
// segment's adjoint in reverse.
#include "pbf_common.h"
#include "pbf_kernels.cuh"

#include <algorithm>
#include <array>
#include <cmath>
#include <limits>
#include <string>
#include <vector>

namespace pbf {
namespace adj {

__device__ __forceinline__ float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) {
    return make_float3(a.x + b.x, a.y + b.y, a.z + b.z);
}
__device__ __forceinline__ float3 operator-(float3 a, float3 b) {
    return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
__device__ __forceinline__ float3 operator*(float s, float3 a) {
    return make_float3(s * a.x, s * a.y, s * a.z);
}
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Analytic derivatives used by the adjoint.  With rr = |r|:
//   spiky gradient g(r) = f(rr) r,  f = c_spiky (1 - rr/h)^2 / rr
//   Hessian        H u = f u + (f'(rr) / rr) (r . u) r
//   poly6 gradient grad W = -6 c_poly6 t^2 / h^2 r,  t = 1 - |r|^2 / h^2
//   s_corr'        ds/d(d2) = 3 k n ratio^(3n-1) / (h^2 - dq^2)
struct PairTerms {
    float3 g;      // spiky gradient (the forward's rounding: spiky())
    float f, fpr;  // f and f'(rr) / rr
    float w;       // poly6
    float3 gw;     // poly6 gradient
    float s, sp;   // s_corr and ds/d(d2)
};

__device__ __forceinline__ PairTerms pair_terms(const StepConst& c, float3 r) {
    PairTerms t;
    const float d2 = dist2(r.x, r.y, r.z);
    spiky(c.k, r.x, r.y, r.z, d2, t.g.x, t.g.y, t.g.z);
    t.w = poly6(c.k, d2);
    t.s = scorr<0>(c.sc, d2);
    t.f = 0.0f;
    t.fpr = 0.0f;
    t.sp = 0.0f;
    t.gw = make_float3(0.0f, 0.0f, 0.0f);
    if (d2 < c.k.h2) {
        const float tp = 1.0f - d2 * c.k.inv_h2;
        t.gw = (-6.0f * c.k.c_poly6 * tp * tp * c.k.inv_h2) * r;
        if (d2 >= kSpikyMinD2) {
            const float rr = sqrtf(d2);
            const float u = 1.0f - rr * c.k.inv_h;
            t.f = c.k.c_spiky * u * u / rr;
            const float fp = -c.k.c_spiky * u / rr * (2.0f * c.k.inv_h + u / rr);
            t.fpr = fp / rr;
        }
        if (c.sc.k != 0.0f && c.sc.n > 0 && c.sc.dq2 < c.sc.h2) {
            const float ratio = (c.sc.h2 - d2) * c.sc.inv_den;
            t.sp = 3.0f * c.sc.k * static_cast<float>(c.sc.n) *
                   powf(ratio, 3.0f * static_cast<float>(c.sc.n) - 1.0f) * c.sc.inv_den;
        }
    }
    return t;
}
__device__ __forceinline__ float3 hess(const PairTerms& t, float3 r, float3 u) {
    return t.f * u + (t.fpr * dot3(r, u)) * r;
}

// ---- taped forward (particle-id order) -------------------------------------

__global__ void k_integrate(const float4* __restrict__ x, const float4* __restrict__ v,
                            StepConst c, int n, float4* __restrict__ v1, float4* __restrict__ p0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 vv = v[i];
    const float4 p = x[i];
    vv.x = ffma(c.gravx, c.dt, vv.x);
    vv.y = ffma(c.gravy, c.dt, vv.y);
    vv.z = ffma(c.gravz, c.dt, vv.z);
    v1[i] = vv;
    p0[i] = make_float4(ffma(vv.x, c.dt, p.x), ffma(vv.y, c.dt, p.y), ffma(vv.z, c.dt, p.z), p.w);
}

// Lists found in sorted order, rewritten in particle-id order.
__global__ void k_map_lists(const uint32_t* __restrict__ perm, const uint32_t* __restrict__ nbr_s,
                            const int* __restrict__ cnt_s, int n, size_t stride, int max_nb,
                            uint32_t* __restrict__ nbr, int* __restrict__ cnt) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    // After a failed search (status set, kernels returned early) perm and
    // the lists may hold stale data: only ids below n are ever written.
    const uint32_t o = perm[s];
    if (o >= static_cast<uint32_t>(n)) return;
    const int k = max(0, cnt_s[s]);
    cnt[o] = k;
    const int m = min(k, max_nb);
    for (int q = 0; q < m; ++q) {
        const uint32_t j = nbr_s[static_cast<size_t>(q) * stride + s];
        const uint32_t id = j < static_cast<uint32_t>(n) ? perm[j] : o;
        nbr[static_cast<size_t>(q) * stride + o] = id < static_cast<uint32_t>(n) ? id : o;
    }
}

// computeLambda over a recorded list (the solver's lambda arithmetic).
__global__ void k_lambda(const float4* __restrict__ p, const uint32_t* __restrict__ nbr,
                         const int* __restrict__ cnt, StepConst c, int n, float* __restrict__ lam) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 pi = p[i];
    const int count = min(cnt[i], c.max_nb);
    float wsum = c.k.c_poly6, s2 = 0.0f, gx = 0.0f, gy = 0.0f, gz = 0.0f;
    for (int k = 0; k < count; ++k) {
        const float4 pj = __ldg(&p[__ldg(&nbr[static_cast<size_t>(k) * c.stride + i])]);
        const float dx = fsub(pi.x, pj.x), dy = fsub(pi.y, pj.y), dz = fsub(pi.z, pj.z);
        const float d2 = dist2(dx, dy, dz);
        wsum = fadd(wsum, poly6(c.k, d2));
        float ax, ay, az;
        spiky(c.k, dx, dy, dz, d2, ax, ay, az);
        s2 = ffma(az, az, ffma(ay, ay, ffma(ax, ax, s2)));
        gx = fadd(gx, ax);
        gy = fadd(gy, ay);
        gz = fadd(gz, az);
    }
    const float rho = fmul(c.mass, wsum);
    const float denom = ffma(c.gs2, fadd(s2, dist2(gx, gy, gz)), c.lambda_eps);
    lam[i] = fdiv(-fsub(fdiv(rho, c.rho0), 1.0f), denom);
}

// delta p + apply + container clamp; q (before the clamp) is recorded.
__global__ void k_delta(const float4* __restrict__ p, const float* __restrict__ lam,
                        const uint32_t* __restrict__ nbr, const int* __restrict__ cnt, StepConst c,
                        int n, float4* __restrict__ q_out, float4* __restrict__ p_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 pi = p[i];
    const float li = lam[i];
    const int count = min(cnt[i], c.max_nb);
    float ax = 0.0f, ay = 0.0f, az = 0.0f;
    for (int k = 0; k < count; ++k) {
        const uint32_t j = __ldg(&nbr[static_cast<size_t>(k) * c.stride + i]);
        const float4 pj = __ldg(&p[j]);
        const float dx = fsub(pi.x, pj.x), dy = fsub(pi.y, pj.y), dz = fsub(pi.z, pj.z);
        const float d2 = dist2(dx, dy, dz);
        float gx, gy, gz;
        spiky(c.k, dx, dy, dz, d2, gx, gy, gz);
        const float ls = fadd(fadd(li, __ldg(&lam[j])), scorr<0>(c.sc, d2));
        ax = ffma(ls, gx, ax);
        ay = ffma(ls, gy, ay);
        az = ffma(ls, gz, az);
    }
    float qx = fadd(pi.x, fmul(c.gs, ax)), qy = fadd(pi.y, fmul(c.gs, ay)),
          qz = fadd(pi.z, fmul(c.gs, az));
    q_out[i] = make_float4(qx, qy, qz, pi.w);
    project_container(c.col, c.particle_radius, qx, qy, qz);
    p_out[i] = make_float4(qx, qy, qz, pi.w);
}

__global__ void k_velocity(const float4* __restrict__ pI, const float4* __restrict__ x,
                           const float4* __restrict__ v1, StepConst c, int n,
                           float4* __restrict__ v2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 q = pI[i], xo = x[i];
    v2[i] = make_float4(fmul(fsub(q.x, xo.x), c.inv_dt), fmul(fsub(q.y, xo.y), c.inv_dt),
                        fmul(fsub(q.z, xo.z), c.inv_dt), v1[i].w);
}

__global__ void k_xsph(const float4* __restrict__ pI, const float4* __restrict__ v2,
                       const uint32_t* __restrict__ nbr, const int* __restrict__ cnt, StepConst c,
                       int n, float4* __restrict__ v3) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 pi = pI[i], vi = v2[i];
    const int count = min(cnt[i], c.max_nb);
    float cx = 0.0f, cy = 0.0f, cz = 0.0f;
    for (int k = 0; k < count; ++k) {
        const uint32_t j = __ldg(&nbr[static_cast<size_t>(k) * c.stride + i]);
        const float4 pj = __ldg(&pI[j]), vj = __ldg(&v2[j]);
        const float w = poly6(c.k, dist2(fsub(pi.x, pj.x), fsub(pi.y, pj.y), fsub(pi.z, pj.z)));
        cx = ffma(fsub(vj.x, vi.x), w, cx);
        cy = ffma(fsub(vj.y, vi.y), w, cy);
        cz = ffma(fsub(vj.z, vi.z), w, cz);
    }
    v3[i] = make_float4(ffma(c.xsph_c, cx, vi.x), ffma(c.xsph_c, cy, vi.y),
                        ffma(c.xsph_c, cz, vi.z), vi.w);
}

__global__ void k_respond(const float4* __restrict__ pI, const float4* __restrict__ v1,
                          const float4* __restrict__ v3, StepConst c, int n,
                          float4* __restrict__ v4, float4* __restrict__ x_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = v3[i];
    const float4 p = pI[i];
    resolve_velocity(c.col, c.particle_radius, c.restitution, c.friction, p, v1[i], v);
    v4[i] = v;
    x_out[i] = p;
}

// ---- adjoint -----------------------------------------------------------------

// Container contacts of one particle in the forward's order: up to three
// walls, each an axis and a normal sign; `active` as resolveContactVelocity
// decides it for the velocity reaching that wall.
struct Walls {
    int m;
    int axis[3];
    float sign[3];
    bool active[3];
};

__device__ __forceinline__ float comp(float4 v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

__device__ __forceinline__ Walls replay_walls(const StepConst& c, float4 p, float4 vin, float4 v) {
    Walls w;
    w.m = 0;
    const float r = c.particle_radius, eps = kContactEpsilon;
    const float ts = fsub(1.0f, c.friction);
    const float minX = fadd(c.col.cminx, r), maxX = fsub(c.col.cmaxx, r);
    const float minY = fadd(c.col.cminy, r);
    const float minZ = fadd(c.col.cminz, r), maxZ = fsub(c.col.cmaxz, r);
    auto wall = [&](int a, float s) {
        const float nx = a == 0 ? s : 0.0f, ny = a == 1 ? s : 0.0f, nz = a == 2 ? s : 0.0f;
        const float vn = ffma(v.z, nz, ffma(v.y, ny, fmul(v.x, nx)));
        const float vinn = ffma(vin.z, nz, ffma(vin.y, ny, fmul(vin.x, nx)));
        const float target = vinn < 0.0f ? fmul(-c.restitution, vinn) : 0.0f;
        w.axis[w.m] = a;
        w.sign[w.m] = s;
        w.active[w.m] = !(vn > target || (vn == target && vinn >= 0.0f));
        ++w.m;
        contact(nx, ny, nz, vin, c.restitution, ts, v);
    };
    if (p.x <= fadd(minX, eps)) wall(0, 1.0f);
    else if (p.x >= fsub(maxX, eps)) wall(0, -1.0f);
    if (p.y <= fadd(minY, eps)) wall(1, 1.0f);
    if (p.z <= fadd(minZ, eps)) wall(2, 1.0f);
    else if (p.z >= fsub(maxZ, eps)) wall(2, -1.0f);
    return w;
}

// gv4 -> gv3 (velocity before the contacts) and gv1 (incoming velocity).
__global__ void k_respond_adj(const float4* __restrict__ pI, const float4* __restrict__ v1,
                              const float4* __restrict__ v3, const float4* __restrict__ gv4,
                              StepConst c, int n, float4* __restrict__ gv3,
                              float4* __restrict__ gv1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 vin = v1[i];
    const Walls w = replay_walls(c, pI[i], vin, v3[i]);
    float g[3] = {gv4[i].x, gv4[i].y, gv4[i].z};
    float gin[3] = {0.0f, 0.0f, 0.0f};
    const float ts = 1.0f - c.friction;
    for (int k = w.m - 1; k >= 0; --k) {
        if (!w.active[k]) continue;
        const int a = w.axis[k];
        // v'_a = -e vin_a when the incoming normal speed is negative, else 0;
        // v'_b = (1 - friction) v_b for the other axes.
        if (w.sign[k] * comp(vin, a) < 0.0f) gin[a] += -c.restitution * g[a];
        g[a] = 0.0f;
        for (int b = 0; b < 3; ++b)
            if (b != a) g[b] *= ts;
    }
    gv3[i] = make_float4(g[0], g[1], g[2], 0.0f);
    gv1[i] = make_float4(gin[0], gin[1], gin[2], 0.0f);
}

// XSPH and velocity-update adjoint, plus the clamp of the last iteration:
//   gv2_i = gv3_i + c sum_j (gv3_j - gv3_i) W_ij
//   gp_I  = gx'_i + gv2_i / dt + c sum_j ((gv3_i - gv3_j).(v2_j - v2_i)) grad W_ij
//   gxs_i = -gv2_i / dt                       (x enters v2)
//   dL/dc += gv3_i . sum_j (v2_j - v2_i) W_ij
//   gq_{I-1} = gp_I where the clamp left q unchanged, 0 elsewhere.
__global__ void k_xsph_adj(const float4* __restrict__ pI, const float4* __restrict__ v2,
                           const float4* __restrict__ gv3, const uint32_t* __restrict__ nbr,
                           const int* __restrict__ cnt, const float4* __restrict__ gx_next,
                           const float4* __restrict__ q_last, StepConst c, int n,
                           float4* __restrict__ gxs, float4* __restrict__ gq,
                           double* __restrict__ acc_c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 pi4 = pI[i];
    const float3 pi = f3(pi4), vi = f3(v2[i]), gi = f3(gv3[i]);
    const int count = min(cnt[i], c.max_nb);
    float3 sg = make_float3(0.0f, 0.0f, 0.0f), sv = sg, pos = sg;
    for (int k = 0; k < count; ++k) {
        const uint32_t j = __ldg(&nbr[static_cast<size_t>(k) * c.stride + i]);
        const float3 r = pi - f3(__ldg(&pI[j]));
        const PairTerms t = pair_terms(c, r);
        const float3 dv = f3(__ldg(&v2[j])) - vi;
        const float3 gj = f3(__ldg(&gv3[j]));
        sg = sg + t.w * (gj - gi);
        sv = sv + t.w * dv;
        pos = pos + dot3(gi - gj, dv) * t.gw;
    }
    const float3 gv2 = gi + c.xsph_c * sg;
    acc_c[i] += static_cast<double>(dot3(gi, sv));
    const float3 gp = f3(gx_next[i]) + c.inv_dt * gv2 + c.xsph_c * pos;
    gxs[i] = make_float4(-c.inv_dt * gv2.x, -c.inv_dt * gv2.y, -c.inv_dt * gv2.z, 0.0f);
    const float4 q = q_last[i];
    gq[i] = make_float4(q.x == pi4.x ? gp.x : 0.0f, q.y == pi4.y ? gp.y : 0.0f,
                        q.z == pi4.z ? gp.z : 0.0f, 0.0f);
}

// First gather pass of one iteration's adjoint (u_ij = gq_i - gq_j):
//   glam_i = gs sum_j u_ij . g_ij
//   gpart_i = gq_i + gs sum_j [(lam_i + lam_j + s_ij) H_ij u_ij + 2 s'_ij (u_ij . g_ij) r_ij]
// and the per-particle terms of the lambda adjoint: C_i, D_i recomputed,
//   gC_i = -glam_i / D_i, gD_i = glam_i C_i / D_i^2, a_i = m gC_i / rho0,
// with the rest-density partial gC_i (-rho_i / rho0^2) + g_gs_i (-m / rho0^2),
// g_gs_i = gq_i . X_i + 2 gs gD_i (S2_i + |G_i|^2), X_i = delta p_i / gs.
__global__ void k_iter_adj_a(const float4* __restrict__ p, const float* __restrict__ lam,
                             const float4* __restrict__ gq, const uint32_t* __restrict__ nbr,
                             const int* __restrict__ cnt, StepConst c, int n,
                             float4* __restrict__ gpart, float4* __restrict__ aux,
                             float* __restrict__ aa, double* __restrict__ acc_rho0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 pi = f3(p[i]), gqi = f3(gq[i]);
    const float li = lam[i];
    const int count = min(cnt[i], c.max_nb);
    float wsum = c.k.c_poly6, s2 = 0.0f, glam = 0.0f;
    float3 G = make_float3(0.0f, 0.0f, 0.0f), X = G, dpos = G;
    for (int k = 0; k < count; ++k) {
        const uint32_t j = __ldg(&nbr[static_cast<size_t>(k) * c.stride + i]);
        const float3 r = pi - f3(__ldg(&p[j]));
        const PairTerms t = pair_terms(c, r);
        const float3 u = gqi - f3(__ldg(&gq[j]));
        const float coef = li + __ldg(&lam[j]) + t.s;
        wsum += t.w;
        s2 += dot3(t.g, t.g);
        G = G + t.g;
        X = X + coef * t.g;
        const float ug = dot3(u, t.g);
        glam += ug;
        dpos = dpos + coef * hess(t, r, u) + (2.0f * t.sp * ug) * r;
    }
    const float rho = c.mass * wsum;
    const float S = s2 + dot3(G, G);
    const float D = c.gs2 * S + c.lambda_eps;
    const float C = rho / c.rho0 - 1.0f;
    const float gl = c.gs * glam;
    const float gC = -gl / D;
    const float gD = gl * C / (D * D);
    gpart[i] = make_float4(gqi.x + c.gs * dpos.x, gqi.y + c.gs * dpos.y, gqi.z + c.gs * dpos.z,
                           0.0f);
    aux[i] = make_float4(G.x, G.y, G.z, gD);
    aa[i] = c.mass * gC / c.rho0;
    const float ggs = dot3(gqi, X) + 2.0f * c.gs * gD * S;
    const double r2 = static_cast<double>(c.rho0) * c.rho0;
    acc_rho0[i] += -static_cast<double>(gC) * rho / r2 - static_cast<double>(ggs) * c.mass / r2;
}

// Second gather pass: the lambda adjoint's position terms,
//   gp_i = gpart_i + sum_j [(a_i + a_j) gradW_ij
//                         + 2 gs^2 H_ij ((gD_i + gD_j) g_ij + gD_i G_i - gD_j G_j)],
// then either the clamp of the previous iteration (gq_{k-1}) or, after the
// first iteration, the integration adjoint (gx_t, gv_t).
__global__ void k_iter_adj_b(const float4* __restrict__ p, const float4* __restrict__ aux,
                             const float* __restrict__ aa, const uint32_t* __restrict__ nbr,
                             const int* __restrict__ cnt, const float4* __restrict__ gpart,
                             const float4* __restrict__ q_prev, const float4* __restrict__ gxs,
                             const float4* __restrict__ gv1, StepConst c, int n,
                             float4* __restrict__ gq_prev, float4* __restrict__ gx_t,
                             float4* __restrict__ gv_t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 pi4 = p[i];
    const float3 pi = f3(pi4);
    const float4 ai4 = aux[i];
    const float3 Gi = f3(ai4);
    const float gDi = ai4.w, ai = aa[i];
    const int count = min(cnt[i], c.max_nb);
    float3 acc = make_float3(0.0f, 0.0f, 0.0f);
    for (int k = 0; k < count; ++k) {
        const uint32_t j = __ldg(&nbr[static_cast<size_t>(k) * c.stride + i]);
        const float3 r = pi - f3(__ldg(&p[j]));
        const PairTerms t = pair_terms(c, r);
        const float4 aj4 = __ldg(&aux[j]);
        const float gDj = aj4.w;
        const float3 w = (gDi + gDj) * t.g + gDi * Gi - gDj * f3(aj4);
        acc = acc + (ai + __ldg(&aa[j])) * t.gw + (2.0f * c.gs2) * hess(t, r, w);
    }
    const float3 gp = f3(gpart[i]) + acc;
    if (q_prev) {
        const float4 q = q_prev[i];
        gq_prev[i] = make_float4(q.x == pi4.x ? gp.x : 0.0f, q.y == pi4.y ? gp.y : 0.0f,
                                 q.z == pi4.z ? gp.z : 0.0f, 0.0f);
    } else {
        // p0 = x + v1 dt, v1 = v + g dt.
        const float4 gs = gxs[i], g1 = gv1[i];
        gx_t[i] = make_float4(gs.x + gp.x, gs.y + gp.y, gs.z + gp.z, 0.0f);
        gv_t[i] = make_float4(g1.x + c.dt * gp.x, g1.y + c.dt * gp.y, g1.z + c.dt * gp.z, 0.0f);
    }
}

constexpr int kB = 256;
inline unsigned grid(int n) { return static_cast<unsigned>((n + kB - 1) / kB); }

}  // namespace adj
}  // namespace pbf

using namespace pbf;

struct pbf_adjoint {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;

    size_t n = 0, stride = 0;
    int max_nb = 128, every = 10, iters = 0;
    int steps_done = 0;
    pbf_params prm{};
    uint64_t cells = 0;
    StepConst c{};
    SortPlan plan{};

    // Neighbour-list builder (sorted order) and its scratch.
    DeviceBuffer keys, skeys, sidx, akeys, aidx, first, xsorted, org, soa, nbr_s, cnt_s, scratch,
        status;
    // Checkpoints (x, v) every `every` steps.
    DeviceBuffer ckpt;
    // Tape of one segment: per step kF4 float4 arrays, I lambdas, I + 1 lists.
    DeviceBuffer tape4, tapel, tapen, tapec;
    // Work arrays.
    DeviceBuffer xa, va, xb, vb, gx, gv, gxs, gv1, gv3, gq0, gq1, gpart, aux, aa, acc_r, acc_c;

    ~pbf_adjoint() {
        if (stream) cudaStreamDestroy(stream);
    }

    int f4_slots() const { return 2 * iters + 5; }
    size_t soa_stride() const { return (n + 1 + 63) / 64 * 64; }
    // Tape slots of step t: 0 x, 1 v1, 2 + k p_k (k = 0..I), 3 + I + k q_k
    // (k < I), 3 + 2I v2, 4 + 2I v3.
    float4* T(int t, int slot) {
        return tape4.as<float4>() + (static_cast<size_t>(t) * f4_slots() + slot) * n;
    }
    float* L(int t, int k) { return tapel.as<float>() + (static_cast<size_t>(t) * iters + k) * n; }
    uint32_t* NB(int t, int k) {
        return tapen.as<uint32_t>() + (static_cast<size_t>(t) * (iters + 1) + k) * stride * max_nb;
    }
    int* CN(int t, int k) { return tapec.as<int>() + (static_cast<size_t>(t) * (iters + 1) + k) * n; }

    void initialize(size_t count, pbf_float3 lo, pbf_float3 hi, const pbf_params& p, int maxnb,
                    int ckpt_every) {
        if (count == 0) fail(PBF_ERR_INVALID_ARGUMENT, "particle count must be greater than zero");
        if (count > static_cast<size_t>(std::numeric_limits<int>::max()))
            fail(PBF_ERR_LENGTH, "Particle count exceeds CUDA kernel index range");
        if (maxnb <= 0) fail(PBF_ERR_INVALID_ARGUMENT, "maxNeighbors must be greater than zero");
        if (ckpt_every <= 0) fail(PBF_ERR_INVALID_ARGUMENT, "checkpoint interval must be positive");
        if (p.substeps != 1) fail(PBF_ERR_INVALID_ARGUMENT, "the adjoint takes one substep per step");
        if (p.vorticityStrength != 0.0f)
            fail(PBF_ERR_INVALID_ARGUMENT,
                 "the adjoint covers integration, the density constraint, container contacts "
                 "and XSPH; vorticityStrength must be 0");
        validate_params(p);
        const double width = double(hi.x) - double(lo.x);
        const double depth = double(hi.z) - double(lo.z);
        if (width < 2.0 * double(p.particleRadius) || depth < 2.0 * double(p.particleRadius))
            fail(PBF_ERR_INVALID_ARGUMENT, "Particle diameter exceeds closed container dimensions");
        const std::array<int, 3> d = grid_dims_checked(lo, hi, p.smoothingRadius);
        cuda_check(cudaSetDevice(device));
        if (!stream) cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        n = count;
        max_nb = maxnb;
        every = ckpt_every;
        iters = p.solverIterations;
        prm = p;
        stride = (n + 255) / 256 * 256;
        cells = uint64_t(d[0]) * uint64_t(d[1]) * uint64_t(d[2]);
        plan = make_sort_plan(static_cast<int>(n), cells);

        c = StepConst{};
        const float h = p.smoothingRadius;
        c.k = make_kernel_const(h);
        c.sc = make_scorr_const(h, p.scorrK, p.scorrN, p.scorrDeltaQ);
        c.g.minx = lo.x;
        c.g.miny = lo.y;
        c.g.minz = lo.z;
        c.g.cell = h;
        c.g.gx = d[0];
        c.g.gy = d[1];
        c.g.gz = d[2];
        c.g.radius = 1;
        c.mass = p.particleMass;
        c.rho0 = p.restDensity;
        c.lambda_eps = p.lambdaEpsilon;
        c.gs = p.particleMass / p.restDensity;
        c.gs2 = c.gs * c.gs;
        c.dt = p.dt;
        c.inv_dt = 1.0f / c.dt;
        c.gravx = p.gravity.x;
        c.gravy = p.gravity.y;
        c.gravz = p.gravity.z;
        c.particle_radius = p.particleRadius;
        c.restitution = p.collisionRestitution;
        c.friction = p.collisionFriction;
        c.xsph_c = p.xsphViscosity;
        c.vort_eps = 0.0f;
        c.max_nb = max_nb;
        c.stride = stride;
        c.col.cminx = lo.x;
        c.col.cminy = lo.y;
        c.col.cminz = lo.z;
        c.col.cmaxx = hi.x;
        c.col.cmaxy = hi.y;
        c.col.cmaxz = hi.z;

        const size_t f4b = n * sizeof(float4), u4b = n * sizeof(uint32_t);
        keys.allocate(u4b);
        skeys.allocate(u4b);
        sidx.allocate(u4b);
        akeys.allocate(u4b);
        aidx.allocate(u4b);
        org.allocate(u4b);
        first.allocate((cells + 1) * sizeof(int));
        xsorted.allocate(f4b);
        soa.allocate(3 * soa_stride() * sizeof(float));
        nbr_s.allocate(stride * size_t(max_nb) * sizeof(uint32_t));
        cnt_s.allocate(u4b);
        scratch.allocate(sort_scratch_bytes(static_cast<int>(n)));
        status.allocate(sizeof(unsigned));
        tape4.allocate(static_cast<size_t>(every) * f4_slots() * f4b);
        tapel.allocate(static_cast<size_t>(every) * iters * n * sizeof(float));
        tapen.allocate(static_cast<size_t>(every) * (iters + 1) * stride * max_nb *
                       sizeof(uint32_t));
        tapec.allocate(static_cast<size_t>(every) * (iters + 1) * u4b);
        for (DeviceBuffer* b : {&xa, &va, &xb, &vb, &gx, &gv, &gxs, &gv1, &gv3, &gq0, &gq1,
                                &gpart, &aux})
            b->allocate(f4b);
        // Lists and counts start empty, so no stale index is ever read.
        cuda_check(cudaMemsetAsync(tapen.get(), 0, tapen.bytes(), stream));
        cuda_check(cudaMemsetAsync(tapec.get(), 0, tapec.bytes(), stream));
        cuda_check(cudaMemsetAsync(nbr_s.get(), 0, nbr_s.bytes(), stream));
        cuda_check(cudaMemsetAsync(cnt_s.get(), 0, cnt_s.bytes(), stream));
        cuda_check(cudaMemsetAsync(sidx.get(), 0, sidx.bytes(), stream));
        cuda_check(cudaStreamSynchronize(stream));
        aa.allocate(n * sizeof(float));
        acc_r.allocate(n * sizeof(double));
        acc_c.allocate(n * sizeof(double));
        ckpt = DeviceBuffer();
        steps_done = 0;
    }

    // New rest density and XSPH strength (validated like initialize).
    void set_physics(float rest_density, float xsph) {
        if (n == 0) fail(PBF_ERR_LOGIC, "the adjoint must be initialized first");
        pbf_params p = prm;
        p.restDensity = rest_density;
        p.xsphViscosity = xsph;
        validate_params(p);
        prm = p;
        c.rho0 = rest_density;
        c.gs = prm.particleMass / rest_density;
        c.gs2 = c.gs * c.gs;
        c.xsph_c = xsph;
        ckpt = DeviceBuffer();
        steps_done = 0;
    }

    // Neighbour lists of p (particle-id order) into (nbr, cnt).
    void build_lists(const float4* p, uint32_t* nbr, int* cnt) {
        const int N = static_cast<int>(n);
        unsigned* sp = status.as<unsigned>();
        launch_grid_keys(p, keys.as<uint32_t>(), N, c.g, stream);
        launch_sort(plan, keys.as<uint32_t>(), skeys.as<uint32_t>(), sidx.as<uint32_t>(),
                    akeys.as<uint32_t>(), aidx.as<uint32_t>(), scratch.get(), sp, stream);
        float* s0 = soa.as<float>();
        launch_gather_first(sidx.as<uint32_t>(), p, xsorted.as<float4>(), nullptr,
                            org.as<uint32_t>(), s0, s0 + soa_stride(), s0 + 2 * soa_stride(), N,
                            skeys.as<uint32_t>(), cells, first.as<int>(), sp, stream);
        launch_search(xsorted.as<float4>(), s0, s0 + soa_stride(), s0 + 2 * soa_stride(),
                      first.as<int>(), c, N, nbr_s.as<uint32_t>(), cnt_s.as<int>(), nullptr, sp,
                      false, stream);
        adj::k_map_lists<<<adj::grid(N), adj::kB, 0, stream>>>(sidx.as<uint32_t>(),
                                                               nbr_s.as<uint32_t>(),
                                                               cnt_s.as<int>(), N, stride, max_nb,
                                                               nbr, cnt);
    }

    // One step from (x, v) to (x_out, v_out).  With a tape slot t >= 0 every
    // intermediate goes to the tape; otherwise slot 0 of the tape is scratch.
    void step(const float4* x, const float4* v, float4* x_out, float4* v_out, int t) {
        const int N = static_cast<int>(n);
        const int s = t < 0 ? 0 : t;
        const int I = iters;
        float4* v1 = T(s, 1);
        cuda_check(cudaMemcpyAsync(T(s, 0), x, n * sizeof(float4), cudaMemcpyDeviceToDevice,
                                   stream));
        adj::k_integrate<<<adj::grid(N), adj::kB, 0, stream>>>(x, v, c, N, v1, T(s, 2));
        for (int k = 0; k < I; ++k) {
            build_lists(T(s, 2 + k), NB(s, k), CN(s, k));
            adj::k_lambda<<<adj::grid(N), adj::kB, 0, stream>>>(T(s, 2 + k), NB(s, k), CN(s, k),
                                                                c, N, L(s, k));
            adj::k_delta<<<adj::grid(N), adj::kB, 0, stream>>>(T(s, 2 + k), L(s, k), NB(s, k),
                                                               CN(s, k), c, N, T(s, 3 + I + k),
                                                               T(s, 3 + k));
        }
        float4* pI = T(s, 2 + I);
        build_lists(pI, NB(s, I), CN(s, I));
        adj::k_velocity<<<adj::grid(N), adj::kB, 0, stream>>>(pI, x, v1, c, N, T(s, 3 + 2 * I));
        adj::k_xsph<<<adj::grid(N), adj::kB, 0, stream>>>(pI, T(s, 3 + 2 * I), NB(s, I),
                                                          CN(s, I), c, N, T(s, 4 + 2 * I));
        adj::k_respond<<<adj::grid(N), adj::kB, 0, stream>>>(pI, v1, T(s, 4 + 2 * I), c, N, v_out,
                                                             x_out);
        cuda_check(cudaGetLastError());
    }

    void check_status() {
        unsigned h = 0;
        cuda_check(cudaMemcpyAsync(&h, status.get(), sizeof h, cudaMemcpyDeviceToHost, stream));
        cuda_check(cudaStreamSynchronize(stream));
        if (h & kStatusNeighborOverflow)
            fail(PBF_ERR_OVERFLOW, "Particle neighbor count exceeds solver capacity");
    }

    void forward(const pbf_float4* x0, const pbf_float4* v0, int steps, pbf_float4* x_out,
                 pbf_float4* v_out) {
        if (n == 0) fail(PBF_ERR_LOGIC, "the adjoint must be initialized before the forward");
        if (steps < 0) fail(PBF_ERR_INVALID_ARGUMENT, "step count must not be negative");
        if (!x0 || !v0 || !x_out || !v_out) fail(PBF_ERR_INVALID_ARGUMENT, "null state pointer");
        cuda_check(cudaSetDevice(device));
        const size_t f4b = n * sizeof(float4);
        const int nck = steps / every + 1;
        ckpt = DeviceBuffer(static_cast<size_t>(nck) * 2 * f4b);
        cuda_check(cudaMemsetAsync(status.get(), 0, sizeof(unsigned), stream));
        cuda_check(cudaMemcpyAsync(xa.get(), x0, f4b, cudaMemcpyDefault, stream));
        cuda_check(cudaMemcpyAsync(va.get(), v0, f4b, cudaMemcpyDefault, stream));
        float4 *x = xa.as<float4>(), *v = va.as<float4>();
        float4 *xn = xb.as<float4>(), *vn = vb.as<float4>();
        for (int t = 0; t < steps; ++t) {
            if (t % every == 0) {
                float4* ck = ckpt.as<float4>() + static_cast<size_t>(t / every) * 2 * n;
                cuda_check(cudaMemcpyAsync(ck, x, f4b, cudaMemcpyDeviceToDevice, stream));
                cuda_check(cudaMemcpyAsync(ck + n, v, f4b, cudaMemcpyDeviceToDevice, stream));
            }
            step(x, v, xn, vn, -1);
            std::swap(x, xn);
            std::swap(v, vn);
        }
        cuda_check(cudaMemcpyAsync(x_out, x, f4b, cudaMemcpyDefault, stream));
        cuda_check(cudaMemcpyAsync(v_out, v, f4b, cudaMemcpyDefault, stream));
        check_status();
        steps_done = steps;
    }

    // Adjoint of the tape slot t: (gx, gv) of the step's output -> of its input.
    void step_adjoint(int t) {
        const int N = static_cast<int>(n);
        const int I = iters;
        float4* pI = T(t, 2 + I);
        adj::k_respond_adj<<<adj::grid(N), adj::kB, 0, stream>>>(
            pI, T(t, 1), T(t, 4 + 2 * I), gv.as<float4>(), c, N, gv3.as<float4>(),
            gv1.as<float4>());
        float4* gqa = gq0.as<float4>();
        float4* gqb = gq1.as<float4>();
        adj::k_xsph_adj<<<adj::grid(N), adj::kB, 0, stream>>>(
            pI, T(t, 3 + 2 * I), gv3.as<float4>(), NB(t, I), CN(t, I), gx.as<float4>(),
            T(t, 3 + I + (I - 1)), c, N, gxs.as<float4>(), gqa, acc_c.as<double>());
        for (int k = I - 1; k >= 0; --k) {
            adj::k_iter_adj_a<<<adj::grid(N), adj::kB, 0, stream>>>(
                T(t, 2 + k), L(t, k), gqa, NB(t, k), CN(t, k), c, N, gpart.as<float4>(),
                aux.as<float4>(), aa.as<float>(), acc_r.as<double>());
            adj::k_iter_adj_b<<<adj::grid(N), adj::kB, 0, stream>>>(
                T(t, 2 + k), aux.as<float4>(), aa.as<float>(), NB(t, k), CN(t, k),
                gpart.as<float4>(), k > 0 ? T(t, 3 + I + (k - 1)) : nullptr, gxs.as<float4>(),
                gv1.as<float4>(), c, N, gqb, gx.as<float4>(), gv.as<float4>());
            std::swap(gqa, gqb);
        }
        cuda_check(cudaGetLastError());
    }

    void backward(const pbf_float4* gx_out, const pbf_float4* gv_out, pbf_float4* gx0,
                  pbf_float4* gv0, double* grho0, double* gxsph) {
        if (n == 0 || !ckpt.get()) fail(PBF_ERR_LOGIC, "backward needs a forward first");
        if (!gx_out || !gv_out || !gx0 || !gv0)
            fail(PBF_ERR_INVALID_ARGUMENT, "null gradient pointer");
        cuda_check(cudaSetDevice(device));
        const size_t f4b = n * sizeof(float4);
        cuda_check(cudaMemsetAsync(status.get(), 0, sizeof(unsigned), stream));
        cuda_check(cudaMemcpyAsync(gx.get(), gx_out, f4b, cudaMemcpyDefault, stream));
        cuda_check(cudaMemcpyAsync(gv.get(), gv_out, f4b, cudaMemcpyDefault, stream));
        cuda_check(cudaMemsetAsync(acc_r.get(), 0, n * sizeof(double), stream));
        cuda_check(cudaMemsetAsync(acc_c.get(), 0, n * sizeof(double), stream));
        const int segs = (steps_done + every - 1) / every;
        for (int sg = segs - 1; sg >= 0; --sg) {
            const int t0 = sg * every;
            const int len = std::min(every, steps_done - t0);
            const float4* ck = ckpt.as<float4>() + static_cast<size_t>(sg) * 2 * n;
            cuda_check(cudaMemcpyAsync(xa.get(), ck, f4b, cudaMemcpyDeviceToDevice, stream));
            cuda_check(cudaMemcpyAsync(va.get(), ck + n, f4b, cudaMemcpyDeviceToDevice, stream));
            float4 *x = xa.as<float4>(), *v = va.as<float4>();
            float4 *xn = xb.as<float4>(), *vn = vb.as<float4>();
            for (int t = 0; t < len; ++t) {
                step(x, v, xn, vn, t);
                std::swap(x, xn);
                std::swap(v, vn);
            }
            for (int t = len - 1; t >= 0; --t) step_adjoint(t);
        }
        cuda_check(cudaMemcpyAsync(gx0, gx.get(), f4b, cudaMemcpyDefault, stream));
        cuda_check(cudaMemcpyAsync(gv0, gv.get(), f4b, cudaMemcpyDefault, stream));
        std::vector<double> hr(n), hc(n);
        cuda_check(cudaMemcpyAsync(hr.data(), acc_r.get(), n * sizeof(double),
                                   cudaMemcpyDeviceToHost, stream));
        cuda_check(cudaMemcpyAsync(hc.data(), acc_c.get(), n * sizeof(double),
                                   cudaMemcpyDeviceToHost, stream));
        check_status();
        double sr = 0.0, sc = 0.0;
        for (size_t i = 0; i < n; ++i) {
            sr += hr[i];
            sc += hc[i];
        }
        if (grho0) *grho0 = sr;
        if (gxsph) *gxsph = sc;
    }
};

#define PBF_ADJ_GUARD(a, ...)                                                 \
    do {                                                                      \
        if (!(a)) {                                                           \
            pbf::set_global_error("adjoint handle must not be null");         \
            return PBF_ERR_INVALID_ARGUMENT;                                  \
        }                                                                     \
        return pbf::guarded(&(a)->last_error, [&]() { __VA_ARGS__; });        \
    } while (0)

extern "C" {

pbf_status pbf_adjoint_create(pbf_adjoint** out, int device) {
    return pbf::guarded(nullptr, [&]() {
        if (!out) fail(PBF_ERR_INVALID_ARGUMENT, "output handle pointer must not be null");
        auto* a = new pbf_adjoint();
        if (device < 0) {
            if (cudaGetDevice(&a->device) != cudaSuccess) a->device = 0;
        } else {
            a->device = device;
        }
        *out = a;
    });
}

void pbf_adjoint_destroy(pbf_adjoint* a) { delete a; }

const char* pbf_adjoint_last_error(const pbf_adjoint* a) {
    return a ? a->last_error.c_str() : "adjoint handle must not be null";
}

pbf_status pbf_adjoint_initialize(pbf_adjoint* a, size_t count, pbf_float3 min_bounds,
                                  pbf_float3 max_bounds, const pbf_params* params,
                                  int max_neighbors, int checkpoint_every) {
    PBF_ADJ_GUARD(a, {
        if (!params) fail(PBF_ERR_INVALID_ARGUMENT, "params must not be null");
        a->initialize(count, min_bounds, max_bounds, *params, max_neighbors, checkpoint_every);
    });
}

pbf_status pbf_adjoint_set_physics(pbf_adjoint* a, float rest_density, float xsph_viscosity) {
    PBF_ADJ_GUARD(a, a->set_physics(rest_density, xsph_viscosity));
}

pbf_status pbf_adjoint_forward(pbf_adjoint* a, const pbf_float4* x0, const pbf_float4* v0,
                               int steps, pbf_float4* x_out, pbf_float4* v_out) {
    PBF_ADJ_GUARD(a, a->forward(x0, v0, steps, x_out, v_out));
}

pbf_status pbf_adjoint_backward(pbf_adjoint* a, const pbf_float4* grad_x, const pbf_float4* grad_v,
                                pbf_float4* grad_x0, pbf_float4* grad_v0,
                                double* grad_rest_density, double* grad_xsph) {
    PBF_ADJ_GUARD(a, a->backward(grad_x, grad_v, grad_x0, grad_v0, grad_rest_density, grad_xsph));
}

}  // extern "C"
