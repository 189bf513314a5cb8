// pbf_adjoint.cu -- reverse-mode derivative of the PBF step: gradients of a
// loss on the final particle state with respect to the initial positions and
// velocities, the rest density and the XSPH strength.
//
// Differentiated substep (a step of S substeps is S of them with dt / S,
// each taped as one step):
//   integrate   v1 = v + g dt, p0 = x + v1 dt               (integration.cu:6-32)
//   I times     lambda_i = -C_i / (gs^2 (S2_i + |G_i|^2) + eps),
//               q = p + gs sum_j (lambda_i + lambda_j + s_corr) grad W_ij,
//               p' = collision projection of q (container, spheres, boxes,
//               planes; pbf_solver_kernels.cu:26-193, collision_kernels.cu:47-234)
//   velocity    v2 = (p_I - x) / dt                         (pbf_solver_kernels.cu:195-211)
//   XSPH        v3 = v2 + c sum_j (v2_j - v2_i) W_ij        (pbf_solver_kernels.cu:213-266)
//   vorticity   v5 = v3 + dt eps (N x w), w_i = sum_j grad W_ij x (v3_j - v3_i),
//               N = eta / |eta|, eta_i = sum_j (|w_j| - |w_i|) grad W_ij
//               (pbf_solver_kernels.cu:268-385; only when eps != 0)
//   response    v4 = contacts against v1 (restitution, friction; normals of
//               spheres and boxes depend on the position)
//               (collision_kernels.cu:236-371)
// gs = m / rho0, C_i = rho_i / rho0 - 1, rho_i = m (W(0) + sum_j W_ij),
// G_i = sum_j grad W_ij, S2_i = sum_j |grad W_ij|^2.
//
// The forward is the solver's own step, kernel for kernel (a step of the
// adjoint from particle-id order is bit for bit the solver's step): predict;
// per iteration a stable sort of the cell keys, the gather into the new
// order, the walk with lambda, delta p with the container projection; the
// final sort and gather, the velocity update and the walk with XSPH; then the
// contact response, written back in particle-id order.  The tape of a step
// keeps every sort's permutation, each iteration's positions, lambdas and
// neighbour lists (integer data, not differentiated), which components the
// projection moved, and the velocities entering XSPH and the contacts.
//
// The adjoint of an iteration runs in that iteration's sorted order.  A list
// holds j iff it holds i for j (d2 is computed bit-identically from both
// sides), and grad W is odd while its Hessian is even, so every transposed
// (scatter) term of the adjoint is evaluated as a gather over the particle's
// own list; the forward's gathers through a permutation become stores
// through the same permutation (each target written once).  No atomics: the
// result is deterministic.
//
// Checkpointing: the forward keeps (x, v) every K steps, in particle-id
// order, and records its last segment into the tape; the backward recomputes
// each earlier K-step segment from its checkpoint into the tape and runs the
// segment's adjoint in reverse.  Forward, recompute and adjoint segments run
// as CUDA graphs.
#include "pbf_common.h"
#include "pbf_kernels.cuh"

#include <algorithm>
#include <array>
#include <cmath>
#include <limits>
#include <map>
#include <string>
#include <tuple>
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
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Analytic derivatives used by the adjoint.  With rr = |r|:
//   spiky gradient g(r) = f(rr) r,  f = c_spiky (1 - rr/h)^2 / rr
//   Hessian        H u = f u + (f'(rr) / rr) (r . u) r
//   poly6 gradient grad W = -6 c_poly6 t^2 / h^2 r,  t = 1 - |r|^2 / h^2
//   s_corr'        ds/d(d2) = 3 k n ratio^(3n-1) / (h^2 - dq^2)
struct PairTerms {
    float3 g;      // spiky gradient
    float f, fpr;  // f and f'(rr) / rr
    float w;       // poly6
    float3 gw;     // poly6 gradient
    float s, sp;   // s_corr and ds/d(d2)
};

__device__ __forceinline__ PairTerms pair_terms(const StepConst& c, float3 r) {
    PairTerms t;
    const float d2 = dist2(r.x, r.y, r.z);
    t.g = t.gw = make_float3(0.0f, 0.0f, 0.0f);
    t.f = t.fpr = t.w = t.s = t.sp = 0.0f;
    if (!(d2 < c.k.h2)) return t;  // every term vanishes at |r| >= h
    const float tp = 1.0f - d2 * c.k.inv_h2;
    t.w = poly6(c.k, d2);
    t.gw = (-6.0f * c.k.c_poly6 * tp * tp * c.k.inv_h2) * r;
    if (d2 >= kSpikyMinD2) {
        // One reciprocal square root serves |r|, f, f' and the gradient.
        const float ir = rsqrtf(d2);
        const float rr = d2 * ir;
        const float u = 1.0f - rr * c.k.inv_h;
        t.f = c.k.c_spiky * u * u * ir;
        t.g = t.f * r;
        t.fpr = -c.k.c_spiky * u * ir * (2.0f * c.k.inv_h + u * ir) * ir;
    }
    if (c.sc.k != 0.0f && c.sc.n > 0 && c.sc.dq2 < c.sc.h2) {
        // s = -k ratio^(3n), ds/d(d2) = 3 k n ratio^(3n - 1) / (h^2 - dq^2),
        // with ratio^(3n - 1) = (ratio^3)^(n - 1) ratio^2.
        const float ratio = (c.sc.h2 - d2) * c.sc.inv_den;
        const float r2 = ratio * ratio;
        const float pm1 = ipow(r2 * ratio, c.sc.n - 1);
        t.s = c.sc.negk * pm1 * r2 * ratio;
        t.sp = 3.0f * c.sc.k * static_cast<float>(c.sc.n) * pm1 * r2 * c.sc.inv_den;
    }
    return t;
}
__device__ __forceinline__ float3 hess(const PairTerms& t, float3 r, float3 u) {
    return t.f * u + (t.fpr * dot3(r, u)) * r;
}

// The gather passes give each particle L consecutive threads (L = 2 or 4):
// lane l takes list entries l, l + L, ...; the partial sums are combined by
// a fixed butterfly (deterministic), after which every lane holds the
// total.  More lanes, more warps to hide the gather latency.
constexpr int kLanes = 4;
template <int L>
__device__ __forceinline__ float lane_sum(float v) {
#pragma unroll
    for (int m = 1; m < L; m <<= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
    return v;
}
template <int L>
__device__ __forceinline__ float3 lane_sum(float3 v) {
    return make_float3(lane_sum<L>(v.x), lane_sum<L>(v.y), lane_sum<L>(v.z));
}

// ---- adjoint -----------------------------------------------------------------

// 3x3 matrices (row-major) for the Jacobians of the collision replays.
struct Mat3 {
    float m[9];
};
__device__ __forceinline__ Mat3 mat_diag(float a, float b, float c) {
    Mat3 r = {{a, 0.0f, 0.0f, 0.0f, b, 0.0f, 0.0f, 0.0f, c}};
    return r;
}
__device__ __forceinline__ Mat3 mat_mul(const Mat3& A, const Mat3& B) {
    Mat3 r;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            r.m[3 * i + j] = A.m[3 * i] * B.m[j] + A.m[3 * i + 1] * B.m[3 + j] +
                             A.m[3 * i + 2] * B.m[6 + j];
    return r;
}
__device__ __forceinline__ Mat3 mat_add(const Mat3& A, const Mat3& B) {
    Mat3 r;
#pragma unroll
    for (int k = 0; k < 9; ++k) r.m[k] = A.m[k] + B.m[k];
    return r;
}
// A^T g.
__device__ __forceinline__ float3 mat_tmul(const Mat3& A, float3 g) {
    return make_float3(A.m[0] * g.x + A.m[3] * g.y + A.m[6] * g.z,
                       A.m[1] * g.x + A.m[4] * g.y + A.m[7] * g.z,
                       A.m[2] * g.x + A.m[5] * g.y + A.m[8] * g.z);
}
// s (I - n n^T).
__device__ __forceinline__ Mat3 mat_perp(float3 n, float s) {
    Mat3 r;
    const float v[3] = {n.x, n.y, n.z};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) r.m[3 * i + j] = s * ((i == j ? 1.0f : 0.0f) - v[i] * v[j]);
    return r;
}

// The projection's Jacobian M = d p / d q over a replay of project_all.
struct ProjJac {
    Mat3 M = mat_diag(1.0f, 1.0f, 1.0f);
    __device__ __forceinline__ void fix(int a) {
        M.m[3 * a] = M.m[3 * a + 1] = M.m[3 * a + 2] = 0.0f;
    }
    __device__ __forceinline__ void sphere(float ox, float oy, float oz, float len, float minD) {
        const float il = 1.0f / len;
        M = mat_mul(mat_perp(make_float3(ox * il, oy * il, oz * il), minD * il), M);
    }
    // p' = cl + (r / len) o: (I - P) + (r / len) (P - n n^T), P = diag(outside);
    // n has no component along the inside axes (o_a = 0 there).
    __device__ __forceinline__ void box(float ox, float oy, float oz, float len, float r,
                                        bool outx, bool outy, bool outz) {
        const float il = 1.0f / len;
        Mat3 J = mat_perp(make_float3(ox * il, oy * il, oz * il), r * il);
        const bool out[3] = {outx, outy, outz};
#pragma unroll
        for (int a = 0; a < 3; ++a)
            if (!out[a]) J.m[4 * a] += 1.0f - r * il;
        M = mat_mul(J, M);
    }
    __device__ __forceinline__ void plane(float nx, float ny, float nz) {
        M = mat_mul(mat_perp(make_float3(nx, ny, nz), 1.0f), M);
    }
    __device__ __forceinline__ void contact(float, float, float, float, bool, bool, bool, float4,
                                            float4, float, float, float) {}
};

// The velocity response's Jacobians over a replay of resolve_velocity: with
// respect to the velocity entering it (A), the incoming velocity v_in (B)
// and the position (C, through normals that depend on it).  Per active
// contact with unit normal n:
//   v' = ts (v - vn n) + target n, vn = v.n, target = -e vin.n when vin.n < 0
//   dv'/dv = ts (I - n n^T), dv'/dvin = -e n n^T (vin.n < 0),
//   dv'/dn = -ts (n v^T + vn I) + target I - e n vin^T (vin.n < 0),
//   dn/dp = (I - n n^T) / len, restricted to the clamped axes for boxes.
struct RespJac {
    Mat3 A = mat_diag(1.0f, 1.0f, 1.0f), B = mat_diag(0.0f, 0.0f, 0.0f),
         C = mat_diag(0.0f, 0.0f, 0.0f);
    float e = 0.0f, ts = 1.0f;
    __device__ __forceinline__ void fix(int) {}
    __device__ __forceinline__ void sphere(float, float, float, float, float) {}
    __device__ __forceinline__ void box(float, float, float, float, float, bool, bool, bool) {}
    __device__ __forceinline__ void plane(float, float, float) {}
    __device__ __forceinline__ void contact(float nx, float ny, float nz, float len, bool outx,
                                            bool outy, bool outz, float4 vin, float4 v,
                                            float vn, float vinn, float target) {
        const float3 n = make_float3(nx, ny, nz);
        const Mat3 Fv = mat_perp(n, ts);
        A = mat_mul(Fv, A);
        B = mat_mul(Fv, B);
        C = mat_mul(Fv, C);
        const float nv[3] = {nx, ny, nz};
        const bool hit = vinn < 0.0f;
        if (hit) {
            Mat3 Fvin;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) Fvin.m[3 * i + j] = -e * nv[i] * nv[j];
            B = mat_add(B, Fvin);
        }
        if (len > 0.0f) {
            const float vv[3] = {v.x, v.y, v.z}, vi[3] = {vin.x, vin.y, vin.z};
            Mat3 Fn;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    Fn.m[3 * i + j] = -ts * nv[i] * vv[j] + (i == j ? target - ts * vn : 0.0f) -
                                      (hit ? e * nv[i] * vi[j] : 0.0f);
            Mat3 Np = mat_perp(n, 1.0f / len);
            const bool out[3] = {outx, outy, outz};
#pragma unroll
            for (int j = 0; j < 3; ++j)
                if (!out[j]) Np.m[j] = Np.m[3 + j] = Np.m[6 + j] = 0.0f;
            C = mat_add(C, mat_mul(Fn, Np));
        }
    }
};

// gv' (velocity leaving the contacts, particle-id order through org) ->
// gradient of the velocity entering the contacts (final sorted order), of
// the incoming velocity v1 (particle-id order; vin_F[s] = v1[org[s]] in the
// forward) and of the position (gxe, final sorted order: the contact normals
// of spheres and boxes depend on it).
__global__ void k_respond_adj(const float4* __restrict__ pF, const float4* __restrict__ vinF,
                              const float4* __restrict__ vc, const float4* __restrict__ gv4,
                              const uint32_t* __restrict__ org, StepConst c, int n,
                              float4* __restrict__ gv3, float4* __restrict__ gv1,
                              float4* __restrict__ gxe) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t o = org[s];
    if (o >= static_cast<uint32_t>(n)) return;  // only after a failed forward
    RespJac jac;
    jac.e = c.restitution;
    jac.ts = fsub(1.0f, c.friction);
    float4 v = vc[s];
    resolve_velocity(c.col, c.particle_radius, c.restitution, c.friction, pF[s], vinF[s], v, jac);
    const float3 g = f3(gv4[o]);
    const float3 a = mat_tmul(jac.A, g), b = mat_tmul(jac.B, g), x = mat_tmul(jac.C, g);
    gv3[s] = make_float4(a.x, a.y, a.z, 0.0f);
    gv1[o] = make_float4(b.x, b.y, b.z, 0.0f);
    gxe[s] = make_float4(x.x, x.y, x.z, 0.0f);
}

// The gradient of q where the projection moved no component, 0 elsewhere.
__device__ __forceinline__ float4 unmoved(uint8_t m, float3 g) {
    return make_float4((m & 1u) ? 0.0f : g.x, (m & 2u) ? 0.0f : g.y, (m & 4u) ? 0.0f : g.z, 0.0f);
}

// Gradient of the position before the collision projection at slot r: with
// sphere / box / plane colliders the transpose of the projection's Jacobian,
// replayed from the recorded position before it (pre); with the container
// alone the moved bits say which components were clamped.
__device__ __forceinline__ float4 project_adj(const StepConst& c, const float4* __restrict__ pre,
                                              const uint8_t* __restrict__ moved, uint32_t r,
                                              float3 g) {
    if (!pre) return unmoved(moved[r], g);
    const float4 q = pre[r];
    float px = q.x, py = q.y, pz = q.z;
    ProjJac jac;
    project_all(c.col, c.particle_radius, px, py, pz, jac);
    const float3 t = mat_tmul(jac.M, g);
    return make_float4(t.x, t.y, t.z, 0.0f);
}

// XSPH and velocity-update adjoint in the final sorted order, then the final
// gather and the projection of the last iteration:
//   gv2_i = gv3_i + c sum_j (gv3_j - gv3_i) W_ij
//   gp_F  = gx'_i + gv2_i / dt + c sum_j ((gv3_i - gv3_j).(v2_j - v2_i)) grad W_ij
//   gxs   = -gv2_i / dt at the particle's id        (x enters v2)
//   dL/dc += gv3_i . sum_j (v2_j - v2_i) W_ij
//   gq_{I-1} at slot rel[s] of the last iteration's order = gp_F where the
//   projection left the component unchanged, 0 elsewhere.
// gx_extra: position gradient from the contact normals and the vorticity
// confinement.
template <int L>
__global__ void k_xsph_adj(const float4* __restrict__ pF, const float4* __restrict__ v2,
                           const float4* __restrict__ gv3, const uint32_t* __restrict__ nbr,
                           const int* __restrict__ cnt, const float4* __restrict__ gx_next,
                           const uint32_t* __restrict__ org, const uint32_t* __restrict__ rel,
                           const uint8_t* __restrict__ moved_last,
                           const float4* __restrict__ pre_last,
                           const float4* __restrict__ gx_extra, StepConst c, int n,
                           float4* __restrict__ gxs, float4* __restrict__ gq,
                           double* __restrict__ acc_c) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = tid / L, lane = tid % L;
    const bool live = i < n;
    const int ii = live ? i : 0;
    const float3 pi = f3(pF[ii]), vi = f3(v2[ii]), gi = f3(gv3[ii]);
    const int count = live ? min(cnt[i], c.max_nb) : 0;
    float3 sg = make_float3(0.0f, 0.0f, 0.0f), sv = sg, pos = sg;
    for (int k = lane; k < count; k += L) {
        const uint32_t j = __ldg(&nbr[static_cast<size_t>(k) * c.stride + i]);
        const float3 r = pi - f3(__ldg(&pF[j]));
        const PairTerms t = pair_terms(c, r);
        const float3 dv = f3(__ldg(&v2[j])) - vi;
        const float3 gj = f3(__ldg(&gv3[j]));
        sg = sg + t.w * (gj - gi);
        sv = sv + t.w * dv;
        pos = pos + dot3(gi - gj, dv) * t.gw;
    }
    sg = lane_sum<L>(sg);
    sv = lane_sum<L>(sv);
    pos = lane_sum<L>(pos);
    if (!live || lane != 0) return;
    const float3 gv2 = gi + c.xsph_c * sg;
    acc_c[i] += static_cast<double>(dot3(gi, sv));
    const uint32_t o = org[i], r = rel[i];
    if (o >= static_cast<uint32_t>(n) || r >= static_cast<uint32_t>(n)) return;
    float3 gp = f3(gx_next[o]) + c.inv_dt * gv2 + c.xsph_c * pos;
    gp = gp + f3(gx_extra[i]);  // contact normals' and vorticity confinement's terms
    gxs[o] = make_float4(-c.inv_dt * gv2.x, -c.inv_dt * gv2.y, -c.inv_dt * gv2.z, 0.0f);
    gq[r] = project_adj(c, pre_last, moved_last, r, gp);
}

// First gather pass of one iteration's adjoint (u_ij = gq_i - gq_j):
//   glam_i = gs sum_j u_ij . g_ij
//   gpart_i = gq_i + gs sum_j [(lam_i + lam_j + s_ij) H_ij u_ij + 2 s'_ij (u_ij . g_ij) r_ij]
// and the per-particle terms of the lambda adjoint: C_i, D_i recomputed,
//   gC_i = -glam_i / D_i, gD_i = glam_i C_i / D_i^2, a_i = m gC_i / rho0,
// with the rest-density partial gC_i (-rho_i / rho0^2) + g_gs_i (-m / rho0^2),
// g_gs_i = gq_i . X_i + 2 gs gD_i (S2_i + |G_i|^2), X_i = delta p_i / gs.
template <int L>
__global__ void k_iter_adj_a(const float4* __restrict__ p, const float* __restrict__ lam,
                             const float4* __restrict__ gq, const uint32_t* __restrict__ nbr,
                             const int* __restrict__ cnt, StepConst c, int n,
                             float4* __restrict__ gpart, float4* __restrict__ aux,
                             float* __restrict__ aa, double* __restrict__ acc_rho0) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = tid / L, lane = tid % L;
    const bool live = i < n;
    const int ii = live ? i : 0;
    const float3 pi = f3(p[ii]), gqi = f3(gq[ii]);
    const float li = lam[ii];
    const int count = live ? min(cnt[i], c.max_nb) : 0;
    float wsum = 0.0f, s2 = 0.0f, glam = 0.0f;
    float3 G = make_float3(0.0f, 0.0f, 0.0f), X = G, dpos = G;
    for (int k = lane; k < count; k += L) {
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
    wsum = lane_sum<L>(wsum) + c.k.c_poly6;
    s2 = lane_sum<L>(s2);
    glam = lane_sum<L>(glam);
    G = lane_sum<L>(G);
    X = lane_sum<L>(X);
    dpos = lane_sum<L>(dpos);
    if (!live || lane != 0) return;
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
// then the transposed gather of the iteration (slot rel[s] of the previous
// order): either the projection of the previous iteration (gq_{k-1}) or,
// after the first iteration, the integration adjoint (gx_t, gv_t in
// particle-id order).
template <int L>
__global__ void k_iter_adj_b(const float4* __restrict__ p, const float4* __restrict__ aux,
                             const float* __restrict__ aa, const uint32_t* __restrict__ nbr,
                             const int* __restrict__ cnt, const float4* __restrict__ gpart,
                             const uint32_t* __restrict__ rel,
                             const uint8_t* __restrict__ moved_prev,
                             const float4* __restrict__ pre_prev,
                             const float4* __restrict__ gxs, const float4* __restrict__ gv1,
                             StepConst c, int n, float4* __restrict__ gq_prev,
                             float4* __restrict__ gx_t, float4* __restrict__ gv_t) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = tid / L, lane = tid % L;
    const bool live = i < n;
    const int ii = live ? i : 0;
    const float3 pi = f3(p[ii]);
    const float4 ai4 = aux[ii];
    const float3 Gi = f3(ai4);
    const float gDi = ai4.w, ai = aa[ii];
    const int count = live ? min(cnt[i], c.max_nb) : 0;
    float3 acc = make_float3(0.0f, 0.0f, 0.0f);
    for (int k = lane; k < count; k += L) {
        const uint32_t j = __ldg(&nbr[static_cast<size_t>(k) * c.stride + i]);
        const float3 r = pi - f3(__ldg(&p[j]));
        const PairTerms t = pair_terms(c, r);
        const float4 aj4 = __ldg(&aux[j]);
        const float gDj = aj4.w;
        const float3 w = (gDi + gDj) * t.g + gDi * Gi - gDj * f3(aj4);
        acc = acc + (ai + __ldg(&aa[j])) * t.gw + (2.0f * c.gs2) * hess(t, r, w);
    }
    acc = lane_sum<L>(acc);
    if (!live || lane != 0) return;
    const float3 gp = f3(gpart[i]) + acc;
    const uint32_t r = rel[i];
    if (r >= static_cast<uint32_t>(n)) return;  // only after a failed forward
    if (moved_prev) {
        gq_prev[r] = project_adj(c, pre_prev, moved_prev, r, gp);
    } else {
        // p0 = x + v1 dt, v1 = v + g dt.
        const float4 gs = gxs[r], g1 = gv1[r];
        gx_t[r] = make_float4(gs.x + gp.x, gs.y + gp.y, gs.z + gp.z, 0.0f);
        gv_t[r] = make_float4(g1.x + c.dt * gp.x, g1.y + c.dt * gp.y, g1.z + c.dt * gp.z, 0.0f);
    }
}

// Vorticity confinement adjoint (computeVorticity, applyVorticityConfinement,
// pbf_solver_kernels.cu:268-385), in the final sorted order.  Forward, with
// g_kj the spiky gradient at x_k - x_j and v the velocities after XSPH:
//   w_k = sum_j g_kj x (v_j - v_k),  m_k = |w_k|,
//   eta_k = sum_j (m_j - m_k) g_kj,  N_k = eta_k / |eta_k| (0 when |eta_k| <= 1e-6),
//   v'_k = v_k + dt eps (N_k x w_k).
// First pass (a = dt eps gv'_k): gN = w x a, geta = (gN - N (N . gN)) / |eta|,
// and the direct part of gw = a x N.
template <int L>
__global__ void k_conf_adj_a(const float4* __restrict__ pF, const float4* __restrict__ om,
                             const uint32_t* __restrict__ nbr, const int* __restrict__ cnt,
                             const float4* __restrict__ gv5, StepConst c, int n,
                             float4* __restrict__ geta, float4* __restrict__ gw_direct) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = tid / L, lane = tid % L;
    const bool live = i < n;
    const int ii = live ? i : 0;
    const float3 pi = f3(pF[ii]);
    const float mi = om[ii].w;
    const int count = live ? min(cnt[i], c.max_nb) : 0;
    float3 eta = make_float3(0.0f, 0.0f, 0.0f);
    for (int k = lane; k < count; k += L) {
        const uint32_t j = __ldg(&nbr[static_cast<size_t>(k) * c.stride + i]);
        const PairTerms t = pair_terms(c, pi - f3(__ldg(&pF[j])));
        eta = eta + (__ldg(&om[j]).w - mi) * t.g;
    }
    eta = lane_sum<L>(eta);
    if (!live || lane != 0) return;
    const float3 w = f3(om[i]);
    const float3 a = (c.dt * c.vort_eps) * f3(gv5[i]);
    const float len = sqrtf(dot3(eta, eta));
    float3 N = make_float3(0.0f, 0.0f, 0.0f), ge = N;
    if (len > kEtaEpsilon) {
        N = (1.0f / len) * eta;
        const float3 gN = cross3(w, a);
        ge = (1.0f / len) * (gN - dot3(N, gN) * N);
    }
    geta[i] = make_float4(ge.x, ge.y, ge.z, 0.0f);
    const float3 gw = cross3(a, N);
    gw_direct[i] = make_float4(gw.x, gw.y, gw.z, 0.0f);
}

// Second pass: the magnitude terms of eta,
//   gm_k = -sum_j (geta_k + geta_j) . g_kj,
//   gx_k = sum_j (m_j - m_k) H_kj (geta_k + geta_j),
// (added to gx) and gw_k = direct + gm_k w_k / m_k.
template <int L>
__global__ void k_conf_adj_b(const float4* __restrict__ pF, const float4* __restrict__ om,
                             const uint32_t* __restrict__ nbr, const int* __restrict__ cnt,
                             const float4* __restrict__ geta,
                             const float4* __restrict__ gw_direct, StepConst c, int n,
                             float4* __restrict__ gw, float4* __restrict__ gx) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = tid / L, lane = tid % L;
    const bool live = i < n;
    const int ii = live ? i : 0;
    const float3 pi = f3(pF[ii]), gei = f3(geta[ii]);
    const float mi = om[ii].w;
    const int count = live ? min(cnt[i], c.max_nb) : 0;
    float gm = 0.0f;
    float3 pos = make_float3(0.0f, 0.0f, 0.0f);
    for (int k = lane; k < count; k += L) {
        const uint32_t j = __ldg(&nbr[static_cast<size_t>(k) * c.stride + i]);
        const float3 r = pi - f3(__ldg(&pF[j]));
        const PairTerms t = pair_terms(c, r);
        const float3 sg = gei + f3(__ldg(&geta[j]));
        gm -= dot3(sg, t.g);
        pos = pos + (__ldg(&om[j]).w - mi) * hess(t, r, sg);
    }
    gm = lane_sum<L>(gm);
    pos = lane_sum<L>(pos);
    if (!live || lane != 0) return;
    float3 g = f3(gw_direct[i]);
    if (mi > 0.0f) g = g + (gm / mi) * f3(om[i]);
    gw[i] = make_float4(g.x, g.y, g.z, 0.0f);
    const float4 x0 = gx[i];
    gx[i] = make_float4(x0.x + pos.x, x0.y + pos.y, x0.z + pos.z, 0.0f);
}

// Third pass: the vorticity sum,
//   gv_k = gv'_k - sum_j (gw_k + gw_j) x g_kj,
//   gx_k += sum_j H_kj ((v_j - v_k) x (gw_k + gw_j)).
template <int L>
__global__ void k_vort_adj(const float4* __restrict__ pF, const float4* __restrict__ v3,
                           const uint32_t* __restrict__ nbr, const int* __restrict__ cnt,
                           const float4* __restrict__ gw, const float4* __restrict__ gv5,
                           StepConst c, int n, float4* __restrict__ gv3,
                           float4* __restrict__ gx) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = tid / L, lane = tid % L;
    const bool live = i < n;
    const int ii = live ? i : 0;
    const float3 pi = f3(pF[ii]), vi = f3(v3[ii]), gwi = f3(gw[ii]);
    const int count = live ? min(cnt[i], c.max_nb) : 0;
    float3 acc = make_float3(0.0f, 0.0f, 0.0f), pos = acc;
    for (int k = lane; k < count; k += L) {
        const uint32_t j = __ldg(&nbr[static_cast<size_t>(k) * c.stride + i]);
        const float3 r = pi - f3(__ldg(&pF[j]));
        const PairTerms t = pair_terms(c, r);
        const float3 sg = gwi + f3(__ldg(&gw[j]));
        acc = acc + cross3(sg, t.g);
        pos = pos + hess(t, r, cross3(f3(__ldg(&v3[j])) - vi, sg));
    }
    acc = lane_sum<L>(acc);
    pos = lane_sum<L>(pos);
    if (!live || lane != 0) return;
    const float3 g = f3(gv5[i]) - acc;
    gv3[i] = make_float4(g.x, g.y, g.z, 0.0f);
    const float4 x0 = gx[i];
    gx[i] = make_float4(x0.x + pos.x, x0.y + pos.y, x0.z + pos.z, 0.0f);
}

// Contact response of the forward (resolveVelocitiesKernel, the solver's
// arithmetic), with positions and velocities stored back in particle-id order.
__global__ void k_respond_out(const float4* __restrict__ pF, const float4* __restrict__ vinF,
                              const float4* __restrict__ v3, const uint32_t* __restrict__ org,
                              StepConst c, int n, float4* __restrict__ x_out,
                              float4* __restrict__ v_out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t o = org[s];
    if (o >= static_cast<uint32_t>(n)) return;  // only after a failed forward
    const float4 p = pF[s];
    float4 v = v3[s];
    resolve_velocity(c.col, c.particle_radius, c.restitution, c.friction, p, vinF[s], v);
    x_out[o] = p;
    v_out[o] = v;
}

constexpr int kB = 256;
inline unsigned grid(int n) { return static_cast<unsigned>((n + kB - 1) / kB); }
// Grid of the gather passes (L threads per particle).
inline unsigned grid_lanes(int n, int L) {
    return static_cast<unsigned>((static_cast<size_t>(n) * L + kB - 1) / kB);
}
// Lanes per particle of the gather passes: four while fewer than 2^17
// particles leave the SMs short of warps, two above.  Backward time over
// the solver's forward, 60 steps, lanes 1 / 2 / 4: 1.97 / 1.64 / 1.62 at
// 65,536 particles, 2.04 / 1.89 / 1.95 at 262,144, 2.20 / 2.19 / 2.39 at
// 1,048,576.
constexpr int kLanesBelow = 1 << 17;
inline int lanes_for(int n) { return n < kLanesBelow ? kLanes : 2; }

}  // namespace adj
}  // namespace pbf

using namespace pbf;

struct pbf_adjoint {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;

    size_t n = 0, stride = 0;
    int max_nb = 128, every = 10, iters = 0, subs = 1;
    int steps_done = 0;
    pbf_params prm{};
    uint64_t cells = 0;
    StepConst c{};
    SortPlan plan{};

    // Scratch of one step: keys, sort buffers, composed permutations, the
    // cell table, component arrays and the predicted / projected positions.
    DeviceBuffer keys, skeys, akeys, aidx, orgs, first, soa, xs0, vin, pn, scratch, status;
    // Tape of one segment (`every` step slots), see the accessors below.
    DeviceBuffer tf4, tu32, tlam, tnb, tcn, tmv;
    // States in particle-id order: slot j holds (x, v) entering step j of a
    // recomputed segment; the forward alternates between slots 0 and 1.
    DeviceBuffer states;
    // Checkpoints (x, v) every `every` steps.
    DeviceBuffer ckpt;
    // The tape holds the last segment of the latest forward (recorded by the
    // forward itself, so the backward need not recompute it).
    bool tape_last = false;
    // Adjoint work arrays (gva..gvc: vorticity confinement only; gxe: the
    // position gradient from contact normals and vorticity confinement).
    DeviceBuffer gx, gv, gxs, gv1, gv3, gq0, gq1, gpart, aux, aa, acc_r, acc_c, gxe;
    DeviceBuffer gva, gvb, gvc;
    bool vort = false;  // vorticity confinement in the step
    // Sphere, box and plane colliders (host records as the solver keeps them,
    // and their device copy).
    std::vector<float4> h_col[3];
    DeviceBuffer d_col;
    bool has_col() const { return !h_col[0].empty() || !h_col[1].empty() || !h_col[2].empty(); }
    // Captured segments: (kind, length, parity) -> graph.
    std::map<std::tuple<int, int, int>, cudaGraphExec_t> graphs;

    ~pbf_adjoint() {
        clear_graphs();
        if (stream) cudaStreamDestroy(stream);
    }

    void clear_graphs() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
    }

    // Tape of step slot t.  float4 arrays: P(t, k) positions of sort k in its
    // order (k = 0..I; k = I is the final sort, i.e. the step's new
    // positions), then v2 (entering XSPH), v1 in the final order (entering
    // the contacts) and v3 (leaving XSPH); with vorticity confinement also
    // the vorticity (w = |w|) and v5 (leaving the confinement, entering the
    // contacts).  uint32 arrays: REL(t, k) the
    // permutation of sort k (its slot s takes slot REL[s] of the previous
    // order; for k = 0 that order is particle-id order), and ORG(t) the
    // composed permutation of the final order (slot -> particle id).
    int f4_per_step() const { return iters + (vort ? 6 : 4) + iters; }
    int u32_per_step() const { return iters + 2; }
    float4* P(int t, int k) {
        return tf4.as<float4>() + (static_cast<size_t>(t) * f4_per_step() + k) * n;
    }
    float4* V2(int t) { return P(t, iters + 1); }
    float4* VINF(int t) { return P(t, iters + 2); }
    float4* V3(int t) { return P(t, iters + 3); }
    float4* OM(int t) { return P(t, iters + 4); }
    float4* V5(int t) { return P(t, iters + 5); }
    // Velocities entering the contact response.
    float4* VC(int t) { return vort ? V5(t) : V3(t); }
    // Positions of iteration k before the collision projection (written only
    // with sphere / box / plane colliders).
    float4* PRE(int t, int k) { return P(t, iters + (vort ? 6 : 4) + k); }
    uint32_t* REL(int t, int k) {
        return tu32.as<uint32_t>() + (static_cast<size_t>(t) * u32_per_step() + k) * n;
    }
    uint32_t* ORG(int t) { return REL(t, iters + 1); }
    float* LAM(int t, int k) { return tlam.as<float>() + (static_cast<size_t>(t) * iters + k) * n; }
    uint8_t* MV(int t, int k) { return tmv.as<uint8_t>() + (static_cast<size_t>(t) * iters + k) * n; }
    uint32_t* NB(int t, int k) {
        return tnb.as<uint32_t>() + (static_cast<size_t>(t) * (iters + 1) + k) * stride * max_nb;
    }
    int* CN(int t, int k) { return tcn.as<int>() + (static_cast<size_t>(t) * (iters + 1) + k) * n; }
    float4* SX(int j) { return states.as<float4>() + static_cast<size_t>(2 * j) * n; }
    float4* SV(int j) { return states.as<float4>() + static_cast<size_t>(2 * j + 1) * n; }
    size_t soa_stride() const { return soa_stride_for(n); }

    void initialize(size_t count, pbf_float3 lo, pbf_float3 hi, const pbf_params& p, int maxnb,
                    int ckpt_every) {
        if (count == 0) fail(PBF_ERR_INVALID_ARGUMENT, "particle count must be greater than zero");
        if (count > static_cast<size_t>(std::numeric_limits<int>::max() / adj::kLanes))
            fail(PBF_ERR_LENGTH, "Particle count exceeds CUDA kernel index range");
        if (maxnb <= 0) fail(PBF_ERR_INVALID_ARGUMENT, "maxNeighbors must be greater than zero");
        if (ckpt_every <= 0) fail(PBF_ERR_INVALID_ARGUMENT, "checkpoint interval must be positive");
        validate_params(p);
        if (static_cast<long long>(ckpt_every) * p.substeps > std::numeric_limits<int>::max())
            fail(PBF_ERR_LENGTH, "checkpoint interval times substeps exceeds the int range");
        const double width = double(hi.x) - double(lo.x);
        const double depth = double(hi.z) - double(lo.z);
        if (width < 2.0 * double(p.particleRadius) || depth < 2.0 * double(p.particleRadius))
            fail(PBF_ERR_INVALID_ARGUMENT, "Particle diameter exceeds closed container dimensions");
        const std::array<int, 3> d = grid_dims_checked(lo, hi, p.smoothingRadius);
        cuda_check(cudaSetDevice(device));
        if (!stream) cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        clear_graphs();
        n = count;
        max_nb = maxnb;
        subs = p.substeps;
        every = ckpt_every * subs;  // in substeps: each substep is one taped step
        iters = p.solverIterations;
        vort = p.vorticityStrength != 0.0f;
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
        c.dt = p.dt / static_cast<float>(p.substeps);  // as the solver forms it
        c.inv_dt = 1.0f / c.dt;
        c.gravx = p.gravity.x;
        c.gravy = p.gravity.y;
        c.gravz = p.gravity.z;
        c.particle_radius = p.particleRadius;
        c.restitution = p.collisionRestitution;
        c.friction = p.collisionFriction;
        c.xsph_c = p.xsphViscosity;
        c.vort_eps = p.vorticityStrength;
        c.max_nb = max_nb;
        c.stride = stride;
        c.walk_lanes = default_walk_lanes(n, max_nb);
        c.prune_cells = true;
        c.col.cminx = lo.x;
        c.col.cminy = lo.y;
        c.col.cminz = lo.z;
        c.col.cmaxx = hi.x;
        c.col.cmaxy = hi.y;
        c.col.cmaxz = hi.z;
        apply_colliders();

        const size_t f4b = n * sizeof(float4), u4b = n * sizeof(uint32_t);
        const size_t E = static_cast<size_t>(every), I = static_cast<size_t>(iters);
        keys.allocate(u4b);
        skeys.allocate(u4b);
        akeys.allocate(u4b);
        aidx.allocate(u4b);
        orgs.allocate(2 * u4b);
        first.allocate((cells + 1) * sizeof(int));
        soa.allocate(3 * soa_stride() * sizeof(float));
        scratch.allocate(sort_scratch_bytes(static_cast<int>(n)));
        status.allocate(sizeof(unsigned));
        for (DeviceBuffer* b : {&xs0, &vin, &pn}) b->allocate(f4b);
        tf4.allocate(E * f4_per_step() * f4b);
        tu32.allocate(E * u32_per_step() * u4b);
        tlam.allocate(E * I * n * sizeof(float));
        tmv.allocate(E * I * n);
        tnb.allocate(E * (I + 1) * stride * max_nb * sizeof(uint32_t));
        tcn.allocate(E * (I + 1) * u4b);
        states.allocate((E + 1) * 2 * f4b);
        for (DeviceBuffer* b : {&gx, &gv, &gxs, &gv1, &gv3, &gq0, &gq1, &gpart, &aux, &gxe})
            b->allocate(f4b);
        for (DeviceBuffer* b : {&gva, &gvb, &gvc}) {
            if (vort)
                b->allocate(f4b);
            else
                *b = DeviceBuffer();
        }
        aa.allocate(n * sizeof(float));
        acc_r.allocate(n * sizeof(double));
        acc_c.allocate(n * sizeof(double));
        // Index data starts zeroed, so no index read after a failed step is
        // ever out of range.
        for (DeviceBuffer* b : {&tnb, &tcn, &tu32, &tmv, &orgs, &first, &keys})
            cuda_check(cudaMemsetAsync(b->get(), 0, b->bytes(), stream));
        cuda_check(cudaStreamSynchronize(stream));
        ckpt = DeviceBuffer();
        tape_last = false;
        steps_done = 0;
    }

    // CollisionSystem setters for the differentiated step (kind 0 spheres, 1
    // boxes, 2 planes; validated as the solver's); drops the recorded
    // forward.  Kept across initialize.
    void set_colliders(int kind, const void* data, size_t count) {
        std::vector<float4> next = collider_records(kind, data, count);
        cuda_check(cudaSetDevice(device));
        std::vector<float4> all;
        for (int k = 0; k < 3; ++k) {
            const std::vector<float4>& v = k == kind ? next : h_col[k];
            all.insert(all.end(), v.begin(), v.end());
        }
        DeviceBuffer d(all.size() * sizeof(float4));
        if (!all.empty())
            cuda_check(cudaMemcpy(d.get(), all.data(), all.size() * sizeof(float4),
                                  cudaMemcpyHostToDevice));
        h_col[kind].swap(next);
        d_col = std::move(d);
        apply_colliders();
        clear_graphs();  // the graphs hold the old constants
        ckpt = DeviceBuffer();
        tape_last = false;
        steps_done = 0;
    }
    void apply_colliders() {
        const float4* base = d_col.as<float4>();
        const size_t ns = h_col[0].size(), nb = h_col[1].size() / 2, np = h_col[2].size() / 2;
        c.col.spheres = base;
        c.col.boxes = base ? base + ns : nullptr;
        c.col.planes = base ? base + ns + 2 * nb : nullptr;
        c.col.ns = static_cast<int>(ns);
        c.col.nb = static_cast<int>(nb);
        c.col.np = static_cast<int>(np);
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
        clear_graphs();  // the graphs hold the old constants
        ckpt = DeviceBuffer();
        tape_last = false;
        steps_done = 0;
    }

    // Sort of the current keys into permutation rel, gather of src (the
    // previous order) into dst, composed permutation into org_out.
    void rebuild(const float4* src, float4* dst, uint32_t* rel, const uint32_t* org_in,
                 uint32_t* org_out) {
        const int N = static_cast<int>(n);
        unsigned* sp = status.as<unsigned>();
        float* s0 = soa.as<float>();
        launch_sort(plan, keys.as<uint32_t>(), skeys.as<uint32_t>(), rel, akeys.as<uint32_t>(),
                    aidx.as<uint32_t>(), scratch.get(), sp, stream);
        launch_gather_first(rel, src, dst, org_in, org_out, s0, s0 + soa_stride(),
                            s0 + 2 * soa_stride(), N, skeys.as<uint32_t>(), cells, first.as<int>(),
                            sp, stream);
    }

    // One step of the solver from (x, v) in particle-id order into tape slot
    // t, leaving (x_out, v_out) in particle-id order.
    void step(int t, const float4* x, const float4* v, float4* x_out, float4* v_out) {
        const int N = static_cast<int>(n);
        const int I = iters;
        unsigned* sp = status.as<unsigned>();
        float* s0 = soa.as<float>();
        uint32_t* oa = orgs.as<uint32_t>();
        uint32_t* ob = oa + n;
        launch_predict(x, v, xs0.as<float4>(), vin.as<float4>(), keys.as<uint32_t>(), N, c, sp,
                       stream);
        const float4* src = xs0.as<float4>();
        const uint32_t* org_in = nullptr;
        for (int k = 0; k < I; ++k) {
            uint32_t* org_out = (k & 1) ? ob : oa;
            rebuild(src, P(t, k), REL(t, k), org_in, org_out);
            launch_search(P(t, k), s0, s0 + soa_stride(), s0 + 2 * soa_stride(), first.as<int>(), c,
                          N, NB(t, k), CN(t, k), LAM(t, k), sp, true, stream);
            launch_delta_apply(P(t, k), NB(t, k), CN(t, k), LAM(t, k), c, N, pn.as<float4>(),
                               keys.as<uint32_t>(), sp, stream, MV(t, k),
                               has_col() ? PRE(t, k) : nullptr);
            src = pn.as<float4>();
            org_in = org_out;
        }
        float4* pF = P(t, I);
        rebuild(src, pF, REL(t, I), org_in, ORG(t));
        launch_finalize(ORG(t), x, vin.as<float4>(), v, nullptr, pF, N, c, V2(t), VINF(t),
                        nullptr, sp, stream);
        launch_search_xsph(pF, s0, s0 + soa_stride(), s0 + 2 * soa_stride(), first.as<int>(), c, N,
                           NB(t, I), CN(t, I), V2(t), V3(t), VINF(t), false, sp, stream);
        if (vort) {
            launch_vorticity(pF, V3(t), NB(t, I), CN(t, I), c, N, OM(t), true, sp, stream);
            launch_confine(pF, NB(t, I), CN(t, I), OM(t), V3(t), c, N, V5(t), VINF(t), false, sp,
                           stream);
        }
        adj::k_respond_out<<<adj::grid(N), adj::kB, 0, stream>>>(pF, VINF(t), VC(t), ORG(t), c, N,
                                                                 x_out, v_out);
        cuda_check(cudaGetLastError());
    }

    // Adjoint of tape slot t: (gx, gv) of the step's output -> of its input,
    // both in particle-id order.
    void step_adjoint(int t) {
        if (adj::lanes_for(static_cast<int>(n)) == adj::kLanes)
            step_adjoint_l<adj::kLanes>(t);
        else
            step_adjoint_l<2>(t);
    }

    template <int L>
    void step_adjoint_l(int t) {
        const int N = static_cast<int>(n);
        const int I = iters;
        const unsigned gl = adj::grid_lanes(N, L);
        float4* pF = P(t, I);
        // gv3: gradient of the velocities entering the contacts; gxe: the
        // position terms of contact normals (then of vorticity confinement).
        adj::k_respond_adj<<<adj::grid(N), adj::kB, 0, stream>>>(
            pF, VINF(t), VC(t), gv.as<float4>(), ORG(t), c, N, gv3.as<float4>(),
            gv1.as<float4>(), gxe.as<float4>());
        // With vorticity confinement its three passes turn gv3 into the
        // gradient of the XSPH output (gvb).
        const float4* g_xsph_out = gv3.as<float4>();
        if (vort) {
            adj::k_conf_adj_a<L><<<gl, adj::kB, 0, stream>>>(
                pF, OM(t), NB(t, I), CN(t, I), gv3.as<float4>(), c, N, gva.as<float4>(),
                gvb.as<float4>());
            adj::k_conf_adj_b<L><<<gl, adj::kB, 0, stream>>>(
                pF, OM(t), NB(t, I), CN(t, I), gva.as<float4>(), gvb.as<float4>(), c, N,
                gvc.as<float4>(), gxe.as<float4>());
            adj::k_vort_adj<L><<<gl, adj::kB, 0, stream>>>(
                pF, V3(t), NB(t, I), CN(t, I), gvc.as<float4>(), gv3.as<float4>(), c, N,
                gvb.as<float4>(), gxe.as<float4>());
            g_xsph_out = gvb.as<float4>();
        }
        const bool col = has_col();
        float4* gqa = gq0.as<float4>();
        float4* gqb = gq1.as<float4>();
        adj::k_xsph_adj<L><<<gl, adj::kB, 0, stream>>>(
            pF, V2(t), g_xsph_out, NB(t, I), CN(t, I), gx.as<float4>(), ORG(t), REL(t, I),
            MV(t, I - 1), col ? PRE(t, I - 1) : nullptr, gxe.as<float4>(), c, N,
            gxs.as<float4>(), gqa, acc_c.as<double>());
        for (int k = I - 1; k >= 0; --k) {
            adj::k_iter_adj_a<L><<<gl, adj::kB, 0, stream>>>(
                P(t, k), LAM(t, k), gqa, NB(t, k), CN(t, k), c, N, gpart.as<float4>(),
                aux.as<float4>(), aa.as<float>(), acc_r.as<double>());
            adj::k_iter_adj_b<L><<<gl, adj::kB, 0, stream>>>(
                P(t, k), aux.as<float4>(), aa.as<float>(), NB(t, k), CN(t, k),
                gpart.as<float4>(), REL(t, k), k > 0 ? MV(t, k - 1) : nullptr,
                (k > 0 && col) ? PRE(t, k - 1) : nullptr, gxs.as<float4>(), gv1.as<float4>(), c,
                N, gqb, gx.as<float4>(), gv.as<float4>());
            std::swap(gqa, gqb);
        }
        cuda_check(cudaGetLastError());
    }

    // Runs `enqueue` as a graph cached under key (captured on first use).
    template <class F>
    void run_graph(std::tuple<int, int, int> key, F&& enqueue) {
        auto it = graphs.find(key);
        if (it == graphs.end()) {
            cuda_check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            try {
                enqueue();
            } catch (...) {
                cudaGraph_t g = nullptr;
                cudaStreamEndCapture(stream, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            cudaGraph_t g = nullptr;
            cuda_check(cudaStreamEndCapture(stream, &g));
            cudaGraphExec_t ex = nullptr;
            const cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            cuda_check(e);
            it = graphs.emplace(key, ex).first;
        }
        cuda_check(cudaGraphLaunch(it->second, stream));
    }

    void check_status() {
        unsigned h = 0;
        cuda_check(cudaMemcpyAsync(&h, status.get(), sizeof h, cudaMemcpyDeviceToHost, stream));
        cuda_check(cudaStreamSynchronize(stream));
        if (h & kStatusNeighborOverflow)
            fail(PBF_ERR_OVERFLOW, "Particle neighbor count exceeds solver capacity");
        if (h & kStatusNotConverged) fail(PBF_ERR_RUNTIME, "Collision constraints did not converge");
    }

    // `frames` solver steps of `subs` substeps each.
    void forward(const pbf_float4* x0, const pbf_float4* v0, int frames, pbf_float4* x_out,
                 pbf_float4* v_out) {
        if (n == 0) fail(PBF_ERR_LOGIC, "the adjoint must be initialized before the forward");
        if (frames < 0) fail(PBF_ERR_INVALID_ARGUMENT, "step count must not be negative");
        if (static_cast<long long>(frames) * subs > std::numeric_limits<int>::max())
            fail(PBF_ERR_LENGTH, "step count times substeps exceeds the int range");
        const int steps = frames * subs;  // substeps, one taped step each
        if (!x0 || !v0 || !x_out || !v_out) fail(PBF_ERR_INVALID_ARGUMENT, "null state pointer");
        cuda_check(cudaSetDevice(device));
        const size_t f4b = n * sizeof(float4);
        const int nck = steps / every + 1;
        ckpt = DeviceBuffer(static_cast<size_t>(nck) * 2 * f4b);
        steps_done = 0;
        tape_last = false;
        cuda_check(cudaMemsetAsync(status.get(), 0, sizeof(unsigned), stream));
        cuda_check(cudaMemcpyAsync(SX(0), x0, f4b, cudaMemcpyDefault, stream));
        cuda_check(cudaMemcpyAsync(SV(0), v0, f4b, cudaMemcpyDefault, stream));
        // Before the last segment the state after t steps is in slot t % 2
        // and the tape's slot 0 is scratch; the last segment runs as the
        // backward's recompute would, into the tape.
        int fin = 0;
        for (int t0 = 0; t0 < steps; t0 += every) {
            const int len = std::min(every, steps - t0);
            const int par = t0 & 1;
            float4* ck = ckpt.as<float4>() + static_cast<size_t>(t0 / every) * 2 * n;
            cuda_check(cudaMemcpyAsync(ck, SX(par), f4b, cudaMemcpyDeviceToDevice, stream));
            cuda_check(cudaMemcpyAsync(ck + n, SV(par), f4b, cudaMemcpyDeviceToDevice, stream));
            if (t0 + len < steps) {
                run_graph(std::make_tuple(0, len, par), [&]() {
                    for (int t = 0; t < len; ++t) {
                        const int a = (par + t) & 1;
                        step(0, SX(a), SV(a), SX(1 - a), SV(1 - a));
                    }
                });
                fin = (par + len) & 1;
            } else {
                if (par) {
                    cuda_check(cudaMemcpyAsync(SX(0), ck, f4b, cudaMemcpyDeviceToDevice, stream));
                    cuda_check(
                        cudaMemcpyAsync(SV(0), ck + n, f4b, cudaMemcpyDeviceToDevice, stream));
                }
                run_graph(std::make_tuple(1, len, 0), [&]() { record(len); });
                fin = len;
                tape_last = true;
            }
        }
        cuda_check(cudaMemcpyAsync(x_out, SX(fin), f4b, cudaMemcpyDefault, stream));
        cuda_check(cudaMemcpyAsync(v_out, SV(fin), f4b, cudaMemcpyDefault, stream));
        check_status();
        steps_done = steps;
    }

    // `len` steps from state slot 0 into tape slots 0..len-1 (states 1..len).
    void record(int len) {
        for (int t = 0; t < len; ++t) step(t, SX(t), SV(t), SX(t + 1), SV(t + 1));
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
            if (!(sg == segs - 1 && tape_last)) {
                const float4* ck = ckpt.as<float4>() + static_cast<size_t>(sg) * 2 * n;
                cuda_check(cudaMemcpyAsync(SX(0), ck, f4b, cudaMemcpyDeviceToDevice, stream));
                cuda_check(cudaMemcpyAsync(SV(0), ck + n, f4b, cudaMemcpyDeviceToDevice, stream));
                run_graph(std::make_tuple(1, len, 0), [&]() { record(len); });
            }
            tape_last = false;  // the tape now holds this segment
            run_graph(std::make_tuple(2, len, 0), [&]() {
                for (int t = len - 1; t >= 0; --t) step_adjoint(t);
            });
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

pbf_status pbf_adjoint_set_spheres(pbf_adjoint* a, const pbf_sphere* spheres, size_t count) {
    PBF_ADJ_GUARD(a, a->set_colliders(0, spheres, count));
}

pbf_status pbf_adjoint_set_boxes(pbf_adjoint* a, const pbf_box* boxes, size_t count) {
    PBF_ADJ_GUARD(a, a->set_colliders(1, boxes, count));
}

pbf_status pbf_adjoint_set_planes(pbf_adjoint* a, const pbf_plane* planes, size_t count) {
    PBF_ADJ_GUARD(a, a->set_colliders(2, planes, count));
}

pbf_status pbf_adjoint_forward(pbf_adjoint* a, const pbf_float4* x0, const pbf_float4* v0,
                               int steps, pbf_float4* x_out, pbf_float4* v_out) {
    const NvtxRange range("pbf_adjoint_forward");
    PBF_ADJ_GUARD(a, a->forward(x0, v0, steps, x_out, v_out));
}

pbf_status pbf_adjoint_backward(pbf_adjoint* a, const pbf_float4* grad_x, const pbf_float4* grad_v,
                                pbf_float4* grad_x0, pbf_float4* grad_v0,
                                double* grad_rest_density, double* grad_xsph) {
    const NvtxRange range("pbf_adjoint_backward");
    PBF_ADJ_GUARD(a, a->backward(grad_x, grad_v, grad_x0, grad_v0, grad_rest_density, grad_xsph));
}

}  // extern "C"
