// pbf_collide.cuh -- boundary collision projection and velocity response.
//
// Restates src/pbf/collision_kernels.cu with the explicit rounding of
// pbf_math.cuh.  Positions are projected per particle: a pass that marks no
// correction leaves the particle unchanged, so iterating each particle to its
// own fixed point gives the same positions as the reference's global
// "repeat while any particle was corrected" loop
// (src/pbf/collision_system.cu:133-172) without a host round trip per pass.
#pragma once

#include "pbf_math.cuh"

namespace pbf {

// Collider arrays live in one device buffer; counts travel by value.
struct Colliders {
    const float4* spheres;  // (cx, cy, cz, radius)
    const float4* boxes;    // pairs: (center.xyz, -), (halfExtents.xyz, -)
    const float4* planes;   // pairs: (point.xyz, -), (normal.xyz, -)
    int ns, nb, np;
    float cminx, cminy, cminz, cmaxx, cmaxy, cmaxz;  // container == grid bounds
};

// Derivative hooks.  Every projector and the contact response below report
// each change they make to a hook object: the solver passes NoJac (empty,
// compiled away); the adjoint passes an accumulator of the Jacobians, so its
// replay makes the same decisions with the same float arithmetic.
//   fix(a)                      coordinate a set to a constant
//   sphere(o, len, minD)        p = s + (minD / len) o, o = p - s, len = |o|
//   box(o, len, r, outside)     p = cl + (r / len) o, o = p - cl(p), cl the
//                               clamp into the box (outside[a]: p_a was clamped)
//   plane(n)                    p += n (r - n . (p - pt))
//   contact(n, len, outside, vin, v, vn, vinn, target)
//                               an active contact with unit normal n; len > 0
//                               when n = o / len depends on the position
//                               (spheres, outside[] masks boxes), else 0
struct NoJac {
    __device__ __forceinline__ void fix(int) {}
    __device__ __forceinline__ void sphere(float, float, float, float, float) {}
    __device__ __forceinline__ void box(float, float, float, float, float, bool, bool, bool) {}
    __device__ __forceinline__ void plane(float, float, float) {}
    __device__ __forceinline__ void contact(float, float, float, float, bool, bool, bool, float4,
                                            float4, float, float, float) {}
};

// projectionTolerance (collision_kernels.cu:9-14).
__device__ __forceinline__ float proj_tol(float px, float py, float pz, float ox, float oy,
                                          float oz, float rad) {
    float s = fmaxf(rad, fmaxf(fabsf(px), fabsf(ox)));
    s = fmaxf(s, fmaxf(fabsf(py), fabsf(oy)));
    s = fmaxf(s, fmaxf(fabsf(pz), fabsf(oz)));
    return fmul(kProjectionTolScale, s);
}

// solveContainerKernel (collision_kernels.cu:47-82): open top.
template <class J>
__device__ __forceinline__ bool project_container(const Colliders& c, float r, float& px,
                                                  float& py, float& pz, J& jac) {
    const float minX = fadd(c.cminx, r), maxX = fsub(c.cmaxx, r);
    const float minY = fadd(c.cminy, r);
    const float minZ = fadd(c.cminz, r), maxZ = fsub(c.cmaxz, r);
    const float ox = px, oy = py, oz = pz;
    px = fminf(fmaxf(px, minX), maxX);
    py = fmaxf(py, minY);
    pz = fminf(fmaxf(pz, minZ), maxZ);
    if (px != ox) jac.fix(0);
    if (py != oy) jac.fix(1);
    if (pz != oz) jac.fix(2);
    return px != ox || py != oy || pz != oz;
}
__device__ __forceinline__ bool project_container(const Colliders& c, float r, float& px,
                                                  float& py, float& pz) {
    NoJac j;
    return project_container(c, r, px, py, pz, j);
}

// solveSpheresKernel (collision_kernels.cu:84-124).
template <class J>
__device__ __forceinline__ bool project_spheres(const Colliders& c, float r, float& px,
                                                float& py, float& pz, J& jac) {
    bool mark = false;
    for (int k = 0; k < c.ns; ++k) {
        const float4 s = __ldg(&c.spheres[k]);
        const float minD = fadd(s.w, r);
        const float ox = fsub(px, s.x), oy = fsub(py, s.y), oz = fsub(pz, s.z);
        const float d2 = dist2(ox, oy, oz);
        if (d2 < fmul(minD, minD)) {
            if (fsub(minD, fsqrt(d2)) <= proj_tol(px, py, pz, s.x, s.y, s.z, minD)) continue;
            mark = true;
            if (d2 == 0.0f) {
                px = fadd(s.x, minD);
                jac.fix(0);
            } else {
                const float len = fsqrt(d2);
                const float scale = fdiv(minD, len);
                jac.sphere(ox, oy, oz, len, minD);
                px = ffma(ox, scale, s.x);
                py = ffma(oy, scale, s.y);
                pz = ffma(oz, scale, s.z);
            }
        }
    }
    return mark;
}

// solveBoxesKernel (collision_kernels.cu:126-189).
template <class J>
__device__ __forceinline__ bool project_boxes(const Colliders& c, float r, float& px,
                                              float& py, float& pz, J& jac) {
    bool mark = false;
    for (int k = 0; k < c.nb; ++k) {
        const float4 bc = __ldg(&c.boxes[2 * k]);
        const float4 he = __ldg(&c.boxes[2 * k + 1]);
        const float mnx = fsub(bc.x, he.x), mny = fsub(bc.y, he.y), mnz = fsub(bc.z, he.z);
        const float mxx = fadd(bc.x, he.x), mxy = fadd(bc.y, he.y), mxz = fadd(bc.z, he.z);
        const float clx = fminf(fmaxf(px, mnx), mxx);
        const float cly = fminf(fmaxf(py, mny), mxy);
        const float clz = fminf(fmaxf(pz, mnz), mxz);
        const float ox = fsub(px, clx), oy = fsub(py, cly), oz = fsub(pz, clz);
        const float d2 = dist2(ox, oy, oz);
        if (d2 > 0.0f && d2 < fmul(r, r)) {
            if (fsub(r, fsqrt(d2)) <= proj_tol(px, py, pz, clx, cly, clz, r)) continue;
            mark = true;
            const float len = fsqrt(d2);
            const float scale = fdiv(r, len);
            jac.box(ox, oy, oz, len, r, clx != px, cly != py, clz != pz);
            px = ffma(ox, scale, clx);
            py = ffma(oy, scale, cly);
            pz = ffma(oz, scale, clz);
        } else if (d2 == 0.0f) {
            mark = true;
            const float dX = fminf(fsub(px, mnx), fsub(mxx, px));
            const float dY = fminf(fsub(py, mny), fsub(mxy, py));
            const float dZ = fminf(fsub(pz, mnz), fsub(mxz, pz));
            if (dX <= dY && dX <= dZ) {
                px = fsub(px, mnx) < fsub(mxx, px) ? fsub(mnx, r) : fadd(mxx, r);
                jac.fix(0);
            } else if (dY <= dZ) {
                py = fsub(py, mny) < fsub(mxy, py) ? fsub(mny, r) : fadd(mxy, r);
                jac.fix(1);
            } else {
                pz = fsub(pz, mnz) < fsub(mxz, pz) ? fsub(mnz, r) : fadd(mxz, r);
                jac.fix(2);
            }
        }
    }
    return mark;
}

__device__ __forceinline__ bool plane_normal(const Colliders& c, int k, float& nx, float& ny,
                                             float& nz, float4& pt) {
    pt = __ldg(&c.planes[2 * k]);
    const float4 n = __ldg(&c.planes[2 * k + 1]);
    const float nl2 = dist2(n.x, n.y, n.z);
    if (nl2 == 0.0f) return false;
    const float ns = fdiv(1.0f, fsqrt(nl2));
    nx = fmul(n.x, ns);
    ny = fmul(n.y, ns);
    nz = fmul(n.z, ns);
    return true;
}

__device__ __forceinline__ bool project_spheres(const Colliders& c, float r, float& px,
                                                float& py, float& pz) {
    NoJac j;
    return project_spheres(c, r, px, py, pz, j);
}
__device__ __forceinline__ bool project_boxes(const Colliders& c, float r, float& px,
                                              float& py, float& pz) {
    NoJac j;
    return project_boxes(c, r, px, py, pz, j);
}

// solvePlanesKernel (collision_kernels.cu:191-234).
template <class J>
__device__ __forceinline__ bool project_planes(const Colliders& c, float r, float& px,
                                               float& py, float& pz, J& jac) {
    bool mark = false;
    for (int k = 0; k < c.np; ++k) {
        float nx, ny, nz;
        float4 pt;
        if (!plane_normal(c, k, nx, ny, nz, pt)) continue;
        const float dist =
            ffma(fsub(pz, pt.z), nz, ffma(fsub(py, pt.y), ny, fmul(fsub(px, pt.x), nx)));
        if (dist < r) {
            if (fsub(r, dist) <= proj_tol(px, py, pz, pt.x, pt.y, pt.z, r)) continue;
            mark = true;
            jac.plane(nx, ny, nz);
            const float corr = fsub(r, dist);
            px = ffma(nx, corr, px);
            py = ffma(ny, corr, py);
            pz = ffma(nz, corr, pz);
        }
    }
    return mark;
}
__device__ __forceinline__ bool project_planes(const Colliders& c, float r, float& px,
                                               float& py, float& pz) {
    NoJac j;
    return project_planes(c, r, px, py, pz, j);
}

// Returns false when the particle still needed a correction in its last pass.
template <class J>
__device__ __forceinline__ bool project_all(const Colliders& c, float r, float& px, float& py,
                                            float& pz, J& jac) {
    for (int pass = 0; pass < kMaxCollisionPasses; ++pass) {
        bool mark = project_container(c, r, px, py, pz, jac);
        if (c.ns) mark = project_spheres(c, r, px, py, pz, jac) || mark;
        if (c.nb) mark = project_boxes(c, r, px, py, pz, jac) || mark;
        if (c.np) mark = project_planes(c, r, px, py, pz, jac) || mark;
        if (!mark) return true;
    }
    return false;
}
__device__ __forceinline__ bool project_all(const Colliders& c, float r, float& px, float& py,
                                            float& pz) {
    NoJac j;
    return project_all(c, r, px, py, pz, j);
}

// resolveContactVelocity (collision_kernels.cu:21-43).  len / outside: see
// the hooks above (len = 0 for a normal that does not depend on position).
template <class J>
__device__ __forceinline__ void contact(float nx, float ny, float nz, float4 vin, float e,
                                        float ts, float4& v, J& jac, float len = 0.0f,
                                        bool outx = true, bool outy = true, bool outz = true) {
    const float vn = ffma(v.z, nz, ffma(v.y, ny, fmul(v.x, nx)));
    const float vinn = ffma(vin.z, nz, ffma(vin.y, ny, fmul(vin.x, nx)));
    const float target = vinn < 0.0f ? fmul(-e, vinn) : 0.0f;
    if (vn > target || (vn == target && vinn >= 0.0f)) return;
    jac.contact(nx, ny, nz, len, outx, outy, outz, vin, v, vn, vinn, target);
    const float tx = ffma(-vn, nx, v.x), ty = ffma(-vn, ny, v.y), tz = ffma(-vn, nz, v.z);
    v.x = ffma(ts, tx, fmul(target, nx));
    v.y = ffma(ts, ty, fmul(target, ny));
    v.z = ffma(ts, tz, fmul(target, nz));
}

// resolveVelocitiesKernel (collision_kernels.cu:236-371).
template <class J>
__device__ __forceinline__ void resolve_velocity(const Colliders& c, float r, float e,
                                                 float friction, float4 p, float4 vin,
                                                 float4& v, J& jac) {
    const float ts = fsub(1.0f, friction);
    const float eps = kContactEpsilon;
    const float minX = fadd(c.cminx, r), maxX = fsub(c.cmaxx, r);
    const float minY = fadd(c.cminy, r);
    const float minZ = fadd(c.cminz, r), maxZ = fsub(c.cmaxz, r);
    if (p.x <= fadd(minX, eps)) contact(1.0f, 0.0f, 0.0f, vin, e, ts, v, jac);
    else if (p.x >= fsub(maxX, eps)) contact(-1.0f, 0.0f, 0.0f, vin, e, ts, v, jac);
    if (p.y <= fadd(minY, eps)) contact(0.0f, 1.0f, 0.0f, vin, e, ts, v, jac);
    if (p.z <= fadd(minZ, eps)) contact(0.0f, 0.0f, 1.0f, vin, e, ts, v, jac);
    else if (p.z >= fsub(maxZ, eps)) contact(0.0f, 0.0f, -1.0f, vin, e, ts, v, jac);
    for (int k = 0; k < c.ns; ++k) {
        const float4 s = __ldg(&c.spheres[k]);
        const float minD = fadd(s.w, r);
        const float ox = fsub(p.x, s.x), oy = fsub(p.y, s.y), oz = fsub(p.z, s.z);
        const float d2 = dist2(ox, oy, oz);
        const float cd = fadd(minD, eps);
        if (d2 > 0.0f && d2 <= fmul(cd, cd)) {
            const float len = fsqrt(d2);
            const float sc = fdiv(1.0f, len);
            contact(fmul(ox, sc), fmul(oy, sc), fmul(oz, sc), vin, e, ts, v, jac, len);
        }
    }
    for (int k = 0; k < c.nb; ++k) {
        const float4 bc = __ldg(&c.boxes[2 * k]);
        const float4 he = __ldg(&c.boxes[2 * k + 1]);
        const float mnx = fsub(bc.x, he.x), mny = fsub(bc.y, he.y), mnz = fsub(bc.z, he.z);
        const float mxx = fadd(bc.x, he.x), mxy = fadd(bc.y, he.y), mxz = fadd(bc.z, he.z);
        const float clx = fminf(fmaxf(p.x, mnx), mxx);
        const float cly = fminf(fmaxf(p.y, mny), mxy);
        const float clz = fminf(fmaxf(p.z, mnz), mxz);
        const float ox = fsub(p.x, clx), oy = fsub(p.y, cly), oz = fsub(p.z, clz);
        const float d2 = dist2(ox, oy, oz);
        const float re = fadd(r, eps);
        float nx, ny, nz, len = 0.0f;
        if (d2 > 0.0f && d2 <= fmul(re, re)) {
            len = fsqrt(d2);
            const float sc = fdiv(1.0f, len);
            nx = fmul(ox, sc);
            ny = fmul(oy, sc);
            nz = fmul(oz, sc);
        } else if (d2 == 0.0f) {
            const float dX = fminf(fsub(p.x, mnx), fsub(mxx, p.x));
            const float dY = fminf(fsub(p.y, mny), fsub(mxy, p.y));
            const float dZ = fminf(fsub(p.z, mnz), fsub(mxz, p.z));
            nx = ny = nz = 0.0f;
            if (dX <= dY && dX <= dZ) nx = fsub(p.x, mnx) < fsub(mxx, p.x) ? -1.0f : 1.0f;
            else if (dY <= dZ) ny = fsub(p.y, mny) < fsub(mxy, p.y) ? -1.0f : 1.0f;
            else nz = fsub(p.z, mnz) < fsub(mxz, p.z) ? -1.0f : 1.0f;
        } else {
            continue;
        }
        contact(nx, ny, nz, vin, e, ts, v, jac, len, clx != p.x, cly != p.y, clz != p.z);
    }
    for (int k = 0; k < c.np; ++k) {
        float nx, ny, nz;
        float4 pt;
        if (!plane_normal(c, k, nx, ny, nz, pt)) continue;
        const float dist =
            ffma(fsub(p.z, pt.z), nz, ffma(fsub(p.y, pt.y), ny, fmul(fsub(p.x, pt.x), nx)));
        if (dist <= fadd(r, eps)) contact(nx, ny, nz, vin, e, ts, v, jac);
    }
}
__device__ __forceinline__ void resolve_velocity(const Colliders& c, float r, float e,
                                                 float friction, float4 p, float4 vin,
                                                 float4& v) {
    NoJac j;
    resolve_velocity(c, r, e, friction, p, vin, v, j);
}

}  // namespace pbf
