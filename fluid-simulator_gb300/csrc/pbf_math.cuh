// pbf_math.cuh -- device arithmetic of the PBF step.
//
// Every operation is spelled out with a round-to-nearest intrinsic, so the
// compiler cannot contract or reorder it.  The host oracle performs the same
// sequence with std::fma and -ffp-contract=off, which makes the whole step
// bit-reproducible against it.  Formulas restate the reference kernels:
//   poly6 / spiky gradient  include/pbf/sph_helpers.cuh:13-95
//   cell hash               include/pbf/spatial_grid.cuh:65-102
//   artificial pressure     include/pbf/pbf_solver_kernels.cuh:24-47
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pbf {

constexpr float kPi = 3.14159265358979323846f;
constexpr int kMaxCollisionPasses = 32;   // src/pbf/collision_system.cu:148
constexpr float kContactEpsilon = 1e-4f;  // src/pbf/collision_kernels.cu:254
constexpr float kEtaEpsilon = 1.0e-6f;    // src/pbf/pbf_solver_kernels.cu:367
constexpr float kProjectionTolScale = 9.5367431640625e-07f;  // 8 * FLT_EPSILON = 2^-20

// Status bits shared by every kernel of a step.  Kernels return early once a
// fatal bit is set so the state freezes where the reference would throw.
enum StatusBits : unsigned {
    kStatusNeighborOverflow = 1u << 0,
    kStatusNotConverged = 1u << 1,
    kStatusListOverflow = 1u << 2,  // compact lists: total count over capacity
    kStatusFatalMask = kStatusNeighborOverflow | kStatusNotConverged | kStatusListOverflow,
};

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

// Packed pair of floats for the FP32x2 instructions of sm_100+: each lane is
// rounded exactly like the scalar add/mul/fma.rn, so pairs give the same bits.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pack2(float a, float b) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void unpack2(f32x2 r, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 splat2(float a) { return pack2(a, a); }

// Squared length, rounded as the reference's compiled findNeighbors rounds
// dx*dx + dy*dy + dz*dz (src/pbf/neighbors.cu:73-74): nvcc contracts it to
// fma(dz, dz, fma(dy, dy, dx*dx)).  Neighbour lists can only match the
// reference bit for bit with this exact rounding.
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
    return ffma(dz, dz, ffma(dy, dy, fmul(dx, dx)));
}
__device__ __forceinline__ float len3(float x, float y, float z) { return fsqrt(dist2(x, y, z)); }
// dist2 of two displacements at once (lane-wise identical to dist2).
__device__ __forceinline__ f32x2 dist2x2(f32x2 dx, f32x2 dy, f32x2 dz) {
    return fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
}
// a.y*b.z - a.z*b.y with one rounding of the first product.
__device__ __forceinline__ float crossc(float ay, float az, float by, float bz) {
    return ffma(ay, bz, -fmul(az, by));
}

// Smoothing-kernel constants, computed on the host in float with the same
// operation order as the oracle.
struct KernelConst {
    float h, h2, inv_h, inv_h2, c_poly6, c_spiky;
};

__host__ inline KernelConst make_kernel_const(float h) {
    KernelConst k;
    k.h = h;
    k.h2 = h * h;
    k.inv_h = 1.0f / h;
    k.inv_h2 = 1.0f / k.h2;
    k.c_poly6 = 315.0f / (64.0f * kPi) / h / h / h;
    k.c_spiky = -45.0f / kPi / h / h / h / h;
    return k;
}

// poly6FromDistanceSquared (include/pbf/sph_helpers.cuh:13-34).
__device__ __forceinline__ float poly6(const KernelConst& k, float d2) {
    if (d2 >= k.h2) return 0.0f;
    const float t = ffma(-d2, k.inv_h2, 1.0f);
    const float t2 = fmul(t, t);
    const float t3 = fmul(t2, t);
    return fmul(k.c_poly6, t3);
}

// poly6 of two squared distances (lane-wise identical to poly6).
__device__ __forceinline__ f32x2 poly6_2(const KernelConst& k, f32x2 d2) {
    const f32x2 t = fma2(d2, splat2(-k.inv_h2), splat2(1.0f));
    const f32x2 w = mul2(splat2(k.c_poly6), mul2(mul2(t, t), t));
    float a, b, da, db;
    unpack2(w, a, b);
    unpack2(d2, da, db);
    if (da >= k.h2) a = 0.0f;
    if (db >= k.h2) b = 0.0f;
    return pack2(a, b);
}

// Reciprocal square root by Newton's method from the bit-level seed of
// C. Lomont, "Fast Inverse Square Root" (2003), constant 0x5f375a86: three
// steps y <- y (3/2 - (x/2) y^2), each a correctly rounded multiply or fma,
// so the host restatement reproduces it bit for bit.  For normal x > 0 the
// result is within 2 ulp of 1/sqrt(x).  The spiky gradient takes it in place
// of a square root and a divide: one pass of FP32 arithmetic that also runs
// on FP32x2 pairs.
constexpr uint32_t kRsqrtSeed = 0x5f375a86u;
__device__ __forceinline__ float rsqrt_seed(float x) {
    return __uint_as_float(kRsqrtSeed - (__float_as_uint(x) >> 1));
}
__device__ __forceinline__ float rsqrt_nt(float x) {
    const float nxh = fmul(-0.5f, x);
    float y = rsqrt_seed(x);
#pragma unroll
    for (int it = 0; it < 3; ++it) y = fmul(y, ffma(fmul(nxh, y), y, 1.5f));
    return y;
}
__device__ __forceinline__ f32x2 rsqrt_nt2(f32x2 x) {
    float a, b;
    unpack2(x, a, b);
    const f32x2 nxh = mul2(splat2(-0.5f), x);
    f32x2 y = pack2(rsqrt_seed(a), rsqrt_seed(b));
#pragma unroll
    for (int it = 0; it < 3; ++it) y = mul2(y, fma2(mul2(nxh, y), y, splat2(1.5f)));
    return y;
}

// Below this squared separation (2^-100, separations under 2^-50) the
// gradient is zero, as for coincident particles; the Newton seed needs a
// normal input.
constexpr float kSpikyMinD2 = 7.8886090522101181e-31f;

// spikyGradientFromDistanceSquared (include/pbf/sph_helpers.cuh:48-81):
// c_spiky (1 - r/h)^2 d / r, zero outside 0 < r < h, with r = d2 / sqrt(d2)
// and 1/r from rsqrt_nt: g = d * s, s = c_spiky t^2 * rsqrt(d2).
__device__ __forceinline__ float spiky_scale(const KernelConst& k, float d2) {
    const float rr = rsqrt_nt(d2);
    const float r = fmul(d2, rr);
    const float t = ffma(-r, k.inv_h, 1.0f);
    return fmul(fmul(k.c_spiky, fmul(t, t)), rr);
}
__device__ __forceinline__ void spiky(const KernelConst& k, float dx, float dy, float dz,
                                      float d2, float& gx, float& gy, float& gz) {
    if (d2 < kSpikyMinD2 || d2 >= k.h2) {
        gx = gy = gz = 0.0f;
        return;
    }
    const float s = spiky_scale(k, d2);
    gx = fmul(dx, s);
    gy = fmul(dy, s);
    gz = fmul(dz, s);
}
// The scale s of two squared distances, 0 where spiky() returns zero
// (d * 0 may then be -0, which leaves every sum it enters unchanged).
__device__ __forceinline__ f32x2 spiky_scale2(const KernelConst& k, f32x2 d2) {
    const f32x2 rr = rsqrt_nt2(d2);
    const f32x2 r = mul2(d2, rr);
    const f32x2 t = fma2(r, splat2(-k.inv_h), splat2(1.0f));
    const f32x2 sc = mul2(mul2(splat2(k.c_spiky), mul2(t, t)), rr);
    float a, b, da, db;
    unpack2(sc, a, b);
    unpack2(d2, da, db);
    if (da < kSpikyMinD2 || da >= k.h2) a = 0.0f;
    if (db < kSpikyMinD2 || db >= k.h2) b = 0.0f;
    return pack2(a, b);
}

// Artificial pressure s_corr = -k (W(r)/W(dq))^n with the poly6 normalisation
// cancelled (include/pbf/pbf_solver_kernels.cuh:24-47); the integer power is
// taken by squaring instead of powf.
struct ScorrConst {
    float k, negk, h2, dq2, inv_den;
    int n;
};

__host__ inline ScorrConst make_scorr_const(float h, float k, int n, float dq) {
    ScorrConst s;
    s.k = k;
    s.negk = -k;
    s.n = n;
    s.h2 = h * h;
    s.dq2 = dq * dq;
    s.inv_den = 1.0f / (s.h2 - s.dq2);
    return s;
}

__device__ __forceinline__ float ipow(float b, int n) {
    float r = 1.0f;
    while (n > 0) {
        if (n & 1) r = fmul(r, b);
        n >>= 1;
        if (n) b = fmul(b, b);
    }
    return r;
}

// ipow with the exponent known at compile time: the same products in the
// same order as the loop above (b^2, b^4 = (b^2)^2, 1 * x == x exactly).
template <int N>
__device__ __forceinline__ float ipow_c(float b) {
    if (N == 1) return b;
    if (N == 2) return fmul(b, b);
    if (N == 3) return fmul(b, fmul(b, b));
    if (N == 4) {
        const float b2 = fmul(b, b);
        return fmul(b2, b2);
    }
    return ipow(b, N);
}

template <int N>
__device__ __forceinline__ f32x2 ipow_c2(f32x2 b) {
    if (N == 1) return b;
    if (N == 2) return mul2(b, b);
    if (N == 3) return mul2(b, mul2(b, b));
    if (N == 4) {
        const f32x2 b2 = mul2(b, b);
        return mul2(b2, b2);
    }
    return b;  // not reached: other exponents use the run-time loop
}
__device__ __forceinline__ f32x2 ipow2(f32x2 b, int n) {
    f32x2 r = splat2(1.0f);
    while (n > 0) {
        if (n & 1) r = mul2(r, b);
        n >>= 1;
        if (n) b = mul2(b, b);
    }
    return r;
}

// N > 0: exponent fixed at compile time; N == 0: exponent read from s.n.
template <int N = 0>
__device__ __forceinline__ float scorr(const ScorrConst& s, float d2) {
    if (s.k == 0.0f || s.n <= 0) return 0.0f;
    if (d2 >= s.h2 || s.dq2 >= s.h2) return 0.0f;
    const float ratio = fmul(fsub(s.h2, d2), s.inv_den);
    const float r3 = fmul(fmul(ratio, ratio), ratio);
    return fmul(s.negk, N > 0 ? ipow_c<N>(r3) : ipow(r3, s.n));
}

// scorr of two squared distances (lane-wise identical to scorr<N>).
template <int N = 0>
__device__ __forceinline__ f32x2 scorr2(const ScorrConst& s, f32x2 d2) {
    if (s.k == 0.0f || s.n <= 0 || s.dq2 >= s.h2) return splat2(0.0f);
    const f32x2 ratio = mul2(sub2(splat2(s.h2), d2), splat2(s.inv_den));
    const f32x2 r3 = mul2(mul2(ratio, ratio), ratio);
    const f32x2 p = (N >= 1 && N <= 4) ? ipow_c2<N>(r3) : ipow2(r3, s.n);
    float a, b, da, db;
    unpack2(mul2(splat2(s.negk), p), a, b);
    unpack2(d2, da, db);
    if (da >= s.h2) a = 0.0f;
    if (db >= s.h2) b = 0.0f;
    return pack2(a, b);
}

// Grid geometry: cell = floor((p - min) / cellSize) per axis with an IEEE
// divide, saturating float->int conversion, clamp, u64 key arithmetic
// truncated to u32 (include/pbf/spatial_grid.cuh:65-102).
struct GridConst {
    float minx, miny, minz, cell;
    int gx, gy, gz;
    int radius;  // ceil(h / cellSize), clamped to the largest grid dimension
};

__device__ __forceinline__ void cell_of(const GridConst& g, float px, float py, float pz,
                                        int& cx, int& cy, int& cz) {
    cx = __float2int_rz(floorf(fdiv(fsub(px, g.minx), g.cell)));
    cy = __float2int_rz(floorf(fdiv(fsub(py, g.miny), g.cell)));
    cz = __float2int_rz(floorf(fdiv(fsub(pz, g.minz), g.cell)));
    cx = max(0, min(cx, g.gx - 1));
    cy = max(0, min(cy, g.gy - 1));
    cz = max(0, min(cz, g.gz - 1));
}

__device__ __forceinline__ uint32_t cell_key(const GridConst& g, int cx, int cy, int cz) {
    return static_cast<uint32_t>(static_cast<uint64_t>(cx) +
                                 static_cast<uint64_t>(cy) * static_cast<uint64_t>(g.gx) +
                                 static_cast<uint64_t>(cz) * static_cast<uint64_t>(g.gx) *
                                     static_cast<uint64_t>(g.gy));
}

__device__ __forceinline__ uint32_t key_of(const GridConst& g, float4 p) {
    int cx, cy, cz;
    cell_of(g, p.x, p.y, p.z, cx, cy, cz);
    return cell_key(g, cx, cy, cz);
}

}  // namespace pbf
