// venu_device.cuh -- device building blocks of the GB300 path tracer.
//
// Arithmetic contract (the library is compiled with -fmad=false): every
// float operation rounds once as written; fmaf() appears only where written.
// Camera rays, scattering and the sky follow the reference's device source
// (Core/RayTracer.cu, Core/vec_math.h) operation by operation; the ray/box
// and ray/sphere tests are this library's own (robust slab test, stable
// quadratic with an exactly refined constant term).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include <type_traits>

#include "../../include/venu.h"

#ifndef VENU_MINMAX3
#define VENU_MINMAX3 1
#endif
// Register cap of the fused traverse+shade kernels.  64 registers let 8
// blocks of 128 threads (32 warps) stay resident per SM instead of 6 at the
// 80 the compiler picks on its own, at the cost of a few spilled bytes;
// measured on GB300: +8 % segments/s on the RTIOW scene, +6 % on 1M spheres
// (72: +5 %, 56: +7 %, 48: slower).
#ifndef VENU_TRACE_MAXREG
#define VENU_TRACE_MAXREG 64
#endif
#define VENU_TRACE_BOUNDS __maxnreg__(VENU_TRACE_MAXREG)
// Register cap of the fused kernel over the wide tree.  With 4 children per
// node, 64 registers (8 resident 128-thread blocks per SM, a few spilled
// bytes) beat 72 and 80 (6 and 5 blocks) on RTIOW (+5 %) and 1M spheres
// (+7 %), and lose 3 % on 5k spheres.
#ifndef VENU_WIDE_MAXREG
#define VENU_WIDE_MAXREG 64
#endif
#define VENU_WIDE_BOUNDS __maxnreg__(VENU_WIDE_MAXREG)
// The multi-job kernel of the batch engine keeps a per-ray scene view.
#ifndef VENU_TRACE_MULTI_MAXREG
#define VENU_TRACE_MULTI_MAXREG 64
#endif
#define VENU_TRACE_MULTI_BOUNDS __maxnreg__(VENU_TRACE_MULTI_MAXREG)

namespace venu {

// ---------------------------------------------------------------------------
// float3 operations with Core/vec_math.h semantics.
// ---------------------------------------------------------------------------
struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator-(f3 a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// Core/vec_math.h:483-487: float3 / float multiplies by the reciprocal.
__device__ __forceinline__ f3 divs(f3 a, float s) {
    float inv = 1.0f / s;
    return a * inv;
}
__device__ __forceinline__ f3 normalize(f3 v) {  // Core/vec_math.h:544-549
    float inv = 1.0f / sqrtf(dot(v, v));
    return v * inv;
}
__device__ __forceinline__ f3 reflect(f3 i, f3 n) { return i - (2.0f * n) * dot(n, i); }
__device__ __forceinline__ f3 refract(f3 uv, f3 n, float eta) {  // Core/vec_math.h:563-569
    float cos_theta = fminf(dot(-uv, n), 1.0f);
    f3 r_perp = eta * (uv + cos_theta * n);
    f3 r_par = (-sqrtf(fabsf(1.0f - dot(r_perp, r_perp)))) * n;
    return r_perp + r_par;
}
__device__ __forceinline__ f3 lerp3(f3 a, f3 b, float t) { return a + t * (b - a); }

// ---------------------------------------------------------------------------
// RNG: TEA-4 seed hash and the 24-bit LCG of Core/random.cuh:31-67.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t tea4(uint32_t v0, uint32_t v1) {
    uint32_t s0 = 0;
#pragma unroll
    for (int n = 0; n < 4; ++n) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}
__device__ __forceinline__ float rnd(uint32_t& s) {
    s = 1664525u * s + 1013904223u;
    return (float)(s & 0x00FFFFFFu) / (float)0x01000000;
}
// Core/RayTracer.cu:93-97 with min=-1, max=1; draws x, y, z left to right.
// The rejection loops stop after kMaxTries candidates (the last one is then
// kept): an acceptance rate of 52% (sphere) / 79% (disk) makes that bound
// unreachable in practice, and it guarantees termination on the GPU.
constexpr int kMaxTries = 4096;
__device__ __forceinline__ float rnd_pm1(uint32_t& s) { return -1.0f + (1.0f - -1.0f) * rnd(s); }
__device__ __forceinline__ f3 random_in_unit_sphere(uint32_t& s) {  // :117-125
    f3 p;
    for (int i = 0; i < kMaxTries; ++i) {
        float x = rnd_pm1(s);
        float y = rnd_pm1(s);
        float z = rnd_pm1(s);
        p = mk(x, y, z);
        if (!(dot(p, p) >= 1.0f)) break;
    }
    return p;
}
__device__ __forceinline__ f3 random_in_unit_disk(uint32_t& s) {  // :141-149
    f3 p;
    for (int i = 0; i < kMaxTries; ++i) {
        float x = rnd_pm1(s);
        float y = rnd_pm1(s);
        p = mk(x, y, 0.0f);
        if (!(dot(p, p) >= 1.0f)) break;
    }
    return p;
}
// Core/RayTracer.cu:8-13; for float x, (double)x < 1e-8 <=> x <= 1e-8f.
__device__ __forceinline__ bool near_zero(f3 e) {
    return fabsf(e.x) <= 1e-8f && fabsf(e.y) <= 1e-8f && fabsf(e.z) <= 1e-8f;
}

// ---------------------------------------------------------------------------
// Camera (Params fields) with the per-launch constants normalize(U/V).
// ---------------------------------------------------------------------------
struct DevCamera {
    f3 origin, u, v, w, un, vn;
    float lens;
};

// Core/RayTracer.cu:151-161,173-177: jitter u, jitter v, then the lens disk.
__device__ __forceinline__ void camera_ray(const DevCamera& C, uint32_t x, uint32_t y, uint32_t W,
                                           uint32_t H, uint32_t& seed, f3& o, f3& d) {
    float r1 = rnd(seed);
    float s = 2.0f * ((float)x + r1) / (float)(W - 1) - 1.0f;
    float r2 = rnd(seed);
    float t = 2.0f * ((float)y + r2) / (float)(H - 1) - 1.0f;
    f3 rd = C.lens * random_in_unit_disk(seed);
    f3 offset = C.un * rd.x + C.vn * rd.y;
    o = C.origin + offset;
    d = C.w + (s * C.u) * 0.5f + (t * C.v) * 0.5f - offset;
}

// Core/RayTracer.cu:442-449.  fmaf(0.5, y, 0.5) equals the reference's double
// 0.5 * (y + 1.0) rounded to float (both are one rounding of the same value).
__device__ __forceinline__ f3 sky(f3 d) {
    f3 ud = normalize(d);
    float t = fmaf(0.5f, ud.y, 0.5f);
    return lerp3(mk(1.0f, 1.0f, 1.0f), mk(0.5f, 0.7f, 1.0f), t);
}

// Schlick (Core/RayTracer.cu:373-379) with (1-cos)^5 as an explicit product.
__device__ __forceinline__ float reflectance(float cosine, float ref_idx) {
    float r0 = (1.0f - ref_idx) / (1.0f + ref_idx);
    r0 = r0 * r0;
    float x = 1.0f - cosine;
    float x2 = x * x;
    float x5 = (x2 * x2) * x;
    return r0 + (1.0f - r0) * x5;
}

// x^(1/2.4) for x in [2^-126, 1], the power of the sRGB encode
// (Core/RayTracer.cu:16-47 calls powf), from IEEE +, -, *, / and fmaf only,
// so that the host restatement rounds identically and image bytes can be
// checked exactly.  x = m 2^e with m in [sqrt(1/2), sqrt(2));
// log2 m = s (c1 + c3 s^2 + c5 s^4 + c7 s^6 + c9 s^8), s = (m-1)/(m+1): the
// atanh series of ln m = 2 atanh(s) scaled by 1/ln 2 (c_k = 2/(k ln 2), c1
// as a head and a tail); t = y (e + log2 m) with the product y e split
// exactly (TwoProduct); 2^t = 2^n 2^f with n = rint(t) and 2^f by its Taylor
// series to f^7 (coefficients ln(2)^k / k!).  Error at most 1.16 ulp over
// every float in [0.0031308, 1] (measured against double pow).
__device__ __forceinline__ float srgb_pow(float x) {
    const uint32_t b = __float_as_uint(x);
    int e = (int)(b >> 23) - 127;
    float m = __uint_as_float((b & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421353816986083984375f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float z = s * s;
    float tail = fmaf(z, 0.32059890031814575f, 0.41219857335090637f);
    tail = fmaf(z, tail, 0.5770780444145203f);
    tail = fmaf(z, tail, 0.9617967009544373f);
    tail = fmaf(z, tail, 3.8519259e-08f);
    const float L = fmaf(s, 2.885390043258667f, s * tail);
    const float y = 0.4166666567325592f;  // 1.0f / 2.4f, the reference's exponent
    const float fe = (float)e;
    const float ph = fe * y;
    const float pl = fmaf(fe, y, -ph);
    const float q = fmaf(y, L, pl);
    const float n = rintf(ph + q);
    const float f = (ph - n) + q;
    float p = fmaf(f, 1.5252733646775596e-05f, 1.540352968731895e-04f);
    p = fmaf(f, p, 1.3333557872101665e-03f);
    p = fmaf(f, p, 9.618128649890423e-03f);
    p = fmaf(f, p, 5.550410971045494e-02f);
    p = fmaf(f, p, 2.4022650718688965e-01f);
    p = fmaf(f, p, 6.931471824645996e-01f);
    p = fmaf(f, p, 1.0f);
    return p * __uint_as_float((uint32_t)(127 + (int)n) << 23);
}

// ---------------------------------------------------------------------------
// Scene view: LBVH nodes + spheres/materials in Morton (slot) order.
// ---------------------------------------------------------------------------
// Child words: bit 31 = leaf, bit 30 = leaf already tested before the
// traversal (a hoisted huge sphere), bits 0-29 = slot or internal index.
constexpr int32_t kLeaf = (int32_t)0x80000000u;
constexpr int32_t kHoisted = 0x40000000;
constexpr int32_t kSlotMask = 0x3fffffff;
constexpr int32_t kNone = 0x7fffffff;
constexpr int kMaxHoisted = 4;

// Children per node of the wide traversal tree (4; 8 measured slower on
// every workload here) and its node layout in float4s: per axis a
// the lo planes of the children at 2a*H + h and the hi planes at
// (2a+1)*H + h (h = 0..H-1, four children per float4), then the child words
// at 6H + h and the masks at 7H.
#ifndef VENU_WIDE_CHILDREN
#define VENU_WIDE_CHILDREN 4
#endif
constexpr int kWideW = VENU_WIDE_CHILDREN;
constexpr int kWideH = kWideW / 4;
constexpr int kWideF4 = 8 * kWideH;
static_assert(kWideW == 4 || kWideW == 8, "the wide tree has 4 or 8 children per node");

struct SceneView {
    const float4* __restrict__ nodes;  // 2 float4 per internal node: {lo, left} {hi, right}
    const float4* __restrict__ trav;   // 4 float4 per internal node: both children, see lbvh.cu
    const float4* __restrict__ wide;   // kWideF4 float4 per node of the wide tree, see lbvh.cu
    const float4* __restrict__ sph;    // {center, radius} per slot
    const float4* __restrict__ mat;    // {albedo, fuzz or ir} per slot
    const uint32_t* __restrict__ meta; // original id | material << 30
    uint32_t n;
    uint32_t nhoist;                   // huge spheres tested first by every ray
    int32_t hoist[kMaxHoisted];        // their slots (ascending)
};

// Slab test: a box's entry / exit parameter on axis k is
// fma(lo_k or hi_k, inv_k, offset).  The offset -(o_k inv_k) is rounded, which
// a margin of |o_k inv_k| 2^-21 covers (several times that rounding).
//   Shared margin (almost every ray): one offset n0_k = -(o_k inv_k) per axis
//   and the largest margin of the three axes added once to the exit
//   parameter (n1.x), which keeps four floats live during traversal.
//   Per-axis margins (axis = true): a near-zero direction component (1/d up
//   to 1e20) makes its own margin huge, and shared by all axes it would
//   switch off the culling on the other two (such a ray then visits every
//   node its slab meets).  When the shared margin exceeds 1 (in units of t)
//   the offsets carry each axis's own margin instead, moved outwards: n0_k
//   for the lo plane, n1_k for the hi plane (the entry plane is lo when
//   inv_k >= 0).  Such rays are rare (a direction component below ~1e-5 of
//   the others) and traverse with their own instantiation of the loop.
//   from: slot of the sphere the ray leaves (its origin lies on that
//   sphere's surface), or -1 (camera rays, rays from the caller).
struct RayPre {
    f3 o, d, inv, n0, n1;
    float a, inv_a;
    bool axis;
    int32_t from;
};

constexpr float kSharedMarginMax = 1.0f;

__device__ __forceinline__ RayPre prep(f3 o, f3 d) {
    RayPre R;
    R.from = -1;
    R.o = o;
    R.d = d;
    float dx = fabsf(d.x) < 1e-20f ? copysignf(1e-20f, d.x) : d.x;
    float dy = fabsf(d.y) < 1e-20f ? copysignf(1e-20f, d.y) : d.y;
    float dz = fabsf(d.z) < 1e-20f ? copysignf(1e-20f, d.z) : d.z;
    R.inv = mk(1.0f / dx, 1.0f / dy, 1.0f / dz);
    const float px = o.x * R.inv.x, py = o.y * R.inv.y, pz = o.z * R.inv.z;
    const float mx = fabsf(px) * 4.76837158203125e-07f;  // 2^-21
    const float my = fabsf(py) * 4.76837158203125e-07f;
    const float mz = fabsf(pz) * 4.76837158203125e-07f;
    const float m = fmaxf(fmaxf(mx, my), mz);
    R.axis = m > kSharedMarginMax;
    if (!R.axis) {
        R.n0 = mk(-px, -py, -pz);
        R.n1 = mk(m, 0.0f, 0.0f);
    } else {
        const float lx = -px - mx, hx = -px + mx;
        const float ly = -py - my, hy = -py + my;
        const float lz = -pz - mz, hz = -pz + mz;
        R.n0 = mk(R.inv.x >= 0.0f ? lx : hx, R.inv.y >= 0.0f ? ly : hy, R.inv.z >= 0.0f ? lz : hz);
        R.n1 = mk(R.inv.x >= 0.0f ? hx : lx, R.inv.y >= 0.0f ? hy : ly, R.inv.z >= 0.0f ? hz : lz);
    }
    R.a = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
    R.inv_a = 1.0f / R.a;
    return R;
}

// Three-input min / max (one instruction on sm_100 and later).  The slab
// test never feeds them a NaN (the direction guard keeps 1/d finite), and on
// non-NaN inputs they equal the two-input chains exactly.
__device__ __forceinline__ float fmax3(float a, float b, float c) {
#if VENU_MINMAX3
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fmaxf(fmaxf(a, b), c);
#endif
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
#if VENU_MINMAX3
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fminf(fminf(a, b), c);
#endif
}

// Robust slab test: conservative by a relative 2^-20 plus the rounding
// margins of the slab offsets (shared or per axis, see RayPre), so rounding
// never drops a box the ray touches.
template <bool AXIS>
__device__ __forceinline__ bool box_test(const RayPre& R, float4 lo, float4 hi, float tmin,
                                         float tcap, float& tnear) {
    const f3 nh = AXIS ? R.n1 : R.n0;
    float t0x = fmaf(lo.x, R.inv.x, R.n0.x), t1x = fmaf(hi.x, R.inv.x, nh.x);
    float t0y = fmaf(lo.y, R.inv.y, R.n0.y), t1y = fmaf(hi.y, R.inv.y, nh.y);
    float t0z = fmaf(lo.z, R.inv.z, R.n0.z), t1z = fmaf(hi.z, R.inv.z, nh.z);
    float tn = fmax3(fminf(t0x, t1x), fminf(t0y, t1y), fmaxf(fminf(t0z, t1z), tmin));
    float tf = fmin3(fmaxf(t0x, t1x), fmaxf(t0y, t1y), fminf(fmaxf(t0z, t1z), tcap));
    tnear = tn;
    // tf (1 + 2^-20) covers the roundings of the two fmas; the shared margin
    // is added here
    return AXIS ? tn <= tf * 1.00000095367431640625f : tn <= fmaf(tf, 1.00000095367431640625f, R.n1.x);
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    float bp = s - a;
    float ap = s - bp;
    e = (a - ap) + (b - bp);
}

// Ray/sphere: the discriminant is formed from the perpendicular distance of
// the centre to the ray line, disc = a (r^2 - |f|^2) with f = h - (h.d/a) d
// (Haines et al., "Precision Improvements for Ray/Sphere Intersection", Ray
// Tracing Gems ch. 7), so its error scales with r^2 instead of |h|^2; the
// roots come from q = -(b + sign(b) sqrt(disc)) as q/a and c/q (no
// cancellation).  When the origin is close to the surface relative to the
// radius (|c| < (|h|^2 + r^2)/16), c = |o-C|^2 - r^2 and h are refined with
// TwoDiff/TwoProduct/TwoSum error terms, so the near root c/q keeps full
// relative accuracy even for the r = 1000 ground sphere.  Root selection
// follows Core/RayTracer.cu:248-253: the smaller root in [tmin, tmax], else
// the larger.
__device__ __forceinline__ bool sphere_test(const RayPre& R, float4 S, float tmin, float tmax,
                                            float& tout) {
    const float r = S.w;
    float hx = R.o.x - S.x, hy = R.o.y - S.y, hz = R.o.z - S.z;
    float hb = fmaf(hx, R.d.x, fmaf(hy, R.d.y, hz * R.d.z));
    float hh = fmaf(hx, hx, fmaf(hy, hy, hz * hz));
    float r2 = r * r;
    float c = hh - r2;
    // Origin clearly outside (c above its rounding bound) and moving away from
    // the centre (h.d > 0): both roots are negative, no hit.
    if (hb > 0.0f && c > (hh + r2) * 9.5367431640625e-07f) return false;  // 2^-20
    float discp;
    if (fabsf(c) < (hh + r2) * 0.0625f) {
        // exact residuals of h = o - C (TwoDiff)
        float bvx = R.o.x - hx, bvy = R.o.y - hy, bvz = R.o.z - hz;
        float ex = (R.o.x - (hx + bvx)) + (bvx - S.x);
        float ey = (R.o.y - (hy + bvy)) + (bvy - S.y);
        float ez = (R.o.z - (hz + bvz)) + (bvz - S.z);
        // c = |h + e|^2 - r^2 from exact squares and compensated sums
        float px = hx * hx, py = hy * hy, pz = hz * hz;
        float qx = fmaf(hx, hx, -px), qy = fmaf(hy, hy, -py), qz = fmaf(hz, hz, -pz);
        float qr = fmaf(r, r, -r2);
        float s1, e1, s2, e2, s3, e3;
        two_sum(px, py, s1, e1);
        two_sum(s1, pz, s2, e2);
        two_sum(s2, -r2, s3, e3);
        float lo = (e1 + e2) + e3;
        lo = lo + ((qx + qy) + qz);
        lo = lo - qr;
        float he = fmaf(hx, ex, fmaf(hy, ey, hz * ez));
        lo = fmaf(2.0f, he, lo);
        c = s3 + lo;
        hb = hb + fmaf(ex, R.d.x, fmaf(ey, R.d.y, ez * R.d.z));
        // f = (h + e) - s d as head + tail, then r^2 - |f|^2 compensated
        const float s = hb * R.inv_a;
        float mx = s * R.d.x, my = s * R.d.y, mz = s * R.d.z;
        float mex = fmaf(s, R.d.x, -mx), mey = fmaf(s, R.d.y, -my), mez = fmaf(s, R.d.z, -mz);
        float fx, fy, fz, fex, fey, fez;
        two_sum(hx, -mx, fx, fex);
        two_sum(hy, -my, fy, fey);
        two_sum(hz, -mz, fz, fez);
        float tx = (fex - mex) + ex, ty = (fey - mey) + ey, tz = (fez - mez) + ez;
        float gx = fx * fx, gy = fy * fy, gz = fz * fz;
        float gex = fmaf(fx, fx, -gx), gey = fmaf(fy, fy, -gy), gez = fmaf(fz, fz, -gz);
        float u1, v1, u2, v2, w, we;
        two_sum(gx, gy, u1, v1);
        two_sum(u1, gz, u2, v2);
        two_sum(r2, -u2, w, we);
        float dl = (we + qr) - (v1 + v2);
        dl = dl - ((gex + gey) + gez);
        dl = fmaf(-2.0f, fmaf(fx, tx, fmaf(fy, ty, fz * tz)), dl);
        discp = w + dl;
    } else {
        const float s = hb * R.inv_a;
        const float fx = fmaf(-s, R.d.x, hx);
        const float fy = fmaf(-s, R.d.y, hy);
        const float fz = fmaf(-s, R.d.z, hz);
        const float ff = fmaf(fx, fx, fmaf(fy, fy, fz * fz));
        discp = fmaf(r, r, -ff);
    }
    if (!(discp >= 0.0f)) return false;
    const float sd = sqrtf(R.a * discp);
    const float q = -(hb + copysignf(sd, hb));
    if (q == 0.0f) return false;
    const float ta = q * R.inv_a;
    const float tb = c / q;
    const float t0 = fminf(ta, tb), t1 = fmaxf(ta, tb);
    if (t0 >= tmin && t0 <= tmax) {
        tout = t0;
        return true;
    }
    if (t1 >= tmin && t1 <= tmax) {
        tout = t1;
        return true;
    }
    return false;
}

// ---------------------------------------------------------------------------
// Closest-hit traversal of the binary LBVH.
//
// Children are tested at their parent, from the parent's 64-byte record in
// the traversal layout (one contiguous 4 x float4 load): internal children by
// their box, leaf children directly by their sphere, stored inline.  The
// nearer hit child is descended; the farther one's index and entry distance
// go on a per-thread stack whose top kShared entries live in shared
// memory (ring buffer, layout [entry][thread] so a warp touches 32 distinct
// banks) and whose older entries spill to local memory.  Ties on t go to the
// smaller slot, so the result does not depend on traversal order.
// ---------------------------------------------------------------------------
constexpr int kShared = 8;   // shared-memory entries per thread (power of two)
constexpr int kSharedShallow = 4;  // the fused kernel's choice for shallow trees (small scenes)
constexpr int kSpill = 64;   // local-memory entries beyond those

struct StackSmem {
    int* node;   // [kShared][block]
    float* tn;   // [kShared][block]
};

// Counting builds only.  lane_steps / warp_steps: traversal steps summed over
// lanes, and over warps (one per step instruction the warp issues, with
// however many lanes are converged on it): their ratio / 32 is the SIMD
// utilisation of the traversal loop.
struct TraceCounters {
    uint32_t nodes, spheres, lane_steps, warp_steps;
};

// Adds a warp's counters to stats[1..4] (nodes, spheres, lane steps, warp
// steps); every lane of the warp calls it.
__device__ __forceinline__ void flush_counters(const TraceCounters& K, unsigned long long* stats) {
    unsigned long long a = K.nodes, b = K.spheres, c = K.lane_steps, d = K.warp_steps;
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off);
        b += __shfl_xor_sync(0xffffffffu, b, off);
        c += __shfl_xor_sync(0xffffffffu, c, off);
        d += __shfl_xor_sync(0xffffffffu, d, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(stats + 1, a);
        atomicAdd(stats + 2, b);
        atomicAdd(stats + 3, c);
        atomicAdd(stats + 4, d);
    }
}

// Per-lane traversal state.  begin() prepares a ray and tests the root;
// step() tests both children of the current node (from its 64-byte record in
// the traversal layout: boxes of internal children, spheres of leaf children
// inline) and descends or pops; both return whether more work remains.  The
// same state machine serves the one-ray-per-thread kernels (trace_closest)
// and the persistent kernels that refill idle lanes.
template <bool COUNT, bool AXIS = false, int KS = kShared>
struct Tracer {
    RayPre R;
    float tmin, tmax, best_t;
    int32_t best, cur;
    int sp;
    uint32_t guard;

    __device__ __forceinline__ void leaf(int32_t k, float4 s4, TraceCounters& K) {
        float t;
        if (COUNT) ++K.spheres;
        if (sphere_test(R, s4, tmin, tmax, t) && (t < best_t || (t == best_t && k < best))) {
            best_t = t;
            best = k;
        }
    }

    // Tested up front, with the whole warp converged: first the sphere the
    // ray leaves (R.from; its origin lies within r/16 of that surface, so its
    // test takes sphere_test's long refined branch, which in the walk would
    // run at a different step in each lane), then the huge hoisted spheres
    // (the ground) but that one.  Both are skipped during traversal, and
    // their hit distances already cull boxes behind them.  The closest hit
    // does not depend on the order of the tests.
    __device__ __forceinline__ void from_first(const SceneView& S, TraceCounters& K) {
        if (R.from >= 0) leaf(R.from, __ldg(S.sph + R.from), K);
        for (uint32_t h = 0; h < S.nhoist; ++h)
            if (S.hoist[h] != R.from) leaf(S.hoist[h], __ldg(S.sph + S.hoist[h]), K);
    }

    // R_ from prep(); its axis flag must equal AXIS.
    __device__ __forceinline__ bool begin(const SceneView& S, const RayPre& R_, float tmin_, float tmax_,
                                          TraceCounters& K) {
        R = R_;
        tmin = tmin_;
        tmax = tmax_;
        best_t = tmax_;
        best = kNone;
        sp = 0;
        const uint32_t n = S.n;
        if (n == 0) return false;
        from_first(S, K);
        if (n == 1) {
            if (R.from != 0) leaf(0, __ldg(S.sph), K);
            return false;
        }
        float tn;
        float4 rlo = __ldg(S.nodes + 0), rhi = __ldg(S.nodes + 1);
        if (COUNT) ++K.nodes;
        if (!box_test<AXIS>(R, rlo, rhi, tmin, best_t, tn)) return false;
        cur = 0;
        // A tree has n-1 internal nodes and each step expands a different one;
        // the guard turns a cyclic (corrupt) tree into an error flag instead
        // of a hang.
        guard = 2u * n + 8u;
        return true;
    }

    // spill / spill_tn: this thread's local-memory stack entries beyond the
    // kShared in shared memory.
    __device__ __forceinline__ bool step(const SceneView& S, StackSmem sm, uint32_t tid, uint32_t bdim,
                                         int* spill, float* spill_tn, bool& overflow, TraceCounters& K) {
        // Every word of the traversal records is in range (checked when the
        // records are written), so only termination needs guarding here.
        if (--guard == 0u) {
            overflow = true;
            return false;
        }
        if (COUNT) {
            ++K.lane_steps;
            const uint32_t am = __activemask();
            if ((tid & 31u) == (uint32_t)(__ffs(am) - 1)) ++K.warp_steps;
        }
        const float4* T = S.trav + 4 * (size_t)cur;
        const float4 a0 = __ldg(T), b0 = __ldg(T + 1), a1 = __ldg(T + 2), b1 = __ldg(T + 3);
        const int32_t w0 = __float_as_int(a0.w), w1 = __float_as_int(a1.w);
        bool h0 = false, h1 = false;
        float tn0 = 0.0f, tn1 = 0.0f;
        if (w0 & kLeaf) {
            if (!(w0 & kHoisted) && (w0 & kSlotMask) != R.from)
                leaf(w0 & kSlotMask, make_float4(a0.x, a0.y, a0.z, b0.x), K);
        } else {
            if (COUNT) ++K.nodes;
            h0 = box_test<AXIS>(R, a0, b0, tmin, best_t, tn0);
        }
        if (w1 & kLeaf) {
            if (!(w1 & kHoisted) && (w1 & kSlotMask) != R.from)
                leaf(w1 & kSlotMask, make_float4(a1.x, a1.y, a1.z, b1.x), K);
        } else {
            if (COUNT) ++K.nodes;
            h1 = box_test<AXIS>(R, a1, b1, tmin, best_t, tn1);
        }
        if (h0 && h1) {
            int32_t far;
            float far_tn;
            if (tn1 < tn0) {
                far = w0;
                far_tn = tn0;
                cur = w1;
            } else {
                far = w1;
                far_tn = tn1;
                cur = w0;
            }
            const uint32_t j = (uint32_t)(sp & (KS - 1)) * bdim + tid;
            if (sp >= KS) {
                const int g = sp - KS;
                if (g >= kSpill) {
                    overflow = true;
                    return false;
                }
                spill[g] = sm.node[j];
                spill_tn[g] = sm.tn[j];
            }
            sm.node[j] = far;
            sm.tn[j] = far_tn;
            ++sp;
            return true;
        }
        if (h0) {
            cur = w0;
            return true;
        }
        if (h1) {
            cur = w1;
            return true;
        }
        while (sp > 0) {
            --sp;
            const uint32_t j = (uint32_t)(sp & (KS - 1)) * bdim + tid;
            const int32_t e = sm.node[j];
            const float etn = sm.tn[j];
            if (sp >= KS) {
                sm.node[j] = spill[sp - KS];
                sm.tn[j] = spill_tn[sp - KS];
            }
            if (etn <= best_t) {
                cur = e;
                return true;
            }
        }
        return false;
    }

    __device__ __forceinline__ int32_t result(float& t) const {
        if (best == kNone) {
            t = tmax;
            return -1;
        }
        t = best_t;
        return best;
    }
};

// ---------------------------------------------------------------------------
// Closest-hit traversal of the wide tree (node layout in lbvh.cu).
//
// A step loads one node and tests all of its child boxes with the same
// instructions in every lane (structure-of-arrays loads, four children per
// float4), pushes the hit internal children but the nearest farthest first
// onto the same shared-memory / local-memory stack as the binary traversal
// (ordered by a sorting network on keys of entry distance and child number
// when more than two are hit), tests the spheres of the leaf children whose
// boxes were hit, then descends to the nearest child unless a sphere hit now
// culls it, else pops (popped entries are culled against the closest hit).
// ---------------------------------------------------------------------------
template <bool AXIS>
__device__ __forceinline__ bool box_test_s(const RayPre& R, float lx, float ly, float lz, float hx, float hy,
                                           float hz, float tmin, float tcap, float& tnear) {
    const f3 nh = AXIS ? R.n1 : R.n0;
    float t0x = fmaf(lx, R.inv.x, R.n0.x), t1x = fmaf(hx, R.inv.x, nh.x);
    float t0y = fmaf(ly, R.inv.y, R.n0.y), t1y = fmaf(hy, R.inv.y, nh.y);
    float t0z = fmaf(lz, R.inv.z, R.n0.z), t1z = fmaf(hz, R.inv.z, nh.z);
    float tn = fmax3(fminf(t0x, t1x), fminf(t0y, t1y), fmaxf(fminf(t0z, t1z), tmin));
    float tf = fmin3(fmaxf(t0x, t1x), fmaxf(t0y, t1y), fminf(fmaxf(t0z, t1z), tcap));
    tnear = tn;
    return AXIS ? tn <= tf * 1.00000095367431640625f : tn <= fmaf(tf, 1.00000095367431640625f, R.n1.x);
}

__device__ __forceinline__ void cswap(uint32_t& a, uint32_t& b) {
    const uint32_t lo = min(a, b), hi = max(a, b);
    a = lo;
    b = hi;
}

// Batcher's odd-even merge sort of 8 keys, ascending (19 comparators).
__device__ __forceinline__ void sort4(uint32_t k[4]) {
    cswap(k[0], k[1]); cswap(k[2], k[3]);
    cswap(k[0], k[2]); cswap(k[1], k[3]);
    cswap(k[1], k[2]);
}

__device__ __forceinline__ void sort8(uint32_t k[8]) {
    cswap(k[0], k[1]); cswap(k[2], k[3]); cswap(k[4], k[5]); cswap(k[6], k[7]);
    cswap(k[0], k[2]); cswap(k[1], k[3]); cswap(k[4], k[6]); cswap(k[5], k[7]);
    cswap(k[1], k[2]); cswap(k[5], k[6]);
    cswap(k[0], k[4]); cswap(k[1], k[5]); cswap(k[2], k[6]); cswap(k[3], k[7]);
    cswap(k[2], k[4]); cswap(k[3], k[5]);
    cswap(k[1], k[2]); cswap(k[3], k[4]); cswap(k[5], k[6]);
}

template <bool COUNT, bool AXIS = false, int KS = kShared>
struct WideTracer {
    RayPre R;
    float tmin, tmax, best_t;
    int32_t best, cur;
    int sp;
    uint32_t guard;

    __device__ __forceinline__ void leaf(int32_t k, float4 s4, TraceCounters& K) {
        float t;
        if (COUNT) ++K.spheres;
        if (sphere_test(R, s4, tmin, tmax, t) && (t < best_t || (t == best_t && k < best))) {
            best_t = t;
            best = k;
        }
    }

    // as Tracer::from_first
    __device__ __forceinline__ void from_first(const SceneView& S, TraceCounters& K) {
        if (R.from >= 0) leaf(R.from, __ldg(S.sph + R.from), K);
        for (uint32_t h = 0; h < S.nhoist; ++h)
            if (S.hoist[h] != R.from) leaf(S.hoist[h], __ldg(S.sph + S.hoist[h]), K);
    }

    __device__ __forceinline__ bool begin(const SceneView& S, const RayPre& R_, float tmin_, float tmax_,
                                          TraceCounters& K) {
        R = R_;
        tmin = tmin_;
        tmax = tmax_;
        best_t = tmax_;
        best = kNone;
        sp = 0;
        const uint32_t n = S.n;
        if (n == 0) return false;
        from_first(S, K);
        if (n == 1) {
            if (R.from != 0) leaf(0, __ldg(S.sph), K);
            return false;
        }
        float tn;
        float4 rlo = __ldg(S.nodes + 0), rhi = __ldg(S.nodes + 1);
        if (COUNT) ++K.nodes;
        if (!box_test<AXIS>(R, rlo, rhi, tmin, best_t, tn)) return false;
        cur = 0;
        // every wide node is expanded at most once per ray, and there are
        // fewer than n of them: the guard turns a cyclic tree into an error
        guard = n + 8u;
        return true;
    }

    __device__ __forceinline__ void push(StackSmem sm, uint32_t tid, uint32_t bdim, int* spill, float* spill_tn,
                                         bool& overflow, int32_t node, float tn) {
        const uint32_t j = (uint32_t)(sp & (KS - 1)) * bdim + tid;
        if (sp >= KS) {
            const int g = sp - KS;
            if (g >= kSpill) {
                overflow = true;
                return;
            }
            spill[g] = sm.node[j];
            spill_tn[g] = sm.tn[j];
        }
        sm.node[j] = node;
        sm.tn[j] = tn;
        ++sp;
    }

    __device__ __forceinline__ bool step(const SceneView& S, StackSmem sm, uint32_t tid, uint32_t bdim,
                                         int* spill, float* spill_tn, bool& overflow, TraceCounters& K) {
        if (--guard == 0u) {
            overflow = true;
            return false;
        }
        if (COUNT) {
            ++K.lane_steps;
            const uint32_t am = __activemask();
            if ((tid & 31u) == (uint32_t)(__ffs(am) - 1)) ++K.warp_steps;
        }
        const float4* N = S.wide + kWideF4 * (size_t)cur;
        const uint32_t masks = __float_as_uint(__ldg(N + 7 * kWideH).x);
        const uint32_t leafm = (masks >> 8) & 0xffu, intm = masks & ~leafm & 0xffu;
        // key of child c: its entry distance's bits with c in the low three
        // bits (distances are >= tmin > 0, so the bits order like the
        // values; the cut makes a key's distance a lower bound), all ones
        // unless it is a hit internal child
        uint32_t key[kWideW];
        uint32_t lhit = 0;
#pragma unroll
        for (int h = 0; h < kWideH; ++h) {
            const float4 lx = __ldg(N + h), hx = __ldg(N + kWideH + h);
            const float4 ly = __ldg(N + 2 * kWideH + h), hy = __ldg(N + 3 * kWideH + h);
            const float4 lz = __ldg(N + 4 * kWideH + h), hz = __ldg(N + 5 * kWideH + h);
            float t;
#define VENU_WIDE_CHILD(J, C)                                                                       \
    {                                                                                               \
        const bool ok = box_test_s<AXIS>(R, lx.C, ly.C, lz.C, hx.C, hy.C, hz.C, tmin, best_t, t); \
        lhit |= (uint32_t)ok << (J);                                                                \
        key[J] = (ok && ((intm >> (J)) & 1u)) ? ((__float_as_uint(t) & ~7u) | (uint32_t)(J)) : 0xffffffffu; \
    }
            VENU_WIDE_CHILD(4 * h + 0, x)
            VENU_WIDE_CHILD(4 * h + 1, y)
            VENU_WIDE_CHILD(4 * h + 2, z)
            VENU_WIDE_CHILD(4 * h + 3, w)
#undef VENU_WIDE_CHILD
        }
        lhit &= leafm;
        if (COUNT) K.nodes += (uint32_t)__popc(masks & 0xffu);
        const int32_t* words = reinterpret_cast<const int32_t*>(N + 6 * kWideH);
        // the hit internal children but the nearest onto the stack, farthest
        // first (one or two hits without sorting); the nearest is descended
        // unless the leaf tests below cull it
        uint32_t kmin = key[0];
#pragma unroll
        for (int c = 1; c < kWideW; ++c) kmin = min(kmin, key[c]);
        if (kmin != 0xffffffffu) {
            uint32_t nhit = 0;
#pragma unroll
            for (int c = 0; c < kWideW; ++c) nhit += key[c] != 0xffffffffu;
            if (nhit == 2u) {
                uint32_t kmax = 0;
#pragma unroll
                for (int c = 0; c < kWideW; ++c) kmax = key[c] != 0xffffffffu ? max(kmax, key[c]) : kmax;
                push(sm, tid, bdim, spill, spill_tn, overflow, __ldg(words + (kmax & 7u)),
                     __uint_as_float(kmax & ~7u));
            } else if (nhit > 2u) {
                if (kWideW == 8) sort8(key); else sort4(key);
#pragma unroll
                for (int i = kWideW - 1; i >= 1; --i) {
                    if (key[i] != 0xffffffffu)
                        push(sm, tid, bdim, spill, spill_tn, overflow, __ldg(words + (key[i] & 7u)),
                             __uint_as_float(key[i] & ~7u));
                }
            }
            if (overflow) return false;
        }
        // then the spheres of the hit leaf children, which may shorten the
        // ray and cull the pushed entries and the nearest child
        for (uint32_t lm = lhit; lm; lm &= lm - 1u) {
            const int32_t k = __ldg(words + (__ffs(lm) - 1)) & kSlotMask;
            if (k != R.from) leaf(k, __ldg(S.sph + k), K);
        }
        if (kmin != 0xffffffffu && __uint_as_float(kmin & ~7u) <= best_t) {
            cur = __ldg(words + (kmin & 7u));
            return true;
        }
        while (sp > 0) {
            --sp;
            const uint32_t j = (uint32_t)(sp & (KS - 1)) * bdim + tid;
            const int32_t e = sm.node[j];
            const float etn = sm.tn[j];
            if (sp >= KS) {
                sm.node[j] = spill[sp - KS];
                sm.tn[j] = spill_tn[sp - KS];
            }
            if (etn <= best_t) {
                cur = e;
                return true;
            }
        }
        return false;
    }

    __device__ __forceinline__ int32_t result(float& t) const {
        if (best == kNone) {
            t = tmax;
            return -1;
        }
        t = best_t;
        return best;
    }
};

template <bool COUNT, bool AXIS, int KS = kShared, bool WIDE = false>
__device__ __forceinline__ int32_t trace_closest_as(const SceneView& S, const RayPre& R, float tmin,
                                                    float tmax, float& t_out, StackSmem sm,
                                                    uint32_t tid, uint32_t bdim, bool& overflow,
                                                    TraceCounters& K) {
    typename std::conditional<WIDE, WideTracer<COUNT, AXIS, KS>, Tracer<COUNT, AXIS, KS>>::type T;
    int spill[kSpill];
    float spill_tn[kSpill];
    if (T.begin(S, R, tmin, tmax, K))
        while (T.step(S, sm, tid, bdim, spill, spill_tn, overflow, K)) {
        }
    return T.result(t_out);
}

// Closest hit of one ray (R from prep): the shared-margin loop, or the
// per-axis one for the rare near-axis-parallel ray.  KS: shared-memory stack
// entries per thread (the kernel's StackSmem holds KS of them).
template <bool COUNT, int KS = kShared, bool WIDE = false>
__device__ __forceinline__ int32_t trace_closest(const SceneView& S, const RayPre& R, float tmin,
                                                 float tmax, float& t_out, StackSmem sm,
                                                 uint32_t tid, uint32_t bdim, bool& overflow,
                                                 TraceCounters& K) {
    if (R.axis)
        return trace_closest_as<COUNT, true, KS, WIDE>(S, R, tmin, tmax, t_out, sm, tid, bdim, overflow, K);
    return trace_closest_as<COUNT, false, KS, WIDE>(S, R, tmin, tmax, t_out, sm, tid, bdim, overflow, K);
}

// ---------------------------------------------------------------------------
// Path state in the wavefront queues (48 bytes per path; 52 in the batch
// engine):
//   o4 = {origin.xyz, slot (int bits)}
//   d4 = {direction.xyz, remaining depth (bits 0-7) | job index (batch
//         engine) or 1 + slot of the sphere the ray leaves (single-scene
//         renderer) (bits 8-31)}
//   t4 = {throughput.rgb, bounce seed (uint bits)}
//   from = the batch engine's slot of the sphere the ray leaves
//          (RayPre::from), -1 for a camera ray; null in the single-scene
//          renderer
// ---------------------------------------------------------------------------
struct Queue {
    float4* o;
    float4* d;
    float4* t;
    int32_t* from;
};

}  // namespace venu
