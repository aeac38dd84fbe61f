// render_kernels.cuh -- wavefront stages shared by the plain single-scene
// renderer and the batched multi-scene renderer.
#pragma once

#include "venu_device.cuh"

namespace venu {

// Per-sample camera ray into a queue entry (Core/RayTracer.cu:163-202 up to
// optixTrace).  The bounce seed is the raygen seed after the sample's jitter
// and lens draws; the raygen seed continues from that same state to the next
// sample (the reference copies it into the PRD and never copies it back).
// d4.w packs the remaining depth (low 8 bits) and, above it, the job index
// in the batch engine, or 1 + the slot of the sphere the ray leaves in the
// single-scene renderer (0 for a camera ray; see packed_from).
constexpr uint32_t kDepthMask = 0xFFu;
__device__ __forceinline__ void write_primary(const Queue& q, uint32_t pos, f3 o, f3 d, uint32_t slot,
                                              int depth, uint32_t seed, uint32_t job = 0) {
    q.o[pos] = make_float4(o.x, o.y, o.z, __int_as_float((int)slot));
    q.d[pos] = make_float4(d.x, d.y, d.z, __uint_as_float((job << 8) | ((uint32_t)depth & kDepthMask)));
    q.t[pos] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(seed));
}

// The sphere a continuing ray leaves (RayPre::from) is carried for slots up
// to kFromMax: 1 + slot fits the 24 bits above the depth in d4.w.  A ray
// leaving a sphere of a larger slot carries none and meets that sphere in
// the walk instead (same closest hit).  The single-scene renderer keeps it
// in d4.w (its queue entry stays 48 bytes; a separate 4-byte array measured
// 1-4 % slower); the batch engine, whose d4.w holds the job index, in
// Queue::from.
constexpr uint32_t kFromMax = (1u << 24) - 2u;
__device__ __forceinline__ int32_t from_of_hit(int32_t k) { return (uint32_t)k <= kFromMax ? k : -1; }
__device__ __forceinline__ int32_t packed_from(float d4w) { return (int32_t)(__float_as_uint(d4w) >> 8) - 1; }

__device__ __forceinline__ DevCamera load_camera(const venu_camera& c) {
    DevCamera k;
    k.origin = mk(c.origin[0], c.origin[1], c.origin[2]);
    k.u = mk(c.u[0], c.u[1], c.u[2]);
    k.v = mk(c.v[0], c.v[1], c.v[2]);
    k.w = mk(c.w[0], c.w[1], c.w[2]);
    k.un = normalize(k.u);
    k.vn = normalize(k.v);
    k.lens = c.lens_radius;
    return k;
}

// Division of x < 2^31 by an invariant d (1 <= d <= 2^30) as a multiply and a
// shift (Granlund & Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994, with N = 31): l = ceil(log2 d),
// m = floor(2^(31+l) / d) + 1 < 2^32, and x / d = (x m) >> (31 + l) exactly.
struct FastDiv {
    uint32_t m, shift;
};

__host__ __device__ inline FastDiv make_fastdiv(uint32_t d) {
    uint32_t l = 0;
    while (l < 31u && (1u << l) < d) ++l;
    FastDiv f;
    f.m = (uint32_t)((1ull << (31u + l)) / d + 1ull);
    f.shift = 31u + l;
    return f;
}

__device__ __forceinline__ uint32_t fast_div(uint32_t x, FastDiv f) {
    return (uint32_t)(((unsigned long long)x * f.m) >> f.shift);
}

// The primary rays of one wave of the single-scene renderer, made inside the
// fused kernel from each path's raygen seed (k_raygen writes only the seeds):
// the same queue entry as write_primary, without the round trip through
// memory.  path_seeds == nullptr: rays come from the queue.
struct PrimaryGen {
    venu_camera cam;
    const uint32_t* path_seeds;  // [k * P], path pos = s * P + pl
    uint32_t W, H, p0, P;
    int depth;                   // max_depth - 1
    FastDiv div_P, div_W;        // make_fastdiv(P), make_fastdiv(W)
    uint32_t in_place_factor;    // venu_tuning.in_place_factor (>= 1)
};

// C: load_camera(g.cam), made once per block
__device__ __forceinline__ void gen_primary(const PrimaryGen& g, const DevCamera& C, uint32_t pos, float4& o4,
                                            float4& d4, uint32_t& seed) {
    const uint32_t s = fast_div(pos, g.div_P);
    const uint32_t pix = g.p0 + (pos - s * g.P);
    const uint32_t y = fast_div(pix, g.div_W);
    seed = g.path_seeds[pos];
    f3 o, d;
    camera_ray(C, pix - y * g.W, y, g.W, g.H, seed, o, d);
    o4 = make_float4(o.x, o.y, o.z, __int_as_float((int)pos));
    d4 = make_float4(d.x, d.y, d.z, __uint_as_float((uint32_t)g.depth & kDepthMask));
}

struct ShadeOut {
    bool cont;
    float4 o, d, t;   // next queue entry when cont
    int32_t from;     // the sphere the next ray leaves (from_of_hit of the hit)
    float4 result;    // final path radiance when !cont
};

// One hit/miss record -> scatter (Core/RayTracer.cu:272-449, iterative):
// forward throughput, black at depth 0 or on metal absorption, sky on miss.
// PACK_FROM (single-scene renderer): the next ray's d4.w carries `from`
// above the depth; otherwise it keeps the job index there.
template <bool PACK_FROM>
__device__ __forceinline__ ShadeOut shade_one(const SceneView& S, float4 o4, float4 d4, float4 t4, int2 h) {
    ShadeOut out;
    out.cont = false;
    f3 o = mk(o4.x, o4.y, o4.z), d = mk(d4.x, d4.y, d4.z);
    const uint32_t dbits = __float_as_uint(d4.w);
    int depth = (int)(dbits & kDepthMask);
    f3 T = mk(t4.x, t4.y, t4.z);
    uint32_t seed = __float_as_uint(t4.w);
    if (h.y < 0) {
        f3 L = T * sky(d);
        out.result = make_float4(L.x, L.y, L.z, 0.0f);
        return out;
    }
    if (!(depth > 0)) {
        out.result = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return out;
    }
    const int k = h.y;
    const float t = __int_as_float(h.x);
    float4 sp = __ldg(S.sph + k);
    float4 m = __ldg(S.mat + k);
    uint32_t type = __ldg(S.meta + k) >> 30;
    f3 C = mk(sp.x, sp.y, sp.z);
    f3 p = o + d * t;
    f3 outward = divs(p - C, sp.w);
    bool front = dot(d, outward) < 0.0f;
    f3 n = front ? outward : -outward;
    f3 dir;
    if (type <= 1u) {
        // Lambertian and metal draw one point in the unit ball each; one call
        // serves both, so a warp holding both kinds runs the rejection loop
        // once instead of once per branch (each ray draws the same values)
        const f3 u = random_in_unit_sphere(seed);
        if (type == 0u) {
            dir = n + normalize(u);
            if (near_zero(dir)) dir = n;
        } else {
            dir = reflect(normalize(d), n) + m.w * u;
            if (!(dot(dir, n) > 0.0f)) {
                out.result = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                return out;
            }
        }
        T = T * mk(m.x, m.y, m.z);
    } else {
        float ratio = front ? (1.0f / m.w) : m.w;
        f3 ud = normalize(d);
        float cos_t = fminf(dot(-ud, n), 1.0f);
        float sin_t = sqrtf(1.0f - cos_t * cos_t);
        bool cannot = ratio * sin_t > 1.0f;
        if (cannot || reflectance(cos_t, ratio) > rnd(seed))
            dir = reflect(ud, n);
        else
            dir = refract(ud, n, ratio);
    }
    out.cont = true;
    out.from = from_of_hit(k);
    out.o = make_float4(p.x, p.y, p.z, o4.w);
    const uint32_t high = PACK_FROM ? (uint32_t)(out.from + 1) << 8 : (dbits & ~kDepthMask);
    out.d = make_float4(dir.x, dir.y, dir.z, __uint_as_float(high | (uint32_t)(depth - 1)));
    out.t = make_float4(T.x, T.y, T.z, __uint_as_float(seed));
    return out;
}

// Warp-aggregated append: one atomic per warp, positions from the ballot.
__device__ __forceinline__ uint32_t warp_append(bool pred, uint32_t* counter) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t m = __ballot_sync(0xffffffffu, pred);
    uint32_t base = 0;
    if (lane == 0 && m) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    return base + (uint32_t)__popc(m & ((1u << lane) - 1u));
}

// Kahan-compensated add of one sample into {sum.rgb, n} {comp.rgb, 0}.
__device__ __forceinline__ void kahan_add(float4& a0, float4& a1, float4 v) {
    float y, t;
    y = v.x - a1.x; t = a0.x + y; a1.x = (t - a0.x) - y; a0.x = t;
    y = v.y - a1.y; t = a0.y + y; a1.y = (t - a0.y) - y; a0.y = t;
    y = v.z - a1.z; t = a0.z + y; a1.z = (t - a0.z) - y; a0.z = t;
    a0.w = a0.w + 1.0f;
}

// Core/RayTracer.cu:16-47: clamp, sRGB (x^(1/2.4) by srgb_pow in place of
// powf), x*256 truncated.
__device__ __forceinline__ unsigned char quant8(float x) {
    x = fmaxf(0.0f, fminf(x, 1.0f));
    uint32_t q = (uint32_t)(x * 256.0f);
    return (unsigned char)min(q, 255u);
}
__device__ __forceinline__ uchar4 make_color(f3 c) {
    float v[3] = {fmaxf(0.0f, fminf(c.x, 1.0f)), fmaxf(0.0f, fminf(c.y, 1.0f)), fmaxf(0.0f, fminf(c.z, 1.0f))};
    unsigned char q[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float srgb = v[i] < 0.0031308f ? 12.92f * v[i] : 1.055f * srgb_pow(v[i]) - 0.055f;
        q[i] = quant8(srgb);
    }
    return make_uchar4(q[0], q[1], q[2], 255);
}

}  // namespace venu
