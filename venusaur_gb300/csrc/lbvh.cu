// lbvh.cu -- linear BVH over spheres, built on the device.
//
// Replaces Renderer::BuildAccelerationStructures (Core/Renderer.h:160-255):
//   1. centroid bounds (order-preserving integer atomics: exact min/max),
//   2. 30-bit Morton codes of the centroids quantised to 10 bits per axis,
//   3. stable LSD radix sort of (code, original index), 4 passes of 8 bits,
//      one warp per 512-key tile, stable ranking with __match_any_sync,
//   4. Karras 2012 hierarchy ("Maximizing Parallelism in the Construction of
//      BVHs, Octrees, and k-d Trees"), ties on equal codes broken by index,
//   5. bottom-up refit with per-node arrival counters; leaf boxes are the
//      sphere AABBs rounded outward (__fsub_rd / __fadd_ru, |radius|),
//   6. gather of spheres and materials into Morton (slot) order.
// Every step is integer work or exact float min/max, so the result is
// bit-identical to a host build of the same algorithm.
#include "venu_device.cuh"
#include "venu_internal.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace venu {
namespace {

constexpr int kTileKeys = 512;  // keys per warp tile
constexpr int kWarpsPerBlock = 8;
constexpr int kRadixBits = 8;
constexpr int kBuckets = 1 << kRadixBits;

__device__ __forceinline__ uint32_t f2u(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float u2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Build-time control block: centroid bounds (order-preserving encoded),
// the bounds used for quantisation, and the hoisted-sphere list.
struct LbvhCtl {
    uint32_t b0[6];       // all centroids: lo.xyz, hi.xyz
    float bounds[6];      // the same bounds as floats
    uint32_t hoist_cnt;   // huge spheres found
    uint32_t nhoist;      // hoisted (<= kMaxHoisted), 0 if more than kHoistCandidates
    int32_t hoist[kMaxHoisted];
    uint32_t hoist_buf[64];
    uint32_t bad_words;   // child words k_trav_layout had to replace (never, for a sound build)
};
constexpr uint32_t kHoistCandidates = 64;

// A sphere is huge when its radius exceeds a quarter of the largest extent of
// all centroids (the r = 1000 ground sphere of the RTIOW scene).
__device__ __forceinline__ float huge_threshold(const uint32_t* b0) {
    float m = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) m = fmaxf(m, u2f(b0[3 + a]) - u2f(b0[a]));
    return 0.25f * m;
}

__global__ void k_lbvh_init(LbvhCtl* c) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        for (int a = 0; a < 3; ++a) {
            c->b0[a] = 0xffffffffu;
            c->b0[3 + a] = 0u;
        }
        c->hoist_cnt = 0;
        c->nhoist = 0;
        c->bad_words = 0;
    }
}

// Centroid bounds (exact min/max through order-preserving integer atomics).
__global__ void k_bounds(const venu_sphere* __restrict__ s, uint32_t n, uint32_t* __restrict__ bu) {
    uint32_t lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0, 0, 0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            uint32_t u = f2u(s[i].center[a]);
            lo[a] = min(lo[a], u);
            hi[a] = max(hi[a], u);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            lo[a] = min(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], off));
            hi[a] = max(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], off));
        }
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            atomicMin(bu + a, lo[a]);
            atomicMax(bu + 3 + a, hi[a]);
        }
    }
}

// Karras's bit spreading: bit i of v goes to bit 3i.
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3ffu;
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
__device__ __forceinline__ uint32_t quant10(float c, float lo, float ext) {
    if (!(ext > 0.0f)) return 0;
    float t = (c - lo) / ext;
    float f = t * 1024.0f;
    f = fminf(fmaxf(f, 0.0f), 1023.0f);
    return (uint32_t)f;
}

// Morton codes quantised to the centroid bounds with one scale for all three
// axes (the largest extent), so cells stay cubic: a flat scene is split flat
// instead of its thin axis being stretched over 1024 levels.  (Measured on
// the oracle: 27 % fewer box tests per segment on a 200 000-sphere scene and
// 18 % on 1 M spheres than per-axis scaling, equal on the RTIOW scene.)
__global__ void k_morton(const venu_sphere* __restrict__ s, uint32_t n, LbvhCtl* c, uint32_t* __restrict__ keys,
                         uint32_t* __restrict__ vals) {
    const uint32_t* bu = c->b0;
    float lo[3], ext = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = u2f(bu[a]);
        float hi = u2f(bu[3 + a]);
        ext = fmaxf(ext, hi - lo[a]);
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            c->bounds[a] = lo[a];
            c->bounds[3 + a] = hi;
        }
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t qx = quant10(s[i].center[0], lo[0], ext);
        uint32_t qy = quant10(s[i].center[1], lo[1], ext);
        uint32_t qz = quant10(s[i].center[2], lo[2], ext);
        keys[i] = (spread10(qx) << 2) | (spread10(qy) << 1) | spread10(qz);
        vals[i] = i;
    }
}

// Huge spheres in slot order -> candidates (unordered, at most 64).
__global__ void k_hoist_collect(const float4* __restrict__ sph, uint32_t n, LbvhCtl* c) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float thr = huge_threshold(c->b0);
    if (fabsf(sph[k].w) > thr) {
        const uint32_t i = atomicAdd(&c->hoist_cnt, 1u);
        if (i < kHoistCandidates) c->hoist_buf[i] = k;
    }
}

// The (at most 4) lowest huge slots are hoisted and their leaf words flagged;
// with more than 64 huge spheres nothing is hoisted (deterministically).
__global__ void k_hoist_finalize(LbvhCtl* c, const int32_t* __restrict__ pleaf, float4* nodes, uint32_t n) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const uint32_t cnt = c->hoist_cnt;
    if (cnt == 0 || cnt > kHoistCandidates) {
        c->nhoist = 0;
        return;
    }
    uint32_t buf[kHoistCandidates];
    for (uint32_t i = 0; i < cnt; ++i) buf[i] = c->hoist_buf[i];
    for (uint32_t i = 1; i < cnt; ++i) {  // insertion sort
        uint32_t v = buf[i], j = i;
        while (j > 0 && buf[j - 1] > v) {
            buf[j] = buf[j - 1];
            --j;
        }
        buf[j] = v;
    }
    const uint32_t nh = cnt < (uint32_t)kMaxHoisted ? cnt : (uint32_t)kMaxHoisted;
    for (uint32_t i = 0; i < nh; ++i) {
        const uint32_t k = buf[i];
        const int32_t p = pleaf[k];
        c->hoist[i] = (int32_t)k;
        if (p < 0 || (uint32_t)p >= n - 1) continue;
        const int32_t want = (int32_t)k | kLeaf;
        if (__float_as_int(nodes[2 * p].w) == want)
            nodes[2 * p].w = __int_as_float(want | kHoisted);
        else if (__float_as_int(nodes[2 * p + 1].w) == want)
            nodes[2 * p + 1].w = __int_as_float(want | kHoisted);
    }
    c->nhoist = nh;
}

// Per-tile digit histogram, digit-major: hist[d * ntiles + tile].
__global__ void k_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift, uint32_t ntiles,
                       uint32_t* __restrict__ hist) {
    __shared__ uint32_t cnt[kWarpsPerBlock][kBuckets];
    const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t tile = blockIdx.x * kWarpsPerBlock + w;
    for (int d = lane; d < kBuckets; d += 32) cnt[w][d] = 0;
    __syncwarp();
    if (tile < ntiles) {
        for (int j = 0; j < kTileKeys / 32; ++j) {
            uint32_t idx = tile * kTileKeys + j * 32 + lane;
            if (idx < n) atomicAdd(&cnt[w][(keys[idx] >> shift) & (kBuckets - 1)], 1u);
        }
        __syncwarp();
        for (int d = lane; d < kBuckets; d += 32) hist[(size_t)d * ntiles + tile] = cnt[w][d];
    }
}

// Exclusive scan of `total` counters in place (one block of 1024 threads).
__global__ void k_scan(uint32_t* __restrict__ a, uint32_t total) {
    __shared__ uint32_t part[1024];
    const uint32_t t = threadIdx.x;
    const uint32_t per = (total + blockDim.x - 1) / blockDim.x;
    const uint32_t b = t * per, e = min(total, b + per);
    uint32_t sum = 0;
    for (uint32_t i = b; i < e; ++i) sum += a[i];
    part[t] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < blockDim.x; off <<= 1) {
        uint32_t v = t >= off ? part[t - off] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = part[t] - sum;  // exclusive prefix of this thread's chunk
    for (uint32_t i = b; i < e; ++i) {
        uint32_t v = a[i];
        a[i] = run;
        run += v;
    }
}

// Stable scatter: keys of a tile are ranked in tile order within their digit.
__global__ void k_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t n,
                          int shift, uint32_t ntiles, const uint32_t* __restrict__ offs,
                          uint32_t* __restrict__ kout, uint32_t* __restrict__ vout) {
    __shared__ uint32_t base[kWarpsPerBlock][kBuckets];
    const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t tile = blockIdx.x * kWarpsPerBlock + w;
    if (tile >= ntiles) return;  // whole warp leaves together
    for (int d = lane; d < kBuckets; d += 32) base[w][d] = offs[(size_t)d * ntiles + tile];
    __syncwarp();
    const uint32_t lt = (1u << lane) - 1u;
    for (int j = 0; j < kTileKeys / 32; ++j) {
        uint32_t idx = tile * kTileKeys + j * 32 + lane;
        bool valid = idx < n;
        uint32_t k = valid ? kin[idx] : 0u;
        uint32_t d = valid ? ((k >> shift) & (kBuckets - 1)) : (uint32_t)kBuckets + lane;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t rank = __popc(peers & lt);
        uint32_t pos = valid ? base[w][d] + rank : 0u;
        __syncwarp();
        if (valid && rank == 0) base[w][d] += __popc(peers);
        __syncwarp();
        if (valid) {
            kout[pos] = k;
            vout[pos] = vin[idx];
        }
    }
}

__device__ __forceinline__ int delta(const uint32_t* __restrict__ k, int n, int i, int j) {
    if (j < 0 || j > n - 1) return -1;
    uint32_t a = k[i], b = k[j];
    if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clz(a ^ b);
}

// One thread per internal node i in [0, n-2].
__global__ void k_karras(const uint32_t* __restrict__ keys, int n, float4* __restrict__ nodes,
                         int32_t* __restrict__ parent_int, int32_t* __restrict__ parent_leaf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(keys, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;  // ceil(l/2), ceil(l/4), ..., 1
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * d + min(d, 0);
    int left = (min(i, j) == gamma) ? (gamma | kLeaf) : gamma;
    int right = (max(i, j) == gamma + 1) ? ((gamma + 1) | kLeaf) : gamma + 1;
    nodes[2 * i].w = __int_as_float(left);
    nodes[2 * i + 1].w = __int_as_float(right);
    if (left & kLeaf) parent_leaf[left & ~kLeaf] = i; else parent_int[left] = i;
    if (right & kLeaf) parent_leaf[right & ~kLeaf] = i; else parent_int[right] = i;
    if (i == 0) parent_int[0] = -1;
}

// Leaf boxes + bottom-up refit.  The second thread to arrive at a node
// computes its box; a __threadfence before each arrival publishes the
// children's boxes, and they are read back through L2 (__ldcg).
// ids[k] & id_mask = original index of the sphere in slot k (the sorted
// values during a build, the meta words during a refit of moved spheres).
// Leaf words may carry the hoisted flag (refit after a build).
__global__ void k_refit(const venu_sphere* __restrict__ s, const uint32_t* __restrict__ ids, uint32_t id_mask, int n,
                        float4* nodes, const int32_t* __restrict__ parent_int,
                        const int32_t* __restrict__ parent_leaf, float4* leafbox,
                        uint32_t* __restrict__ arrive) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const venu_sphere& sp = s[ids[k] & id_mask];
    float r = fabsf(sp.radius);
    // An exactly-zero difference rounds down to -0.0; "+ 0.0f" makes it +0.0
    // (still a lower bound) so boxes never carry a signed zero.
    float4 lo = make_float4(__fsub_rd(sp.center[0], r) + 0.0f, __fsub_rd(sp.center[1], r) + 0.0f,
                            __fsub_rd(sp.center[2], r) + 0.0f, 0.0f);
    float4 hi = make_float4(__fadd_ru(sp.center[0], r), __fadd_ru(sp.center[1], r), __fadd_ru(sp.center[2], r), 0.0f);
    leafbox[2 * k] = lo;
    leafbox[2 * k + 1] = hi;
    int p = parent_leaf[k];
    // A Karras tree over unique (code, index) keys is at most 63 levels deep;
    // the bound only guards against a corrupt parent chain.
    for (int level = 0; p >= 0 && p < n - 1 && level < 128; ++level) {
        __threadfence();
        if (atomicAdd(arrive + p, 1u) == 0u) return;
        __threadfence();
        int32_t cl = __float_as_int(__ldcg(&nodes[2 * p].w));
        int32_t cr = __float_as_int(__ldcg(&nodes[2 * p + 1].w));
        const bool ok_l = (cl & kLeaf) ? (cl & kSlotMask) < n : cl < n - 1;
        const bool ok_r = (cr & kLeaf) ? (cr & kSlotMask) < n : cr < n - 1;
        if (!ok_l || !ok_r) return;
        float4 l0 = (cl & kLeaf) ? __ldcg(leafbox + 2 * (cl & kSlotMask)) : __ldcg(nodes + 2 * cl);
        float4 h0 = (cl & kLeaf) ? __ldcg(leafbox + 2 * (cl & kSlotMask) + 1) : __ldcg(nodes + 2 * cl + 1);
        float4 l1 = (cr & kLeaf) ? __ldcg(leafbox + 2 * (cr & kSlotMask)) : __ldcg(nodes + 2 * cr);
        float4 h1 = (cr & kLeaf) ? __ldcg(leafbox + 2 * (cr & kSlotMask) + 1) : __ldcg(nodes + 2 * cr + 1);
        nodes[2 * p] = make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), __int_as_float(cl));
        nodes[2 * p + 1] = make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), __int_as_float(cr));
        p = parent_int[p];
    }
}

// ---------------------------------------------------------------------------
// Treelet restructuring (Karras & Aila, HPG 2013), one bottom-up pass after
// the refit: at every internal node N, once both of its subtrees are final,
// a treelet of up to 7 leaves is grown from N's children by opening the
// internal treelet leaf with the largest surface area (first on ties); a
// dynamic program over the 2^7 subsets finds the topology with the least
// total internal surface area, and the treelet is rewired that way if that
// is strictly less than its current total.  Leaves keep their Morton slots,
// N stays the treelet root, the treelet's internal nodes are reused in the
// order they were opened and handed out in depth-first order of the new
// topology.  Same arithmetic, same order as the host LBVH of the oracle, so
// the tree stays bit-exact.  One thread per leaf walks up as in k_refit;
// the second thread to reach a node restructures it.
// ---------------------------------------------------------------------------
constexpr int kTreeletLeaves = 7;

struct TBox {
    float lo[3], hi[3];
};

__device__ __forceinline__ float tbox_area(const TBox& b) {
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return 2.0f * ((dx * dy + dy * dz) + dz * dx);
}

__device__ __forceinline__ TBox tbox_of(const float4* nodes, const float4* leafbox, int32_t c) {
    const float4 lo = (c & kLeaf) ? __ldcg(leafbox + 2 * (c & kSlotMask)) : __ldcg(nodes + 2 * c);
    const float4 hi = (c & kLeaf) ? __ldcg(leafbox + 2 * (c & kSlotMask) + 1) : __ldcg(nodes + 2 * c + 1);
    TBox b;
    b.lo[0] = lo.x;
    b.lo[1] = lo.y;
    b.lo[2] = lo.z;
    b.hi[0] = hi.x;
    b.hi[1] = hi.y;
    b.hi[2] = hi.z;
    return b;
}

__device__ __forceinline__ int32_t child_word(const float4* nodes, int32_t p, int side) {
    return __float_as_int(__ldcg(&nodes[2 * p + side].w));
}

// Restructures the treelet rooted at N with the whole warp.  The treelet's
// entries are spread over lanes 0..6 (lane i holds entry i), so every
// memory round trip serves all entries at once: the growth step reads the
// open entries' boxes in parallel and picks the largest area (first on
// ties) with a warp reduction; the DP's subsets of one size are shared out
// over the lanes (each subset's cost computed exactly as a single thread
// would: the same members in the same order, the same partition order and
// tie rule); lane 0 rewires the treelet, and each rewired node's box is the
// union of its subset's entry boxes (min / max are exact, so this equals
// refitting it from its children).  Every lane of the warp calls it with
// the same N.  cost / split: this warp's shared-memory DP tables.
__device__ void restructure_treelet_warp(int32_t N, int n, float4* nodes, int32_t* parent_int,
                                         int32_t* parent_leaf, const float4* leafbox, float* cost,
                                         uint8_t* split) {
    const int lane = threadIdx.x & 31;
    int32_t internals[kTreeletLeaves - 1];
    int nl = 2, ni = 0;
    int32_t mine = lane < 2 ? child_word(nodes, N, lane) : 0;  // entry `lane` of the treelet
    internals[ni++] = N;
    bool bad = false;
    while (nl < kTreeletLeaves) {
        float a = -1.0f;
        if (lane < nl && !(mine & kLeaf)) a = tbox_area(tbox_of(nodes, leafbox, mine));
        float ba = a;
        int bi = lane;
        for (int off = 16; off > 0; off >>= 1) {
            const float oa = __shfl_xor_sync(0xffffffffu, ba, off);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (oa > ba || (oa == ba && oi < bi)) {
                ba = oa;
                bi = oi;
            }
        }
        if (ba < 0.0f) break;  // no internal entry left
        const int32_t c = __shfl_sync(0xffffffffu, mine, bi);
        if ((uint32_t)c >= (uint32_t)(n - 1)) {  // never for a sound tree
            bad = true;
            break;
        }
        internals[ni++] = c;
        if (lane == bi) mine = child_word(nodes, c, 0);
        if (lane == nl) mine = child_word(nodes, c, 1);
        ++nl;
    }
    const bool my_bad = lane < nl && ((mine & kLeaf) ? (mine & kSlotMask) >= n : (uint32_t)mine >= (uint32_t)(n - 1));
    if (__any_sync(0xffffffffu, my_bad)) bad = true;
    if (bad || nl < 3) return;  // the same decision in every lane
    const int full = (1 << nl) - 1;
    TBox bx[kTreeletLeaves];
    {
        TBox b{};
        if (lane < nl) b = tbox_of(nodes, leafbox, mine);
        for (int i = 0; i < nl; ++i)
            for (int ax = 0; ax < 3; ++ax) {
                bx[i].lo[ax] = __shfl_sync(0xffffffffu, b.lo[ax], i);
                bx[i].hi[ax] = __shfl_sync(0xffffffffu, b.hi[ax], i);
            }
    }
    for (int S = 1 + lane; S <= full; S += 32)
        if ((S & (S - 1)) == 0) {
            cost[S] = 0.0f;
            split[S] = 0;
        }
    for (int k = 2; k <= nl; ++k) {
        __syncwarp();
        for (int S = 1 + lane; S <= full; S += 32) {
            if (__popc(S) != k) continue;
            TBox u;
            for (int ax = 0; ax < 3; ++ax) {
                u.lo[ax] = INFINITY;
                u.hi[ax] = -INFINITY;
            }
            for (int i = 0; i < nl; ++i)
                if (S >> i & 1)
                    for (int ax = 0; ax < 3; ++ax) {
                        u.lo[ax] = fminf(u.lo[ax], bx[i].lo[ax]);
                        u.hi[ax] = fmaxf(u.hi[ax], bx[i].hi[ax]);
                    }
            const float area = tbox_area(u);
            const int low = S & -S, rest = S ^ low;
            float bc = INFINITY;
            int bp = 0;
            for (int Q = (rest - 1) & rest;; Q = (Q - 1) & rest) {  // the subsets of rest but rest, largest first
                const int P = Q | low;
                const float c = cost[P] + cost[S ^ P];
                if (c < bc) {
                    bc = c;
                    bp = P;
                }
                if (Q == 0) break;
            }
            cost[S] = area + bc;
            split[S] = (uint8_t)bp;
        }
    }
    __syncwarp();
    // the treelet's current internal area, summed in the same order as a
    // single thread would (internals[0], [1], ...)
    float my_area = 0.0f;
    {
        int32_t my_int = 0;
        for (int i = 0; i < ni; ++i)
            if (lane == i) my_int = internals[i];
        if (lane < ni) my_area = tbox_area(tbox_of(nodes, leafbox, my_int));
    }
    float current = 0.0f;
    for (int i = 0; i < ni; ++i) current = current + __shfl_sync(0xffffffffu, my_area, i);
    const bool better = cost[full] < current;
    int32_t L[kTreeletLeaves];
    for (int i = 0; i < nl; ++i) L[i] = __shfl_sync(0xffffffffu, mine, i);
    __syncwarp();
    if (better && lane == 0) {
        // order[i]: the subset of the i-th internal node in depth-first
        // preorder; it is given internals[i]
        int order[kTreeletLeaves - 1];
        int no = 0;
        {
            int stack[kTreeletLeaves];
            int sp = 0;
            stack[sp++] = full;
            while (sp > 0) {
                const int S = stack[--sp];
                if ((S & (S - 1)) == 0) continue;
                order[no++] = S;
                stack[sp++] = S ^ split[S];
                stack[sp++] = split[S];
            }
        }
        auto word = [&](int T) -> int32_t {
            if ((T & (T - 1)) == 0) return L[__ffs(T) - 1];
            for (int i = 0; i < no; ++i)
                if (order[i] == T) return internals[i];
            return internals[0];  // unreachable: every internal subset is in order[]
        };
        for (int i = 0; i < no; ++i) {
            const int S = order[i];
            const int32_t me = internals[i];
            const int32_t l = word(split[S]), r = word(S ^ split[S]);
            TBox u;
            for (int ax = 0; ax < 3; ++ax) {
                u.lo[ax] = INFINITY;
                u.hi[ax] = -INFINITY;
            }
            for (int j = 0; j < nl; ++j)
                if (S >> j & 1)
                    for (int ax = 0; ax < 3; ++ax) {
                        u.lo[ax] = fminf(u.lo[ax], bx[j].lo[ax]);
                        u.hi[ax] = fmaxf(u.hi[ax], bx[j].hi[ax]);
                    }
            nodes[2 * me] = make_float4(u.lo[0], u.lo[1], u.lo[2], __int_as_float(l));
            nodes[2 * me + 1] = make_float4(u.hi[0], u.hi[1], u.hi[2], __int_as_float(r));
            if (l & kLeaf) parent_leaf[l & kSlotMask] = me;
            else parent_int[l] = me;
            if (r & kLeaf) parent_leaf[r & kSlotMask] = me;
            else parent_int[r] = me;
        }
    }
    // lane 0's rewiring is published before any lane moves on (the arrival
    // atomics order it for the other warps)
    __syncwarp();
    __threadfence();
}

// One thread per leaf walks up as in k_refit; a node is restructured once
// both of its subtrees are final, by the warp of the thread that arrived
// second.  Every lane of a warp stays in the loop until none of them is
// walking, so that it can help: the lanes that won a node in a round are
// served one after another by the whole warp.
constexpr int kTreeletBlock = 128;
__global__ void __launch_bounds__(kTreeletBlock) k_treelets(int n, float4* nodes, int32_t* parent_int,
                                                             int32_t* parent_leaf, const float4* __restrict__ leafbox,
                                                             uint32_t* __restrict__ arrive) {
    __shared__ float s_cost[kTreeletBlock / 32][1 << kTreeletLeaves];
    __shared__ uint8_t s_split[kTreeletBlock / 32][1 << kTreeletLeaves];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int w = threadIdx.x >> 5;
    int p = k < n ? parent_leaf[k] : -1;
    bool walking = k < n;
    for (int level = 0; level < 128; ++level) {
        bool want = false;
        if (walking) {
            if (p < 0 || p >= n - 1) {
                walking = false;
            } else {
                __threadfence();
                if (atomicAdd(arrive + p, 1u) == 0u) {
                    walking = false;  // the other subtree is not final yet
                } else {
                    __threadfence();
                    want = true;
                }
            }
        }
        for (uint32_t m = __ballot_sync(0xffffffffu, want); m; m &= m - 1u) {
            const int32_t q = __shfl_sync(0xffffffffu, p, __ffs(m) - 1);
            restructure_treelet_warp(q, n, nodes, parent_int, parent_leaf, leafbox, s_cost[w], s_split[w]);
        }
        if (want) p = __ldcg(parent_int + p);
        if (!__any_sync(0xffffffffu, walking)) break;
    }
}

// Slot-ordered sphere / material / meta records.  ids may alias meta (a
// refit regathers from the meta words): each thread reads its slot's word
// before writing it.
__global__ void k_gather(const venu_sphere* __restrict__ s, const uint32_t* ids, uint32_t id_mask, uint32_t n,
                         float4* __restrict__ sph, float4* __restrict__ mat, uint32_t* meta) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t id = ids[k] & id_mask;
    const venu_sphere& sp = s[id];
    uint32_t type = sp.material > 2u ? 2u : sp.material;
    sph[k] = make_float4(sp.center[0], sp.center[1], sp.center[2], sp.radius);
    float param = type == 1u ? sp.fuzz : (type == 2u ? sp.ir : 0.0f);
    mat[k] = make_float4(sp.albedo[0], sp.albedo[1], sp.albedo[2], param);
    meta[k] = id | (type << 30);
}

// Traversal layout: internal node p becomes one 64-byte record holding both
// children, child c in float4s 4p+2c and 4p+2c+1:
//   internal child q: {lo.xyz, q}, {hi.xyz, 0}   (q's box from nodes)
//   leaf child:       {center, word}, {radius, 0, 0, 0}   (word keeps the
//                     leaf and hoisted flags; the sphere is inlined)
// A step of the traversal then reads one record instead of two boxes or
// spheres at two addresses.  Runs after k_hoist_finalize, so the flags are
// final; the canonical nodes array stays the exported form.
//
// Every word written here is in range by construction -- an internal child
// in [1, n-1), a leaf slot below n -- so the traversal needs no per-step
// index checks: a word that is not (which a sound build never produces) is
// replaced by a skipped leaf and counted in *bad.
__global__ void k_trav_layout(const float4* __restrict__ nodes, const float4* __restrict__ sph, uint32_t n,
                              float4* __restrict__ trav, uint32_t* bad) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2u * (n - 1u)) return;
    const uint32_t p = i >> 1, c = i & 1u;
    int32_t w = __float_as_int(nodes[2 * p + c].w);
    const bool ok = (w & kLeaf) ? (uint32_t)(w & kSlotMask) < n && !(w & ~(kLeaf | kHoisted | kSlotMask))
                                : (uint32_t)w - 1u < n - 2u;  // 1 <= w < n-1 (the root is nobody's child)
    if (!ok) {
        w = kLeaf | kHoisted;  // slot 0, never tested
        if (bad) atomicAdd(bad, 1u);
    }
    float4 a, b;
    if (w & kLeaf) {
        const float4 s4 = sph[w & kSlotMask];
        a = make_float4(s4.x, s4.y, s4.z, __int_as_float(w));
        b = make_float4(s4.w, 0.0f, 0.0f, 0.0f);
    } else {
        const float4 lo = nodes[2 * w], hi = nodes[2 * w + 1];
        a = make_float4(lo.x, lo.y, lo.z, __int_as_float(w));
        b = make_float4(hi.x, hi.y, hi.z, 0.0f);
    }
    trav[4 * (size_t)p + 2 * c] = a;
    trav[4 * (size_t)p + 2 * c + 1] = b;
}

// ---------------------------------------------------------------------------
// The wide traversal tree (renderer variants 4 and 5), collapsed from the
// binary LBVH after its build.  A wide node stands for a binary node r and
// holds up to kWideW (4) of r's descendants: starting from r's two
// children, the internal entry of largest box surface area (the first such
// entry on ties) is replaced by its two children until there are kWideW
// entries or only leaves.  Internal entries become wide nodes themselves.
// The wide nodes are numbered in increasing order of the binary nodes they
// stand for (root first), so the tree is deterministic.  Results do not
// depend on it: the closest hit is the same for any conservative traversal
// (minimum t, ties to the smaller slot).
//
// Node layout (kWideF4 float4s: 128 bytes for 4 children, 256 for 8), with
// H = kWideW / 4 float4s per plane:
//   [0, 6H)   child boxes, structure of arrays: lo.x, hi.x, lo.y, hi.y,
//             lo.z, hi.z, each H float4s of four children
//   [6H, 7H)  child words: an internal child's wide index, or a leaf's
//             0x80000000 | slot (an unused entry or a hoisted leaf:
//             0x80000000 | 0x40000000, never tested)
//   [7H]      {valid mask | leaf mask << 8 (int bits), 0, 0, 0}
// wide_src[kWideW w + c] keeps the binary word of child c (internal node
// index or leaf word), so a refit of moved spheres can recompute the boxes
// in place.
// ---------------------------------------------------------------------------
constexpr int kWideChildren = kWideW;

__device__ __forceinline__ float box_area(float4 lo, float4 hi) {
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}

__device__ int wide_collapse(const float4* __restrict__ nodes, int32_t r, int32_t w[kWideChildren]) {
    w[0] = __float_as_int(nodes[2 * r].w);
    w[1] = __float_as_int(nodes[2 * r + 1].w);
    int cnt = 2;
    while (cnt < kWideChildren) {
        int best = -1;
        float best_a = -1.0f;
        for (int i = 0; i < cnt; ++i) {
            if (w[i] & kLeaf) continue;
            const float a = box_area(nodes[2 * w[i]], nodes[2 * w[i] + 1]);
            if (a > best_a) {
                best_a = a;
                best = i;
            }
        }
        if (best < 0) break;
        const int32_t q = w[best];
        w[best] = __float_as_int(nodes[2 * q].w);
        w[cnt++] = __float_as_int(nodes[2 * q + 1].w);
    }
    return cnt;
}

// One level of the collapse: every binary node of the frontier expands;
// its internal entries are flagged as wide nodes and form the next frontier.
__global__ void k_wide_frontier(const float4* __restrict__ nodes, const int32_t* __restrict__ fin, uint32_t nin,
                                int32_t* __restrict__ fout, uint32_t* __restrict__ nout, uint32_t* __restrict__ flag) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nin) return;
    int32_t w[kWideChildren];
    const int c = wide_collapse(nodes, fin[i], w);
    for (int j = 0; j < c; ++j) {
        if (w[j] & kLeaf) continue;
        flag[w[j]] = 1u;
        fout[atomicAdd(nout, 1u)] = w[j];
    }
}

// Box of a leaf: the sphere's box rounded outwards (as k_refit makes it).
__device__ __forceinline__ void leaf_box(float4 s4, float4& lo, float4& hi) {
    const float r = fabsf(s4.w);
    lo = make_float4(__fsub_rd(s4.x, r) + 0.0f, __fsub_rd(s4.y, r) + 0.0f, __fsub_rd(s4.z, r) + 0.0f, 0.0f);
    hi = make_float4(__fadd_ru(s4.x, r), __fadd_ru(s4.y, r), __fadd_ru(s4.z, r), 0.0f);
}

// Writes wide node w from the binary words of its children (src[0..7];
// kLeaf | kHoisted for an unused entry).  idx maps a binary internal node to
// its wide index.
__device__ void wide_write_node(const float4* __restrict__ nodes, const float4* __restrict__ sph,
                                const uint32_t* __restrict__ idx, const int32_t* src, float4* __restrict__ W) {
    float lo[3][kWideChildren], hi[3][kWideChildren];
    int32_t word[kWideChildren];
    uint32_t valid = 0, leafm = 0;
    for (int c = 0; c < kWideChildren; ++c) {
        const int32_t b = src[c];
        float4 l = make_float4(0.0f, 0.0f, 0.0f, 0.0f), h = l;
        if (b & kLeaf) {
            word[c] = b;
            if (!(b & kHoisted)) {
                leaf_box(sph[b & kSlotMask], l, h);
                valid |= 1u << c;
                leafm |= 1u << c;
            }
        } else {
            l = nodes[2 * b];
            h = nodes[2 * b + 1];
            word[c] = (int32_t)idx[b];
            valid |= 1u << c;
        }
        lo[0][c] = l.x; lo[1][c] = l.y; lo[2][c] = l.z;
        hi[0][c] = h.x; hi[1][c] = h.y; hi[2][c] = h.z;
    }
    for (int a = 0; a < 3; ++a) {
        for (int half = 0; half < kWideH; ++half) {
            const int c = 4 * half;
            W[2 * a * kWideH + half] = make_float4(lo[a][c], lo[a][c + 1], lo[a][c + 2], lo[a][c + 3]);
            W[(2 * a + 1) * kWideH + half] = make_float4(hi[a][c], hi[a][c + 1], hi[a][c + 2], hi[a][c + 3]);
        }
    }
    for (int half = 0; half < kWideH; ++half) {
        const int c = 4 * half;
        W[6 * kWideH + half] = make_float4(__int_as_float(word[c]), __int_as_float(word[c + 1]),
                                           __int_as_float(word[c + 2]), __int_as_float(word[c + 3]));
    }
    W[7 * kWideH] = make_float4(__int_as_float((int)(valid | (leafm << 8))), 0.0f, 0.0f, 0.0f);
    if (kWideH == 2) W[15] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// One thread per binary internal node; the flagged ones write their wide node.
__global__ void k_wide_write(const float4* __restrict__ nodes, const float4* __restrict__ sph, uint32_t n,
                             const uint32_t* __restrict__ flag, const uint32_t* __restrict__ idx,
                             float4* __restrict__ wide, int32_t* __restrict__ wide_src) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n - 1 || !flag[r]) return;
    int32_t w[kWideChildren];
    const int c = wide_collapse(nodes, (int32_t)r, w);
    for (int j = c; j < kWideChildren; ++j) w[j] = kLeaf | kHoisted;
    const uint32_t k = idx[r];
    for (int j = 0; j < kWideChildren; ++j) wide_src[(size_t)kWideChildren * k + j] = w[j];
    wide_write_node(nodes, sph, idx, w, wide + kWideF4 * (size_t)k);
}

// Refit of moved spheres: the same topology, boxes recomputed from the
// refit binary nodes and the new spheres.  idx is not needed: the child
// words of internal children stay as they are.
__global__ void k_wide_refit(const float4* __restrict__ nodes, const float4* __restrict__ sph, uint32_t nwide,
                             const int32_t* __restrict__ wide_src, float4* __restrict__ wide) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nwide) return;
    float4* W = wide + kWideF4 * (size_t)k;
    float lo[3][kWideChildren], hi[3][kWideChildren];
    for (int c = 0; c < kWideChildren; ++c) {
        const int32_t b = wide_src[(size_t)kWideChildren * k + c];
        float4 l = make_float4(0.0f, 0.0f, 0.0f, 0.0f), h = l;
        if (b & kLeaf) {
            if (!(b & kHoisted)) leaf_box(sph[b & kSlotMask], l, h);
        } else {
            l = nodes[2 * b];
            h = nodes[2 * b + 1];
        }
        lo[0][c] = l.x; lo[1][c] = l.y; lo[2][c] = l.z;
        hi[0][c] = h.x; hi[1][c] = h.y; hi[2][c] = h.z;
    }
    for (int a = 0; a < 3; ++a) {
        for (int half = 0; half < kWideH; ++half) {
            const int c = 4 * half;
            W[2 * a * kWideH + half] = make_float4(lo[a][c], lo[a][c + 1], lo[a][c + 2], lo[a][c + 3]);
            W[(2 * a + 1) * kWideH + half] = make_float4(hi[a][c], hi[a][c + 1], hi[a][c + 2], hi[a][c + 3]);
        }
    }
}

inline uint32_t cdiv(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

// Device buffers of one LBVH build: outputs and scratch.  trav may be null
// (the build then stops at the canonical layout).
struct LbvhBuffers {
    float4 *nodes, *trav, *sph, *mat;
    uint32_t *meta, *keys;
    LbvhCtl* ctl;
    uint32_t *keys_alt, *vals, *vals_alt, *hist, *arrive;
    int32_t *pint, *pleaf;
    float4* leafbox;
};

// The whole build, asynchronously on `st`; both venu_scene_create and
// venu_lbvh_build_noalloc run exactly this sequence.
cudaError_t launch_lbvh(const venu_sphere* s, uint32_t n, cudaStream_t st, const LbvhBuffers& B) {
    const uint32_t nint = n > 1 ? n - 1 : 1;
    const uint32_t ntiles = cdiv(n, kTileKeys);
    k_lbvh_init<<<1, 32, 0, st>>>(B.ctl);
    cudaError_t e = cudaMemsetAsync(B.arrive, 0, sizeof(uint32_t) * nint, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.pint, 0xff, sizeof(int32_t) * nint, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.pleaf, 0xff, sizeof(int32_t) * n, st);
    if (e != cudaSuccess) return e;
    const uint32_t blocks = std::min(cdiv(n, 256), (uint32_t)(sm_count() * 8));
    k_bounds<<<blocks, 256, 0, st>>>(s, n, B.ctl->b0);
    k_morton<<<blocks, 256, 0, st>>>(s, n, B.ctl, B.keys, B.vals);
    uint32_t *kin = B.keys, *kout = B.keys_alt, *vin = B.vals, *vout = B.vals_alt;
    const uint32_t sblocks = cdiv(ntiles, kWarpsPerBlock);
    for (int shift = 0; shift < 32; shift += kRadixBits) {
        k_hist<<<sblocks, 32 * kWarpsPerBlock, 0, st>>>(kin, n, shift, ntiles, B.hist);
        k_scan<<<1, 1024, 0, st>>>(B.hist, kBuckets * ntiles);
        k_scatter<<<sblocks, 32 * kWarpsPerBlock, 0, st>>>(kin, vin, n, shift, ntiles, B.hist, kout, vout);
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    // four passes: the sorted codes / ids are back in B.keys / B.vals
    if (n > 1) {
        k_karras<<<cdiv(n - 1, 256), 256, 0, st>>>(B.keys, (int)n, B.nodes, B.pint, B.pleaf);
        k_refit<<<cdiv(n, 256), 256, 0, st>>>(s, B.vals, 0xffffffffu, (int)n, B.nodes, B.pint, B.pleaf, B.leafbox,
                                              B.arrive);
        e = cudaMemsetAsync(B.arrive, 0, sizeof(uint32_t) * nint, st);
        if (e != cudaSuccess) return e;
        k_treelets<<<cdiv(n, kTreeletBlock), kTreeletBlock, 0, st>>>((int)n, B.nodes, B.pint, B.pleaf, B.leafbox,
                                                                     B.arrive);
    }
    k_gather<<<cdiv(n, 256), 256, 0, st>>>(s, B.vals, 0xffffffffu, n, B.sph, B.mat, B.meta);
    if (n > 1) {
        k_hoist_collect<<<cdiv(n, 256), 256, 0, st>>>(B.sph, n, B.ctl);
        k_hoist_finalize<<<1, 32, 0, st>>>(B.ctl, B.pleaf, B.nodes, n);
        if (B.trav) k_trav_layout<<<cdiv(2 * (n - 1), 256), 256, 0, st>>>(B.nodes, B.sph, n, B.trav, &B.ctl->bad_words);
    }
    return cudaGetLastError();
}

}  // namespace

void free_scene(venu_scene* s) {
    if (!s) return;
    cudaFree(s->nodes);
    cudaFree(s->trav);
    cudaFree(s->sph);
    cudaFree(s->mat);
    cudaFree(s->meta);
    cudaFree(s->keys);
    cudaFree(s->parents);
    cudaFree(s->wide);
    cudaFree(s->wide_src);
    s->wide = nullptr;
    s->wide_src = nullptr;
    s->nwide = 0;
    s->parents = nullptr;
    s->nodes = s->trav = nullptr;
    s->sph = s->mat = nullptr;
    s->meta = s->keys = nullptr;
}

// The wide tree of a built scene (n > 1): the collapse level by level from
// the root (the host reads each level's size), then one write pass.
venu_status build_wide(const venu_scene* S, cudaStream_t st) {
    const uint32_t n = S->n;
    if (n < 2) return VENU_OK;
    const uint32_t nint = n - 1;
    uint32_t *flag = nullptr, *idx = nullptr, *cnt = nullptr;
    int32_t *fa = nullptr, *fb = nullptr;
    venu_status rc = VENU_OK;
    uint32_t nwide = 0;
#define WSTEP(call)                    \
    do {                               \
        cudaError_t _e = (call);       \
        if (_e != cudaSuccess) {       \
            rc = cuda_fail(_e, #call); \
            goto wdone;                \
        }                              \
    } while (0)
    WSTEP(cudaMalloc(&flag, sizeof(uint32_t) * nint));
    WSTEP(cudaMalloc(&idx, sizeof(uint32_t) * nint));
    WSTEP(cudaMalloc(&cnt, sizeof(uint32_t)));
    WSTEP(cudaMalloc(&fa, sizeof(int32_t) * nint));
    WSTEP(cudaMalloc(&fb, sizeof(int32_t) * nint));
    WSTEP(cudaMemsetAsync(flag, 0, sizeof(uint32_t) * nint, st));
    WSTEP(cudaMemsetAsync(flag, 0x01, 1, st));  // the root
    WSTEP(cudaMemsetAsync(fa, 0, sizeof(int32_t), st));
    {
        // a binary tree over n leaves has fewer than n levels, and each level
        // of the collapse takes at least one of them
        uint32_t nin = 1;
        for (uint32_t level = 0; nin > 0 && level < n; ++level) {
            WSTEP(cudaMemsetAsync(cnt, 0, sizeof(uint32_t), st));
            k_wide_frontier<<<cdiv(nin, 128), 128, 0, st>>>(S->nodes, fa, nin, fb, cnt, flag);
            WSTEP(cudaGetLastError());
            WSTEP(cudaMemcpyAsync(&nin, cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
            WSTEP(cudaStreamSynchronize(st));
            std::swap(fa, fb);
        }
        if (nin > 0) {  // a cyclic (corrupt) binary tree: no wide tree
            set_error("venu_scene_create: the wide-tree collapse did not end");
            rc = VENU_ERR_INVALID;
            goto wdone;
        }
    }
    WSTEP(cudaMemcpyAsync(idx, flag, sizeof(uint32_t) * nint, cudaMemcpyDeviceToDevice, st));
    k_scan<<<1, 1024, 0, st>>>(idx, nint);
    WSTEP(cudaGetLastError());
    {
        uint32_t last_idx = 0, last_flag = 0;
        WSTEP(cudaMemcpyAsync(&last_idx, idx + nint - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        WSTEP(cudaMemcpyAsync(&last_flag, flag + nint - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        WSTEP(cudaStreamSynchronize(st));
        nwide = last_idx + last_flag;
    }
    WSTEP(cudaMalloc(&S->wide, sizeof(float4) * kWideF4 * (size_t)nwide));
    WSTEP(cudaMalloc(&S->wide_src, sizeof(int32_t) * kWideChildren * (size_t)nwide));
    S->nwide = nwide;
    S->bytes += sizeof(float4) * kWideF4 * (size_t)nwide + sizeof(int32_t) * kWideChildren * (size_t)nwide;
    k_wide_write<<<cdiv(nint, 128), 128, 0, st>>>(S->nodes, S->sph, n, flag, idx, S->wide, S->wide_src);
    WSTEP(cudaGetLastError());
    WSTEP(cudaStreamSynchronize(st));
#undef WSTEP
wdone:
    cudaFree(flag);
    cudaFree(idx);
    cudaFree(cnt);
    cudaFree(fa);
    cudaFree(fb);
    return rc;
}

venu_status build_scene(const venu_sphere* spheres_dev, uint32_t n, cudaStream_t st, venu_scene* S) {
    S->n = n;
    if (n == 0) return VENU_OK;
    if (n > (1u << 28)) {
        set_error("venu_scene_create: more than 2^28 spheres");
        return VENU_ERR_TOO_LARGE;
    }
    const uint32_t ntiles = cdiv(n, kTileKeys);
    const size_t hist_n = (size_t)kBuckets * ntiles;
    size_t bytes = 0;
    auto alloc = [&](void** p, size_t b) -> cudaError_t {
        bytes += b;
        return cudaMalloc(p, b ? b : 16);
    };
    const uint32_t nint = n > 1 ? n - 1 : 1;
    VENU_CUDA(alloc((void**)&S->nodes, sizeof(float4) * 2 * nint));
    VENU_CUDA(alloc((void**)&S->trav, sizeof(float4) * 4 * nint));
    VENU_CUDA(alloc((void**)&S->sph, sizeof(float4) * n));
    VENU_CUDA(alloc((void**)&S->mat, sizeof(float4) * n));
    VENU_CUDA(alloc((void**)&S->meta, sizeof(uint32_t) * n));
    VENU_CUDA(alloc((void**)&S->keys, sizeof(uint32_t) * n));
    VENU_CUDA(alloc((void**)&S->parents, sizeof(int32_t) * ((size_t)nint + n)));
    S->bytes = bytes;
    LbvhBuffers B{};
    B.nodes = S->nodes;
    B.trav = S->trav;
    B.sph = S->sph;
    B.mat = S->mat;
    B.meta = S->meta;
    B.keys = S->keys;
    B.pint = S->parents;
    B.pleaf = S->parents + nint;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    venu_status rc = VENU_OK;
    LbvhCtl hc;
#define STEP(call)                               \
    do {                                         \
        cudaError_t _e = (call);                 \
        if (_e != cudaSuccess) {                 \
            rc = cuda_fail(_e, #call);           \
            goto done;                           \
        }                                        \
    } while (0)
    STEP(cudaMalloc(&B.ctl, sizeof(LbvhCtl)));
    STEP(cudaMalloc(&B.keys_alt, sizeof(uint32_t) * n));
    STEP(cudaMalloc(&B.vals, sizeof(uint32_t) * n));
    STEP(cudaMalloc(&B.vals_alt, sizeof(uint32_t) * n));
    STEP(cudaMalloc(&B.hist, sizeof(uint32_t) * hist_n));
    STEP(cudaMalloc(&B.arrive, sizeof(uint32_t) * nint));
    STEP(cudaMalloc(&B.leafbox, sizeof(float4) * 2 * n));
    STEP(cudaEventCreate(&e0));
    STEP(cudaEventCreate(&e1));
    STEP(cudaEventRecord(e0, st));
    STEP(launch_lbvh(spheres_dev, n, st, B));
    STEP(cudaEventRecord(e1, st));
    STEP(cudaMemcpyAsync(&hc, B.ctl, sizeof(LbvhCtl), cudaMemcpyDeviceToHost, st));
    STEP(cudaStreamSynchronize(st));
    {
        float ms = 0.0f;
        STEP(cudaEventElapsedTime(&ms, e0, e1));
        S->build_ms = ms;
        std::memcpy(S->bounds, hc.bounds, sizeof(S->bounds));
        S->nhoist = n > 1 ? hc.nhoist : 0u;
        for (int i = 0; i < kMaxHoisted; ++i) S->hoist[i] = hc.hoist[i];
        if (n > 1 && hc.bad_words) {
            set_error("venu_scene_create: the LBVH build produced " + std::to_string(hc.bad_words) +
                      " out-of-range child words");
            rc = VENU_ERR_INVALID;
        }
    }
#undef STEP
done:
    cudaFree(B.ctl);
    cudaFree(B.keys_alt);
    cudaFree(B.vals);
    cudaFree(B.vals_alt);
    cudaFree(B.hist);
    cudaFree(B.arrive);
    cudaFree(B.leafbox);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return rc;
}

venu_status ensure_wide(const venu_scene* S, cudaStream_t st) {
    std::lock_guard<std::mutex> lock(S->wide_mu);
    if (S->n < 2 || S->wide) return VENU_OK;
    const auto t0 = std::chrono::steady_clock::now();
    const venu_status rc = build_wide(S, st);
    S->wide_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (rc != VENU_OK) {  // no half-built tree stays behind
        cudaStreamSynchronize(st);
        cudaFree(S->wide);
        cudaFree(S->wide_src);
        if (S->nwide)
            S->bytes -= sizeof(float4) * kWideF4 * (size_t)S->nwide + sizeof(int32_t) * kWideChildren * (size_t)S->nwide;
        S->wide = nullptr;
        S->wide_src = nullptr;
        S->nwide = 0;
    }
    return rc;
}

venu_status update_scene(venu_scene* S, const venu_sphere* s, cudaStream_t st) {
    const uint32_t n = S->n;
    if (n == 0) return VENU_OK;
    // New sphere records into the same slots (meta holds each slot's
    // original index), then the boxes bottom-up over the kept parent links,
    // then the traversal records.  Topology, slot order and the hoisted set
    // stay those of the build.
    k_gather<<<cdiv(n, 256), 256, 0, st>>>(s, S->meta, 0x3fffffffu, n, S->sph, S->mat, S->meta);
    VENU_CUDA(cudaGetLastError());
    if (n == 1) return VENU_OK;
    float4* leafbox = nullptr;
    uint32_t* arrive = nullptr;
    VENU_CUDA(cudaMallocAsync(&leafbox, sizeof(float4) * 2 * n, st));
    cudaError_t e = cudaMallocAsync(&arrive, sizeof(uint32_t) * (n - 1), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(arrive, 0, sizeof(uint32_t) * (n - 1), st);
    if (e == cudaSuccess) {
        k_refit<<<cdiv(n, 256), 256, 0, st>>>(s, S->meta, 0x3fffffffu, (int)n, S->nodes, S->parents,
                                              S->parents + (n - 1), leafbox, arrive);
        k_trav_layout<<<cdiv(2 * (n - 1), 256), 256, 0, st>>>(S->nodes, S->sph, n, S->trav, nullptr);
        if (S->nwide) k_wide_refit<<<cdiv(S->nwide, 128), 128, 0, st>>>(S->nodes, S->sph, S->nwide, S->wide_src,
                                                                      S->wide);
        e = cudaGetLastError();
    }
    cudaFreeAsync(leafbox, st);
    if (arrive) cudaFreeAsync(arrive, st);
    if (e != cudaSuccess) return cuda_fail(e, "venu_scene_update");
    return VENU_OK;
}

}  // namespace venu

// ---------------------------------------------------------------------------
// venu_lbvh_build_noalloc: the same LBVH build into caller-owned buffers,
// with its scratch in a fixed file-scope device array instead of cudaMalloc.
// ---------------------------------------------------------------------------
namespace venu {
namespace {

constexpr uint32_t kNoAllocMaxSpheres = VENU_NOALLOC_MAX_SPHERES;
constexpr uint32_t kNoAllocMaxTiles = (kNoAllocMaxSpheres + kTileKeys - 1) / kTileKeys;
constexpr size_t al256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kNA = kNoAllocMaxSpheres;
constexpr size_t kOffCtl = 0;                                         // LbvhCtl
constexpr size_t kOffKeysAlt = al256(kOffCtl + sizeof(LbvhCtl));
constexpr size_t kOffVals = al256(kOffKeysAlt + 4 * kNA);
constexpr size_t kOffValsAlt = al256(kOffVals + 4 * kNA);
constexpr size_t kOffHist = al256(kOffValsAlt + 4 * kNA);
constexpr size_t kOffArrive = al256(kOffHist + 4 * (size_t)kBuckets * kNoAllocMaxTiles);
constexpr size_t kOffParentInt = al256(kOffArrive + 4 * kNA);
constexpr size_t kOffParentLeaf = al256(kOffParentInt + 4 * kNA);
constexpr size_t kOffLeafBox = al256(kOffParentLeaf + 4 * kNA);
constexpr size_t kNoAllocScratchBytes = al256(kOffLeafBox + 32 * kNA);  // about 3.8 MB

}  // namespace
}  // namespace venu

// Every GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) unsigned char g_lbvh_noalloc_scratch[venu::kNoAllocScratchBytes];

namespace venu {
namespace {

std::mutex g_noalloc_mu;
constexpr int kMaxDevices = 64;
void* g_noalloc_scratch[kMaxDevices] = {};

// Device address of the scratch array on the current device.  The host-side
// name g_lbvh_noalloc_scratch is only a stand-in: its device address comes
// from cudaGetSymbolAddress, once per device, with that device current.
venu_status noalloc_scratch(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "venu_lbvh_build_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("venu_lbvh_build_noalloc: device ordinal out of range");
        return VENU_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_scratch[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_lbvh_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "venu_lbvh_build_noalloc: cudaGetSymbolAddress");
        g_noalloc_scratch[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_noalloc_scratch[dev]);
    return VENU_OK;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace
}  // namespace venu

extern "C" venu_status venu_lbvh_build_noalloc(const venu_sphere* spheres_dev, uint32_t n, float* nodes_out,
                                               float* spheres_out, float* materials_out, uint32_t* meta_out,
                                               uint32_t* morton_out, void* stream) {
    using namespace venu;
    if (n > kNoAllocMaxSpheres) {
        set_error("venu_lbvh_build_noalloc: " + std::to_string(n) + " spheres exceed the limit of " +
                  std::to_string(kNoAllocMaxSpheres) + " (VENU_NOALLOC_MAX_SPHERES); use venu_scene_create");
        return VENU_ERR_TOO_LARGE;
    }
    if (n == 0) return VENU_OK;
    if (!spheres_dev || !spheres_out || !materials_out || !meta_out || !morton_out || (n > 1 && !nodes_out)) {
        set_error("venu_lbvh_build_noalloc: NULL buffer");
        return VENU_ERR_INVALID;
    }
    if (!aligned16(spheres_out) || !aligned16(materials_out) || (n > 1 && !aligned16(nodes_out))) {
        set_error("venu_lbvh_build_noalloc: nodes/spheres/materials outputs must be 16-byte aligned");
        return VENU_ERR_INVALID;
    }
    venu_status ds = require_device();
    if (ds != VENU_OK) return ds;
    unsigned char* base = nullptr;
    venu_status ss = noalloc_scratch(&base);
    if (ss != VENU_OK) return ss;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    LbvhBuffers B{};
    B.nodes = reinterpret_cast<float4*>(nodes_out);
    B.sph = reinterpret_cast<float4*>(spheres_out);
    B.mat = reinterpret_cast<float4*>(materials_out);
    B.meta = meta_out;
    B.keys = morton_out;
    B.ctl = reinterpret_cast<LbvhCtl*>(base + kOffCtl);
    B.keys_alt = reinterpret_cast<uint32_t*>(base + kOffKeysAlt);
    B.vals = reinterpret_cast<uint32_t*>(base + kOffVals);
    B.vals_alt = reinterpret_cast<uint32_t*>(base + kOffValsAlt);
    B.hist = reinterpret_cast<uint32_t*>(base + kOffHist);
    B.arrive = reinterpret_cast<uint32_t*>(base + kOffArrive);
    B.pint = reinterpret_cast<int32_t*>(base + kOffParentInt);
    B.pleaf = reinterpret_cast<int32_t*>(base + kOffParentLeaf);
    B.leafbox = reinterpret_cast<float4*>(base + kOffLeafBox);
    // The scratch keeps the previous call's contents; launch_lbvh resets what
    // must start from a known value (bounds seeds, hoist counters, arrival
    // counters, parent links) before using it.
    VENU_CUDA(launch_lbvh(spheres_dev, n, st, B));
    VENU_CUDA(cudaGetLastError());
    return VENU_OK;
}
