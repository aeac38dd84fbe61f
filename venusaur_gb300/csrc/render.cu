// render.cu -- the plain single-scene wavefront renderer.
//
// Replaces Renderer::Draw (Core/Renderer.h:35-78) and the OptiX programs of
// Core/RayTracer.cu.  A render call is cut into waves of up to max_paths
// paths (pixels x a run of consecutive samples).  Per wave:
//   raygen     one thread per pixel, the wave's samples in order;
//   bounce b   traverse (closest hit for every queued ray)
//              shade    (scatter; survivors compacted into the next queue
//                        with __ballot_sync + a warp prefix, finished paths
//                        write their radiance to their sample slot);
//   accumulate one thread per pixel, Kahan-adds the wave's samples in
//              sample order.
// A resolve pass writes the running mean (RGBA32F) and sRGB RGBA8.
// Queue counts live on the device; the host never waits inside a render.
#include "render_kernels.cuh"
#include "venu_internal.h"

#include <algorithm>
#include <cstring>
#include <vector>

namespace venu {

// The bounce loop of a wave run as one CUDA graph (fused variants): the
// first bounce's kernel, then a while node over a body of two bounce kernels
// (odd: queue 1 -> 0, even: queue 0 -> 1), each with its queues and
// counters as fixed parameters.  The last block of each bounce launch
// advances the loop: it clears the counters the next bounce writes to,
// counts the bounce, and keeps the while node going only while the bounce
// left rays to trace -- so a wave whose paths all finish early (in place, or
// by depth) launches no empty bounces.
struct WaveCtl {
    uint32_t b;            // bounces of the wave traced so far
    uint32_t nb;           // at most this many (the maximum depth)
    uint32_t blocks_done;  // blocks of the running bounce launch that finished
    uint32_t pad;
};

// Camera rays of one wave (P pixels from p0, k samples from s0): path
// pos = s * P + pl.  With path_seeds, only each path's raygen seed is written
// (4 bytes instead of a 48-byte queue entry) and the fused kernel makes the
// camera ray itself (PrimaryGen); the pixel's seed still advances through
// every sample's draws, which is what fixes the next sample's seed.
__global__ void k_raygen(venu_camera cam, uint32_t W, uint32_t H, uint32_t p0, uint32_t P, uint32_t s0,
                         uint32_t k, uint32_t subframe, int max_depth, uint32_t* __restrict__ seeds,
                         Queue q, uint32_t* __restrict__ path_seeds, uint32_t* __restrict__ cnt,
                         uint32_t* __restrict__ work, int nbounce, WaveCtl* __restrict__ ctl) {
    const uint32_t pl = blockIdx.x * blockDim.x + threadIdx.x;
    if (pl == 0) {
        cnt[0] = P * k;
        for (int b = 1; b <= nbounce; ++b) cnt[b] = 0;
        for (int b = 0; b <= nbounce; ++b) work[b] = 0;
        if (ctl) {
            ctl->b = 0u;
            ctl->nb = (uint32_t)nbounce;
        }
    }
    if (pl >= P) return;
    const DevCamera C = load_camera(cam);
    const uint32_t pix = p0 + pl;
    const uint32_t x = pix % W, y = pix / W;
    uint32_t seed = (s0 == 0) ? tea4(pix, subframe) : seeds[pix];
    for (uint32_t s = 0; s < k; ++s) {
        const uint32_t pos = s * P + pl;
        if (path_seeds) path_seeds[pos] = seed;
        f3 o, d;
        camera_ray(C, x, y, W, H, seed, o, d);
        if (!path_seeds) write_primary(q, pos, o, d, pos, max_depth - 1, seed);
    }
    seeds[pix] = seed;
}

// WIDE: over the 4-wide tree (variant 5's later bounces).
// The separate traversal and shading kernels read each queue entry and hit
// record once: they load and store them evict-first (ld/st.global.cs), which
// leaves more of L1 and L2 to the node set (1M spheres, variant 3: +0.5 %).
// The fused kernel keeps plain accesses: the same hints measured -0.45 % on
// the RTIOW scene there.
template <bool COUNT, bool WIDE = false>
__global__ void __launch_bounds__(256) k_traverse(SceneView S, Queue q, const uint32_t* __restrict__ cnt,
                                                  uint32_t* __restrict__ work, int2* __restrict__ hits,
                                                  uint32_t* __restrict__ err,
                                                  unsigned long long* __restrict__ stats) {
    extern __shared__ unsigned char smem[];
    StackSmem sm;
    sm.node = reinterpret_cast<int*>(smem);
    sm.tn = reinterpret_cast<float*>(smem + sizeof(int) * kShared * blockDim.x);
    const uint32_t n = *cnt;
    const uint32_t lane = threadIdx.x & 31;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(stats, (unsigned long long)n);
    TraceCounters K{0, 0};
    bool overflow = false;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(work, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane;
        if (i < n) {
            float4 o4 = __ldcs(q.o + i), d4 = __ldcs(q.d + i);
            RayPre R = prep(mk(o4.x, o4.y, o4.z), mk(d4.x, d4.y, d4.z));
            R.from = packed_from(d4.w);
            float t;
            int32_t k = trace_closest<COUNT, kShared, WIDE>(S, R, 0.001f, 1e16f, t, sm, threadIdx.x, blockDim.x,
                                                           overflow, K);
            __stcs(hits + i, make_int2(__float_as_int(t), k));
        }
    }
    if (overflow) atomicOr(err, 1u);
    if (COUNT) flush_counters(K, stats);
}

// Persistent lanes: a lane whose ray is finished takes a new one as soon as
// at least `refill_min` lanes of its warp are idle (one atomic per refill),
// so warps stay full while the queue lasts instead of waiting for their
// slowest ray (dynamic fetch, Aila & Laine 2009).
template <bool COUNT>
__global__ void __launch_bounds__(256) k_traverse_dyn(SceneView S, Queue q, const uint32_t* __restrict__ cnt,
                                                      uint32_t* __restrict__ work, int2* __restrict__ hits,
                                                      uint32_t* __restrict__ err,
                                                      unsigned long long* __restrict__ stats, uint32_t refill_min) {
    extern __shared__ unsigned char smem[];
    StackSmem sm;
    sm.node = reinterpret_cast<int*>(smem);
    sm.tn = reinterpret_cast<float*>(smem + sizeof(int) * kShared * blockDim.x);
    const uint32_t n = *cnt;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1u;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(stats, (unsigned long long)n);
    TraceCounters K{0, 0};
    bool overflow = false;
    Tracer<COUNT> T;
    int spill[kSpill];
    float spill_tn[kSpill];
    uint32_t ray = 0;
    bool active = false, exhausted = false;
    for (;;) {
        const uint32_t idle = __ballot_sync(0xffffffffu, !active);
        if (!exhausted && (idle == 0xffffffffu || (uint32_t)__popc(idle) >= refill_min)) {
            const uint32_t k = (uint32_t)__popc(idle);
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(work, k);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base + k >= n) exhausted = true;
            if (!active) {
                const uint32_t my = base + (uint32_t)__popc(idle & lt);
                if (my < n) {
                    ray = my;
                    const float4 o4 = __ldcs(q.o + my), d4 = __ldcs(q.d + my);
                    RayPre R = prep(mk(o4.x, o4.y, o4.z), mk(d4.x, d4.y, d4.z));
                    R.from = packed_from(d4.w);
                    if (R.axis) {
                        // a near-axis-parallel ray (rare): traced to the end now with
                        // the per-axis loop, on this lane's free stack; the lane
                        // stays idle
                        float t;
                        const int32_t kk = trace_closest_as<COUNT, true>(S, R, 0.001f, 1e16f, t, sm, threadIdx.x,
                                                                         blockDim.x, overflow, K);
                        __stcs(hits + my, make_int2(__float_as_int(t), kk));
                    } else if (T.begin(S, R, 0.001f, 1e16f, K)) {
                        active = true;
                    } else {
                        float t;
                        const int32_t kk = T.result(t);
                        __stcs(hits + my, make_int2(__float_as_int(t), kk));
                    }
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (exhausted) break;
            continue;
        }
        if (active && !T.step(S, sm, threadIdx.x, blockDim.x, spill, spill_tn, overflow, K)) {
            active = false;
            float t;
            const int32_t kk = T.result(t);
            __stcs(hits + ray, make_int2(__float_as_int(t), kk));
        }
    }
    if (overflow) atomicOr(err, 1u);
    if (COUNT) flush_counters(K, stats);
}

// One warp-batch loop of the fused kernel: each warp takes 32 rays, traces
// and shades them, and appends the continuing paths to the next queue.
template <bool COUNT, int KS, bool WIDE>
__device__ __forceinline__ void trace_shade_loop(const SceneView& S, const Queue& qin, uint32_t n,
                                                 uint32_t* __restrict__ work, const Queue& qout,
                                                 uint32_t* __restrict__ cnt_out, float4* __restrict__ slots,
                                                 const PrimaryGen& gen, const DevCamera& cam, StackSmem sm,
                                                 bool& overflow, TraceCounters& K) {
    const uint32_t lane = threadIdx.x & 31;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(work, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane;
        const bool valid = i < n;
        ShadeOut r;
        r.cont = false;
        uint32_t slot = 0;
        if (valid) {
            float4 o4, d4;
            uint32_t seed = 0;
            if (gen.path_seeds) {
                gen_primary(gen, cam, i, o4, d4, seed);
            } else {
                o4 = qin.o[i];
                d4 = qin.d[i];
            }
            slot = (uint32_t)__float_as_int(o4.w);
            RayPre R = prep(mk(o4.x, o4.y, o4.z), mk(d4.x, d4.y, d4.z));
            R.from = packed_from(d4.w);
            float t;
            const int32_t k =
                trace_closest<COUNT, KS, WIDE>(S, R, 0.001f, 1e16f, t, sm, threadIdx.x, blockDim.x, overflow, K);
            const float4 t4 = gen.path_seeds ? make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(seed)) : qin.t[i];
            r = shade_one<true>(S, o4, d4, t4, make_int2(__float_as_int(t), k));
        }
        const uint32_t pos = warp_append(r.cont, cnt_out);
        if (r.cont) {
            qout.o[pos] = r.o;
            qout.d[pos] = r.d;
            qout.t[pos] = r.t;
        } else if (valid) {
            slots[slot] = r.result;
        }
    }
}

// The in-place launch (no more rays than the grid has threads): block b
// takes rays [b * blockDim, (b + 1) * blockDim) and finishes them bounce by
// bounce.  Between bounces the block's surviving paths are compacted to its
// first threads (their state staged through the unused output queue, at the
// block's own positions), so its warps stay full while paths end at
// different bounces instead of idling around the few long paths.  Each path
// goes through exactly the same arithmetic as in the ordinary loop; only
// the thread that runs it changes.
template <bool COUNT, int KS, bool WIDE>
__device__ __forceinline__ void trace_shade_in_place(const SceneView& S, const Queue& qin, uint32_t n,
                                                     const Queue& qout, float4* __restrict__ slots,
                                                     const PrimaryGen& gen, const DevCamera& cam, StackSmem sm,
                                                     bool& overflow, TraceCounters& K, uint32_t& extra) {
    __shared__ uint32_t warp_live[32];
    const uint32_t t = threadIdx.x, lane = t & 31u, w = t >> 5;
    const uint32_t base = blockIdx.x * blockDim.x;
    const uint32_t i = base + t;  // this thread's state lives at i
    bool live = i < n;
    float4 o4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), d4 = o4;
    if (live) {
        uint32_t seed = 0;
        if (gen.path_seeds) {
            gen_primary(gen, cam, i, o4, d4, seed);
            qout.t[i] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(seed));
        } else {
            o4 = qin.o[i];
            d4 = qin.d[i];
            qout.t[i] = qin.t[i];
        }
    }
    uint32_t held = (uint32_t)__syncthreads_count(live);  // threads holding a state, from thread 0 on
    for (bool first = true;; first = false) {
        const uint32_t cnt = (uint32_t)__syncthreads_count(live);
        if (cnt == 0) break;
        if (cnt < held) {
            // compaction: the live states to threads [0, cnt)
            const uint32_t m = __ballot_sync(0xffffffffu, live);
            if (lane == 0) warp_live[w] = (uint32_t)__popc(m);
            float4 t4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (live) t4 = qout.t[i];
            __syncthreads();
            uint32_t pos = (uint32_t)__popc(m & ((1u << lane) - 1u));
            for (uint32_t v = 0; v < w; ++v) pos += warp_live[v];
            if (live) {
                qout.o[base + pos] = o4;
                qout.d[base + pos] = d4;
                qout.t[base + pos] = t4;
            }
            __syncthreads();
            live = t < cnt;
            if (live) {
                o4 = qout.o[i];
                d4 = qout.d[i];
            }
            held = cnt;
        }
        if (live) {
            RayPre R = prep(mk(o4.x, o4.y, o4.z), mk(d4.x, d4.y, d4.z));
            R.from = packed_from(d4.w);
            float th;
            const int32_t k = trace_closest<COUNT, KS, WIDE>(S, R, 0.001f, 1e16f, th, sm, t, blockDim.x, overflow, K);
            const ShadeOut r = shade_one<true>(S, o4, d4, qout.t[i], make_int2(__float_as_int(th), k));
            if (!first) ++extra;
            if (r.cont) {
                o4 = r.o;
                d4 = r.d;
                qout.t[i] = r.t;
            } else {
                slots[(uint32_t)__float_as_int(o4.w)] = r.result;
                live = false;
            }
        }
    }
}

// The in-place launch with refills (in_place_factor > 1, its own kernel
// instantiation, REFILL): a launch with at most in_place_factor rays per
// thread of the grid finishes every path it takes bounce after bounce
// instead of appending survivors to the next queue.  A block takes rays from the launch
// with one atomic per refill (the same dynamic hand-out as the ordinary
// loop), and at each bounce boundary compacts its surviving paths to its
// first threads (their state staged through the unused output queue) and
// gives the threads behind them fresh rays, so its warps stay full while
// paths end at different bounces.  Each path goes through exactly the same
// arithmetic as in the ordinary loop; only the thread that runs it changes.
// A block's staging positions are those of the first rays it took, base0 +
// [0, blockDim): it never holds more paths than that first chunk had rays
// (a short first chunk is the launch's last), so they stay inside the queue.
// The factor is a tuning field (venu_tuning.in_place_factor): finishing in
// place keeps the warps of a block in step bounce by bounce, which pays on
// scenes with long, divergent paths and costs on short ones.

template <bool COUNT, int KS, bool WIDE>
__device__ __forceinline__ void trace_shade_in_place_refill(const SceneView& S, const Queue& qin, uint32_t n,
                                                     uint32_t* __restrict__ work, const Queue& qout,
                                                     float4* __restrict__ slots, const PrimaryGen& gen,
                                                     const DevCamera& cam, StackSmem sm, bool& overflow,
                                                     TraceCounters& K, uint32_t& extra) {
    __shared__ uint32_t warp_live[32];
    __shared__ uint32_t s_base;
    const uint32_t t = threadIdx.x, lane = t & 31u, w = t >> 5;
    uint32_t base0 = 0xffffffffu;  // the block's staging positions start here (its first chunk)
    uint32_t held = 0;             // threads [0, held) hold the block's paths
    bool exhausted = false, live = false, first = false;
    float4 o4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), d4 = o4;
    for (;;) {
        const uint32_t cnt = (uint32_t)__syncthreads_count(live);
        if (cnt == 0 && exhausted) break;
        if (cnt < held || (!exhausted && cnt < blockDim.x)) {
            const uint32_t i = base0 + t;
            if (cnt < held) {  // the live states to threads [0, cnt)
                const uint32_t m = __ballot_sync(0xffffffffu, live);
                if (lane == 0) warp_live[w] = (uint32_t)__popc(m);
                float4 t4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (live) t4 = qout.t[i];
                __syncthreads();
                uint32_t pos = (uint32_t)__popc(m & ((1u << lane) - 1u));
                for (uint32_t v = 0; v < w; ++v) pos += warp_live[v];
                if (live) {
                    qout.o[base0 + pos] = o4;
                    qout.d[base0 + pos] = d4;
                    qout.t[base0 + pos] = t4;
                }
                __syncthreads();
                if (t < cnt) {
                    o4 = qout.o[i];
                    d4 = qout.d[i];
                }
            }
            uint32_t take = 0, base = 0;
            if (!exhausted) {  // fresh rays for threads [cnt, blockDim)
                const uint32_t need = blockDim.x - cnt;
                if (t == 0) s_base = atomicAdd(work, need);
                __syncthreads();
                base = s_base;
                take = base < n ? min(need, n - base) : 0u;
                exhausted = take < need;
                if (base0 == 0xffffffffu) base0 = base;  // the first chunk (cnt == 0 then)
            }
            live = t < cnt + take;
            first = t >= cnt && live;
            if (first) {
                const uint32_t ray = base + (t - cnt);
                const uint32_t j = base0 + t;
                if (gen.path_seeds) {
                    uint32_t seed = 0;
                    gen_primary(gen, cam, ray, o4, d4, seed);
                    qout.t[j] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(seed));
                } else {
                    o4 = qin.o[ray];
                    d4 = qin.d[ray];
                    qout.t[j] = qin.t[ray];
                }
            }
            held = cnt + take;
        }
        if (live) {
            const uint32_t i = base0 + t;
            RayPre R = prep(mk(o4.x, o4.y, o4.z), mk(d4.x, d4.y, d4.z));
            R.from = packed_from(d4.w);
            float th;
            const int32_t k = trace_closest<COUNT, KS, WIDE>(S, R, 0.001f, 1e16f, th, sm, t, blockDim.x, overflow, K);
            const ShadeOut r = shade_one<true>(S, o4, d4, qout.t[i], make_int2(__float_as_int(th), k));
            if (!first) ++extra;
            first = false;
            if (r.cont) {
                o4 = r.o;
                d4 = r.d;
                qout.t[i] = r.t;
            } else {
                slots[(uint32_t)__float_as_int(o4.w)] = r.result;
                live = false;
            }
        }
    }
}

// Traverse and shade in one pass: each warp takes 32 rays, traverses them,
// then shades all 32 together once the warp has reconverged and appends the
// continuing paths with one ballot and one atomic.  Saves the hit record
// round trip, the second read of the rays and one launch per bounce.
// WIDE: the 4-wide tree instead of the binary traversal layout (variant 4,
// k_trace_shade_wide, with its own register cap).
// The end of a bounce launch run inside the wave graph (see WaveCtl).
__device__ __forceinline__ void wave_advance(WaveCtl* ctl, uint32_t* cnt_in, uint32_t* work,
                                             const uint32_t* cnt_out, unsigned long long* stats,
                                             cudaGraphConditionalHandle handle) {
    __syncthreads();  // every thread of the block is done
    if (threadIdx.x != 0) return;
    __threadfence();
    if (atomicAdd(&ctl->blocks_done, 1u) != gridDim.x - 1u) return;
    // the last block: every ray of this bounce is traced and shaded, and its
    // input counters are read by nobody any more
    __threadfence();
    ctl->blocks_done = 0u;
    *cnt_in = 0u;  // the output count of the next bounce
    *work = 0u;    // the hand-out counter of the bounce after it
    const uint32_t b = ctl->b + 1u;
    ctl->b = b;
    atomicAdd(stats + 5, 1ull);  // bounce launches run
    const uint32_t more = b < ctl->nb && *reinterpret_cast<const volatile uint32_t*>(cnt_out) > 0u;
    cudaGraphSetConditional(handle, more);
}

template <bool COUNT, int KS, bool WIDE, bool REFILL>
__device__ __forceinline__ void trace_shade_body(const SceneView& S, const Queue& qin,
                                                 uint32_t* __restrict__ cnt_in, uint32_t* __restrict__ work,
                                                 const Queue& qout, uint32_t* __restrict__ cnt_out,
                                                 float4* __restrict__ slots, uint32_t* __restrict__ err,
                                                 unsigned long long* __restrict__ stats, const PrimaryGen& gen,
                                                 WaveCtl* ctl, cudaGraphConditionalHandle handle) {
    extern __shared__ unsigned char smem[];
    StackSmem sm;
    sm.node = reinterpret_cast<int*>(smem);
    sm.tn = reinterpret_cast<float*>(smem + sizeof(int) * KS * blockDim.x);
    __shared__ DevCamera cam;  // the primary rays' camera basis, once per block
    if (gen.path_seeds) {      // a kernel parameter: the same in every thread
        if (threadIdx.x == 0) cam = load_camera(gen.cam);
        __syncthreads();
    }
    const uint32_t n = *cnt_in;
    const uint32_t lane = threadIdx.x & 31;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(stats, (unsigned long long)n);
    TraceCounters K{0, 0};
    bool overflow = false;
    uint32_t extra = 0;  // segments traced in place after a ray's first
    if (n <= (REFILL ? gen.in_place_factor : 1u) * gridDim.x * blockDim.x) {
        if (REFILL)
            trace_shade_in_place_refill<COUNT, KS, WIDE>(S, qin, n, work, qout, slots, gen, cam, sm, overflow, K,
                                                         extra);
        else
            trace_shade_in_place<COUNT, KS, WIDE>(S, qin, n, qout, slots, gen, cam, sm, overflow, K, extra);
        for (int off = 16; off > 0; off >>= 1) extra += __shfl_xor_sync(0xffffffffu, extra, off);
        if (lane == 0 && extra) atomicAdd(stats, (unsigned long long)extra);
    } else {
        trace_shade_loop<COUNT, KS, WIDE>(S, qin, n, work, qout, cnt_out, slots, gen, cam, sm, overflow, K);
    }
    if (overflow) atomicOr(err, 1u);
    if (COUNT) flush_counters(K, stats);
    if (ctl) wave_advance(ctl, cnt_in, work, cnt_out, stats, handle);
}

// REFILL: launches of up to in_place_factor rays per thread finish in place
// with refills (a separate instantiation, so the ordinary kernel keeps its
// registers).  ctl: the wave graph's loop control (nullptr for a launch
// from the host's bounce loop).
template <bool COUNT, int KS, bool REFILL = false>
__global__ void VENU_TRACE_BOUNDS k_trace_shade(SceneView S, Queue qin, uint32_t* __restrict__ cnt_in,
                                                uint32_t* __restrict__ work, Queue qout,
                                                uint32_t* __restrict__ cnt_out, float4* __restrict__ slots,
                                                uint32_t* __restrict__ err, unsigned long long* __restrict__ stats,
                                                PrimaryGen gen, WaveCtl* ctl, cudaGraphConditionalHandle handle) {
    trace_shade_body<COUNT, KS, false, REFILL>(S, qin, cnt_in, work, qout, cnt_out, slots, err, stats, gen, ctl,
                                               handle);
}

template <bool COUNT, int KS, bool REFILL = false>
__global__ void VENU_WIDE_BOUNDS k_trace_shade_wide(SceneView S, Queue qin, uint32_t* __restrict__ cnt_in,
                                                    uint32_t* __restrict__ work, Queue qout,
                                                    uint32_t* __restrict__ cnt_out, float4* __restrict__ slots,
                                                    uint32_t* __restrict__ err,
                                                    unsigned long long* __restrict__ stats, PrimaryGen gen,
                                                    WaveCtl* ctl, cudaGraphConditionalHandle handle) {
    trace_shade_body<COUNT, KS, true, REFILL>(S, qin, cnt_in, work, qout, cnt_out, slots, err, stats, gen, ctl,
                                              handle);
}

__global__ void __launch_bounds__(512) k_shade(SceneView S, Queue qin, const int2* __restrict__ hits,
                                               const uint32_t* __restrict__ cnt_in, Queue qout,
                                               uint32_t* __restrict__ cnt_out, float4* __restrict__ slots) {
    const uint32_t n = *cnt_in;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        const uint32_t i = base + lane;
        ShadeOut r;
        r.cont = false;
        uint32_t slot = 0;
        const bool valid = i < n;
        if (valid) {
            float4 o4 = __ldcs(qin.o + i), d4 = __ldcs(qin.d + i), t4 = __ldcs(qin.t + i);
            slot = (uint32_t)__float_as_int(o4.w);
            r = shade_one<true>(S, o4, d4, t4, __ldcs(hits + i));
        }
        const uint32_t pos = warp_append(r.cont, cnt_out);
        if (r.cont) {
            __stcs(qout.o + pos, r.o);
            __stcs(qout.d + pos, r.d);
            __stcs(qout.t + pos, r.t);
        } else if (valid) {
            __stcs(slots + slot, r.result);
        }
    }
}

// Kahan-adds samples [0, k) of pixels [p0, p0+P) from their slots, in order.
__global__ void k_accumulate(const float4* __restrict__ slots, uint32_t p0, uint32_t P, uint32_t k,
                             float4* __restrict__ accum) {
    const uint32_t pl = blockIdx.x * blockDim.x + threadIdx.x;
    if (pl >= P) return;
    const uint32_t pix = p0 + pl;
    float4 a0 = accum[2 * (size_t)pix], a1 = accum[2 * (size_t)pix + 1];
    for (uint32_t s = 0; s < k; ++s) kahan_add(a0, a1, __ldcs(slots + (size_t)s * P + pl));
    accum[2 * (size_t)pix] = a0;
    accum[2 * (size_t)pix + 1] = a1;
}

__global__ void k_resolve(const float4* __restrict__ accum, uint32_t npix, float4* __restrict__ image_f,
                          uchar4* __restrict__ image8) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    float4 a0 = accum[2 * (size_t)pix];
    f3 mean = mk(a0.x / a0.w, a0.y / a0.w, a0.z / a0.w);
    if (image_f) image_f[pix] = make_float4(mean.x, mean.y, mean.z, 1.0f);
    if (image8) image8[pix] = make_color(mean);
}

// Arbitrary rays -> closest hit (t, original id, front face).
__global__ void __launch_bounds__(128) k_trace_rays(SceneView S, const float* __restrict__ rays, uint32_t n,
                                                    float tmin, float tmax, float* __restrict__ t_out,
                                                    int32_t* __restrict__ id_out, uint32_t* __restrict__ front_out,
                                                    uint32_t* __restrict__ err) {
    extern __shared__ unsigned char smem[];
    StackSmem sm;
    sm.node = reinterpret_cast<int*>(smem);
    sm.tn = reinterpret_cast<float*>(smem + sizeof(int) * kShared * blockDim.x);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f3 o = mk(rays[6 * (size_t)i], rays[6 * (size_t)i + 1], rays[6 * (size_t)i + 2]);
    f3 d = mk(rays[6 * (size_t)i + 3], rays[6 * (size_t)i + 4], rays[6 * (size_t)i + 5]);
    RayPre R = prep(o, d);
    TraceCounters K{0, 0};
    bool overflow = false;
    float t;
    int32_t k = trace_closest<false>(S, R, tmin, tmax, t, sm, threadIdx.x, blockDim.x, overflow, K);
    if (overflow) atomicOr(err, 1u);
    if (t_out) t_out[i] = t;
    uint32_t front = 0;
    int32_t id = -1;
    if (k >= 0) {
        id = (int32_t)(__ldg(S.meta + k) & 0x3fffffffu);
        float4 sp = __ldg(S.sph + k);
        f3 p = o + d * t;
        f3 outward = divs(p - mk(sp.x, sp.y, sp.z), sp.w);
        front = dot(d, outward) < 0.0f ? 1u : 0u;
    }
    if (id_out) id_out[i] = id;
    if (front_out) front_out[i] = front;
}

SceneView view_of(const venu_scene* s) {
    SceneView v;
    v.nodes = s->nodes;
    v.sph = s->sph;
    v.mat = s->mat;
    v.meta = s->meta;
    v.trav = s->trav;
    v.wide = s->wide;
    v.n = s->n;
    v.nhoist = s->nhoist;
    for (int i = 0; i < kMaxHoisted; ++i) v.hoist[i] = s->hoist[i];
    return v;
}

size_t traverse_smem(int block, int entries) { return (size_t)block * entries * (sizeof(int) + sizeof(float)); }
size_t traverse_smem(int block) { return traverse_smem(block, kShared); }

}  // namespace venu

using namespace venu;

// Everything the wave graph's kernels take as parameters, and their launch
// shape: the graph is rebuilt when any of it changes (zero-initialised, so
// that whole objects compare with memcmp).
struct WaveGraphKey {
    SceneView S;
    PrimaryGen pg;
    Queue q0, q1;
    uint32_t* cnt;
    uint32_t* work;
    float4* slots;
    uint32_t* err;
    unsigned long long* stats;
    WaveCtl* ctl;
    size_t fsm;
    int grid, block;
    uint32_t kind;  // bits: 4-wide tree, shallow stack, counting build, in-place refills
};

struct venu_renderer {
    uint32_t Q = 0;     // paths the queues hold now (grown on demand up to Qmax)
    uint32_t Qmax = 0;  // the wave size asked for at creation
    uint32_t flags = 0;
    Queue q[2] = {};
    int2* hits = nullptr;
    float4* slots = nullptr;
    uint32_t* seeds = nullptr;
    uint32_t seeds_cap = 0;
    uint32_t* cnt = nullptr;   // [65]
    uint32_t* work = nullptr;  // [65]
    uint32_t* err = nullptr;
    unsigned long long* stats = nullptr;  // segments, nodes, spheres, lane / warp steps, graph bounces
    venu_tuning tune = {2u, 32u, 128u, 0u, 128u, 0u, 1u};
    int trav_blocks = 0, shade_blocks = 0, fused_blocks = 0;
    venu_render_stats last = {};
    uint32_t host_launches = 0;  // kernels the last render launched from the host
    bool graph_off = false;      // the wave graph could not be built: host bounce loops only
    // the wave graph (fused variants): built on first use, kept while its key holds
    WaveCtl* ctl = nullptr;
    cudaStream_t cap = nullptr;
    cudaGraph_t wgraph = nullptr;
    cudaGraphExec_t wexec = nullptr;
    WaveGraphKey wkey;
    // VENU_RENDERER_PROFILE: event pairs around traverse (even) / shade (odd) launches
    std::vector<cudaEvent_t> ev;
    size_t ev_used = 0;
};

namespace {
constexpr int kTravBlock = 128;  // venu_trace
constexpr uint32_t kMaxDepth = 64;

template <typename K>
cudaError_t occupancy_grid(K kernel, int block, size_t smem, uint32_t per_sm_cap, int& grid) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
    if (e != cudaSuccess) return e;
    per_sm = std::max(1, per_sm);
    if (per_sm_cap) per_sm = std::min(per_sm, (int)per_sm_cap);
    grid = per_sm * sm_count();
    return cudaSuccess;
}

template <typename K>
cudaError_t set_smem_refill(K kernel, size_t smem) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// Persistent grids: as many resident blocks as fit (or the tuned cap) on every SM.
cudaError_t configure(venu_renderer* r) {
    const venu_tuning& t = r->tune;
    const size_t sm = traverse_smem((int)t.traverse_block);
    cudaError_t e;
    if (t.traverse_variant == 4) {  // the fused kernel over the 4-wide tree
        e = occupancy_grid(k_trace_shade_wide<false, kShared>, (int)t.traverse_block, sm,
                           t.traverse_blocks_per_sm, r->fused_blocks);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_trace_shade_wide<true, kShared>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sm);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_trace_shade_wide<false, kSharedShallow>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_trace_shade_wide<true, kSharedShallow>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e == cudaSuccess) e = set_smem_refill(k_trace_shade_wide<false, kShared, true>, sm);
        if (e == cudaSuccess) e = set_smem_refill(k_trace_shade_wide<true, kShared, true>, sm);
        if (e == cudaSuccess) e = set_smem_refill(k_trace_shade_wide<false, kSharedShallow, true>, sm);
        if (e == cudaSuccess) e = set_smem_refill(k_trace_shade_wide<true, kSharedShallow, true>, sm);
        if (e != cudaSuccess) return e;
        r->trav_blocks = r->fused_blocks;
    } else if (t.traverse_variant >= 2) {  // the fused kernel: every bounce (2), the primary one (3, 5)
        e = occupancy_grid(k_trace_shade<false, kShared>, (int)t.traverse_block, sm, t.traverse_blocks_per_sm,
                           r->fused_blocks);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_trace_shade<true, kShared>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        // the shallow-tree instantiation needs less shared memory; same grid
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_trace_shade<false, kSharedShallow>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sm);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_trace_shade<true, kSharedShallow>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sm);
        if (e == cudaSuccess) e = set_smem_refill(k_trace_shade<false, kShared, true>, sm);
        if (e == cudaSuccess) e = set_smem_refill(k_trace_shade<true, kShared, true>, sm);
        if (e == cudaSuccess) e = set_smem_refill(k_trace_shade<false, kSharedShallow, true>, sm);
        if (e == cudaSuccess) e = set_smem_refill(k_trace_shade<true, kSharedShallow, true>, sm);
        if (e != cudaSuccess) return e;
    }
    if (t.traverse_variant == 4) {
    } else if (t.traverse_variant == 5) {  // later bounces: the separate traversal over the wide tree
        e = occupancy_grid(k_traverse<false, true>, (int)t.traverse_block, sm, t.traverse_blocks_per_sm,
                           r->trav_blocks);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_traverse<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    } else if (t.traverse_variant == 0 || t.traverse_variant == 3) {
        e = occupancy_grid(k_traverse<false>, (int)t.traverse_block, sm, t.traverse_blocks_per_sm, r->trav_blocks);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_traverse<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    } else if (t.traverse_variant == 2) {
        r->trav_blocks = r->fused_blocks;
    } else {
        e = occupancy_grid(k_traverse_dyn<false>, (int)t.traverse_block, sm, t.traverse_blocks_per_sm, r->trav_blocks);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_traverse_dyn<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    }
    if (e == cudaSuccess) e = occupancy_grid(k_shade, (int)t.shade_block, 0, t.shade_blocks_per_sm, r->shade_blocks);
    if (e != cudaSuccess) return e;
    {
        const int nsm = std::max(1, sm_count());
        const int pf = std::max(1, r->fused_blocks / nsm), pt = std::max(1, r->trav_blocks / nsm);
        const size_t shallow = traverse_smem((int)t.traverse_block, kSharedShallow);
        if (t.traverse_variant == 4) {
            if (e == cudaSuccess) e = prefer_l1(k_trace_shade_wide<false, kShared>, pf, sm);
            if (e == cudaSuccess) e = prefer_l1(k_trace_shade_wide<false, kSharedShallow>, pf, shallow);
            if (e == cudaSuccess) e = prefer_l1(k_trace_shade_wide<false, kShared, true>, pf, sm);
            if (e == cudaSuccess) e = prefer_l1(k_trace_shade_wide<false, kSharedShallow, true>, pf, shallow);
        } else if (t.traverse_variant >= 2) {
            if (e == cudaSuccess) e = prefer_l1(k_trace_shade<false, kShared>, pf, sm);
            if (e == cudaSuccess) e = prefer_l1(k_trace_shade<false, kSharedShallow>, pf, shallow);
            if (e == cudaSuccess) e = prefer_l1(k_trace_shade<false, kShared, true>, pf, sm);
            if (e == cudaSuccess) e = prefer_l1(k_trace_shade<false, kSharedShallow, true>, pf, shallow);
        }
        if (t.traverse_variant == 5 && e == cudaSuccess) e = prefer_l1(k_traverse<false, true>, pt, sm);
        if ((t.traverse_variant == 0 || t.traverse_variant == 3) && e == cudaSuccess)
            e = prefer_l1(k_traverse<false>, pt, sm);
        if (t.traverse_variant == 1 && e == cudaSuccess) e = prefer_l1(k_traverse_dyn<false>, pt, sm);
        if (e == cudaSuccess) e = prefer_l1(k_shade, std::max(1, r->shade_blocks / nsm), 0);
    }
    return e;
}

// Returns an event pair for the next profiled launch, growing the pool.
cudaError_t next_events(venu_renderer* r, cudaEvent_t& a, cudaEvent_t& b) {
    while (r->ev_used + 2 > r->ev.size()) {
        cudaEvent_t e;
        cudaError_t err = cudaEventCreate(&e);
        if (err != cudaSuccess) return err;
        r->ev.push_back(e);
    }
    a = r->ev[r->ev_used];
    b = r->ev[r->ev_used + 1];
    r->ev_used += 2;
    return cudaSuccess;
}

void free_queues(venu_renderer* r) {
    for (int i = 0; i < 2; ++i) {
        cudaFree(r->q[i].o);
        cudaFree(r->q[i].d);
        cudaFree(r->q[i].t);
        r->q[i] = Queue{};
    }
    cudaFree(r->hits);
    cudaFree(r->slots);
    r->hits = nullptr;
    r->slots = nullptr;
    r->Q = 0;
}

// Path queues for waves of Q paths (96 B + 8 B hit + 16 B slot per path).
cudaError_t alloc_queues(venu_renderer* r, uint32_t Q) {
    free_queues(r);
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        if (e == cudaSuccess) e = cudaMalloc(&r->q[i].o, sizeof(float4) * (size_t)Q);
        if (e == cudaSuccess) e = cudaMalloc(&r->q[i].d, sizeof(float4) * (size_t)Q);
        if (e == cudaSuccess) e = cudaMalloc(&r->q[i].t, sizeof(float4) * (size_t)Q);
    }
    if (e == cudaSuccess) e = cudaMalloc(&r->hits, sizeof(int2) * (size_t)Q);
    if (e == cudaSuccess) e = cudaMalloc(&r->slots, sizeof(float4) * (size_t)Q);
    if (e != cudaSuccess) {
        free_queues(r);
        return e;
    }
    r->Q = Q;
    return cudaSuccess;
}

void destroy_wave_graph(venu_renderer* r);
constexpr uint32_t kFusedWide = 1u, kFusedShallow = 2u, kFusedCount = 4u, kFusedRefill = 8u;

// One bounce of the fused kernel (variant 2, or 4 over the 4-wide tree)
// with the renderer's launch shape.  ctl / handle: the wave graph's loop
// control, or nullptr / 0 for a launch from the host's bounce loop.
cudaError_t launch_fused(const venu_renderer* r, cudaStream_t st, uint32_t kind, size_t fsm, const SceneView& S,
                         const Queue& qi, uint32_t* cnt_in, uint32_t* work, const Queue& qo, uint32_t* cnt_out,
                         const PrimaryGen& pg, WaveCtl* ctl, cudaGraphConditionalHandle h) {
    const int grid = r->fused_blocks, tb = (int)r->tune.traverse_block;
#define VENU_FUSED(KERNEL, C, KS, RF)                                                                       \
    KERNEL<C, KS, RF><<<grid, tb, fsm, st>>>(S, qi, cnt_in, work, qo, cnt_out, r->slots, r->err, r->stats, pg, ctl, h)
#define VENU_FUSED_RF(KERNEL, C, KS)                  \
    do {                                              \
        if (kind & kFusedRefill)                      \
            VENU_FUSED(KERNEL, C, KS, true);          \
        else                                          \
            VENU_FUSED(KERNEL, C, KS, false);         \
    } while (0)
#define VENU_FUSED_CS(KERNEL, KS)                     \
    do {                                              \
        if (kind & kFusedCount)                       \
            VENU_FUSED_RF(KERNEL, true, KS);          \
        else                                          \
            VENU_FUSED_RF(KERNEL, false, KS);         \
    } while (0)
    if (kind & kFusedWide) {
        if (kind & kFusedShallow) VENU_FUSED_CS(k_trace_shade_wide, kSharedShallow);
        else VENU_FUSED_CS(k_trace_shade_wide, kShared);
    } else {
        if (kind & kFusedShallow) VENU_FUSED_CS(k_trace_shade, kSharedShallow);
        else VENU_FUSED_CS(k_trace_shade, kShared);
    }
#undef VENU_FUSED_CS
#undef VENU_FUSED_RF
#undef VENU_FUSED
    return cudaGetLastError();
}

// Builds the wave graph for `key` (see WaveCtl): the first bounce (camera
// rays from the per-path seeds, queue 0 -> 1), then while (rays left) {
// queue 1 -> 0; queue 0 -> 1 }.  After an odd bounce that leaves no rays the
// even one still starts and finds none, so a wave runs at most one empty
// launch.
venu_status build_wave_graph(venu_renderer* r, const WaveGraphKey& key) {
    destroy_wave_graph(r);
    if (!r->cap) VENU_CUDA(cudaStreamCreateWithFlags(&r->cap, cudaStreamNonBlocking));
    VENU_CUDA(cudaGraphCreate(&r->wgraph, 0));
    cudaGraph_t g = r->wgraph;
    cudaGraphConditionalHandle h = 0;
    VENU_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
    PrimaryGen later = key.pg;
    later.path_seeds = nullptr;  // bounces after the first read their rays from the queue
    VENU_CUDA(cudaStreamBeginCaptureToGraph(r->cap, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    cudaError_t le = launch_fused(r, r->cap, key.kind, key.fsm, key.S, key.q0, key.cnt, key.work, key.q1,
                                  key.cnt + 1, key.pg, key.ctl, h);
    cudaGraph_t captured = nullptr;
    cudaError_t ee = cudaStreamEndCapture(r->cap, &captured);
    if (le != cudaSuccess) return cuda_fail(le, "venu_render: capture of the first bounce");
    if (ee != cudaSuccess) return cuda_fail(ee, "venu_render: cudaStreamEndCapture");
    cudaGraphNode_t first = nullptr;
    size_t nn = 1;
    VENU_CUDA(cudaGraphGetNodes(g, &first, &nn));
    if (nn != 1) {
        set_error("venu_render: the first bounce captured as " + std::to_string(nn) + " graph nodes");
        return VENU_ERR_CUDA;
    }
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t loop = nullptr;
    VENU_CUDA(cudaGraphAddNode(&loop, g, &first, nullptr, 1, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    VENU_CUDA(cudaStreamBeginCaptureToGraph(r->cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    le = launch_fused(r, r->cap, key.kind, key.fsm, key.S, key.q1, key.cnt + 1, key.work + 1, key.q0, key.cnt,
                      later, key.ctl, h);
    if (le == cudaSuccess)
        le = launch_fused(r, r->cap, key.kind, key.fsm, key.S, key.q0, key.cnt, key.work, key.q1, key.cnt + 1,
                          later, key.ctl, h);
    ee = cudaStreamEndCapture(r->cap, &captured);
    if (le != cudaSuccess) return cuda_fail(le, "venu_render: capture of the bounce loop");
    if (ee != cudaSuccess) return cuda_fail(ee, "venu_render: cudaStreamEndCapture");
    VENU_CUDA(cudaGraphInstantiate(&r->wexec, g, 0));
    r->wkey = key;
    return VENU_OK;
}

void destroy_wave_graph(venu_renderer* r) {
    if (r->wexec) cudaGraphExecDestroy(r->wexec);
    if (r->wgraph) cudaGraphDestroy(r->wgraph);
    r->wexec = nullptr;
    r->wgraph = nullptr;
}

void free_renderer(venu_renderer* r) {
    for (cudaEvent_t e : r->ev) cudaEventDestroy(e);
    r->ev.clear();
    destroy_wave_graph(r);
    if (r->cap) cudaStreamDestroy(r->cap);
    r->cap = nullptr;
    cudaFree(r->ctl);
    free_queues(r);
    cudaFree(r->seeds);
    cudaFree(r->cnt);
    cudaFree(r->work);
    cudaFree(r->err);
    cudaFree(r->stats);
}
}  // namespace

extern "C" venu_status venu_renderer_create(uint32_t max_paths, uint32_t flags, venu_renderer** out) {
    if (!out) {
        set_error("venu_renderer_create: out is NULL");
        return VENU_ERR_INVALID;
    }
    *out = nullptr;
    venu_status ds = require_device();
    if (ds != VENU_OK) return ds;
    if (max_paths == 0) max_paths = 64u << 20;
    // 2^30 keeps every path position and slot below 2^31 (signed slot words,
    // FastDiv's range) at ~120 B per path (~129 GB at the maximum)
    if (max_paths > (1u << 30)) {
        set_error("venu_renderer_create: max_paths above 2^30");
        return VENU_ERR_TOO_LARGE;
    }
    venu_renderer* r = new venu_renderer();
    r->Qmax = max_paths;  // the queues are sized by the first render that needs them
    r->flags = flags;
    cudaError_t e = cudaMalloc(&r->cnt, sizeof(uint32_t) * (kMaxDepth + 1));
    if (e == cudaSuccess) e = cudaMalloc(&r->work, sizeof(uint32_t) * (kMaxDepth + 1));
    if (e == cudaSuccess) e = cudaMalloc(&r->err, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&r->stats, sizeof(unsigned long long) * 6);
    if (e == cudaSuccess) e = cudaMemset(r->err, 0, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(r->stats, 0, sizeof(unsigned long long) * 6);
    if (e == cudaSuccess) e = cudaMalloc(&r->ctl, sizeof(WaveCtl));
    if (e == cudaSuccess) e = cudaMemset(r->ctl, 0, sizeof(WaveCtl));
    if (e == cudaSuccess) e = configure(r);
    if (e != cudaSuccess) {
        free_renderer(r);
        delete r;
        return e == cudaErrorMemoryAllocation ? (set_error("venu_renderer_create: out of device memory"), VENU_ERR_OOM)
                                              : cuda_fail(e, "venu_renderer_create");
    }
    *out = r;
    return VENU_OK;
}

extern "C" venu_status venu_renderer_set_tuning(venu_renderer* r, const venu_tuning* t) {
    if (!r || !t) {
        set_error("venu_renderer_set_tuning: NULL argument");
        return VENU_ERR_INVALID;
    }
    const bool ok = t->traverse_variant <= 5u && t->refill_min >= 1u && t->refill_min <= 32u &&
                    (t->traverse_block == 64u || t->traverse_block == 128u || t->traverse_block == 256u) &&
                    t->shade_block >= 64u && t->shade_block <= 512u && (t->shade_block % 32u) == 0u &&
                    t->traverse_blocks_per_sm <= 32u && t->shade_blocks_per_sm <= 32u && t->in_place_factor <= 16u;
    if (!ok) {
        set_error("venu_renderer_set_tuning: value out of range");
        return VENU_ERR_INVALID;
    }
    const venu_tuning old = r->tune;
    r->tune = *t;
    cudaError_t e = configure(r);
    if (e != cudaSuccess) {
        r->tune = old;
        configure(r);
        return cuda_fail(e, "venu_renderer_set_tuning");
    }
    return VENU_OK;
}

extern "C" venu_status venu_renderer_get_tuning(const venu_renderer* r, venu_tuning* t) {
    if (!r || !t) {
        set_error("venu_renderer_get_tuning: NULL argument");
        return VENU_ERR_INVALID;
    }
    *t = r->tune;
    return VENU_OK;
}

extern "C" venu_status venu_renderer_destroy(venu_renderer* r) {
    if (!r) return VENU_OK;
    free_renderer(r);
    delete r;
    return VENU_OK;
}

extern "C" venu_status venu_render(venu_renderer* r, const venu_scene* scene, const venu_camera* camera,
                                   const venu_render_opts* opts, float* accum_dev, float* image_f_dev,
                                   uint8_t* image8_dev, void* stream) {
    if (!r || !scene || !camera || !opts || !accum_dev) {
        set_error("venu_render: NULL argument");
        return VENU_ERR_INVALID;
    }
    const uint32_t W = opts->width, H = opts->height, spp = opts->samples_per_pixel;
    const uint32_t maxd = opts->max_depth;
    if (W < 2 || H < 2 || spp == 0 || maxd == 0 || maxd > kMaxDepth) {
        set_error("venu_render: need width,height >= 2, spp >= 1, 1 <= max_depth <= 64");
        return VENU_ERR_INVALID;
    }
    const uint64_t npix64 = (uint64_t)W * H;
    if (npix64 > (1u << 30)) {
        set_error("venu_render: image above 2^30 pixels");
        return VENU_ERR_TOO_LARGE;
    }
    const uint32_t npix = (uint32_t)npix64;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (npix > r->seeds_cap) {
        cudaFree(r->seeds);
        r->seeds = nullptr;
        r->seeds_cap = 0;
        VENU_CUDA(cudaMalloc(&r->seeds, sizeof(uint32_t) * npix));
        r->seeds_cap = npix;
    }
    if (opts->flags & VENU_FLAG_RESET_ACCUM)
        VENU_CUDA(cudaMemsetAsync(accum_dev, 0, sizeof(float) * VENU_ACCUM_FLOATS_PER_PIXEL * npix64, st));
    VENU_CUDA(cudaMemsetAsync(r->stats, 0, sizeof(unsigned long long) * 6, st));
    if (r->tune.traverse_variant == 4u || r->tune.traverse_variant == 5u) {
        const venu_status ws = ensure_wide(scene, st);  // the first such render builds it
        if (ws != VENU_OK) return ws;
    }
    const SceneView S = view_of(scene);
    const bool count = (r->flags & VENU_RENDERER_COUNT) != 0;
    const bool prof = (r->flags & VENU_RENDERER_PROFILE) != 0;
    r->ev_used = 0;
    {
        // queues for waves of min(all paths of this call, Qmax): a small render
        // holds no more memory than it uses; grown (never shrunk) on demand
        const uint64_t want = std::min<uint64_t>((uint64_t)npix * spp, r->Qmax);
        if (want > r->Q) {
            VENU_CUDA(cudaStreamSynchronize(st));
            const cudaError_t ae = alloc_queues(r, (uint32_t)want);
            if (ae != cudaSuccess) {
                set_error("venu_render: cannot allocate path queues for " + std::to_string(want) + " paths");
                return VENU_ERR_OOM;
            }
        }
    }
    const venu_tuning& tu = r->tune;
    const size_t tsm = traverse_smem((int)tu.traverse_block);
    const int tb = (int)tu.traverse_block, sb = (int)tu.shade_block;
    float4* accum = reinterpret_cast<float4*>(accum_dev);
    uint32_t launches = 0, waves = 0;
    // wave shape: all pixels x k samples, or P pixels x 1 sample
    uint32_t P, k;
    if (npix <= r->Q) {
        P = npix;
        k = std::min(spp, r->Q / npix);
    } else {
        P = r->Q;
        k = 1;
    }
    const int nb = (int)maxd;
    // the fused first bounce (variants 2 and 3) makes its camera rays from
    // per-path seeds, kept in the first queue's throughput array (bounce 0
    // reads no queue and writes the other one)
    const bool gen0 = tu.traverse_variant >= 2u;
    // small scenes have shallow trees: a 4-entry shared stack leaves more of
    // the SM's memory to L1 (measured: RTIOW +0.5 %; 1M spheres -4.5 %)
    const bool shallow = scene->n <= 4096u;
    uint32_t* const path_seeds = gen0 ? reinterpret_cast<uint32_t*>(r->q[0].t) : nullptr;
    // the fused variants run each wave's bounce loop as one graph launch
    // (WaveCtl) when every wave covers all pixels, so that the graph's
    // parameters are the same for every wave; the profiling build times
    // every launch from the host
    const bool fused = tu.traverse_variant == 2u || tu.traverse_variant == 4u;
    // a caller capturing the stream into a graph of its own gets the
    // host's bounce loop captured (no graph launched inside the capture)
    cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
    VENU_CUDA(cudaStreamIsCapturing(st, &cap_status));
    bool use_graph = fused && !prof && P == npix && !r->graph_off && cap_status == cudaStreamCaptureStatusNone;
    const uint32_t kind = (tu.traverse_variant == 4u ? kFusedWide : 0u) | (shallow ? kFusedShallow : 0u) |
                          (count ? kFusedCount : 0u) | (tu.in_place_factor > 1u ? kFusedRefill : 0u);
    const size_t fsm = shallow ? traverse_smem(tb, kSharedShallow) : tsm;
    // the camera-ray generator of the wave of pixels [p0, p0 + PP)
    auto primary_gen = [&](uint32_t p0, uint32_t PP) {
        PrimaryGen pg;
        std::memset(&pg, 0, sizeof pg);  // the graph key compares whole objects
        pg.cam = *camera;
        pg.W = W;
        pg.H = H;
        pg.p0 = p0;
        pg.P = PP;
        pg.depth = (int)maxd - 1;
        pg.div_P = make_fastdiv(PP);
        pg.div_W = make_fastdiv(W);
        pg.in_place_factor = tu.in_place_factor ? tu.in_place_factor : 1u;
        return pg;
    };
    if (use_graph) {
        WaveGraphKey key;
        std::memset(&key, 0, sizeof key);
        key.S = S;
        key.pg = primary_gen(0u, npix);
        key.pg.path_seeds = path_seeds;
        key.q0 = r->q[0];
        key.q1 = r->q[1];
        key.cnt = r->cnt;
        key.work = r->work;
        key.slots = r->slots;
        key.err = r->err;
        key.stats = r->stats;
        key.ctl = r->ctl;
        key.fsm = fsm;
        key.grid = r->fused_blocks;
        key.block = tb;
        key.kind = kind;
        if (!r->wexec || std::memcmp(&key, &r->wkey, sizeof key) != 0) {
            if (build_wave_graph(r, key) != VENU_OK) {
                // graphs unavailable here: the host's bounce loop from now on
                destroy_wave_graph(r);
                (void)cudaGetLastError();
                r->graph_off = true;
                use_graph = false;
            }
        }
    }
    for (uint32_t s0 = 0; s0 < spp; s0 += k) {
        const uint32_t kk = std::min(k, spp - s0);
        for (uint32_t p0 = 0; p0 < npix; p0 += P) {
            const uint32_t PP = std::min(P, npix - p0);
            k_raygen<<<(PP + 255) / 256, 256, 0, st>>>(*camera, W, H, p0, PP, s0, kk, opts->subframe_index,
                                                       (int)maxd, r->seeds, r->q[0], path_seeds, r->cnt, r->work,
                                                       nb, use_graph ? r->ctl : nullptr);
            PrimaryGen pg = primary_gen(p0, PP);
            ++launches;
            if (use_graph) {  // the bounce loop of this wave: one graph launch
                VENU_CUDA(cudaGraphLaunch(r->wexec, st));
                k_accumulate<<<(PP + 255) / 256, 256, 0, st>>>(r->slots, p0, PP, kk, accum);
                ++launches;
                ++waves;
                continue;
            }
            for (int b = 0; b < nb; ++b) {
                const Queue& qi = r->q[b & 1];
                const Queue& qo = r->q[(b + 1) & 1];
                cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr, e3 = nullptr;
                if (prof) {
                    VENU_CUDA(next_events(r, e0, e1));
                    VENU_CUDA(next_events(r, e2, e3));
                    VENU_CUDA(cudaEventRecord(e0, st));
                }
                // variant 3: the coherent primary rays fused, the divergent
                // later bounces with the separate traversal kernel
                const uint32_t v = tu.traverse_variant <= 2u ? tu.traverse_variant
                                   : tu.traverse_variant == 4u ? 4u
                                   : tu.traverse_variant == 5u ? (b == 0 ? 2u : 5u)
                                                               : (b == 0 ? 2u : 0u);
                if ((v == 4 || v == 5) && scene->nwide == 0u && scene->n > 1u) {
                    set_error("venu_render: the scene has no wide tree");
                    return VENU_ERR_INVALID;
                }
                if (v == 2 || v == 4) {
                    pg.path_seeds = (b == 0) ? path_seeds : nullptr;
                    VENU_CUDA(launch_fused(r, st, kind, fsm, S, qi, r->cnt + b, r->work + b, qo, r->cnt + b + 1,
                                           pg, nullptr, 0));
                    if (prof) {
                        VENU_CUDA(cudaEventRecord(e1, st));
                        VENU_CUDA(cudaEventRecord(e2, st));
                        VENU_CUDA(cudaEventRecord(e3, st));
                    }
                    launches += 1;
                    // a first bounce that the fused kernel finishes in place
                    // finishes every path: no later bounce has rays
                    if (b == 0 && (uint64_t)PP * kk <= (uint64_t)pg.in_place_factor * r->fused_blocks * (uint64_t)tb)
                        break;
                    continue;
                }
                if (v == 0) {
                    if (count)
                        k_traverse<true><<<r->trav_blocks, tb, tsm, st>>>(S, qi, r->cnt + b, r->work + b, r->hits,
                                                                         r->err, r->stats);
                    else
                        k_traverse<false><<<r->trav_blocks, tb, tsm, st>>>(S, qi, r->cnt + b, r->work + b, r->hits,
                                                                          r->err, r->stats);
                } else if (v == 5) {
                    if (count)
                        k_traverse<true, true><<<r->trav_blocks, tb, tsm, st>>>(S, qi, r->cnt + b, r->work + b,
                                                                               r->hits, r->err, r->stats);
                    else
                        k_traverse<false, true><<<r->trav_blocks, tb, tsm, st>>>(S, qi, r->cnt + b, r->work + b,
                                                                                r->hits, r->err, r->stats);
                } else {
                    if (count)
                        k_traverse_dyn<true><<<r->trav_blocks, tb, tsm, st>>>(S, qi, r->cnt + b, r->work + b, r->hits,
                                                                             r->err, r->stats, tu.refill_min);
                    else
                        k_traverse_dyn<false><<<r->trav_blocks, tb, tsm, st>>>(S, qi, r->cnt + b, r->work + b,
                                                                              r->hits, r->err, r->stats, tu.refill_min);
                }
                if (prof) {
                    VENU_CUDA(cudaEventRecord(e1, st));
                    VENU_CUDA(cudaEventRecord(e2, st));
                }
                k_shade<<<r->shade_blocks, sb, 0, st>>>(S, qi, r->hits, r->cnt + b, qo, r->cnt + b + 1, r->slots);
                if (prof) VENU_CUDA(cudaEventRecord(e3, st));
                launches += 2;
            }
            k_accumulate<<<(PP + 255) / 256, 256, 0, st>>>(r->slots, p0, PP, kk, accum);
            ++launches;
            ++waves;
        }
    }
    if (image_f_dev || image8_dev) {
        k_resolve<<<(npix + 255) / 256, 256, 0, st>>>(accum, npix, reinterpret_cast<float4*>(image_f_dev),
                                                      reinterpret_cast<uchar4*>(image8_dev));
        ++launches;
    }
    VENU_CUDA(cudaGetLastError());
    r->last = venu_render_stats{};
    r->last.paths = (uint64_t)npix * spp;
    r->last.waves = waves;
    r->last.kernel_launches = launches;  // plus the wave graphs' bounces, counted on the device
    r->host_launches = launches;
    return VENU_OK;
}

extern "C" venu_status venu_renderer_stats(venu_renderer* r, venu_render_stats* out) {
    if (!r || !out) {
        set_error("venu_renderer_stats: NULL argument");
        return VENU_ERR_INVALID;
    }
    unsigned long long st[6] = {0, 0, 0, 0, 0, 0};
    uint32_t err = 0;
    VENU_CUDA(cudaMemcpy(st, r->stats, sizeof(st), cudaMemcpyDeviceToHost));
    VENU_CUDA(cudaMemcpy(&err, r->err, sizeof(err), cudaMemcpyDeviceToHost));
    r->last.segments = st[0];
    r->last.nodes_visited = st[1];
    r->last.spheres_tested = st[2];
    r->last.lane_steps = st[3];
    r->last.warp_steps = st[4];
    r->last.kernel_launches = r->host_launches + (uint32_t)st[5];
    // event pairs alternate traverse, shade (4 events per bounce)
    float tms = 0.0f, sms = 0.0f;
    uint32_t tn = 0, sn = 0;
    for (size_t i = 0; i + 3 < r->ev_used; i += 4) {
        float a = 0.0f, b = 0.0f;
        VENU_CUDA(cudaEventElapsedTime(&a, r->ev[i], r->ev[i + 1]));
        VENU_CUDA(cudaEventElapsedTime(&b, r->ev[i + 2], r->ev[i + 3]));
        tms += a;
        sms += b;
        ++tn;
        ++sn;
    }
    r->last.traverse_ms = tms;
    r->last.shade_ms = sms;
    r->last.traverse_launches = tn;
    r->last.shade_launches = sn;
    *out = r->last;
    if (err) {
        set_error("traversal stack overflow (result of at least one ray is incomplete)");
        return VENU_ERR_STACK;
    }
    return VENU_OK;
}

extern "C" venu_status venu_trace(const venu_scene* scene, const float* rays_dev, uint32_t n, float tmin,
                                  float tmax, float* t_dev, int32_t* id_dev, uint32_t* front_dev, void* stream) {
    if (!scene || (!rays_dev && n)) {
        set_error("venu_trace: NULL argument");
        return VENU_ERR_INVALID;
    }
    venu_status ds = require_device();
    if (ds != VENU_OK) return ds;
    if (n == 0) return VENU_OK;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    uint32_t* err = nullptr;
    VENU_CUDA(cudaMalloc(&err, sizeof(uint32_t)));
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(uint32_t), st);
    const size_t tsm = traverse_smem(kTravBlock);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_trace_rays, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm);
    if (e == cudaSuccess) {
        k_trace_rays<<<(n + kTravBlock - 1) / kTravBlock, kTravBlock, tsm, st>>>(view_of(scene), rays_dev, n, tmin,
                                                                               tmax, t_dev, id_dev, front_dev, err);
        e = cudaGetLastError();
    }
    uint32_t herr = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(err);
    if (e != cudaSuccess) return cuda_fail(e, "venu_trace");
    if (herr) {
        set_error("venu_trace: traversal stack overflow");
        return VENU_ERR_STACK;
    }
    return VENU_OK;
}
