// batch.cu -- many render jobs in one shared path pool (batched and served
// rendering).
//
// Every admitted job is a Renderer::Draw (Core/Renderer.h:35-78) of its own
// scene.  Instead of one wavefront per job, all jobs feed one pool of paths
// in flight:
//
//   trace+shade  every ray of the iteration against its own job's LBVH,
//                shaded, the survivors compacted into the other queue (the
//                job index rides in the upper bits of the depth word).  The
//                iteration's rays are the queued survivors followed by the
//                new paths the last plan handed out: those camera rays are
//                made in the kernel, from each job's precomputed raygen
//                seed table, and never pass through memory;
//   plan         one thread hands the free pool slots to the admitted jobs
//                in plan order (submission order, or shortest first);
//
// repeated under a device-side while condition, so the whole loop is one
// CUDA graph launch.  Which of the two queues is the input alternates each
// iteration through a parity word in device memory, so one iteration is one
// pass of the loop body and a run can end after any iteration.  Paths finish into per-job sample slots; a job whose
// paths are all done is accumulated (Kahan, sample order) and resolved by
// venu_batch_collect.  The seed table holds, for every (sample, pixel), the
// raygen RNG state at the start of that sample (Core/RayTracer.cu:169-177),
// which makes every path independent of generation order: results are
// bit-identical to venu_render of each job alone.
#include "render_kernels.cuh"
#include "venu_internal.h"

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

namespace venu {

struct DevJob {
    SceneView scene;
    venu_camera cam;
    DevCamera dcam;  // load_camera(cam), written by k_seed_tables
    uint32_t W, H, npix, spp, max_depth, subframe;
    FastDiv div_npix, div_W;  // make_fastdiv(npix), make_fastdiv(W)
    const uint32_t* seeds;  // [spp * npix], sample-major
    float4* slots;          // [spp * npix], sample-major
    unsigned long long total;
};

struct LoopCtl {  // device-owned loop state
    uint32_t cnt[2], work[2];
    uint32_t iter, running;
    uint32_t gen_n;     // new paths of this iteration (made by the trace kernel) ...
    uint32_t gen_base;  // ... at input indices [gen_base, gen_base + gen_n), after the survivors
    uint32_t plan_n, err;
    uint32_t job_finished;  // set when a job's last path finishes (reset per run)
    uint32_t parity;        // the queue traced in this iteration; flipped by k_plan
    uint32_t chunk_end;     // this step traces input rays [chunk_start, chunk_end)
    uint32_t chunk_start;
    unsigned long long segments, paths_done, iterations;
};

struct RunCtl {  // host-written before each run
    uint32_t max_iter, nactive, stop_on_finish, sequential;
    uint32_t chunk, pad[3];  // rays traced per step (0: the whole input queue)
};

struct CollectEntry {
    float4* accum;
    float4* image_f;
    uchar4* image8;
    const float4* slots;
    uint32_t npix, spp, reset, pix_off;
};

// Up to kSeedGroup jobs admitted by one launch, passed by value (no staging
// copy): their table entries, table slots and pixel offsets.
constexpr uint32_t kSeedGroup = 32;
struct SeedGroup {
    DevJob job[kSeedGroup];
    uint32_t slot[kSeedGroup];
    uint32_t pix_off[kSeedGroup + 1];  // pix_off[k]: first thread of job k; pix_off[n]: all pixels
    uint32_t n;
};

// Admits a group of jobs: each job's raygen RNG state at the start of every
// sample of every pixel (the seed table, one thread per pixel), and -- from
// each job's first thread -- its table entry with the camera basis and
// zeroed counters.  A submit is one allocation per job and one launch per
// group.
__global__ void k_seed_tables(const __grid_constant__ SeedGroup g, DevJob* __restrict__ jobs,
                              unsigned long long* __restrict__ job_next, unsigned long long* __restrict__ job_done,
                              uint32_t* __restrict__ job_seen) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.pix_off[g.n]) return;
    uint32_t lo = 0, hi = g.n;  // last job k with pix_off[k] <= t
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (g.pix_off[mid] <= t) lo = mid; else hi = mid;
    }
    const DevJob& dj = g.job[lo];
    const uint32_t pix = t - g.pix_off[lo];
    const uint32_t W = dj.W, npix = dj.npix;
    const DevCamera C = load_camera(dj.cam);
    if (pix == 0) {
        const uint32_t slot = g.slot[lo];
        DevJob w = dj;
        w.dcam = C;
        jobs[slot] = w;
        job_next[slot] = 0ull;
        job_done[slot] = 0ull;
        job_seen[slot] = 0u;
    }
    uint32_t* __restrict__ seeds = const_cast<uint32_t*>(dj.seeds);
    const uint32_t x = pix % W, y = pix / W;
    uint32_t seed = tea4(pix, dj.subframe);
    for (uint32_t s = 0; s < dj.spp; ++s) {
        seeds[(size_t)s * npix + pix] = seed;
        f3 o, d;
        camera_ray(C, x, y, W, dj.H, seed, o, d);  // advances the seed past the sample's draws
    }
}

// Hands the free pool slots to the jobs (plan order) and flips the parity;
// returns whether any work is left.  sequential: a job gets slots only once
// every job before it in the order has finished all its paths (one job at a
// time, as rendering them in turn).  One warp: jobs go 32 at a time, one per
// lane.  The greedy hand-out -- each job in order takes min(its remaining
// paths, the slots still free) -- has a closed form: the slots taken by jobs
// 0..k together are min(free, the sum of their remaining paths), so a warp
// prefix sum gives every job's share and offset at once.
__device__ uint32_t plan_iteration(const DevJob* __restrict__ jobs, unsigned long long* __restrict__ job_next,
                                   const unsigned long long* __restrict__ job_done,
                                   const uint32_t* __restrict__ order, const RunCtl* __restrict__ run,
                                   LoopCtl* ctl, uint32_t* __restrict__ plan_job,
                                   unsigned long long* __restrict__ plan_start, uint32_t* __restrict__ plan_off,
                                   uint32_t Q, int in, int out, uint32_t chunk) {
    const uint32_t lane = threadIdx.x;  // a single 32-thread block
    const uint32_t survivors = ctl->cnt[out];
    const unsigned long long free = survivors < Q ? Q - survivors : 0u;
    const uint32_t na = run->nactive;
    const bool sequential = run->sequential != 0u;
    unsigned long long carry = 0;  // remaining paths of the unblocked jobs before this chunk
    bool blocked_before = false, more = false;
    for (uint32_t base = 0; base < na; base += 32u) {
        const uint32_t i = base + lane;
        const bool valid = i < na;
        uint32_t j = 0;
        unsigned long long total = 0, nx = 0;
        if (valid) {
            j = order[i];
            total = jobs[j].total;
            nx = job_next[j];
        }
        const bool unfinished = valid && sequential && job_done[j] < total;
        const uint32_t um = __ballot_sync(0xffffffffu, unfinished);
        // blocked: an earlier job of the order has not finished (the job that
        // has not finished itself still takes slots)
        const bool blocked = blocked_before || (um & ((1u << lane) - 1u)) != 0u;
        const unsigned long long rem = (valid && !blocked) ? total - nx : 0ull;
        unsigned long long incl = rem;  // inclusive prefix sum over the lanes
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long v = __shfl_up_sync(0xffffffffu, incl, d);
            if ((int)lane >= d) incl += v;
        }
        const unsigned long long before = min(free, carry + incl - rem);
        const unsigned long long upto = min(free, carry + incl);
        const unsigned long long take = upto - before;
        if (valid) {
            plan_job[i] = j;
            plan_start[i] = nx;
            plan_off[i] = (uint32_t)before;
            job_next[j] = nx + take;
        }
        more = more || __any_sync(0xffffffffu, valid && nx + take < total);
        carry += __shfl_sync(0xffffffffu, incl, 31);
        blocked_before = blocked_before || um != 0u;
    }
    const uint32_t off = (uint32_t)min(free, carry);
    __syncwarp();  // every lane has read the loop state before lane 0 rewrites it
    if (lane == 0) {
        plan_off[na] = off;
        ctl->plan_n = na;
        ctl->gen_n = off;
        ctl->gen_base = survivors;
        ctl->cnt[out] = survivors + off;
        ctl->cnt[in] = 0;    // the next trace writes into the other queue
        ctl->work[out] = 0;  // and fetches from this one, chunk by chunk
        ctl->chunk_start = 0u;
        ctl->chunk_end = min(chunk, survivors + off);
        ctl->parity = (uint32_t)out;
    }
    return (survivors + off > 0u || more) ? 1u : 0u;
}

// Decides the next step and whether there is one (one warp).  The loop
// condition: more rays or paths to generate, and none of the step cap, "a
// job just finished" (stop-on-finish) or the host's interrupt word (mapped
// host memory, read volatile).  A step traces a chunk of the input queue
// (RunCtl::chunk rays, all of them when 0); while input rays are left the
// next step takes the next chunk, else this plans the next iteration and
// flips the queue parity: the queue filled now is the one traced next.
__global__ void __launch_bounds__(32) k_plan(const DevJob* __restrict__ jobs,
                                             unsigned long long* __restrict__ job_next,
                                             const unsigned long long* __restrict__ job_done,
                                             uint32_t* __restrict__ job_seen, const uint32_t* __restrict__ order,
                                             const RunCtl* __restrict__ run, LoopCtl* ctl,
                                             uint32_t* __restrict__ plan_job,
                                             unsigned long long* __restrict__ plan_start,
                                             uint32_t* __restrict__ plan_off, uint32_t Q,
                                             const volatile uint32_t* interrupt,
                                             cudaGraphConditionalHandle handle, int use_handle) {
    const uint32_t lane = threadIdx.x;
    // jobs whose last path finished in this step
    bool fin = false;
    const uint32_t na = run->nactive;
    for (uint32_t i = lane; i < na; i += 32u) {
        const uint32_t j = order[i];
        if (!job_seen[j] && job_done[j] >= jobs[j].total) {
            job_seen[j] = 1u;
            fin = true;
        }
    }
    if (__any_sync(0xffffffffu, fin) && lane == 0) ctl->job_finished = 1u;
    const int in = (int)(ctl->parity & 1u), out = 1 - in;
    const uint32_t chunk = run->chunk ? run->chunk : 0xffffffffu;
    const uint32_t it = ctl->iter + 1u;
    const uint32_t n_in = ctl->cnt[in], done_to = ctl->chunk_end;
    __syncwarp();
    uint32_t go;
    if (done_to < n_in) {  // input rays left: the next chunk of this queue
        if (lane == 0) {
            ctl->work[in] = done_to;
            ctl->chunk_start = done_to;
            ctl->chunk_end = done_to + min(chunk, n_in - done_to);
        }
        go = 1u;
    } else {
        go = plan_iteration(jobs, job_next, job_done, order, run, ctl, plan_job, plan_start, plan_off, Q, in, out,
                            chunk);
    }
    if (lane != 0) return;
    ctl->iter = it;
    ctl->iterations += 1u;
    if (run->max_iter && it >= run->max_iter) go = 0u;
    if (run->stop_on_finish && ctl->job_finished) go = 0u;  // hand finished jobs to the host now
    if (*interrupt) go = 0u;                                 // the host has new work to admit
    ctl->running = go;
    if (use_handle) cudaGraphSetConditional(handle, go);
}

// The camera ray of new path t of the iteration (t < gen_n): its plan entry
// (the last entry i with plan_off[i] <= t; entries may be empty), job, sample
// and pixel, from the job's seed table -- what k_raygen writes to the queue
// for venu_render.  Path numbers within a job fit 31 bits (venu_batch_submit).
__device__ __forceinline__ void gen_primary(const DevJob* __restrict__ jobs, const uint32_t* __restrict__ plan_job,
                                            const unsigned long long* __restrict__ plan_start,
                                            const uint32_t* __restrict__ plan_off, uint32_t np, uint32_t t,
                                            float4& o4, float4& d4, uint32_t& seed) {
    uint32_t lo = 0, hi = np;  // invariant: plan_off[lo] <= t < plan_off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (plan_off[mid] <= t) lo = mid; else hi = mid;
    }
    const uint32_t j = plan_job[lo];
    const DevJob& J = jobs[j];
    const uint32_t l = (uint32_t)(plan_start[lo] + (t - plan_off[lo]));
    const uint32_t npix = J.npix, W = J.W;
    const uint32_t s = fast_div(l, J.div_npix);
    const uint32_t pix = l - s * npix;
    const uint32_t y = fast_div(pix, J.div_W);
    seed = J.seeds[l];
    f3 o, d;
    camera_ray(J.dcam, pix - y * W, y, W, J.H, seed, o, d);
    o4 = make_float4(o.x, o.y, o.z, __int_as_float((int)l));
    d4 = make_float4(d.x, d.y, d.z, __uint_as_float((j << 8) | ((uint32_t)((int)J.max_depth - 1) & kDepthMask)));
}

// A pointer read that the compiler may not merge with an earlier read of the
// same field (so the value is not kept live in a register meanwhile).
template <typename T>
__device__ __forceinline__ T ld_volatile_ptr(const T* p) {
    return *reinterpret_cast<const volatile T*>(p);
}

// One warp-batch loop of the batch kernel.  IN_PLACE (a step with no more
// rays than the grid has threads): each path is finished in place, bounce
// after bounce (the step leaves no survivors); the output queue is unused
// then, and its throughput slot i carries ray i's state between bounces.
// (Chunked steps: survivors of earlier chunks of the iteration sit below
// chunk_start, which no scratch index reaches.)  A separate instantiation,
// so the ordinary loop keeps its registers.
template <bool COUNT, bool IN_PLACE>
__device__ __forceinline__ void trace_shade_multi_loop(const DevJob* __restrict__ jobs,
                                                       unsigned long long* __restrict__ job_done, LoopCtl* ctl,
                                                       const uint32_t* __restrict__ plan_job,
                                                       const unsigned long long* __restrict__ plan_start,
                                                       const uint32_t* __restrict__ plan_off, const Queue& qin,
                                                       const Queue& qout, int in, int out, StackSmem sm,
                                                       bool& overflow, TraceCounters& K, uint32_t& finished,
                                                       uint32_t& traced) {
    const uint32_t n = ctl->chunk_end;  // this step: input rays [chunk_start, chunk_end)
    const uint32_t gen_base = ctl->gen_base, np = ctl->plan_n;  // new paths from gen_base on
    const uint32_t lane = threadIdx.x & 31;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&ctl->work[in], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane;
        const bool valid = i < n;
        uint32_t job = 0xFFFFFFFFu;
        ShadeOut r;
        r.cont = false;
        if (valid) {
            const bool fresh = i >= gen_base;
            float4 o4, d4;
            uint32_t seed = 0;
            int32_t from = -1;
            if (fresh) {
                gen_primary(jobs, plan_job, plan_start, plan_off, np, i - gen_base, o4, d4, seed);
            } else {
                o4 = qin.o[i];
                d4 = qin.d[i];
                from = qin.from[i];
            }
            job = __float_as_uint(d4.w) >> 8;
            for (bool first = true;; first = false) {
                RayPre R = prep(mk(o4.x, o4.y, o4.z), mk(d4.x, d4.y, d4.z));
                R.from = from;
                float t;
                int32_t k;
                {
                    const SceneView S = jobs[job].scene;
                    k = trace_closest<COUNT>(S, R, 0.001f, 1e16f, t, sm, threadIdx.x, blockDim.x, overflow, K);
                }
                ++traced;  // per lane: one segment
                // the shading pointers are read again here instead of being kept in
                // registers through the traversal (the job table is L1/L2-resident)
                SceneView S2;
                const SceneView* G = &jobs[job].scene;
                S2.sph = ld_volatile_ptr(&G->sph);
                S2.mat = ld_volatile_ptr(&G->mat);
                S2.meta = ld_volatile_ptr(&G->meta);
                const float4 t4 = (IN_PLACE && !first) ? qout.t[i]
                                  : fresh                ? make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(seed))
                                                         : qin.t[i];
                const float4 ow = o4;  // .w: the path's slot
                r = shade_one<false>(S2, o4, d4, t4, make_int2(__float_as_int(t), k));
                if (!r.cont) jobs[job].slots[(uint32_t)__float_as_int(ow.w)] = r.result;
                if (!IN_PLACE || !r.cont) break;
                o4 = r.o;
                d4 = r.d;
                from = r.from;
                qout.t[i] = r.t;
            }
        }
        const uint32_t pos = warp_append(r.cont, &ctl->cnt[out]);
        if (r.cont) {
            qout.o[pos] = r.o;
            qout.d[pos] = r.d;
            qout.t[pos] = r.t;
            qout.from[pos] = r.from;
        }
        // finished paths per job: one atomic per distinct job in the warp
        const bool fin = valid && !r.cont;
        const uint32_t key = fin ? job : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        // (the result is not read: a fire-and-forget reduction; k_plan
        // notices finished jobs)
        if (fin && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&job_done[job], (unsigned long long)__popc(peers));
        finished += __popc(__ballot_sync(0xffffffffu, fin));
    }
}

template <bool COUNT>
__global__ void VENU_TRACE_MULTI_BOUNDS k_trace_shade_multi(const DevJob* __restrict__ jobs,
                                                           unsigned long long* __restrict__ job_done, LoopCtl* ctl,
                                                           const uint32_t* __restrict__ plan_job,
                                                           const unsigned long long* __restrict__ plan_start,
                                                           const uint32_t* __restrict__ plan_off,
                                                           Queue q0, Queue q1) {
    extern __shared__ unsigned char smem[];
    StackSmem sm;
    sm.node = reinterpret_cast<int*>(smem);
    sm.tn = reinterpret_cast<float*>(smem + sizeof(int) * kShared * blockDim.x);
    const int in = (int)(ctl->parity & 1u), out = 1 - in;
    const Queue qin = in ? q1 : q0, qout = in ? q0 : q1;
    const uint32_t lane = threadIdx.x & 31;
    TraceCounters K{0, 0};
    bool overflow = false;
    uint32_t finished = 0, traced = 0;
    if (ctl->chunk_end - ctl->chunk_start <= gridDim.x * blockDim.x)
        trace_shade_multi_loop<COUNT, true>(jobs, job_done, ctl, plan_job, plan_start, plan_off, qin, qout, in, out,
                                            sm, overflow, K, finished, traced);
    else
        trace_shade_multi_loop<COUNT, false>(jobs, job_done, ctl, plan_job, plan_start, plan_off, qin, qout, in, out,
                                             sm, overflow, K, finished, traced);
    for (int off = 16; off > 0; off >>= 1) traced += __shfl_xor_sync(0xffffffffu, traced, off);
    if (lane == 0 && finished) atomicAdd(&ctl->paths_done, (unsigned long long)finished);
    if (lane == 0 && traced) atomicAdd(&ctl->segments, (unsigned long long)traced);
    if (overflow) atomicOr(&ctl->err, 1u);
}


// Accumulate (Kahan, sample order) and resolve finished jobs: one thread per
// pixel of the listed jobs.
__global__ void k_collect(const CollectEntry* __restrict__ ent, uint32_t nent, uint32_t total_pix) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total_pix) return;
    uint32_t lo = 0, hi = nent;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (ent[mid].pix_off <= t) lo = mid; else hi = mid;
    }
    const CollectEntry& E = ent[lo];
    const uint32_t pix = t - E.pix_off;
    float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0;
    if (!E.reset) {
        a0 = E.accum[2 * (size_t)pix];
        a1 = E.accum[2 * (size_t)pix + 1];
    }
    for (uint32_t s = 0; s < E.spp; ++s) kahan_add(a0, a1, E.slots[(size_t)s * E.npix + pix]);
    E.accum[2 * (size_t)pix] = a0;
    E.accum[2 * (size_t)pix + 1] = a1;
    const f3 mean = mk(a0.x / a0.w, a0.y / a0.w, a0.z / a0.w);
    if (E.image_f) E.image_f[pix] = make_float4(mean.x, mean.y, mean.z, 1.0f);
    if (E.image8) E.image8[pix] = make_color(mean);
}

SceneView view_of(const venu_scene* s);
size_t traverse_smem(int block);

}  // namespace venu

using namespace venu;

namespace {

struct JobHost {
    bool active = false;
    venu_job_desc desc{};
    uint64_t total = 0, bytes = 0;
    uint64_t seq = 0;        // submission number
    uint64_t remaining = 0;  // paths not finished at the last collect
    uint32_t* seeds = nullptr;
    float4* slots = nullptr;
};

constexpr uint32_t kMaxJobs = 4096;

}  // namespace

struct venu_batch {
    uint32_t Q = 0, max_jobs = 0, flags = 0;
    Queue q[2] = {};
    DevJob* d_jobs = nullptr;
    unsigned long long *d_next = nullptr, *d_done = nullptr, *d_plan_start = nullptr;
    uint32_t* d_seen = nullptr;  // per job: finish already reported by k_plan
    uint32_t *d_order = nullptr, *d_plan_job = nullptr, *d_plan_off = nullptr;
    LoopCtl* d_ctl = nullptr;
    RunCtl* d_run = nullptr;
    CollectEntry* d_collect = nullptr;
    std::vector<JobHost> jobs;
    std::vector<uint32_t> order;  // active job slots in plan order (policy)
    uint32_t policy = VENU_POLICY_FIFO;
    bool order_dirty = false;     // b->order changed since it was last uploaded (at the next run)
    uint32_t chunk = 0;  // rays traced per step (0: a whole iteration per step)
    uint64_t next_seq = 0;
    uint32_t* h_interrupt = nullptr;  // mapped host word
    uint32_t* d_interrupt = nullptr;  // its device address
    venu_tuning tune = {2u, 8u, 256u, 0u, 256u, 0u, 1u};
    int trav_blocks = 0;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphConditionalHandle handle = 0;
    uint64_t graph_launches = 0, resident = 0;
};

namespace {

cudaError_t batch_configure(venu_batch* b) {
    const size_t sm = traverse_smem((int)b->tune.traverse_block);
    cudaError_t e = cudaFuncSetAttribute(k_trace_shade_multi<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    int per_sm = 0;
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_shade_multi<false>,
                                                          (int)b->tune.traverse_block, sm);
    if (e != cudaSuccess) return e;
    per_sm = std::max(1, per_sm);
    if (b->tune.traverse_blocks_per_sm) per_sm = std::min(per_sm, (int)b->tune.traverse_blocks_per_sm);
    b->trav_blocks = per_sm * sm_count();
    return prefer_l1(k_trace_shade_multi<false>, per_sm, sm);
}

// One iteration of the path loop: trace the parity queue and the planned new
// paths, then plan (which also sets the loop condition and flips the parity).
cudaError_t launch_body(venu_batch* b, cudaStream_t st, bool use_handle) {
    const size_t sm = traverse_smem((int)b->tune.traverse_block);
    k_trace_shade_multi<false><<<b->trav_blocks, b->tune.traverse_block, sm, st>>>(
        b->d_jobs, b->d_done, b->d_ctl, b->d_plan_job, b->d_plan_start, b->d_plan_off, b->q[0], b->q[1]);
    k_plan<<<1, 32, 0, st>>>(b->d_jobs, b->d_next, b->d_done, b->d_seen, b->d_order, b->d_run, b->d_ctl, b->d_plan_job,
                             b->d_plan_start, b->d_plan_off, b->Q, b->d_interrupt, b->handle, use_handle ? 1 : 0);
    return cudaGetLastError();
}

void destroy_graph(venu_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->handle = 0;
}

// while (condition) { body } as one executable graph.
venu_status build_graph(venu_batch* b) {
    destroy_graph(b);
    VENU_CUDA(cudaGraphCreate(&b->graph, 0));
    VENU_CUDA(cudaGraphConditionalHandleCreate(&b->handle, b->graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = b->handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    VENU_CUDA(cudaGraphAddNode(&node, b->graph, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    VENU_CUDA(cudaStreamBeginCaptureToGraph(b->cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    cudaError_t le = launch_body(b, b->cap, true);
    cudaGraph_t captured = nullptr;
    cudaError_t ee = cudaStreamEndCapture(b->cap, &captured);
    if (le != cudaSuccess) return cuda_fail(le, "venu_batch: capture of the path loop");
    if (ee != cudaSuccess) return cuda_fail(ee, "venu_batch: cudaStreamEndCapture");
    VENU_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    return VENU_OK;
}

void free_batch(venu_batch* b) {
    destroy_graph(b);
    for (auto& j : b->jobs) cudaFree(j.slots);  // seeds share the allocation
    for (int i = 0; i < 2; ++i) {
        cudaFree(b->q[i].o);
        cudaFree(b->q[i].d);
        cudaFree(b->q[i].t);
        cudaFree(b->q[i].from);
    }
    cudaFree(b->d_jobs);
    cudaFree(b->d_next);
    cudaFree(b->d_done);
    cudaFree(b->d_seen);
    cudaFree(b->d_plan_start);
    cudaFree(b->d_order);
    cudaFree(b->d_plan_job);
    cudaFree(b->d_plan_off);
    cudaFree(b->d_ctl);
    cudaFree(b->d_run);
    cudaFree(b->d_collect);
    if (b->h_interrupt) cudaFreeHost(b->h_interrupt);
    if (b->cap) cudaStreamDestroy(b->cap);
}

// Plan order: submission order (FIFO), or fewest unfinished paths first
// (shortest remaining first; ties by submission).  The order decides only
// which job's new paths take free pool slots first -- never the results.
venu_status upload_order(venu_batch* b, cudaStream_t st) {
    if (b->policy == VENU_POLICY_SHORTEST_FIRST)
        std::stable_sort(b->order.begin(), b->order.end(), [b](uint32_t x, uint32_t y) {
            const JobHost &X = b->jobs[x], &Y = b->jobs[y];
            return X.remaining != Y.remaining ? X.remaining < Y.remaining : X.seq < Y.seq;
        });
    else
        std::stable_sort(b->order.begin(), b->order.end(),
                         [b](uint32_t x, uint32_t y) { return b->jobs[x].seq < b->jobs[y].seq; });
    if (!b->order.empty())
        VENU_CUDA(cudaMemcpyAsync(b->d_order, b->order.data(), sizeof(uint32_t) * b->order.size(),
                                  cudaMemcpyHostToDevice, st));
    return VENU_OK;
}

}  // namespace

extern "C" uint64_t venu_batch_job_bytes(uint32_t width, uint32_t height, uint32_t spp) {
    const uint64_t paths = (uint64_t)width * height * spp;
    return paths * (sizeof(uint32_t) + sizeof(float4));
}

extern "C" venu_status venu_batch_create(uint32_t pool_paths, uint32_t max_jobs, uint32_t flags, venu_batch** out) {
    if (!out) {
        set_error("venu_batch_create: out is NULL");
        return VENU_ERR_INVALID;
    }
    *out = nullptr;
    venu_status ds = require_device();
    if (ds != VENU_OK) return ds;
    if (pool_paths == 0) pool_paths = 64u << 20;
    if (max_jobs == 0 || max_jobs > kMaxJobs || pool_paths > (1u << 28)) {
        set_error("venu_batch_create: need 1 <= max_jobs <= 4096 and pool_paths <= 2^28");
        return VENU_ERR_INVALID;
    }
    venu_batch* b = new venu_batch();
    b->Q = pool_paths;
    b->max_jobs = max_jobs;
    b->flags = flags;
    b->jobs.resize(max_jobs);
    cudaError_t e = cudaSuccess;
    const size_t Q = pool_paths;
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        if (e == cudaSuccess) e = cudaMalloc(&b->q[i].o, sizeof(float4) * Q);
        if (e == cudaSuccess) e = cudaMalloc(&b->q[i].d, sizeof(float4) * Q);
        if (e == cudaSuccess) e = cudaMalloc(&b->q[i].t, sizeof(float4) * Q);
        if (e == cudaSuccess) e = cudaMalloc(&b->q[i].from, sizeof(int32_t) * Q);
    }
    if (e == cudaSuccess) e = cudaMalloc(&b->d_jobs, sizeof(DevJob) * max_jobs);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_next, sizeof(unsigned long long) * max_jobs);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_done, sizeof(unsigned long long) * max_jobs);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_seen, sizeof(uint32_t) * max_jobs);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_plan_start, sizeof(unsigned long long) * max_jobs);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_order, sizeof(uint32_t) * max_jobs);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_plan_job, sizeof(uint32_t) * max_jobs);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_plan_off, sizeof(uint32_t) * (max_jobs + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_ctl, sizeof(LoopCtl));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_run, sizeof(RunCtl));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_collect, sizeof(CollectEntry) * max_jobs);
    if (e == cudaSuccess) e = cudaMemset(b->d_ctl, 0, sizeof(LoopCtl));
    if (e == cudaSuccess) e = cudaMemset(b->d_run, 0, sizeof(RunCtl));
    if (e == cudaSuccess) e = cudaMemset(b->d_jobs, 0, sizeof(DevJob) * max_jobs);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaHostAlloc(&b->h_interrupt, sizeof(uint32_t), cudaHostAllocMapped);
    if (e == cudaSuccess) {
        *b->h_interrupt = 0u;
        e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&b->d_interrupt), b->h_interrupt, 0);
    }
    if (e == cudaSuccess) e = batch_configure(b);
    if (e != cudaSuccess) {
        venu_status s = cuda_fail(e, "venu_batch_create");
        free_batch(b);
        delete b;
        return s;
    }
    *out = b;
    return VENU_OK;
}

extern "C" venu_status venu_batch_set_tuning(venu_batch* b, const venu_tuning* t) {
    if (!b || !t) {
        set_error("venu_batch_set_tuning: NULL argument");
        return VENU_ERR_INVALID;
    }
    if (!(t->traverse_block == 64u || t->traverse_block == 128u || t->traverse_block == 256u) ||
        t->traverse_blocks_per_sm > 32u) {
        set_error("venu_batch_set_tuning: traverse_block must be 64, 128 or 256");
        return VENU_ERR_INVALID;
    }
    b->tune = *t;
    b->tune.traverse_variant = 2u;  // the batch loop always traces and shades in one kernel
    cudaError_t e = batch_configure(b);
    if (e != cudaSuccess) return cuda_fail(e, "venu_batch_set_tuning");
    destroy_graph(b);  // rebuilt with the new launch shapes on the next run
    return VENU_OK;
}

namespace {

venu_status check_job(const venu_job_desc* job, uint32_t k) {
    const std::string at = "venu_batch_submit: job " + std::to_string(k) + ": ";
    if (!job->scene || !job->accum) {
        set_error(at + "NULL scene or accumulator");
        return VENU_ERR_INVALID;
    }
    const venu_render_opts& o = job->opts;
    if (o.width < 2 || o.height < 2 || o.samples_per_pixel == 0 || o.max_depth == 0 || o.max_depth > 64) {
        set_error(at + "need width,height >= 2, spp >= 1, 1 <= max_depth <= 64");
        return VENU_ERR_INVALID;
    }
    const uint64_t npix = (uint64_t)o.width * o.height, total = npix * o.samples_per_pixel;
    if (npix > (1u << 30) || total > 0x7fffffffull) {
        set_error(at + "a job may have at most 2^31 - 1 paths");
        return VENU_ERR_TOO_LARGE;
    }
    return VENU_OK;
}

cudaError_t launch_seed_group(venu_batch* b, SeedGroup& g, cudaStream_t st) {
    if (g.n == 0) return cudaSuccess;
    const uint32_t threads = g.pix_off[g.n];
    k_seed_tables<<<(threads + 255) / 256, 256, 0, st>>>(g, b->d_jobs, b->d_next, b->d_done, b->d_seen);
    g.n = 0;
    g.pix_off[0] = 0;
    return cudaGetLastError();
}

}  // namespace

extern "C" venu_status venu_batch_submit_many(venu_batch* b, const venu_job_desc* jobs, uint32_t n, void* stream,
                                              uint32_t* job_ids) {
    if (!b || (n && !jobs)) {
        set_error("venu_batch_submit: NULL argument");
        return VENU_ERR_INVALID;
    }
    for (uint32_t k = 0; k < n; ++k) {
        const venu_status v = check_job(jobs + k, k);
        if (v != VENU_OK) return v;
    }
    std::vector<uint32_t> slots;
    for (uint32_t i = 0; i < b->max_jobs && slots.size() < n; ++i)
        if (!b->jobs[i].active) slots.push_back(i);
    if (slots.size() < n) {
        set_error("venu_batch_submit: max_jobs jobs are already admitted");
        return VENU_ERR_TOO_LARGE;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    SeedGroup g;
    std::memset(&g, 0, sizeof(g));
    for (uint32_t k = 0; k < n; ++k) {
        const venu_job_desc* job = jobs + k;
        const venu_render_opts& o = job->opts;
        const uint64_t npix = (uint64_t)o.width * o.height, total = npix * o.samples_per_pixel;
        const uint32_t slot = slots[k];
        JobHost& J = b->jobs[slot];
        J = JobHost{};
        // one allocation: the sample slots, then the seed table
        void* buf = nullptr;
        cudaError_t e = cudaMallocAsync(&buf, (sizeof(float4) + sizeof(uint32_t)) * total, st);
        // a group holds kSeedGroup jobs and at most 2^31 pixels (one job has at most 2^30)
        if (e == cudaSuccess && (g.n == kSeedGroup || (uint64_t)g.pix_off[g.n] + npix > (1ull << 31)))
            e = launch_seed_group(b, g, st);
        if (e != cudaSuccess) {
            // nothing of this call is admitted: free what it allocated
            if (buf) cudaFreeAsync(buf, st);
            for (uint32_t m = 0; m < k; ++m) {
                JobHost& P = b->jobs[slots[m]];
                cudaFreeAsync(P.slots, st);
                P = JobHost{};
            }
            b->jobs[slot] = JobHost{};
            return cuda_fail(e, "venu_batch_submit: job buffers");
        }
        J.slots = static_cast<float4*>(buf);
        J.seeds = reinterpret_cast<uint32_t*>(J.slots + total);
        J.active = true;
        J.desc = *job;
        J.total = total;
        J.remaining = total;
        J.bytes = venu_batch_job_bytes(o.width, o.height, o.samples_per_pixel);
        DevJob& dj = g.job[g.n];
        dj.scene = view_of(job->scene);
        dj.cam = job->camera;
        dj.W = o.width;
        dj.H = o.height;
        dj.npix = (uint32_t)npix;
        dj.div_npix = make_fastdiv((uint32_t)npix);
        dj.div_W = make_fastdiv(o.width);
        dj.spp = o.samples_per_pixel;
        dj.max_depth = o.max_depth;
        dj.subframe = o.subframe_index;
        dj.seeds = J.seeds;
        dj.slots = J.slots;
        dj.total = total;
        g.slot[g.n] = slot;
        g.pix_off[g.n + 1] = g.pix_off[g.n] + (uint32_t)npix;
        ++g.n;
    }
    const cudaError_t le = launch_seed_group(b, g, st);
    if (le != cudaSuccess) return cuda_fail(le, "venu_batch_submit: seed tables");
    for (uint32_t k = 0; k < n; ++k) {
        JobHost& J = b->jobs[slots[k]];
        J.seq = b->next_seq++;
        b->order.push_back(slots[k]);
        b->resident += J.bytes;
        if (job_ids) job_ids[k] = slots[k];
    }
    if (n) b->order_dirty = true;  // uploaded by the next run
    return VENU_OK;
}

extern "C" venu_status venu_batch_submit(venu_batch* b, const venu_job_desc* job, void* stream, uint32_t* job_id) {
    if (!job) {
        set_error("venu_batch_submit: NULL argument");
        return VENU_ERR_INVALID;
    }
    return venu_batch_submit_many(b, job, 1, stream, job_id);
}

extern "C" venu_status venu_batch_run(venu_batch* b, uint32_t max_iterations, uint32_t flags, void* stream) {
    if (!b) {
        set_error("venu_batch_run: NULL batch");
        return VENU_ERR_INVALID;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (b->order_dirty) {
        venu_status us = upload_order(b, st);
        if (us != VENU_OK) return us;
        b->order_dirty = false;
    }
    RunCtl rc;
    rc.max_iter = max_iterations;
    rc.nactive = (uint32_t)b->order.size();
    rc.stop_on_finish = (flags & VENU_RUN_STOP_ON_FINISH) ? 1u : 0u;
    rc.sequential = b->policy == VENU_POLICY_SEQUENTIAL ? 1u : 0u;
    rc.chunk = b->chunk;
    rc.pad[0] = rc.pad[1] = rc.pad[2] = 0u;
    VENU_CUDA(cudaMemcpyAsync(b->d_run, &rc, sizeof(rc), cudaMemcpyHostToDevice, st));
    VENU_CUDA(cudaMemsetAsync(&b->d_ctl->iter, 0, sizeof(uint32_t), st));
    VENU_CUDA(cudaMemsetAsync(&b->d_ctl->job_finished, 0, sizeof(uint32_t), st));
    if (b->flags & VENU_BATCH_NO_GRAPH) {
        // host-driven loop: one body, then read the device's running flag
        for (;;) {
            cudaError_t e = launch_body(b, st, false);
            if (e != cudaSuccess) return cuda_fail(e, "venu_batch_run");
            uint32_t running = 0;
            VENU_CUDA(cudaMemcpyAsync(&running, &b->d_ctl->running, sizeof(running), cudaMemcpyDeviceToHost, st));
            VENU_CUDA(cudaStreamSynchronize(st));
            if (!running || __atomic_load_n(b->h_interrupt, __ATOMIC_ACQUIRE)) break;
        }
        return VENU_OK;
    }
    if (!b->exec) {
        venu_status gs = build_graph(b);
        if (gs != VENU_OK) return gs;
    }
    VENU_CUDA(cudaGraphLaunch(b->exec, st));
    ++b->graph_launches;
    return VENU_OK;
}

extern "C" venu_status venu_batch_collect(venu_batch* b, void* stream, uint32_t* finished_ids, uint32_t cap,
                                          uint32_t* count) {
    if (!b) {
        set_error("venu_batch_collect: NULL batch");
        return VENU_ERR_INVALID;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    VENU_CUDA(cudaStreamSynchronize(st));
    uint32_t err = 0;
    VENU_CUDA(cudaMemcpy(&err, &b->d_ctl->err, sizeof(err), cudaMemcpyDeviceToHost));
    std::vector<unsigned long long> done(b->max_jobs);
    VENU_CUDA(cudaMemcpy(done.data(), b->d_done, sizeof(unsigned long long) * b->max_jobs, cudaMemcpyDeviceToHost));
    std::vector<CollectEntry> ent;
    std::vector<uint32_t> fin;
    uint32_t pix_off = 0;
    // one k_collect per group of finished jobs with at most 2^31 pixels
    // (a job has at most 2^30), so the thread index stays 32-bit
    auto flush = [&]() -> cudaError_t {
        if (ent.empty()) return cudaSuccess;
        cudaError_t e = cudaMemcpyAsync(b->d_collect, ent.data(), sizeof(CollectEntry) * ent.size(),
                                        cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return e;
        k_collect<<<(pix_off + 255) / 256, 256, 0, st>>>(b->d_collect, (uint32_t)ent.size(), pix_off);
        ent.clear();
        pix_off = 0;
        return cudaGetLastError();
    };
    for (uint32_t slot : b->order) {
        JobHost& J = b->jobs[slot];
        J.remaining = J.total - std::min<uint64_t>(done[slot], J.total);
        if (done[slot] < J.total) continue;
        const venu_render_opts& o = J.desc.opts;
        if ((uint64_t)pix_off + (uint64_t)o.width * o.height > (1ull << 31)) VENU_CUDA(flush());
        CollectEntry c;
        c.accum = reinterpret_cast<float4*>(J.desc.accum);
        c.image_f = reinterpret_cast<float4*>(J.desc.image_f);
        c.image8 = reinterpret_cast<uchar4*>(J.desc.image8);
        c.slots = J.slots;
        c.npix = o.width * o.height;
        c.spp = o.samples_per_pixel;
        c.reset = (o.flags & VENU_FLAG_RESET_ACCUM) ? 1u : 0u;
        c.pix_off = pix_off;
        pix_off += c.npix;
        ent.push_back(c);
        fin.push_back(slot);
    }
    VENU_CUDA(flush());
    if (!fin.empty()) {
        for (uint32_t slot : fin) {
            JobHost& J = b->jobs[slot];
            VENU_CUDA(cudaFreeAsync(J.slots, st));  // seeds share the allocation
            b->resident -= J.bytes;
            J = JobHost{};
        }
        std::vector<uint32_t> keep;
        for (uint32_t slot : b->order)
            if (b->jobs[slot].active) keep.push_back(slot);
        b->order.swap(keep);
    }
    if (!fin.empty() || b->policy == VENU_POLICY_SHORTEST_FIRST) b->order_dirty = true;
    const uint32_t n = (uint32_t)fin.size();
    if (finished_ids)
        for (uint32_t i = 0; i < n && i < cap; ++i) finished_ids[i] = fin[i];
    if (count) *count = n;
    if (err) {
        set_error("venu_batch: traversal stack overflow");
        return VENU_ERR_STACK;
    }
    return VENU_OK;
}

extern "C" venu_status venu_batch_set_policy(venu_batch* b, uint32_t policy) {
    if (!b || policy > VENU_POLICY_SEQUENTIAL) {
        set_error("venu_batch_set_policy: NULL batch or unknown policy");
        return VENU_ERR_INVALID;
    }
    b->policy = policy;
    b->order_dirty = true;  // re-sorted and uploaded by the next run
    return VENU_OK;
}

extern "C" venu_status venu_batch_set_chunk(venu_batch* b, uint32_t rays) {
    if (!b) {
        set_error("venu_batch_set_chunk: NULL batch");
        return VENU_ERR_INVALID;
    }
    b->chunk = rays;
    return VENU_OK;
}

extern "C" venu_status venu_batch_interrupt(venu_batch* b, uint32_t on) {
    if (!b) {
        set_error("venu_batch_interrupt: NULL batch");
        return VENU_ERR_INVALID;
    }
    __atomic_store_n(b->h_interrupt, on ? 1u : 0u, __ATOMIC_RELEASE);
    return VENU_OK;
}

extern "C" venu_status venu_batch_stats_get(venu_batch* b, venu_batch_stats* out) {
    if (!b || !out) {
        set_error("venu_batch_stats_get: NULL argument");
        return VENU_ERR_INVALID;
    }
    LoopCtl c;
    VENU_CUDA(cudaMemcpy(&c, b->d_ctl, sizeof(c), cudaMemcpyDeviceToHost));
    out->segments = c.segments;
    out->paths_done = c.paths_done;
    out->iterations = c.iterations;
    out->graph_launches = b->graph_launches;
    out->resident_bytes = b->resident;
    out->active_jobs = (uint32_t)b->order.size();
    out->reserved = 0;
    return VENU_OK;
}

extern "C" venu_status venu_batch_destroy(venu_batch* b) {
    if (!b) return VENU_OK;
    cudaDeviceSynchronize();
    free_batch(b);
    delete b;
    return VENU_OK;
}
