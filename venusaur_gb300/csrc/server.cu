// server.cu -- render server: continuous batching over venu_batch.
//
// One host thread per server.  Requests are queued first-come first-served
// and admitted while their device memory (scene BVH unless already resident,
// the job's seed table and sample slots, accumulator and image) fits the HBM
// budget; admitted jobs advance together in a shared path pool a few
// iterations per step; finished jobs are collected, their images copied to
// host memory and their buffers released.  Scene BVHs stay resident across
// requests with the same scene_key and are evicted least-recently-used when
// the budget needs room.
//
// Two lanes, each its own venu_batch: requests of at most express_paths
// paths (when set) go to a small express pool, the rest to the bulk pool.
// Each step runs the express lane first when it has work, then the bulk
// lane; a submit interrupts the running step at its next iteration, so a
// small request waits for at most one bulk iteration instead of sharing
// every bounce with the large jobs in the bulk pool.
#include "venu_internal.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

double seconds_since(Clock::time_point t0) {
    return std::chrono::duration<double>(Clock::now() - t0).count();
}

struct Request {
    uint64_t id = 0;
    venu_request req{};
    std::vector<venu_sphere> spheres;
    bool no_spheres = false;  // keyed request relying on a resident scene
    int32_t status = VENU_ERR_NOT_READY;
    bool done = false, cancelled = false;
    double t_submit = 0, t_admit = 0, t_done = 0;
    std::vector<uint8_t> image;
    // while admitted
    uint64_t scene_key = 0;
    int lane = 0;
    bool session_accum = false;  // accum belongs to a progressive session, not to the request
    float* accum = nullptr;
    uint8_t* image8 = nullptr;
    uint64_t job_bytes = 0;
};

// A progressive session (Renderer::Draw served over requests): its
// accumulator stays on the device between requests.
struct Session {
    float* accum = nullptr;
    uint32_t width = 0, height = 0;
    bool busy = false;         // a request of the session is admitted
    bool end_pending = false;  // ended while busy: freed when that request completes
    uint64_t bytes = 0;
};

struct SceneEntry {
    venu_scene* scene = nullptr;
    uint64_t bytes = 0;
    uint32_t refs = 0;
    uint64_t last_use = 0;
};

constexpr uint64_t kPrivateKey = 1ull << 63;  // scenes of requests without a key
constexpr uint32_t kExpressPool = 2u << 20;    // paths in flight in the express lane
constexpr uint32_t kBulkChunk = 4u << 20;      // bulk rays per step while the express lane is on

// Device bytes of a scene of n spheres, for admission before it is built:
// binary nodes 32 + traversal records 64 + spheres, materials 32 + meta,
// keys 8 + parent links 8 bytes per sphere, and the 4-wide tree (about one
// node of 128 + 16 bytes per two spheres).  Once built, the
// scene's own byte count replaces the estimate.
uint64_t scene_estimate(uint32_t n) { return (uint64_t)n * 240u + 4096u; }
uint64_t image_bytes(const venu_render_opts& o) {
    return (uint64_t)o.width * o.height * (sizeof(float) * VENU_ACCUM_FLOATS_PER_PIXEL + 4u);
}

}  // namespace

struct venu_server {
    uint64_t budget = 0;
    uint32_t pool = 0, max_jobs = 0, iters = 0;
    int device = 0;
    Clock::time_point t0 = Clock::now();

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    std::deque<uint64_t> pending;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    uint64_t next_id = 1;
    uint32_t inject = 0;
    uint64_t submitted = 0, completed = 0, failed = 0, segments = 0;
    std::vector<double> lat_ms;
    double busy = 0;
    uint32_t n_active = 0;
    uint64_t resident_shared = 0;
    venu_status fatal = VENU_OK;
    std::string fatal_msg;
    std::atomic<uint32_t> policy{VENU_POLICY_FIFO};  // plan order, applied by the server thread
    uint32_t applied_policy = VENU_POLICY_FIFO;
    uint64_t applied_express = 0;

    std::atomic<uint64_t> express_paths{0};  // 0: one lane
    // owned by the server thread
    std::thread th;
    venu_batch* batch = nullptr;    // bulk lane
    venu_batch* express = nullptr;  // express lane
    cudaStream_t st = nullptr;
    std::unordered_map<uint64_t, SceneEntry> scenes;
    std::unordered_map<uint32_t, uint64_t> active[2];  // per lane: batch job id -> request id
    std::unordered_map<uint64_t, Session> sessions;
    std::vector<uint64_t> sessions_to_end;  // guarded by mu; ended by the server thread
    uint64_t resident = 0, use_clock = 0;
    // guarded by mu
    uint64_t evictions = 0;        // scenes evicted to make room
    uint64_t admission_waits = 0;  // steps at which the queue head waited for room
    uint64_t peak_resident = 0;    // most device bytes held at once
    size_t n_active_all() const { return active[0].size() + active[1].size(); }
    venu_batch* lane(int l) const { return l ? express : batch; }
};

namespace {

void complete(venu_server* s, Request& R, int32_t status) {
    std::lock_guard<std::mutex> lock(s->mu);
    R.status = status;
    R.t_done = seconds_since(s->t0);
    R.done = true;
    ++s->completed;
    if (status == VENU_OK)
        s->lat_ms.push_back(1000.0 * (R.t_done - R.t_submit));
    else
        ++s->failed;
    s->cv_done.notify_all();
}

void release_scene(venu_server* s, uint64_t key) {
    auto it = s->scenes.find(key);
    if (it == s->scenes.end()) return;
    if (it->second.refs) --it->second.refs;
    if (it->second.refs == 0 && (key & kPrivateKey)) {  // a request's own scene is not kept
        venu_scene_destroy(it->second.scene);
        s->resident -= it->second.bytes;
        s->scenes.erase(it);
    }
}

// Least recently used unreferenced scenes go until `need` more bytes fit.
void evict_for(venu_server* s, uint64_t need) {
    while (s->resident + need > s->budget) {
        uint64_t victim = 0;
        uint64_t best = UINT64_MAX;
        for (auto& kv : s->scenes)
            if (kv.second.refs == 0 && kv.second.last_use < best) {
                best = kv.second.last_use;
                victim = kv.first;
            }
        if (best == UINT64_MAX) return;
        venu_scene_destroy(s->scenes[victim].scene);
        s->resident -= s->scenes[victim].bytes;
        s->scenes.erase(victim);
        std::lock_guard<std::mutex> lock(s->mu);
        ++s->evictions;
    }
}

// The request's accumulator: freed if it is the request's own; a session's
// stays (and the session is free for its next request).
void release_accum(venu_server* s, Request& R) {
    if (R.session_accum) {
        auto it = s->sessions.find(R.req.session);
        if (it != s->sessions.end()) {
            it->second.busy = false;
            if (it->second.end_pending) {
                if (it->second.accum) cudaFreeAsync(it->second.accum, s->st);
                s->resident -= it->second.bytes;
                s->sessions.erase(it);
            }
        }
    } else if (R.accum) {
        cudaFreeAsync(R.accum, s->st);
    }
    R.accum = nullptr;
}

// Admits one request; on failure it is completed with its status.
void admit(venu_server* s, Request& R) {
    const venu_render_opts& o = R.req.opts;
    uint32_t inj;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        inj = s->inject;
        s->inject &= ~(VENU_INJECT_ALLOC);
        if (!(inj & VENU_INJECT_ALLOC)) s->inject &= ~(VENU_INJECT_SCENE);
    }
    if (inj & VENU_INJECT_ALLOC) {
        complete(s, R, VENU_ERR_OOM);
        return;
    }
    const uint64_t key = R.req.scene_key ? R.req.scene_key : (kPrivateKey | R.id);
    auto it = s->scenes.find(key);
    if (it == s->scenes.end()) {
        if (R.no_spheres) {  // its scene was never sent or has been evicted
            complete(s, R, VENU_ERR_INVALID);
            return;
        }
        if (inj & VENU_INJECT_SCENE) {
            complete(s, R, VENU_ERR_CUDA);
            return;
        }
        venu_scene* sc = nullptr;
        venu_status st = venu_scene_create(R.spheres.data(), (uint32_t)R.spheres.size(), s->st, &sc);
        if (st != VENU_OK) {
            complete(s, R, st);
            return;
        }
        venu_scene_info info{};
        venu_scene_info_get(sc, &info);
        SceneEntry e;
        e.scene = sc;
        e.bytes = info.device_bytes;
        s->resident += e.bytes;
        it = s->scenes.emplace(key, e).first;
        R.spheres.clear();
        R.spheres.shrink_to_fit();
    }
    it->second.refs += 1;
    it->second.last_use = ++s->use_clock;
    const uint64_t npix = (uint64_t)o.width * o.height;
    const uint64_t accum_bytes = npix * sizeof(float) * VENU_ACCUM_FLOATS_PER_PIXEL;
    bool reset = true;
    cudaError_t e = cudaSuccess;
    if (R.req.session) {
        // continue the session's accumulator unless it is new, resized or reset
        Session& S = s->sessions[R.req.session];
        reset = !S.accum || S.width != o.width || S.height != o.height || (o.flags & VENU_FLAG_RESET_ACCUM);
        if (S.accum && (S.width != o.width || S.height != o.height)) {
            cudaFreeAsync(S.accum, s->st);
            s->resident -= S.bytes;
            S.accum = nullptr;
        }
        if (!S.accum) {
            e = cudaMallocAsync(&S.accum, accum_bytes, s->st);
            if (e == cudaSuccess) {
                S.width = o.width;
                S.height = o.height;
                S.bytes = accum_bytes;
                s->resident += accum_bytes;
            } else {
                S.accum = nullptr;
            }
        }
        R.accum = S.accum;
        R.session_accum = true;
        S.busy = e == cudaSuccess;
    } else {
        e = cudaMallocAsync(&R.accum, accum_bytes, s->st);
    }
    if (e == cudaSuccess) e = cudaMallocAsync(&R.image8, npix * 4u, s->st);
    if (e != cudaSuccess) {
        release_accum(s, R);
        release_scene(s, key);
        complete(s, R, VENU_ERR_OOM);
        return;
    }
    const uint64_t paths = (uint64_t)o.width * o.height * o.samples_per_pixel;
    const uint64_t xp = s->express_paths.load();
    R.lane = (xp && paths <= xp) ? 1 : 0;
    venu_job_desc d{};
    d.scene = it->second.scene;
    d.camera = R.req.camera;
    d.opts = o;
    if (reset) d.opts.flags |= VENU_FLAG_RESET_ACCUM;
    else d.opts.flags &= ~VENU_FLAG_RESET_ACCUM;
    d.accum = R.accum;
    d.image8 = R.image8;
    uint32_t jid = 0;
    venu_status bs = venu_batch_submit(s->lane(R.lane), &d, s->st, &jid);
    if (bs != VENU_OK) {
        release_accum(s, R);
        cudaFreeAsync(R.image8, s->st);
        R.image8 = nullptr;
        release_scene(s, key);
        complete(s, R, bs);
        return;
    }
    R.scene_key = key;
    R.job_bytes = venu_batch_job_bytes(o.width, o.height, o.samples_per_pixel) + image_bytes(o) -
                  (R.session_accum ? accum_bytes : 0u);  // a session's accumulator is counted with the session
    s->resident += R.job_bytes;
    s->active[R.lane][jid] = R.id;
    std::lock_guard<std::mutex> lock(s->mu);
    R.t_admit = seconds_since(s->t0);
}

void free_session(venu_server* s, std::unordered_map<uint64_t, Session>::iterator it) {
    if (it->second.accum) cudaFreeAsync(it->second.accum, s->st);
    s->resident -= it->second.bytes;
    s->sessions.erase(it);
}

// Frees a session's accumulator, now or -- while one of its requests is
// admitted -- when that request completes.
void end_session(venu_server* s, uint64_t id) {
    auto it = s->sessions.find(id);
    if (it == s->sessions.end()) return;
    if (it->second.busy) it->second.end_pending = true;
    else free_session(s, it);
}

void fail_all_active(venu_server* s, venu_status st) {
    for (auto& act : s->active) {
        for (auto& kv : act) {
            Request* R;
            {
                std::lock_guard<std::mutex> lock(s->mu);
                R = s->reqs[kv.second].get();
            }
            complete(s, *R, st);
        }
        act.clear();
    }
}

// One step of one lane: run (ends when a job finishes, after max_iter
// iterations, or at an interrupt), collect, hand finished images back.
venu_status run_lane(venu_server* s, int l, uint32_t max_iter, std::vector<uint32_t>& fin) {
    venu_batch* b = s->lane(l);
    venu_status rs = venu_batch_run(b, max_iter, VENU_RUN_STOP_ON_FINISH, s->st);
    uint32_t nfin = 0;
    if (rs == VENU_OK) rs = venu_batch_collect(b, s->st, fin.data(), (uint32_t)fin.size(), &nfin);
    if (rs != VENU_OK) return rs;
    std::vector<Request*> done;
    nfin = std::min<uint32_t>(nfin, (uint32_t)fin.size());  // fin holds max_jobs ids, the most a collect returns
    for (uint32_t i = 0; i < nfin; ++i) {
        auto it = s->active[l].find(fin[i]);
        if (it == s->active[l].end()) continue;
        Request* R;
        {
            std::lock_guard<std::mutex> lock(s->mu);
            R = s->reqs[it->second].get();
        }
        s->active[l].erase(it);
        const uint64_t npix = (uint64_t)R->req.opts.width * R->req.opts.height;
        R->image.resize(npix * 4u);
        cudaMemcpyAsync(R->image.data(), R->image8, npix * 4u, cudaMemcpyDeviceToHost, s->st);
        done.push_back(R);
    }
    cudaError_t ce = cudaStreamSynchronize(s->st);
    for (Request* R : done) {
        release_accum(s, *R);
        cudaFreeAsync(R->image8, s->st);
        R->image8 = nullptr;
        s->resident -= R->job_bytes;
        release_scene(s, R->scene_key);
        complete(s, *R, ce == cudaSuccess ? VENU_OK : VENU_ERR_CUDA);
    }
    return VENU_OK;
}

void server_loop(venu_server* s) {
    cudaSetDevice(s->device);
    std::vector<uint32_t> fin(s->max_jobs);
    for (;;) {
        // Clear the interrupt before looking at the queue: a request queued
        // after this point sets it again and ends the next run early.
        venu_batch_interrupt(s->batch, 0u);
        venu_batch_interrupt(s->express, 0u);
        {
            const uint32_t pol = s->policy.load();
            if (pol != s->applied_policy) {
                venu_batch_set_policy(s->batch, pol);  // the express lane stays FIFO
                s->applied_policy = pol;
            }
            // with the express lane on, the bulk pool yields every kBulkChunk
            // rays, so small requests wait at most one chunk, not one whole
            // bulk iteration
            const uint64_t xp = s->express_paths.load();
            if ((xp != 0) != (s->applied_express != 0)) venu_batch_set_chunk(s->batch, xp ? kBulkChunk : 0u);
            s->applied_express = xp;
        }
        // admission, first come first served
        for (;;) {
            Request* R = nullptr;
            bool skipped = false;
            std::vector<uint64_t> ending;
            {
                std::lock_guard<std::mutex> lock(s->mu);
                // session ends requested before this request was submitted
                // apply to it: take them in the same critical section
                ending.swap(s->sessions_to_end);
                if (!s->pending.empty()) {
                    R = s->reqs[s->pending.front()].get();
                    if (R->cancelled) {
                        s->pending.pop_front();
                        R = nullptr;
                        skipped = true;
                    }
                }
            }
            for (uint64_t id : ending) end_session(s, id);
            if (skipped) continue;
            if (!R) break;
            if (R->cancelled) continue;
            if (R->req.session) {  // one request of a session at a time, in order
                auto si = s->sessions.find(R->req.session);
                if (si != s->sessions.end() && si->second.busy) break;
            }
            const venu_render_opts& o = R->req.opts;
            const uint64_t key = R->req.scene_key ? R->req.scene_key : (kPrivateKey | R->id);
            const bool cached = s->scenes.count(key) != 0;
            const uint64_t need = venu_batch_job_bytes(o.width, o.height, o.samples_per_pixel) + image_bytes(o) +
                                  (cached ? 0u : scene_estimate((uint32_t)R->spheres.size()));
            if (need > s->budget) {
                {
                    std::lock_guard<std::mutex> lock(s->mu);
                    s->pending.pop_front();
                }
                complete(s, *R, VENU_ERR_OOM);
                continue;
            }
            if (s->resident + need > s->budget) evict_for(s, need);
            if (s->resident + need > s->budget || s->n_active_all() >= s->max_jobs) {  // wait for room
                std::lock_guard<std::mutex> lock(s->mu);
                ++s->admission_waits;
                break;
            }
            {
                std::lock_guard<std::mutex> lock(s->mu);
                s->pending.pop_front();
            }
            admit(s, *R);
        }
        {
            std::lock_guard<std::mutex> lock(s->mu);
            s->n_active = (uint32_t)s->n_active_all();
            s->resident_shared = s->resident;
            s->peak_resident = std::max(s->peak_resident, s->resident);
        }
        if (s->n_active_all() == 0) {
            std::unique_lock<std::mutex> lock(s->mu);
            if (s->stop) break;
            if (s->pending.empty()) s->cv_work.wait_for(lock, std::chrono::milliseconds(20));
            if (s->stop) break;
            continue;
        }
        const Clock::time_point tb = Clock::now();
        // The express lane first.  The bulk lane gets one iteration per step
        // while express work remains (so small requests wait at most one bulk
        // iteration, and a stream of them cannot stall the bulk lane), and
        // up to `iters` when there is none.
        venu_status rs = VENU_OK;
        const bool express_work = !s->active[1].empty();
        if (express_work) rs = run_lane(s, 1, s->iters, fin);
        if (rs == VENU_OK && !s->active[0].empty()) rs = run_lane(s, 0, express_work ? 1u : s->iters, fin);
        if (rs != VENU_OK) {
            std::string msg = venu_last_error();
            fail_all_active(s, rs);
            std::lock_guard<std::mutex> lock(s->mu);
            s->fatal = rs;
            s->fatal_msg = msg;
            s->stop = true;
            break;
        }
        venu_batch_stats bst{}, bsx{};
        venu_batch_stats_get(s->batch, &bst);
        venu_batch_stats_get(s->express, &bsx);
        std::lock_guard<std::mutex> lock(s->mu);
        s->busy += seconds_since(tb);
        s->segments = bst.segments + bsx.segments;
        if (s->stop && s->n_active_all() == 0) break;
    }
    // shut down: fail what is left, drop the sessions
    fail_all_active(s, VENU_ERR_CANCELLED);
    for (auto& kv : s->sessions)
        if (kv.second.accum) cudaFreeAsync(kv.second.accum, s->st);
    s->sessions.clear();
    cudaStreamSynchronize(s->st);
    std::deque<uint64_t> left;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        left.swap(s->pending);
    }
    for (uint64_t id : left) {
        Request* R;
        {
            std::lock_guard<std::mutex> lock(s->mu);
            R = s->reqs[id].get();
        }
        complete(s, *R, VENU_ERR_CANCELLED);
    }
    cudaStreamSynchronize(s->st);
    for (auto& kv : s->scenes) venu_scene_destroy(kv.second.scene);
    s->scenes.clear();
}

}  // namespace

using namespace venu;

extern "C" venu_status venu_server_create(uint64_t hbm_budget_bytes, uint32_t pool_paths, uint32_t max_jobs,
                                          uint32_t iterations_per_step, venu_server** out) {
    if (!out || hbm_budget_bytes == 0 || max_jobs == 0) {
        set_error("venu_server_create: need out, a budget and max_jobs > 0");
        return VENU_ERR_INVALID;
    }
    *out = nullptr;
    venu_status ds = require_device();
    if (ds != VENU_OK) return ds;
    venu_server* s = new venu_server();
    s->budget = hbm_budget_bytes;
    s->pool = pool_paths;
    s->max_jobs = max_jobs;
    s->iters = iterations_per_step ? iterations_per_step : 8;
    cudaGetDevice(&s->device);
    venu_status bs = venu_batch_create(pool_paths, max_jobs, 0, &s->batch);
    if (bs != VENU_OK) {
        delete s;
        return bs;
    }
    bs = venu_batch_create(kExpressPool, max_jobs, 0, &s->express);
    if (bs != VENU_OK) {
        venu_batch_destroy(s->batch);
        delete s;
        return bs;
    }
    cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        venu_batch_destroy(s->express);
        venu_batch_destroy(s->batch);
        delete s;
        return cuda_fail(e, "venu_server_create");
    }
    s->th = std::thread(server_loop, s);
    *out = s;
    return VENU_OK;
}

extern "C" venu_status venu_server_submit(venu_server* s, const venu_request* req, uint64_t* request_id) {
    if (!s || !req) {
        set_error("venu_server_submit: NULL argument");
        return VENU_ERR_INVALID;
    }
    const venu_render_opts& o = req->opts;
    if (o.width < 2 || o.height < 2 || o.samples_per_pixel == 0 || o.max_depth == 0 || o.max_depth > 64 ||
        (req->num_spheres && !req->spheres) || req->num_spheres > (1u << 28)) {
        set_error("venu_server_submit: malformed request");
        return VENU_ERR_INVALID;
    }
    auto R = std::make_unique<Request>();
    R->req = *req;
    if (req->num_spheres) R->spheres.assign(req->spheres, req->spheres + req->num_spheres);
    R->no_spheres = (req->scene_key != 0 && req->spheres == nullptr);
    R->req.spheres = nullptr;
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) {
        set_error("venu_server_submit: server stopped: " + s->fatal_msg);
        return s->fatal != VENU_OK ? s->fatal : VENU_ERR_CANCELLED;
    }
    R->id = s->next_id++;
    R->t_submit = seconds_since(s->t0);
    const uint64_t id = R->id;
    s->reqs.emplace(id, std::move(R));
    s->pending.push_back(id);
    ++s->submitted;
    s->cv_work.notify_all();
    venu_batch_interrupt(s->batch, 1u);  // end the running step early: admit this request sooner
    venu_batch_interrupt(s->express, 1u);
    if (request_id) *request_id = id;
    return VENU_OK;
}

extern "C" venu_status venu_server_set_policy(venu_server* s, uint32_t policy) {
    if (!s || policy > VENU_POLICY_SEQUENTIAL) {
        set_error("venu_server_set_policy: NULL server or unknown policy");
        return VENU_ERR_INVALID;
    }
    s->policy.store(policy);
    venu_batch_interrupt(s->batch, 1u);  // applied at the start of the next step
    return VENU_OK;
}

extern "C" venu_status venu_server_end_session(venu_server* s, uint64_t session) {
    if (!s || session == 0) {
        set_error("venu_server_end_session: NULL server or session 0");
        return VENU_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    s->sessions_to_end.push_back(session);
    s->cv_work.notify_all();
    return VENU_OK;
}

extern "C" venu_status venu_server_set_express(venu_server* s, uint64_t max_paths) {
    if (!s) {
        set_error("venu_server_set_express: NULL server");
        return VENU_ERR_INVALID;
    }
    s->express_paths.store(max_paths);  // requests admitted from now on
    return VENU_OK;
}

extern "C" venu_status venu_server_wait(venu_server* s, uint64_t request_id, double timeout_s, venu_result* out) {
    if (!s || !out) {
        set_error("venu_server_wait: NULL argument");
        return VENU_ERR_INVALID;
    }
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->reqs.find(request_id);
    if (it == s->reqs.end()) {
        set_error("venu_server_wait: unknown request");
        return VENU_ERR_INVALID;
    }
    Request* R = it->second.get();
    // NaN or <= 0: one look; above 1e9 s (infinity included): 1e9 s, whose
    // count of nanoseconds still fits the clock's 64-bit duration
    const double tw = timeout_s > 0.0 ? (timeout_s < 1e9 ? timeout_s : 1e9) : 0.0;
    const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(tw));
    while (!R->done)
        if (s->cv_done.wait_until(lock, deadline) == std::cv_status::timeout && !R->done) {
            set_error("venu_server_wait: timed out");
            return VENU_ERR_NOT_READY;
        }
    out->request_id = R->id;
    out->tag = R->req.tag;
    out->status = R->status;
    out->width = R->req.opts.width;
    out->height = R->req.opts.height;
    out->reserved = 0;
    out->image8 = R->image.empty() ? nullptr : R->image.data();
    out->t_submit = R->t_submit;
    out->t_admit = R->t_admit;
    out->t_done = R->t_done;
    return VENU_OK;
}

extern "C" venu_status venu_server_cancel(venu_server* s, uint64_t request_id) {
    if (!s) return VENU_ERR_INVALID;
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->reqs.find(request_id);
    if (it == s->reqs.end()) {
        set_error("venu_server_cancel: unknown request");
        return VENU_ERR_INVALID;
    }
    Request* R = it->second.get();
    auto p = std::find(s->pending.begin(), s->pending.end(), request_id);
    if (p == s->pending.end()) {
        set_error("venu_server_cancel: request already admitted or done");
        return VENU_ERR_NOT_READY;
    }
    s->pending.erase(p);
    R->cancelled = true;
    R->status = VENU_ERR_CANCELLED;
    R->t_done = seconds_since(s->t0);
    R->done = true;
    ++s->completed;
    ++s->failed;
    s->cv_done.notify_all();
    return VENU_OK;
}

extern "C" venu_status venu_server_release(venu_server* s, uint64_t request_id) {
    if (!s) return VENU_ERR_INVALID;
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->reqs.find(request_id);
    if (it == s->reqs.end() || !it->second->done) {
        set_error("venu_server_release: unknown or unfinished request");
        return VENU_ERR_INVALID;
    }
    s->reqs.erase(it);
    return VENU_OK;
}

extern "C" venu_status venu_server_inject(venu_server* s, uint32_t what) {
    if (!s) return VENU_ERR_INVALID;
    std::lock_guard<std::mutex> lock(s->mu);
    s->inject |= what;
    return VENU_OK;
}

extern "C" venu_status venu_server_stats_get(venu_server* s, venu_server_stats* out) {
    if (!s || !out) return VENU_ERR_INVALID;
    std::lock_guard<std::mutex> lock(s->mu);
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->failed = s->failed;
    out->resident_bytes = s->resident_shared;
    out->budget_bytes = s->budget;
    out->segments = s->segments;
    out->active = s->n_active;
    out->pending = (uint32_t)s->pending.size();
    std::vector<double> l = s->lat_ms;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) {
        if (l.empty()) return 0.0;
        const size_t i = (size_t)std::min<double>((double)l.size() - 1, std::ceil(q * l.size()) - 1);
        return l[i];
    };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    out->busy_seconds = s->busy;
    out->evictions = s->evictions;
    out->admission_waits = s->admission_waits;
    out->peak_resident_bytes = s->peak_resident;
    return VENU_OK;
}

extern "C" venu_status venu_server_destroy(venu_server* s) {
    if (!s) return VENU_OK;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->th.joinable()) s->th.join();
    venu_batch_destroy(s->batch);
    venu_batch_destroy(s->express);
    if (s->st) cudaStreamDestroy(s->st);
    delete s;
    return VENU_OK;
}
