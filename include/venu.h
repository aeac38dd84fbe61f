/*
 * venu.h -- C ABI of the Venusaur-GB300 path tracer (libvenusaur_gb300.so).
 *
 * A drop-in for the reference's OptiX hot path: the LBVH replaces
 * Renderer::BuildAccelerationStructures, venu_render replaces the
 * Renderer::Draw -> optixLaunch -> __raygen__rg/__intersection__/
 * __closesthit__/__miss__ chain.  Citations are relative to the reference
 * project root (TienYoung/Venusaur).
 *
 * Conventions:
 *  - plain C types only; every call returns a venu_status (no exceptions
 *    cross the ABI); venu_last_error() gives the message of the last failure
 *    on the calling thread;
 *  - device pointers are CUDA device addresses on the current device;
 *    `stream` is a cudaStream_t passed as void* (NULL = legacy stream);
 *  - handles are thread-compatible, not thread-safe: one thread per handle
 *    at a time;
 *  - the library has no CPU fallback: without a usable sm_103 device every
 *    GPU entry point returns VENU_ERR_NO_DEVICE.
 */
#ifndef VENU_H
#define VENU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define VENU_API __attribute__((visibility("default")))
#else
#define VENU_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum venu_status {
    VENU_OK = 0,
    VENU_ERR_INVALID = 1,    /* bad argument */
    VENU_ERR_CUDA = 2,       /* CUDA runtime error */
    VENU_ERR_OOM = 3,        /* device allocation failed or over budget */
    VENU_ERR_NO_DEVICE = 4,  /* no CUDA device / not sm_103 */
    VENU_ERR_STACK = 5,      /* traversal stack overflow (reported, never expected) */
    VENU_ERR_TIMEOUT = 6,    /* a bounded device wait gave up */
    VENU_ERR_CANCELLED = 7,  /* job cancelled (server) */
    VENU_ERR_TOO_LARGE = 8,  /* size beyond a stated limit */
    VENU_ERR_NOT_READY = 9   /* result not available yet (server poll) */
} venu_status;

/* Material::Type (Core/material.h:8-13). */
typedef enum venu_material_type {
    VENU_LAMBERTIAN = 0,
    VENU_METAL = 1,
    VENU_DIELECTRIC = 2
} venu_material_type;

/* Sphere(center, radius, Material(type, albedo, fuzz, ir))
 * (Core/sphere.h:8-13, Core/material.h:16-19); 48 bytes. */
typedef struct venu_sphere {
    float center[3];
    float radius;
    float albedo[3];
    float fuzz;
    float ir;
    uint32_t material; /* venu_material_type */
    uint32_t pad[2];
} venu_sphere;

/* Camera fields of Params (Core/RayTracer.h:10-14): origin, the U/V/W frame
 * of Camera::UVWFrame (Core/Camera.cpp:16-37) and the lens radius
 * (Core/camera.h:20). */
typedef struct venu_camera {
    float origin[3];
    float u[3];
    float v[3];
    float w[3];
    float lens_radius;
} venu_camera;

/* Per-call render parameters (Params width/height/samples_per_pixel/
 * subframe_index, Core/RayTracer.h:6-9; Core/RayTracer.cu:172 max_depth). */
typedef struct venu_render_opts {
    uint32_t width;
    uint32_t height;
    uint32_t samples_per_pixel;
    uint32_t subframe_index; /* seeds tea<4>(pixel, subframe_index) */
    uint32_t max_depth;      /* ray casts per path, >= 1 (reference: 4) */
    uint32_t flags;          /* VENU_FLAG_* */
} venu_render_opts;

#define VENU_FLAG_RESET_ACCUM 1u /* zero the accumulator first (camera change) */

/* Accumulator layout: 8 floats per pixel {sum.r, sum.g, sum.b, n,
 * comp.r, comp.g, comp.b, 0} -- a Kahan-compensated running sum of path
 * radiance over every sample since the last reset. */
#define VENU_ACCUM_FLOATS_PER_PIXEL 8

typedef struct venu_scene venu_scene;
typedef struct venu_renderer venu_renderer;

typedef struct venu_scene_info {
    uint32_t num_spheres;
    uint32_t num_nodes;      /* internal LBVH nodes (num_spheres - 1) */
    uint64_t device_bytes;   /* resident bytes owned by the scene */
    float bounds[6];         /* centroid bounds used for Morton quantisation */
    float build_ms;          /* device time of the last LBVH build */
    uint32_t num_wide_nodes; /* nodes of the 4-wide traversal tree collapsed from the LBVH: built
                                by the first venu_render with traversal variant 4 or 5 (0 until
                                then; device_bytes grows by its size) */
    float wide_ms;           /* wall time of that collapse (host-driven, level by level) */
} venu_scene_info;

typedef struct venu_render_stats {
    uint64_t segments;       /* ray casts of the last render (primary + bounces) */
    uint64_t paths;          /* paths of the last render (W*H*spp) */
    uint32_t waves;          /* waves of the last render */
    uint32_t kernel_launches;/* kernels launched by the last render */
    uint64_t nodes_visited;  /* counting renders only (VENU_RENDERER_COUNT) */
    uint64_t spheres_tested; /* counting renders only */
    float traverse_ms;       /* profiling renders only (VENU_RENDERER_PROFILE): */
    float shade_ms;          /*   summed CUDA-event times of each kernel's launches */
    uint32_t traverse_launches;
    uint32_t shade_launches;
    uint64_t lane_steps;     /* counting renders only: traversal steps summed over lanes, */
    uint64_t warp_steps;     /*   and over warps (one per step the warp issues); */
                             /*   lane_steps / (32 warp_steps) = SIMD utilisation of traversal */
} venu_render_stats;

/* ---- errors / device -------------------------------------------------- */
VENU_API const char* venu_last_error(void);
/* Checks that the current device is usable (sm_103, kernels load). */
VENU_API venu_status venu_device_check(int* sm_count_out, int* cc_major_out, int* cc_minor_out);

/* ---- host-side scene and camera helpers ------------------------------ */
/* The RTIOW final scene (Core/Scene.h:13-80) from a seeded generator with a
 * fixed draw order; returns the sphere count (<= 488) and writes up to cap. */
VENU_API uint32_t venu_scene_generate_rtiow(uint32_t seed, venu_sphere* out, uint32_t cap);
/* Ground sphere plus n-1 random spheres: centers uniform in [box_lo, box_hi],
 * radii log-uniform in [rmin, rmax], materials 80/15/5 as Core/Scene.h:28-64. */
VENU_API venu_status venu_scene_generate_random(uint32_t n, uint32_t seed, const float box_lo[3],
                                       const float box_hi[3], float rmin, float rmax,
                                       venu_sphere* out);
/* Camera(origin, vfov, aspect, aperture, focal) + SetForward(lookat - origin)
 * + UVWFrame (Core/camera.h:14, Core/Camera.cpp:24-37, Core/Core.cpp:355). */
VENU_API void venu_camera_look_at(const float eye[3], const float lookat[3], float vfov_deg, float aspect,
                         float aperture, float focal, venu_camera* out);
/* Camera::UpdateUVW (Core/Camera.cpp:27-37) for a unit forward vector. */
VENU_API void venu_camera_frame(const float eye[3], const float forward[3], float vfov_deg, float aspect,
                       float aperture, float focal, venu_camera* out);
/* Camera::Pitch / Yaw / Roll (Core/camera.h:56-78): the unit forward vector
 * rotated by `degrees` about `axis` (the camera's u, v or w) with GLM's
 * quaternion semantics (forward * rotate(identity, radians(degrees), axis)),
 * then normalised.  Host only; out may alias forward. */
VENU_API void venu_camera_rotate(const float forward[3], const float axis[3], float degrees, float out[3]);

/* ---- image files: the headless stand-in for the GL display
 *      (Core/CUDAOutputBuffer.h:284-339, Core/Core.cpp:396-426).  Host
 *      buffers in the renderer's pixel order (row 0 = bottom). ------------- */
/* Binary PPM (P6), top row first, alpha dropped. */
VENU_API venu_status venu_image_write_ppm(const char* path, const uint8_t* rgba8, uint32_t width, uint32_t height);
/* PFM (RGB float32, little-endian, bottom row first), alpha dropped. */
VENU_API venu_status venu_image_write_pfm(const char* path, const float* rgba32f, uint32_t width, uint32_t height);

/* ---- scene: LBVH build (replaces Renderer::BuildAccelerationStructures,
 *      Core/Renderer.h:160-255, and CreateSBT's per-sphere records,
 *      Core/Renderer.h:452-520) ------------------------------------------ */
/* Uploads `n` spheres from host memory and builds the LBVH on the device
 * (Morton30, radix sort, Karras hierarchy, refit).  Blocks until built. */
VENU_API venu_status venu_scene_create(const venu_sphere* spheres_host, uint32_t n, void* stream,
                              venu_scene** out);
/* Same, from spheres already in device memory. */
VENU_API venu_status venu_scene_create_device(const venu_sphere* spheres_dev, uint32_t n, void* stream,
                                     venu_scene** out);
/* Moving spheres (no counterpart in the reference, which builds once in
 * Renderer::Init, Core/Renderer.h:25-33): the scene's spheres replaced by `n` new ones (the same count and original order as at
 * creation; centres, radii and materials may change) and the LBVH refit --
 * same topology and slot order, boxes recomputed bottom-up -- instead of
 * rebuilt.  Renders afterwards equal renders of a fresh build of the new
 * spheres (the closest hit does not depend on the tree; ties between equal
 * distances aside).  Quality degrades as spheres move far from where the
 * tree was built: rebuild with venu_scene_create then.  The host variant
 * uploads and returns when done; the device variant is asynchronous on
 * `stream` and `spheres_dev` must stay valid until it completes. */
VENU_API venu_status venu_scene_update(venu_scene* scene, const venu_sphere* spheres_host, uint32_t n, void* stream);
VENU_API venu_status venu_scene_update_device(venu_scene* scene, const venu_sphere* spheres_dev, uint32_t n,
                                              void* stream);
VENU_API venu_status venu_scene_info_get(const venu_scene* scene, venu_scene_info* out);
/* Copies the built LBVH to host buffers (any may be NULL): sorted Morton
 * codes [n], sorted original ids [n], internal nodes [(n-1) x 32 bytes:
 * lo[3], left, hi[3], right; child >= 0 internal, 0x80000000 | slot leaf,
 * and 0x40000000 also set on the leaf of a hoisted sphere -- one of at most
 * four huge spheres (radius above a quarter of the largest centroid extent)
 * that every ray tests before the traversal]. */
VENU_API venu_status venu_scene_export_bvh(const venu_scene* scene, uint32_t* morton, uint32_t* ids,
                                  void* nodes);
VENU_API venu_status venu_scene_destroy(venu_scene* scene);

/* ---- LBVH build that allocates nothing --------------------------------
 * No counterpart in the reference (OptiX sizes and allocates its own build
 * buffers).  For callers that must not allocate device memory: an engine or
 * server that hands every byte of HBM out from its own pool or budget and
 * cannot let a library call cudaMalloc behind it, or a per-frame rebuild of
 * moving spheres that cannot afford the device-wide synchronisation that
 * cudaMalloc/cudaFree may cause.  It runs the same kernels as
 * venu_scene_create into buffers the caller owns, asynchronously on
 * `stream`, and calls no cudaMalloc, cudaFree or other allocating routine.
 *
 * Scratch lives in one fixed device array inside the library (about 3.8 MB
 * for VENU_NOALLOC_MAX_SPHERES spheres), which every GPU that loads the
 * library holds until the process exits.  n above VENU_NOALLOC_MAX_SPHERES
 * returns VENU_ERR_TOO_LARGE.  The first call on a device looks up that
 * array's device address (once per device, with the device current); make
 * that first call before any stream capture.  All calls share the array and
 * it keeps the last call's contents: calls whose work overlaps on the GPU
 * (other streams, other host threads) race and must be serialised.
 *
 * The device address of that array is looked up once per device ordinal and
 * kept for the life of the process; it belongs to the CUDA context current at
 * that first call, so this entry point must not be used after that device's
 * context is destroyed (cudaDeviceReset) in the same process.
 *
 * Outputs (device, 16-byte aligned where float4):
 *   nodes_out      (n-1) x 8 floats: {lo.xyz, left} {hi.xyz, right} (n > 1;
 *                  may be NULL for n = 1).  Child words as
 *                  venu_scene_export_bvh writes them: >= 0 an internal node,
 *                  0x80000000 | slot a leaf, and 0x40000000 also set on the
 *                  leaf of a hoisted sphere (one of at most four huge spheres,
 *                  radius above a quarter of the largest centroid extent).  A
 *                  traversal of these nodes must test the hoisted spheres
 *                  before the walk and skip their leaves in it, as this
 *                  library's does; their slots are the leaf words that carry
 *                  0x40000000
 *   spheres_out    n x 4 floats {center, radius} in Morton slot order
 *   materials_out  n x 4 floats {albedo, fuzz or ir}
 *   meta_out       n uint32: original index | material << 30
 *   morton_out     n uint32: sorted Morton codes
 * They equal venu_scene_create's LBVH (venu_scene_export_bvh) bit for bit. */
#define VENU_NOALLOC_MAX_SPHERES 65536u
VENU_API venu_status venu_lbvh_build_noalloc(const venu_sphere* spheres_dev, uint32_t n, float* nodes_out,
                                             float* spheres_out, float* materials_out, uint32_t* meta_out,
                                             uint32_t* morton_out, void* stream);

/* ---- device self-tests ------------------------------------------------
 * The device arithmetic that results depend on bit for bit, exposed so a
 * caller can compare it word for word with a host restatement.  All pointers
 * are device memory; asynchronous on `stream`. */
/* tea_out[i] = tea<4>(a[i], b[i]) for i < n (Core/random.cuh:31-46); then
 * nsteps steps of the LCG from `seed` (Core/random.cuh:49-67): rnd_out[k] the
 * k-th draw, states_out[k] the state after it (either may be NULL). */
VENU_API venu_status venu_selftest_rng(const uint32_t* a_dev, const uint32_t* b_dev, uint32_t n,
                                       uint32_t* tea_out_dev, uint32_t seed, uint32_t nsteps,
                                       float* rnd_out_dev, uint32_t* states_out_dev, void* stream);
/* out[i] = x[i]^(1/2.4) for i < n: which = 0 the library's own power routine,
 * used by every sRGB encode (Core/RayTracer.cu:16-47 calls powf; this one
 * is built from IEEE operations only, so a host restatement matches it bit
 * for bit; x in [2^-126, 1]); which = 1 CUDA's powf(x, 1.0f/2.4f). */
VENU_API venu_status venu_selftest_srgb_pow(const float* x_dev, uint64_t n, uint32_t which, float* out_dev,
                                            void* stream);

/* ---- closest hit for arbitrary rays (optixTrace without programs) ----- */
/* rays_dev: n x 6 floats (origin, direction).  Writes, per ray, the hit
 * distance t (tmax on a miss), the original sphere index (-1 on a miss) and
 * front = 1 when the ray hits the outside (set_face_normal,
 * Core/RayTracer.cu:219-224). */
VENU_API venu_status venu_trace(const venu_scene* scene, const float* rays_dev, uint32_t n, float tmin,
                       float tmax, float* t_dev, int32_t* id_dev, uint32_t* front_dev,
                       void* stream);

/* ---- renderer: the plain single-scene wavefront method ---------------- */
#define VENU_RENDERER_COUNT 1u   /* count nodes visited / spheres tested */
#define VENU_RENDERER_PROFILE 2u /* CUDA events around every traverse / shade launch */

/* max_paths: paths in flight per wave (0 = default 64 Mi; about 120 B of
 * queues and slots per path, 8 GB at 64 Mi; at most 2^30).  The queues are
 * allocated by the first render that needs them, for min(its paths,
 * max_paths).  Larger waves mean fewer wave tails -- the last bounces of a
 * wave, when few paths are left -- and are faster: 16 -> 128 Mi gives +24 %
 * on a 1920x1080x256 RTIOW render, 16 -> 64 Mi +22 % on 1M spheres, and
 * that whole render (530.8 M paths) as one wave instead of two of 2^28
 * +0.6 %. */
VENU_API venu_status venu_renderer_create(uint32_t max_paths, uint32_t flags, venu_renderer** out);
/* One Renderer::Draw: spp samples per pixel for every pixel, added to the
 * accumulator (VENU_ACCUM_FLOATS_PER_PIXEL floats per pixel, device), then
 * the running mean written to image_f (RGBA32F, may be NULL) and image8
 * (sRGB RGBA8 as Core/RayTracer.cu:16-47, may be NULL).  Asynchronous on
 * `stream`; statistics are final once the stream has been synchronised.
 * With the fused traversal variants (2, 4) each wave's bounce loop is one
 * CUDA graph launch whose while node stops when no rays are left (the graph
 * is built by the first such render and rebuilt when the scene, camera,
 * image size, depth or tuning change); the renderer must not be used from
 * two streams at once.  On a stream that is being captured, every bounce is
 * launched from the host instead, so the render can be captured into the
 * caller's graph.  Replaces Core/Renderer.h:35-78. */
VENU_API venu_status venu_render(venu_renderer* r, const venu_scene* scene, const venu_camera* camera,
                        const venu_render_opts* opts, float* accum_dev, float* image_f_dev,
                        uint8_t* image8_dev, void* stream);
VENU_API venu_status venu_renderer_stats(venu_renderer* r, venu_render_stats* out);

/* Launch shapes and traversal variant of a renderer (chosen by the
 * autotuner, venusaur_gb300/tune.py; results do not depend on them). */
typedef struct venu_tuning {
    uint32_t traverse_variant;       /* 0: each warp takes 32 rays and runs them to the end;
                                        1: idle lanes take new rays;
                                        2: as 0, then the warp shades its 32 hits in the same
                                           kernel (no separate shade launch; default);
                                        3: 2 for the primary rays, 0 for later bounces;
                                        4: as 2, over the 4-wide tree collapsed from the
                                           LBVH (4 child boxes tested per step);
                                        5: 2 for the primary rays, then 0 over the 4-wide tree
                                        (4 and 5: the first such render of a scene builds its
                                        4-wide tree and blocks until it is built) */
    uint32_t refill_min;             /* variant 1: refill when >= this many lanes are idle (1..32) */
    uint32_t traverse_block;         /* threads per traversal block: 64, 128 or 256 */
    uint32_t traverse_blocks_per_sm; /* 0 = as many as fit */
    uint32_t shade_block;            /* threads per shade block: 64..512, multiple of 32 */
    uint32_t shade_blocks_per_sm;    /* 0 = as many as fit */
    uint32_t in_place_factor;        /* fused variants: a launch with at most this many rays per
                                        thread of its grid finishes its paths in place, bounce
                                        after bounce, refilling finished threads (1..16; 0 = 1;
                                        the batch engine ignores it) */
} venu_tuning;
VENU_API venu_status venu_renderer_set_tuning(venu_renderer* r, const venu_tuning* t);
VENU_API venu_status venu_renderer_get_tuning(const venu_renderer* r, venu_tuning* t);

/* ---- batched / served rendering ----------------------------------------
 * No single counterpart in the reference (it renders one scene per
 * optixLaunch); each job is one Renderer::Draw of its own scene, camera and
 * image.  All admitted jobs share one pool of paths in flight: every ray
 * carries its job, finished paths are replaced by new camera rays of the
 * jobs in plan order (their camera rays made inside the trace kernel), and
 * the whole path loop -- trace+shade, plan, repeat -- is one CUDA graph
 * launch driven by a device-side
 * while condition.  Results are bit-identical to venu_render of each job
 * alone (same seeds, same per-pixel sample order). */
typedef struct venu_batch venu_batch;

typedef struct venu_job_desc {
    const venu_scene* scene;
    venu_camera camera;
    venu_render_opts opts;  /* width, height, spp, subframe_index, max_depth, flags */
    float* accum;           /* device, VENU_ACCUM_FLOATS_PER_PIXEL per pixel, caller-owned */
    float* image_f;         /* optional RGBA32F mean */
    uint8_t* image8;        /* optional sRGB RGBA8 */
} venu_job_desc;

typedef struct venu_batch_stats {
    uint64_t segments;        /* ray casts since creation */
    uint64_t paths_done;      /* finished paths since creation */
    uint64_t iterations;      /* path-loop iterations since creation */
    uint64_t graph_launches;  /* venu_batch_run calls that launched the graph */
    uint64_t resident_bytes;  /* device bytes held for admitted jobs (seed tables, sample slots) */
    uint32_t active_jobs;
    uint32_t reserved;
} venu_batch_stats;

#define VENU_BATCH_NO_GRAPH 1u /* run the path loop from the host (one launch per stage) */

/* pool_paths: paths in flight (0 = 64 Mi, about 7 GB); max_jobs: concurrently admitted jobs (<= 4096). */
VENU_API venu_status venu_batch_create(uint32_t pool_paths, uint32_t max_jobs, uint32_t flags, venu_batch** out);
VENU_API venu_status venu_batch_set_tuning(venu_batch* b, const venu_tuning* t);
/* Bytes venu_batch_submit allocates for a job of this size (seed table + slots). */
VENU_API uint64_t venu_batch_job_bytes(uint32_t width, uint32_t height, uint32_t spp);
/* Admits a job: allocates its seed table and per-sample slots and computes the
 * seeds on `stream`.  The scene and output buffers must stay valid until the
 * job is collected.  VENU_ERR_TOO_LARGE when max_jobs are admitted. */
VENU_API venu_status venu_batch_submit(venu_batch* b, const venu_job_desc* job, void* stream, uint32_t* job_id);
/* n jobs at once (one call, one seed-table launch per 32 jobs): job_ids[k]
 * gets job k's id.  All or nothing: on an error no job of the call is
 * admitted.  venu_batch_submit is this with n = 1. */
VENU_API venu_status venu_batch_submit_many(venu_batch* b, const venu_job_desc* jobs, uint32_t n, void* stream,
                                            uint32_t* job_ids);
/* Runs the shared path loop for at most max_iterations steps (0 = until
 * every admitted job has finished) as one graph launch on `stream`; a step
 * is one iteration (every queued ray traced once) unless venu_batch_set_chunk
 * splits iterations.  With VENU_RUN_STOP_ON_FINISH the loop also ends after
 * the step in which a job's last path finished, so a server can hand results
 * out at once. */
#define VENU_RUN_STOP_ON_FINISH 1u
VENU_API venu_status venu_batch_run(venu_batch* b, uint32_t max_iterations, uint32_t flags, void* stream);
/* Waits for `stream`, then accumulates, resolves and releases every finished
 * job; writes their ids (up to cap) and the count. */
VENU_API venu_status venu_batch_collect(venu_batch* b, void* stream, uint32_t* finished_ids, uint32_t cap,
                                        uint32_t* count);
/* Plan order of the admitted jobs: which job's new paths take free pool slots
 * first.  FIFO (default): submission order.  SHORTEST_FIRST: fewest
 * unfinished paths first (as of the last collect; ties by submission) --
 * small jobs overtake large ones, which lowers typical latency; a steady
 * stream of small jobs can delay a large one indefinitely.  SEQUENTIAL:
 * submission order, and a job gets slots only once every earlier job has
 * finished all its paths (no overlap: a job's last bounces are not slowed
 * by the next job's rays; the pool runs part-empty meanwhile).  Results do
 * not depend on the order.  Call between runs, not while a venu_batch_run
 * is in flight. */
#define VENU_POLICY_FIFO 0u
#define VENU_POLICY_SHORTEST_FIRST 1u
#define VENU_POLICY_SEQUENTIAL 2u
VENU_API venu_status venu_batch_set_policy(venu_batch* b, uint32_t policy);
/* Sets (on != 0) or clears a flag in mapped host memory that the device loop
 * reads once per iteration: while set, a running venu_batch_run ends at its
 * next iteration boundary (and later runs after one iteration), so
 * a host with new jobs can admit them without waiting for the run.  The only
 * batch call that may be made from another host thread. */
VENU_API venu_status venu_batch_interrupt(venu_batch* b, uint32_t on);
/* Rays traced per loop step (0, the default: a whole iteration, every queued
 * ray, per step).  With a chunk, an iteration over a large pool is split into
 * steps of at most `rays` rays, and the iteration cap, stop-on-finish and the
 * interrupt take effect at step boundaries: a host can admit or run other
 * work after at most one chunk instead of one whole-pool iteration.  Results
 * do not depend on it. */
VENU_API venu_status venu_batch_set_chunk(venu_batch* b, uint32_t rays);
VENU_API venu_status venu_batch_stats_get(venu_batch* b, venu_batch_stats* out);
VENU_API venu_status venu_batch_destroy(venu_batch* b);

/* ---- render server (continuous batching) ------------------------------
 * No counterpart in the reference (it serves one interactive window).  A
 * server owns one host thread and one venu_batch.  Requests arrive at any
 * time from any thread; the server admits them first-come first-served
 * while the device memory they need fits the HBM budget, keeps scene BVHs
 * resident across requests that share a scene_key (evicting unused ones,
 * least recently used first, when the budget needs room), advances every
 * admitted job together in the shared path pool a few iterations at a time,
 * and retires finished jobs: image copied to host memory, buffers freed,
 * latency recorded.  A request that can never fit the budget fails with
 * VENU_ERR_OOM; a cancelled pending request completes with
 * VENU_ERR_CANCELLED; a failure of one request never stops the others. */
typedef struct venu_server venu_server;

typedef struct venu_request {
    const venu_sphere* spheres; /* host; copied by venu_server_submit.  NULL with a
                                   scene_key: use the resident scene of that key
                                   (VENU_ERR_INVALID if it is not resident) */
    uint32_t num_spheres;
    uint32_t reserved;
    uint64_t scene_key;         /* != 0: requests with the same key share one resident BVH */
    venu_camera camera;
    venu_render_opts opts;      /* accumulation is reset per request, except in a session */
    uint64_t tag;               /* returned with the result */
    uint64_t session;           /* != 0: a progressive session (Renderer::Draw served over
                                   requests, Core/Renderer.h:35-78): the samples are added to
                                   the session's resident accumulator and the image is the
                                   running mean, unless opts.flags has VENU_FLAG_RESET_ACCUM or
                                   the size changed (then it restarts); the caller advances
                                   opts.subframe_index.  Requests of one session run one at a
                                   time in submission order. */
} venu_request;

typedef struct venu_result {
    uint64_t request_id;
    uint64_t tag;
    int32_t status;             /* venu_status of the request */
    uint32_t width, height;
    uint32_t reserved;
    const uint8_t* image8;      /* host sRGB RGBA8, valid until venu_server_release */
    double t_submit, t_admit, t_done; /* seconds, steady clock of the server */
} venu_result;

typedef struct venu_server_stats {
    uint64_t submitted, completed, failed;
    uint64_t resident_bytes;    /* scenes + admitted jobs */
    uint64_t budget_bytes;
    uint64_t segments;          /* ray casts traced by the server */
    uint32_t active, pending;
    double p50_ms, p99_ms;      /* request latency (submit -> image on host), completed requests */
    double busy_seconds;        /* wall time with at least one admitted job */
    uint64_t evictions;         /* resident scenes evicted to make room under the budget */
    uint64_t admission_waits;   /* server steps at which the next request waited for room */
    uint64_t peak_resident_bytes; /* most device bytes held at once (scenes, jobs, sessions) */
} venu_server_stats;

/* Test hooks: make the next admission fail as if its allocation failed
 * (VENU_INJECT_ALLOC) or its BVH build failed (VENU_INJECT_SCENE). */
#define VENU_INJECT_ALLOC 1u
#define VENU_INJECT_SCENE 2u

VENU_API venu_status venu_server_create(uint64_t hbm_budget_bytes, uint32_t pool_paths, uint32_t max_jobs,
                                        uint32_t iterations_per_step, venu_server** out);
VENU_API venu_status venu_server_submit(venu_server* s, const venu_request* req, uint64_t* request_id);
/* Plan order of the bulk lane (VENU_POLICY_FIFO, the default,
 * VENU_POLICY_SHORTEST_FIRST or VENU_POLICY_SEQUENTIAL; see
 * venu_batch_set_policy); the express lane is always FIFO and admission
 * first come first served.  Takes effect at the server's next step. */
VENU_API venu_status venu_server_set_policy(venu_server* s, uint32_t policy);
/* Express lane: requests of at most max_paths paths (width x height x spp)
 * admitted from now on run in a second, small pool (2 Mi paths) that the
 * server advances ahead of the bulk pool at every step, and the bulk pool
 * yields every 4 Mi traced rays; 0 (the default) turns it off.  A small
 * request then waits for at most one bulk chunk instead of sharing every
 * bounce with the large jobs. */
VENU_API venu_status venu_server_set_express(venu_server* s, uint64_t max_paths);
/* Frees a progressive session's accumulator (after its admitted request, if
 * any, completes); a later request with the same id starts a new session. */
VENU_API venu_status venu_server_end_session(venu_server* s, uint64_t session);
/* Blocks until the request completes or timeout_s passes (VENU_ERR_NOT_READY).
 * timeout_s <= 0 (or NaN) looks once without waiting; values above 1e9 s,
 * infinity included, wait 1e9 s (about 32 years). */
VENU_API venu_status venu_server_wait(venu_server* s, uint64_t request_id, double timeout_s, venu_result* out);
VENU_API venu_status venu_server_cancel(venu_server* s, uint64_t request_id);
VENU_API venu_status venu_server_release(venu_server* s, uint64_t request_id);
VENU_API venu_status venu_server_inject(venu_server* s, uint32_t what);
VENU_API venu_status venu_server_stats_get(venu_server* s, venu_server_stats* out);
VENU_API venu_status venu_server_destroy(venu_server* s);
VENU_API venu_status venu_renderer_destroy(venu_renderer* r);

#ifdef __cplusplus
}
#endif
#endif /* VENU_H */
