/*
 * venu_oracle.h -- CPU oracle for the Venusaur-GB300 path tracer.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code: only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference arm use it, always as the checker.
 *
 * It restates, on the host, the reference's per-pixel path tracer
 * (Core/RayTracer.cu:8-449, Core/random.cuh:31-67, Core/Camera.cpp:24-37)
 * in two arithmetic modes:
 *
 *   VO_MODE_REF    the reference's source semantics literally: recursive
 *                  attenuation order, double cos/sin in the dielectric,
 *                  pow() in Schlick, plain half-b quadratic, spp-sum then
 *                  multiply by 1/spp, lerp across subframes, max depth 4
 *                  unless overridden, brute-force closest hit.
 *   VO_MODE_REF_BVH  VO_MODE_REF with the closest hit found through the host
 *                  LBVH instead of by brute force (the reference's
 *                  intersection program on the spheres the walk reaches;
 *                  the same hit as the brute force: smallest root, exact
 *                  ties to the smaller index).  The reference's arithmetic
 *                  at the cost of an accelerated CPU tracer.
 *   VO_MODE_GB300  the arithmetic the CUDA kernels implement (stable
 *                  quadratic with exact c, FP32 dielectric, pow5 as a product,
 *                  forward throughput, Kahan accumulation, LBVH traversal).
 *
 * plus the host LBVH (Morton30 -> stable sort -> Karras -> refit) and an
 * FP64 brute-force closest-hit oracle.
 *
 * The sphere / camera structs have the same byte layout as the product's
 * venu_sphere / venu_camera (include/venu.h).
 */
#ifndef VENU_ORACLE_H
#define VENU_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vo_sphere {
    float center[3];
    float radius;
    float albedo[3];
    float fuzz;
    float ir;
    uint32_t material; /* 0 lambertian, 1 metal, 2 dielectric */
    uint32_t pad[2];
} vo_sphere;

typedef struct vo_camera {
    float origin[3];
    float u[3];
    float v[3];
    float w[3];
    float lens_radius;
} vo_camera;

typedef struct vo_node {
    float lo[3];
    int32_t left;
    float hi[3];
    int32_t right;
} vo_node;

enum { VO_MODE_REF = 0, VO_MODE_GB300 = 1, VO_MODE_REF_BVH = 2 };

typedef struct vo_render_opts {
    uint32_t width, height;
    uint32_t spp;
    uint32_t subframe_index;
    uint32_t max_depth;
    uint32_t mode;      /* VO_MODE_* */
    uint32_t nthreads;  /* 0 = hardware concurrency */
    uint32_t row_begin; /* render rows [row_begin, row_end) only; 0,0 = all */
    uint32_t row_end;
} vo_render_opts;

/* --- RNG (Core/random.cuh:31-67) --- */
uint32_t vo_tea4(uint32_t v0, uint32_t v1);
void vo_rnd_stream(uint32_t seed, uint32_t n, float* out, uint32_t* states_out);

/* --- scenes (Core/Scene.h:13-80 with a fixed, documented draw order) --- */
uint32_t vo_scene_rtiow(uint32_t seed, vo_sphere* out, uint32_t cap);
uint32_t vo_scene_random(uint32_t n, uint32_t seed, const float box_lo[3],
                         const float box_hi[3], float rmin, float rmax,
                         vo_sphere* out);

/* --- camera (Core/Camera.cpp:24-37, Core/camera.h:20) --- */
void vo_camera_look_at(const float eye[3], const float lookat[3], float vfov_deg,
                       float aspect, float aperture, float focal, vo_camera* out);

/* --- LBVH --- */
int vo_lbvh_build(const vo_sphere* s, uint32_t n, uint32_t* morton_sorted,
                  uint32_t* sorted_ids, vo_node* nodes, float bounds[6],
                  uint32_t* depth_out);
/* Build on s_build, then move every sphere to s_new (same count and original
 * indices) keeping topology, slot order and hoisted set, and refit the boxes
 * (the product's venu_scene_update). */
int vo_lbvh_refit(const vo_sphere* s_build, const vo_sphere* s_new, uint32_t n, vo_node* nodes);

/* --- closest hit --- */
/* rays: n x 6 floats (ox,oy,oz,dx,dy,dz).  FP64 brute force over the float
 * inputs converted exactly to double; id = original sphere index or -1. */
void vo_trace_fp64(const vo_sphere* s, uint32_t ns, const float* rays, uint32_t n,
                   float tmin, float tmax, int32_t* id, double* t, double* disc_rel,
                   double* t_second);
/* GB300-mode FP32 LBVH traversal (same arithmetic as the CUDA kernel).
 * id = original sphere index or -1; front = 1 if the ray hits the outside. */
void vo_trace_bvh(const vo_sphere* s, uint32_t ns, const float* rays, uint32_t n,
                  float tmin, float tmax, int32_t* id, float* t, uint32_t* front,
                  uint32_t* nodes_visited, uint32_t* spheres_tested);
/* Per ray, the deepest traversal stack of vo_trace_bvh's walk (entries). */
void vo_trace_bvh_stack(const vo_sphere* s, uint32_t ns, const float* rays, uint32_t n, float tmin, float tmax,
                        uint32_t* max_stack);
/* REF-mode FP32 brute force (reference quadratic, OptiX-like strict tmax). */
void vo_trace_ref(const vo_sphere* s, uint32_t ns, const float* rays, uint32_t n,
                  float tmin, float tmax, int32_t* id, float* t);

/* --- render ---
 * GB300 mode: accum is 8 floats per pixel {sum.rgb, n, comp.rgb, 0} (the
 *   device layout), updated in place; image_f gets {mean.rgb, 1}.
 * REF / REF_BVH modes: accum is 4 floats per pixel {mean.rgb, 1} (Params::accum).
 * image8 gets sRGB RGBA8 in both modes (may be NULL).
 * samples_out (may be NULL): per (s, pixel) final path radiance, 3 floats,
 *   layout [s][pixel][3] for the rendered rows.
 * Returns the number of path segments (ray casts) traced. */
uint64_t vo_render(const vo_sphere* s, uint32_t ns, const vo_camera* cam,
                   const vo_render_opts* opts, float* accum, float* image_f,
                   uint8_t* image8, float* samples_out, uint64_t* nodes_visited,
                   uint64_t* spheres_tested);
/* vo_render of spheres s through the LBVH built on s_build and refit to s
 * (vo_lbvh_refit); s_build = NULL is vo_render. */
uint64_t vo_render_refit(const vo_sphere* s_build, const vo_sphere* s, uint32_t ns,
                         const vo_camera* cam, const vo_render_opts* opts, float* accum,
                         float* image_f, uint8_t* image8, float* samples_out,
                         uint64_t* nodes_visited, uint64_t* spheres_tested);

/* sRGB encode of linear RGB (Core/RayTracer.cu:16-47) with pow() (REF) and
 * with the GB300 arithmetic's own power routine (the kernels' bytes). */
void vo_make_color(const float* rgb, uint32_t n, uint8_t* out4);
void vo_make_color_gb300(const float* rgb, uint32_t n, uint8_t* out4);
/* x^(1/2.4) by the GB300 power routine, for x in [2^-126, 1]. */
void vo_srgb_pow(const float* x, uint64_t n, float* out);

#ifdef __cplusplus
}
#endif
#endif
