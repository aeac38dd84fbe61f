// api.cu -- C ABI: errors, device check, scene lifecycle, host-side scene
// generators and camera frame.
#include "venu_device.cuh"
#include "venu_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <random>
#include <string>
#include <vector>

namespace venu {

namespace {
thread_local std::string g_error;
std::once_flag g_dev_once;
venu_status g_dev_status = VENU_ERR_NO_DEVICE;
int g_sms = 0, g_major = 0, g_minor = 0;

__global__ void k_probe(int* out) {
    if (out) *out = 103;
}

void probe_device() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    cudaDeviceProp p;
    if (e == cudaSuccess) e = cudaGetDeviceProperties(&p, dev);
    if (e != cudaSuccess) {
        g_dev_status = VENU_ERR_NO_DEVICE;
        g_error = std::string("no usable CUDA device: ") + cudaGetErrorString(e);
        return;
    }
    g_sms = p.multiProcessorCount;
    g_major = p.major;
    g_minor = p.minor;
    if (!(p.major == 10 && p.minor == 3)) {
        g_dev_status = VENU_ERR_NO_DEVICE;
        g_error = "libvenusaur_gb300 is built for sm_103a only; device is sm_" + std::to_string(p.major) +
                  std::to_string(p.minor);
        return;
    }
    cudaFuncAttributes a;
    e = cudaFuncGetAttributes(&a, k_probe);
    if (e != cudaSuccess) {
        g_dev_status = VENU_ERR_NO_DEVICE;
        g_error = std::string("kernels do not load on this device: ") + cudaGetErrorString(e);
        return;
    }
    g_dev_status = VENU_OK;
}
}  // namespace

void set_error(const std::string& msg) { g_error = msg; }

venu_status cuda_fail(cudaError_t e, const char* what) {
    g_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return e == cudaErrorMemoryAllocation ? VENU_ERR_OOM : VENU_ERR_CUDA;
}

venu_status require_device() {
    std::call_once(g_dev_once, probe_device);
    if (g_dev_status != VENU_OK) {
        // keep the probe's message for this thread too
        std::string msg = g_error.empty() ? std::string("no usable sm_103 CUDA device") : g_error;
        g_error = msg;
    }
    return g_dev_status;
}

int sm_count() { return g_sms > 0 ? g_sms : 1; }

// ---------------------------------------------------------------------------
// Scene generators (host).  Scene RNG: std::mt19937 (its output sequence is
// fixed by the C++ standard) with u = (x >> 8) * 2^-24.  exp/log of the
// log-uniform radius use only +,-,*,/ so scenes are identical on x86-64 and
// aarch64 hosts.
// ---------------------------------------------------------------------------
namespace {
struct Rng {
    std::mt19937 g;
    explicit Rng(uint32_t s) : g(s) {}
    float U() { return (float)(g() >> 8) * (1.0f / 16777216.0f); }
};
double dexp(double x) {
    const double ln2_hi = 6.93147180369123816490e-01, ln2_lo = 1.90821492927058770002e-10;
    double kf = std::floor(x * 1.44269504088896338700 + 0.5);
    double r = (x - kf * ln2_hi) - kf * ln2_lo;
    double term = 1.0, sum = 1.0;
    for (int i = 1; i < 24; ++i) {
        term = term * r / (double)i;
        sum = sum + term;
    }
    return std::ldexp(sum, (int)kf);
}
double dlog(double x) {
    const double ln2_hi = 6.93147180369123816490e-01, ln2_lo = 1.90821492927058770002e-10;
    int e = 0;
    double m = std::frexp(x, &e);
    if (m < 0.70710678118654752440) {
        m = m * 2.0;
        e -= 1;
    }
    double s = (m - 1.0) / (m + 1.0), s2 = s * s, term = s, sum = 0.0;
    for (int i = 1; i < 60; i += 2) {
        sum = sum + term / (double)i;
        term = term * s2;
    }
    return 2.0 * sum + (double)e * ln2_hi + (double)e * ln2_lo;
}
venu_sphere sphere(float cx, float cy, float cz, float r, uint32_t mat, float ar, float ag, float ab, float fuzz,
                   float ir) {
    venu_sphere s;
    std::memset(&s, 0, sizeof(s));
    s.center[0] = cx;
    s.center[1] = cy;
    s.center[2] = cz;
    s.radius = r;
    s.albedo[0] = ar;
    s.albedo[1] = ag;
    s.albedo[2] = ab;
    s.fuzz = fuzz;
    s.ir = ir;
    s.material = mat;
    return s;
}
// Core/Scene.h:28-64 material choice (argument lists drawn left to right).
venu_sphere material_sphere(Rng& R, float choose, float cx, float cy, float cz, float r) {
    if ((double)choose < 0.8) {
        float a[3], b[3];
        for (int i = 0; i < 3; ++i) a[i] = R.U();
        for (int i = 0; i < 3; ++i) b[i] = R.U();
        return sphere(cx, cy, cz, r, VENU_LAMBERTIAN, a[0] * b[0], a[1] * b[1], a[2] * b[2], 0.0f, 0.0f);
    }
    if ((double)choose < 0.95) {
        float a[3];
        for (int i = 0; i < 3; ++i) a[i] = 0.5f + (1.0f - 0.5f) * R.U();
        float fz = 0.0f + (0.5f - 0.0f) * R.U();
        return sphere(cx, cy, cz, r, VENU_METAL, a[0], a[1], a[2], fz, 0.0f);
    }
    return sphere(cx, cy, cz, r, VENU_DIELECTRIC, 0.0f, 0.0f, 0.0f, 0.0f, 1.5f);
}
}  // namespace

}  // namespace venu

using namespace venu;

extern "C" const char* venu_last_error(void) { return g_error.c_str(); }

extern "C" venu_status venu_device_check(int* sm_count_out, int* cc_major_out, int* cc_minor_out) {
    venu_status s = require_device();
    if (sm_count_out) *sm_count_out = g_sms;
    if (cc_major_out) *cc_major_out = g_major;
    if (cc_minor_out) *cc_minor_out = g_minor;
    return s;
}

extern "C" uint32_t venu_scene_generate_rtiow(uint32_t seed, venu_sphere* out, uint32_t cap) {
    std::vector<venu_sphere> v;
    Rng R(seed);
    v.push_back(sphere(0.0f, -1000.0f, 0.0f, 1000.0f, VENU_LAMBERTIAN, 0.5f, 0.5f, 0.5f, 0.0f, 0.0f));
    for (int a = -11; a < 11; a++) {
        for (int b = -11; b < 11; b++) {
            float choose = R.U();
            float ux = R.U();
            float cx = (float)((double)a + 0.9 * (double)ux);
            float uz = R.U();
            float cz = (float)((double)b + 0.9 * (double)uz);
            float dx = cx - 4.0f, dy = 0.2f - 0.2f, dz = cz - 0.0f;
            float len = std::sqrt(dx * dx + dy * dy + dz * dz);
            if ((double)len > 0.9) v.push_back(material_sphere(R, choose, cx, 0.2f, cz, 0.2f));
        }
    }
    v.push_back(sphere(0.0f, 1.0f, 0.0f, 1.0f, VENU_DIELECTRIC, 0.0f, 0.0f, 0.0f, 0.0f, 1.5f));
    v.push_back(sphere(-4.0f, 1.0f, 0.0f, 1.0f, VENU_LAMBERTIAN, 0.4f, 0.2f, 0.1f, 0.0f, 0.0f));
    v.push_back(sphere(4.0f, 1.0f, 0.0f, 1.0f, VENU_METAL, 0.7f, 0.6f, 0.5f, 0.0f, 0.0f));
    const uint32_t n = (uint32_t)v.size();
    if (out) std::memcpy(out, v.data(), sizeof(venu_sphere) * std::min(n, cap));
    return n;
}

extern "C" venu_status venu_scene_generate_random(uint32_t n, uint32_t seed, const float box_lo[3],
                                                  const float box_hi[3], float rmin, float rmax, venu_sphere* out) {
    if (!out || !box_lo || !box_hi || !(rmin > 0.0f) || !(rmax >= rmin)) {
        set_error("venu_scene_generate_random: bad argument");
        return VENU_ERR_INVALID;
    }
    if (n == 0) return VENU_OK;
    Rng R(seed);
    out[0] = sphere(0.0f, -1000.0f, 0.0f, 1000.0f, VENU_LAMBERTIAN, 0.5f, 0.5f, 0.5f, 0.0f, 0.0f);
    const double lrat = dlog((double)rmax / (double)rmin);
    for (uint32_t i = 1; i < n; ++i) {
        float choose = R.U();
        float cx = box_lo[0] + (box_hi[0] - box_lo[0]) * R.U();
        float cy = box_lo[1] + (box_hi[1] - box_lo[1]) * R.U();
        float cz = box_lo[2] + (box_hi[2] - box_lo[2]) * R.U();
        float ur = R.U();
        float r = (float)((double)rmin * dexp((double)ur * lrat));
        out[i] = material_sphere(R, choose, cx, cy, cz, r);
    }
    return VENU_OK;
}

namespace {
// glm semantics: dot = (x*x + y*y) + z*z, normalize = v * (1 / sqrt(dot)).
float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
void norm3(float* v) {
    float inv = 1.0f / std::sqrt(dot3(v, v));
    v[0] = v[0] * inv;
    v[1] = v[1] * inv;
    v[2] = v[2] * inv;
}
}  // namespace

extern "C" void venu_camera_look_at(const float eye[3], const float lookat[3], float vfov_deg, float aspect,
                                    float aperture, float focal, venu_camera* out) {
    // Camera::SetForward (Core/camera.h:27) normalises lookat - eye.
    float fwd[3] = {lookat[0] - eye[0], lookat[1] - eye[1], lookat[2] - eye[2]};
    norm3(fwd);
    venu_camera_frame(eye, fwd, vfov_deg, aspect, aperture, focal, out);
}

extern "C" void venu_camera_frame(const float eye[3], const float forward[3], float vfov_deg, float aspect,
                                  float aperture, float focal, venu_camera* out) {
    // Camera::UpdateUVW (Core/Camera.cpp:27-37) for an already unit forward.
    auto cross3 = [](const float* x, const float* y, float* o) {
        o[0] = x[1] * y[2] - y[1] * x[2];
        o[1] = x[2] * y[0] - y[2] * x[0];
        o[2] = x[0] * y[1] - y[0] * x[1];
    };
    const float* fwd = forward;
    float w[3] = {fwd[0] * focal, fwd[1] * focal, fwd[2] * focal};
    const float up[3] = {0.0f, 1.0f, 0.0f};
    float u[3], v[3];
    cross3(w, up, u);
    norm3(u);
    cross3(u, w, v);
    norm3(v);
    float theta = vfov_deg * 0.01745329251994329576923690768489f;
    float h = std::tan(theta * 0.5f);
    float vh = 2.0f * h;
    float vw = aspect * vh;
    float su = focal * vw, sv = focal * vh;
    for (int i = 0; i < 3; ++i) {
        out->origin[i] = eye[i];
        out->u[i] = u[i] * su;
        out->v[i] = v[i] * sv;
        out->w[i] = w[i];
    }
    out->lens_radius = aperture * 0.5f;
}

extern "C" void venu_camera_rotate(const float forward[3], const float axis[3], float degrees, float out[3]) {
    // Camera::Pitch / Yaw / Roll (Core/camera.h:56-78):
    //   q = glm::rotate(quat(1,0,0,0), glm::radians(degrees), axis)
    //   forward = normalize(forward * q)
    // restated from GLM's published quaternion functions: rotate() normalises
    // the axis only when its length is off 1 by more than 0.001 and builds
    // q = (cos(a/2), axis*sin(a/2)) (the product with the identity is exact);
    // vec3 * quat rotates by inverse(q) = conjugate(q) / dot(q, q), applied as
    // v + 2*(cross(qv, v)*w + cross(qv, cross(qv, v))).
    float ax[3] = {axis[0], axis[1], axis[2]};
    const float len = std::sqrt(dot3(ax, ax));
    if (std::fabs(len - 1.0f) > 0.001f) {
        const float inv = 1.0f / len;
        ax[0] *= inv;
        ax[1] *= inv;
        ax[2] *= inv;
    }
    const float a = degrees * 0.01745329251994329576923690768489f;
    const float sh = std::sin(a * 0.5f), ch = std::cos(a * 0.5f);
    const float qw = ch, qx = ax[0] * sh, qy = ax[1] * sh, qz = ax[2] * sh;
    const float d = (qw * qw + qx * qx) + (qy * qy + qz * qz);
    const float iw = qw / d, ix = -qx / d, iy = -qy / d, iz = -qz / d;
    const float v[3] = {forward[0], forward[1], forward[2]};
    const float uv[3] = {iy * v[2] - v[1] * iz, iz * v[0] - v[2] * ix, ix * v[1] - v[0] * iy};
    const float uuv[3] = {iy * uv[2] - uv[1] * iz, iz * uv[0] - uv[2] * ix, ix * uv[1] - uv[0] * iy};
    float r[3];
    for (int i = 0; i < 3; ++i) r[i] = v[i] + (uv[i] * iw + uuv[i]) * 2.0f;
    norm3(r);
    out[0] = r[0];
    out[1] = r[1];
    out[2] = r[2];
}

// ---- image files (the headless replacement of the GL display path,
// Core/CUDAOutputBuffer.h:284-339 and Core/Core.cpp:396-426) --------------
extern "C" venu_status venu_image_write_ppm(const char* path, const uint8_t* rgba8, uint32_t width, uint32_t height) {
    if (!path || (!rgba8 && width && height)) {
        set_error("venu_image_write_ppm: NULL argument");
        return VENU_ERR_INVALID;
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        set_error(std::string("venu_image_write_ppm: cannot open ") + path);
        return VENU_ERR_INVALID;
    }
    std::fprintf(f, "P6\n%u %u\n255\n", width, height);
    std::vector<uint8_t> row(3u * (size_t)width);
    bool ok = true;
    for (uint32_t y = height; y-- > 0 && ok;) {  // pixel row 0 is the bottom of the image
        const uint8_t* src = rgba8 + 4u * (size_t)y * width;
        for (uint32_t x = 0; x < width; ++x) {
            row[3 * x] = src[4 * x];
            row[3 * x + 1] = src[4 * x + 1];
            row[3 * x + 2] = src[4 * x + 2];
        }
        ok = std::fwrite(row.data(), 1, row.size(), f) == row.size();
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) {
        set_error(std::string("venu_image_write_ppm: write failed: ") + path);
        return VENU_ERR_INVALID;
    }
    return VENU_OK;
}

extern "C" venu_status venu_image_write_pfm(const char* path, const float* rgba32f, uint32_t width, uint32_t height) {
    if (!path || (!rgba32f && width && height)) {
        set_error("venu_image_write_pfm: NULL argument");
        return VENU_ERR_INVALID;
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        set_error(std::string("venu_image_write_pfm: cannot open ") + path);
        return VENU_ERR_INVALID;
    }
    // PFM: "PF", size, negative scale = little-endian floats, rows bottom to
    // top (the pixel order of the buffers); byte order fixed explicitly.
    std::fprintf(f, "PF\n%u %u\n-1.0\n", width, height);
    std::vector<uint8_t> row(12u * (size_t)width);
    bool ok = true;
    for (uint32_t y = 0; y < height && ok; ++y) {
        const float* src = rgba32f + 4u * (size_t)y * width;
        for (uint32_t x = 0; x < width; ++x)
            for (int c = 0; c < 3; ++c) {
                uint32_t b;
                std::memcpy(&b, &src[4 * x + c], 4);
                uint8_t* d = &row[12 * x + 4 * c];
                d[0] = (uint8_t)b;
                d[1] = (uint8_t)(b >> 8);
                d[2] = (uint8_t)(b >> 16);
                d[3] = (uint8_t)(b >> 24);
            }
        ok = std::fwrite(row.data(), 1, row.size(), f) == row.size();
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) {
        set_error(std::string("venu_image_write_pfm: write failed: ") + path);
        return VENU_ERR_INVALID;
    }
    return VENU_OK;
}

extern "C" venu_status venu_scene_create_device(const venu_sphere* spheres_dev, uint32_t n, void* stream,
                                                venu_scene** out) {
    if (!out || (!spheres_dev && n)) {
        set_error("venu_scene_create: NULL argument");
        return VENU_ERR_INVALID;
    }
    *out = nullptr;
    venu_status ds = require_device();
    if (ds != VENU_OK) return ds;
    venu_scene* s = new venu_scene();
    venu_status rc = build_scene(spheres_dev, n, reinterpret_cast<cudaStream_t>(stream), s);
    if (rc != VENU_OK) {
        free_scene(s);
        delete s;
        return rc;
    }
    *out = s;
    return VENU_OK;
}

extern "C" venu_status venu_scene_create(const venu_sphere* spheres_host, uint32_t n, void* stream,
                                         venu_scene** out) {
    if (!out || (!spheres_host && n)) {
        set_error("venu_scene_create: NULL argument");
        return VENU_ERR_INVALID;
    }
    *out = nullptr;
    venu_status ds = require_device();
    if (ds != VENU_OK) return ds;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    venu_sphere* d = nullptr;
    if (n) {
        VENU_CUDA(cudaMalloc(&d, sizeof(venu_sphere) * n));
        cudaError_t e = cudaMemcpyAsync(d, spheres_host, sizeof(venu_sphere) * n, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) {
            cudaFree(d);
            return cuda_fail(e, "venu_scene_create: upload");
        }
    }
    venu_status rc = venu_scene_create_device(d, n, stream, out);
    cudaStreamSynchronize(st);
    cudaFree(d);
    return rc;
}

extern "C" venu_status venu_scene_update_device(venu_scene* scene, const venu_sphere* spheres_dev, uint32_t n,
                                                void* stream) {
    if (!scene || (!spheres_dev && n)) {
        set_error("venu_scene_update: NULL argument");
        return VENU_ERR_INVALID;
    }
    if (n != scene->n) {
        set_error("venu_scene_update: sphere count differs from the scene's (" + std::to_string(n) + " vs " +
                  std::to_string(scene->n) + "); a different count needs venu_scene_create");
        return VENU_ERR_INVALID;
    }
    venu_status ds = require_device();
    if (ds != VENU_OK) return ds;
    return update_scene(scene, spheres_dev, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" venu_status venu_scene_update(venu_scene* scene, const venu_sphere* spheres_host, uint32_t n,
                                         void* stream) {
    if (!scene || (!spheres_host && n)) {
        set_error("venu_scene_update: NULL argument");
        return VENU_ERR_INVALID;
    }
    if (n != scene->n) return venu_scene_update_device(scene, nullptr, n, stream);  // reports the mismatch
    venu_status ds = require_device();
    if (ds != VENU_OK) return ds;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (n == 0) return VENU_OK;
    venu_sphere* d = nullptr;
    VENU_CUDA(cudaMallocAsync(&d, sizeof(venu_sphere) * n, st));
    cudaError_t e = cudaMemcpyAsync(d, spheres_host, sizeof(venu_sphere) * n, cudaMemcpyHostToDevice, st);
    venu_status rc = e == cudaSuccess ? update_scene(scene, d, st) : cuda_fail(e, "venu_scene_update: upload");
    cudaFreeAsync(d, st);
    cudaError_t se = cudaStreamSynchronize(st);
    if (rc == VENU_OK && se != cudaSuccess) rc = cuda_fail(se, "venu_scene_update");
    return rc;
}

extern "C" venu_status venu_scene_info_get(const venu_scene* s, venu_scene_info* out) {
    if (!s || !out) {
        set_error("venu_scene_info_get: NULL argument");
        return VENU_ERR_INVALID;
    }
    out->num_spheres = s->n;
    out->num_nodes = s->n > 1 ? s->n - 1 : 0;
    out->device_bytes = s->bytes;
    std::memcpy(out->bounds, s->bounds, sizeof(out->bounds));
    out->build_ms = s->build_ms;
    out->num_wide_nodes = s->nwide;
    out->wide_ms = s->wide_ms;
    return VENU_OK;
}

extern "C" venu_status venu_scene_export_bvh(const venu_scene* s, uint32_t* morton, uint32_t* ids, void* nodes) {
    if (!s) {
        set_error("venu_scene_export_bvh: NULL scene");
        return VENU_ERR_INVALID;
    }
    const uint32_t n = s->n;
    if (n == 0) return VENU_OK;
    if (morton) VENU_CUDA(cudaMemcpy(morton, s->keys, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
    if (ids) {
        VENU_CUDA(cudaMemcpy(ids, s->meta, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < n; ++i) ids[i] &= 0x3fffffffu;
    }
    if (nodes && n > 1) VENU_CUDA(cudaMemcpy(nodes, s->nodes, sizeof(float4) * 2 * (n - 1), cudaMemcpyDeviceToHost));
    return VENU_OK;
}

extern "C" venu_status venu_scene_destroy(venu_scene* s) {
    if (!s) return VENU_OK;
    free_scene(s);
    delete s;
    return VENU_OK;
}
