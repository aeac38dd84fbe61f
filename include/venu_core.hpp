// venu_core.hpp -- C++17 mirror of the reference's Core/ interface
// (Material, Sphere, Scene, Camera, CUDAOutputBuffer, Renderer) over the C ABI
// in venu.h.  Header-only; link libvenusaur_gb300.so and the CUDA runtime.
//
// It replaces Core/material.h, Core/sphere.h, Core/Scene.h, Core/camera.h,
// Core/CUDAOutputBuffer.h (the CUDA_DEVICE and ZERO_COPY buffer types) and
// Core/Renderer.h so that a main loop written against the reference
// (Init / Draw / Cleanup) compiles unchanged apart from the includes; glm is
// replaced by a small vec3.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "venu.h"

namespace venu_core {

struct vec3 {
    float x = 0, y = 0, z = 0;
    vec3() = default;
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};
// the glm::vec3 operations the reference's main loop uses (lookat - lookfrom)
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }

class Exception : public std::runtime_error {
   public:
    Exception(venu_status s, const std::string& what)
        : std::runtime_error(what + ": " + venu_last_error()), status(s) {}
    venu_status status;
};

inline void check(venu_status s, const char* what) {
    if (s != VENU_OK) throw Exception(s, what);
}
inline void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// Core/material.h:6-33
class Material {
   public:
    enum Type { Lambertian = 0, Metal, Dielectric };
    explicit Material(Type type, const vec3& albedo = vec3(), float fuzz = 0, float ir = 0)
        : m_type(type), m_albedo(albedo), m_fuzz(fuzz), m_ir(ir) {}
    Type GetType() const { return m_type; }
    vec3 GetAlbedo() const { return m_albedo; }
    float GetFuzz() const { return m_fuzz; }
    float GetIR() const { return m_ir; }

   private:
    Type m_type;
    vec3 m_albedo;
    float m_fuzz, m_ir;
};

// Core/sphere.h:5-36 (GetAABB uses |radius|)
class Sphere {
   public:
    Sphere(const vec3& center, float radius, const Material& material)
        : m_center(center), m_radius(radius), m_material(material) {}
    vec3 GetCenter() const { return m_center; }
    float GetRadius() const { return m_radius; }
    const Material& GetMaterial() const { return m_material; }
    void SetMaterial(const Material& m) { m_material = m; }
    void GetAABB(float lo[3], float hi[3]) const {
        float r = std::fabs(m_radius);
        lo[0] = m_center.x - r; lo[1] = m_center.y - r; lo[2] = m_center.z - r;
        hi[0] = m_center.x + r; hi[1] = m_center.y + r; hi[2] = m_center.z + r;
    }
    venu_sphere record() const {
        venu_sphere s{};
        s.center[0] = m_center.x; s.center[1] = m_center.y; s.center[2] = m_center.z;
        s.radius = m_radius;
        vec3 a = m_material.GetAlbedo();
        s.albedo[0] = a.x; s.albedo[1] = a.y; s.albedo[2] = a.z;
        s.fuzz = m_material.GetFuzz();
        s.ir = m_material.GetIR();
        s.material = (uint32_t)m_material.GetType();
        return s;
    }

   private:
    vec3 m_center;
    float m_radius;
    Material m_material;
};

// Core/Scene.h:13-84: the default constructor builds the RTIOW final scene.
class Scene {
   public:
    explicit Scene(uint32_t seed = 0) {
        std::vector<venu_sphere> buf(600);
        uint32_t n = venu_scene_generate_rtiow(seed, buf.data(), (uint32_t)buf.size());
        buf.resize(n);
        set(buf);
    }
    explicit Scene(const std::vector<Sphere>& spheres) : m_spheres(spheres) {
        for (uint32_t i = 0; i < m_spheres.size(); ++i) m_indices.push_back(i);
    }
    void set(const std::vector<venu_sphere>& recs) {
        m_spheres.clear();
        m_indices.clear();
        for (const auto& r : recs) {
            Material m((Material::Type)r.material, vec3(r.albedo[0], r.albedo[1], r.albedo[2]), r.fuzz, r.ir);
            m_spheres.emplace_back(vec3(r.center[0], r.center[1], r.center[2]), r.radius, m);
            m_indices.push_back((uint32_t)m_indices.size());
        }
    }
    std::vector<venu_sphere> records() const {
        std::vector<venu_sphere> out;
        for (const auto& s : m_spheres) out.push_back(s.record());
        return out;
    }
    std::vector<Sphere> m_spheres;
    std::vector<uint32_t> m_indices;
};

// Core/camera.h:9-100, Core/Camera.cpp:16-37
class Camera {
   public:
    Camera() { UpdateUVW(); }
    Camera(const vec3& origin, float vfov, float aspect, float aperture, float focalLength)
        : m_position(origin), m_vfov(vfov), m_aspect(aspect), m_aperture(aperture), m_focalLength(focalLength) {
        UpdateUVW();
    }
    void SetForward(vec3 d) {
        m_forward = normalize(d);
        m_changed = true;
    }
    void UVWFrame(vec3& U, vec3& V, vec3& W) {
        UpdateUVW();
        U = m_u;
        V = m_v;
        W = m_w;
    }
    float GetLensRadius() const { return m_aperture * 0.5f; }
    const vec3& GetPosition() const { return m_position; }
    float GetFocalLength() const { return m_focalLength; }
    void SetFocalLength(float f) {
        if (m_focalLength != f) {
            m_focalLength = f;
            m_changed = true;
        }
    }
    void MoveForward(float speed) {
        m_position = add_scaled(m_position, m_forward, speed);
        m_changed = true;
    }
    // Core/camera.h:42-78; u/v/w are those of the last UVWFrame (or Draw).
    void MoveRight(float speed) {
        m_position = add_scaled(m_position, normalize(m_u), speed);
        m_changed = true;
    }
    void MoveUp(float speed) {
        m_position = add_scaled(m_position, normalize(m_v), speed);
        m_changed = true;
    }
    void Pitch(float speed) { rotate(m_u, speed); }
    void Yaw(float speed) { rotate(m_v, speed); }
    void Roll(float speed) { rotate(m_w, speed); }
    bool Changed() {
        bool c = m_changed;
        m_changed = false;
        return c;
    }
    venu_camera params() const {
        venu_camera c{};
        const float e[3] = {m_position.x, m_position.y, m_position.z};
        const float f[3] = {m_forward.x, m_forward.y, m_forward.z};
        venu_camera_frame(e, f, m_vfov, m_aspect, m_aperture, m_focalLength, &c);
        return c;
    }

    // Renderer::Draw takes the frame through here, refreshing u/v/w as the
    // reference's UVWFrame does.
    venu_camera frame() {
        venu_camera c = params();
        m_u = vec3(c.u[0], c.u[1], c.u[2]);
        m_v = vec3(c.v[0], c.v[1], c.v[2]);
        m_w = vec3(c.w[0], c.w[1], c.w[2]);
        return c;
    }

   private:
    static vec3 normalize(const vec3& d) {
        float inv = 1.0f / std::sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
        return vec3(d.x * inv, d.y * inv, d.z * inv);
    }
    static vec3 add_scaled(const vec3& p, const vec3& d, float s) {
        return vec3(p.x + d.x * s, p.y + d.y * s, p.z + d.z * s);
    }
    void UpdateUVW() { frame(); }
    void rotate(const vec3& axis, float degrees) {
        const float f[3] = {m_forward.x, m_forward.y, m_forward.z};
        const float a[3] = {axis.x, axis.y, axis.z};
        float o[3];
        venu_camera_rotate(f, a, degrees, o);
        m_forward = vec3(o[0], o[1], o[2]);
        m_changed = true;
    }
    vec3 m_position;
    vec3 m_forward{0.0f, 0.0f, -1.0f};
    float m_vfov = 45.0f, m_aspect = 1.6f, m_aperture = 0.0f, m_focalLength = 1.0f;
    vec3 m_u, m_v, m_w;
    bool m_changed = true;
};

// Core/CUDAOutputBuffer.h:56-61
enum class CUDAOutputBufferType {
    CUDA_DEVICE = 0,  // device memory (supported)
    GL_INTEROP = 1,   // an OpenGL pixel buffer: no display here, rejected
    ZERO_COPY = 2,    // mapped pinned host memory the kernels write to (supported)
    CUDA_P2P = 3      // device memory shared with a GL display: rejected
};

// Core/CUDAOutputBuffer.h:64-106,108-382 (template, constructor, map / unmap,
// getHostPointer) for the headless buffer types.  The GL types need the
// display path, which this library replaces by writePPM / writePFM: their
// construction throws.  Besides the reference's PIXEL_FORMAT pixels the
// buffer holds the RGBA32F running mean that venu_render writes (floatPixels,
// writePFM).
template <typename PIXEL_FORMAT>
class CUDAOutputBuffer {
   public:
    CUDAOutputBuffer(CUDAOutputBufferType type, int32_t width, int32_t height) : m_type(type) {
        if (type == CUDAOutputBufferType::GL_INTEROP || type == CUDAOutputBufferType::CUDA_P2P)
            throw Exception(VENU_ERR_INVALID, "CUDAOutputBuffer: GL_INTEROP and CUDA_P2P need an OpenGL display");
        resize(width, height);
    }
    ~CUDAOutputBuffer() { release(); }
    CUDAOutputBuffer(const CUDAOutputBuffer&) = delete;
    CUDAOutputBuffer& operator=(const CUDAOutputBuffer&) = delete;

    void setDevice(int32_t device_idx) { m_device_idx = device_idx; }
    void setStream(cudaStream_t s) { m_stream = s; }

    // Core/CUDAOutputBuffer.h:173-234; sizes below 1 become 1 (ensureMinimumSize)
    void resize(int32_t width, int32_t height) {
        width = width < 1 ? 1 : width;
        height = height < 1 ? 1 : height;
        if (m_pixels && width == m_width && height == m_height) return;
        release();
        m_width = width;
        m_height = height;
        makeCurrent();
        const size_t n = (size_t)m_width * m_height;
        if (m_type == CUDAOutputBufferType::CUDA_DEVICE) {
            cuda_check(cudaMalloc(reinterpret_cast<void**>(&m_pixels), sizeof(PIXEL_FORMAT) * n), "CUDAOutputBuffer");
        } else {
            cuda_check(cudaHostAlloc(reinterpret_cast<void**>(&m_host_zcopy_pixels), sizeof(PIXEL_FORMAT) * n,
                                     cudaHostAllocPortable | cudaHostAllocMapped),
                       "CUDAOutputBuffer");
            cuda_check(cudaHostGetDevicePointer(reinterpret_cast<void**>(&m_pixels), m_host_zcopy_pixels, 0),
                       "CUDAOutputBuffer");
        }
        cuda_check(cudaMalloc(&m_pixels_f, 16u * n), "CUDAOutputBuffer");
    }

    // Device address of the pixels for the kernels (Core/CUDAOutputBuffer.h:236-262).
    PIXEL_FORMAT* map() { return m_pixels; }
    // Waits for the stream (Core/CUDAOutputBuffer.h:264-282).
    void unmap() {
        makeCurrent();
        cuda_check(cudaStreamSynchronize(m_stream), "unmap");
    }

    int32_t width() const { return m_width; }
    int32_t height() const { return m_height; }

    // Core/CUDAOutputBuffer.h:284-339: the GL pixel buffer of the display.
    unsigned int getPBO() {
        throw Exception(VENU_ERR_INVALID, "CUDAOutputBuffer::getPBO: no OpenGL display (use writePPM)");
    }
    void deletePBO() {}

    // Core/CUDAOutputBuffer.h:348-382: a host copy of the pixels.
    PIXEL_FORMAT* getHostPointer() {
        if (m_type == CUDAOutputBufferType::ZERO_COPY) {
            unmap();
            return m_host_zcopy_pixels;
        }
        m_host_pixels.resize((size_t)m_width * m_height);
        makeCurrent();
        cuda_check(cudaMemcpy(m_host_pixels.data(), m_pixels, sizeof(PIXEL_FORMAT) * m_host_pixels.size(),
                              cudaMemcpyDeviceToHost),
                   "getHostPointer");
        return m_host_pixels.data();
    }

    cudaStream_t stream() const { return m_stream; }
    float* floatPixels() { return m_pixels_f; }
    std::vector<float> getHostFloat() {
        std::vector<float> h(4u * m_width * m_height);
        makeCurrent();
        cuda_check(cudaMemcpy(h.data(), m_pixels_f, h.size() * sizeof(float), cudaMemcpyDeviceToHost),
                   "getHostFloat");
        return h;
    }
    // Headless stand-ins for the GL display (Core/CUDAOutputBuffer.h:284-339).
    void writePPM(const char* path) {
        static_assert(sizeof(PIXEL_FORMAT) == 4, "writePPM needs 4-byte RGBA8 pixels");
        const PIXEL_FORMAT* h = getHostPointer();
        check(venu_image_write_ppm(path, reinterpret_cast<const uint8_t*>(h), (uint32_t)m_width,
                                   (uint32_t)m_height),
              "writePPM");
    }
    void writePFM(const char* path) {
        std::vector<float> h = getHostFloat();
        check(venu_image_write_pfm(path, h.data(), (uint32_t)m_width, (uint32_t)m_height), "writePFM");
    }

   private:
    void makeCurrent() { cuda_check(cudaSetDevice(m_device_idx), "cudaSetDevice"); }
    void release() {
        if (m_type == CUDAOutputBufferType::CUDA_DEVICE && m_pixels) cudaFree(m_pixels);
        if (m_host_zcopy_pixels) cudaFreeHost(m_host_zcopy_pixels);
        if (m_pixels_f) cudaFree(m_pixels_f);
        m_pixels = nullptr;
        m_host_zcopy_pixels = nullptr;
        m_pixels_f = nullptr;
    }
    CUDAOutputBufferType m_type;
    int32_t m_width = 0, m_height = 0;
    PIXEL_FORMAT* m_pixels = nullptr;            // device address (mapped, for ZERO_COPY)
    PIXEL_FORMAT* m_host_zcopy_pixels = nullptr;  // ZERO_COPY host memory
    std::vector<PIXEL_FORMAT> m_host_pixels;
    float* m_pixels_f = nullptr;
    cudaStream_t m_stream = nullptr;
    int32_t m_device_idx = 0;
};

// Core/Renderer.h:22-97 over venu_scene / venu_render.
class Renderer {
   public:
    explicit Renderer(uint32_t samples_per_pixel = 16, uint32_t max_depth = 4, uint32_t max_paths = 0)
        : m_spp(samples_per_pixel), m_max_depth(max_depth), m_max_paths(max_paths) {}
    // ptxSource is accepted for signature parity and ignored (no PTX JIT).
    void Init(const Scene& scene, const std::string& ptxSource = std::string()) {
        (void)ptxSource;
        std::vector<venu_sphere> recs = scene.records();
        check(venu_scene_create(recs.data(), (uint32_t)recs.size(), nullptr, &m_scene), "venu_scene_create");
        check(venu_renderer_create(m_max_paths, 0, &m_renderer), "venu_renderer_create");
    }
    // Moving spheres (no reference counterpart): the same spheres re-posed;
    // the LBVH is refit and the progressive accumulation restarts.
    void Update(const Scene& scene) {
        std::vector<venu_sphere> recs = scene.records();
        check(venu_scene_update(m_scene, recs.data(), (uint32_t)recs.size(), nullptr), "venu_scene_update");
        m_scene_changed = true;
    }
    // Core/Renderer.h:35-78: one progressive subframe of samples_per_pixel
    // samples (16, the reference's fixed count, by default).
    void Draw(Camera& camera, CUDAOutputBuffer<uchar4>& out) {
        const uint64_t npix = (uint64_t)out.width() * out.height();
        uint32_t flags = 0;
        const bool scene_changed = m_scene_changed;
        m_scene_changed = false;
        if (camera.Changed() || scene_changed || npix != m_accum_pixels) {
            if (m_accum) cudaFree(m_accum);
            cuda_check(cudaMalloc(&m_accum, sizeof(float) * VENU_ACCUM_FLOATS_PER_PIXEL * npix), "accum");
            m_accum_pixels = npix;
            m_subframe = 0;
            flags = VENU_FLAG_RESET_ACCUM;
        }
        ++m_subframe;
        venu_camera cam = camera.frame();
        venu_render_opts o{(uint32_t)out.width(), (uint32_t)out.height(), m_spp, m_subframe, m_max_depth, flags};
        check(venu_render(m_renderer, m_scene, &cam, &o, m_accum, out.floatPixels(),
                          reinterpret_cast<uint8_t*>(out.map()), out.stream()),
              "venu_render");
        out.unmap();
    }
    void Cleanup() {
        if (m_renderer) venu_renderer_destroy(m_renderer);
        if (m_scene) venu_scene_destroy(m_scene);
        if (m_accum) cudaFree(m_accum);
        m_renderer = nullptr;
        m_scene = nullptr;
        m_accum = nullptr;
        m_accum_pixels = 0;
    }
    uint32_t subframe_index() const { return m_subframe; }

   private:
    uint32_t m_spp, m_max_depth, m_max_paths;
    venu_scene* m_scene = nullptr;
    venu_renderer* m_renderer = nullptr;
    float* m_accum = nullptr;
    uint64_t m_accum_pixels = 0;
    uint32_t m_subframe = 0;
    bool m_scene_changed = false;
};

}  // namespace venu_core
