// ref_harness.cpp -- builds the reference's own device code
// (Core/RayTracer.cu, Core/random.cuh, Core/vec_math.h, Core/RayTracer.h)
// for the host, in place under the reference checkout, against the OptiX
// device-API stand-in in ref_shim/optix.h.  TEST INFRASTRUCTURE ONLY: the
// resulting oracle/_ref/libvenu_ref.so pins the oracle restatement.
//
// Two host-build details make the result follow the device semantics:
//  * CUDA device code resolves sqrt/fabs on a float argument to the float
//    overloads; `using std::sqrt` etc. gives the host build the same choice.
//  * The reference draws random numbers inside make_float3(...) argument
//    lists (Core/RayTracer.cu:101-105,110-114,145), whose evaluation order
//    C++ leaves unspecified; nvcc device code evaluates them left to right,
//    g++ right to left.  make_float3 is redirected to a braced initializer,
//    which C++ evaluates left to right.
#include "optix.h"

#include <cmath>
using std::fabs;
using std::sqrt;

#include "vec_math.h"
#include "random.cuh"

namespace vshim {
struct lr3 {
    float3 v;
    template <class A, class B, class C>
    lr3(A a, B b, C c) : v(::make_float3((float)a, (float)b, (float)c)) {}
    lr3(float s) : v(::make_float3(s, s, s)) {}
    lr3(double s) : v(::make_float3((float)s, (float)s, (float)s)) {}
    lr3(const float4& q) : v(::make_float3(q.x, q.y, q.z)) {}
};
}  // namespace vshim
#define make_float3(...) (::vshim::lr3{__VA_ARGS__}.v)

#include "RayTracer.cu"

#undef make_float3

#include <atomic>
#include <thread>
#include <vector>

namespace vshim {
Launch g_launch;
thread_local Trace* g_top = nullptr;
thread_local uint3 g_launch_index;
}  // namespace vshim

void optixTrace(OptixTraversableHandle, float3 origin, float3 direction, float tmin, float tmax,
                float, OptixVisibilityMask, unsigned int, unsigned int, unsigned int, unsigned int,
                unsigned int& p0, unsigned int& p1) {
    vshim::Trace T;
    T.o = origin;
    T.d = direction;
    T.tmin = tmin;
    T.tmax = tmax;
    T.p0 = p0;
    T.p1 = p1;
    T.hit = false;
    T.prim = 0;
    T.kind = 0;
    vshim::Trace* saved = vshim::g_top;
    vshim::g_top = &T;
    const vshim::Launch& L = vshim::g_launch;
    for (unsigned i = 0; i < L.n; ++i) {
        T.cur_prim = i;
        T.sbt = &L.recs[i];
        __intersection__hit_sphere();
    }
    if (T.hit) {
        T.sbt = &L.recs[T.prim];
        switch (L.types[T.prim]) {
            case 0: __closesthit__lambertian(); break;
            case 1: __closesthit__metal(); break;
            default: __closesthit__dielectric(); break;
        }
    } else {
        T.sbt = nullptr;
        __miss__ms();
    }
    p0 = T.p0;
    p1 = T.p1;
    vshim::g_top = saved;
}

extern "C" {

typedef struct vr_sphere {  // same layout as venu_sphere / vo_sphere
    float center[3];
    float radius;
    float albedo[3];
    float fuzz;
    float ir;
    uint32_t material;
    uint32_t pad[2];
} vr_sphere;

unsigned vr_tea4(unsigned a, unsigned b) { return tea<4>(a, b); }

void vr_rnd_stream(unsigned seed, unsigned n, float* out, unsigned* states) {
    for (unsigned i = 0; i < n; ++i) {
        out[i] = rnd(seed);
        if (states) states[i] = seed;
    }
}

// Runs __raygen__rg for every pixel of a width x height launch.
// cam = {origin[3], u[3], v[3], w[3], lens_radius}; accum is float4 per pixel
// (read when subframe_index > 0, as Core/RayTracer.cu:208-213 does).
void vr_render(const vr_sphere* s, unsigned ns, const float* cam, unsigned width, unsigned height,
               unsigned spp, unsigned subframe_index, float* accum, unsigned char* image,
               unsigned nthreads) {
    std::vector<vshim::SphereRec> recs(ns);
    std::vector<unsigned> types(ns);
    for (unsigned i = 0; i < ns; ++i) {
        recs[i].center = ::make_float3(s[i].center[0], s[i].center[1], s[i].center[2]);
        recs[i].radius = s[i].radius;
        std::memset(recs[i].mat, 0, sizeof(recs[i].mat));
        types[i] = s[i].material;
        // Renderer::CreateSBT (Core/Renderer.h:487-503)
        if (s[i].material == 0) {
            recs[i].mat[0] = s[i].albedo[0]; recs[i].mat[1] = s[i].albedo[1]; recs[i].mat[2] = s[i].albedo[2];
        } else if (s[i].material == 1) {
            recs[i].mat[0] = s[i].albedo[0]; recs[i].mat[1] = s[i].albedo[1]; recs[i].mat[2] = s[i].albedo[2];
            recs[i].mat[3] = s[i].fuzz;
        } else {
            recs[i].mat[0] = s[i].ir;
        }
    }
    static_assert(sizeof(vshim::SphereRec) == sizeof(SphereHitGroupData), "record layout");
    vshim::g_launch.recs = recs.data();
    vshim::g_launch.types = types.data();
    vshim::g_launch.n = ns;
    params.image = reinterpret_cast<uchar4*>(image);
    params.accum = reinterpret_cast<float4*>(accum);
    params.width = width;
    params.height = height;
    params.samples_per_pixel = spp;
    params.subframe_index = subframe_index;
    params.origin = ::make_float3(cam[0], cam[1], cam[2]);
    params.u = ::make_float3(cam[3], cam[4], cam[5]);
    params.v = ::make_float3(cam[6], cam[7], cam[8]);
    params.w = ::make_float3(cam[9], cam[10], cam[11]);
    params.lens_radius = cam[12];
    params.handle = 0;
    unsigned nt = nthreads ? nthreads : std::max(1u, std::thread::hardware_concurrency());
    std::atomic<unsigned> next{0};
    auto worker = [&]() {
        for (;;) {
            unsigned y = next.fetch_add(1);
            if (y >= height) break;
            for (unsigned x = 0; x < width; ++x) {
                vshim::g_launch_index = ::make_uint3(x, y, 0);
                __raygen__rg();
            }
        }
    };
    std::vector<std::thread> th;
    for (unsigned i = 1; i < nt; ++i) th.emplace_back(worker);
    worker();
    for (auto& t : th) t.join();
}

}  // extern "C"
