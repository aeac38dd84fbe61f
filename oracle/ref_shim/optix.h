// optix.h -- host-side stand-in for the few OptiX *device* functions that the
// reference's Core/RayTracer.cu calls, so that file can be compiled by g++
// and run on CPU cores as a pinned reference (TEST INFRASTRUCTURE ONLY).
//
// Written from the documented behaviour of the OptiX 8 device API; no OptiX
// header is used.  optixTrace() is a brute-force loop over the scene's
// spheres in index order that calls the reference's own intersection
// program, then its closest-hit or miss program, recursively.  A reported
// intersection is accepted when tmin <= t <= tmax and it is strictly closer
// than the current one (so an exact tie keeps the lower sphere index).
#pragma once

#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#ifndef __global__
#define __global__
#endif
#ifndef __constant__
#define __constant__
#endif

#include <vector_functions.h>
#include <vector_types.h>

#include <cmath>
#include <cstdint>
#include <cstring>

typedef unsigned long long OptixTraversableHandle;
typedef unsigned long long CUdeviceptr_shim;
typedef unsigned int OptixVisibilityMask;
enum { OPTIX_RAY_FLAG_NONE = 0 };

namespace vshim {

struct SphereRec {  // SphereHitGroupData layout (Core/RayTracer.h:40-45)
    float3 center;
    float radius;
    float mat[4];   // MaterialData union
};

struct Launch {
    const SphereRec* recs = nullptr;
    const unsigned* types = nullptr;  // 0 lambertian, 1 metal, 2 dielectric
    unsigned n = 0;
};
extern Launch g_launch;

struct Trace {
    float3 o, d;
    float tmin, tmax;
    unsigned p0, p1;
    bool hit;
    unsigned prim, kind;
    unsigned attr[6];
    unsigned cur_prim;  // primitive whose intersection program runs
    const void* sbt;    // SBT data of the program that runs
};
extern thread_local Trace* g_top;
extern thread_local uint3 g_launch_index;

}  // namespace vshim

inline unsigned int __float_as_uint(float f) {
    unsigned int u;
    std::memcpy(&u, &f, 4);
    return u;
}
inline float __uint_as_float(unsigned int u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
// The device intrinsic is an approximation; the host build uses powf.
inline float __powf(float x, float y) { return std::pow(x, y); }

inline uint3 optixGetLaunchIndex() { return vshim::g_launch_index; }
inline CUdeviceptr_shim optixGetSbtDataPointer() {
    return (CUdeviceptr_shim)(uintptr_t)vshim::g_top->sbt;
}
inline unsigned int optixGetPayload_0() { return vshim::g_top->p0; }
inline unsigned int optixGetPayload_1() { return vshim::g_top->p1; }
inline unsigned int optixGetAttribute_0() { return vshim::g_top->attr[0]; }
inline unsigned int optixGetAttribute_1() { return vshim::g_top->attr[1]; }
inline unsigned int optixGetAttribute_2() { return vshim::g_top->attr[2]; }
inline unsigned int optixGetAttribute_3() { return vshim::g_top->attr[3]; }
inline unsigned int optixGetAttribute_4() { return vshim::g_top->attr[4]; }
inline unsigned int optixGetAttribute_5() { return vshim::g_top->attr[5]; }
inline unsigned int optixGetHitKind() { return vshim::g_top->kind; }
inline int optixGetPrimitiveIndex() { return (int)vshim::g_top->cur_prim; }
inline float3 optixGetWorldRayOrigin() { return vshim::g_top->o; }
inline float3 optixGetWorldRayDirection() { return vshim::g_top->d; }
inline float optixGetRayTmin() { return vshim::g_top->tmin; }
inline float optixGetRayTmax() { return vshim::g_top->tmax; }

inline bool optixReportIntersection(float t, unsigned int kind, unsigned int a0, unsigned int a1,
                                    unsigned int a2, unsigned int a3, unsigned int a4,
                                    unsigned int a5) {
    vshim::Trace* T = vshim::g_top;
    if (!(t >= T->tmin && t <= T->tmax)) return false;
    if (T->hit && !(t < T->tmax)) return false;
    T->hit = true;
    T->tmax = t;
    T->prim = T->cur_prim;
    T->kind = kind;
    T->attr[0] = a0; T->attr[1] = a1; T->attr[2] = a2;
    T->attr[3] = a3; T->attr[4] = a4; T->attr[5] = a5;
    return true;
}

// Provided by the harness after the reference programs are defined.
void optixTrace(OptixTraversableHandle handle, float3 origin, float3 direction, float tmin,
                float tmax, float rayTime, OptixVisibilityMask mask, unsigned int rayFlags,
                unsigned int sbtOffset, unsigned int sbtStride, unsigned int missSbtIndex,
                unsigned int& p0, unsigned int& p1);
