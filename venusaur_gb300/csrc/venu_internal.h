// venu_internal.h -- host-side internals shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/venu.h"

namespace venu {

void set_error(const std::string& msg);
venu_status cuda_fail(cudaError_t e, const char* what);

#define VENU_CUDA(call)                                          \
    do {                                                         \
        cudaError_t _e = (call);                                 \
        if (_e != cudaSuccess) return ::venu::cuda_fail(_e, #call); \
    } while (0)

venu_status require_device();  // sm_103 device present and kernels loadable
int sm_count();

// Shared-memory carveout preference: just what `per_sm` resident blocks of
// `kernel` need (static + dynamic + the 1 KB the system reserves per block),
// so that the rest of the SM's unified memory is L1 (the node records and
// spheres stay in L1 longer: RTIOW 1080p x 256 +0.5 %, the batch engine on
// the 64-scene mix +0.3 %).
template <typename K>
cudaError_t prefer_l1(K kernel, int per_sm, size_t dyn) {
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    int dev = 0, maxsm = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess) return e;
    const size_t need = (size_t)(per_sm > 1 ? per_sm : 1) * (fa.sharedSizeBytes + dyn + 1024);
    const size_t pct = (need * 100 + (size_t)maxsm - 1) / (size_t)maxsm + 1;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, (int)(pct < 100 ? pct : 100));
}

}  // namespace venu

struct venu_scene {
    uint32_t n = 0;
    float4* nodes = nullptr;   // 2 per internal node
    float4* trav = nullptr;    // 4 per internal node: both children (traversal layout)
    float4* sph = nullptr;     // slot order
    float4* mat = nullptr;
    uint32_t* meta = nullptr;  // original id | material << 30
    uint32_t* keys = nullptr;  // sorted Morton codes
    int32_t* parents = nullptr;  // [n-1] parent of each internal node, then [n] of each leaf (for refits)
    // The 4-wide traversal tree (lbvh.cu), built on first use by a render
    // with traversal variant 4 or 5 (ensure_wide); a cache of the binary
    // tree, so it may be filled in through a const scene.
    mutable float4* wide = nullptr;      // kWideF4 float4 per wide node
    mutable int32_t* wide_src = nullptr; // kWideChildren per wide node: binary word of each child (for refits)
    mutable uint32_t nwide = 0;
    mutable float wide_ms = 0.0f;        // wall time of the wide tree's collapse
    mutable std::mutex wide_mu;          // serialises that first build
    float bounds[6] = {0, 0, 0, 0, 0, 0};
    uint32_t nhoist = 0;          // huge spheres tested before traversal
    int32_t hoist[4] = {0, 0, 0, 0};
    float build_ms = 0.0f;
    mutable uint64_t bytes = 0;   // device bytes held (grows when the wide tree is built)
};

namespace venu {
// Builds the LBVH for `n` device spheres into `s` (allocates its buffers).
venu_status build_scene(const venu_sphere* spheres_dev, uint32_t n, cudaStream_t stream, venu_scene* s);
void free_scene(venu_scene* s);
// Moves the scene's spheres to `spheres_dev` (same count, original order) and
// refits the boxes on `stream` (asynchronous).
venu_status update_scene(venu_scene* s, const venu_sphere* spheres_dev, cudaStream_t stream);
// Builds the scene's 4-wide tree on `stream` unless it exists (blocking: the
// collapse reads each level's size on the host).  Thread-safe.
venu_status ensure_wide(const venu_scene* s, cudaStream_t stream);
}  // namespace venu
