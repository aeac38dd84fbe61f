// selftest.cu -- the device arithmetic that results depend on bit for bit,
// exposed so that it can be compared word for word with the host
// restatement: the TEA-4 seed hash and the LCG of Core/random.cuh:31-67, and
// the sRGB power routine (with CUDA's powf beside it for comparison).
#include "venu_device.cuh"
#include "venu_internal.h"

namespace venu {
namespace {

__global__ void k_selftest_tea(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, uint32_t n,
                               uint32_t* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = tea4(a[i], b[i]);
}

// One thread walks the LCG: the stream is sequential by definition.
__global__ void k_selftest_lcg(uint32_t seed, uint32_t nsteps, float* __restrict__ vals,
                               uint32_t* __restrict__ states) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    uint32_t s = seed;
    for (uint32_t k = 0; k < nsteps; ++k) {
        const float v = rnd(s);
        if (vals) vals[k] = v;
        if (states) states[k] = s;
    }
}

__global__ void k_selftest_pow(const float* __restrict__ x, uint64_t n, uint32_t which, float* __restrict__ out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = which == 0 ? srgb_pow(x[i]) : powf(x[i], 1.0f / 2.4f);
}

}  // namespace
}  // namespace venu

using namespace venu;

extern "C" venu_status venu_selftest_rng(const uint32_t* a_dev, const uint32_t* b_dev, uint32_t n,
                                         uint32_t* tea_out_dev, uint32_t seed, uint32_t nsteps,
                                         float* rnd_out_dev, uint32_t* states_out_dev, void* stream) {
    if ((n && (!a_dev || !b_dev || !tea_out_dev)) || (nsteps && !rnd_out_dev && !states_out_dev)) {
        set_error("venu_selftest_rng: NULL argument");
        return VENU_ERR_INVALID;
    }
    venu_status ds = require_device();
    if (ds != VENU_OK) return ds;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (n) k_selftest_tea<<<(n + 255) / 256, 256, 0, st>>>(a_dev, b_dev, n, tea_out_dev);
    if (nsteps) k_selftest_lcg<<<1, 32, 0, st>>>(seed, nsteps, rnd_out_dev, states_out_dev);
    VENU_CUDA(cudaGetLastError());
    return VENU_OK;
}

extern "C" venu_status venu_selftest_srgb_pow(const float* x_dev, uint64_t n, uint32_t which, float* out_dev,
                                              void* stream) {
    if (n && (!x_dev || !out_dev)) {
        set_error("venu_selftest_srgb_pow: NULL argument");
        return VENU_ERR_INVALID;
    }
    if (which > 1) {
        set_error("venu_selftest_srgb_pow: which must be 0 (library routine) or 1 (powf)");
        return VENU_ERR_INVALID;
    }
    venu_status ds = require_device();
    if (ds != VENU_OK) return ds;
    if (n == 0) return VENU_OK;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    k_selftest_pow<<<sm_count() * 8, 256, 0, st>>>(x_dev, n, which, out_dev);
    VENU_CUDA(cudaGetLastError());
    return VENU_OK;
}
