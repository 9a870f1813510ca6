// static_scratch.cu -- working memory for insta_field_eval_static, the one entry point that
// allocates nothing.  Its scratch is a file-scope device array, reserved when a device first
// loads this library and kept until the process exits.
#include <mutex>

#include "device_common.cuh"
#include "mlp_tiles.cuh"
#include "kernels.h"

namespace insta {

// Largest batch insta_field_eval_static accepts, and the scratch it needs: encoded input
// tiles (up to 144 + 16 FP16 columns per sample: 128 hash features, 16 expression dims, SH) plus
// packed FP16 and FP32 network outputs.
constexpr int64_t kStaticMaxSamples = 16384;
constexpr size_t kStaticTileBytes = (size_t)kStaticMaxSamples / 128 * (128 * (144 + 16) * 2);
constexpr size_t kStaticOutBytes = (size_t)kStaticMaxSamples * sizeof(uint2);
constexpr size_t kStaticOutF32Bytes = (size_t)kStaticMaxSamples * sizeof(float4);
constexpr size_t kStaticBytes = kStaticTileBytes + kStaticOutBytes + kStaticOutF32Bytes;

static __device__ __align__(256) uint8_t g_static_scratch[kStaticBytes];

// In host code g_static_scratch names a host-side stand-in, not device memory: the kernels
// get the device address, looked up once per device with that device current.
static std::mutex g_static_mutex;
static void* g_static_ptr[64] = {};

int64_t static_max_samples() { return kStaticMaxSamples; }

cudaError_t static_scratch(int device, uint8_t** tiles, uint2** out, float4** out_f32) {
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_static_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return e;
        g_static_ptr[device] = p;
    }
    uint8_t* base = static_cast<uint8_t*>(g_static_ptr[device]);
    *tiles = base;
    *out = reinterpret_cast<uint2*>(base + kStaticTileBytes);
    *out_f32 = reinterpret_cast<float4*>(base + kStaticTileBytes + kStaticOutBytes);
    return cudaSuccess;
}

}  // namespace insta
