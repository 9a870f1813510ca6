// Stand-in for the tiny-cuda-nn helpers the hot-path headers call (the submodule is empty).
#pragma once
#include <cstdint>
#include <utility>
// host stand-in for the CUDA stream handle named in interface signatures
typedef struct CUstream_st* cudaStream_t;
namespace tcnn {
template <typename T>
inline T clamp(T val, T lower, T upper) { return val < lower ? lower : (upper < val ? upper : val); }
template <typename T>
inline void host_device_swap(T& a, T& b) { T c(a); a = b; b = c; }
}  // namespace tcnn
namespace tcnn {
// 3-D Morton code of three 10-bit coordinates (x in bit 0, y in bit 1, z in bit 2 of each triple),
// the standard bit-interleaving construction.
inline uint32_t expand_bits_3d(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
inline uint32_t morton3D(uint32_t x, uint32_t y, uint32_t z) { return expand_bits_3d(x) | (expand_bits_3d(y) << 1) | (expand_bits_3d(z) << 2); }
}  // namespace tcnn
