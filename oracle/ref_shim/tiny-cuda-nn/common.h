// Stand-in for the tiny-cuda-nn helpers the hot-path headers call (the submodule is empty).
#pragma once
#include <utility>
// host stand-in for the CUDA stream handle named in interface signatures
typedef struct CUstream_st* cudaStream_t;
namespace tcnn {
template <typename T>
inline T clamp(T val, T lower, T upper) { return val < lower ? lower : (upper < val ? upper : val); }
template <typename T>
inline void host_device_swap(T& a, T& b) { T c(a); a = b; b = c; }
}  // namespace tcnn
