// Stand-in: GPUMemory as a host vector (only named by TriangleBvh's interface here).
#pragma once
#include <vector>
#include <tiny-cuda-nn/common.h>
namespace tcnn {
template <typename T>
struct GPUMemory {
    std::vector<T> v;
    T* data() const { return const_cast<T*>(v.data()); }
    void free_memory() { v.clear(); }
    void resize_and_copy_from_host(const std::vector<T>& h) { v = h; }
};
}  // namespace tcnn
