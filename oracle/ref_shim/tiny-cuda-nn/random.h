// Stand-in: the random-number generator type random_val.cuh names (its templates that use it
// are never instantiated by the reference build in oracle/).
#pragma once
#include <cstdint>
namespace tcnn {
struct default_rng_t {
    uint64_t state = 0;
    float next_float() { return 0.f; }
    uint32_t next_uint() { return 0u; }
};
}  // namespace tcnn
