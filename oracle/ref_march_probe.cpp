// ref_march_probe.cpp -- the reference's march helpers compiled for the host, behind a C ABI, so
// the oracle's march can be pinned against them.  TEST INFRASTRUCTURE ONLY: built by
// oracle/build_ref.py into oracle/_ref/ (git-ignored) when the INSTA sources are present.
//
// instant-ngp/src/testbed_nerf.cu is a CUDA translation unit full of kernels and cannot be compiled
// for the host whole; oracle/build_ref.py takes the text of its march helpers from the reference
// file at build time (NERF_* step constants :48-56, grid_mip_offset :78-80, calc_cone_angle
// :82-89, calc_dt :91-93, distance_to_next_voxel / advance_to_next_voxel :186-208,
// warp_dt / unwarp_dt :300-311, cascaded_grid_idx_at / density_grid_occupied_at :313-337,
// mip_from_pos / mip_from_dt :471-485) into oracle/_ref/march_helpers.inc, included here
// unmodified.  NERF_GRIDSIZE comes from the reference's nerf.h.
#define __host__
#define __device__
#define __global__
#define __forceinline__ inline

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>

#include <neural-graphics-primitives/common.h>
#include <neural-graphics-primitives/nerf.h>

// CUDA's integer min/max overloads for mixed signedness (min(unsigned int, int) compares as
// unsigned), which the device code relies on; float min through std.
static inline uint32_t min(uint32_t a, int b) { return std::min(a, (uint32_t)b); }
static inline int max(int a, int b) { return std::max(a, b); }
static inline float min(float a, float b) { return fminf(a, b); }

namespace ngp {
using namespace Eigen;
using ::min;
using ::max;
#include "march_helpers.inc"
}  // namespace ngp

static Eigen::Vector3f v3(const float* p) { return Eigen::Vector3f(p[0], p[1], p[2]); }

extern "C" {

float ref_calc_dt(float t, float cone_angle) { return ngp::calc_dt(t, cone_angle); }

float ref_calc_cone_angle(float cosine, float fx, float fy, float cone_angle_constant) {
    return ngp::calc_cone_angle(cosine, Eigen::Vector2f(fx, fy), cone_angle_constant);
}

float ref_warp_dt(float dt) { return ngp::warp_dt(dt); }
float ref_unwarp_dt(float dt) { return ngp::unwarp_dt(dt); }

int ref_mip_from_pos(const float* pos) { return ngp::mip_from_pos(v3(pos)); }
int ref_mip_from_dt(float dt, const float* pos) { return ngp::mip_from_dt(dt, v3(pos)); }

uint32_t ref_cascaded_grid_idx_at(const float* pos, uint32_t mip) { return ngp::cascaded_grid_idx_at(v3(pos), mip); }
int ref_density_grid_occupied_at(const float* pos, const uint8_t* bitfield, uint32_t mip) {
    return ngp::density_grid_occupied_at(v3(pos), bitfield, mip) ? 1 : 0;
}

float ref_distance_to_next_voxel(const float* pos, const float* dir, const float* idir, uint32_t res) {
    return ngp::distance_to_next_voxel(v3(pos), v3(dir), v3(idir), res);
}
float ref_advance_to_next_voxel(float t, float cone_angle, const float* pos, const float* dir, const float* idir, uint32_t res) {
    return ngp::advance_to_next_voxel(t, cone_angle, v3(pos), v3(dir), v3(idir), res);
}

}  // extern "C"
