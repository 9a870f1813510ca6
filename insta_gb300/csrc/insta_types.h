// insta_types.h -- plain views of device-resident avatar state, passed to kernels by value.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define INSTA_STACK 48
#define INSTA_MAX_LEVELS 12
#define INSTA_MAX_HASH_LEVELS 32

// device error word bits (read back by the host after each call)
#define INSTA_DEVERR_STACK 0x1u      // BVH traversal stack overflow
#define INSTA_DEVERR_TIMEOUT 0x2u    // a bounded wait on an mbarrier ran out
#define INSTA_DEVERR_NO_TRI 0x4u     // no nearest triangle found (empty mesh)
#define INSTA_DEVERR_MARCH 0x8u      // march iteration guard reached

namespace insta {

struct TriFrame;

// Per-frame deformed mesh: 4-wide LBVH over Morton-ordered triangles.
//   leaf_tris: [n_tris][INSTA_TRI_F4] float4 in Morton order -- (a.xyz, b.x) (b.yz, c.xy)
//              (c.z, id bits, |v21|^2, |v32|^2) (v21, |v13|^2) (v32, |n|^2) (v13, n.x)
//              (v21 x n, n.y) (v32 x n, n.z) (v13 x n, 0): the vertices plus every point-independent
//              term of Triangle::distance_sq, computed with the same operations (same bits)
//   nodes:     [n_nodes][7] float4 -- child boxes SoA (min.x[4] min.y[4] min.z[4] max.x[4] max.y[4]
//              max.z[4]) and the four child references (int bits): >= 0 internal node index,
//              INSTA_LEAF_BIT | (first slot << 3) | count for a leaf, -1 for an empty slot.
//   Node 0 is the root.
#define INSTA_LEAF_BIT 0x40000000
#define INSTA_LEAF_SIZE 4   // triangles per leaf at most (the reference's N_PRIMITIVES_LEAF is 2; see bvh.cuh)
#define INSTA_TRI_F4 9
struct FrameView {
    const float4* leaf_tris;
    // [n_tris][2] float4 per Morton slot, the triangle's bounding disk: (centre, radius), (unit
    // normal, 0) -- every point of the triangle lies in the plane through the centre with that
    // normal, within the radius of the centre (leaf_bound_sq)
    const float4* leaf_bounds;
    const float4* nodes;
    const TriFrame* frames;   // per original triangle, see device_common.cuh
    int n_tris;
    int n_nodes;
};

struct DeformView {
    const TriFrame* canon;    // canonical frame records (original order)
    const int32_t* adjacency; // [F][3]
    int disable_interp;
    float aabb_min[3], aabb_max[3];   // Testbed::m_aabb (the warp kernel's render_bbox)
};

struct FieldView {
    const uint16_t* table;    // hash table, [entries][n_features] FP16
    const uint8_t* mlp_smem;  // pre-laid-out MLP weight image (see umma.cuh)
    uint32_t mlp_smem_bytes;
    uint32_t n_levels, n_features, n_extra;
    float level_scale[INSTA_MAX_HASH_LEVELS];
    uint32_t level_res[INSTA_MAX_HASH_LEVELS];
    uint32_t level_size[INSTA_MAX_HASH_LEVELS];
    uint32_t level_off[INSTA_MAX_HASH_LEVELS];   // in entries
    uint8_t level_dense[INSTA_MAX_HASH_LEVELS];
    int precision;            // 0 fp16, 1 bf16, 2 fp8 e4m3 (weight scales inside the MLP image)
};

struct RenderView {
    int width, height;
    float focal[2];
    float screen_center[2];
    float cam[12];
    float aabb_min[3], aabb_max[3];       // render box
    float train_min[3], train_max[3];     // Testbed::m_aabb
    float cone_angle;
    float min_transmittance;
    uint32_t spp;
    uint32_t max_samples_per_ray;
    int snap_to_pixel_centers;
    int frame_id;
    int linear_colors;
};

}  // namespace insta
