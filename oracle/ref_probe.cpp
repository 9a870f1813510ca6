// ref_probe.cpp -- the reference's own hot-path headers compiled for the host, behind a C ABI,
// so the oracle can be pinned against them.  TEST INFRASTRUCTURE ONLY: built by
// oracle/build_ref.py into oracle/_ref/ (git-ignored) when the INSTA sources are present.
//
// Compiled unmodified from the reference tree (paths relative to the INSTA repository):
//   instant-ngp/include/neural-graphics-primitives/triangle.cuh      Triangle::distance_sq, tbn
//   instant-ngp/include/neural-graphics-primitives/bounding_box.cuh  BoundingBox::distance_sq
//   instant-ngp/include/neural-graphics-primitives/triangle_bvh.cuh  TriangleBvhNode, FixedStack
//   instant-ngp/include/neural-graphics-primitives/bvh.cuh           closest_triangle
//   include/rta/affine.cuh                                           tri2projection,
//                                                                    interpolate_transformation,
//                                                                    transform_point/direction
//   instant-ngp/include/neural-graphics-primitives/random_val.cuh    sobol, ld_random_val,
//                                                                    ld_random_pixel_offset
// against oracle/ref_shim (an Eigen subset and stand-ins for the absent tiny-cuda-nn pieces).
#define __host__
#define __device__
#define __global__
#define __forceinline__ inline
#define __expf expf

#include <array>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <memory>
#include <stack>
#include <vector>

#include <neural-graphics-primitives/triangle.cuh>
#include <neural-graphics-primitives/bounding_box.cuh>
#include <neural-graphics-primitives/triangle_bvh.cuh>
#include <neural-graphics-primitives/bvh.cuh>
#include <rta/affine.cuh>
#include <neural-graphics-primitives/random_val.cuh>

static_assert(sizeof(ngp::Triangle) == 48, "Triangle layout");
static_assert(sizeof(ngp::TriangleBvhNode) == 32, "TriangleBvhNode layout");

static Eigen::Vector3f v3(const float* p) { return Eigen::Vector3f(p[0], p[1], p[2]); }

static void store4(const Eigen::Matrix4f& M, float* out) {
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[r * 4 + c] = M(r, c);
}

extern "C" {

float ref_tri_distance_sq(const ngp::Triangle* t, const float* p) { return t->distance_sq(v3(p)); }

float ref_box_distance_sq(const float* mn, const float* mx, const float* p) {
    ngp::BoundingBox bb(v3(mn), v3(mx));
    return bb.distance_sq(v3(p));
}

void ref_tbn(const ngp::Triangle* t, float* m9) {
    Eigen::Matrix3f m = t->tbn();
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) m9[r * 3 + c] = m(r, c);
}

void ref_tri2projection(const ngp::Triangle* t, const float* p, float* M16) { store4(tri2projection(v3(p), *t), M16); }

void ref_interpolate_transformation(const float* p, const int32_t* adjacency, const ngp::Triangle* tris, uint32_t id, int invert,
                                    float* M16) {
    store4(interpolate_transformation(v3(p), adjacency, tris, tris[id], invert != 0), M16);
}

void ref_transform(const float* p, const float* dir, const float* Mw16, const float* Mc16, float* out_p, float* out_d) {
    Eigen::Matrix4f Mw, Mc;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) { Mw(r, c) = Mw16[r * 4 + c]; Mc(r, c) = Mc16[r * 4 + c]; }
    Eigen::Vector3f x = transform_point(v3(p), Mw, Mc);
    Eigen::Vector3f d = transform_direction(v3(dir), Mw, Mc);
    for (int k = 0; k < 3; ++k) { out_p[k] = x[k]; out_d[k] = d[k]; }
}

int ref_closest_triangle(const ngp::TriangleBvhNode* nodes, const ngp::Triangle* sorted, const float* p, float* dist) {
    auto r = closest_triangle(v3(p), nodes, sorted);
    *dist = r.second;
    return r.first;
}

uint32_t ref_sobol(uint32_t index, uint32_t dim) { return ngp::sobol(index, dim); }

float ref_ld_random_val(uint32_t index, uint32_t seed, uint32_t dim) { return ngp::ld_random_val(index, seed, dim); }

void ref_ld_random_pixel_offset(uint32_t spp, float* out) {
    Eigen::Vector2f o = ngp::ld_random_pixel_offset(spp);
    out[0] = o.x();
    out[1] = o.y();
}

}  // extern "C"
