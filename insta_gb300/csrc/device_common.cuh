// device_common.cuh -- per-sample device routines of the INSTA hot path on sm_103a.
//
// Geometry that decides the nearest-triangle index (squared point-triangle and
// point-box distances) is written with explicit round-to-nearest intrinsics so
// no multiply-add is contracted: the index is bit-exact against the host
// restatement (which is compiled with -ffp-contract=off) and follows the
// reference's expression order (Eigen's 3-term reduction x0 + (x1 + x2)).
#pragma once

#include <cstdint>
#include <cstring>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include "insta_types.h"

namespace insta {

// ---------------------------------------------------------------- vector helpers
struct V3 { float x, y, z; };

__device__ __forceinline__ V3 v3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ V3 sub_rn(V3 a, V3 b) { return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }
__device__ __forceinline__ float dot_rn(V3 a, V3 b) {
    return __fadd_rn(__fmul_rn(a.x, b.x), __fadd_rn(__fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)));
}
__device__ __forceinline__ V3 cross_rn(V3 a, V3 b) {
    return {__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
            __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
            __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x))};
}
// Eigen normalized(): v / sqrt(|v|^2), unchanged for a zero vector.
__device__ __forceinline__ V3 normalize_rn(V3 v) {
    float z = dot_rn(v, v);
    if (z > 0.f) {
        float s = __fsqrt_rn(z);
        return {__fdiv_rn(v.x, s), __fdiv_rn(v.y, s), __fdiv_rn(v.z, s)};
    }
    return v;
}
__device__ __forceinline__ float sign_f(float x) { return copysignf(1.0f, x); }
__device__ __forceinline__ float clamp01_like(float v, float lo, float hi) { return v < lo ? lo : (hi < v ? hi : v); }

// ----------------------------------------------------- exact point-triangle distance
// Triangle::distance_sq (NGP/triangle.cuh:88-107), identical operation order.
__device__ __forceinline__ float tri_distance_sq(V3 a, V3 b, V3 c, V3 pos) {
    V3 v21 = sub_rn(b, a), p1 = sub_rn(pos, a);
    V3 v32 = sub_rn(c, b), p2 = sub_rn(pos, b);
    V3 v13 = sub_rn(a, c), p3 = sub_rn(pos, c);
    V3 nor = cross_rn(v21, v13);
    float s1 = sign_f(dot_rn(cross_rn(v21, nor), p1));
    float s2 = sign_f(dot_rn(cross_rn(v32, nor), p2));
    float s3 = sign_f(dot_rn(cross_rn(v13, nor), p3));
    float s = __fadd_rn(__fadd_rn(s1, s2), s3);
    if (s < 2.0f) {
        float f1 = clamp01_like(__fdiv_rn(dot_rn(v21, p1), dot_rn(v21, v21)), 0.f, 1.f);
        float f2 = clamp01_like(__fdiv_rn(dot_rn(v32, p2), dot_rn(v32, v32)), 0.f, 1.f);
        float f3 = clamp01_like(__fdiv_rn(dot_rn(v13, p3), dot_rn(v13, v13)), 0.f, 1.f);
        V3 e1 = {__fsub_rn(__fmul_rn(v21.x, f1), p1.x), __fsub_rn(__fmul_rn(v21.y, f1), p1.y), __fsub_rn(__fmul_rn(v21.z, f1), p1.z)};
        V3 e2 = {__fsub_rn(__fmul_rn(v32.x, f2), p2.x), __fsub_rn(__fmul_rn(v32.y, f2), p2.y), __fsub_rn(__fmul_rn(v32.z, f2), p2.z)};
        V3 e3 = {__fsub_rn(__fmul_rn(v13.x, f3), p3.x), __fsub_rn(__fmul_rn(v13.y, f3), p3.y), __fsub_rn(__fmul_rn(v13.z, f3), p3.z)};
        float d1 = dot_rn(e1, e1), d2 = dot_rn(e2, e2), d3 = dot_rn(e3, e3);
        float m = d1;
        if (d2 < m) m = d2;
        if (d3 < m) m = d3;
        return m;
    }
    float nd = dot_rn(nor, p1);
    return __fdiv_rn(__fmul_rn(nd, nd), dot_rn(nor, nor));
}

// Point-independent terms of tri_distance_sq for one triangle, written as INSTA_TRI_F4 float4.
__device__ __forceinline__ void tri_record(V3 a, V3 b, V3 c, uint32_t id, float4* dst) {
    const V3 v21 = sub_rn(b, a), v32 = sub_rn(c, b), v13 = sub_rn(a, c);
    const V3 nor = cross_rn(v21, v13);
    const V3 c1 = cross_rn(v21, nor), c2 = cross_rn(v32, nor), c3 = cross_rn(v13, nor);
    dst[0] = make_float4(a.x, a.y, a.z, b.x);
    dst[1] = make_float4(b.y, b.z, c.x, c.y);
    dst[2] = make_float4(c.z, __uint_as_float(id), dot_rn(v21, v21), dot_rn(v32, v32));
    dst[3] = make_float4(v21.x, v21.y, v21.z, dot_rn(v13, v13));
    dst[4] = make_float4(v32.x, v32.y, v32.z, dot_rn(nor, nor));
    dst[5] = make_float4(v13.x, v13.y, v13.z, nor.x);
    dst[6] = make_float4(c1.x, c1.y, c1.z, nor.y);
    dst[7] = make_float4(c2.x, c2.y, c2.z, nor.z);
    dst[8] = make_float4(c3.x, c3.y, c3.z, 0.f);
}

// The bounding disk of a triangle (FrameView::leaf_bounds), in FP64: centre = centroid, radius =
// the largest vertex distance from it, widened by 2^-16 relative + 2e-7 absolute so that the FP32
// centre and radius still enclose every vertex, with the rounding of p - centre in FP32 (below
// 1e-7 for coordinates of order one) to spare; unit normal of (b - a) x (c - a), zero for a
// degenerate triangle (the disk is then the sphere of the same radius).
__device__ __forceinline__ void tri_bound(const float* A, const float* B, const float* C, float4* dst) {
    double c[3], n[3], r2 = 0.0;
    for (int k = 0; k < 3; ++k) c[k] = ((double)A[k] + (double)B[k] + (double)C[k]) / 3.0;
    const float* v[3] = {A, B, C};
    for (int i = 0; i < 3; ++i) {
        double d2 = 0.0;
        for (int k = 0; k < 3; ++k) d2 += ((double)v[i][k] - c[k]) * ((double)v[i][k] - c[k]);
        r2 = fmax(r2, d2);
    }
    const double e1[3] = {(double)B[0] - A[0], (double)B[1] - A[1], (double)B[2] - A[2]};
    const double e2[3] = {(double)C[0] - A[0], (double)C[1] - A[1], (double)C[2] - A[2]};
    n[0] = e1[1] * e2[2] - e1[2] * e2[1];
    n[1] = e1[2] * e2[0] - e1[0] * e2[2];
    n[2] = e1[0] * e2[1] - e1[1] * e2[0];
    const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    const double inv = nn > 0.0 ? 1.0 / nn : 0.0;
    const double r = sqrt(r2) * (1.0 + 1.0 / 65536.0) + 2e-7;
    dst[0] = make_float4((float)c[0], (float)c[1], (float)c[2], (float)r);
    dst[1] = make_float4((float)(n[0] * inv), (float)(n[1] * inv), (float)(n[2] * inv), 0.f);
}

// A lower bound on the squared distance from p to the triangle of a leaf_bounds entry: with
// v = p - centre, h = n.v the signed distance to the triangle's plane and l = |v - h n| the
// distance of p's projection from the centre, the triangle lies within the disk of the radius
// around the centre, so d^2 >= h^2 + max(l - radius, 0)^2.  In FP32: |h| is reduced by 2e-7
// (the rounding of v and of the stored normal, for coordinates of order one and distances below
// 0.1), the radius carries its own margin, and the result is shrunk by 2^-12 relative, which
// covers the rounding of l where the radius matters (l >= radius, millimetres); so the bound
// stays below the exact squared distance, and a triangle it skips (bound > prune limit) cannot
// reach the running minimum.
__device__ __forceinline__ float leaf_bound_sq(const float4* b, V3 p) {
    const float4 b0 = __ldg(b), b1 = __ldg(b + 1);
    const float vx = p.x - b0.x, vy = p.y - b0.y, vz = p.z - b0.z;
    const float h = fmaf(b1.x, vx, fmaf(b1.y, vy, b1.z * vz));
    const float vv = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
    const float l = sqrtf(fmaxf(fmaf(-h, h, vv), 0.f));
    const float ex = fmaxf(l - b0.w, 0.f);
    const float hs = fmaxf(fabsf(h) - 2e-7f, 0.f);
    return fmaf(hs, hs, ex * ex) * (1.0f - 1.0f / 4096.0f);
}

// tri_distance_sq from a precomputed record: only the point-dependent operations remain, in the
// same order, so the result is bit-identical.
__device__ __forceinline__ float tri_distance_rec(const float4* tr, V3 pos, int32_t& id) {
    const float4 q0 = __ldg(tr), q1 = __ldg(tr + 1), q2 = __ldg(tr + 2), q3 = __ldg(tr + 3), q4 = __ldg(tr + 4);
    const float4 q5 = __ldg(tr + 5), q6 = __ldg(tr + 6), q7 = __ldg(tr + 7), q8 = __ldg(tr + 8);
    id = __float_as_int(q2.y);
    const V3 p1 = sub_rn(pos, v3(q0.x, q0.y, q0.z)), p2 = sub_rn(pos, v3(q0.w, q1.x, q1.y)), p3 = sub_rn(pos, v3(q1.z, q1.w, q2.x));
    const V3 v21 = v3(q3.x, q3.y, q3.z), v32 = v3(q4.x, q4.y, q4.z), v13 = v3(q5.x, q5.y, q5.z);
    const V3 nor = v3(q5.w, q6.w, q7.w);
    const float s1 = sign_f(dot_rn(v3(q6.x, q6.y, q6.z), p1));
    const float s2 = sign_f(dot_rn(v3(q7.x, q7.y, q7.z), p2));
    const float s3 = sign_f(dot_rn(v3(q8.x, q8.y, q8.z), p3));
    const float s = __fadd_rn(__fadd_rn(s1, s2), s3);
    if (s < 2.0f) {
        float f1 = clamp01_like(__fdiv_rn(dot_rn(v21, p1), q2.z), 0.f, 1.f);
        float f2 = clamp01_like(__fdiv_rn(dot_rn(v32, p2), q2.w), 0.f, 1.f);
        float f3 = clamp01_like(__fdiv_rn(dot_rn(v13, p3), q3.w), 0.f, 1.f);
        V3 e1 = {__fsub_rn(__fmul_rn(v21.x, f1), p1.x), __fsub_rn(__fmul_rn(v21.y, f1), p1.y), __fsub_rn(__fmul_rn(v21.z, f1), p1.z)};
        V3 e2 = {__fsub_rn(__fmul_rn(v32.x, f2), p2.x), __fsub_rn(__fmul_rn(v32.y, f2), p2.y), __fsub_rn(__fmul_rn(v32.z, f2), p2.z)};
        V3 e3 = {__fsub_rn(__fmul_rn(v13.x, f3), p3.x), __fsub_rn(__fmul_rn(v13.y, f3), p3.y), __fsub_rn(__fmul_rn(v13.z, f3), p3.z)};
        float d1 = dot_rn(e1, e1), d2 = dot_rn(e2, e2), d3 = dot_rn(e3, e3);
        float m = d1;
        if (d2 < m) m = d2;
        if (d3 < m) m = d3;
        return m;
    }
    const float nd = dot_rn(nor, p1);
    return __fdiv_rn(__fmul_rn(nd, nd), q4.w);
}


// PCG32 (O'Neill's permuted congruential generator with 64-bit state, XSH-RR output), the
// pcg32 class tiny-cuda-nn uses as default_rng_t, restated from the published algorithm:
// LCG step with multiplier 6364136223846793005 and odd increment, output of the old state,
// floats from the top 23 bits, and the logarithmic-time jump ahead.
struct Pcg32 {
    uint64_t state, inc;
    __host__ __device__ uint32_t next_uint() {
        const uint64_t old = state;
        state = old * 0x5851f42d4c957f2dull + inc;
        const uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((~rot + 1u) & 31u));
    }
    __host__ __device__ float next_float() {
        const uint32_t bits = (next_uint() >> 9) | 0x3f800000u;
        float f;
        memcpy(&f, &bits, 4);
        return f - 1.0f;
    }
    __host__ __device__ void advance(int64_t delta_) {
        uint64_t cur_mult = 0x5851f42d4c957f2dull, cur_plus = inc, acc_mult = 1u, acc_plus = 0u;
        uint64_t delta = (uint64_t)delta_;
        while (delta > 0) {
            if (delta & 1) {
                acc_mult *= cur_mult;
                acc_plus = acc_plus * cur_mult + cur_plus;
            }
            cur_plus = (cur_mult + 1) * cur_plus;
            cur_mult *= cur_mult;
            delta /= 2;
        }
        state = acc_mult * state + acc_plus;
    }
};

}  // namespace insta

#include "bvh.cuh"

namespace insta {

// ------------------------------------------------------------------ frame math
// 4-term row product with the halving order (x0 + x1) + (x2 + x3).
__device__ __forceinline__ float row4_rn(float m0, float m1, float m2, float m3, float v0, float v1, float v2, float v3) {
    return __fadd_rn(__fadd_rn(__fmul_rn(m0, v0), __fmul_rn(m1, v1)), __fadd_rn(__fmul_rn(m2, v2), __fmul_rn(m3, v3)));
}

// General 4x4 inverse by 2x2 sub-determinant expansion (row-major).  Returns false when singular.
__device__ __forceinline__ bool inverse4(const float* m, float* o) {
    float s0 = __fsub_rn(__fmul_rn(m[0], m[5]), __fmul_rn(m[4], m[1]));
    float s1 = __fsub_rn(__fmul_rn(m[0], m[6]), __fmul_rn(m[4], m[2]));
    float s2 = __fsub_rn(__fmul_rn(m[0], m[7]), __fmul_rn(m[4], m[3]));
    float s3 = __fsub_rn(__fmul_rn(m[1], m[6]), __fmul_rn(m[5], m[2]));
    float s4 = __fsub_rn(__fmul_rn(m[1], m[7]), __fmul_rn(m[5], m[3]));
    float s5 = __fsub_rn(__fmul_rn(m[2], m[7]), __fmul_rn(m[6], m[3]));
    float c5 = __fsub_rn(__fmul_rn(m[10], m[15]), __fmul_rn(m[14], m[11]));
    float c4 = __fsub_rn(__fmul_rn(m[9], m[15]), __fmul_rn(m[13], m[11]));
    float c3 = __fsub_rn(__fmul_rn(m[9], m[14]), __fmul_rn(m[13], m[10]));
    float c2 = __fsub_rn(__fmul_rn(m[8], m[15]), __fmul_rn(m[12], m[11]));
    float c1 = __fsub_rn(__fmul_rn(m[8], m[14]), __fmul_rn(m[12], m[10]));
    float c0 = __fsub_rn(__fmul_rn(m[8], m[13]), __fmul_rn(m[12], m[9]));
    // det = s0*c5 - s1*c4 + s2*c3 + s3*c2 - s4*c1 + s5*c0, evaluated left to right
    float det = __fadd_rn(__fsub_rn(__fadd_rn(__fadd_rn(__fsub_rn(__fmul_rn(s0, c5), __fmul_rn(s1, c4)), __fmul_rn(s2, c3)), __fmul_rn(s3, c2)), __fmul_rn(s4, c1)), __fmul_rn(s5, c0));
    if (det == 0.f) return false;
    float id = __fdiv_rn(1.f, det);
#define T3(a, b, c) __fmul_rn(__fadd_rn(__fsub_rn((a), (b)), (c)), id)
    o[0] = T3(__fmul_rn(m[5], c5), __fmul_rn(m[6], c4), __fmul_rn(m[7], c3));
    o[1] = T3(__fmul_rn(-m[1], c5), -__fmul_rn(m[2], c4), -__fmul_rn(m[3], c3));
    o[2] = T3(__fmul_rn(m[13], s5), __fmul_rn(m[14], s4), __fmul_rn(m[15], s3));
    o[3] = T3(__fmul_rn(-m[9], s5), -__fmul_rn(m[10], s4), -__fmul_rn(m[11], s3));
    o[4] = T3(__fmul_rn(-m[4], c5), -__fmul_rn(m[6], c2), -__fmul_rn(m[7], c1));
    o[5] = T3(__fmul_rn(m[0], c5), __fmul_rn(m[2], c2), __fmul_rn(m[3], c1));
    o[6] = T3(__fmul_rn(-m[12], s5), -__fmul_rn(m[14], s2), -__fmul_rn(m[15], s1));
    o[7] = T3(__fmul_rn(m[8], s5), __fmul_rn(m[10], s2), __fmul_rn(m[11], s1));
    o[8] = T3(__fmul_rn(m[4], c4), __fmul_rn(m[5], c2), __fmul_rn(m[7], c0));
    o[9] = T3(__fmul_rn(-m[0], c4), -__fmul_rn(m[1], c2), -__fmul_rn(m[3], c0));
    o[10] = T3(__fmul_rn(m[12], s4), __fmul_rn(m[13], s2), __fmul_rn(m[15], s0));
    o[11] = T3(__fmul_rn(-m[8], s4), -__fmul_rn(m[9], s2), -__fmul_rn(m[11], s0));
    o[12] = T3(__fmul_rn(-m[4], c3), -__fmul_rn(m[5], c1), -__fmul_rn(m[6], c0));
    o[13] = T3(__fmul_rn(m[0], c3), __fmul_rn(m[1], c1), __fmul_rn(m[2], c0));
    o[14] = T3(__fmul_rn(-m[12], s3), -__fmul_rn(m[13], s1), -__fmul_rn(m[14], s0));
    o[15] = T3(__fmul_rn(m[8], s3), __fmul_rn(m[9], s1), __fmul_rn(m[10], s0));
#undef T3
    return true;
}

// Per-triangle frame record (128 B, original triangle order):
//   r[0..2]  rows of tri2projection: [tbn * (mask==1 ? scaling : 1) | a]   (include/rta/affine.cuh:26-39)
//   r[3..6]  rows of its 4x4 inverse (deformed frames only)
//   r[7]     centroid xyz, mask id (bits)
struct TriFrame { float4 r[8]; };

__device__ __forceinline__ V3 load_centroid(const TriFrame* f, uint32_t id, uint32_t* mask) {
    float4 c = __ldg(&f[id].r[7]);
    if (mask) *mask = __float_as_uint(c.w);
    return v3(c.x, c.y, c.z);
}

// interpolate_transformation (include/rta/affine.cuh:45-100) on precomputed projections:
// M = sum_i w_i P_i with w = exp(-4|c_i - p|) (neighbours) and exp(-|c - p|) (self), normalised.
__device__ __forceinline__ void blend_projection(const TriFrame* frames, const int32_t* adj, uint32_t id, V3 p, float* M) {
    int32_t nb[3];
    nb[0] = __ldg(adj + id * 3 + 0); nb[1] = __ldg(adj + id * 3 + 1); nb[2] = __ldg(adj + id * 3 + 2);
    float a[4];
    float sum = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        a[i] = 0.f;
        if (nb[i] >= 0) {
            V3 c = load_centroid(frames, (uint32_t)nb[i], nullptr);
            V3 d = sub_rn(c, p);
            a[i] = expf(__fmul_rn(-4.f, __fsqrt_rn(dot_rn(d, d))));
            sum = __fadd_rn(sum, a[i]);
        }
    }
    {
        V3 c = load_centroid(frames, id, nullptr);
        V3 d = sub_rn(c, p);
        a[3] = expf(__fmul_rn(-1.f, __fsqrt_rn(dot_rn(d, d))));
        sum = __fadd_rn(sum, a[3]);
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) M[k] = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        uint32_t t = i < 3 ? (uint32_t)nb[i] : id;
        if (i < 3 && nb[i] < 0) continue;
        float w = __fdiv_rn(a[i], sum);
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            float4 q = __ldg(&frames[t].r[r]);
            M[r * 4 + 0] = __fadd_rn(__fmul_rn(w, q.x), M[r * 4 + 0]);
            M[r * 4 + 1] = __fadd_rn(__fmul_rn(w, q.y), M[r * 4 + 1]);
            M[r * 4 + 2] = __fadd_rn(__fmul_rn(w, q.z), M[r * 4 + 2]);
            M[r * 4 + 3] = __fadd_rn(__fmul_rn(w, q.w), M[r * 4 + 3]);
        }
        M[15] = __fadd_rn(__fmul_rn(w, 1.f), M[15]);
        M[12] = __fadd_rn(__fmul_rn(w, 0.f), M[12]);
        M[13] = __fadd_rn(__fmul_rn(w, 0.f), M[13]);
        M[14] = __fadd_rn(__fmul_rn(w, 0.f), M[14]);
    }
}

// The deformed->canonical map of the `warp` kernel (src/core.cu:487-513) for the nearest
// triangle `id`: canonical position and (optionally) canonical warped direction.
__device__ __forceinline__ void map_to_canonical(const DeformView& dv, const TriFrame* def, uint32_t id, V3 p,
                                                 const float* dir_w, float* out_pos, float* out_dir_w, uint32_t* out_mask) {
    uint32_t mask;
    load_centroid(def, id, &mask);
    float Mw[16], Mc[16];
    if (mask == 2u && !dv.disable_interp) {
        float Mb[16];
        blend_projection(def, dv.adjacency, id, p, Mb);
        if (!inverse4(Mb, Mw)) {
#pragma unroll
            for (int k = 0; k < 16; ++k) Mw[k] = (k % 5 == 0) ? 1.f : 0.f;
        }
        blend_projection(dv.canon, dv.adjacency, id, p, Mc);
    } else {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            float4 q = __ldg(&def[id].r[3 + r]);
            Mw[r * 4 + 0] = q.x; Mw[r * 4 + 1] = q.y; Mw[r * 4 + 2] = q.z; Mw[r * 4 + 3] = q.w;
        }
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            float4 q = __ldg(&dv.canon[id].r[r]);
            Mc[r * 4 + 0] = q.x; Mc[r * 4 + 1] = q.y; Mc[r * 4 + 2] = q.z; Mc[r * 4 + 3] = q.w;
        }
        Mc[12] = 0.f; Mc[13] = 0.f; Mc[14] = 0.f; Mc[15] = 1.f;
    }
    // transform_point (include/rta/affine.cuh:102-108)
    float l[4], o[3];
#pragma unroll
    for (int r = 0; r < 4; ++r) l[r] = row4_rn(Mw[r * 4], Mw[r * 4 + 1], Mw[r * 4 + 2], Mw[r * 4 + 3], p.x, p.y, p.z, 1.f);
#pragma unroll
    for (int r = 0; r < 3; ++r) o[r] = row4_rn(Mc[r * 4], Mc[r * 4 + 1], Mc[r * 4 + 2], Mc[r * 4 + 3], l[0], l[1], l[2], l[3]);
    out_pos[0] = o[0]; out_pos[1] = o[1]; out_pos[2] = o[2];
    if (dir_w) {
        // unwarp_direction, transform_direction, warp_direction (src/core.cu:62-68, affine.cuh:110-116)
        V3 dd = v3(__fsub_rn(__fmul_rn(dir_w[0], 2.f), 1.f), __fsub_rn(__fmul_rn(dir_w[1], 2.f), 1.f), __fsub_rn(__fmul_rn(dir_w[2], 2.f), 1.f));
        V3 ld = v3(dot_rn(v3(Mw[0], Mw[1], Mw[2]), dd), dot_rn(v3(Mw[4], Mw[5], Mw[6]), dd), dot_rn(v3(Mw[8], Mw[9], Mw[10]), dd));
        V3 cd = v3(dot_rn(v3(Mc[0], Mc[1], Mc[2]), ld), dot_rn(v3(Mc[4], Mc[5], Mc[6]), ld), dot_rn(v3(Mc[8], Mc[9], Mc[10]), ld));
        cd = normalize_rn(cd);
        out_dir_w[0] = __fmul_rn(__fadd_rn(cd.x, 1.f), 0.5f);
        out_dir_w[1] = __fmul_rn(__fadd_rn(cd.y, 1.f), 0.5f);
        out_dir_w[2] = __fmul_rn(__fadd_rn(cd.z, 1.f), 0.5f);
    }
    if (out_mask) *out_mask = mask;
}

// ------------------------------------------------------------------- march
// Constants and helpers of ngp/src/testbed_nerf.cu:48-93,186-208,303-337,471-485.
constexpr float SQRT3F = 1.73205080757f;
constexpr float MIN_CONE = SQRT3F / 1024.0f;
constexpr float MAX_CONE = MIN_CONE * 128.0f * 1024.0f / 128.0f;
constexpr uint32_t GRID = 128u;
constexpr uint32_t GRID3 = GRID * GRID * GRID;

__device__ __forceinline__ float calc_dt(float t, float cone) { return clamp01_like(__fmul_rn(t, cone), MIN_CONE, MAX_CONE); }
__device__ __forceinline__ float warp_dt(float dt) {
    const float mx = MIN_CONE * 128.0f;
    return __fdiv_rn(__fsub_rn(dt, MIN_CONE), __fsub_rn(mx, MIN_CONE));
}
__device__ __forceinline__ float unwarp_dt(float dt) {
    const float mx = MIN_CONE * 128.0f;
    return __fadd_rn(__fmul_rn(dt, __fsub_rn(mx, MIN_CONE)), MIN_CONE);
}
__device__ __forceinline__ int mip_from_pos(V3 p) {
    float m = fabsf(__fsub_rn(p.x, 0.5f));
    float a1 = fabsf(__fsub_rn(p.y, 0.5f)), a2 = fabsf(__fsub_rn(p.z, 0.5f));
    if (a1 > m) m = a1;
    if (a2 > m) m = a2;
    int e; frexpf(m, &e);
    int v = max(0, e + 1);
    return min(6, v);
}
__device__ __forceinline__ int mip_from_dt(float dt, V3 p) {
    int mip = mip_from_pos(p);
    dt = __fmul_rn(dt, 256.0f);
    if (dt < 1.f) return mip;
    int e; frexpf(dt, &e);
    return min(6, max(e, mip));
}
__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
__device__ __forceinline__ uint32_t morton3d(uint32_t x, uint32_t y, uint32_t z) {
    return expand_bits(x) | (expand_bits(y) << 1) | (expand_bits(z) << 2);
}
__device__ __forceinline__ uint32_t morton_invert(uint32_t x) {
    x = x & 0x49249249u;
    x = (x | (x >> 2)) & 0xc30c30c3u;
    x = (x | (x >> 4)) & 0x0f00f00fu;
    x = (x | (x >> 8)) & 0xff0000ffu;
    x = (x | (x >> 16)) & 0x0000ffffu;
    return x;
}
__device__ __forceinline__ int grid_coord(float v, float s) {
    float q = __fadd_rn(__fmul_rn(__fsub_rn(v, 0.5f), s), 0.5f);
    int i = (int)__fmul_rn(q, 128.0f);
    return min(127, max(0, i));
}
__device__ __forceinline__ bool occupied_at(V3 p, const uint8_t* bf, int mip) {
    float s = scalbnf(1.0f, -mip);
    uint32_t idx = morton3d((uint32_t)grid_coord(p.x, s), (uint32_t)grid_coord(p.y, s), (uint32_t)grid_coord(p.z, s));
    return (__ldg(bf + idx / 8 + (size_t)mip * (GRID3 / 8)) >> (idx % 8)) & 1u;
}
__device__ __forceinline__ float advance_to_next_voxel(float t, float cone, V3 pos, V3 dir, V3 idir, uint32_t res) {
    float fr = (float)res;
    float px = __fmul_rn(fr, pos.x), py = __fmul_rn(fr, pos.y), pz = __fmul_rn(fr, pos.z);
    float tx = __fmul_rn(__fsub_rn(floorf(__fadd_rn(__fadd_rn(px, 0.5f), __fmul_rn(0.5f, sign_f(dir.x)))), px), idir.x);
    float ty = __fmul_rn(__fsub_rn(floorf(__fadd_rn(__fadd_rn(py, 0.5f), __fmul_rn(0.5f, sign_f(dir.y)))), py), idir.y);
    float tz = __fmul_rn(__fsub_rn(floorf(__fadd_rn(__fadd_rn(pz, 0.5f), __fmul_rn(0.5f, sign_f(dir.z)))), pz), idir.z);
    float tm = fminf(fminf(tx, ty), tz);
    float target = __fadd_rn(t, fmaxf(__fdiv_rn(tm, fr), 0.0f));
    int guard = 0;
    do { t = __fadd_rn(t, calc_dt(t, cone)); } while (t < target && ++guard < 1 << 20);
    return t;
}
__device__ __forceinline__ bool box_contains(const float* mn, const float* mx, V3 p) {
    return p.x >= mn[0] && p.x <= mx[0] && p.y >= mn[1] && p.y <= mx[1] && p.z >= mn[2] && p.z <= mx[2];
}
__device__ __forceinline__ V3 ray_at(V3 o, V3 d, float t) {
    return v3(__fadd_rn(o.x, __fmul_rn(d.x, t)), __fadd_rn(o.y, __fmul_rn(d.y, t)), __fadd_rn(o.z, __fmul_rn(d.z, t)));
}

// ------------------------------------------------------- low-discrepancy jitter
// Owen-scrambled Sobol (NGP/random_val.cuh:159-322), dimensions 0 and 1.
__device__ __forceinline__ uint32_t sobol_dim(uint32_t index, uint32_t dim) {
    uint32_t X = 0, v = 0x80000000u;
#pragma unroll 4
    for (uint32_t bit = 0; bit < 32; ++bit) {
        uint32_t dirn = dim == 0 ? (0x80000000u >> bit) : v;
        if ((index >> bit) & 1u) X ^= dirn;
        v = v ^ (v >> 1);
    }
    return X;
}
__device__ __forceinline__ uint32_t hash_combine(uint32_t seed, uint32_t v) { return seed ^ (v + (seed << 6) + (seed >> 2)); }
__device__ __forceinline__ uint32_t owen_scramble(uint32_t x, uint32_t seed) {
    x = __brev(x);
    x += seed;
    x ^= x * 0x6c50b47cu;
    x ^= x * 0xb82f1e52u;
    x ^= x * 0xc7afe638u;
    x ^= x * 0x8d22f6e6u;
    return __brev(x);
}
__device__ __forceinline__ float ld_random_val(uint32_t index, uint32_t seed, uint32_t dim) {
    const float S = (float)(1.0 / 4294967296.0);
    index = owen_scramble(index, seed);
    return __fmul_rn(__uint2float_rn(owen_scramble(sobol_dim(index, dim), hash_combine(seed, dim))), S);
}
__device__ __forceinline__ void ld_random_pixel_offset(uint32_t spp, float* out) {
    const float S = (float)(1.0 / 4294967296.0);
    uint32_t i0 = owen_scramble(0u, 0xdeadbeefu), i1 = owen_scramble(spp, 0xdeadbeefu);
#pragma unroll
    for (uint32_t d = 0; d < 2; ++d) {
        float v0 = __fmul_rn(__uint2float_rn(owen_scramble(sobol_dim(i0, d), hash_combine(0xdeadbeefu, d))), S);
        float v1 = __fmul_rn(__uint2float_rn(owen_scramble(sobol_dim(i1, d), hash_combine(0xdeadbeefu, d))), S);
        float o = __fadd_rn(__fsub_rn(0.5f, v0), v1);
        out[d] = __fsub_rn(o, floorf(o));
    }
}

__device__ __forceinline__ float aabb_ray_tmin(const float* mn, const float* mx, V3 o, V3 d) {
    float tmin = __fdiv_rn(__fsub_rn(mn[0], o.x), d.x), tmax = __fdiv_rn(__fsub_rn(mx[0], o.x), d.x);
    if (tmin > tmax) { float t = tmin; tmin = tmax; tmax = t; }
    float tymin = __fdiv_rn(__fsub_rn(mn[1], o.y), d.y), tymax = __fdiv_rn(__fsub_rn(mx[1], o.y), d.y);
    if (tymin > tymax) { float t = tymin; tymin = tymax; tymax = t; }
    if (tmin > tymax || tymin > tmax) return 3.402823466e38f;
    if (tymin > tmin) tmin = tymin;
    if (tymax < tmax) tmax = tymax;
    float tzmin = __fdiv_rn(__fsub_rn(mn[2], o.z), d.z), tzmax = __fdiv_rn(__fsub_rn(mx[2], o.z), d.z);
    if (tzmin > tzmax) { float t = tzmin; tzmin = tzmax; tzmax = t; }
    if (tmin > tzmax || tzmin > tmax) return 3.402823466e38f;
    if (tzmin > tmin) tmin = tzmin;
    return tmin;
}

struct RayState { V3 o, d, idir; float t; };

// init_rays_with_payload_kernel_nerf (:1854-1963) + pixel_to_ray (NGP/common_device.cuh:260-315)
// + advance_pos_nerf (:634-686).  Returns false when the ray misses the render box.
__device__ __forceinline__ bool ray_init(const RenderView& rv, uint32_t x, uint32_t y, const uint8_t* bf, RayState& r) {
    float off[2];
    ld_random_pixel_offset(rv.snap_to_pixel_centers ? 0u : rv.spp, off);
    float u = __fdiv_rn(__fadd_rn((float)x, off[0]), (float)rv.width);
    float v = __fdiv_rn(__fadd_rn((float)y, off[1]), (float)rv.height);
    V3 dc = v3(__fdiv_rn(__fmul_rn(__fsub_rn(u, rv.screen_center[0]), (float)rv.width), rv.focal[0]),
               __fdiv_rn(__fmul_rn(__fsub_rn(v, rv.screen_center[1]), (float)rv.height), rv.focal[1]), 1.0f);
    V3 d = v3(dot_rn(v3(rv.cam[0], rv.cam[1], rv.cam[2]), dc), dot_rn(v3(rv.cam[4], rv.cam[5], rv.cam[6]), dc),
              dot_rn(v3(rv.cam[8], rv.cam[9], rv.cam[10]), dc));
    d = normalize_rn(d);
    r.o = v3(rv.cam[3], rv.cam[7], rv.cam[11]);
    r.d = d;
    r.idir = v3(__fdiv_rn(1.f, d.x), __fdiv_rn(1.f, d.y), __fdiv_rn(1.f, d.z));
    float tm = aabb_ray_tmin(rv.aabb_min, rv.aabb_max, r.o, r.d);
    float t = __fadd_rn(fmaxf(tm, 0.05f), 1e-6f);
    if (!box_contains(rv.aabb_min, rv.aabb_max, ray_at(r.o, r.d, t))) return false;
    uint32_t idx = x + (uint32_t)rv.width * y;
    float dt = calc_dt(t, rv.cone_angle);
    t = __fadd_rn(t, __fmul_rn(ld_random_val(rv.spp, idx * 786433u, 0u), dt));
    for (int guard = 0; guard < (1 << 16); ++guard) {
        V3 p = ray_at(r.o, r.d, t);
        if (!box_contains(rv.aabb_min, rv.aabb_max, p)) return false;
        dt = calc_dt(t, rv.cone_angle);
        int mip = mip_from_dt(dt, p);
        if (occupied_at(p, bf, mip)) break;
        t = advance_to_next_voxel(t, rv.cone_angle, p, r.d, r.idir, GRID >> mip);
    }
    r.t = t;
    return true;
}

// One sample of generate_next_nerf_network_inputs (:760-791).  False when the ray leaves the box.
__device__ __forceinline__ bool ray_next_sample(const RenderView& rv, const uint8_t* bf, RayState& r, V3& pos, float& dt, float* t_sample = nullptr) {
    float t = r.t;
    for (int guard = 0; guard < (1 << 16); ++guard) {
        pos = ray_at(r.o, r.d, t);
        if (!box_contains(rv.aabb_min, rv.aabb_max, pos)) { r.t = t; return false; }
        dt = calc_dt(t, rv.cone_angle);
        int mip = mip_from_dt(dt, pos);
        if (occupied_at(pos, bf, mip)) { if (t_sample) *t_sample = t; r.t = __fadd_rn(t, dt); return true; }
        t = advance_to_next_voxel(t, rv.cone_angle, pos, r.d, r.idir, GRID >> mip);
    }
    r.t = t;
    return false;
}

// ------------------------------------------------------------ hash-grid encode
// Published multiresolution hash encoding, this library's documented table layout
// (per-level dense index x + y*res + z*res^2 or spatial hash with primes
// 1, 2654435761, 805459861; trilinear weights; FP32 accumulation).
// Level l's two features at x (trilinear over the cell's 8 corners).
__device__ __forceinline__ float2 half2_bits(uint32_t b) {
    __half2 h;
    memcpy(&h, &b, 4);
    return __half22float2(h);
}

// Trilinear interpolation of level l's two features at x (the published multiresolution hash
// encoding: dense index x + y res + z res^2 for levels whose grid fits the table, else the spatial
// hash x ^ y * 2654435761 ^ z * 805459861).  The eight corners are summed in the order
// (x, y, z) = 000, 100, 010, 110, 001, 101, 011, 111.  Dense levels (the coarse ones) fetch the
// two x-neighbours of each (y, z) pair together: one 8-byte load when the pair starts on an even
// entry (level offsets are multiples of 8 entries), else two 4-byte loads; the values and their
// order are unchanged.  (Measured on the 512x512 frame: 8-byte pairs ~2 % faster than per-corner
// loads; 16-byte groups and L2 evict_last cache hints on the dense levels were slower.)
__device__ __forceinline__ void hash_level(const FieldView& fv, const __half2* table, V3 x, uint32_t l, float& a0, float& a1) {
    const float s = fv.level_scale[l];
    float px = fmaf(x.x, s, 0.5f), py = fmaf(x.y, s, 0.5f), pz = fmaf(x.z, s, 0.5f);
    float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    float rx = __fsub_rn(px, fx), ry = __fsub_rn(py, fy), rz = __fsub_rn(pz, fz);
    uint32_t gx = (uint32_t)(int32_t)fx, gy = (uint32_t)(int32_t)fy, gz = (uint32_t)(int32_t)fz;
    const uint32_t res = fv.level_res[l], size = fv.level_size[l];
    const bool dense = fv.level_dense[l];
    const __half2* lt = table + fv.level_off[l];
    // The weights and the weighted sum run as packed FP32 pairs (the two x-neighbours' weights,
    // the two features), each half with the rounding of the scalar operations, in the same order:
    // w = (wx * wy) * wz, then a += w * e corner by corner.
    const float2 wx = make_float2(__fsub_rn(1.f, rx), rx);
    float2 acc = make_float2(0.f, 0.f);
    if (dense) {
#pragma unroll
        for (uint32_t c2 = 0; c2 < 4; ++c2) {
            const uint32_t by = c2 & 1u, bz = c2 >> 1;
            uint32_t i0 = gx + (gy + by) * res + (gz + bz) * res * res;
            uint32_t i1 = i0 + 1u;
            if (i0 >= size) i0 %= size;   // only cells on the far boundary wrap
            if (i1 >= size) i1 %= size;
            float2 e0, e1;
            if (i1 == i0 + 1u && (i0 & 1u) == 0u) {
                const uint2 u = __ldg(reinterpret_cast<const uint2*>(lt + i0));
                e0 = half2_bits(u.x);
                e1 = half2_bits(u.y);
            } else {
                e0 = __half22float2(__ldg(lt + i0));
                e1 = __half22float2(__ldg(lt + i1));
            }
            const float wy = by ? ry : __fsub_rn(1.f, ry), wz = bz ? rz : __fsub_rn(1.f, rz);
            const float2 w = __fmul2_rn(__fmul2_rn(wx, make_float2(wy, wy)), make_float2(wz, wz));
            acc = __fadd2_rn(acc, __fmul2_rn(make_float2(w.x, w.x), e0));
            acc = __fadd2_rn(acc, __fmul2_rn(make_float2(w.y, w.y), e1));
        }
        a0 = acc.x;
        a1 = acc.y;
        return;
    }
#pragma unroll
    for (uint32_t c2 = 0; c2 < 4; ++c2) {
        const uint32_t by = c2 & 1u, bz = c2 >> 1;
        const float wy = by ? ry : __fsub_rn(1.f, ry), wz = bz ? rz : __fsub_rn(1.f, rz);
        const float2 w = __fmul2_rn(__fmul2_rn(wx, make_float2(wy, wy)), make_float2(wz, wz));
        const uint32_t hyz = ((gy + by) * 2654435761u) ^ ((gz + bz) * 805459861u);
        const uint32_t idx0 = (gx ^ hyz) & (size - 1u), idx1 = ((gx + 1u) ^ hyz) & (size - 1u);
        const float2 e0 = __half22float2(__ldg(lt + idx0)), e1 = __half22float2(__ldg(lt + idx1));
        acc = __fadd2_rn(acc, __fmul2_rn(make_float2(w.x, w.x), e0));
        acc = __fadd2_rn(acc, __fmul2_rn(make_float2(w.y, w.y), e1));
    }
    a0 = acc.x;
    a1 = acc.y;
}

// Level l's F = 4 or 8 features at x: the corners, weights and summation order of hash_level,
// each corner's F FP16 values in one 8-byte (F = 4) or 16-byte (F = 8) load; entry i of the
// level starts at FP16 element (level_off + i) F (16-byte aligned for F = 8: the table follows the
// MLP weights, whose sizes are multiples of 16 elements).
template <int F>
__device__ __forceinline__ void hash_level_wide(const FieldView& fv, const __half2* table, V3 x, uint32_t l, float* out) {
    static_assert(F == 4 || F == 8, "4 or 8 features per level");
    const float s = fv.level_scale[l];
    const float px = fmaf(x.x, s, 0.5f), py = fmaf(x.y, s, 0.5f), pz = fmaf(x.z, s, 0.5f);
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    const float rx = __fsub_rn(px, fx), ry = __fsub_rn(py, fy), rz = __fsub_rn(pz, fz);
    const uint32_t gx = (uint32_t)(int32_t)fx, gy = (uint32_t)(int32_t)fy, gz = (uint32_t)(int32_t)fz;
    const uint32_t res = fv.level_res[l], size = fv.level_size[l];
    const bool dense = fv.level_dense[l];
    const __half2* lt = table + (size_t)fv.level_off[l] * (F / 2);
    const float2 wx = make_float2(__fsub_rn(1.f, rx), rx);
    float2 acc[F / 2];
#pragma unroll
    for (int q = 0; q < F / 2; ++q) acc[q] = make_float2(0.f, 0.f);
#pragma unroll
    for (uint32_t c2 = 0; c2 < 4; ++c2) {
        const uint32_t by = c2 & 1u, bz = c2 >> 1;
        uint32_t i0, i1;
        if (dense) {
            i0 = gx + (gy + by) * res + (gz + bz) * res * res;
            i1 = i0 + 1u;
            if (i0 >= size) i0 %= size;   // only cells on the far boundary wrap
            if (i1 >= size) i1 %= size;
        } else {
            const uint32_t hyz = ((gy + by) * 2654435761u) ^ ((gz + bz) * 805459861u);
            i0 = (gx ^ hyz) & (size - 1u);
            i1 = ((gx + 1u) ^ hyz) & (size - 1u);
        }
        uint32_t e0[F / 2], e1[F / 2];
        if constexpr (F == 8) {
            const uint4 u0 = __ldg(reinterpret_cast<const uint4*>(lt + (size_t)i0 * 4u));
            const uint4 u1 = __ldg(reinterpret_cast<const uint4*>(lt + (size_t)i1 * 4u));
            e0[0] = u0.x; e0[1] = u0.y; e0[2] = u0.z; e0[3] = u0.w;
            e1[0] = u1.x; e1[1] = u1.y; e1[2] = u1.z; e1[3] = u1.w;
        } else {
            const uint2 u0 = __ldg(reinterpret_cast<const uint2*>(lt + (size_t)i0 * 2u));
            const uint2 u1 = __ldg(reinterpret_cast<const uint2*>(lt + (size_t)i1 * 2u));
            e0[0] = u0.x; e0[1] = u0.y;
            e1[0] = u1.x; e1[1] = u1.y;
        }
        const float wy = by ? ry : __fsub_rn(1.f, ry), wz = bz ? rz : __fsub_rn(1.f, rz);
        const float2 w = __fmul2_rn(__fmul2_rn(wx, make_float2(wy, wy)), make_float2(wz, wz));
#pragma unroll
        for (int q = 0; q < F / 2; ++q) acc[q] = __fadd2_rn(acc[q], __fmul2_rn(make_float2(w.x, w.x), half2_bits(e0[q])));
#pragma unroll
        for (int q = 0; q < F / 2; ++q) acc[q] = __fadd2_rn(acc[q], __fmul2_rn(make_float2(w.y, w.y), half2_bits(e1[q])));
    }
#pragma unroll
    for (int q = 0; q < F / 2; ++q) { out[2 * q] = acc[q].x; out[2 * q + 1] = acc[q].y; }
}

// Real spherical harmonics up to degree 4 of the unwarped direction (16 values).
__device__ __forceinline__ void sh4(float dx, float dy, float dz, float* out) {
    float x = __fsub_rn(__fmul_rn(dx, 2.f), 1.f), y = __fsub_rn(__fmul_rn(dy, 2.f), 1.f), z = __fsub_rn(__fmul_rn(dz, 2.f), 1.f);
    float xx = x * x, yy = y * y, zz = z * z;
    float s[16];
    s[0] = 0.28209479177387814f;
    s[1] = -0.48860251190291987f * y;
    s[2] = 0.48860251190291987f * z;
    s[3] = -0.48860251190291987f * x;
    s[4] = 1.0925484305920792f * x * y;
    s[5] = -1.0925484305920792f * y * z;
    s[6] = 0.94617469575755997f * zz - 0.31539156525251999f;
    s[7] = -1.0925484305920792f * x * z;
    s[8] = 0.54627421529603959f * (xx - yy);
    s[9] = 0.59004358992664352f * y * (-3.f * xx + yy);
    s[10] = 2.8906114426405538f * x * y * z;
    s[11] = 0.45704579946446572f * y * (1.f - 5.f * zz);
    s[12] = 0.3731763325901154f * z * (5.f * zz - 3.f);
    s[13] = 0.45704579946446572f * x * (1.f - 5.f * zz);
    s[14] = 1.4453057213202769f * z * (xx - yy);
    s[15] = 0.59004358992664352f * x * (-xx + 3.f * yy);
#pragma unroll
    for (int k = 0; k < 16; ++k) out[k] = s[k];
}

}  // namespace insta
