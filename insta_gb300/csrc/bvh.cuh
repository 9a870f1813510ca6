// bvh.cuh -- exact nearest-triangle query over the per-frame 4-wide LBVH.
//
// Depth-first, nearest-child-first traversal (the order of closest_triangle,
// NGP/bvh.cuh:48-96: child boxes sorted with the 4-input network, nearest popped
// first).  Differences from the reference, both deliberate:
//   * ties resolve to the lowest original triangle id (the reference keeps the last
//     triangle in BVH order, which depends on the build);
//   * a subtree is pruned only when its box distance exceeds best * (1 + 2^-10) + 1e-12,
//     so a rounding-level difference between box and triangle distances can never hide
//     the true minimum -- the result equals the brute-force minimum over all triangles.
// The search can start from a distance bound (occupancy marking).
#pragma once

#include "insta_types.h"

namespace insta {

struct Nearest {
    int32_t id;     // original triangle id, -1 when nothing within the bound
    int32_t slot;   // position in the frame's Morton-ordered triangle array
    float d2;       // squared distance
};

// Point-box squared distance for pruning only: fused multiply-adds are fine here because the
// prune limit carries a relative slack far larger than any rounding difference.
// The offset to the box is p minus p clamped into the box (zero inside).
__device__ __forceinline__ float box_dist_fast(float mnx, float mny, float mnz, float mxx, float mxy, float mxz, V3 p) {
    const float dx = p.x - fminf(fmaxf(p.x, mnx), mxx);
    const float dy = p.y - fminf(fmaxf(p.y, mny), mxy);
    const float dz = p.z - fminf(fmaxf(p.z, mnz), mxz);
    return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

__device__ __forceinline__ float prune_limit(float best) {
    return isinf(best) ? best : __fadd_rn(__fadd_rn(best, __fmul_rn(best, 0.0009765625f)), 1e-12f);
}

// Exact squared distance of p to the triangle at Morton slot `slot`; its original id in `id`.
__device__ __forceinline__ float slot_distance(const FrameView& fr, int32_t slot, V3 p, int32_t& id) {
    return tri_distance_rec(fr.leaf_tris + (size_t)slot * INSTA_TRI_F4, p, id);
}

__device__ __forceinline__ Nearest nearest_bvh(const FrameView& fr, V3 p, float best, int32_t bid, int32_t bslot, uint32_t* err) {
    uint32_t stack_r[INSTA_STACK];
    float stack_d[INSTA_STACK];
    int sp = 0;
    stack_r[sp] = 0u;
    stack_d[sp] = 0.f;
    ++sp;
    while (sp > 0) {
        --sp;
        const uint32_t ref = stack_r[sp];
        if (stack_d[sp] > prune_limit(best)) continue;
        if (ref & INSTA_LEAF_BIT) {
            const uint32_t first = (ref & ~INSTA_LEAF_BIT) >> 3, count = ref & 7u;
            for (uint32_t i = 0; i < count; ++i) {
                if (leaf_bound_sq(fr.leaf_bounds + (size_t)(first + i) * 2, p) > prune_limit(best)) continue;
                int32_t id;
                float d = slot_distance(fr, (int32_t)(first + i), p, id);
                if (d < best || (d == best && (uint32_t)id < (uint32_t)bid)) { best = d; bid = id; bslot = (int32_t)(first + i); }
            }
            continue;
        }
        const float4* nd = fr.nodes + (size_t)ref * 7;
        const float4 mnx = __ldg(nd + 0), mny = __ldg(nd + 1), mnz = __ldg(nd + 2);
        const float4 mxx = __ldg(nd + 3), mxy = __ldg(nd + 4), mxz = __ldg(nd + 5);
        const int4 ch = __ldg(reinterpret_cast<const int4*>(nd + 6));
        float cd[4];
        uint32_t ci[4] = {(uint32_t)ch.x, (uint32_t)ch.y, (uint32_t)ch.z, (uint32_t)ch.w};
        cd[0] = box_dist_fast(mnx.x, mny.x, mnz.x, mxx.x, mxy.x, mxz.x, p);
        cd[1] = box_dist_fast(mnx.y, mny.y, mnz.y, mxx.y, mxy.y, mxz.y, p);
        cd[2] = box_dist_fast(mnx.z, mny.z, mnz.z, mxx.z, mxy.z, mxz.z, p);
        cd[3] = box_dist_fast(mnx.w, mny.w, mnz.w, mxx.w, mxy.w, mxz.w, p);
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (ci[i] == 0xffffffffu) cd[i] = __int_as_float(0x7f800000);
        // 4-input sorting network, descending (NGP/bvh.cuh:28-46): the nearest child is pushed last
#define INSTA_CAS(x, y) if (cd[x] < cd[y]) { float td = cd[x]; cd[x] = cd[y]; cd[y] = td; uint32_t ti = ci[x]; ci[x] = ci[y]; ci[y] = ti; }
        INSTA_CAS(0, 2) INSTA_CAS(1, 3) INSTA_CAS(0, 1) INSTA_CAS(2, 3) INSTA_CAS(1, 2)
#undef INSTA_CAS
        const float lim = prune_limit(best);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (ci[i] != 0xffffffffu && cd[i] <= lim) {
                if (sp < INSTA_STACK) { stack_r[sp] = ci[i]; stack_d[sp] = cd[i]; ++sp; }
                else if (err) atomicOr(err, INSTA_DEVERR_STACK);
            }
        }
    }
    return {bid, bslot, best};
}

// Leaves hold up to INSTA_LEAF_SIZE triangles (a 3-bit count in the leaf reference).  Wider leaves
// than the reference's two trade inner-node visits -- the expensive part of a warp walk: four box
// tests per lane, the warp-wide child ordering, the stack pushes -- for bounding-disk tests,
// which are cheap; measured on the 512x512 frame, leaves of 2 / 3 / 4 triangles: 29.8 / 26.1 /
// 23.1 inner nodes per warp walk, nearest stage 1.12 / 1.09 / 1.07 ms.
static_assert(INSTA_LEAF_SIZE >= 1 && INSTA_LEAF_SIZE <= 7, "leaf counts are 3 bits");
constexpr uint32_t kWarpQueue = 32u * (INSTA_LEAF_SIZE + 1);   // < 32 pending + a leaf's tests for 32 lanes

// Per-warp shared scratch of nearest_warp.
struct WarpScratch {
    uint32_t stack[INSTA_STACK];   // node references of the shared traversal stack
    uint32_t skey[INSTA_STACK];    // per entry: the smallest box distance (bits) of the lanes that pushed it
    uint32_t queue[kWarpQueue];    // pending exact tests: Morton slot << 5 | owner lane
    unsigned long long best[32];   // per lane: (distance bits << 32) | triangle id, the running minimum
};

// Run the first n queued exact tests, one per lane: lane t tests entry t against its owner's
// point and folds (distance, id) into the owner's running minimum; the rest of the queue moves to
// the front.  Returns the refreshed (best, bid) of the calling lane.
__device__ __forceinline__ void flush_tests(const FrameView& fr, WarpScratch& ws, V3 p, uint32_t n, uint32_t& qlen,
                                            float& best, int32_t& bid) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t e = lane < n ? ws.queue[lane] : 0u;
    const uint32_t owner = e & 31u;
    const V3 q = v3(__shfl_sync(0xffffffffu, p.x, owner), __shfl_sync(0xffffffffu, p.y, owner), __shfl_sync(0xffffffffu, p.z, owner));
    if (lane < n) {
        int32_t id;
        const float d = slot_distance(fr, (int32_t)(e >> 5), q, id);
        atomicMin(&ws.best[owner], ((unsigned long long)__float_as_uint(d) << 32) | (uint32_t)id);
    }
    const uint32_t rest = qlen - n;   // < 32 * INSTA_LEAF_SIZE
    uint32_t tq[INSTA_LEAF_SIZE];
#pragma unroll
    for (int j = 0; j < INSTA_LEAF_SIZE; ++j) tq[j] = lane + 32u * j < rest ? ws.queue[n + 32u * j + lane] : 0u;
    __syncwarp();
#pragma unroll
    for (int j = 0; j < INSTA_LEAF_SIZE; ++j)
        if (lane + 32u * j < rest) ws.queue[32u * j + lane] = tq[j];
    __syncwarp();
    qlen = rest;
    const unsigned long long k = ws.best[lane];
    best = __uint_as_float((uint32_t)(k >> 32));
    bid = (int32_t)(uint32_t)k;
}

// Warp-cooperative variant for spatially coherent queries (one point per lane, all 32 lanes call
// it together).  The warp walks the union of the nodes its lanes need with one shared stack: a
// node is fetched once per warp, every lane tests it against its own point and bound, and a child
// is pushed when any lane may find a nearer triangle in it.  The stack holds, beside each node,
// the smallest box distance among the lanes that wanted it (warp-uniform, in shared memory): a
// popped node is skipped when that exceeds every lane's current prune limit, so no per-lane
// distances are kept (no local-memory stack; measured on the 512x512 frame: 6 % more inner nodes,
// nearest stage 0.965 -> 0.920 ms).  At a leaf, the (triangle, lane) pairs
// that lanes need are queued and run 32 at a time, one per lane, so the exact tests are not
// replicated across lanes that do not need them.  Each lane's result is exactly its own nearest
// triangle, ties to the lowest id (the union holds every node that lane's own traversal would
// visit; pruning with a not yet updated bound only tests more).  Control flow stays uniform.
// Lanes with active == false only ride along.  The slot of the result is not tracked (-1).
// `top`: when not null, the warp's shared-memory copy of the frame's first n_top nodes (the top
// levels: nodes are numbered level by level, see stage_top_nodes); those are read from there.
// `stats`: when not null, lane 0 adds the walk's counts (walks, inner nodes, leaves, bounding-disk
// tests, exact tests) to stats[0..4].
__device__ __forceinline__ Nearest nearest_warp(const FrameView& fr, V3 p, bool active, WarpScratch& ws, uint32_t* err,
                                                float bound = __builtin_huge_valf(), const float4* top = nullptr,
                                                uint32_t n_top = 0, unsigned long long* stats = nullptr) {
    uint32_t c_inner = 0, c_leaf = 0, c_bound = 0, c_exact = 0;
    const float INF = __int_as_float(0x7f800000);
    const uint32_t lane = threadIdx.x & 31u, lt_mask = (1u << lane) - 1u;
    float best = active ? bound : -INF;
    int32_t bid = -1;
    int sp = 0;
    uint32_t qlen = 0;
    __syncwarp();
    ws.best[lane] = ((unsigned long long)__float_as_uint(best) << 32) | 0xffffffffull;
    if (lane == 0) { ws.stack[0] = 0u; ws.skey[0] = 0u; }
    __syncwarp();
    sp = 1;
    float lim = prune_limit(best);   // changes only when a flush lowers best
    // the warp's largest prune limit (bits; limits are >= 0, inactive lanes count as 0)
    uint32_t lim_max = __reduce_max_sync(0xffffffffu, active ? __float_as_uint(lim) : 0u);
    while (sp > 0) {
        --sp;
        const uint32_t ref = ws.stack[sp];
        if (ws.skey[sp] > lim_max) continue;   // no lane can find anything nearer below it
        const bool need = active;
        const uint32_t nm = __ballot_sync(0xffffffffu, need);
        if (ref & INSTA_LEAF_BIT) {
            // a lane queues a triangle of the leaf only when the triangle's bounding disk may
            // hold a point nearer than its prune limit (leaf_bound_sq)
            const uint32_t first = (ref & ~INSTA_LEAF_BIT) >> 3, count = ref & 7u;
            __syncwarp();   // the popped entry has been read by every lane
            ++c_leaf;
            c_bound += count * (uint32_t)__popc(nm);
            for (uint32_t i = 0; i < count; ++i) {
                const bool want = need && leaf_bound_sq(fr.leaf_bounds + (size_t)(first + i) * 2, p) <= lim;
                const uint32_t m = __ballot_sync(0xffffffffu, want);
                if (want) ws.queue[qlen + __popc(m & lt_mask)] = ((first + i) << 5) | lane;
                qlen += __popc(m);
                c_exact += (uint32_t)__popc(m);
            }
            __syncwarp();
            if (qlen >= 32u) {
                do flush_tests(fr, ws, p, 32u, qlen, best, bid);
                while (qlen >= 32u);
                lim = prune_limit(best);
                lim_max = __reduce_max_sync(0xffffffffu, active ? __float_as_uint(lim) : 0u);
            }
            continue;
        }
        ++c_inner;
        float4 mnx, mny, mnz, mxx, mxy, mxz;
        int4 ch;
        if (ref < n_top) {   // warp-uniform: the staged top levels
            const float4* nd = top + (size_t)ref * 7;
            mnx = nd[0]; mny = nd[1]; mnz = nd[2]; mxx = nd[3]; mxy = nd[4]; mxz = nd[5];
            ch = reinterpret_cast<const int4*>(nd)[6];
        } else {
            const float4* nd = fr.nodes + (size_t)ref * 7;
            mnx = __ldg(nd + 0); mny = __ldg(nd + 1); mnz = __ldg(nd + 2);
            mxx = __ldg(nd + 3); mxy = __ldg(nd + 4); mxz = __ldg(nd + 5);
            ch = __ldg(reinterpret_cast<const int4*>(nd + 6));
        }
        float cd[4];
        uint32_t ci[4] = {(uint32_t)ch.x, (uint32_t)ch.y, (uint32_t)ch.z, (uint32_t)ch.w};
        cd[0] = box_dist_fast(mnx.x, mny.x, mnz.x, mxx.x, mxy.x, mxz.x, p);
        cd[1] = box_dist_fast(mnx.y, mny.y, mnz.y, mxx.y, mxy.y, mxz.y, p);
        cd[2] = box_dist_fast(mnx.z, mny.z, mnz.z, mxx.z, mxy.z, mxz.z, p);
        cd[3] = box_dist_fast(mnx.w, mny.w, mnz.w, mxx.w, mxy.w, mxz.w, p);
        // per child: the warp's smallest distance among lanes that need it (bits order like floats >= 0)
        uint32_t key[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const bool want = ci[i] != 0xffffffffu && cd[i] <= lim;
            key[i] = __reduce_min_sync(0xffffffffu, want ? __float_as_uint(cd[i]) : 0xffffffffu);
        }
        // sort the children farthest-first (keys are warp-uniform; every index is static, so the
        // pairs stay in registers) and push the needed ones: the warp pops the nearest next.
        // With at most one child wanted there is nothing to order.
        const int wanted = (key[0] != 0xffffffffu) + (key[1] != 0xffffffffu) + (key[2] != 0xffffffffu) + (key[3] != 0xffffffffu);
        if (wanted > 1) {
#define INSTA_CASK(x, y)                                                                  \
    if (key[x] < key[y]) {                                                                \
        uint32_t tk = key[x]; key[x] = key[y]; key[y] = tk;                               \
        uint32_t tc = ci[x]; ci[x] = ci[y]; ci[y] = tc;                                   \
    }
            INSTA_CASK(0, 2) INSTA_CASK(1, 3) INSTA_CASK(0, 1) INSTA_CASK(2, 3) INSTA_CASK(1, 2)
#undef INSTA_CASK
        }
        __syncwarp();   // every lane has read the popped entry before lane 0 overwrites it
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (key[i] != 0xffffffffu) {
                if (sp < INSTA_STACK) {
                    if (lane == 0) { ws.stack[sp] = ci[i]; ws.skey[sp] = key[i]; }
                    ++sp;
                } else if (err && lane == 0) {
                    atomicOr(err, INSTA_DEVERR_STACK);
                }
            }
        }
        __syncwarp();
    }
    if (qlen) flush_tests(fr, ws, p, qlen, qlen, best, bid);
    if (stats && lane == 0) {
        atomicAdd(stats + 0, 1ull);
        atomicAdd(stats + 1, (unsigned long long)c_inner);
        atomicAdd(stats + 2, (unsigned long long)c_leaf);
        atomicAdd(stats + 3, (unsigned long long)c_bound);
        atomicAdd(stats + 4, (unsigned long long)c_exact);
    }
    return {bid, -1, best};
}

// ------------------------------------------------------------------ ray queries
// Triangle::ray_intersect (NGP/triangle.cuh:66-80) from a leaf record, same operations and order:
// FLT_MAX for a miss.  v1v0 = b - a is the record's v21; v2v0 = c - a is -v13 and the triangle
// normal (b - a) x (c - a) is -(v21 x v13), both exact negations.
__device__ __forceinline__ float tri_ray_rec(const float4* tr, V3 ro, V3 rd, int32_t& id) {
    const float4 q0 = __ldg(tr), q2 = __ldg(tr + 2), q3 = __ldg(tr + 3), q5 = __ldg(tr + 5), q6 = __ldg(tr + 6), q7 = __ldg(tr + 7);
    id = __float_as_int(q2.y);
    const V3 v1v0 = v3(q3.x, q3.y, q3.z), v2v0 = v3(-q5.x, -q5.y, -q5.z), n = v3(-q5.w, -q6.w, -q7.w);
    const V3 rov0 = sub_rn(ro, v3(q0.x, q0.y, q0.z));
    const V3 q = cross_rn(rov0, rd);
    const float d = __fdiv_rn(1.0f, dot_rn(rd, n));
    const float u = __fmul_rn(d, -dot_rn(q, v2v0));
    const float v = __fmul_rn(d, dot_rn(q, v1v0));
    const float t = __fmul_rn(d, -dot_rn(n, rov0));
    if (u < 0.0f || u > 1.0f || v < 0.0f || __fadd_rn(u, v) > 1.0f || t < 0.0f) return 3.402823466e38f;
    return t;
}

// Entry distance of a ray into a box for pruning (slab test; NaN slabs from zero direction
// components count as inside): +inf when the ray misses it.
__device__ __forceinline__ float box_ray_entry(float mnx, float mny, float mnz, float mxx, float mxy, float mxz, V3 o, V3 inv) {
    const float tx1 = (mnx - o.x) * inv.x, tx2 = (mxx - o.x) * inv.x;
    const float ty1 = (mny - o.y) * inv.y, ty2 = (mxy - o.y) * inv.y;
    const float tz1 = (mnz - o.z) * inv.z, tz2 = (mxz - o.z) * inv.z;
    const float tmin = fmaxf(fmaxf(fminf(tx1, tx2), fminf(ty1, ty2)), fmaxf(fminf(tz1, tz2), 0.f));
    const float tmax = fminf(fminf(fmaxf(tx1, tx2), fmaxf(ty1, ty2)), fmaxf(tz1, tz2));
    return tmax * 1.0001f + 1e-6f < tmin ? __int_as_float(0x7f800000) : tmin;
}

// Closest hit with t < t_max (TriangleBvh4::ray_intersect, ngp/src/triangle_bvh.cu:271-311): the
// exact minimum of tri_ray_rec over all triangles, ties to the lowest triangle id (the reference
// keeps the first in its BVH order).  A subtree is skipped only when its entry exceeds the
// running minimum by the prune slack.  Returns {id or -1, Morton slot or -1, t (t_max for no hit)}.
__device__ __forceinline__ Nearest ray_closest(const FrameView& fr, V3 o, V3 d, float t_max, uint32_t* err) {
    const V3 inv = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    uint32_t stack[INSTA_STACK];
    int sp = 0;
    stack[sp++] = 0u;
    float best = t_max;
    int32_t bid = -1, bslot = -1;
    while (sp > 0) {
        const uint32_t ref = stack[--sp];
        if (ref & INSTA_LEAF_BIT) {
            const uint32_t first = (ref & ~INSTA_LEAF_BIT) >> 3, count = ref & 7u;
            for (uint32_t i = 0; i < count; ++i) {
                int32_t id;
                const float t = tri_ray_rec(fr.leaf_tris + (size_t)(first + i) * INSTA_TRI_F4, o, d, id);
                if (t < best || (t == best && bid >= 0 && (uint32_t)id < (uint32_t)bid)) { best = t; bid = id; bslot = (int32_t)(first + i); }
            }
            continue;
        }
        const float4* nd = fr.nodes + (size_t)ref * 7;
        const float4 mnx = __ldg(nd + 0), mny = __ldg(nd + 1), mnz = __ldg(nd + 2);
        const float4 mxx = __ldg(nd + 3), mxy = __ldg(nd + 4), mxz = __ldg(nd + 5);
        const int4 ch = __ldg(reinterpret_cast<const int4*>(nd + 6));
        uint32_t ci[4] = {(uint32_t)ch.x, (uint32_t)ch.y, (uint32_t)ch.z, (uint32_t)ch.w};
        float ct[4];
        ct[0] = box_ray_entry(mnx.x, mny.x, mnz.x, mxx.x, mxy.x, mxz.x, o, inv);
        ct[1] = box_ray_entry(mnx.y, mny.y, mnz.y, mxx.y, mxy.y, mxz.y, o, inv);
        ct[2] = box_ray_entry(mnx.z, mny.z, mnz.z, mxx.z, mxy.z, mxz.z, o, inv);
        ct[3] = box_ray_entry(mnx.w, mny.w, mnz.w, mxx.w, mxy.w, mxz.w, o, inv);
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (ci[i] == 0xffffffffu) ct[i] = __int_as_float(0x7f800000);
#define INSTA_CAS(x, y) if (ct[x] < ct[y]) { float td = ct[x]; ct[x] = ct[y]; ct[y] = td; uint32_t ti = ci[x]; ci[x] = ci[y]; ci[y] = ti; }
        INSTA_CAS(0, 2) INSTA_CAS(1, 3) INSTA_CAS(0, 1) INSTA_CAS(2, 3) INSTA_CAS(1, 2)
#undef INSTA_CAS
        const float lim = best + best * 0.0009765625f + 1e-6f;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (ci[i] != 0xffffffffu && ct[i] <= lim) {
                if (sp < INSTA_STACK) stack[sp++] = ci[i];
                else if (err) atomicOr(err, INSTA_DEVERR_STACK);
            }
        }
    }
    return {bid, bslot, best};
}

// Unbounded exact nearest triangle.
__device__ __forceinline__ Nearest nearest_triangle(const FrameView& fr, V3 p, uint32_t* err) {
    return nearest_bvh(fr, p, __int_as_float(0x7f800000), -1, -1, err);
}


}  // namespace insta
