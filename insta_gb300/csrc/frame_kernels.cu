// frame_kernels.cu -- per-frame tracked-mesh upload on the device: triangle frame
// records, Morton-ordered implicit 4-ary BVH (single-CTA shared-memory sort), occupancy
// bitfield from the mesh, and the canonical-map kernels (the `warp` hook).
#include <algorithm>
#include <vector>

#include "device_common.cuh"
#include "kernels.h"

namespace insta {

// ----------------------------------------------------------------- frame records
__device__ __forceinline__ float tri_area_rn(V3 a, V3 b, V3 c) {
    V3 n = cross_rn(sub_rn(b, a), sub_rn(c, a));
    return __fmul_rn(0.5f, __fsqrt_rn(dot_rn(n, n)));
}

// Triangles whose edges are almost parallel (sin^2 of the corner angle <= 1e-12) get their
// frame built in FP64; everything else in FP32 with the reference's operation order.
__device__ __forceinline__ bool near_degenerate(V3 e1, V3 e2) {
    V3 n = cross_rn(e1, e2);
    float nn = dot_rn(n, n), l1 = dot_rn(e1, e1), l2 = dot_rn(e2, e2);
    return nn <= 1e-12f * l1 * l2;
}

struct D3 { double x, y, z; };
__device__ __forceinline__ D3 d3cross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
__device__ __forceinline__ double d3dot(D3 a, D3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
__device__ __forceinline__ D3 d3norm(D3 v) {
    double z = d3dot(v, v);
    if (z > 0.0) { double s = sqrt(z); return {v.x / s, v.y / s, v.z / s}; }
    return v;
}

__device__ bool inverse4_d(const double* m, double* o) {
    double s0 = m[0] * m[5] - m[4] * m[1], s1 = m[0] * m[6] - m[4] * m[2], s2 = m[0] * m[7] - m[4] * m[3];
    double s3 = m[1] * m[6] - m[5] * m[2], s4 = m[1] * m[7] - m[5] * m[3], s5 = m[2] * m[7] - m[6] * m[3];
    double c5 = m[10] * m[15] - m[14] * m[11], c4 = m[9] * m[15] - m[13] * m[11], c3 = m[9] * m[14] - m[13] * m[10];
    double c2 = m[8] * m[15] - m[12] * m[11], c1 = m[8] * m[14] - m[12] * m[10], c0 = m[8] * m[13] - m[12] * m[9];
    double det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    if (det == 0.0) return false;
    double id = 1.0 / det;
    o[0] = (m[5] * c5 - m[6] * c4 + m[7] * c3) * id;   o[1] = (-m[1] * c5 + m[2] * c4 - m[3] * c3) * id;
    o[2] = (m[13] * s5 - m[14] * s4 + m[15] * s3) * id; o[3] = (-m[9] * s5 + m[10] * s4 - m[11] * s3) * id;
    o[4] = (-m[4] * c5 + m[6] * c2 - m[7] * c1) * id;  o[5] = (m[0] * c5 - m[2] * c2 + m[3] * c1) * id;
    o[6] = (-m[12] * s5 + m[14] * s2 - m[15] * s1) * id; o[7] = (m[8] * s5 - m[10] * s2 + m[11] * s1) * id;
    o[8] = (m[4] * c4 - m[5] * c2 + m[7] * c0) * id;   o[9] = (-m[0] * c4 + m[1] * c2 - m[3] * c0) * id;
    o[10] = (m[12] * s4 - m[13] * s2 + m[15] * s0) * id; o[11] = (-m[8] * s4 + m[9] * s2 - m[11] * s0) * id;
    o[12] = (-m[4] * c3 + m[5] * c1 - m[6] * c0) * id; o[13] = (m[0] * c3 - m[1] * c1 + m[2] * c0) * id;
    o[14] = (-m[12] * s3 + m[13] * s1 - m[14] * s0) * id; o[15] = (m[8] * s3 - m[9] * s1 + m[10] * s0) * id;
    return true;
}

// TinyMesh::build_triangles (src/tiny_mesh.cu:134-164) + tri2projection (include/rta/affine.cuh:26-39)
// for every face; `canon_area` == nullptr builds the canonical mesh (scaling 1).
__global__ void tri_frame_kernel(int F, const float* __restrict__ verts, const int32_t* __restrict__ faces,
                                 const uint32_t* __restrict__ mask, const float* __restrict__ canon_area,
                                 float* __restrict__ area_out, TriFrame* __restrict__ out, int with_inverse,
                                 const FrameJob* __restrict__ jobs) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    if (jobs) {   // a batch of frames of one avatar: frame blockIdx.y
        verts = jobs[blockIdx.y].verts;
        out = jobs[blockIdx.y].frames;
    }
    int i0 = faces[f * 3], i1 = faces[f * 3 + 1], i2 = faces[f * 3 + 2];
    V3 a = v3(verts[i0 * 3], verts[i0 * 3 + 1], verts[i0 * 3 + 2]);
    V3 b = v3(verts[i1 * 3], verts[i1 * 3 + 1], verts[i1 * 3 + 2]);
    V3 c = v3(verts[i2 * 3], verts[i2 * 3 + 1], verts[i2 * 3 + 2]);
    uint32_t m = mask ? mask[f] : 15u;
    float area = tri_area_rn(a, b, c);
    if (area_out) area_out[f] = area;
    float s = canon_area ? __fmul_rn(1.0f, __fdiv_rn(area, canon_area[f])) : 1.0f;
    V3 e1 = sub_rn(b, a), e2 = sub_rn(c, a);
    float P[16];
    if (!near_degenerate(e1, e2)) {
        V3 n = normalize_rn(cross_rn(e1, e2));
        V3 bt = normalize_rn(cross_rn(e1, n));
        V3 tg = normalize_rn(cross_rn(bt, n));
        float cols[3][3] = {{tg.x, bt.x, n.x}, {tg.y, bt.y, n.y}, {tg.z, bt.z, n.z}};
        float av[3] = {a.x, a.y, a.z};
        for (int r = 0; r < 3; ++r) {
            for (int q = 0; q < 3; ++q) P[r * 4 + q] = m == 1u ? __fmul_rn(cols[r][q], s) : cols[r][q];
            P[r * 4 + 3] = av[r];
        }
        P[12] = 0.f; P[13] = 0.f; P[14] = 0.f; P[15] = 1.f;
        float Pi[16];
        if (with_inverse) {
            if (!inverse4(P, Pi))
                for (int k = 0; k < 16; ++k) Pi[k] = (k % 5 == 0) ? 1.f : 0.f;
            for (int r = 0; r < 4; ++r) out[f].r[3 + r] = make_float4(Pi[r * 4], Pi[r * 4 + 1], Pi[r * 4 + 2], Pi[r * 4 + 3]);
        }
    } else {
        D3 A = {a.x, a.y, a.z}, E1 = {(double)b.x - a.x, (double)b.y - a.y, (double)b.z - a.z};
        D3 E2 = {(double)c.x - a.x, (double)c.y - a.y, (double)c.z - a.z};
        D3 n = d3norm(d3cross(E1, E2));
        D3 bt = d3norm(d3cross(E1, n));
        D3 tg = d3norm(d3cross(bt, n));
        double cols[3][3] = {{tg.x, bt.x, n.x}, {tg.y, bt.y, n.y}, {tg.z, bt.z, n.z}};
        double av[3] = {A.x, A.y, A.z}, Pd[16];
        for (int r = 0; r < 3; ++r) {
            for (int q = 0; q < 3; ++q) Pd[r * 4 + q] = m == 1u ? cols[r][q] * (double)s : cols[r][q];
            Pd[r * 4 + 3] = av[r];
        }
        Pd[12] = 0.0; Pd[13] = 0.0; Pd[14] = 0.0; Pd[15] = 1.0;
        for (int k = 0; k < 16; ++k) P[k] = (float)Pd[k];
        if (with_inverse) {
            double Pi[16];
            if (!inverse4_d(Pd, Pi))
                for (int k = 0; k < 16; ++k) Pi[k] = (k % 5 == 0) ? 1.0 : 0.0;
            for (int r = 0; r < 4; ++r)
                out[f].r[3 + r] = make_float4((float)Pi[r * 4], (float)Pi[r * 4 + 1], (float)Pi[r * 4 + 2], (float)Pi[r * 4 + 3]);
        }
    }
    for (int r = 0; r < 3; ++r) out[f].r[r] = make_float4(P[r * 4], P[r * 4 + 1], P[r * 4 + 2], P[r * 4 + 3]);
    if (!with_inverse)
        for (int r = 0; r < 4; ++r) out[f].r[3 + r] = make_float4(0.f, 0.f, 0.f, 0.f);
    float cx = __fdiv_rn(__fadd_rn(__fadd_rn(a.x, b.x), c.x), 3.0f);
    float cy = __fdiv_rn(__fadd_rn(__fadd_rn(a.y, b.y), c.y), 3.0f);
    float cz = __fdiv_rn(__fadd_rn(__fadd_rn(a.z, b.z), c.z), 3.0f);
    out[f].r[7] = make_float4(cx, cy, cz, __uint_as_float(m));
}

// --------------------------------------------------------------- BVH build (1 CTA)
struct BvhBuildArgs {
    int F;
    const float* verts;
    const int32_t* faces;
    const TriFrame* frames;
    float4* leaf_tris;
    float4* nodes;        // [max_nodes][7]
    int2* node_range;     // scratch [max_nodes]
    float* node_box;      // scratch [max_nodes][6]
    int* n_nodes_out;
    int max_nodes;
    int np2;
};

__device__ __forceinline__ void box_union(float* b, const float* o) {
    b[0] = fminf(b[0], o[0]); b[1] = fminf(b[1], o[1]); b[2] = fminf(b[2], o[2]);
    b[3] = fmaxf(b[3], o[3]); b[4] = fmaxf(b[4], o[4]); b[5] = fmaxf(b[5], o[5]);
}

// First position in [b, e) whose key has the highest bit in which keys[b] and keys[e-1] differ set:
// the split of a binary radix tree over sorted Morton codes (Karras 2012).
__device__ __forceinline__ int radix_split(const uint64_t* keys, int b, int e) {
    const uint64_t x = keys[b], y = keys[e - 1];
    if (x == y) return (b + e) >> 1;
    const uint64_t m = 1ull << (63 - __clzll((long long)(x ^ y)));
    int lo = b, hi = e - 1;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (keys[mid] & m) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// Up to 4 child ranges of [b, e): split once, then split each half again if it is not a leaf.
__device__ __forceinline__ int child_ranges(const uint64_t* keys, int b, int e, int2* out) {
    const int m = radix_split(keys, b, e);
    int n = 0;
    const int2 h[2] = {make_int2(b, m), make_int2(m, e)};
    for (int i = 0; i < 2; ++i) {
        if (h[i].y - h[i].x > INSTA_LEAF_SIZE) {
            const int q = radix_split(keys, h[i].x, h[i].y);
            out[n++] = make_int2(h[i].x, q);
            out[n++] = make_int2(q, h[i].y);
        } else {
            out[n++] = h[i];
        }
    }
    return n;
}

// Block-wide exclusive scan of cnt[0, n) in place (1024 threads); returns the total.
__device__ int block_scan(int* cnt, int n, int* warp_tot) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int per = (n + nt - 1) / nt;
    const int b = tid * per, e = min(n, b + per);
    int s = 0;
    for (int i = b; i < e; ++i) s += cnt[i];
    int incl = s;
    for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(0xffffffffu, incl, o);
        if ((tid & 31) >= o) incl += v;
    }
    if ((tid & 31) == 31) warp_tot[tid >> 5] = incl;
    __syncthreads();
    if (tid < 32) {
        int v = tid < (nt >> 5) ? warp_tot[tid] : 0;
        int w = v;
        for (int o = 1; o < 32; o <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, w, o);
            if (tid >= o) w += u;
        }
        warp_tot[tid] = w - v;   // exclusive warp offsets
        if (tid == 31) warp_tot[32] = w;
    }
    __syncthreads();
    int run = warp_tot[tid >> 5] + incl - s;
    for (int i = b; i < e; ++i) { int c = cnt[i]; cnt[i] = run; run += c; }
    __syncthreads();
    int total = warp_tot[32];
    __syncthreads();
    return total;
}

// LSD radix sort, in shared memory, of the 64-bit keys (Morton code << 32 | face id) on their
// high word.  The keys start in id order and every pass is stable, so the result is ordered by
// (code, id).  8 passes of 4 bits; the active threads each own ipt consecutive keys, count their
// digits into cnt16[digit][thread], and one block-wide exclusive scan over that digit-major table
// gives every key its destination.  While sorting, key p lives at p + p / 16 (one 8-byte pad per
// 16 keys keeps a thread's consecutive keys off a single bank); the keys end unpadded.  Called by
// all 1024 threads of the block; `keys` holds np2 + np2 / 16 entries.
__device__ __forceinline__ int padded(int p) { return p + (p >> 4); }

__device__ void block_radix_sort_hi(uint64_t* keys, int np2, uint16_t* cnt16, int* warp_tot) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int active = np2 < 1024 ? np2 : 1024;
    const int ipt = np2 / active;   // 1..16
    const bool owns = tid < active;
    // pad: striped, so each step moves 32 consecutive keys; reads all land before the writes
    {
        uint64_t v[16];
        for (int i = 0; i < ipt; ++i) v[i] = tid < active ? keys[i * active + tid] : 0ull;
        __syncthreads();
        for (int i = 0; i < ipt; ++i) if (tid < active) keys[padded(i * active + tid)] = v[i];
        __syncthreads();
    }
    for (int shift = 32; shift < 64; shift += 4) {
#pragma unroll
        for (int d = 0; d < 16; ++d) cnt16[d * 1024 + tid] = 0;
        if (owns)
            for (int i = 0; i < ipt; ++i) ++cnt16[(int)((keys[padded(tid * ipt + i)] >> shift) & 15u) * 1024 + tid];
        __syncthreads();
        // exclusive scan over the 16 x 1024 table in digit-major order, 16 entries per thread
        uint32_t loc[16], sum = 0;
#pragma unroll
        for (int e = 0; e < 16; ++e) { loc[e] = sum; sum += cnt16[tid * 16 + e]; }
        uint32_t x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[warp] = (int)x;
        __syncthreads();
        if (warp == 0) {
            uint32_t t = (uint32_t)warp_tot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            warp_tot[lane] = (int)t;
        }
        __syncthreads();
        const uint32_t base = (warp ? (uint32_t)warp_tot[warp - 1] : 0u) + x - sum;
#pragma unroll
        for (int e = 0; e < 16; ++e) cnt16[tid * 16 + e] = (uint16_t)(base + loc[e]);
        __syncthreads();
        uint64_t kk[16];
        if (owns)
            for (int i = 0; i < ipt; ++i) kk[i] = keys[padded(tid * ipt + i)];
        __syncthreads();   // every key is in registers before any is overwritten
        if (owns)
            for (int i = 0; i < ipt; ++i) {
                const int d = (int)((kk[i] >> shift) & 15u);
                keys[padded(cnt16[d * 1024 + tid]++)] = kk[i];
            }
        __syncthreads();
    }
    // unpad (striped)
    {
        uint64_t v[16];
        for (int i = 0; i < ipt; ++i) v[i] = tid < active ? keys[padded(i * active + tid)] : 0ull;
        __syncthreads();
        for (int i = 0; i < ipt; ++i) if (tid < active) keys[i * active + tid] = v[i];
        __syncthreads();
    }
}

// LBVH: sort triangles by the 30-bit Morton code of their centroid (ties by id), build the
// binary radix tree top-down level by level and collapse every two binary levels into one
// 4-wide node; boxes are then filled bottom-up.  Leaves hold <= INSTA_LEAF_SIZE triangles (the
// reference's build uses N_PRIMITIVES_LEAF = 2, src/tiny_mesh.cu:28-32; query results do not
// depend on the structure).
__global__ void __launch_bounds__(1024) bvh_build_kernel(BvhBuildArgs one, const BvhBuildArgs* __restrict__ many) {
    const BvhBuildArgs a = many ? many[blockIdx.x] : one;   // a batch builds one frame per CTA
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t* keys = reinterpret_cast<uint64_t*>(smem_raw);
    int* cnt = reinterpret_cast<int*>(smem_raw + (size_t)(a.np2 + a.np2 / 16) * 8);   // per node of the current level
    __shared__ float red[6][32];
    __shared__ float ext[6];
    __shared__ int warp_tot[33];
    __shared__ int lvl_off[66];
    __shared__ int n_levels;
    const int tid = threadIdx.x, nt = blockDim.x;
    // 1. centroid bounds
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int f = tid; f < a.F; f += nt) {
        float4 c = a.frames[f].r[7];
        lo[0] = fminf(lo[0], c.x); lo[1] = fminf(lo[1], c.y); lo[2] = fminf(lo[2], c.z);
        hi[0] = fmaxf(hi[0], c.x); hi[1] = fmaxf(hi[1], c.y); hi[2] = fmaxf(hi[2], c.z);
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    if ((tid & 31) == 0)
        for (int k = 0; k < 3; ++k) { red[k][tid >> 5] = lo[k]; red[3 + k][tid >> 5] = hi[k]; }
    __syncthreads();
    if (tid < 32) {
        int nw = nt >> 5;
        for (int k = 0; k < 3; ++k) {
            lo[k] = tid < nw ? red[k][tid] : 3.4e38f;
            hi[k] = tid < nw ? red[3 + k][tid] : -3.4e38f;
        }
        for (int o = 16; o > 0; o >>= 1)
            for (int k = 0; k < 3; ++k) {
                lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
                hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
            }
        if (tid == 0)
            for (int k = 0; k < 3; ++k) { ext[k] = lo[k]; float e = hi[k] - lo[k]; ext[3 + k] = e > 0.f ? 1.f / e : 0.f; }
    }
    __syncthreads();
    // 2. Morton keys (code << 32 | face id: unique)
    for (int i = tid; i < a.np2; i += nt) {
        uint64_t key = ~0ull;
        if (i < a.F) {
            float4 c = a.frames[i].r[7];
            float q[3] = {(c.x - ext[0]) * ext[3], (c.y - ext[1]) * ext[4], (c.z - ext[2]) * ext[5]};
            uint32_t v[3];
            for (int k = 0; k < 3; ++k) v[k] = (uint32_t)fminf(fmaxf(q[k] * 1024.f, 0.f), 1023.f);
            key = ((uint64_t)morton3d(v[0], v[1], v[2]) << 32) | (uint32_t)i;
        }
        keys[i] = key;
    }
    __syncthreads();
    // 3. sort ascending (the count region doubles as the radix counters)
    block_radix_sort_hi(keys, a.np2, reinterpret_cast<uint16_t*>(cnt), warp_tot);
    // 4. the face of each Morton slot; tri_record_kernel builds the records across the GPU
    for (int s = tid; s < a.F; s += nt) a.leaf_tris[(size_t)s * INSTA_TRI_F4 + 2].y = __uint_as_float((uint32_t)(keys[s] & 0xffffffffu));
    // 5. topology, top-down, one level of 4-wide nodes at a time
    if (tid == 0) {
        a.node_range[0] = make_int2(0, a.F);
        lvl_off[0] = 0;
        lvl_off[1] = 1;
        n_levels = 1;
    }
    __syncthreads();
    for (int L = 0; L < 64; ++L) {
        const int lb = lvl_off[L], le = lvl_off[L + 1];
        if (lb == le) break;
        for (int n = lb + tid; n < le; n += nt) {
            int2 r = a.node_range[n];
            int2 ch[4];
            int nc = r.y - r.x > INSTA_LEAF_SIZE ? child_ranges(keys, r.x, r.y, ch) : 0;
            if (nc == 0) { ch[0] = r; nc = 1; }   // a root that is already a leaf
            int inner = 0;
            for (int i = 0; i < nc; ++i) inner += (ch[i].y - ch[i].x > INSTA_LEAF_SIZE) ? 1 : 0;
            cnt[n - lb] = inner;
        }
        __syncthreads();
        const int total = block_scan(cnt, le - lb, warp_tot);
        for (int n = lb + tid; n < le; n += nt) {
            int2 r = a.node_range[n];
            int2 ch[4];
            int nc = r.y - r.x > INSTA_LEAF_SIZE ? child_ranges(keys, r.x, r.y, ch) : 0;
            if (nc == 0) { ch[0] = r; nc = 1; }
            int next = le + cnt[n - lb];
            int refs[4] = {-1, -1, -1, -1};
            for (int i = 0; i < nc; ++i) {
                if (ch[i].y - ch[i].x > INSTA_LEAF_SIZE) {
                    if (next < a.max_nodes) { a.node_range[next] = ch[i]; refs[i] = next; }
                    ++next;
                } else {
                    refs[i] = (int)(INSTA_LEAF_BIT | ((uint32_t)ch[i].x << 3) | (uint32_t)(ch[i].y - ch[i].x));
                }
            }
            reinterpret_cast<int4*>(a.nodes)[(size_t)n * 7 + 6] = make_int4(refs[0], refs[1], refs[2], refs[3]);
        }
        __syncthreads();
        if (tid == 0) {
            lvl_off[L + 2] = min(le + total, a.max_nodes);
            n_levels = L + 1;
        }
        __syncthreads();
    }
    // 6. boxes, bottom-up
    for (int L = n_levels - 1; L >= 0; --L) {
        const int lb = lvl_off[L], le = lvl_off[L + 1];
        for (int n = lb + tid; n < le; n += nt) {
            const int4 refs = reinterpret_cast<const int4*>(a.nodes)[(size_t)n * 7 + 6];
            const int rr[4] = {refs.x, refs.y, refs.z, refs.w};
            float mn[3][4], mx[3][4];
            float nb[6] = {3.4e38f, 3.4e38f, 3.4e38f, -3.4e38f, -3.4e38f, -3.4e38f};
            for (int i = 0; i < 4; ++i) {
                float cb[6] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000),
                               -__int_as_float(0x7f800000), -__int_as_float(0x7f800000), -__int_as_float(0x7f800000)};
                if (rr[i] != -1) {
                    if ((uint32_t)rr[i] & INSTA_LEAF_BIT) {
                        const uint32_t first = ((uint32_t)rr[i] & ~(uint32_t)INSTA_LEAF_BIT) >> 3, count = (uint32_t)rr[i] & 7u;
                        for (uint32_t t = first; t < first + count; ++t) {
                            const uint32_t f = (uint32_t)(keys[t] & 0xffffffffu);
                            const float* A = a.verts + a.faces[f * 3] * 3;
                            const float* B = a.verts + a.faces[f * 3 + 1] * 3;
                            const float* Cv = a.verts + a.faces[f * 3 + 2] * 3;
                            float pts[9] = {A[0], A[1], A[2], B[0], B[1], B[2], Cv[0], Cv[1], Cv[2]};
                            for (int p = 0; p < 3; ++p) {
                                float pb[6] = {pts[p * 3], pts[p * 3 + 1], pts[p * 3 + 2], pts[p * 3], pts[p * 3 + 1], pts[p * 3 + 2]};
                                box_union(cb, pb);
                            }
                        }
                    } else {
                        for (int k = 0; k < 6; ++k) cb[k] = a.node_box[(size_t)rr[i] * 6 + k];
                    }
                    box_union(nb, cb);
                }
                for (int k = 0; k < 3; ++k) { mn[k][i] = cb[k]; mx[k][i] = cb[3 + k]; }
            }
            float4* nd = a.nodes + (size_t)n * 7;
            for (int k = 0; k < 3; ++k) {
                nd[k] = make_float4(mn[k][0], mn[k][1], mn[k][2], mn[k][3]);
                nd[3 + k] = make_float4(mx[k][0], mx[k][1], mx[k][2], mx[k][3]);
            }
            for (int k = 0; k < 6; ++k) a.node_box[(size_t)n * 6 + k] = nb[k];
        }
        __syncthreads();
    }
    if (tid == 0) *a.n_nodes_out = lvl_off[n_levels];
}

// --------------------------------------------------------------------- occupancy
// mark_flame_density_grid (ngp/src/testbed_nerf.cu:364-389) over the deformed mesh, fused with
// grid_to_bitfield (:585-609): one thread per cell, a nearest-triangle query bounded by the marking
// radius; a warp covers 32 Morton-consecutive cells and writes their bits as one 32-bit word.
// One cell per thread (not eight) spreads the few expensive cells near the surface over many warps;
// per-thread queries beat a shared warp traversal here because most cells leave at the root.
__global__ void __launch_bounds__(256) occupancy_kernel(FrameView fr, double radius, float bound, uint8_t* __restrict__ bits, uint32_t* err) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t n_warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t base = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32u; base < GRID3; base += n_warps * 32u) {
        const uint32_t cell = base + lane;
        const uint32_t x = morton_invert(cell), y = morton_invert(cell >> 1), z = morton_invert(cell >> 2);
        const V3 p = v3(__fdiv_rn((float)x + 0.5f, 128.f), __fdiv_rn((float)y + 0.5f, 128.f), __fdiv_rn((float)z + 0.5f, 128.f));
        const Nearest r = nearest_bvh(fr, p, bound, -1, -1, err);
        bool on = false;
        if (r.id >= 0) {
            uint32_t m;
            load_centroid(fr.frames, (uint32_t)r.id, &m);
            on = (double)__fsqrt_rn(r.d2) < radius && m != 0u;
        }
        // bit j of byte b is cell 8b + j: the ballot word is the four bytes of this warp's cells
        const uint32_t word = __ballot_sync(0xffffffffu, on);
        if (lane == 0) reinterpret_cast<uint32_t*>(bits)[base >> 5] = word;
        // bitfield_max_pool (:611-632) for mips 1..7 at once: a mip-l cell is occupied iff some
        // occupied mip-0 cell maps onto it under l halvings toward the centre (x -> x / 2 + 32)
        if (on) {
            uint32_t cx = x, cy = y, cz = z;
            for (uint32_t l = 1; l < 8; ++l) {
                cx = cx / 2 + GRID / 4; cy = cy / 2 + GRID / 4; cz = cz / 2 + GRID / 4;
                const uint32_t c = l * GRID3 + morton3d(cx, cy, cz);
                atomicOr(reinterpret_cast<uint32_t*>(bits) + (c >> 5), 1u << (c & 31u));
            }
        }
    }
}

// bitfield_max_pool (:611-632) for one mip level; `next` must be zeroed.
__global__ void maxpool_kernel(const uint8_t* __restrict__ prev, uint8_t* __restrict__ next) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= GRID3 / 64) return;
    uint8_t bits = 0;
    for (int j = 0; j < 8; ++j) bits |= prev[i * 8 + j] > 0 ? (uint8_t)(1u << j) : 0;
    uint32_t x = morton_invert(i) + GRID / 8, y = morton_invert(i >> 1) + GRID / 8, z = morton_invert(i >> 2) + GRID / 8;
    next[morton3d(x, y, z)] |= bits;
}

// ---------------------------------------------------------------- density grid -> bitfield
// update_density_grid_mean_and_bitfield (ngp/src/testbed_nerf.cu:2863-2878) for a loaded grid.
// The mean of max(v, 0) / 128^3 over cascade 0 is reduced deterministically: fixed per-block
// trees, then one block over the block sums in index order.
constexpr uint32_t kMeanBlocks = 1024;

__global__ void __launch_bounds__(256) density_convert_kernel(const uint16_t* __restrict__ half_grid, float* __restrict__ grid, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        grid[i] = __half2float(__ushort_as_half(half_grid[i]));
}

__global__ void __launch_bounds__(256) density_mean_partial_kernel(const float* __restrict__ grid, float* __restrict__ partial) {
    __shared__ float red[256];
    const uint32_t per = GRID3 / kMeanBlocks;   // 2048 cells per block
    float acc = 0.f;
    for (uint32_t k = threadIdx.x; k < per; k += blockDim.x)
        acc = __fadd_rn(acc, __fdiv_rn(fmaxf(grid[blockIdx.x * per + k], 0.f), (float)GRID3));
    red[threadIdx.x] = acc;
    __syncthreads();
    for (uint32_t o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] = __fadd_rn(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(256) density_mean_final_kernel(float* __restrict__ partial, float* __restrict__ thresh_out) {
    __shared__ float red[256];
    float acc = 0.f;
    for (uint32_t k = threadIdx.x; k < kMeanBlocks; k += blockDim.x) acc = __fadd_rn(acc, partial[k]);
    red[threadIdx.x] = acc;
    __syncthreads();
    for (uint32_t o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] = __fadd_rn(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) thresh_out[0] = fminf(0.01f, red[0]);   // NERF_MIN_OPTICAL_THICKNESS
}

// grid_to_bitfield (:585-609): one byte (8 Morton-consecutive cells) per thread over all mips.
__global__ void __launch_bounds__(256) grid_to_bitfield_kernel(const float* __restrict__ grid, uint32_t n_cascades,
                                                               const float* __restrict__ thresh, uint8_t* __restrict__ bits) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= GRID3 / 8 * 8) return;
    uint8_t b = 0;
    if (i < GRID3 / 8 * n_cascades) {
        const float t = *thresh;
        const float4 lo = reinterpret_cast<const float4*>(grid)[(size_t)i * 2];
        const float4 hi = reinterpret_cast<const float4*>(grid)[(size_t)i * 2 + 1];
        const float v[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
#pragma unroll
        for (int j = 0; j < 8; ++j) b |= v[j] > t ? (uint8_t)(1u << j) : (uint8_t)0;
    }
    bits[i] = b;
}

// ------------------------------------------------------------- density-grid maintenance
// update_density_grid_nerf (ngp/src/testbed_nerf.cu:2774-2861) with INSTA's deformation hook:
//   grid_samples_kernel  generate_grid_samples_nerf_nonuniform (:487-516) for the uniform and the
//                        non-uniform set in one launch (the reference hands both calls the same
//                        generator state)
//   warp_random_kernel   warp_random_samples (src/core.cu:528-579): a random tracked frame per
//                        sample, its nearest triangle, the deformed -> canonical position
//   (encode + MLPs)      NerfNetwork::density at the canonical positions
//   splat_max_kernel     splat_grid_samples_nerf_max_nearest_neighbor (:518-531)
//   ema_kernel           ema_grid_samples_nerf (:554-583): max(previous * decay, new), negative
//                        cells (never updated) kept
__global__ void __launch_bounds__(256) grid_samples_kernel(uint32_t n_uniform, uint32_t n_nonuniform, Pcg32 rng, uint32_t step,
                                                           float3 aabb_min, float3 aabb_max, const float* __restrict__ grid,
                                                           uint32_t n_cascades, float* __restrict__ coords, uint32_t stride,
                                                           uint32_t* __restrict__ indices) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_uniform + n_nonuniform) return;
    const bool uniform = i < n_uniform;
    const uint32_t li = uniform ? i : i - n_uniform, ne = uniform ? n_uniform : n_nonuniform;
    const float thresh = uniform ? -0.01f : 0.01f;   // NERF_MIN_OPTICAL_THICKNESS for the non-uniform set
    Pcg32 r = rng;
    r.advance((int64_t)(uint32_t)(li * 4u));
    const uint32_t level = (uint32_t)__fmul_rn(r.next_float(), (float)n_cascades) % n_cascades;
    uint32_t idx = 0;
    for (uint32_t j = 0; j < 10; ++j) {
        idx = ((li + step * ne) * 56924617u + j * 19349663u + 96925573u) % GRID3;
        idx += level * GRID3;
        if (grid[idx] > thresh) break;
    }
    const uint32_t cell = idx % GRID3;
    const float cc[3] = {(float)morton_invert(cell), (float)morton_invert(cell >> 1), (float)morton_invert(cell >> 2)};
    const float rr[3] = {r.next_float(), r.next_float(), r.next_float()};
    const float scale = scalbnf(1.0f, (int)level);
    const float mn[3] = {aabb_min.x, aabb_min.y, aabb_min.z}, mx[3] = {aabb_max.x, aabb_max.y, aabb_max.z};
    float* c = coords + (size_t)i * stride;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float pos = __fadd_rn(__fmul_rn(__fsub_rn(__fdiv_rn(__fadd_rn(cc[k], rr[k]), (float)GRID), 0.5f), scale), 0.5f);
        c[k] = __fdiv_rn(__fsub_rn(pos, mn[k]), __fsub_rn(mx[k], mn[k]));   // warp_position = aabb.relative_pos
        c[8 + k] = 0.5f;                                                     // no direction (density only)
    }
    c[3] = 0.f;   // warp_dt(MIN_CONE_STEPSIZE)
    c[4] = 0.f;
    indices[i] = idx;
}

__global__ void __launch_bounds__(256) warp_random_kernel(const FrameView* __restrict__ frames, uint32_t n_frames, DeformView dv,
                                                          float* __restrict__ coords, uint32_t stride, uint32_t n, Pcg32 rng,
                                                          uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float* c = coords + (size_t)i * stride;
    const V3 p = v3(c[0], c[1], c[2]);
    Pcg32 r = rng;
    r.advance((int64_t)(uint32_t)(i * n_frames));
    const uint32_t fid = (uint32_t)__fmul_rn(r.next_float(), (float)n_frames);
    if (fid >= n_frames || frames[fid].n_tris == 0) { atomicOr(err, INSTA_DEVERR_NO_TRI); return; }
    const FrameView& fr = frames[fid];
    const Nearest q = nearest_triangle(fr, p, err);
    if (q.id < 0) { atomicOr(err, INSTA_DEVERR_NO_TRI); return; }
    float o[3];
    map_to_canonical(dv, fr.frames, (uint32_t)q.id, p, nullptr, o, nullptr, nullptr);
    c[0] = o[0]; c[1] = o[1]; c[2] = o[2];
}

__global__ void __launch_bounds__(256) splat_max_kernel(uint32_t n, const uint32_t* __restrict__ indices, const uint2* __restrict__ out,
                                                        const float4* __restrict__ out_f32, int f32_out, float* __restrict__ tmp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float raw;
    if (f32_out) {
        raw = out_f32[i].w;
    } else {
        const uint2 u = out[i];
        raw = __half2float(__ushort_as_half((unsigned short)(u.y >> 16)));
    }
    const float thickness = __fmul_rn(__expf(raw), MIN_CONE);   // network_to_density (exponential) x the smallest step
    atomicMax(reinterpret_cast<uint32_t*>(tmp) + indices[i], __float_as_uint(thickness));
}

__global__ void __launch_bounds__(256) ema_kernel(uint32_t n, float decay, float* __restrict__ grid, const float* __restrict__ tmp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float prev = grid[i];
    grid[i] = prev < 0.f ? prev : fmaxf(__fmul_rn(prev, decay), tmp[i]);
}

// ---------------------------------------------------------------- canonical map
__global__ void __launch_bounds__(256) canonical_map_soa_kernel(FrameView fr, DeformView dv, const float* __restrict__ pts, int64_t n,
                                                                int32_t* __restrict__ out_idx, float* __restrict__ out_canon, uint32_t* err) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        V3 p = v3(pts[i * 3], pts[i * 3 + 1], pts[i * 3 + 2]);
        Nearest r = nearest_triangle(fr, p, err);
        out_idx[i] = r.id;
        if (r.id < 0) {
            atomicOr(err, INSTA_DEVERR_NO_TRI);
            out_canon[i * 3] = p.x; out_canon[i * 3 + 1] = p.y; out_canon[i * 3 + 2] = p.z;
            continue;
        }
        float o[3];
        map_to_canonical(dv, fr.frames, (uint32_t)r.id, p, nullptr, o, nullptr, nullptr);
        out_canon[i * 3] = o[0]; out_canon[i * 3 + 1] = o[1]; out_canon[i * 3 + 2] = o[2];
    }
}

// warp (src/core.cu:442-526) in place on NerfCoordinate records (NGP/nerf.h:86-115); the frame
// is fixed (frame_id >= 0, render_deformed) or read from `holder` (surface_closest_point).
__global__ void __launch_bounds__(256) canonical_map_coords_kernel(const FrameView* __restrict__ frames, uint32_t n_frames, DeformView dv,
                                                                   float* __restrict__ coords, uint32_t stride, uint32_t n_extra, int64_t n,
                                                                   int32_t frame_id, uint32_t* err, const uint32_t* __restrict__ n_dev) {
    if (n_dev && (int64_t)*n_dev < n) n = (int64_t)*n_dev;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float* c = coords + i * stride;
        float holder = c[4];
        if (holder < 0.f) continue;
        uint32_t fid = frame_id < 0 ? (uint32_t)holder : (uint32_t)frame_id;
        if (fid >= n_frames) continue;
        V3 p = v3(c[0], c[1], c[2]);
        if (!box_contains(dv.aabb_min, dv.aabb_max, p)) continue;
        const FrameView& fr = frames[fid];
        if (fr.n_tris == 0) continue;
        Nearest r = nearest_triangle(fr, p, err);
        if (r.id < 0) { atomicOr(err, INSTA_DEVERR_NO_TRI); continue; }
        float pos[3], dir[3], dw[3] = {c[8], c[9], c[10]};
        uint32_t mask;
        map_to_canonical(dv, fr.frames, (uint32_t)r.id, p, dw, pos, dir, &mask);
        c[0] = pos[0]; c[1] = pos[1]; c[2] = pos[2];
        c[8] = dir[0]; c[9] = dir[1]; c[10] = dir[2];
        if (mask != 7u)
            for (uint32_t m = 0; m < n_extra; ++m) c[stride - n_extra + m] = 1.f;
    }
}

static int sm_count_frames() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    return sms;
}

// ------------------------------------------------------------------- launchers
// The Morton-ordered triangle records from the face id the build left in each slot: vertices
// plus the point-independent terms of the exact distance (tri_record).  A batch passes the build
// arguments of every frame (blockIdx.y picks one).
__global__ void tri_record_kernel(BvhBuildArgs one, const BvhBuildArgs* __restrict__ many) {
    const BvhBuildArgs& a = many ? many[blockIdx.y] : one;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.F) return;
    float4* dst = a.leaf_tris + (size_t)s * INSTA_TRI_F4;
    const uint32_t f = __float_as_uint(dst[2].y);
    const float* A = a.verts + a.faces[f * 3] * 3;
    const float* B = a.verts + a.faces[f * 3 + 1] * 3;
    const float* C = a.verts + a.faces[f * 3 + 2] * 3;
    tri_record(v3(A[0], A[1], A[2]), v3(B[0], B[1], B[2]), v3(C[0], C[1], C[2]), f, dst);
    tri_bound(A, B, C, a.leaf_tris + (size_t)a.F * INSTA_TRI_F4 + (size_t)s * 2);
}

cudaError_t launch_tri_frames(int F, const float* verts, const int32_t* faces, const uint32_t* mask, const float* canon_area,
                              float* area_out, TriFrame* out, int with_inverse, cudaStream_t s) {
    tri_frame_kernel<<<(F + 255) / 256, 256, 0, s>>>(F, verts, faces, mask, canon_area, area_out, out, with_inverse, nullptr);
    return cudaGetLastError();
}

size_t bvh_scratch_bytes(int F) { return (size_t)F * (sizeof(int2) + 6 * sizeof(float)) + 16; }

static BvhBuildArgs bvh_args(const FrameView& fv, const float* verts, const int32_t* faces, void* scratch) {
    BvhBuildArgs a;
    a.F = fv.n_tris;
    a.verts = verts; a.faces = faces; a.frames = fv.frames;
    a.leaf_tris = const_cast<float4*>(fv.leaf_tris);
    a.nodes = const_cast<float4*>(fv.nodes);
    a.max_nodes = fv.n_nodes;
    a.node_range = reinterpret_cast<int2*>(scratch);
    a.node_box = reinterpret_cast<float*>(reinterpret_cast<char*>(scratch) + (size_t)fv.n_tris * sizeof(int2));
    a.n_nodes_out = reinterpret_cast<int*>(reinterpret_cast<char*>(scratch) + (size_t)fv.n_tris * (sizeof(int2) + 6 * sizeof(float)));
    int np2 = 2;
    while (np2 < fv.n_tris) np2 <<= 1;
    a.np2 = np2;
    return a;
}

static size_t bvh_smem(int F) {
    int np2 = 2;
    while (np2 < F) np2 <<= 1;
    // keys, then the per-node counts of the topology pass, which first serve as the 16 x 1024
    // 16-bit radix counters
    return (size_t)(np2 + np2 / 16) * 8 + std::max((size_t)F * 4, (size_t)16 * 1024 * 2) + 16;
}

cudaError_t launch_bvh_build(const FrameView& fv, const float* verts, const int32_t* faces, void* scratch, cudaStream_t s) {
    const size_t smem = bvh_smem(fv.n_tris);
    cudaError_t e = cudaFuncSetAttribute(bvh_build_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const BvhBuildArgs args = bvh_args(fv, verts, faces, scratch);
    bvh_build_kernel<<<1, 1024, smem, s>>>(args, nullptr);
    tri_record_kernel<<<(fv.n_tris + 255) / 256, 256, 0, s>>>(args, nullptr);
    return cudaGetLastError();
}

size_t frame_batch_table_bytes(int n) { return (size_t)n * (sizeof(FrameJob) + sizeof(BvhBuildArgs)); }

cudaError_t launch_frames_batch(int n, int F, const FrameView* views, const float* const* verts, const int32_t* faces,
                                const uint32_t* mask, const float* canon_area, void* scratch, void* table, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    std::vector<FrameJob> jobs((size_t)n);
    std::vector<BvhBuildArgs> args((size_t)n);
    for (int i = 0; i < n; ++i) {
        jobs[(size_t)i].verts = verts[i];
        jobs[(size_t)i].frames = const_cast<TriFrame*>(views[i].frames);
        args[(size_t)i] = bvh_args(views[i], verts[i], faces, static_cast<char*>(scratch) + (size_t)i * bvh_scratch_bytes(F));
    }
    FrameJob* djobs = static_cast<FrameJob*>(table);
    BvhBuildArgs* dargs = reinterpret_cast<BvhBuildArgs*>(static_cast<char*>(table) + (size_t)n * sizeof(FrameJob));
    // pageable sources: the copies are staged before these calls return
    cudaError_t e = cudaMemcpyAsync(djobs, jobs.data(), jobs.size() * sizeof(FrameJob), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dargs, args.data(), args.size() * sizeof(BvhBuildArgs), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    tri_frame_kernel<<<dim3((F + 255) / 256, n), 256, 0, s>>>(F, nullptr, faces, mask, canon_area, nullptr, nullptr, 1, djobs);
    const size_t smem = bvh_smem(F);
    e = cudaFuncSetAttribute(bvh_build_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    bvh_build_kernel<<<n, 1024, smem, s>>>(BvhBuildArgs{}, dargs);
    tri_record_kernel<<<dim3((F + 255) / 256, n), 256, 0, s>>>(BvhBuildArgs{}, dargs);
    return cudaGetLastError();
}

cudaError_t launch_occupancy(const FrameView& fv, double radius, uint8_t* bitfield, uint32_t* err, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(bitfield + GRID3 / 8, 0, (size_t)7 * GRID3 / 8, s);
    if (e != cudaSuccess) return e;
    float bound = (float)(radius * radius * 1.0001);
    occupancy_kernel<<<sm_count_frames() * 8, 256, 0, s>>>(fv, radius, bound, bitfield, err);
    return cudaGetLastError();
}

size_t density_scratch_bytes(uint32_t n_cascades) { return (size_t)n_cascades * GRID3 * 4 + (kMeanBlocks + 4) * 4; }

cudaError_t launch_density_grid(const void* grid, int fp16, uint32_t n_cascades, void* scratch, uint8_t* bitfield, cudaStream_t s) {
    float* g = static_cast<float*>(scratch);
    float* partial = g + (size_t)n_cascades * GRID3;
    float* thresh = partial + kMeanBlocks;
    const uint32_t n = n_cascades * GRID3;
    cudaError_t e = cudaSuccess;
    if (fp16) density_convert_kernel<<<sm_count_frames() * 8, 256, 0, s>>>(static_cast<const uint16_t*>(grid), g, n);
    else e = cudaMemcpyAsync(g, grid, (size_t)n * 4, cudaMemcpyDefault, s);
    if (e != cudaSuccess) return e;
    density_mean_partial_kernel<<<kMeanBlocks, 256, 0, s>>>(g, partial);
    density_mean_final_kernel<<<1, 256, 0, s>>>(partial, thresh);
    grid_to_bitfield_kernel<<<GRID3 / 8 * 8 / 256, 256, 0, s>>>(g, n_cascades, thresh, bitfield);
    for (int lvl = 1; lvl < 8; ++lvl)
        maxpool_kernel<<<(GRID3 / 64 + 255) / 256, 256, 0, s>>>(bitfield + (size_t)(lvl - 1) * GRID3 / 8, bitfield + (size_t)lvl * GRID3 / 8);
    return cudaGetLastError();
}

cudaError_t launch_grid_samples(uint32_t n_uniform, uint32_t n_nonuniform, uint64_t rng_state, uint64_t rng_inc, uint32_t step,
                                const float* aabb_min, const float* aabb_max, const float* grid, uint32_t n_cascades, float* coords,
                                uint32_t stride, uint32_t* indices, cudaStream_t s) {
    const uint32_t n = n_uniform + n_nonuniform;
    if (n == 0) return cudaSuccess;
    Pcg32 r{rng_state, rng_inc};
    grid_samples_kernel<<<(n + 255) / 256, 256, 0, s>>>(n_uniform, n_nonuniform, r, step, make_float3(aabb_min[0], aabb_min[1], aabb_min[2]),
                                                        make_float3(aabb_max[0], aabb_max[1], aabb_max[2]), grid, n_cascades, coords, stride,
                                                        indices);
    return cudaGetLastError();
}

cudaError_t launch_warp_random(const FrameView* frames_dev, uint32_t n_frames, const DeformView& dv, float* coords, uint32_t stride,
                               uint32_t n, uint64_t rng_state, uint64_t rng_inc, uint32_t* err, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    Pcg32 r{rng_state, rng_inc};
    warp_random_kernel<<<(n + 255) / 256, 256, 0, s>>>(frames_dev, n_frames, dv, coords, stride, n, r, err);
    return cudaGetLastError();
}

cudaError_t launch_splat_ema(uint32_t n, const uint32_t* indices, const uint2* out, const float4* out_f32, int f32_out, float* tmp,
                             float* grid, uint32_t n_cells, float decay, cudaStream_t s) {
    if (n) splat_max_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, indices, out, out_f32, f32_out, tmp);
    ema_kernel<<<(n_cells + 255) / 256, 256, 0, s>>>(n_cells, decay, grid, tmp);
    return cudaGetLastError();
}

cudaError_t launch_canonical_map_soa(const FrameView& fv, const DeformView& dv, const float* pts, int64_t n, int32_t* out_idx,
                                     float* out_canon, uint32_t* err, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    int grid = (int)(blocks < sm_count_frames() * 16 ? blocks : sm_count_frames() * 16);
    canonical_map_soa_kernel<<<grid, 256, 0, s>>>(fv, dv, pts, n, out_idx, out_canon, err);
    return cudaGetLastError();
}

cudaError_t launch_canonical_map_coords(const FrameView* frames_dev, uint32_t n_frames, const DeformView& dv, float* coords,
                                        uint32_t stride, uint32_t n_extra, int64_t n, int32_t frame_id, uint32_t* err, cudaStream_t s,
                                        const uint32_t* n_dev) {
    if (n <= 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    int grid = (int)(blocks < sm_count_frames() * 16 ? blocks : sm_count_frames() * 16);
    canonical_map_coords_kernel<<<grid, 256, 0, s>>>(frames_dev, n_frames, dv, coords, stride, n_extra, n, frame_id, err, n_dev);
    return cudaGetLastError();
}

}  // namespace insta
