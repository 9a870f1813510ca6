// render_kernels.cu -- the render path as a device-driven wavefront, one round per STEPS samples:
//   ray_init_kernel       camera rays in 8x4-pixel tiles, render-box entry, jitter, first occupied cell
//   march_kernel          per alive ray, up to STEPS samples through the occupancy grid; a warp's
//                         samples are written step-major so 32 neighbouring rays' k-th samples sit
//                         together in the compacted sample stream
//   nearest_stage_kernel  per 32 sorted samples: warp-cooperative nearest triangle
//   map_encode_kernel     per sample: deformed->canonical map, hash encode + SH written as
//                         ready-made tensor-core operand tiles
//   mlp256_kernel         density + colour MLPs on 128-sample tiles (tcgen05, TMEM accumulators)
//   composite_kernel      front-to-back compositing, early termination, shading, compaction
// Ray lists and counts stay on the device; the host only decides when to stop issuing rounds.
#include "device_common.cuh"
#include "mlp_tiles.cuh"
#include "kernels.h"

namespace insta {

__device__ __forceinline__ float srgb_to_linear(float s) { return s <= 0.04045f ? s / 12.92f : powf((s + 0.055f) / 1.055f, 2.4f); }

__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred) {
    const uint32_t mask = __ballot_sync(0xffffffffu, pred);
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t base = 0;
    if (mask) {
        const int leader = __ffs(mask) - 1;
        if ((int)lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
        base = __shfl_sync(0xffffffffu, base, leader);
    }
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ void write_pixel(const RenderView& rv, float* out_rgba, float* out_depth, uint32_t pix, float4 rgba, float depth) {
    // shade_kernel_nerf (ngp/src/testbed_nerf.cu:1794-1827) into a zeroed frame buffer
    if (rgba.w > 0.001f) {
        float o[4] = {rgba.x, rgba.y, rgba.z, rgba.w};
        if (!rv.linear_colors) for (int k = 0; k < 3; ++k) o[k] = srgb_to_linear(o[k]);
        reinterpret_cast<float4*>(out_rgba)[pix] = make_float4(o[0], o[1], o[2], o[3]);
        if (o[3] > 0.2f) out_depth[pix] = depth;
    }
}

// ------------------------------------------------------------------ ray init
// Rays are issued in 8x4-pixel tiles, one tile per warp: the samples a warp later takes at one
// step then lie close together, so the warp-cooperative nearest-triangle search visits a small
// union of BVH nodes (about 40% fewer than for 32x1 pixel rows).
constexpr uint32_t kTileW = 8, kTileH = 4;

// Entry k of the launch's init list that owns ray tile `tile`: the last k with init_tile[k] <= tile.
__device__ __forceinline__ uint32_t init_entry(const uint32_t* init_tile, uint32_t n_init, uint32_t tile) {
    uint32_t lo = 0, hi = n_init;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(init_tile + mid) <= tile) lo = mid; else hi = mid;
    }
    return lo;
}

// Warp-aggregated add of `delta` per lane to the counter of each lane's request (lanes may belong
// to different requests): one atomic per distinct request in the warp.
__device__ __forceinline__ void count_per_request(uint32_t* counters, uint32_t req, bool pred, int delta) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t key = pred ? req : 0xffffffffu;
    const uint32_t peers = __match_any_sync(0xffffffffu, key);
    if (pred && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(counters + req, (uint32_t)(delta * __popc(peers)));
}

__global__ void ray_init_kernel(const __grid_constant__ WaveArgs A, uint32_t total_tiles) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t tile = t / (kTileW * kTileH), in = t % (kTileW * kTileH);
    bool alive = false;
    RayState r;
    uint32_t req = 0, idx = 0;
    if (tile < total_tiles) {
        const uint32_t k = init_entry(A.init_tile, A.n_init, tile);
        req = A.init_slot[k];
        const ReqView& R = A.reqs[req];
        const uint32_t w = (uint32_t)R.rv.width, h = (uint32_t)R.rv.height;
        const uint32_t lt = tile - A.init_tile[k];
        const uint32_t x = (lt % R.tiles_x) * kTileW + in % kTileW, y = (lt / R.tiles_x) * kTileH + in / kTileW;
        if (x < w && y < h) {
            idx = y * w + x;
            reinterpret_cast<float4*>(R.out_rgba)[idx] = make_float4(0.f, 0.f, 0.f, 0.f);
            R.out_depth[idx] = 1e10f;
            if (R.out_samples) R.out_samples[idx] = 0u;
            alive = ray_init(R.rv, x, y, R.bitfield, r);
        }
    }
    if (A.req_alive) count_per_request(A.req_alive, req, alive, 1);
    uint32_t slot = warp_append(A.n_alive_out, alive);
    if (alive) {
        RayBuf b = A.rays_out;
        b.a[slot] = make_float4(r.o.x, r.o.y, r.o.z, r.t);
        b.b[slot] = make_float4(r.d.x, r.d.y, r.d.z, 0.f);
        b.c[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
        b.d[slot] = make_float4(0.f, __uint_as_float(idx), __uint_as_float(0u), __uint_as_float(req));
    }
}

// ------------------------------------------------------------------ march + deform + encode
__device__ __forceinline__ uint32_t pack_act(float a, float b, bool bf16) { return pack2_act(a, b, bf16); }

// Parts of one sample's operand rows: hash features of 8-feature groups [g0, g1) (four levels of
// two features, two of four, or one of eight per group; each group stored as one 16-byte chunk
// of the row), the expression dims, and SH of the direction into the SH tile.  No per-sample
// array is materialised.
__device__ __forceinline__ uint32_t feature_groups(const FieldView& fv) { return fv.n_levels * fv.n_features / 8u; }
// F = fv.n_features (2, 4 or 8), a template parameter so that each kernel holds one variant.
template <int F>
__device__ __forceinline__ void encode_levels(const FieldView& fv, const uint16_t* table, const float* pos, uint8_t* rec, uint32_t row,
                                              uint32_t k_in, uint32_t g0, uint32_t g1) {
    const bool bf16 = fv.precision == 1;
    const __half2* t2 = reinterpret_cast<const __half2*>(table);
    const V3 x = v3(pos[0], pos[1], pos[2]);
#pragma unroll 1
    for (uint32_t g = g0; g < g1; ++g) {
        float v[8];
        if constexpr (F == 8) {
            hash_level_wide<8>(fv, t2, x, g, v);
        } else if constexpr (F == 4) {
            hash_level_wide<4>(fv, t2, x, 2 * g, v);
            hash_level_wide<4>(fv, t2, x, 2 * g + 1, v + 4);
        } else {
#pragma unroll
            for (uint32_t j = 0; j < 4; ++j) hash_level(fv, t2, x, 4 * g + j, v[2 * j], v[2 * j + 1]);
        }
        uint4 q;
        q.x = pack_act(v[0], v[1], bf16); q.y = pack_act(v[2], v[3], bf16);
        q.z = pack_act(v[4], v[5], bf16); q.w = pack_act(v[6], v[7], bf16);
        *reinterpret_cast<uint4*>(rec + tile_offset(row, 8 * g, k_in)) = q;
    }
}
template <int F>
__device__ __forceinline__ void encode_extra(const FieldView& fv, const float* extra, uint32_t mask, uint8_t* rec, uint32_t row, uint32_t k_in) {
    const bool bf16 = fv.precision == 1;
    for (uint32_t g = 0; g < fv.n_extra / 8; ++g) {
        float v[8];
#pragma unroll
        for (uint32_t j = 0; j < 8; ++j) v[j] = mask != 7u ? 1.f : (extra ? __ldg(extra + 8 * g + j) : 0.f);
        uint4 q;
        q.x = pack_act(v[0], v[1], bf16); q.y = pack_act(v[2], v[3], bf16);
        q.z = pack_act(v[4], v[5], bf16); q.w = pack_act(v[6], v[7], bf16);
        *reinterpret_cast<uint4*>(rec + tile_offset(row, fv.n_levels * F + 8 * g, k_in)) = q;
    }
}
__device__ __forceinline__ void encode_sh(const FieldView& fv, const float* dirw, uint8_t* rec, uint32_t row, uint32_t k_in) {
    const bool bf16 = fv.precision == 1;
    float d[16];
    sh4(dirw[0], dirw[1], dirw[2], d);
    uint8_t* sh = rec + hash_tile_bytes(k_in);
#pragma unroll
    for (uint32_t g = 0; g < 2; ++g) {
        uint4 q;
        q.x = pack_act(d[8 * g + 0], d[8 * g + 1], bf16); q.y = pack_act(d[8 * g + 2], d[8 * g + 3], bf16);
        q.z = pack_act(d[8 * g + 4], d[8 * g + 5], bf16); q.w = pack_act(d[8 * g + 6], d[8 * g + 7], bf16);
        *reinterpret_cast<uint4*>(sh + tile_offset(row, 8 * g, 16)) = q;
    }
}

// One sample's operand rows: hash features (+ expression dims) into the hash tile, SH of the
// direction into the SH tile.
template <int F>
__device__ __forceinline__ void encode_sample(const FieldView& fv, const uint16_t* table, const float* extra, uint32_t mask,
                                              const float* pos, const float* dirw, uint8_t* rec, uint32_t row, uint32_t k_in) {
    encode_levels<F>(fv, table, pos, rec, row, k_in, 0, feature_groups(fv));
    encode_extra<F>(fv, extra, mask, rec, row, k_in);
    encode_sh(fv, dirw, rec, row, k_in);
}

// One thread per alive ray: the next `steps` sample positions (generate_next_nerf_network_inputs,
// ngp/src/testbed_nerf.cu:722-795).  The march counts the samples, keeping each one's t; then the
// write pass places them -- position and step rebuilt from t -- so the samples of a warp's 32
// neighbouring rays land in one compacted block (base from a warp-aggregated atomic), ordered
// step-major: step k of all lanes, then step k + 1.  Neighbouring entries of the stream are
// then the same step of adjacent pixels, which keeps the cooperative BVH queries coherent.
// sample_ray packs the ray slot and the step k; the deform stage, which runs in spatially sorted
// order, records in sample_index[k * n_alive + r] where sample k of ray r went.
__global__ void __launch_bounds__(256) march_kernel(const __grid_constant__ WaveArgs A) {
    const uint32_t n_alive = *A.n_alive_in;
    const uint32_t steps = A.steps_dev ? *A.steps_dev : A.steps;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t n_iter = (n_alive + stride - 1) / stride;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt_mask = (1u << lane) - 1u;
    for (uint32_t it = 0; it < n_iter; ++it) {
        const uint32_t r = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
        const bool valid = r < n_alive;
        RayState ray;
        uint32_t ns = 0, j = 0;
        float t0 = 0.f;
        RenderView rv;   // the ray's request, held in registers through both march passes
        const uint8_t* bitfield = nullptr;
        if (valid) {
            const float4 ra = A.rays_in.a[r], rb = A.rays_in.b[r], rd = A.rays_in.d[r];
            ns = __float_as_uint(rd.z);
            const ReqView& R = A.reqs[__float_as_uint(rd.w)];
            rv = R.rv;
            bitfield = R.bitfield;
            ray.o = v3(ra.x, ra.y, ra.z);
            ray.d = v3(rb.x, rb.y, rb.z);
            ray.idir = v3(__fdiv_rn(1.f, rb.x), __fdiv_rn(1.f, rb.y), __fdiv_rn(1.f, rb.z));
            ray.t = t0 = ra.w;
            for (; j < steps; ++j) {
                V3 pos;
                float dt, ts;
                if (ns + j >= rv.max_samples_per_ray || !ray_next_sample(rv, bitfield, ray, pos, dt, &ts)) break;
                A.march_t[(size_t)j * n_alive + r] = ts;   // the write pass rebuilds the sample from its t
            }
        }
        const uint32_t total = __reduce_add_sync(0xffffffffu, j);
        const uint32_t max_j = __reduce_max_sync(0xffffffffu, j);
        uint32_t base = 0;
        if (lane == 0 && total) base = atomicAdd(A.n_samples_round, total);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (valid) ray.t = t0;
        uint32_t offset = 0;
        for (uint32_t k = 0; k < max_j; ++k) {
            const bool act = k < j;
            const uint32_t m = __ballot_sync(0xffffffffu, act);
            if (act) {
                // position and step of the sample at ts, as ray_next_sample produced them; the ray
                // then continues from ts + dt, where ray_next_sample leaves it
                const float ts = A.march_t[(size_t)k * n_alive + r];
                const V3 pos = ray_at(ray.o, ray.d, ts);
                const float dt = calc_dt(ts, rv.cone_angle);
                ray.t = __fadd_rn(ts, dt);
                const uint32_t idx = base + offset + (uint32_t)__popc(m & lt_mask);
                A.samples[idx] = make_float4(pos.x, pos.y, pos.z, dt);
                A.sample_ray[idx] = r | (k << kStepShift);
            }
            offset += (uint32_t)__popc(m);
        }
        if (valid) {
            A.rays_in.a[r].w = ray.t;
            A.n_round[r] = j;
        }
    }
}

// ------------------------------------------------------------------ spatial sort of a round's samples
__device__ __forceinline__ uint32_t spread3(uint32_t v) {   // 10 bits -> every third bit
    v &= 1023u;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Cell of a sample: a (2^(bits/3))^3 Morton grid over the frame mesh's box (the union of the
// root's child boxes) widened by 1/8 on each side; positions outside fall into border cells.
__device__ __forceinline__ uint32_t sample_cell(const FrameView& fr, float4 p, uint32_t bits) {
    const float4* nd = fr.nodes;
    const float4 mnx = __ldg(nd + 0), mny = __ldg(nd + 1), mnz = __ldg(nd + 2);
    const float4 mxx = __ldg(nd + 3), mxy = __ldg(nd + 4), mxz = __ldg(nd + 5);
    const int4 ch = __ldg(reinterpret_cast<const int4*>(nd + 6));
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    const float cmn[4][3] = {{mnx.x, mny.x, mnz.x}, {mnx.y, mny.y, mnz.y}, {mnx.z, mny.z, mnz.z}, {mnx.w, mny.w, mnz.w}};
    const float cmx[4][3] = {{mxx.x, mxy.x, mxz.x}, {mxx.y, mxy.y, mxz.y}, {mxx.z, mxy.z, mxz.z}, {mxx.w, mxy.w, mxz.w}};
    const int cref[4] = {ch.x, ch.y, ch.z, ch.w};
#pragma unroll
    for (int c = 0; c < 4; ++c)
        if (cref[c] != -1)
#pragma unroll
            for (int k = 0; k < 3; ++k) { lo[k] = fminf(lo[k], cmn[c][k]); hi[k] = fmaxf(hi[k], cmx[c][k]); }
    const float ext = fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), fmaxf(hi[2] - lo[2], 1e-6f)) * 1.25f;
    const uint32_t per_axis = 1u << (bits / 3);
    const float scale = (float)per_axis / ext, top = (float)(per_axis - 1);
    const float pp[3] = {p.x, p.y, p.z};
    uint32_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float c = (pp[k] - (0.5f * (lo[k] + hi[k]) - 0.5f * ext)) * scale;
        q[k] = (uint32_t)fminf(fmaxf(c, 0.f), top);
    }
    return spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
}

// Count per (request, cell) bin (warp-aggregated: lanes with the same key add once) and remember
// each sample's key.
__global__ void __launch_bounds__(256) sort_count_kernel(const __grid_constant__ WaveArgs A) {
    const uint32_t n = *A.n_samples_round;
    const uint32_t n_alive = *A.n_alive_in;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += stride) {
        const uint32_t s = b + threadIdx.x;
        const bool valid = s < n;
        uint32_t key = 0xffffffffu;
        if (valid) {
            const uint32_t r = A.sample_ray[s] & kRayMask;
            const uint32_t req = r < n_alive ? __float_as_uint(A.rays_in.d[r].w) : 0u;
            key = (req << A.cell_bits) | sample_cell(A.reqs[req].fr, A.samples[s], A.cell_bits);
            A.sample_key[s] = key;
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        if (valid && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(A.sort_bins + key, (uint32_t)__popc(peers));
    }
}

// Exclusive scan of each block of kSortBlock bin counts, in place; block totals to sort_block_sums.
__global__ void __launch_bounds__(kSortBlock) sort_scan_kernel(uint32_t* bins, uint32_t* block_sums) {
    __shared__ uint32_t warp_tot[kSortBlock / 32];
    const uint32_t i = blockIdx.x * kSortBlock + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t v = bins[i];
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= (uint32_t)o) t += y;
        }
        warp_tot[lane] = t;   // inclusive
    }
    __syncthreads();
    const uint32_t before = warp ? warp_tot[warp - 1] : 0u;
    bins[i] = before + x - v;
    if (threadIdx.x == kSortBlock - 1) block_sums[blockIdx.x] = before + x;
}

// Block-wide exclusive scan of one value per thread (kSortBlock threads); returns the total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* before, uint32_t* warp_tot) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    __syncthreads();
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= (uint32_t)o) t += y;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    *before = (warp ? warp_tot[warp - 1] : 0u) + x - v;
    return warp_tot[31];
}

// One block: offsets of the bin blocks, each request's unpadded start and padded segment
// (runs rounded up to 128 samples), padding markers, and the padded sample count.
__global__ void __launch_bounds__(kSortBlock) sort_offsets_kernel(const __grid_constant__ WaveArgs A, uint32_t n_blocks) {
    __shared__ uint32_t warp_tot[32];
    // 1. block offsets (n_blocks <= kMaxSortBins / kSortBlock = 16 per thread)
    const uint32_t per = (n_blocks + kSortBlock - 1) / kSortBlock;
    const uint32_t b0 = threadIdx.x * per;
    uint32_t local[16];
    uint32_t sum = 0;
    for (uint32_t k = 0; k < per; ++k) {
        const uint32_t v = b0 + k < n_blocks ? A.sort_block_sums[b0 + k] : 0u;
        local[k] = sum;
        sum += v;
    }
    uint32_t before;
    const uint32_t total = block_exclusive_scan(sum, &before, warp_tot);
    for (uint32_t k = 0; k < per; ++k)
        if (b0 + k < n_blocks) A.sort_block_sums[b0 + k] = before + local[k];
    __syncthreads();
    // 2. requests: start of each run (its first bin begins a bin block) and padded segments
    const uint32_t shift = A.cell_bits - 10u;   // bins per request / kSortBlock = 2^shift
    const uint32_t rper = (A.n_reqs + kSortBlock - 1) / kSortBlock;   // <= kMaxRequests / kSortBlock
    const uint32_t r0 = threadIdx.x * rper;
    uint32_t cnt[4], pad_sum = 0;
    for (uint32_t k = 0; k < rper; ++k) {
        const uint32_t r = r0 + k;
        cnt[k] = 0;
        if (r < A.n_reqs) {
            const uint32_t st = A.sort_block_sums[r << shift];
            const uint32_t en = r + 1 < A.n_reqs ? A.sort_block_sums[(r + 1) << shift] : total;
            A.req_start[r] = st;
            cnt[k] = en - st;
        }
        pad_sum += (cnt[k] + 127u) & ~127u;
    }
    uint32_t pbefore;
    const uint32_t padded_total = block_exclusive_scan(pad_sum, &pbefore, warp_tot);
    for (uint32_t k = 0; k < rper; ++k) {
        const uint32_t r = r0 + k;
        if (r < A.n_reqs) {
            A.req_seg[r] = pbefore;
            for (uint32_t q = pbefore + cnt[k]; q < pbefore + ((cnt[k] + 127u) & ~127u); ++q) A.sample_order[q] = kNoSample;
        }
        pbefore += (cnt[k] + 127u) & ~127u;
    }
    if (threadIdx.x == 0) {
        A.req_seg[A.n_reqs] = padded_total;
        A.req_start[A.n_reqs] = total;
        *A.n_samples_padded = padded_total;
    }
}

// Place every sample: its bin's start plus a running cursor (warp-aggregated), moved from the
// request's unpadded start to its padded segment.  Order within a bin is arbitrary; each
// sample's result does not depend on it.
__global__ void __launch_bounds__(256) sort_place_kernel(const __grid_constant__ WaveArgs A) {
    const uint32_t n = *A.n_samples_round;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += stride) {
        const uint32_t s = b + threadIdx.x;
        const bool valid = s < n;
        uint32_t key = valid ? A.sample_key[s] : 0xffffffffu;
        const bool placed = key != 0xffffffffu;   // unsorted records (skipped by the caller) carry no key
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (placed && lane == (uint32_t)leader) base = atomicAdd(A.sort_bins + key, (uint32_t)__popc(peers));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (placed) {
            const uint32_t req = key >> A.cell_bits;
            const uint32_t pos = A.sort_block_sums[key / kSortBlock] + base + (uint32_t)__popc(peers & lt_mask);
            A.sample_order[pos - A.req_start[req] + A.req_seg[req]] = s;
        }
    }
}

// The deform + encode stage, two kernels over the spatially sorted stream (split so that each
// gets the registers and occupancy it needs):
//   nearest_stage_kernel  a warp per 32 consecutive samples: the warp-cooperative nearest-triangle
//                         walk (the samples share a few grid cells, so the union of visited nodes
//                         is small); the triangle id of each sample goes to sample_key[position]
//   map_encode_kernel     a thread per sample: the warp hook (src/core.cu:470-519) on
//                         warp_position(pos) / warp_direction(dir) with that triangle, then the
//                         hash encode and SH written as tensor-core operand rows at the sample's
//                         sorted position
// With A.top_nodes > 0 each warp keeps a shared-memory copy of the first top_nodes nodes of its
// frame's tree (the top levels: nodes are numbered level by level), brought in by one bulk copy
// (cp.async.bulk, completion on the warp's mbarrier) whenever the warp moves to another frame;
// the walk reads those nodes from shared memory and the rest through the L1.
__global__ void __launch_bounds__(256, 4) nearest_stage_kernel(const __grid_constant__ WaveArgs A) {
    __shared__ WarpScratch wscratch[8];
    __shared__ alignas(8) uint64_t top_bar[8];
    extern __shared__ __align__(128) float4 top_dyn[];   // [8][top_nodes * 7]
    const uint32_t n = *A.n_samples_padded;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t n_warps = gridDim.x * (blockDim.x >> 5);
    float4* top = top_dyn + (size_t)warp * A.top_nodes * 7;
    const float4* staged = nullptr;   // the nodes array whose top levels `top` holds
    uint32_t n_top = 0, top_phase = 0;
    bool top_ok = A.top_nodes > 0;    // false after a copy that did not complete in time
    if (top_ok) {
        if (lane == 0) {
            mbar_init(&top_bar[warp], 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncwarp();
    }
    // 32-sample chunks are handed out by a device cursor (walk costs vary from chunk to chunk, so
    // a fixed share per warp leaves SMs idle at the end); the last warp to finish resets it
    for (;;) {
        uint32_t chunk = 0;
        if (lane == 0) chunk = atomicAdd(A.nearest_work, 1u);
        const uint32_t base = __shfl_sync(0xffffffffu, chunk, 0) * 32u;
        if (base >= n) break;
        const uint32_t s = base + lane;
        const uint32_t m = A.sample_order[s];
        const bool valid = m != kNoSample;
        const uint32_t any = __ballot_sync(0xffffffffu, valid);
        if (!any) continue;
        uint32_t req = 0;
        float4 smp = make_float4(0.5f, 0.5f, 0.5f, 0.f);
        if (valid) {
            const uint32_t rk = A.sample_ray[m];
            smp = A.samples[m];
            req = __float_as_uint(A.rays_in.d[rk & kRayMask].w);
        }
        req = __shfl_sync(0xffffffffu, req, __ffs(any) - 1);
        const ReqView& R = A.reqs[req];
        const RenderView& rv = R.rv;
        const float pp[3] = {smp.x, smp.y, smp.z};
        float cw[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) cw[k] = __fdiv_rn(__fsub_rn(pp[k], rv.train_min[k]), __fsub_rn(rv.train_max[k], rv.train_min[k]));
        const V3 p = v3(cw[0], cw[1], cw[2]);
        const bool in_box = valid && box_contains(R.dv.aabb_min, R.dv.aabb_max, p);
        if (top_ok && R.fr.nodes != staged) {
            const uint32_t k = min(A.top_nodes, (uint32_t)R.fr.n_nodes);   // never past the node array
            __syncwarp();   // every lane is done reading the previous copy
            if (lane == 0) {
                fence_async_smem();
                bulk_load(top, R.fr.nodes, k * 112u, &top_bar[warp]);
            }
            top_ok = __all_sync(0xffffffffu, mbar_wait(&top_bar[warp], top_phase));   // warp-uniform
            if (top_ok) {
                top_phase ^= 1u;
                staged = R.fr.nodes;
                n_top = k;
            } else {
                n_top = 0;
                if (lane == 0) atomicOr(A.err, INSTA_DEVERR_TIMEOUT);
            }
        }
        Nearest q = nearest_warp(R.fr, p, in_box, wscratch[warp], A.err, __builtin_huge_valf(), top, n_top, A.walk_stats);
        if (valid) A.sample_key[s] = in_box ? (uint32_t)q.id : 0xfffffffeu;
    }
    // a copy that timed out may still land: wait for it (bounded) before the CTA's shared memory goes
    if (A.top_nodes > 0 && !top_ok) mbar_wait(&top_bar[warp], top_phase);
    if (lane == 0) {
        __threadfence();   // this warp's last cursor increment before its count
        if (atomicAdd(A.nearest_work + 1, 1u) == n_warps - 1u) {
            A.nearest_work[0] = 0u;
            A.nearest_work[1] = 0u;
            __threadfence();
        }
    }
}

// The deform half of the stage for sorted position s holding march-order sample m: the warp hook
// (src/core.cu:470-519) on warp_position(pos) / warp_direction(dir) with the nearest triangle the
// nearest stage left in sample_key[s]; records where the sample went (sample_index) and its
// (dt, depth candidate) for the composite.  Returns the request slot.
__device__ __forceinline__ uint32_t deform_sample(const WaveArgs& A, uint32_t s, uint32_t m, uint32_t n_alive, float* cpos, float* cdir,
                                                  uint32_t& mask) {
    const uint32_t rk = A.sample_ray[m];
    const float4 smp = A.samples[m];
    const float4 rb = A.rays_in.b[rk & kRayMask];
    const uint32_t req = __float_as_uint(A.rays_in.d[rk & kRayMask].w);
    A.sample_index[(size_t)(rk >> kStepShift) * n_alive + (rk & kRayMask)] = s;
    const ReqView& R = A.reqs[req];
    const RenderView& rv = R.rv;
    float cw[3], dw[3], dp[3];
    const float pp[3] = {smp.x, smp.y, smp.z}, dd[3] = {rb.x, rb.y, rb.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        cw[k] = __fdiv_rn(__fsub_rn(pp[k], rv.train_min[k]), __fsub_rn(rv.train_max[k], rv.train_min[k]));
        dw[k] = __fmul_rn(__fadd_rn(dd[k], 1.0f), 0.5f);
        dp[k] = __fadd_rn(rv.train_min[k], __fmul_rn(cw[k], __fsub_rn(rv.train_max[k], rv.train_min[k])));
    }
    cpos[0] = cw[0]; cpos[1] = cw[1]; cpos[2] = cw[2];
    cdir[0] = dw[0]; cdir[1] = dw[1]; cdir[2] = dw[2];
    mask = 7u;
    const V3 p = v3(cw[0], cw[1], cw[2]);
    const uint32_t id = A.sample_key[s];
    if (id != 0xfffffffeu) {
        if ((int32_t)id >= 0) map_to_canonical(R.dv, R.fr.frames, id, p, dw, cpos, cdir, &mask);
        else atomicOr(A.err, INSTA_DEVERR_NO_TRI);
    }
    const V3 cam_fwd = v3(rv.cam[2], rv.cam[6], rv.cam[10]);
    const V3 cam_pos = v3(rv.cam[3], rv.cam[7], rv.cam[11]);
    const V3 dv = v3(__fsub_rn(dp[0], cam_pos.x), __fsub_rn(dp[1], cam_pos.y), __fsub_rn(dp[2], cam_pos.z));
    A.aux[s] = make_float2(smp.w, dot_rn(cam_fwd, dv));
    return req;
}

template <int F>
__global__ void __launch_bounds__(256, 4) map_encode_kernel(const __grid_constant__ WaveArgs A) {
    const uint32_t n = *A.n_samples_padded;
    const uint32_t n_alive = *A.n_alive_in;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const uint32_t m = A.sample_order[s];
        if (m == kNoSample) continue;
        float cpos[3], cdir[3];
        uint32_t mask;
        const uint32_t req = deform_sample(A, s, m, n_alive, cpos, cdir, mask);
        const ReqView& R = A.reqs[req];
        uint8_t* rec = A.tiles + (size_t)(s >> 7) * A.tile_bytes;
        encode_sample<F>(A.fv, R.table, R.extra, mask, cpos, cdir, rec, s & 127u, A.k_in);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(A.sample_counter, (unsigned long long)*A.n_samples_round);
}

// ------------------------------------------------------------------ MLP over tiles
// Request slot of tile t: the request whose padded run holds it (render batches; 0 otherwise).
__device__ __forceinline__ uint32_t tile_request(const MlpArgs& A, uint32_t t) {
    if (!A.seg) return 0;
    const uint32_t row = t * 128u;
    uint32_t lo = 0, hi = A.n_reqs;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(A.seg + mid) <= row) lo = mid; else hi = mid;
    }
    return lo;
}

// Weight image of tile t: its request's (render batches), else the field's.
__device__ __forceinline__ const uint8_t* tile_weights(const MlpArgs& A, uint32_t t) {
    return A.seg ? A.reqs[tile_request(A, t)].mlp : A.fv.mlp_smem;
}

// The MLPs over ready-made operand tiles in global memory, 256 threads per CTA: each
// CTA takes a contiguous range of tiles (consecutive tiles mostly share a request, so the weight
// image is reloaded only where a range crosses into another avatar's requests); tile t + 1's
// hash rows are bulk-copied in as soon as tile t's density layer 0 has run, its SH rows as soon
// as colour layer 0 has, so the copies overlap the chain; the epilogues split the accumulator
// columns between the two warpgroups (FP8: each warpgroup re-quantises half of a row, the row
// maximum exchanged through shared memory).
template <bool FP8>
__global__ void __launch_bounds__(256, 4) mlp256_kernel(const __grid_constant__ MlpArgs A) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    Mlp2Ctl& ctl = *reinterpret_cast<Mlp2Ctl*>(smem_raw);
    Mlp2View sm{ctl.bar_mma, ctl.tmem_base, smem_raw + mlp2_stage_off(), smem_raw + mlp2_a_h_off(),
                smem_raw + mlp2_dens_off(A.plan.tile_bytes), smem_raw + mlp2_w_off(A.plan.tile_bytes)};
    uint8_t* w = sm.w;
    const uint32_t n_samples = A.n_alive ? *A.n_alive : (uint32_t)A.n_samples;
    const uint32_t n_tiles = (n_samples + 127u) / 128u;
    const uint32_t per = (n_tiles + gridDim.x - 1) / gridDim.x;
    const uint32_t t0 = blockIdx.x * per, t1 = min(n_tiles, t0 + per);
    if (t0 >= t1) return;
    const uint32_t hash_bytes = hash_tile_bytes(A.plan.k_in), sh_bytes = sh_tile_bytes();
    if (threadIdx.x == 0) {
        mbar_init(&ctl.bar_mma, 1);
        mbar_init(&ctl.bar_load, 2);
        mbar_init(&ctl.bar_w, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x < 32) tmem_alloc(&ctl.tmem_base, 128);
    const uint8_t* loaded = tile_weights(A, t0);
    if (threadIdx.x == 0) {
        bulk_load(w, loaded, A.plan.bytes, &ctl.bar_w);
        const uint8_t* src = A.tiles + (size_t)t0 * A.plan.tile_bytes;
        bulk_load(sm.stage, src, hash_bytes, &ctl.bar_load);
        bulk_load(sm.stage + hash_bytes, src + hash_bytes, sh_bytes, &ctl.bar_load);
    }
    uint32_t w_phase = 0, load_phase = 0, phase = 0;
    bool ok = mbar_wait(&ctl.bar_w, w_phase);
    w_phase ^= 1u;
    tc_fence_before();
    ok = __syncthreads_and(ok ? 1 : 0) != 0;   // uniform: the tile loop holds CTA barriers
    tc_fence_after();
    const bool bf16 = A.fv.precision == 1;
    float* xch = reinterpret_cast<float*>(smem_raw + mlp2_xch_off());
    bool pending = true;   // a tile's copies are in flight
    for (uint32_t t = t0; t < t1 && ok; ++t) {
        ok &= mbar_wait(&ctl.bar_load, load_phase);
        load_phase ^= 1u;
        pending = false;
        const uint8_t* need = tile_weights(A, t);
        if (need != loaded) {
            // the previous tile's MMAs have completed (mlp256 waited on them); swap the image
            if (threadIdx.x == 0) bulk_load(w, need, A.plan.bytes, &ctl.bar_w);
            ok &= mbar_wait(&ctl.bar_w, w_phase);
            w_phase ^= 1u;
            loaded = need;
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
        }
        const bool next = t + 1 < t1;
        const uint8_t* nsrc = A.tiles + (size_t)(t + 1) * A.plan.tile_bytes;
        auto hash_free = [&] {
            if (next && threadIdx.x == 0) bulk_load(sm.stage, nsrc, hash_bytes, &ctl.bar_load);
        };
        auto sh_free = [&] {
            if (next && threadIdx.x == 0) bulk_load(sm.stage + hash_bytes, nsrc + hash_bytes, sh_bytes, &ctl.bar_load);
        };
        pending = next;
        float o4[4];
        if constexpr (FP8) ok &= mlp256_8(sm, xch, sm.a_dens, w, A.plan, reinterpret_cast<const float*>(w + A.plan.scales), phase, o4, hash_free, sh_free);
        else ok &= mlp256(sm, sm.a_dens, w, A.plan, bf16, phase, o4, hash_free, sh_free);
        const uint32_t s = t * 128u + threadIdx.x;
        if (threadIdx.x < 128u && s < n_samples) {
            if (A.fv.precision != 0) {
                A.out_f32[s] = make_float4(o4[0], o4[1], o4[2], o4[3]);
            } else {
                __half2 rg = __floats2half2_rn(o4[0], o4[1]);
                __half2 bd = __floats2half2_rn(o4[2], o4[3]);
                uint2 u;
                u.x = *reinterpret_cast<uint32_t*>(&rg);
                u.y = *reinterpret_cast<uint32_t*>(&bd);
                A.out[s] = u;
            }
        }
        ok = __syncthreads_and(ok ? 1 : 0) != 0;
    }
    if (!ok && threadIdx.x == 0) atomicOr(A.err, INSTA_DEVERR_TIMEOUT);
    // drain the copies of a tile that will not run (bounded wait) before shared memory is released
    if (pending) mbar_wait(&ctl.bar_load, load_phase);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32) tmem_dealloc(ctl.tmem_base, 128);
}

// ------------------------------------------------------------------ fused deform + encode + MLP
// The stage after the nearest-triangle walk in one launch over the sorted stream (FP16 / BF16
// MLPs): a CTA of 256 threads takes a contiguous range of 128-sample tiles.  Per tile, warpgroup 0
// runs the deform half (deform_sample, a sample per thread) and hands canonical position,
// direction and region to the encode through shared memory; both warpgroups encode (half the hash
// levels each, SH and expression dims split between them) straight into the tile's operand rows
// in shared memory; then the MLP chain runs on the tensor cores (mlp256: one thread issues,
// the epilogues split the accumulator columns between the warpgroups).  Several CTAs per SM
// overlap one CTA's gathers with another's MMAs, and the operand rows never go to global memory.
// Same arithmetic as map_encode_kernel + mlp256_kernel, so the outputs are the same bits.
__global__ void __launch_bounds__(256, 4) field_tile_kernel(const __grid_constant__ WaveArgs A, const __grid_constant__ MlpArgs M) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    FusedSmem& sm = *reinterpret_cast<FusedSmem*>(smem_raw);
    uint8_t* w = smem_raw + ((sizeof(FusedSmem) + 1023) & ~size_t(1023));
    const uint32_t n_samples = *A.n_samples_padded;
    const uint32_t n_alive = *A.n_alive_in;
    const uint32_t n_tiles = (n_samples + 127u) / 128u;
    const uint32_t per = (n_tiles + gridDim.x - 1) / gridDim.x;
    const uint32_t t0 = blockIdx.x * per, t1 = min(n_tiles, t0 + per);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(A.sample_counter, (unsigned long long)*A.n_samples_round);
    if (t0 >= t1) return;
    const uint32_t r = threadIdx.x & 127u, wg = threadIdx.x >> 7;
    if (threadIdx.x == 0) {
        mbar_init(&sm.bar_mma, 1);
        mbar_init(&sm.bar_w, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x < 32) tmem_alloc(&sm.tmem_base, 128);
    const uint8_t* loaded = tile_weights(M, t0);
    if (threadIdx.x == 0) bulk_load(w, loaded, M.plan.bytes, &sm.bar_w);
    uint32_t w_phase = 0, phase = 0;
    bool ok = mbar_wait(&sm.bar_w, w_phase);
    w_phase ^= 1u;
    tc_fence_before();
    ok = __syncthreads_and(ok ? 1 : 0) != 0;   // uniform: the tile loop holds CTA barriers
    tc_fence_after();
    const bool bf16 = A.fv.precision == 1;
    const uint32_t ng = feature_groups(A.fv), half = ng / 2;   // feature groups; warpgroup 0 takes [0, half)
    float4* hand = reinterpret_cast<float4*>(sm.a_h);      // [128][2]: (position, region), (direction, valid)
    for (uint32_t t = t0; t < t1 && ok; ++t) {
        const uint32_t req = tile_request(M, t);
        const uint8_t* need = M.seg ? M.reqs[req].mlp : M.fv.mlp_smem;
        if (need != loaded) {
            // the previous tile's MMAs have completed (mlp256 waited on them); swap the image
            if (threadIdx.x == 0) bulk_load(w, need, M.plan.bytes, &sm.bar_w);
            ok &= mbar_wait(&sm.bar_w, w_phase);
            w_phase ^= 1u;
            loaded = need;
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
        }
        const uint32_t s = t * 128u + r;
        if (wg == 0) {
            const uint32_t m = A.sample_order[s];
            float cpos[3] = {0.f, 0.f, 0.f}, cdir[3] = {0.5f, 0.5f, 0.5f};
            uint32_t mask = 7u;
            if (m != kNoSample) deform_sample(A, s, m, n_alive, cpos, cdir, mask);
            hand[r * 2] = make_float4(cpos[0], cpos[1], cpos[2], __uint_as_float(mask));
            hand[r * 2 + 1] = make_float4(cdir[0], cdir[1], cdir[2], __uint_as_float(m != kNoSample ? 1u : 0u));
        }
        __syncthreads();
        const float4 h0 = hand[r * 2], h1 = hand[r * 2 + 1];
        {
            // padding rows are encoded at a fixed point; their outputs are never read
            const ReqView& R = A.reqs[req];
            const float cpos[3] = {h0.x, h0.y, h0.z}, cdir[3] = {h1.x, h1.y, h1.z};
            if (wg == 0) {
                encode_levels<2>(A.fv, R.table, cpos, sm.stage, r, A.k_in, 0, half);
                encode_sh(A.fv, cdir, sm.stage, r, A.k_in);
            } else {
                encode_levels<2>(A.fv, R.table, cpos, sm.stage, r, A.k_in, half, ng);
                encode_extra<2>(A.fv, R.extra, __float_as_uint(h0.w), sm.stage, r, A.k_in);
            }
        }
        // mlp256's first chain fences these generic writes for the tensor core and syncs the CTA;
        // the density output rows go to the hash rows, dead once density layer 0 has run
        float o4[4];
        ok &= mlp256(sm, sm.stage, w, M.plan, bf16, phase, o4);
        if (wg == 0 && __float_as_uint(h1.w) != 0u) {
            if (A.fv.precision != 0) {
                M.out_f32[s] = make_float4(o4[0], o4[1], o4[2], o4[3]);
            } else {
                __half2 rg = __floats2half2_rn(o4[0], o4[1]);
                __half2 bd = __floats2half2_rn(o4[2], o4[3]);
                uint2 u;
                u.x = *reinterpret_cast<uint32_t*>(&rg);
                u.y = *reinterpret_cast<uint32_t*>(&bd);
                M.out[s] = u;
            }
        }
        ok = __syncthreads_and(ok ? 1 : 0) != 0;
    }
    if (!ok && threadIdx.x == 0) atomicOr(A.err, INSTA_DEVERR_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32) tmem_dealloc(sm.tmem_base, 128);
}

// ------------------------------------------------------------------ composite + compaction
__global__ void composite_kernel(const __grid_constant__ WaveArgs A) {
    const uint32_t n_alive = *A.n_alive_in;
    const uint32_t steps = A.steps_dev ? *A.steps_dev : A.steps;
    const bool f32_out = A.fv.precision != 0;   // the MLP wrote FP32 outputs
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t n_iter = (n_alive + stride - 1) / stride;
    for (uint32_t it = 0; it < n_iter; ++it) {
        const uint32_t r = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
        bool keep = false;
        float4 ra, rb, rc, rd;
        if (r < n_alive) {
            ra = A.rays_in.a[r]; rb = A.rays_in.b[r]; rc = A.rays_in.c[r]; rd = A.rays_in.d[r];
            const ReqView& R = A.reqs[__float_as_uint(rd.w)];
            const uint32_t m = A.n_round[r];
            bool done = m < steps;
            float4 rgba = rc;
            float depth = rd.x, maxw = rb.w;
            uint32_t j = 0, used = m;   // samples composited this round
            // The loads run ahead of the arithmetic: the next sample's outputs and the sorted
            // position of the one after are in flight while this sample is composited (loads
            // past an early termination are dropped unused).
            auto load = [&](uint32_t s, float4& v, float2& ax) {
                if (f32_out) {
                    v = A.out_f32[s];
                } else {
                    const uint2 u = A.out[s];
                    const float2 rg = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
                    const float2 bd = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
                    v = make_float4(rg.x, rg.y, bd.x, bd.y);
                }
                ax = A.aux[s];
            };
            float4 v_next = make_float4(0.f, 0.f, 0.f, 0.f);
            float2 ax_next = make_float2(0.f, 0.f);
            uint32_t s_after = 0;
            if (m > 0) load(A.sample_index[r], v_next, ax_next);
            if (m > 1) s_after = A.sample_index[(size_t)n_alive + r];
            for (; j < m; ++j) {
                const float4 v = v_next;
                const float2 ax = ax_next;
                if (j + 1 < m) load(s_after, v_next, ax_next);
                if (j + 2 < m) s_after = A.sample_index[(size_t)(j + 2) * n_alive + r];
                const float o[4] = {v.x, v.y, v.z, v.w};
                // composite_kernel_nerf (ngp/src/testbed_nerf.cu:840-999)
                const float T = 1.f - rgba.w;
                const float dtu = unwarp_dt(warp_dt(ax.x));
                const float alpha = 1.f - expf(-expf(o[3]) * dtu);
                const float wgt = alpha * T;
                rgba.x += (1.0f / (1.0f + expf(-o[0]))) * wgt;
                rgba.y += (1.0f / (1.0f + expf(-o[1]))) * wgt;
                rgba.z += (1.0f / (1.0f + expf(-o[2]))) * wgt;
                rgba.w += wgt;
                if (wgt > maxw) { maxw = wgt; depth = ax.y; }
                if (rgba.w > 1.0f - R.rv.min_transmittance) {
                    const float a = rgba.w;
                    rgba.x /= a; rgba.y /= a; rgba.z /= a; rgba.w /= a;
                    done = true;
                    used = j + 1;
                    break;
                }
            }
            const uint32_t ns = __float_as_uint(rd.z) + m;
            if (done) {
                write_pixel(R.rv, R.out_rgba, R.out_depth, __float_as_uint(rd.y), rgba, depth);
                if (R.out_samples) R.out_samples[__float_as_uint(rd.y)] = __float_as_uint(rd.z) + used;
            } else {
                keep = true;
                rb.w = maxw;
                rc = rgba;
                rd.x = depth;
                rd.z = __uint_as_float(ns);
            }
        }
        if (A.req_alive) count_per_request(A.req_alive, r < n_alive ? __float_as_uint(rd.w) : 0u, r < n_alive && !keep, -1);
        const uint32_t slot = warp_append(A.n_alive_out, keep);
        if (keep) {
            A.rays_out.a[slot] = ra; A.rays_out.b[slot] = rb; A.rays_out.c[slot] = rc; A.rays_out.d[slot] = rd;
        }
    }
}

// ------------------------------------------------------------------ field eval (parity entry)
// mask: 7 = the expression dims from the record's last n_extra floats; any other value = every
// expression dim 1 (the density-grid update, as NerfNetwork::density feeds them,
// NGP/nerf_network.h:107-127,401-410).
template <int F>
__global__ void __launch_bounds__(256) encode_coords_kernel(FieldView fv, const float* __restrict__ coords, uint32_t stride,
                                                            int64_t n, uint8_t* tiles, uint32_t tile_bytes, uint32_t k_in, uint32_t mask) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* c = coords + i * stride;
    float pos[3] = {c[0], c[1], c[2]}, dir[3] = {c[8], c[9], c[10]};
    uint8_t* rec = tiles + (size_t)(i >> 7) * tile_bytes;
    encode_sample<F>(fv, fv.table, mask == 7u ? c + stride - fv.n_extra : nullptr, mask, pos, dir, rec, (uint32_t)(i & 127), k_in);
}

__global__ void unpack_outputs_kernel(const uint2* __restrict__ out, const float4* __restrict__ out_f32, int bf16, int64_t n, float4* dst) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (bf16) { dst[i] = out_f32[i]; return; }
    uint2 u = out[i];
    float2 rg = __half22float2(*reinterpret_cast<__half2*>(&u.x));
    float2 bd = __half22float2(*reinterpret_cast<__half2*>(&u.y));
    dst[i] = make_float4(rg.x, rg.y, bd.x, bd.y);
}

// ------------------------------------------------------------------ training samples
// generate_training_samples_nerf (ngp/src/testbed_nerf.cu:1105-1285) for caller-supplied rays:
// two passes per ray (count up to NERF_STEPS = 1024 occupied steps through the train box, then
// reserve a block atomically and write NerfCoordinate records with holder = image).  Batches of
// up to kTrainMarchOnceMaxRays rays take training_march_kernel + training_write_kernel instead.
__global__ void __launch_bounds__(256) training_samples_kernel(const __grid_constant__ TrainArgs A) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n_rays) return;
    const float* r = A.rays + i * 6;
    const V3 o = v3(r[0], r[1], r[2]);
    const V3 d = normalize_rn(v3(r[3], r[4], r[5]));
    const V3 idir = v3(__fdiv_rn(1.f, d.x), __fdiv_rn(1.f, d.y), __fdiv_rn(1.f, d.z));
    float startt = fmaxf(aabb_ray_tmin(A.aabb_min, A.aabb_max, o, d), 0.0f);
    startt = __fadd_rn(startt, __fmul_rn(calc_dt(startt, A.cone_angle), A.start_rand[i]));
    uint32_t j = 0;
    float t = startt;
    for (int guard = 0; guard < (1 << 16) && j < 1024u; ++guard) {
        const V3 pos = ray_at(o, d, t);
        if (!box_contains(A.aabb_min, A.aabb_max, pos)) break;
        const float dt = calc_dt(t, A.cone_angle);
        const int mip = mip_from_dt(dt, pos);
        if (occupied_at(pos, A.bitfield, mip)) { ++j; t = __fadd_rn(t, dt); }
        else t = advance_to_next_voxel(t, A.cone_angle, pos, d, idir, GRID >> mip);
    }
    if (j == 0) return;
    const uint32_t base = atomicAdd(A.counters + 1, j);
    if (base + j > A.max_samples) {
        // the block does not fit (dropped, as in the reference); mark the part that lies inside the
        // buffer as unused so the warp pass skips it
        for (uint32_t q = base; q < A.max_samples; ++q) A.coords[(size_t)q * A.stride + 4] = -1.f;
        return;
    }
    const uint32_t ri = atomicAdd(A.counters + 0, 1u);
    A.ray_indices[ri] = (uint32_t)i;
    A.numsteps[2 * ri] = j;
    A.numsteps[2 * ri + 1] = base;
    const uint32_t img = A.image[i];
    const float wd[3] = {__fmul_rn(__fadd_rn(d.x, 1.0f), 0.5f), __fmul_rn(__fadd_rn(d.y, 1.0f), 0.5f), __fmul_rn(__fadd_rn(d.z, 1.0f), 0.5f)};
    const float* ex = (A.extra && img < A.n_images) ? A.extra + (size_t)img * A.n_extra : nullptr;
    t = startt;
    uint32_t w = 0;
    for (int guard = 0; guard < (1 << 16) && w < j; ++guard) {
        const V3 pos = ray_at(o, d, t);
        if (!box_contains(A.aabb_min, A.aabb_max, pos)) break;
        const float dt = calc_dt(t, A.cone_angle);
        const int mip = mip_from_dt(dt, pos);
        if (occupied_at(pos, A.bitfield, mip)) {
            float* c = A.coords + (size_t)(base + w) * A.stride;
            const float p3[3] = {pos.x, pos.y, pos.z};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float rel = __fdiv_rn(__fsub_rn(p3[k], A.aabb_min[k]), __fsub_rn(A.aabb_max[k], A.aabb_min[k]));
                c[k] = rel;
                c[5 + k] = rel;
                c[8 + k] = wd[k];
            }
            c[3] = warp_dt(dt);
            c[4] = (float)img;
            for (uint32_t m = 0; m < A.n_extra; ++m) c[A.stride - A.n_extra + m] = ex ? ex[m] : 0.f;
            ++w;
            t = __fadd_rn(t, dt);
        } else {
            t = advance_to_next_voxel(t, A.cone_angle, pos, d, idir, GRID >> mip);
        }
    }
}

// The same training march run once: the counting pass keeps each occupied sample's t (at most 1024
// per ray) and reserves the ray's block, then a warp per kept ray writes the records from those t
// with the write pass's arithmetic -- the records depend only on t and the ray -- so the records
// are bit-identical to training_samples_kernel's.
__global__ void __launch_bounds__(256) training_march_kernel(const __grid_constant__ TrainArgs A, float* __restrict__ tbuf) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n_rays) return;
    const float* r = A.rays + i * 6;
    const V3 o = v3(r[0], r[1], r[2]);
    const V3 d = normalize_rn(v3(r[3], r[4], r[5]));
    const V3 idir = v3(__fdiv_rn(1.f, d.x), __fdiv_rn(1.f, d.y), __fdiv_rn(1.f, d.z));
    float startt = fmaxf(aabb_ray_tmin(A.aabb_min, A.aabb_max, o, d), 0.0f);
    startt = __fadd_rn(startt, __fmul_rn(calc_dt(startt, A.cone_angle), A.start_rand[i]));
    float* tr = tbuf + (size_t)i * 1024u;
    uint32_t j = 0;
    float t = startt;
    for (int guard = 0; guard < (1 << 16) && j < 1024u; ++guard) {
        const V3 pos = ray_at(o, d, t);
        if (!box_contains(A.aabb_min, A.aabb_max, pos)) break;
        const float dt = calc_dt(t, A.cone_angle);
        const int mip = mip_from_dt(dt, pos);
        if (occupied_at(pos, A.bitfield, mip)) { tr[j] = t; ++j; t = __fadd_rn(t, dt); }
        else t = advance_to_next_voxel(t, A.cone_angle, pos, d, idir, GRID >> mip);
    }
    if (j == 0) return;
    const uint32_t base = atomicAdd(A.counters + 1, j);
    if (base + j > A.max_samples) {
        for (uint32_t q = base; q < A.max_samples; ++q) A.coords[(size_t)q * A.stride + 4] = -1.f;
        return;
    }
    const uint32_t ri = atomicAdd(A.counters + 0, 1u);
    A.ray_indices[ri] = (uint32_t)i;
    A.numsteps[2 * ri] = j;
    A.numsteps[2 * ri + 1] = base;
}

__global__ void __launch_bounds__(256) training_write_kernel(const __grid_constant__ TrainArgs A, const float* __restrict__ tbuf) {
    const uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if ((int64_t)k >= min((int64_t)A.counters[0], A.n_rays)) return;
    const uint32_t i = A.ray_indices[k], j = A.numsteps[2 * k], base = A.numsteps[2 * k + 1];
    const float* r = A.rays + (size_t)i * 6;
    const V3 o = v3(r[0], r[1], r[2]);
    const V3 d = normalize_rn(v3(r[3], r[4], r[5]));
    const uint32_t img = A.image[i];
    const float wd[3] = {__fmul_rn(__fadd_rn(d.x, 1.0f), 0.5f), __fmul_rn(__fadd_rn(d.y, 1.0f), 0.5f), __fmul_rn(__fadd_rn(d.z, 1.0f), 0.5f)};
    const float* ex = (A.extra && img < A.n_images) ? A.extra + (size_t)img * A.n_extra : nullptr;
    const float* tr = tbuf + (size_t)i * 1024u;
    for (uint32_t w = lane; w < j; w += 32u) {
        const float t = tr[w];
        const V3 pos = ray_at(o, d, t);
        const float dt = calc_dt(t, A.cone_angle);
        float* c = A.coords + (size_t)(base + w) * A.stride;
        const float p3[3] = {pos.x, pos.y, pos.z};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float rel = __fdiv_rn(__fsub_rn(p3[q], A.aabb_min[q]), __fsub_rn(A.aabb_max[q], A.aabb_min[q]));
            c[q] = rel;
            c[5 + q] = rel;
            c[8 + q] = wd[q];
        }
        c[3] = warp_dt(dt);
        c[4] = (float)img;
        for (uint32_t m = 0; m < A.n_extra; ++m) c[A.stride - A.n_extra + m] = ex ? ex[m] : 0.f;
    }
}

// ------------------------------------------------------------------ march debug
__global__ void march_debug_kernel(RenderView rv, const uint8_t* __restrict__ bf, int max_out, float* out_t, float* out_dt, int32_t* out_n) {
    uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (uint32_t)rv.width * (uint32_t)rv.height) return;
    RayState r;
    int n = 0;
    if (ray_init(rv, idx % (uint32_t)rv.width, idx / (uint32_t)rv.width, bf, r)) {
        V3 pos;
        float dt;
        while (n < max_out && n < (int)rv.max_samples_per_ray) {
            float ts;
            if (!ray_next_sample(rv, bf, r, pos, dt, &ts)) break;
            out_t[(size_t)idx * max_out + n] = ts;
            out_dt[(size_t)idx * max_out + n] = dt;
            ++n;
        }
    }
    out_n[idx] = n;
}

// ------------------------------------------------------------------ launchers

static int g_sms = 0;
static int sm_count() {
    if (!g_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    }
    return g_sms;
}

cudaError_t launch_ray_init(const WaveArgs& a, uint32_t total_tiles, cudaStream_t s) {
    const uint64_t n = (uint64_t)total_tiles * kTileW * kTileH;
    ray_init_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, total_tiles);
    return cudaGetLastError();
}

cudaError_t launch_march(const WaveArgs& a, cudaStream_t s) {
    march_kernel<<<sm_count() * 8, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_sort_samples(const WaveArgs& a, cudaStream_t s) {
    const uint32_t n_bins = a.n_reqs << a.cell_bits;
    cudaError_t e = cudaMemsetAsync(a.sort_bins, 0, (size_t)n_bins * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    sort_count_kernel<<<sm_count() * 8, 256, 0, s>>>(a);
    sort_scan_kernel<<<n_bins / kSortBlock, kSortBlock, 0, s>>>(a.sort_bins, a.sort_block_sums);
    sort_offsets_kernel<<<1, kSortBlock, 0, s>>>(a, n_bins / kSortBlock);
    sort_place_kernel<<<sm_count() * 8, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_nearest_stage(const WaveArgs& a, uint32_t blocks_per_sm, cudaStream_t s) {
    const uint32_t bps = blocks_per_sm ? blocks_per_sm : 16u;
    nearest_stage_kernel<<<sm_count() * bps, 256, (size_t)8 * a.top_nodes * 112u, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_map_encode(const WaveArgs& a, uint32_t blocks_per_sm, cudaStream_t s) {
    const uint32_t bps = blocks_per_sm ? blocks_per_sm : 16u;
    const unsigned grid = sm_count() * bps;
    if (a.fv.n_features == 8) map_encode_kernel<8><<<grid, 256, 0, s>>>(a);
    else if (a.fv.n_features == 4) map_encode_kernel<4><<<grid, 256, 0, s>>>(a);
    else map_encode_kernel<2><<<grid, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_deform_encode(const WaveArgs& a, uint32_t blocks_per_sm, cudaStream_t s) {
    cudaError_t e = launch_nearest_stage(a, blocks_per_sm, s);
    if (e != cudaSuccess) return e;
    return launch_map_encode(a, blocks_per_sm, s);
}

cudaError_t launch_field_fused(const WaveArgs& a, const MlpArgs& m, uint32_t max_tiles, cudaStream_t s, uint32_t ctas_per_sm) {
    const size_t smem = ((sizeof(FusedSmem) + 1023) & ~size_t(1023)) + m.plan.bytes;
    cudaError_t e = cudaFuncSetAttribute(field_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, smem_sm = 0, reserved = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    // as many CTAs as shared memory lets reside, at most 4 (4 x 128 TMEM columns fill an SM)
    int per_sm = smem_sm / (int)(smem + (size_t)reserved);
    per_sm = per_sm < 1 ? 1 : (per_sm > 4 ? 4 : per_sm);
    if (ctas_per_sm && (int)ctas_per_sm < per_sm) per_sm = (int)ctas_per_sm;
    // the shared-memory carveout just large enough for them: the rest stays L1 for the gathers
    const int pct = (int)((100 * (size_t)per_sm * (smem + (size_t)reserved) + (size_t)smem_sm - 1) / (size_t)smem_sm);
    e = cudaFuncSetAttribute(field_tile_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct > 100 ? 100 : pct);
    if (e != cudaSuccess) return e;
    uint32_t grid = (uint32_t)sm_count() * (uint32_t)per_sm;
    if (max_tiles < grid) grid = max_tiles ? max_tiles : 1;
    field_tile_kernel<<<grid, 256, smem, s>>>(a, m);
    return cudaGetLastError();
}

cudaError_t launch_mlp(const MlpArgs& a, uint32_t max_tiles, cudaStream_t s, uint32_t ctas_per_sm, uint32_t slots) {
    const size_t smem = (size_t)mlp2_w_off(a.plan.tile_bytes) + a.plan.bytes;
    const bool fp8 = a.fv.precision == 2;
    const uint8_t* image = a.seg ? a.single : a.fv.mlp_smem;
    if (image && slots == 8 && !fp8 && a.plan.k_in <= 64u) return launch_mlp_pairs(a, image, max_tiles, sm_count(), ctas_per_sm, s);
    // built in: slots for FP8, for batches on one weight image, and for encodings wider than 64
    // (the per-CTA kernel fits two CTAs per SM there; four slots share one copy of the weights)
    const bool want_slots = (slots >= 2 && slots <= 7) || (slots == 0 && (fp8 || (a.seg && a.batch) || a.plan.k_in > 64u));
    if (image && want_slots) {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        uint32_t n_slots = mlp_slots_for(a.plan, optin, fp8);
        if (slots >= 2 && slots < n_slots) n_slots = slots;
        if (n_slots) return launch_mlp_slots(a, image, n_slots, max_tiles, sm_count(), s);
    }
    const void* fn = fp8 ? (const void*)mlp256_kernel<true> : (const void*)mlp256_kernel<false>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    int dev = 0, smem_sm = 0, reserved = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    // contiguous tile ranges: as many CTAs as shared memory lets reside at once (the carveout set
    // to all-shared), at most 4 (4 x 128 TMEM columns fill an SM)
    int per_sm = smem_sm / (int)(smem + (size_t)reserved);
    per_sm = per_sm < 1 ? 1 : (per_sm > 4 ? 4 : per_sm);
    if (ctas_per_sm && (int)ctas_per_sm < per_sm) per_sm = (int)ctas_per_sm;
    uint32_t grid = (uint32_t)sm_count() * (uint32_t)per_sm;
    if (max_tiles < grid) grid = max_tiles ? max_tiles : 1;
    if (fp8) mlp256_kernel<true><<<grid, 256, smem, s>>>(a);
    else mlp256_kernel<false><<<grid, 256, smem, s>>>(a);
    return cudaGetLastError();
}

__global__ void round_begin_kernel(const uint32_t* n_alive_in, uint32_t* n_alive_out, uint32_t* n_samples_round, uint32_t* steps,
                                   uint64_t round_cap, uint32_t max_steps) {
    const uint64_t n = *n_alive_in;
    const uint64_t per = round_cap / (n > 0 ? n : 1);
    *steps = (uint32_t)(per < 1 ? 1 : (per > max_steps ? max_steps : per));
    *n_alive_out = 0u;
    *n_samples_round = 0u;
}

// Between the body's two rounds: the second runs only when the first left rays alive; when it
// does not, its output count (the first round's input count, consumed) is cleared so that the
// loop condition and the host see no ray alive.
__global__ void round_mid_kernel(const uint32_t* a_alive_out, uint32_t* b_alive_out, uint32_t* b_ran, cudaGraphConditionalHandle c) {
    const bool more = *a_alive_out > 0u;
    if (!more) *b_alive_out = 0u;
    *b_ran = more ? 1u : 0u;
    cudaGraphSetConditional(c, more ? 1u : 0u);
}

__global__ void round_end_kernel(const uint32_t* n_alive, uint32_t* rounds, const uint32_t* b_ran, unsigned long long* rounds_total,
                                 uint32_t max_rounds, cudaGraphConditionalHandle cond) {
    const uint32_t ran = 1u + *b_ran;
    const uint32_t r = *rounds + ran;
    *rounds = r;
    *rounds_total += (unsigned long long)ran + (1ull << 40);   // rounds in the low 40 bits, loop iterations above
    cudaGraphSetConditional(cond, (*n_alive > 0u && r < max_rounds) ? 1u : 0u);
}

cudaError_t launch_round_begin(const uint32_t* n_alive_in, uint32_t* n_alive_out, uint32_t* n_samples_round, uint32_t* steps,
                               uint64_t round_cap, uint32_t max_steps, cudaStream_t s) {
    round_begin_kernel<<<1, 1, 0, s>>>(n_alive_in, n_alive_out, n_samples_round, steps, round_cap, max_steps);
    return cudaGetLastError();
}

cudaError_t launch_round_mid(const uint32_t* a_alive_out, uint32_t* b_alive_out, uint32_t* b_ran, cudaGraphConditionalHandle c,
                             cudaStream_t s) {
    round_mid_kernel<<<1, 1, 0, s>>>(a_alive_out, b_alive_out, b_ran, c);
    return cudaGetLastError();
}

cudaError_t launch_round_end(const uint32_t* n_alive, uint32_t* rounds, const uint32_t* b_ran, unsigned long long* rounds_total,
                             uint32_t max_rounds, cudaGraphConditionalHandle cond, cudaStream_t s) {
    round_end_kernel<<<1, 1, 0, s>>>(n_alive, rounds, b_ran, rounds_total, max_rounds, cond);
    return cudaGetLastError();
}

cudaError_t launch_composite(const WaveArgs& a, cudaStream_t s) {
    composite_kernel<<<sm_count() * 8, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_encode_coords(const FieldView& fv, const float* coords, uint32_t stride, int64_t n, uint8_t* tiles,
                                 uint32_t tile_bytes, uint32_t k_in, cudaStream_t s, bool extra_ones) {
    if (n <= 0) return cudaSuccess;
    const unsigned grid = (unsigned)((n + 255) / 256);
    const uint32_t mask = extra_ones ? 0u : 7u;
    if (fv.n_features == 8) encode_coords_kernel<8><<<grid, 256, 0, s>>>(fv, coords, stride, n, tiles, tile_bytes, k_in, mask);
    else if (fv.n_features == 4) encode_coords_kernel<4><<<grid, 256, 0, s>>>(fv, coords, stride, n, tiles, tile_bytes, k_in, mask);
    else encode_coords_kernel<2><<<grid, 256, 0, s>>>(fv, coords, stride, n, tiles, tile_bytes, k_in, mask);
    return cudaGetLastError();
}

cudaError_t launch_unpack(const uint2* out, const float4* out_f32, int bf16, int64_t n, float4* dst, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    unpack_outputs_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, out_f32, bf16, n, dst);
    return cudaGetLastError();
}

cudaError_t launch_training_samples(const TrainArgs& a, float* tbuf, cudaStream_t s) {
    if (a.n_rays <= 0) return cudaSuccess;
    // one ray per thread; small batches (a few thousand rays) in 32-thread blocks so that they spread over every SM
    const int threads = a.n_rays < 152 * 128 ? 32 : 128;
    const unsigned blocks = (unsigned)((a.n_rays + threads - 1) / threads);
    if (tbuf) {
        training_march_kernel<<<blocks, threads, 0, s>>>(a, tbuf);
        training_write_kernel<<<(unsigned)((a.n_rays * 32 + 255) / 256), 256, 0, s>>>(a, tbuf);
    } else {
        training_samples_kernel<<<blocks, threads, 0, s>>>(a);
    }
    return cudaGetLastError();
}

// ------------------------------------------------------------------ canonical map, sorted
// insta_canonical_map_soa on large point sets (the warp hook of src/core.cu:442-526 on bare
// points): a counting sort by 64^3 cell of the frame's box, the warp-cooperative nearest walk over
// 32 sorted neighbours at a time (ids scattered back to the callers' order), then the
// deformed->canonical map per point in the callers' order.
constexpr uint32_t kMapCellBits = 18, kMapBins = 1u << kMapCellBits, kMapBlocks = kMapBins / kSortBlock;

__global__ void __launch_bounds__(256) map_count_kernel(FrameView fr, const float* __restrict__ pts, uint32_t n,
                                                        uint32_t* __restrict__ keys, uint32_t* __restrict__ bins) {
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x) {
        const uint32_t i = b + threadIdx.x;
        const bool valid = i < n;
        uint32_t key = 0xffffffffu;
        if (valid) {
            key = sample_cell(fr, make_float4(pts[(size_t)i * 3], pts[(size_t)i * 3 + 1], pts[(size_t)i * 3 + 2], 0.f), kMapCellBits);
            keys[i] = key;
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        if (valid && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(bins + key, (uint32_t)__popc(peers));
    }
}

// Exclusive scan of the kMapBlocks block totals in place (one block, one total per thread).
__global__ void __launch_bounds__(kSortBlock) map_offsets_kernel(uint32_t* __restrict__ block_sums) {
    __shared__ uint32_t warp_tot[32];
    const uint32_t v = threadIdx.x < kMapBlocks ? block_sums[threadIdx.x] : 0u;
    uint32_t before;
    block_exclusive_scan(v, &before, warp_tot);
    if (threadIdx.x < kMapBlocks) block_sums[threadIdx.x] = before;
}

__global__ void __launch_bounds__(256) map_place_kernel(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ bins,
                                                        const uint32_t* __restrict__ block_sums, uint32_t* __restrict__ order) {
    const uint32_t lane = threadIdx.x & 31u, lt_mask = (1u << lane) - 1u;
    for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x) {
        const uint32_t i = b + threadIdx.x;
        const bool valid = i < n;
        const uint32_t key = valid ? keys[i] : 0xffffffffu;
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (valid && lane == (uint32_t)leader) base = atomicAdd(bins + key, (uint32_t)__popc(peers));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (valid) order[block_sums[key / kSortBlock] + base + __popc(peers & lt_mask)] = i;
    }
}

__global__ void __launch_bounds__(256, 4) map_nearest_kernel(FrameView fr, const float* __restrict__ pts, uint32_t n,
                                                             const uint32_t* __restrict__ order, int32_t* __restrict__ out_idx,
                                                             uint32_t* err) {
    __shared__ WarpScratch wscratch[8];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t n_warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t base = (blockIdx.x * (blockDim.x >> 5) + warp) * 32u; base < n; base += n_warps * 32u) {
        const uint32_t s = base + lane;
        const bool valid = s < n;
        const uint32_t i = valid ? order[s] : 0u;
        const V3 p = valid ? v3(pts[(size_t)i * 3], pts[(size_t)i * 3 + 1], pts[(size_t)i * 3 + 2]) : v3(0.5f, 0.5f, 0.5f);
        const Nearest q = nearest_warp(fr, p, valid, wscratch[warp], err);
        if (valid) out_idx[i] = q.id;
    }
}

__global__ void __launch_bounds__(256) map_canon_kernel(FrameView fr, DeformView dv, const float* __restrict__ pts, uint32_t n,
                                                        const int32_t* __restrict__ idx, float* __restrict__ out_canon, uint32_t* err) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const V3 p = v3(pts[(size_t)i * 3], pts[(size_t)i * 3 + 1], pts[(size_t)i * 3 + 2]);
        const int32_t id = idx[i];
        float o[3] = {p.x, p.y, p.z};
        if (id < 0) atomicOr(err, INSTA_DEVERR_NO_TRI);
        else map_to_canonical(dv, fr.frames, (uint32_t)id, p, nullptr, o, nullptr, nullptr);
        out_canon[(size_t)i * 3] = o[0]; out_canon[(size_t)i * 3 + 1] = o[1]; out_canon[(size_t)i * 3 + 2] = o[2];
    }
}

size_t map_sorted_scratch_bytes(int64_t n) { return ((size_t)n * 2 + kMapBins + kMapBlocks) * sizeof(uint32_t); }

cudaError_t launch_canonical_map_sorted(const FrameView& fv, const DeformView& dv, const float* pts, int64_t n64, int32_t* out_idx,
                                        float* out_canon, void* scratch, uint32_t* err, cudaStream_t s) {
    if (n64 <= 0) return cudaSuccess;
    if (n64 >= (int64_t)1 << 31) return cudaErrorInvalidValue;
    const uint32_t n = (uint32_t)n64;
    uint32_t* keys = static_cast<uint32_t*>(scratch);
    uint32_t* order = keys + n;
    uint32_t* bins = order + n;
    uint32_t* block_sums = bins + kMapBins;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned grid = (unsigned)std::min<int64_t>((n64 + 255) / 256, (int64_t)sms * 8);
    cudaError_t e = cudaMemsetAsync(bins, 0, kMapBins * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    map_count_kernel<<<grid, 256, 0, s>>>(fv, pts, n, keys, bins);
    sort_scan_kernel<<<kMapBlocks, kSortBlock, 0, s>>>(bins, block_sums);
    map_offsets_kernel<<<1, kSortBlock, 0, s>>>(block_sums);
    map_place_kernel<<<grid, 256, 0, s>>>(keys, n, bins, block_sums, order);
    const unsigned grid_w = (unsigned)std::min<int64_t>((n64 + 255) / 256, (int64_t)sms * 4);
    map_nearest_kernel<<<grid_w, 256, 0, s>>>(fv, pts, n, order, out_idx, err);
    map_canon_kernel<<<grid, 256, 0, s>>>(fv, dv, pts, n, out_idx, out_canon, err);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ density-grid warp, sorted
// warp_random_samples (src/core.cu:528-579) for the density-grid update with the samples grouped
// by (frame, 64^3 cell of the sample domain): the frame each sample draws decides its run, the
// render's counting sort (runs padded to 128) orders them, and the warp-cooperative walk runs 32
// neighbours of one frame at a time -- the grid samples lie mostly far from the mesh, where a
// per-sample walk visits a large part of the tree and 32 neighbours share almost all of it.
__global__ void __launch_bounds__(256) gwarp_key_kernel(uint32_t n_frames, const float* __restrict__ coords, uint32_t stride, uint32_t n,
                                                        Pcg32 rng, float3 lo, float3 inv_ext, uint32_t cell_bits,
                                                        uint32_t* __restrict__ keys, uint32_t* __restrict__ bins, uint32_t* __restrict__ n_round) {
    const uint32_t lane = threadIdx.x & 31u;
    if (blockIdx.x == 0 && threadIdx.x == 0) *n_round = n;
    const uint32_t per_axis = 1u << (cell_bits / 3);
    const float top = (float)(per_axis - 1);
    for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x) {
        const uint32_t i = b + threadIdx.x;
        const bool valid = i < n;
        uint32_t key = 0xffffffffu;
        if (valid) {
            Pcg32 r = rng;
            r.advance((int64_t)(uint32_t)(i * n_frames));
            uint32_t fid = (uint32_t)__fmul_rn(r.next_float(), (float)n_frames);
            fid = fid < n_frames ? fid : n_frames - 1;   // next_float < 1, so fid < n_frames already
            const float* c = coords + (size_t)i * stride;
            const float pp[3] = {c[0], c[1], c[2]}, l[3] = {lo.x, lo.y, lo.z}, s[3] = {inv_ext.x, inv_ext.y, inv_ext.z};
            uint32_t q[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) q[k] = (uint32_t)fminf(fmaxf((pp[k] - l[k]) * s[k] * (float)per_axis, 0.f), top);
            key = (fid << cell_bits) | spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
            keys[i] = key;
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        if (valid && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(bins + key, (uint32_t)__popc(peers));
    }
}

__global__ void __launch_bounds__(256, 4) gwarp_nearest_kernel(const FrameView* __restrict__ frames, const float* __restrict__ coords,
                                                               uint32_t stride, const uint32_t* __restrict__ order,
                                                               const uint32_t* __restrict__ keys, const uint32_t* __restrict__ n_padded,
                                                               uint32_t cell_bits, int32_t* __restrict__ ids, uint32_t* err) {
    __shared__ WarpScratch wscratch[8];
    const uint32_t n = *n_padded;   // runs padded to 128: a warp's 32 positions hold one frame
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t n_warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t base = (blockIdx.x * (blockDim.x >> 5) + warp) * 32u; base < n; base += n_warps * 32u) {
        const uint32_t m = order[base + lane];
        const bool valid = m != kNoSample;
        const uint32_t any = __ballot_sync(0xffffffffu, valid);
        if (!any) continue;
        const uint32_t fid = __shfl_sync(0xffffffffu, valid ? keys[m] >> cell_bits : 0u, __ffs(any) - 1);
        const float* c = coords + (size_t)(valid ? m : 0u) * stride;
        const V3 p = valid ? v3(c[0], c[1], c[2]) : v3(0.5f, 0.5f, 0.5f);
        const Nearest q = nearest_warp(frames[fid], p, valid, wscratch[warp], err);
        if (valid) ids[m] = q.id;
    }
}

__global__ void __launch_bounds__(256) gwarp_map_kernel(const FrameView* __restrict__ frames, DeformView dv, float* __restrict__ coords,
                                                        uint32_t stride, uint32_t n, const uint32_t* __restrict__ keys,
                                                        const int32_t* __restrict__ ids, uint32_t cell_bits, uint32_t* err) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int32_t id = ids[i];
        if (id < 0) { atomicOr(err, INSTA_DEVERR_NO_TRI); continue; }
        float* c = coords + (size_t)i * stride;
        float o[3];
        map_to_canonical(dv, frames[keys[i] >> cell_bits].frames, (uint32_t)id, v3(c[0], c[1], c[2]), nullptr, o, nullptr, nullptr);
        c[0] = o[0]; c[1] = o[1]; c[2] = o[2];
    }
}

// The warp hook on NerfCoordinate records in bulk (insta_canonical_map, src/core.cu:442-526):
// the records the hook maps (holder >= 0, a known frame, inside the train box) are sorted by
// (frame, 64^3 cell of the train box) and walked 32 neighbours at a time; the others keep no key
// and stay untouched.
__global__ void __launch_bounds__(256) coords_key_kernel(const FrameView* __restrict__ frames, uint32_t n_frames, int fixed, DeformView dv,
                                                         const float* __restrict__ coords, uint32_t stride, uint32_t n, uint32_t cell_bits,
                                                         uint32_t* __restrict__ keys, uint32_t* __restrict__ bins, uint32_t* __restrict__ n_round,
                                                         const uint32_t* __restrict__ n_dev) {
    const uint32_t lane = threadIdx.x & 31u;
    if (blockIdx.x == 0 && threadIdx.x == 0) *n_round = n;
    const uint32_t n_live = n_dev ? min(n, *n_dev) : n;   // records past a device count get no key
    const uint32_t per_axis = 1u << (cell_bits / 3);
    const float top = (float)(per_axis - 1);
    for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x) {
        const uint32_t i = b + threadIdx.x;
        uint32_t key = 0xffffffffu;
        if (i < n_live) {
            const float* c = coords + (size_t)i * stride;
            const float holder = c[4];
            const V3 p = v3(c[0], c[1], c[2]);
            const uint32_t fid = fixed ? 0u : (uint32_t)holder;
            if (holder >= 0.f && fid < n_frames && box_contains(dv.aabb_min, dv.aabb_max, p) && frames[fid].n_tris > 0) {
                const float pp[3] = {p.x, p.y, p.z};
                uint32_t q[3];
#pragma unroll
                for (int k = 0; k < 3; ++k)
                    q[k] = (uint32_t)fminf(fmaxf((pp[k] - dv.aabb_min[k]) / (dv.aabb_max[k] - dv.aabb_min[k]) * (float)per_axis, 0.f), top);
                key = (fid << cell_bits) | spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
            }
        }
        if (i < n) keys[i] = key;
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        if (key != 0xffffffffu && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(bins + key, (uint32_t)__popc(peers));
    }
}

__global__ void __launch_bounds__(256) coords_map_kernel(const FrameView* __restrict__ frames, DeformView dv, float* __restrict__ coords,
                                                         uint32_t stride, uint32_t n_extra, uint32_t n, const uint32_t* __restrict__ keys,
                                                         const int32_t* __restrict__ ids, uint32_t cell_bits, uint32_t* err) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t key = keys[i];
        if (key == 0xffffffffu) continue;
        const int32_t id = ids[i];
        if (id < 0) { atomicOr(err, INSTA_DEVERR_NO_TRI); continue; }
        float* c = coords + (size_t)i * stride;
        float pos[3], dir[3], dw[3] = {c[8], c[9], c[10]};
        uint32_t mask;
        map_to_canonical(dv, frames[key >> cell_bits].frames, (uint32_t)id, v3(c[0], c[1], c[2]), dw, pos, dir, &mask);
        c[0] = pos[0]; c[1] = pos[1]; c[2] = pos[2];
        c[8] = dir[0]; c[9] = dir[1]; c[10] = dir[2];
        if (mask != 7u)
            for (uint32_t m = 0; m < n_extra; ++m) c[stride - n_extra + m] = 1.f;
    }
}

cudaError_t launch_canonical_map_coords_sorted(const FrameView* frames_dev, uint32_t n_frames, int fixed, const DeformView& dv, float* coords,
                                               uint32_t stride, uint32_t n_extra, uint32_t n, void* scratch, uint32_t* err, cudaStream_t s,
                                               const uint32_t* n_dev) {
    if (n == 0) return cudaSuccess;
    const uint32_t cb = map_cell_bits(n_frames);
    const uint32_t n_bins = n_frames << cb;
    uint32_t* keys = static_cast<uint32_t*>(scratch);
    int32_t* ids = reinterpret_cast<int32_t*>(keys + n);
    uint32_t* order = keys + 2 * (size_t)n;
    uint32_t* bins = order + n + 128u * (size_t)n_frames;
    uint32_t* block_sums = bins + n_bins;
    uint32_t* req_start = block_sums + n_bins / kSortBlock;
    uint32_t* req_seg = req_start + n_frames + 1;
    uint32_t* counters = req_seg + n_frames + 1;
    WaveArgs a{};
    a.n_reqs = n_frames;
    a.cell_bits = cb;
    a.sort_bins = bins;
    a.sort_block_sums = block_sums;
    a.req_start = req_start;
    a.req_seg = req_seg;
    a.sample_order = order;
    a.sample_key = keys;
    a.n_samples_round = counters;
    a.n_samples_padded = counters + 1;
    cudaError_t e = cudaMemsetAsync(bins, 0, (size_t)n_bins * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)std::min<uint32_t>((n + 255) / 256, (uint32_t)sm_count() * 8);
    coords_key_kernel<<<grid, 256, 0, s>>>(frames_dev, n_frames, fixed, dv, coords, stride, n, cb, keys, bins, counters, n_dev);
    sort_scan_kernel<<<n_bins / kSortBlock, kSortBlock, 0, s>>>(bins, block_sums);
    sort_offsets_kernel<<<1, kSortBlock, 0, s>>>(a, n_bins / kSortBlock);
    sort_place_kernel<<<sm_count() * 8, 256, 0, s>>>(a);
    gwarp_nearest_kernel<<<sm_count() * 16, 256, 0, s>>>(frames_dev, coords, stride, order, keys, counters + 1, cb, ids, err);
    coords_map_kernel<<<grid, 256, 0, s>>>(frames_dev, dv, coords, stride, n_extra, n, keys, ids, cb, err);
    return cudaGetLastError();
}

size_t warp_sorted_scratch_bytes(uint32_t n, uint32_t n_frames) {
    const uint32_t cb = map_cell_bits(n_frames);
    const size_t bins = (size_t)n_frames << cb;
    return ((size_t)n * 2 + (size_t)n + 128u * (size_t)n_frames + bins + bins / kSortBlock + 2u * (n_frames + 1u) + 2u) * sizeof(uint32_t);
}

cudaError_t launch_warp_random_sorted(const FrameView* frames_dev, uint32_t n_frames, const DeformView& dv, float* coords, uint32_t stride,
                                      uint32_t n, uint64_t rng_state, uint64_t rng_inc, const float* dom_lo, const float* dom_hi,
                                      void* scratch, uint32_t* err, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint32_t cb = map_cell_bits(n_frames);
    const uint32_t n_bins = n_frames << cb;
    uint32_t* keys = static_cast<uint32_t*>(scratch);
    int32_t* ids = reinterpret_cast<int32_t*>(keys + n);
    uint32_t* order = keys + 2 * (size_t)n;
    uint32_t* bins = order + n + 128u * (size_t)n_frames;
    uint32_t* block_sums = bins + n_bins;
    uint32_t* req_start = block_sums + n_bins / kSortBlock;
    uint32_t* req_seg = req_start + n_frames + 1;
    uint32_t* counters = req_seg + n_frames + 1;
    WaveArgs a{};
    a.n_reqs = n_frames;
    a.cell_bits = cb;
    a.sort_bins = bins;
    a.sort_block_sums = block_sums;
    a.req_start = req_start;
    a.req_seg = req_seg;
    a.sample_order = order;
    a.sample_key = keys;
    a.n_samples_round = counters;
    a.n_samples_padded = counters + 1;
    cudaError_t e = cudaMemsetAsync(bins, 0, (size_t)n_bins * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    Pcg32 r{rng_state, rng_inc};
    const float3 lo = make_float3(dom_lo[0], dom_lo[1], dom_lo[2]);
    const float3 inv = make_float3(1.f / (dom_hi[0] - dom_lo[0]), 1.f / (dom_hi[1] - dom_lo[1]), 1.f / (dom_hi[2] - dom_lo[2]));
    const unsigned grid = (unsigned)std::min<uint32_t>((n + 255) / 256, (uint32_t)sm_count() * 8);
    gwarp_key_kernel<<<grid, 256, 0, s>>>(n_frames, coords, stride, n, r, lo, inv, cb, keys, bins, counters);
    sort_scan_kernel<<<n_bins / kSortBlock, kSortBlock, 0, s>>>(bins, block_sums);
    sort_offsets_kernel<<<1, kSortBlock, 0, s>>>(a, n_bins / kSortBlock);
    sort_place_kernel<<<sm_count() * 8, 256, 0, s>>>(a);
    gwarp_nearest_kernel<<<sm_count() * 16, 256, 0, s>>>(frames_dev, coords, stride, order, keys, counters + 1, cb, ids, err);
    gwarp_map_kernel<<<grid, 256, 0, s>>>(frames_dev, dv, coords, stride, n, keys, ids, cb, err);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ raycast (visualisation)
// rta::Core::raycast_flame (src/core.cu:350-402): init_rays_with_payload_kernel_sdf
// (ngp/src/testbed_sdf.cu:505-577; no slice plane, aperture or octree), the closest hit
// (raytrace_kernel, ngp/src/triangle_bvh.cu:150-166, hits at t < 10), INSTA's shade_kernel_sdf
// (src/core.cu:74-113).  One thread per pixel in 8x4 tiles.
__global__ void __launch_bounds__(256) raycast_kernel(RenderView rv, FrameView fr, float3 center, int color_normal, float* __restrict__ out_rgba,
                                                      float* __restrict__ out_depth, int32_t* __restrict__ out_tri, uint32_t* err) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t tiles_x = ((uint32_t)rv.width + 7u) / 8u;
    const uint32_t tile = t / 32u, in = t % 32u;
    const uint32_t x = (tile % tiles_x) * 8u + in % 8u, y = (tile / tiles_x) * 4u + in / 8u;
    if (x >= (uint32_t)rv.width || y >= (uint32_t)rv.height) return;
    const uint32_t idx = x + (uint32_t)rv.width * y;
    float off[2];
    ld_random_pixel_offset(rv.snap_to_pixel_centers ? 0u : rv.spp, off);
    const float u = __fdiv_rn(__fadd_rn((float)x, off[0]), (float)rv.width);
    const float v = __fdiv_rn(__fadd_rn((float)y, off[1]), (float)rv.height);
    const V3 dc = v3(__fdiv_rn(__fmul_rn(__fsub_rn(u, rv.screen_center[0]), (float)rv.width), rv.focal[0]),
                     __fdiv_rn(__fmul_rn(__fsub_rn(v, rv.screen_center[1]), (float)rv.height), rv.focal[1]), 1.0f);
    const V3 d = normalize_rn(v3(dot_rn(v3(rv.cam[0], rv.cam[1], rv.cam[2]), dc), dot_rn(v3(rv.cam[4], rv.cam[5], rv.cam[6]), dc),
                                 dot_rn(v3(rv.cam[8], rv.cam[9], rv.cam[10]), dc)));
    V3 o = v3(rv.cam[3], rv.cam[7], rv.cam[11]);
    const float t0 = __fadd_rn(fmaxf(aabb_ray_tmin(rv.aabb_min, rv.aabb_max, o, d), 0.0f), 1e-6f);
    o = v3(__fadd_rn(o.x, __fmul_rn(t0, d.x)), __fadd_rn(o.y, __fmul_rn(t0, d.y)), __fadd_rn(o.z, __fmul_rn(t0, d.z)));
    const Nearest h = ray_closest(fr, o, d, 10.0f, err);
    const V3 pos = v3(__fadd_rn(o.x, __fmul_rn(h.d2, d.x)), __fadd_rn(o.y, __fmul_rn(h.d2, d.y)), __fadd_rn(o.z, __fmul_rn(h.d2, d.z)));
    if (h.id < 0 || !box_contains(rv.aabb_min, rv.aabb_max, pos)) {
        if (out_tri) out_tri[idx] = -1;
        return;
    }
    if (out_tri) out_tri[idx] = h.id;
    // Triangle::normal() of the hit, normalised again by the shader
    float col[3];
    {
        const float4* tr = fr.leaf_tris + (size_t)h.slot * INSTA_TRI_F4;
        const float4 q0 = __ldg(tr), q1 = __ldg(tr + 1), q2 = __ldg(tr + 2);
        const V3 a = v3(q0.x, q0.y, q0.z), b = v3(q0.w, q1.x, q1.y), c = v3(q1.z, q1.w, q2.x);
        const V3 nrm = normalize_rn(normalize_rn(cross_rn(sub_rn(b, a), sub_rn(c, a))));
        if (color_normal) {
            col[0] = srgb_to_linear(__fadd_rn(__fmul_rn(0.5f, nrm.x), 0.5f));
            col[1] = srgb_to_linear(__fadd_rn(__fmul_rn(0.5f, nrm.y), 0.5f));
            col[2] = srgb_to_linear(__fadd_rn(__fmul_rn(0.5f, nrm.z), 0.5f));
        } else {
            const float lo[3][3] = {{0.f, 0.f, 1.f}, {1.5f, 0.25f, 0.5f}, {-1.5f, 0.25f, 0.5f}};
            float cs = 0.f;
#pragma unroll
            for (int l = 0; l < 3; ++l) {
                const V3 light = v3(__fadd_rn(center.x, lo[l][0]), __fadd_rn(center.y, lo[l][1]), __fadd_rn(center.z, lo[l][2]));
                cs = __fadd_rn(cs, __fmul_rn(__fmul_rn(1.f / 3.f, fminf(1.f, fmaxf(dot_rn(nrm, light), 0.f))), 0.75f));
            }
            col[0] = col[1] = col[2] = srgb_to_linear(cs);
        }
    }
    reinterpret_cast<float4*>(out_rgba)[idx] = make_float4(col[0], col[1], col[2], 1.0f);
    out_depth[idx] = pos.z;
}

cudaError_t launch_raycast(const RenderView& rv, const FrameView& fr, const float* center, int color_normal, float* out_rgba,
                           float* out_depth, int32_t* out_tri, uint32_t* err, cudaStream_t s) {
    const uint32_t tiles = (((uint32_t)rv.width + 7u) / 8u) * (((uint32_t)rv.height + 3u) / 4u);
    if (tiles == 0) return cudaSuccess;
    raycast_kernel<<<(tiles * 32u + 255u) / 256u, 256, 0, s>>>(rv, fr, make_float3(center[0], center[1], center[2]), color_normal,
                                                              out_rgba, out_depth, out_tri, err);
    return cudaGetLastError();
}

// The deform stage's nearest-triangle query on caller points (32 consecutive points per warp).
__global__ void __launch_bounds__(256, 4) nearest_debug_kernel(FrameView fr, const float* __restrict__ pts, int64_t n,
                                                               int32_t* __restrict__ out, uint32_t* err) {
    __shared__ WarpScratch wscratch[8];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const int64_t n_warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t base = ((int64_t)blockIdx.x * (blockDim.x >> 5) + warp) * 32; base < n; base += n_warps * 32) {
        const int64_t i = base + lane;
        const bool valid = i < n;
        const V3 p = valid ? v3(pts[i * 3], pts[i * 3 + 1], pts[i * 3 + 2]) : v3(0.5f, 0.5f, 0.5f);
        const Nearest q = nearest_warp(fr, p, valid, wscratch[warp], err);
        if (valid) out[i] = q.id;
    }
}

cudaError_t launch_nearest_debug(const FrameView& fr, const float* pts, int64_t n, int32_t* out, uint32_t* err, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 16);
    nearest_debug_kernel<<<(unsigned)blocks, 256, 0, s>>>(fr, pts, n, out, err);
    return cudaGetLastError();
}

cudaError_t launch_march_debug(const RenderView& rv, const uint8_t* bitfield, int max_out, float* out_t, float* out_dt,
                               int32_t* out_n, cudaStream_t s) {
    uint32_t n = (uint32_t)rv.width * (uint32_t)rv.height;
    march_debug_kernel<<<(n + 127) / 128, 128, 0, s>>>(rv, bitfield, max_out, out_t, out_dt, out_n);
    return cudaGetLastError();
}

}  // namespace insta
