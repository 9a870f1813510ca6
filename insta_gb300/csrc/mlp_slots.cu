// mlp_slots.cu -- the avatar MLPs over ready-made operand tiles with several tiles in flight per
// SM: one persistent CTA per SM holds the weight image once, and up to kMaxSlots tile slots, each
// a warpgroup of 128 threads (one sample row per thread) with its own shared-memory tile, its own
// 64 TMEM columns and its own chain (one thread issues the layer's MMAs, every thread of the slot
// waits on the commit mbarrier -- the slot's named barrier is taken once per layer, before the
// issue, and also agrees on the waits' outcome --, the epilogue converts the accumulator into the
// next layer's operand).  The slots synchronise only within themselves, so one
// slot's epilogue overlaps the others' MMAs; compared with mlp256_kernel (four CTAs of 256
// threads per SM, each with its own copy of the weights) more tiles are in flight per SM.  Same
// arithmetic and rounding as mlp256_kernel (FP16 / BF16): NerfNetwork::
// inference_mixed_precision_impl's density and colour MLPs (NGP/nerf_network.h:159-232).
//
// Per slot s: full[s] completes when the tile record has landed (two bulk copies: hash rows, SH
// rows), done[s] at the commit of the slot's current layer.  Hidden activations stay in TMEM as
// the next layer's A operand (after the slots' accumulators: 32 columns per slot for FP16 / BF16,
// 16 for E4M3, so at most 5 / 6 slots fit the 512 columns); only layer 0 (hash rows) and colour
// layer 0 ([density output | SH] rows) read A from shared memory, and the next record is copied
// in once colour layer 0 has completed.  Every wait is bounded (about a second), after which the
// kernel sets INSTA_DEVERR_TIMEOUT and the slot leaves.
#include <cstdint>

#include "device_common.cuh"
#include "mlp_tiles.cuh"
#include "kernels.h"

namespace insta {

namespace {

constexpr uint32_t kMaxSlots = 7;
// TMEM columns of the hidden activations per slot (A operand, 64 values per row)
__host__ __device__ constexpr uint32_t a_cols(bool fp8) { return fp8 ? 16u : 32u; }
__host__ __device__ constexpr uint32_t max_slots_tmem(bool fp8) { return 512u / (64u + a_cols(fp8)); }
constexpr uint32_t kSlotBytes = 24576;    // FP16 / BF16 up to 64 density inputs: [0, 16 KiB) hash rows; SH rows; density rows
constexpr uint32_t kSlotBytes8 = 32768;   // FP8: hash rows (FP16); SH rows (FP16); E4M3 layer input; E4M3 colour input
// FP16 / BF16 slots hold the hash rows in max(16 KiB, the hash tile rounded to 1 KiB), then 4 KiB
// of SH rows and 4 KiB of density rows (wider encodings: 128 hash features + 16 expression dims
// take 36 KiB); FP8 slots take at most 64 density inputs.
__host__ __device__ inline uint32_t hash_region(const TilePlan& P, bool fp8) {
    const uint32_t h = (hash_tile_bytes(P.k_in) + 1023u) & ~1023u;
    return fp8 || h < 16384u ? 16384u : h;
}
__host__ __device__ inline uint32_t slot_bytes(const TilePlan& P, bool fp8) { return fp8 ? kSlotBytes8 : hash_region(P, false) + 8192u; }
constexpr uint32_t kCtlBytes = 1024;

struct SlotCtl {
    uint64_t full[kMaxSlots];
    uint64_t done[kMaxSlots];
    uint64_t bar_w;
    uint32_t tmem_base;
};

// The slot's 128 threads meet at named barrier `id`; true when every thread passed true.
__device__ __forceinline__ bool slot_sync_and(uint32_t id, bool v) {
    uint32_t r;
    asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n barrier.cta.red.and.pred q, %2, 128, p;\n selp.u32 %0, 1, 0, q;\n}\n"
                 : "=r"(r) : "r"(v ? 1u : 0u), "r"(id) : "memory");
    return r != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Layer l of the chain: n_dh density hidden layers, the density output (N = 16), n_rh colour
// hidden layers (the first over [density output | SH]), the colour output (N = 16).
struct LayerOps {
    const uint8_t* a[2];
    const uint8_t* b[2];
    uint32_t k[2];
    int n_ops;
    uint32_t n;
};

__device__ __forceinline__ LayerOps layer_ops(const TilePlan& P, const uint8_t* w, const uint8_t* stage, const uint8_t* sh,
                                              const uint8_t* dens, uint32_t l) {
    LayerOps o{};
    o.n_ops = 1;
    o.n = 64;
    o.a[0] = stage;
    o.k[0] = 64;
    if (l < P.n_dh) {
        o.b[0] = w + P.d_off[l];
        if (l == 0) o.k[0] = P.k_in;
    } else if (l == P.n_dh) {
        o.b[0] = w + P.d_out;
        o.n = 16;
    } else if (l == P.n_dh + 1) {
        o.n_ops = 2;
        o.a[0] = dens; o.b[0] = w + P.r0_dens; o.k[0] = 16;
        o.a[1] = sh; o.b[1] = w + P.r0_sh; o.k[1] = 16;
    } else if (l < P.n_dh + 1 + P.n_rh) {
        o.b[0] = w + P.r_off[l - (P.n_dh + 1)];
    } else {
        o.b[0] = w + P.r_out;
        o.n = 16;
    }
    return o;
}

// FP8 layer l: A the E4M3 layer input (density input padded to k8, then 64-wide hidden rows) or
// the [density output | SH] rows; the image stores colour layer 0 as one K = 32 tile at r0_dens.
__device__ __forceinline__ LayerOps layer_ops8(const TilePlan& P, const uint8_t* w, const uint8_t* a8, const uint8_t* rgb8, uint32_t l) {
    LayerOps o{};
    o.n_ops = 1;
    o.n = 64;
    o.a[0] = a8;
    o.k[0] = 64;
    if (l < P.n_dh) {
        o.b[0] = w + P.d_off[l];
        if (l == 0) o.k[0] = P.k8;
    } else if (l == P.n_dh) {
        o.b[0] = w + P.d_out;
        o.n = 16;
    } else if (l == P.n_dh + 1) {
        o.a[0] = rgb8; o.b[0] = w + P.r0_dens; o.k[0] = 32;
    } else if (l < P.n_dh + 1 + P.n_rh) {
        o.b[0] = w + P.r_off[l - (P.n_dh + 1)];
    } else {
        o.b[0] = w + P.r_out;
        o.n = 16;
    }
    return o;
}

// A 64-wide FP8 hidden layer's epilogue for the thread's own row: dequantise (input row scale a,
// layer weight scale sw), ReLU, the row maximum (the whole row is this thread's, no exchange),
// E4M3 with the new row scale into a8 (K = 64).  Returns the new row scale.  The maximum is taken
// over the raw accumulator values and dequantised once: v -> round(round(v a) sw) is monotone for
// positive scales, so this is the maximum of the dequantised values, bit for bit.
__device__ __forceinline__ float hidden8_row(uint32_t col0, uint32_t acol, float a, float sw) {
    float raw = -__int_as_float(0x7f800000);
#pragma unroll 1
    for (uint32_t c = 0; c < 64u; c += 32u) {
        float v[32];
        tmem_ld32(col0 + c, v);
#pragma unroll
        for (int i = 0; i < 32; ++i) raw = fmaxf(raw, v[i]);
    }
    const float mx = fmaxf(__fmul_rn(__fmul_rn(raw, a), sw), 0.f);
    const float inv = row_inv(mx);
#pragma unroll 1
    for (uint32_t c = 0; c < 64u; c += 32u) {
        float v[32];
        tmem_ld32(col0 + c, v);
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = __fmul_rn(fmaxf(__fmul_rn(__fmul_rn(v[i], a), sw), 0.f), inv);
        uint32_t q[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) q[i] = e4m3x4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
        tmem_st8(acol + c / 4u, q);   // the next layer's A operand: 4 values per column
    }
    tmem_st_wait();
    return row_scale(mx);
}

}  // namespace

template <bool FP8>
__global__ void __launch_bounds__(max_slots_tmem(FP8) * 128, 1) mlp_slots_kernel(const __grid_constant__ MlpArgs A, const uint8_t* wimg,
                                                                      uint32_t n_slots) {
    extern __shared__ __align__(1024) uint8_t smem[];
    SlotCtl& ctl = *reinterpret_cast<SlotCtl*>(smem);
    uint8_t* slots = smem + kCtlBytes;
    const TilePlan& P = A.plan;
    uint8_t* w = slots + n_slots * slot_bytes(P, FP8);
    const uint32_t n_samples = A.n_alive ? *A.n_alive : (uint32_t)A.n_samples;
    const uint32_t n_tiles = (n_samples + 127u) / 128u;
    const uint32_t stride = gridDim.x * n_slots;
    const uint32_t n_layers = P.n_dh + P.n_rh + 2u;
    const uint32_t hash_bytes = hash_tile_bytes(P.k_in), sh_bytes = sh_tile_bytes();
    const bool bf16 = A.fv.precision == 1;
    const uint32_t warp = threadIdx.x >> 5;
    const uint32_t s = threadIdx.x >> 7, r = threadIdx.x & 127u, bar_id = 1u + s;
    if (threadIdx.x == 0) {
        for (uint32_t k = 0; k < n_slots; ++k) {
            mbar_init(&ctl.full[k], 2);
            mbar_init(&ctl.done[k], 1);
        }
        mbar_init(&ctl.bar_w, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // 64 accumulator columns per slot, then the slots' activation columns, allocated as a power of two
    const uint32_t used_cols = n_slots * (64u + a_cols(FP8));
    const uint32_t tmem_cols = used_cols <= 128u ? 128u : (used_cols <= 256u ? 256u : 512u);
    if (warp == 0) tmem_alloc(&ctl.tmem_base, tmem_cols);
    if (threadIdx.x == 0) bulk_load(w, wimg, P.bytes, &ctl.bar_w);
    bool ok = mbar_wait(&ctl.bar_w, 0);
    tc_fence_before();
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    tc_fence_after();
    const uint32_t tmem = ctl.tmem_base;

    uint8_t* st = slots + s * slot_bytes(P, FP8);
    uint8_t* sh = st + hash_region(P, FP8);
    uint8_t* dens = sh + 4096;    // FP16 / BF16 density rows; FP8: the E4M3 layer input
    uint8_t* rgb8 = st + 28672;   // FP8: E4M3 [density output | SH] rows
    const uint32_t col0 = tmem + ((warp & 3u) * 32u << 16) + s * 64u;
    const uint32_t a_col = n_slots * 64u + s * a_cols(FP8);            // the slot's A operand columns
    const uint32_t acol0 = tmem + ((warp & 3u) * 32u << 16) + a_col;   // ... at this thread's lane
    const bool waiter = (warp & 3u) == 0;   // the slot's first warp waits on the mbarriers
    uint32_t n_done = 0, n_loads = 0, n_used = 0;
    uint32_t t = blockIdx.x * n_slots + s;
    auto load = [&](uint32_t tt) {
        const uint8_t* src = A.tiles + (size_t)tt * P.tile_bytes;
        bulk_load(st, src, hash_bytes, &ctl.full[s]);
        bulk_load(sh, src + hash_bytes, sh_bytes, &ctl.full[s]);
    };
    if (t < n_tiles && ok) {
        if (r == 0) load(t);
        ++n_loads;
    }
    bool dok = true;   // this thread's commit waits since the slot's last agreement
    for (; t < n_tiles && ok; t += stride) {
        float o4[4] = {0.f, 0.f, 0.f, 0.f};
        if constexpr (FP8) {
            const float* ls = reinterpret_cast<const float*>(w + P.scales);
            float ra = 1.f;
            for (int l = -1; l < (int)n_layers; ++l) {
                fence_async_smem();
                tc_fence_before();
                bool wok = true;
                if (l == -1 && waiter) wok = mbar_wait(&ctl.full[s], n_used & 1u);
                if (l == -1) ++n_used;
                ok = slot_sync_and(bar_id, wok && dok);
                if (!ok) break;
                tc_fence_after();
                if (l == -1) {
                    // the density input: the FP16 hash row, E4M3 with its own row scale, zero-padded to k8
                    float mx = 0.f;
                    for (uint32_t c = 0; c < P.k_in; c += 16u) {
                        float v[16];
                        load16_half_row(st, P.k_in, c, v, r);
#pragma unroll
                        for (int i = 0; i < 16; ++i) mx = fmaxf(mx, fabsf(v[i]));
                    }
                    ra = row_scale(mx);
                    const float inv = row_inv(mx);
                    for (uint32_t c = 0; c < P.k8; c += 16u) {
                        float v[16];
                        if (c < P.k_in) {
                            load16_half_row(st, P.k_in, c, v, r);
                        } else {
#pragma unroll
                            for (int i = 0; i < 16; ++i) v[i] = 0.f;
                        }
                        store16_e4m3_row(dens, P.k8, c, v, inv, r);
                    }
                    continue;
                }
                if (l == (int)P.n_dh + 1 && r == 0 && t + stride < n_tiles) load(t + stride);   // hash and SH rows are read
                if (l == (int)P.n_dh + 1 && t + stride < n_tiles) ++n_loads;
                if (r == 0) {
                    const LayerOps o = layer_ops8(P, w, dens, rgb8, (uint32_t)l);
                    const uint32_t idesc = idesc_f16(128, o.n, false);
                    const uint32_t a0 = smem_addr(o.a[0]), b0 = smem_addr(o.b[0]);
                    const uint32_t sbo = (o.k[0] / 16u) * 128u;
                    if (l == 0 || l == (int)P.n_dh + 1) {
                        for (uint32_t ks = 0; ks < o.k[0] / 32u; ++ks)
                            umma_f8(tmem + s * 64u, smem_desc(a0 + ks * 256u, 128, sbo), smem_desc(b0 + ks * 256u, 128, sbo), idesc, ks ? 1u : 0u);
                    } else {   // A = the hidden activations in TMEM (K = 64)
                        for (uint32_t ks = 0; ks < 2u; ++ks)
                            umma_f8_ts(tmem + s * 64u, tmem + a_col + ks * 8u, smem_desc(b0 + ks * 256u, 128, sbo), idesc, ks ? 1u : 0u);
                    }
                    umma_commit(&ctl.done[s]);
                }
                dok = mbar_wait(&ctl.done[s], n_done & 1u) && dok;   // every thread; agreed at the next sync
                ++n_done;
                __syncwarp();   // the TMEM loads below are warp-collective
                tc_fence_after();
                const float sw = ls[l];
                if (l == (int)P.n_dh) {
                    float v[16], sv[16];
                    tmem_ld16(col0, v);
#pragma unroll
                    for (int i = 0; i < 16; ++i) v[i] = __fmul_rn(__fmul_rn(v[i], ra), sw);
                    o4[3] = v[0];
                    load16_half_row(sh, 16, 0, sv, r);
                    float mx = 0.f;
#pragma unroll
                    for (int i = 0; i < 16; ++i) mx = fmaxf(mx, fmaxf(fabsf(v[i]), fabsf(sv[i])));
                    ra = row_scale(mx);
                    const float inv = row_inv(mx);
                    store16_e4m3_row(rgb8, 32, 0, v, inv, r);
                    store16_e4m3_row(rgb8, 32, 16, sv, inv, r);
                } else if (l + 1 == (int)n_layers) {
                    float v[16];
                    tmem_ld16(col0, v);
                    o4[0] = __fmul_rn(__fmul_rn(v[0], ra), sw);
                    o4[1] = __fmul_rn(__fmul_rn(v[1], ra), sw);
                    o4[2] = __fmul_rn(__fmul_rn(v[2], ra), sw);
                } else {
                    ra = hidden8_row(col0, acol0, ra, sw);
                }
            }
        } else {
            for (uint32_t l = 0; l < n_layers; ++l) {
                // operands: the record (layer 0) or the rows the previous epilogue wrote
                fence_async_smem();
                tc_fence_before();
                bool wok = true;
                if (l == 0 && waiter) wok = mbar_wait(&ctl.full[s], n_used & 1u);
                if (l == 0) ++n_used;
                ok = slot_sync_and(bar_id, wok && dok);
                if (!ok) break;
                tc_fence_after();
                if (r == 0) {
                    const LayerOps o = layer_ops(P, w, st, sh, dens, l);
                    const uint32_t idesc = idesc_f16(128, o.n, bf16);
                    if (l == 0 || l == P.n_dh + 1) {
                        uint32_t acc = 0;
                        for (int i = 0; i < o.n_ops; ++i) {
                            const uint32_t a0 = smem_addr(o.a[i]), b0 = smem_addr(o.b[i]);
                            const uint32_t sbo = (o.k[i] / 8u) * 128u;
                            for (uint32_t ks = 0; ks < o.k[i] / 16u; ++ks) {
                                umma_f16(tmem + s * 64u, smem_desc(a0 + ks * 256u, 128, sbo), smem_desc(b0 + ks * 256u, 128, sbo), idesc, acc);
                                acc = 1;
                            }
                        }
                    } else {   // A = the hidden activations in TMEM (K = 64)
                        const uint32_t b0 = smem_addr(o.b[0]);
                        for (uint32_t ks = 0; ks < 4u; ++ks)
                            umma_f16_ts(tmem + s * 64u, tmem + a_col + ks * 8u, smem_desc(b0 + ks * 256u, 128, 8u * 128u), idesc, ks ? 1u : 0u);
                    }
                    umma_commit(&ctl.done[s]);
                }
                dok = mbar_wait(&ctl.done[s], n_done & 1u) && dok;   // every thread; agreed at the next sync
                ++n_done;
                __syncwarp();   // the TMEM loads below are warp-collective
                tc_fence_after();
                // hash and SH rows are read once colour layer 0 has completed
                if (l == P.n_dh + 1 && r == 0 && t + stride < n_tiles) load(t + stride);
                if (l == P.n_dh + 1 && t + stride < n_tiles) ++n_loads;
                if (l == P.n_dh) {
                    float v[16];
                    tmem_ld16(col0, v);
                    __half h[16];
    #pragma unroll
                    for (int i = 0; i < 16; ++i) h[i] = to_act(v[i], bf16);
                    o4[3] = from_act(h[0], bf16);
                    store_row(dens, r, 16, h);
                } else if (l + 1 == n_layers) {
                    float v[16];
                    tmem_ld16(col0, v);
                    o4[0] = from_act(to_act(v[0], bf16), bf16);
                    o4[1] = from_act(to_act(v[1], bf16), bf16);
                    o4[2] = from_act(to_act(v[2], bf16), bf16);
                } else {
                    // ReLU, rounding to the activation type, into the next layer's A operand in
                    // TMEM (two values per column)
    #pragma unroll 1
                    for (uint32_t c = 0; c < 64u; c += 32u) {
                        float v[32];
                        tmem_ld32(col0 + c, v);
                        uint32_t p[16];
    #pragma unroll
                        for (int i = 0; i < 16; ++i) p[i] = pack2_relu(v[2 * i], v[2 * i + 1], bf16);
                        tmem_st8(acol0 + c / 2u, p);
                        tmem_st8(acol0 + c / 2u + 8u, p + 8);
                    }
                    tmem_st_wait();
                }
            }
        }
        const uint32_t row = t * 128u + r;
        if (ok && row < n_samples) {
            if (A.fv.precision != 0) {
                A.out_f32[row] = make_float4(o4[0], o4[1], o4[2], o4[3]);
            } else {
                const __half2 rg = __floats2half2_rn(o4[0], o4[1]);
                const __half2 bd = __floats2half2_rn(o4[2], o4[3]);
                A.out[row] = make_uint2(*reinterpret_cast<const uint32_t*>(&rg), *reinterpret_cast<const uint32_t*>(&bd));
            }
        }
    }
    ok = slot_sync_and(bar_id, ok && dok);
    // a record whose copies were issued but not consumed (after a timeout): wait for them
    // (bounded) before shared memory is released
    if (r == 0 && n_loads > n_used) mbar_wait(&ctl.full[s], (n_loads - 1u) & 1u);
    if (!ok && r == 0) atomicOr(A.err, INSTA_DEVERR_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, tmem_cols);
}

// ------------------------------------------------------------------ tile pairs, warp-specialised
// FP16 / BF16 MLPs with two tiles per CTA: 256 epilogue threads (two warpgroups splitting each
// row's 64 columns, as mlp256_kernel) alternate between the two tiles' epilogues and publish each
// tile's next operands on an mbarrier; one more warp issues that tile's next layer at once and
// loads the tile records.  The tensor core runs one tile's layer while the epilogue threads
// convert the other's, and the epilogue threads never wait on the issuing thread.  Hidden
// activations stay in TMEM as the next layer's A operand; 256 TMEM columns and a copy of the
// weights per CTA, two CTAs per SM.  Same arithmetic as mlp256_kernel (bit for bit); measured
// slower than it on the render (0.18 vs 0.13 ms per 512x512 frame): a tuning choice
// (insta_tuning.mlp_slots = 8).
namespace {
constexpr uint32_t kPairEpi = 256;
constexpr uint32_t kPairThreads = kPairEpi + 32;

struct PairCtl {
    uint64_t full[2];      // the tile record has landed (two bulk copies)
    uint64_t done[2];      // the commit of the slot's current layer
    uint64_t opready[2];   // the epilogue threads have written the slot's next operands
    uint64_t bar_w;
    uint32_t tmem_base;
};

// The epilogue threads meet at named barrier 1; true when every one passed true.
__device__ __forceinline__ bool pair_sync_and(bool v) {
    uint32_t r;
    asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n barrier.cta.red.and.pred q, 1, %2, p;\n selp.u32 %0, 1, 0, q;\n}\n"
                 : "=r"(r) : "r"(v ? 1u : 0u), "n"(kPairEpi) : "memory");
    return r != 0;
}
}  // namespace

__global__ void __launch_bounds__(kPairThreads, 2) mlp_pairs_kernel(const __grid_constant__ MlpArgs A, const uint8_t* wimg) {
    extern __shared__ __align__(1024) uint8_t smem[];
    PairCtl& ctl = *reinterpret_cast<PairCtl*>(smem);
    const TilePlan& P = A.plan;
    uint8_t* w = smem + kCtlBytes;
    uint8_t* slot0 = w + ((P.bytes + 1023u) & ~1023u);
    const uint32_t n_samples = A.n_alive ? *A.n_alive : (uint32_t)A.n_samples;
    const uint32_t n_tiles = (n_samples + 127u) / 128u, n_pairs = (n_tiles + 1u) / 2u;
    const uint32_t n_layers = P.n_dh + P.n_rh + 2u;
    const uint32_t hash_bytes = hash_tile_bytes(P.k_in), sh_bytes = sh_tile_bytes();
    const bool bf16 = A.fv.precision == 1;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const bool mma_warp = threadIdx.x >= kPairEpi;
    const uint32_t r = threadIdx.x & 127u, c0 = ((threadIdx.x >> 7) & 1u) * 32u;   // epilogue: row, first column
    if (threadIdx.x == 0) {
        for (int k = 0; k < 2; ++k) {
            mbar_init(&ctl.full[k], 2);
            mbar_init(&ctl.done[k], 1);
            mbar_init(&ctl.opready[k], kPairEpi);
        }
        mbar_init(&ctl.bar_w, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (warp == 0) tmem_alloc(&ctl.tmem_base, 256);
    if (threadIdx.x == 0) bulk_load(w, wimg, P.bytes, &ctl.bar_w);
    bool ok = mbar_wait(&ctl.bar_w, 0);
    tc_fence_before();
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    tc_fence_after();
    const uint32_t tmem = ctl.tmem_base;
    auto stage_of = [&](uint32_t s) { return slot0 + s * kSlotBytes; };   // hash rows, then activations
    uint32_t full_phase = 0u, done_phase = 0u, ready_phase = 0u;          // bit s: slot s's parity
    float dens0 = 0.f, dens1 = 0.f;                                        // per slot: the row's density output

    // The MMA warp: issue layer l of slot s (lane 0), then its commit.
    // Slot s's TMEM: accumulator columns [128 s, 128 s + 64), the hidden activations as the next
    // layer's A operand at 128 s + 64 (32 columns).  Layer 0 (hash rows) and colour layer 0
    // ([density output | SH] rows) read A from shared memory.
    auto issue = [&](uint32_t s, uint32_t l) {
        if (lane != 0) return;
        uint8_t* st = stage_of(s);
        const LayerOps o = layer_ops(P, w, st, st + 16384, st + 20480, l);
        const uint32_t idesc = idesc_f16(128, o.n, bf16);
        const uint32_t d = tmem + s * 128u;
        if (l != 0 && l != P.n_dh + 1) {
            const uint32_t b0 = smem_addr(o.b[0]);
            for (uint32_t ks = 0; ks < 4u; ++ks)
                umma_f16_ts(d, d + 64u + ks * 8u, smem_desc(b0 + ks * 256u, 128, 8u * 128u), idesc, ks ? 1u : 0u);
        } else {
            uint32_t acc = 0;
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                if (i >= o.n_ops) break;
                const uint32_t a0 = smem_addr(o.a[i]), b0 = smem_addr(o.b[i]);
                const uint32_t sbo = (o.k[i] / 8u) * 128u;
                for (uint32_t ks = 0; ks < o.k[i] / 16u; ++ks) {
                    umma_f16(d, smem_desc(a0 + ks * 256u, 128, sbo), smem_desc(b0 + ks * 256u, 128, sbo), idesc, acc);
                    acc = 1;
                }
            }
        }
        umma_commit(&ctl.done[s]);
    };
    // (the parity advances only on success: a record still in flight is waited for at the end)
    auto mma_wait = [&](uint64_t* bar, uint32_t& bits, uint32_t s) -> bool {
        const bool v = __all_sync(0xffffffffu, mbar_wait(bar, (bits >> s) & 1u));
        if (v) bits ^= 1u << s;
        tc_fence_after();
        return v;
    };
    uint32_t pending = 0u;   // MMA warp, bit s: slot s's record copies issued, not yet seen landed
    // The epilogue threads: wait for slot s's commit (warp 0 polls), then release the others.
    auto epi_wait = [&](uint32_t s) -> bool {
        bool v = true;
        if (threadIdx.x < 32u) v = mbar_wait(&ctl.done[s], (done_phase >> s) & 1u);
        done_phase ^= 1u << s;
        v = pair_sync_and(v);
        tc_fence_after();
        return v;
    };
    // The epilogue of layer l of slot s (tile t): ReLU into the activation rows, the density
    // output into the density rows, or the outputs.
    auto epilogue = [&](uint32_t s, uint32_t t, uint32_t l) {
        uint8_t* st = stage_of(s);
        const uint32_t col = tmem + (((warp & 3u) * 32u) << 16) + s * 128u;
        const bool wg0 = threadIdx.x < 128u;
        if (l == P.n_dh) {
            if (wg0) {
                float v[16];
                tmem_ld16(col, v);
                __half h[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) h[i] = to_act(v[i], bf16);
                const float d = from_act(h[0], bf16);
                if (s == 0) dens0 = d; else dens1 = d;
                store_row(st + 20480, r, 16, h);
            }
        } else if (l + 1 == n_layers) {
            if (wg0) {
                float v[16];
                tmem_ld16(col, v);
                const uint32_t row = t * 128u + r;
                if (row < n_samples) {
                    const float o0 = from_act(to_act(v[0], bf16), bf16), o1 = from_act(to_act(v[1], bf16), bf16);
                    const float o2 = from_act(to_act(v[2], bf16), bf16), o3 = s == 0 ? dens0 : dens1;
                    if (A.fv.precision != 0) {
                        A.out_f32[row] = make_float4(o0, o1, o2, o3);
                    } else {
                        const __half2 rg = __floats2half2_rn(o0, o1), bd = __floats2half2_rn(o2, o3);
                        A.out[row] = make_uint2(*reinterpret_cast<const uint32_t*>(&rg), *reinterpret_cast<const uint32_t*>(&bd));
                    }
                }
            }
        } else {
#pragma unroll 1
            for (uint32_t c = c0; c < c0 + 32u; c += 16) {
                float v[16];
                tmem_ld16(col + c, v);
                uint32_t p8[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) p8[i] = pack2_relu(v[2 * i], v[2 * i + 1], bf16);
                tmem_st8(col + 64u + c / 2u, p8);
            }
            tmem_st_wait();
        }
    };

    for (uint32_t p = blockIdx.x; p < n_pairs; p += gridDim.x) {
        const uint32_t ta = 2u * p, tb = 2u * p + 1u;
        const bool has_b = tb < n_tiles;
        // both slots' buffers and TMEM columns are free: the previous pair finished on both sides
        tc_fence_before();
        ok = __syncthreads_and(ok ? 1 : 0) != 0;
        tc_fence_after();
        if (!ok) break;
        if (mma_warp) {
            if (lane == 0) {
                for (uint32_t s = 0; s < (has_b ? 2u : 1u); ++s) {
                    const uint8_t* src = A.tiles + (size_t)(2u * p + s) * P.tile_bytes;
                    bulk_load(stage_of(s), src, hash_bytes, &ctl.full[s]);
                    bulk_load(stage_of(s) + 16384, src + hash_bytes, sh_bytes, &ctl.full[s]);
                }
            }
            pending = has_b ? 3u : 1u;
            ok = mma_wait(&ctl.full[0], full_phase, 0);
            if (ok) {
                pending &= ~1u;
                issue(0, 0);
            }
            if (ok && has_b) {
                ok = mma_wait(&ctl.full[1], full_phase, 1);
                if (ok) {
                    pending &= ~2u;
                    issue(1, 0);
                }
            }
            for (uint32_t l = 0; l + 1 < n_layers && ok; ++l) {
                ok = mma_wait(&ctl.opready[0], ready_phase, 0);
                if (!ok) break;
                issue(0, l + 1);
                if (has_b) {
                    ok = mma_wait(&ctl.opready[1], ready_phase, 1);
                    if (!ok) break;
                    issue(1, l + 1);
                }
            }
        } else {
            for (uint32_t l = 0; l < n_layers; ++l) {
                ok = epi_wait(0);
                if (!ok) break;
                epilogue(0, ta, l);
                if (l + 1 < n_layers) {
                    fence_async_smem();
                    tc_fence_before();
                    mbar_arrive(&ctl.opready[0]);
                }
                if (has_b) {
                    ok = epi_wait(1);
                    if (!ok) break;
                    epilogue(1, tb, l);
                    if (l + 1 < n_layers) {
                        fence_async_smem();
                        tc_fence_before();
                        mbar_arrive(&ctl.opready[1]);
                    }
                }
            }
        }
    }
    // records whose copies were issued but not seen landed (after a timeout): wait for them
    // (bounded) before shared memory is released
    if (mma_warp && lane == 0)
        for (uint32_t s = 0; s < 2u; ++s)
            if ((pending >> s) & 1u) mbar_wait(&ctl.full[s], (full_phase >> s) & 1u);
    if (!ok && (threadIdx.x == 0 || (mma_warp && lane == 0))) atomicOr(A.err, INSTA_DEVERR_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 256);
}

cudaError_t launch_mlp_pairs(const MlpArgs& a, const uint8_t* image, uint32_t max_tiles, int n_sms, uint32_t ctas_per_sm, cudaStream_t s) {
    const size_t smem = kCtlBytes + ((a.plan.bytes + 1023u) & ~1023u) + 2u * kSlotBytes;
    cudaError_t e = cudaFuncSetAttribute(mlp_pairs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(mlp_pairs_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    int dev = 0, smem_sm = 0, reserved = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    int per_sm = smem_sm / (int)(smem + (size_t)reserved);
    per_sm = per_sm < 1 ? 1 : (per_sm > 2 ? 2 : per_sm);   // 2 x 256 TMEM columns
    if (ctas_per_sm && (int)ctas_per_sm < per_sm) per_sm = (int)ctas_per_sm;
    uint32_t grid = (uint32_t)n_sms * (uint32_t)per_sm;
    const uint32_t pairs = (max_tiles + 1u) / 2u;
    if (pairs < grid) grid = pairs ? pairs : 1;
    mlp_pairs_kernel<<<grid, kPairThreads, smem, s>>>(a, image);
    return cudaGetLastError();
}

uint32_t mlp_slots_for(const TilePlan& P, int smem_optin, bool fp8) {
    if (fp8 && (P.k_in > 64u || P.k8 > 64u)) return 0;
    const long avail = (long)smem_optin - (long)kCtlBytes - (long)((P.bytes + 1023u) & ~1023u);
    long n = avail / (long)slot_bytes(P, fp8);
    if (n > (long)max_slots_tmem(fp8)) n = max_slots_tmem(fp8);
    return n < 2 ? 0u : (uint32_t)n;
}

cudaError_t launch_mlp_slots(const MlpArgs& a, const uint8_t* image, uint32_t n_slots, uint32_t max_tiles, int n_sms, cudaStream_t s) {
    const bool fp8 = a.fv.precision == 2;
    const size_t smem = kCtlBytes + (size_t)n_slots * slot_bytes(a.plan, fp8) + a.plan.bytes;
    const void* fn = fp8 ? (const void*)mlp_slots_kernel<true> : (const void*)mlp_slots_kernel<false>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    uint32_t grid = (uint32_t)n_sms;
    const uint32_t need = (max_tiles + n_slots - 1) / n_slots;
    if (need < grid) grid = need ? need : 1;
    if (fp8) mlp_slots_kernel<true><<<grid, n_slots * 128, smem, s>>>(a, image, n_slots);
    else mlp_slots_kernel<false><<<grid, n_slots * 128, smem, s>>>(a, image, n_slots);
    return cudaGetLastError();
}

}  // namespace insta
