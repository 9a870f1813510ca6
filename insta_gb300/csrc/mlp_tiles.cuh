// mlp_tiles.cuh -- the avatar MLPs on 128-sample tiles with tcgen05 (M = 128, FP32 accumulators
// in TMEM).  Inputs arrive as ready-made operand tiles in global memory (written by the encode
// stage in the no-swizzle K-major core-matrix layout of umma.cuh) and are moved into shared
// memory by bulk (TMA) copies, double-buffered so tile t+1 loads while tile t computes.
#pragma once

#include "umma.cuh"

namespace insta {

// Weight image layout (each entry one B-operand tile, byte offset into the image):
//   d[0 .. n_dh]      density hidden layers  (N = 64, K = k_in then 64)
//   d_out             density output         (N = 16, K = 64)
//   r0_dens, r0_sh    colour layer 0 split by input columns (N = 64, K = 16 each)
//   r[0 .. n_rh-1)    further colour hidden layers (N = 64, K = 64)
//   r_out             colour output, padded  (N = 16, K = 64)
struct TilePlan {
    uint32_t d_off[4];
    uint32_t n_dh;        // density hidden layers
    uint32_t d_out;
    uint32_t r0_dens, r0_sh;
    uint32_t r_off[4];
    uint32_t n_rh;        // colour hidden layers (>= 1; the first is r0)
    uint32_t r_out;
    uint32_t bytes;       // image size
    uint32_t k_in;        // density input width (32 or 48)
    uint32_t tile_bytes;  // one input tile record: hash tile + SH tile
    // FP8 image: the density input padded to k8 (multiple of 32), colour layer 0 as one K = 32
    // tile at r0_dens ([density out | SH]); every tile stores one byte per weight
    uint32_t k8;
    uint32_t scales;      // FP8 image: byte offset of the 8 per-layer weight scales (float)
};

__host__ __device__ constexpr uint32_t hash_tile_bytes(uint32_t k_in) { return 128u * k_in * 2u; }
__host__ __device__ constexpr uint32_t sh_tile_bytes() { return 128u * 16u * 2u; }

struct ReqView;

struct MlpArgs {
    FieldView fv;
    TilePlan plan;
    const uint8_t* tiles;
    const uint32_t* n_alive;   // render rounds: device count of the round's (padded) samples
    int64_t n_samples;         // used when n_alive is null
    // render batches: tile t belongs to the request r with seg[r] <= 128 t < seg[r + 1] and uses
    // that request's weight image; null when every tile uses fv.mlp_smem
    const uint32_t* seg;
    const ReqView* reqs;
    uint32_t n_reqs;
    uint2* out;                // FP16 (r, g, b, density) per sample
    float4* out_f32;           // BF16 path: FP32 copies of the BF16-rounded values
    uint32_t* err;
    // render batches whose requests all use one weight image: that image (tiles then need no
    // per-tile lookup), else null
    const uint8_t* single;
    uint32_t batch;            // render batch of two or more requests (the built-in slot choice)
};

// slots (insta_tuning.mlp_slots): 2..7 = mlp_slots_kernel with that many slots where every tile
// uses one weight image; 8 = mlp_pairs_kernel there (FP16 / BF16); 1 = mlp256_kernel; 0 =
// mlp_slots_kernel for FP8 fields, for render batches on one weight image and for encodings
// wider than 64, else mlp256_kernel.  ctas_per_sm: mlp256_kernel's resident CTAs per SM
// (0 = as many as shared memory lets reside, at most 4).
cudaError_t launch_mlp(const MlpArgs& a, uint32_t max_tiles, cudaStream_t s, uint32_t ctas_per_sm = 0, uint32_t slots = 0);
// mlp_slots.cu: slots that fit the opt-in shared memory (0 = the kernel does not apply), launch
uint32_t mlp_slots_for(const TilePlan& P, int smem_optin, bool fp8);
cudaError_t launch_mlp_slots(const MlpArgs& a, const uint8_t* image, uint32_t n_slots, uint32_t max_tiles, int n_sms, cudaStream_t s);
// mlp_slots.cu: FP16 / BF16, two tiles per CTA with an MMA-issuing warp
cudaError_t launch_mlp_pairs(const MlpArgs& a, const uint8_t* image, uint32_t max_tiles, int n_sms, uint32_t ctas_per_sm, cudaStream_t s);

// One MMA chain: sum over (A_i, B_i) pairs into TMEM columns [col, col + N).  K in elements;
// f8: E4M3 operands (kind::f8f6f4, 32 elements per instruction), else FP16/BF16 (16 per
// instruction).  Either way one instruction consumes 32 bytes of each row.
template <typename Smem>
__device__ __forceinline__ bool issue_chain(Smem& sm, const uint8_t* const* a, const uint8_t* const* b, const uint32_t* K,
                                            int n, uint32_t N, uint32_t col, bool bf16, uint32_t& phase, bool f8 = false) {
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
        tc_fence_after();
        const uint32_t idesc = idesc_f16(128, N, bf16 && !f8);
        uint32_t acc = 0;
        for (int i = 0; i < n; ++i) {
            const uint32_t a0 = smem_addr(a[i]), b0 = smem_addr(b[i]);
            const uint32_t kbytes = f8 ? K[i] : 2 * K[i];
            const uint32_t sbo = (kbytes / 16) * 128;
            for (uint32_t ks = 0; ks < kbytes / 32; ++ks) {
                if (f8) umma_f8(sm.tmem_base + col, smem_desc(a0 + ks * 256, 128, sbo), smem_desc(b0 + ks * 256, 128, sbo), idesc, acc);
                else umma_f16(sm.tmem_base + col, smem_desc(a0 + ks * 256, 128, sbo), smem_desc(b0 + ks * 256, 128, sbo), idesc, acc);
                acc = 1;
            }
        }
        umma_commit(&sm.bar_mma);
    }
    // every thread waits for the chain's commit on the mbarrier (try_wait suspends the warp until
    // the phase completes, so no CTA barrier is needed after it; measured 0.128 -> 0.124 ms per
    // 512x512 frame against warp 0 polling and a CTA barrier), then orders its TMEM reads after
    // it.  A wait that gives up makes only that thread's result false: the tile loop agrees on it
    // at its closing barrier.
    const bool ok = mbar_wait(&sm.bar_mma, phase);
    phase ^= 1u;
    __syncwarp();   // the epilogue's TMEM loads are warp-collective
    tc_fence_after();
    return ok;
}

// TMEM columns of the 256-thread kernels (128 allocated per CTA): the 64-wide accumulator, the
// 16-wide output-layer accumulator, and a hidden layer's activations as the next layer's A
// operand (64 FP16/BF16 values per row = 32 columns).
constexpr uint32_t kTmemAcc16 = 64u, kTmemA = 96u;

// The same chain with A = the activations in TMEM (kTmemA, K = 64) and B from shared memory.
// Either way one instruction consumes 32 bytes of each row (8 TMEM columns of A).
template <typename Smem>
__device__ __forceinline__ bool issue_chain_ts(Smem& sm, const uint8_t* b, uint32_t N, uint32_t col, bool bf16, uint32_t& phase,
                                               bool f8 = false) {
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
        tc_fence_after();
        const uint32_t idesc = idesc_f16(128, N, bf16 && !f8);
        const uint32_t b0 = smem_addr(b);
        if (f8) {
            for (uint32_t ks = 0; ks < 2u; ++ks)
                umma_f8_ts(sm.tmem_base + col, sm.tmem_base + kTmemA + ks * 8u, smem_desc(b0 + ks * 256u, 128, 4u * 128u), idesc, ks ? 1u : 0u);
        } else {
            for (uint32_t ks = 0; ks < 4u; ++ks)
                umma_f16_ts(sm.tmem_base + col, sm.tmem_base + kTmemA + ks * 8u, smem_desc(b0 + ks * 256u, 128, 8u * 128u), idesc, ks ? 1u : 0u);
        }
        umma_commit(&sm.bar_mma);
    }
    const bool ok = mbar_wait(&sm.bar_mma, phase);
    phase ^= 1u;
    __syncwarp();   // the epilogue's TMEM loads are warp-collective
    tc_fence_after();
    return ok;
}

// ------------------------------------------------------------------ fused tiles (256 threads)
// Shared memory of the fused deform + encode + MLP kernel: one 128-sample tile at a time per CTA,
// encoded in place by the CTA's own threads (two per sample), so the operand rows never leave the
// SM.  a_h first carries the deform stage's hand-off to the encode (canonical position, direction
// and region of each row); the hash rows of `stage` are dead once density layer 0 has run and then
// hold the density output rows (colour input part 1).
struct FusedSmem {
    alignas(1024) uint8_t stage[128 * 64 * 2];   // hash rows [128][k_in], then SH rows [128][16]
    alignas(1024) uint8_t a_h[128 * 64 * 2];     // hidden activations
    alignas(8) uint64_t bar_mma;
    alignas(8) uint64_t bar_w;
    uint32_t tmem_base;
};

// Shared memory of the 256-thread MLP kernel over ready-made operand tiles: the tile record is
// brought in by two bulk copies -- its hash rows once density layer 0 of the previous tile has run,
// its SH rows once colour layer 0 has -- so the next tile loads while this one computes.
// Dynamic shared memory, in 1 KiB-aligned pieces sized by the tile plan: control block, a_h
// [128][64], the tile record (tile_bytes), a_dens [128][16], the weight image.
struct Mlp2Ctl {
    uint64_t bar_mma;
    uint64_t bar_load;   // both parts of the next tile (two arrivals)
    uint64_t bar_w;
    uint32_t tmem_base;
};
struct Mlp2View {
    uint64_t& bar_mma;
    uint32_t& tmem_base;
    uint8_t* stage;
    uint8_t* a_h;
    uint8_t* a_dens;
    uint8_t* w;
};
__host__ __device__ constexpr uint32_t mlp2_round(uint32_t b) { return (b + 1023u) & ~1023u; }
__host__ __device__ constexpr uint32_t mlp2_xch_off() { return 1024u; }   // FP8: [2][128] row maxima
__host__ __device__ constexpr uint32_t mlp2_a_h_off() { return 2048u; }
__host__ __device__ constexpr uint32_t mlp2_stage_off() { return 2048u + 128u * 64u * 2u; }
__host__ __device__ constexpr uint32_t mlp2_dens_off(uint32_t tile_bytes) { return mlp2_stage_off() + mlp2_round(tile_bytes); }
__host__ __device__ constexpr uint32_t mlp2_w_off(uint32_t tile_bytes) { return mlp2_dens_off(tile_bytes) + 128u * 16u * 2u; }

struct NoHook {
    __device__ void operator()() const {}
};

template <typename Smem>
__device__ __forceinline__ uint32_t fused_lane_addr(const Smem& sm, uint32_t col) {
    return sm.tmem_base + ((((uint32_t)threadIdx.x / 32u) % 4u) * 32u << 16) + col;
}

// ReLU + rounding of 64 accumulator columns into the next layer's A operand in TMEM (kTmemA);
// warpgroup g (threads 128 g ...) takes columns [32 g, 32 g + 32) of its row (TMEM lane quarter =
// warp % 4), i.e. A columns [16 g, 16 g + 16).
template <typename Smem>
__device__ __forceinline__ void relu_to_tmem_a(Smem& sm, bool bf16) {
    const uint32_t c0 = (threadIdx.x >> 7) * 32u;
#pragma unroll 1
    for (uint32_t c = c0; c < c0 + 32u; c += 16) {
        float v[16];
        tmem_ld16(fused_lane_addr(sm, c), v);
        uint32_t p[8];   // ReLU, then both values of a pair rounded by one packed conversion
#pragma unroll
        for (int i = 0; i < 8; ++i) p[i] = pack2_relu(v[2 * i], v[2 * i + 1], bf16);
        tmem_st8(fused_lane_addr(sm, kTmemA + c / 2u), p);
    }
    tmem_st_wait();
}

// Both MLPs (FP16 or BF16) with 256 threads on the tile in sm.stage; warpgroup 0 returns its
// row's (r, g, b, raw density): the density MLP's hidden layers (ReLU), its 16 outputs (raw
// density in column 0) rounded to the activation type, then the colour MLP on [those | SH].  hash_free / sh_free run
// (all threads) as soon as the tensor core is done with the hash rows / the SH rows.
template <typename Smem, typename HashFree = NoHook, typename ShFree = NoHook>
__device__ __forceinline__ bool mlp256(Smem& sm, uint8_t* a_dens, const uint8_t* w, const TilePlan& P, bool bf16, uint32_t& phase,
                                       float* out4, HashFree hash_free = HashFree(), ShFree sh_free = ShFree()) {
    bool ok = true;
    const uint8_t* hash = sm.stage;
    const uint8_t* sh = sm.stage + hash_tile_bytes(P.k_in);
    const bool wg0 = threadIdx.x < 128u;
    const uint8_t* a;
    const uint8_t* b;
    uint32_t K;
    a = hash; b = w + P.d_off[0]; K = P.k_in;
    ok &= issue_chain(sm, &a, &b, &K, 1, 64, 0, bf16, phase);
    hash_free();
    relu_to_tmem_a(sm, bf16);
    for (uint32_t l = 1; l < P.n_dh; ++l) {
        ok &= issue_chain_ts(sm, w + P.d_off[l], 64, 0, bf16, phase);
        relu_to_tmem_a(sm, bf16);
    }
    ok &= issue_chain_ts(sm, w + P.d_out, 16, kTmemAcc16, bf16, phase);
    if (wg0) {
        float v[16];
        tmem_ld16(fused_lane_addr(sm, kTmemAcc16), v);
        __half h[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) h[i] = to_act(v[i], bf16);
        out4[3] = from_act(h[0], bf16);
        store_row(a_dens, threadIdx.x, 16, h);
    }
    {
        const uint8_t* as[2] = {a_dens, sh};
        const uint8_t* bs[2] = {w + P.r0_dens, w + P.r0_sh};
        const uint32_t Ks[2] = {16, 16};
        ok &= issue_chain(sm, as, bs, Ks, 2, 64, 0, bf16, phase);
        sh_free();
        relu_to_tmem_a(sm, bf16);
    }
    for (uint32_t l = 1; l < P.n_rh; ++l) {
        ok &= issue_chain_ts(sm, w + P.r_off[l], 64, 0, bf16, phase);
        relu_to_tmem_a(sm, bf16);
    }
    ok &= issue_chain_ts(sm, w + P.r_out, 16, kTmemAcc16, bf16, phase);
    if (wg0) {
        float v[16];
        tmem_ld16(fused_lane_addr(sm, kTmemAcc16), v);
        out4[0] = from_act(to_act(v[0], bf16), bf16);
        out4[1] = from_act(to_act(v[1], bf16), bf16);
        out4[2] = from_act(to_act(v[2], bf16), bf16);
    }
    return ok;
}

// ------------------------------------------------------------------ FP8 (E4M3) variant
// Every layer input row gets its own scale a = max|x| / 448 (rounded to E4M3 after multiplying by
// 448 / max|x|); weights carry a per-layer scale s; the FP32 accumulator is multiplied back by a,
// then s.
// Four values to E4M3 (round to nearest even, saturating to the finite range), a in the lowest
// byte: two packed conversions of two values each.
__device__ __forceinline__ uint32_t e4m3x4(float a, float b, float c, float d) {
    const uint32_t lo = (uint32_t)__nv_cvt_float2_to_fp8x2(make_float2(a, b), __NV_SATFINITE, __NV_E4M3);
    const uint32_t hi = (uint32_t)__nv_cvt_float2_to_fp8x2(make_float2(c, d), __NV_SATFINITE, __NV_E4M3);
    return (lo & 0xffffu) | (hi << 16);
}

// 16 values of row r, times `inv` (448 / row max), as E4M3 into columns [k, k + 16) of an A tile.
__device__ __forceinline__ void store16_e4m3_row(uint8_t* tile, uint32_t K, uint32_t k, const float* v, float inv, uint32_t r) {
    float q[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) q[i] = __fmul_rn(v[i], inv);
    uint4 u;
    u.x = e4m3x4(q[0], q[1], q[2], q[3]);
    u.y = e4m3x4(q[4], q[5], q[6], q[7]);
    u.z = e4m3x4(q[8], q[9], q[10], q[11]);
    u.w = e4m3x4(q[12], q[13], q[14], q[15]);
    *reinterpret_cast<uint4*>(tile + tile_offset8(r, k, K)) = u;
}

// Row scale a = max / 448 (multiplies the accumulator back) and its quantising factor 448 / max.
__device__ __forceinline__ float row_scale(float mx) { return mx > 0.f ? __fdiv_rn(mx, 448.0f) : 1.0f; }
__device__ __forceinline__ float row_inv(float mx) { return mx > 0.f ? __fdiv_rn(448.0f, mx) : 1.0f; }

__device__ __forceinline__ void load16_half_row(const uint8_t* tile, uint32_t K, uint32_t k, float* v, uint32_t r) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const uint4 u = *reinterpret_cast<const uint4*>(tile + tile_offset(r, k + 8 * q, K));
        const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&w[i]));
            v[8 * q + 2 * i] = f.x;
            v[8 * q + 2 * i + 1] = f.y;
        }
    }
}

// Write one FP16 row of a tile record in global memory (K values, K multiple of 8).
__device__ __forceinline__ void store_row_global(uint8_t* tile, uint32_t r, uint32_t K, const __half* v) {
    for (uint32_t c = 0; c < K / 8; ++c) {
        uint4 q;
        q.x = *reinterpret_cast<const uint32_t*>(&v[c * 8 + 0]);
        q.y = *reinterpret_cast<const uint32_t*>(&v[c * 8 + 2]);
        q.z = *reinterpret_cast<const uint32_t*>(&v[c * 8 + 4]);
        q.w = *reinterpret_cast<const uint32_t*>(&v[c * 8 + 6]);
        *reinterpret_cast<uint4*>(tile + tile_offset(r, c * 8, K)) = q;
    }
}

}  // namespace insta

namespace insta {

// ------------------------------------------------------------------ FP8 with 256 threads
// The FP8 chain with the row work split between the warpgroups: each quantises half of a row's
// columns; the row maximum that sets the row scale is exchanged through `xch` ([2][128] floats),
// so both halves use the same scale.
__device__ __forceinline__ float row_max2(float* xch, float m) {
    const uint32_t r = threadIdx.x & 127u, g = threadIdx.x >> 7;
    xch[g * 128u + r] = m;
    __syncthreads();
    const float o = xch[(g ^ 1u) * 128u + r];
    __syncthreads();   // the buffer is reused by the next exchange
    return fmaxf(m, o);
}

// (The maximum is taken over the raw accumulator values and dequantised once: v ->
// round(round(v a) s) is monotone for positive scales, so this is the maximum of the dequantised
// values, bit for bit.)
template <typename Smem>
__device__ __forceinline__ float hidden_to_e4m3_2(Smem& sm, float* xch, float a, float s) {
    const uint32_t c0 = (threadIdx.x >> 7) * 32u;
    float raw = -__int_as_float(0x7f800000);
#pragma unroll 1
    for (uint32_t c = c0; c < c0 + 32u; c += 16) {
        float v[16];
        tmem_ld16(fused_lane_addr(sm, c), v);
#pragma unroll
        for (int i = 0; i < 16; ++i) raw = fmaxf(raw, v[i]);
    }
    float mx = fmaxf(__fmul_rn(__fmul_rn(raw, a), s), 0.f);
    mx = row_max2(xch, mx);
    const float inv = row_inv(mx);
#pragma unroll 1
    for (uint32_t c = c0; c < c0 + 32u; c += 16) {
        float v[16];
        tmem_ld16(fused_lane_addr(sm, c), v);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = __fmul_rn(fmaxf(__fmul_rn(__fmul_rn(v[i], a), s), 0.f), inv);
        // E4M3 into the next layer's A operand in TMEM: 4 values per column
        tmem_st4(fused_lane_addr(sm, kTmemA + c / 4u), e4m3x4(v[0], v[1], v[2], v[3]), e4m3x4(v[4], v[5], v[6], v[7]),
                 e4m3x4(v[8], v[9], v[10], v[11]), e4m3x4(v[12], v[13], v[14], v[15]));
    }
    tmem_st_wait();
    return row_scale(mx);
}

template <typename Smem, typename HashFree = NoHook, typename ShFree = NoHook>
__device__ __forceinline__ bool mlp256_8(Smem& sm, float* xch, uint8_t* a_rgb8, const uint8_t* w, const TilePlan& P, const float* ls,
                                         uint32_t& phase, float* out4, HashFree hash_free = HashFree(), ShFree sh_free = ShFree()) {
    bool ok = true;
    const uint32_t r = threadIdx.x & 127u, g = threadIdx.x >> 7;
    const bool wg0 = g == 0u;
    const uint8_t* hash = sm.stage;
    const uint8_t* sh = sm.stage + hash_tile_bytes(P.k_in);
    uint8_t* a_in8 = sm.a_h;           // [128][k8 <= 128] E4M3 (the hidden layers' inputs stay in TMEM)
    const uint8_t* a;
    const uint8_t* b;
    uint32_t K;
    int li = 0;
    // density input: the FP16 hash row (k_in values, zero-padded to k8), half the columns each
    const uint32_t half = P.k8 / 2u, c0 = g * half;
    float mx = 0.f;
    for (uint32_t c = c0; c < c0 + half; c += 16) {
        if (c >= P.k_in) continue;
        float v[16];
        load16_half_row(hash, P.k_in, c, v, r);
#pragma unroll
        for (int i = 0; i < 16; ++i) mx = fmaxf(mx, fabsf(v[i]));
    }
    mx = row_max2(xch, mx);
    float ra = row_scale(mx);
    const float inv0 = row_inv(mx);
    for (uint32_t c = c0; c < c0 + half; c += 16) {
        float v[16];
        if (c < P.k_in) load16_half_row(hash, P.k_in, c, v, r);
        else {
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = 0.f;
        }
        store16_e4m3_row(a_in8, P.k8, c, v, inv0, r);
    }
    a = a_in8; b = w + P.d_off[0]; K = P.k8;
    ok &= issue_chain(sm, &a, &b, &K, 1, 64, 0, false, phase, true);
    hash_free();
    ra = hidden_to_e4m3_2(sm, xch, ra, ls[li++]);
    for (uint32_t l = 1; l < P.n_dh; ++l) {
        ok &= issue_chain_ts(sm, w + P.d_off[l], 64, 0, false, phase, true);
        ra = hidden_to_e4m3_2(sm, xch, ra, ls[li++]);
    }
    // density output (16): raw density is column 0; colour input = [density out | SH] (warpgroup 0)
    ok &= issue_chain_ts(sm, w + P.d_out, 16, kTmemAcc16, false, phase, true);
    float dens[16], shv[16];
    mx = 0.f;
    if (wg0) {
        float v[16];
        tmem_ld16(fused_lane_addr(sm, kTmemAcc16), v);
        const float sd = ls[li];
#pragma unroll
        for (int i = 0; i < 16; ++i) dens[i] = __fmul_rn(__fmul_rn(v[i], ra), sd);
        out4[3] = dens[0];
        load16_half_row(sh, 16, 0, shv, r);
#pragma unroll
        for (int i = 0; i < 16; ++i) mx = fmaxf(mx, fmaxf(fabsf(dens[i]), fabsf(shv[i])));
    }
    ++li;
    mx = row_max2(xch, mx);
    ra = row_scale(mx);
    if (wg0) {
        store16_e4m3_row(a_rgb8, 32, 0, dens, row_inv(mx), r);
        store16_e4m3_row(a_rgb8, 32, 16, shv, row_inv(mx), r);
    }
    a = a_rgb8; b = w + P.r0_dens; K = 32;
    ok &= issue_chain(sm, &a, &b, &K, 1, 64, 0, false, phase, true);
    sh_free();
    ra = hidden_to_e4m3_2(sm, xch, ra, ls[li++]);
    for (uint32_t l = 1; l < P.n_rh; ++l) {
        ok &= issue_chain_ts(sm, w + P.r_off[l], 64, 0, false, phase, true);
        ra = hidden_to_e4m3_2(sm, xch, ra, ls[li++]);
    }
    ok &= issue_chain_ts(sm, w + P.r_out, 16, kTmemAcc16, false, phase, true);
    if (wg0) {
        float v[16];
        tmem_ld16(fused_lane_addr(sm, kTmemAcc16), v);
        const float so = ls[li];
        out4[0] = __fmul_rn(__fmul_rn(v[0], ra), so);
        out4[1] = __fmul_rn(__fmul_rn(v[1], ra), so);
        out4[2] = __fmul_rn(__fmul_rn(v[2], ra), so);
    }
    return ok;
}

}  // namespace insta
