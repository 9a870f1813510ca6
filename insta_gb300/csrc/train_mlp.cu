// train_mlp.cu -- the field's forward and backward layer products for training on tcgen05 tensor
// cores: the contraction of tiny-cuda-nn's fully fused MLP training (called from
// NerfNetwork::backward_impl, NGP/nerf_network.h:296-383), here per 128-sample tile with FP16
// operands and FP32 accumulation in TMEM, the activations kept in shared memory between the
// forward and the backward, the ReLU derivatives applied in the epilogues.
//
// Per tile (one persistent CTA of 256 threads per SM, the whole TMEM allocated):
//   forward   X -> H_1 .. H_n -> D (density MLP), [D | SH] -> C_1 .. C_m -> Y (colour MLP), every
//             hidden output rounded to FP16 and kept in shared memory;
//   backward  for each layer from the last: dX = dY W (M = 128 samples) into TMEM, masked by the
//             layer input's ReLU (X > 0) in the epilogue, and dW^T += X^T dY.  The weight
//             gradient contracts over samples, so its M is the layer's input width; to keep
//             M = 128 the tile's samples are split into 128 / K_in blocks and A = X^T is laid
//             out block-diagonally ([X_1^T 0; 0 X_2^T] for K_in = 64): row block b of the
//             accumulator sums the samples of block b, and the blocks are added when the
//             accumulators are flushed.  The dW accumulators stay in TMEM over all the tiles a
//             CTA takes and are added to the gradient once at the end.
//   dX of the first layer goes to global memory (FP32) for the hash-table backward.
#include <cstdint>

#include "device_common.cuh"
#include "mlp_tiles.cuh"
#include "kernels.h"

namespace insta {

namespace {

constexpr uint32_t kThreads = 256;

struct TrainCtl {
    uint64_t bar_mma;
    uint64_t bar_w;
    uint32_t tmem_base;
};

__device__ __forceinline__ uint32_t lane_addr(uint32_t tmem_base, uint32_t col) {
    return tmem_base + ((((uint32_t)threadIdx.x / 32u) % 4u) * 32u << 16) + col;
}

// One chain of MMAs into TMEM column `col` (N columns), A and B K-major no-swizzle tiles in shared
// memory with their own K (so their own 8-row-group stride).  `acc` = accumulate into what is
// there already for the first instruction.
struct Mma {
    const uint8_t* a;
    uint32_t a_k;   // K of the A tile (elements)
    const uint8_t* b;
    uint32_t b_k;   // K of the B tile
    uint32_t k0;    // first K element of this product in both tiles
    uint32_t k;     // K elements of this product (multiple of 16)
    uint32_t n;     // N
    uint32_t col;   // TMEM column of the accumulator
    bool acc;
};

__device__ __forceinline__ void issue(uint32_t tmem_base, const Mma& m) {
    const uint32_t idesc = idesc_f16(128, m.n, false);
    const uint32_t a0 = smem_addr(m.a), b0 = smem_addr(m.b);
    const uint32_t sbo_a = (m.a_k / 8) * 128, sbo_b = (m.b_k / 8) * 128;
    for (uint32_t ks = 0; ks < m.k / 16; ++ks) {
        const uint32_t kb = (m.k0 / 16 + ks) * 256;   // two core matrices (16 elements) per step
        umma_f16(tmem_base + m.col, smem_desc(a0 + kb, 128, sbo_a), smem_desc(b0 + kb, 128, sbo_b), idesc, (m.acc || ks) ? 1u : 0u);
    }
}

// Run up to two chains, then wait for them: the generic-proxy writes of the operands are fenced
// for the tensor core, one thread issues, warp 0 waits on the commit, the CTA syncs.
__device__ __forceinline__ bool run(TrainCtl& ctl, const Mma* ms, int n, uint32_t& phase) {
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
        tc_fence_after();
        for (int i = 0; i < n; ++i) issue(ctl.tmem_base, ms[i]);
        umma_commit(&ctl.bar_mma);
    }
    bool ok = true;
    if (threadIdx.x < 32u) ok = mbar_wait(&ctl.bar_mma, phase);
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    phase ^= 1u;
    tc_fence_after();
    return ok;
}

__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ float2 unpack_h2(uint32_t u) { return __half22float2(*reinterpret_cast<const __half2*>(&u)); }

// Row r, columns [c, c + 16) of a K-wide FP16 tile <- 16 FP32 values.
__device__ __forceinline__ void store16(uint8_t* tile, uint32_t K, uint32_t r, uint32_t c, const float* v) {
#pragma unroll
    for (int q = 0; q < 2; ++q)
        *reinterpret_cast<uint4*>(tile + tile_offset(r, c + 8 * q, K)) =
            make_uint4(pack_h2(v[8 * q], v[8 * q + 1]), pack_h2(v[8 * q + 2], v[8 * q + 3]), pack_h2(v[8 * q + 4], v[8 * q + 5]),
                       pack_h2(v[8 * q + 6], v[8 * q + 7]));
}

// Row r, columns [c, c + 16) of a K-wide FP16 tile -> 16 FP32 values.
__device__ __forceinline__ void load16(const uint8_t* tile, uint32_t K, uint32_t r, uint32_t c, float* v) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const uint4 u = *reinterpret_cast<const uint4*>(tile + tile_offset(r, c + 8 * q, K));
        const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float2 f = unpack_h2(w[i]);
            v[8 * q + 2 * i] = f.x;
            v[8 * q + 2 * i + 1] = f.y;
        }
    }
}

// Core-matrix transposes (a core matrix: 8 rows of 16 bytes, 8 x 8 FP16): a warp moves four at a
// time with one ldmatrix.trans / stmatrix pair, lane l addressing row l % 8 of matrix l / 8 in
// both; the registers carry the transposed fragments, so the stored matrix is the loaded one
// transposed.  Conflict-free: each group of 8 lanes reads or writes 128 contiguous bytes.
__device__ __forceinline__ void cm_transpose4(uint32_t src_row, uint32_t dst_row) {
    uint32_t r0, r1, r2, r3;
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(src_row) : "memory");
    asm volatile("stmatrix.sync.aligned.m8n8.x4.shared.b16 [%0], {%1,%2,%3,%4};" ::"r"(dst_row), "r"(r0), "r"(r1), "r"(r2), "r"(r3)
                 : "memory");
}

// Job j (of n_jobs, a multiple of 4) moves core matrix map(j).src to map(j).dst transposed (byte
// offsets from the tiles' shared-memory addresses); each warp takes four jobs per step.
template <typename Map>
__device__ __forceinline__ void cm_transpose(uint32_t src_base, uint32_t dst_base, uint32_t n_jobs, Map map) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (uint32_t g = warp * 4u; g < n_jobs; g += 4u * (kThreads / 32u)) {
        uint32_t so, d_o;
        map(g + (lane >> 3), so, d_o);
        cm_transpose4(src_base + so + (lane & 7u) * 16u, dst_base + d_o + (lane & 7u) * 16u);
    }
}

// dst[n rows][K = 128 samples] <- src[128 samples][K = n] transposed (n a multiple of 8).
__device__ __forceinline__ void transpose_rows(uint8_t* dst, const uint8_t* src, uint32_t n) {
    const uint32_t gk = n / 8u;
    cm_transpose(smem_addr(src), smem_addr(dst), 16u * gk, [gk](uint32_t j, uint32_t& so, uint32_t& d_o) {
        const uint32_t i = j & 15u, c = j >> 4;   // sample group, output group
        so = (i * gk + c) * 128u;
        d_o = (c * 16u + i) * 128u;
    });
}

// Block-diagonal X^T: dst[128 rows][K = 128 samples], row b * kp + f = feature f of the samples of
// block b ([b kp, b kp + kp)), from src[128 samples][K = src_k] columns [0, width) placed at
// features [f0, f0 + width).  Only the diagonal blocks are written: the rest of dst stays zero
// (cleared once per launch; each kp has its own dst), and features a narrower layer does not
// write hold another layer's values, which only reach accumulator rows that are never read.
__device__ __forceinline__ void transpose_blocks(uint8_t* dst, const uint8_t* src, uint32_t width, uint32_t src_k, uint32_t kp,
                                                 uint32_t f0 = 0) {
    const uint32_t gw = width / 8u, gs = src_k / 8u, gb = kp / 8u, g0 = f0 / 8u;
    cm_transpose(smem_addr(src), smem_addr(dst), 16u * gw, [=](uint32_t j, uint32_t& so, uint32_t& d_o) {
        const uint32_t i = j & 15u, c = j >> 4;   // sample group, feature group
        const uint32_t b = (8u * i) / kp;
        so = (i * gs + c) * 128u;
        d_o = ((b * gb + g0 + c) * 16u + i) * 128u;
    });
}

// Epilogue of a 64-wide accumulator at column `col`: warpgroup g takes columns [32 g, 32 g + 32)
// of its row; optionally ReLU (forward) or the mask of a kept ReLU output (backward), FP16 into
// the K = 64 tile `dst`.
__device__ __forceinline__ void epi64(uint32_t tmem_base, uint32_t col, uint8_t* dst, bool relu, const uint8_t* mask) {
    const uint32_t r = threadIdx.x & 127u, c0 = (threadIdx.x >> 7) * 32u;
#pragma unroll 1
    for (uint32_t c = c0; c < c0 + 32u; c += 16) {
        float v[16];
        tmem_ld16(lane_addr(tmem_base, col + c), v);
        if (relu) {   // ReLU inside the packed conversion (cvt.rn.relu)
            uint32_t p[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) p[i] = pack2_relu(v[2 * i], v[2 * i + 1], false);
#pragma unroll
            for (int q = 0; q < 2; ++q)
                *reinterpret_cast<uint4*>(dst + tile_offset(r, c + 8 * q, 64)) = make_uint4(p[4 * q], p[4 * q + 1], p[4 * q + 2], p[4 * q + 3]);
            continue;
        }
        if (mask) {
            float m[16];
            load16(mask, 64, r, c, m);
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = m[i] > 0.f ? v[i] : 0.f;
        }
        store16(dst, 64, r, c, v);
    }
}

}  // namespace

__global__ void __launch_bounds__(kThreads, 1) train_mlp_kernel(const __grid_constant__ TrainMlpArgs A) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const TrainMlpPlan& P = A.plan;
    TrainCtl& ctl = *reinterpret_cast<TrainCtl*>(smem);
    uint8_t* img = smem + P.s_img;
    uint8_t* xt = smem + P.s_x;      // [128][kd] layer input of the density MLP
    uint8_t* sh = smem + P.s_sh;     // [128][16] SH of the direction
    uint8_t* dens = smem + P.s_dens; // [128][16] density output (colour input part 1)
    uint8_t* dy = smem + P.s_dy;     // [128][<= 64] gradient w.r.t. the current layer's output
    uint8_t* bt = smem + P.s_bt;     // [<= 64][128] the same transposed (B of the weight gradient)
    uint8_t* at32 = smem + P.s_at32; // [128][128] block-diagonal X^T (A of the weight gradient), blocks of 32
    uint8_t* at64 = smem + P.s_at64; // the same with blocks of 64
    const uint32_t r = threadIdx.x & 127u, wg = threadIdx.x >> 7;
    const uint32_t n_tiles = (A.n + 127u) / 128u;
    const bool backward = A.dl_dout != nullptr;
    if (threadIdx.x == 0) {
        mbar_init(&ctl.bar_mma, 1);
        mbar_init(&ctl.bar_w, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < 2u * 128u * 128u * 2u / 16u; i += kThreads)   // both X^T tiles (adjacent)
        reinterpret_cast<uint4*>(at32)[i] = make_uint4(0u, 0u, 0u, 0u);
    if (threadIdx.x < 32) tmem_alloc(&ctl.tmem_base, 512);
    if (threadIdx.x == 0) bulk_load(img, A.images, P.img_bytes, &ctl.bar_w);
    bool ok = mbar_wait(&ctl.bar_w, 0);
    tc_fence_before();
    ok = __syncthreads_and(ok ? 1 : 0) != 0;   // uniform: the tile loop holds CTA barriers
    tc_fence_after();
    const uint32_t tmem = ctl.tmem_base;
    uint32_t phase = 0;
    bool first = true;   // the weight-gradient accumulators start from zero at the CTA's first tile
    const int nd = (int)P.n_density, nl = (int)(P.n_density + P.n_rgb);
    for (uint32_t t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
        const uint32_t s = t * 128u + r;
        const bool valid = s < A.n;
        // ---- inputs: the encoding (FP32 -> FP16) split by columns, SH by warpgroup 0
        {
            const uint32_t half = P.kd / 2u;
            for (uint32_t c = wg * half; c < wg * half + half; c += 8) {
                float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                if (valid) {
                    const float4* src = reinterpret_cast<const float4*>(A.xd + (size_t)s * P.kd + c);
                    const float4 p0 = __ldg(src), p1 = __ldg(src + 1);
                    v[0] = p0.x; v[1] = p0.y; v[2] = p0.z; v[3] = p0.w; v[4] = p1.x; v[5] = p1.y; v[6] = p1.z; v[7] = p1.w;
                }
                *reinterpret_cast<uint4*>(xt + tile_offset(r, c, P.kd)) =
                    make_uint4(pack_h2(v[0], v[1]), pack_h2(v[2], v[3]), pack_h2(v[4], v[5]), pack_h2(v[6], v[7]));
            }
            if (wg == 0) {
                float v[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = valid ? __ldg(A.xr + (size_t)s * 32 + 16 + i) : 0.f;
                store16(sh, 16, r, 0, v);
            }
        }
        // ---- forward, the hidden outputs kept
        Mma m{};
        for (int l = 0; l < nd - 1; ++l) {
            const TrainMlpLayer& L = P.layer[l];
            m = Mma{l == 0 ? xt : smem + P.s_kept[l - 1], l == 0 ? P.kd : 64u, img + L.fwd_img, L.k_pad, 0, L.k_pad, 64, 0, false};
            ok &= run(ctl, &m, 1, phase);
            epi64(tmem, 0, smem + P.s_kept[l], true, nullptr);
        }
        {
            const TrainMlpLayer& L = P.layer[nd - 1];
            m = Mma{nd > 1 ? smem + P.s_kept[nd - 2] : xt, nd > 1 ? 64u : P.kd, img + L.fwd_img, L.k_pad, 0, L.k_pad, 16, 64, false};
            ok &= run(ctl, &m, 1, phase);
            if (wg == 0) {
                float v[16];
                tmem_ld16(lane_addr(tmem, 64), v);
                store16(dens, 16, r, 0, v);
                if (A.out4 && valid) A.out4[(size_t)s * 4 + 3] = __half2float(__float2half_rn(v[0]));
            }
        }
        {
            const TrainMlpLayer& L = P.layer[nd];
            const Mma ms[2] = {Mma{dens, 16, img + L.fwd_img, 16, 0, 16, 64, 0, false},
                               Mma{sh, 16, img + L.fwd_img2, 16, 0, 16, 64, 0, true}};
            ok &= run(ctl, ms, 2, phase);
            epi64(tmem, 0, smem + P.s_kept[nd - 1], true, nullptr);
        }
        for (int l = nd + 1; l < nl - 1; ++l) {
            const TrainMlpLayer& L = P.layer[l];
            m = Mma{smem + P.s_kept[l - 2], 64, img + L.fwd_img, 64, 0, 64, 64, 0, false};
            ok &= run(ctl, &m, 1, phase);
            epi64(tmem, 0, smem + P.s_kept[l - 1], true, nullptr);
        }
        {
            const TrainMlpLayer& L = P.layer[nl - 1];
            m = Mma{smem + P.s_kept[nl - 3], 64, img + L.fwd_img, 64, 0, 64, 16, 64, false};
            ok &= run(ctl, &m, 1, phase);
            if (wg == 0 && A.out4) {   // warp-uniform: tcgen05.ld is a whole-warp instruction
                float v[16];
                tmem_ld16(lane_addr(tmem, 64), v);
                if (valid) {
                    float* o = A.out4 + (size_t)s * 4;
                    o[0] = __half2float(__float2half_rn(v[0]));
                    o[1] = __half2float(__float2half_rn(v[1]));
                    o[2] = __half2float(__float2half_rn(v[2]));
                }
            }
        }
        if (!backward) continue;
        // ---- backward.  dY of the colour output: dL/d raw rgb (columns 3..15 zero)
        if (wg == 0) {
            float v[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = (valid && i < 3) ? __ldg(A.dl_dout + (size_t)s * 4 + i) : 0.f;
            store16(dy, 16, r, 0, v);
        }
        // layers from the last: input tile X (kept), its width, dY width = the layer's n_out
        for (int l = nl - 1; l >= 0; --l) {
            const TrainMlpLayer& L = P.layer[l];
            const uint8_t* x;
            uint32_t xk, xw;
            if (l == 0) { x = xt; xk = P.kd; xw = P.kd; }
            else if (l < nd) { x = smem + P.s_kept[l - 1]; xk = 64; xw = 64; }
            else if (l == nd) { x = nullptr; xk = 32; xw = 32; }   // [density output | SH]
            else { x = smem + P.s_kept[l - 2]; xk = 64; xw = 64; }
            __syncthreads();   // dy complete (the previous epilogue or the output gradient)
            transpose_rows(bt, dy, L.n_out);
            uint8_t* at = L.kp_blk == 32u ? at32 : at64;
            if (x) {
                transpose_blocks(at, x, xw, xk, L.kp_blk);
            } else {
                // colour layer 0 (blocks of 32): features 0..15 the density output, 16..31 SH
                transpose_blocks(at, dens, 16, 16, 32);
                transpose_blocks(at, sh, 16, 16, 32, 16);
            }
            // dX = dY W (into columns 0..), dW^T += X^T dY (its own columns)
            const Mma ms[2] = {Mma{dy, L.n_out, img + L.bwd_img, L.n_out, 0, L.n_out, L.bwd_n, 0, false},
                               Mma{at, 128, bt, 128, 0, 128, L.n_out, L.dw_col, !first}};
            ok &= run(ctl, ms, 2, phase);
            if (l == 0) {
                // dL/d encoding, FP32, for the hash-table backward (warpgroup g: half the columns)
                const uint32_t half = P.kd / 2u;
                for (uint32_t c = wg * half; c < wg * half + half; c += 8) {
                    float v[16];
                    tmem_ld16(lane_addr(tmem, c & ~15u), v);   // 16 columns; use the 8 of this chunk
                    if (valid) {
                        float4* d = reinterpret_cast<float4*>(A.dxd + (size_t)s * P.kd + c);
                        const uint32_t o = c & 15u;
                        d[0] = make_float4(v[o], v[o + 1], v[o + 2], v[o + 3]);
                        d[1] = make_float4(v[o + 4], v[o + 5], v[o + 6], v[o + 7]);
                    }
                }
            } else if (l == nd) {
                // dL/d density output = the colour input's first 16 gradients + the raw density's own
                if (wg == 0) {
                    float v[16];
                    tmem_ld16(lane_addr(tmem, 0), v);
                    if (valid) v[0] += __ldg(A.dl_dout + (size_t)s * 4 + 3);
                    store16(dy, 16, r, 0, v);
                }
            } else {
                // the input is a kept ReLU output: mask
                const uint8_t* mk = l < nd ? smem + P.s_kept[l - 1] : smem + P.s_kept[l - 2];
                epi64(tmem, 0, dy, false, mk);
            }
        }
        first = false;
    }
    if (!ok && threadIdx.x == 0) atomicOr(A.err, INSTA_DEVERR_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // ---- flush the weight gradients: accumulator row b * kp + f = feature f of sample block b
    if (backward && ok && !first) {
        for (int l = 0; l < nl; ++l) {
            const TrainMlpLayer& L = P.layer[l];
            const uint32_t f = r % L.kp_blk;
            const uint32_t cols = L.n_out, c0 = cols == 64u ? wg * 32u : 0u, c1 = cols == 64u ? c0 + 32u : (wg == 0 ? 16u : 0u);
            for (uint32_t c = c0; c < c1; c += 16) {
                float v[16];
                tmem_ld16(lane_addr(tmem, L.dw_col + c), v);
                if (f < L.n_in) {
                    float* g = A.grad + L.w_off;
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        if (c + i < L.n_out_real) atomicAdd(g + (size_t)(c + i) * L.n_in + f, v[i]);
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32) tmem_dealloc(ctl.tmem_base, 512);
}

// Weight images of the plan from the FP32 master weights: tile i of the list holds
// W[row0 + n][col0 + k] (or, transposed, W[row0 + k][col0 + n]) at (n, k) of an N x K FP16 tile,
// zero outside the layer.
__global__ void __launch_bounds__(256) train_images_kernel(TrainImageList L, const float* __restrict__ w32, uint8_t* __restrict__ img) {
    const TrainImageTile& T = L.tile[blockIdx.y];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < T.n * T.k; i += gridDim.x * blockDim.x) {
        const uint32_t n = i / T.k, k = i % T.k;
        const uint32_t row = T.transpose ? T.row0 + k : T.row0 + n, col = T.transpose ? T.col0 + n : T.col0 + k;
        const float v = (row < T.rows && col < T.cols) ? w32[T.w_off + (size_t)row * T.cols + col] : 0.f;
        *reinterpret_cast<__half*>(img + T.dst + tile_offset(n, k, T.k)) = __float2half_rn(v);
    }
}

cudaError_t launch_train_mlp(const TrainMlpArgs& a, const TrainImageList& images, const float* w32, uint8_t* img_dev, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    train_images_kernel<<<dim3(16, images.n_tiles), 256, 0, s>>>(images, w32, img_dev);
    cudaError_t e = cudaFuncSetAttribute(train_mlp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)a.plan.smem_bytes);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t tiles = (a.n + 127u) / 128u;
    train_mlp_kernel<<<tiles < (uint32_t)sms ? tiles : (uint32_t)sms, kThreads, a.plan.smem_bytes, s>>>(a);
    return cudaGetLastError();
}

}  // namespace insta
