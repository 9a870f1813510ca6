// train_mlp.cu -- the field's forward and backward layer products for training on tcgen05 tensor
// cores: the contraction of tiny-cuda-nn's fully fused MLP training (called from
// NerfNetwork::backward_impl, NGP/nerf_network.h:296-383), here per 128-sample tile with FP16
// operands and FP32 accumulation in TMEM, the activations kept in shared memory between the
// forward and the backward, the ReLU derivatives applied in the epilogues.
//
// One persistent CTA per SM (the whole TMEM allocated) takes two tiles at a time and pipelines
// them: 512 epilogue threads alternate between the two tiles' epilogues, and one more warp issues
// each tile's next MMAs as soon as that tile's epilogue has written their operands, so the tensor
// core runs one tile's step while the epilogue threads work on the other's.  One thread issues
// every MMA, so the two tiles' additions into the shared weight-gradient accumulators happen in
// issue order.
//
// Per tile, steps 0 .. n-1 are the forward and n .. 2n-1 the backward of the n layers:
//   forward   X -> H_1 .. H_n -> D (density MLP), [D | SH] -> C_1 .. C_m -> Y (colour MLP), every
//             hidden output rounded to FP16 and kept in shared memory;
//   backward  for each layer from the last: dX = dY W (M = 128 samples) into TMEM, masked by the
//             layer input's ReLU (X > 0) in the epilogue, and dW^T += X^T dY.  The weight
//             gradient contracts over the tile's samples: its A operand is the layer's input
//             tile read as an MN-major matrix (features along M, samples along K) and its B
//             operand the dY tile read the same way, so neither is transposed in shared memory.
//             With M = 128 the accumulator rows past the layer's input width hold products of
//             neighbouring data and are never read.  The dW accumulators stay in TMEM over all
//             the tiles a CTA takes and are added to the gradient once at the end.
//   dX of the first layer goes to global memory (FP32) for the hash-table backward.
#include <cstdint>

#include "device_common.cuh"
#include "mlp_tiles.cuh"
#include "kernels.h"

namespace insta {

namespace {

constexpr uint32_t kEpiThreads = 512;              // four warpgroups: each epilogue splits a row's columns four ways
constexpr uint32_t kThreads = kEpiThreads + 32;    // and one warp that issues the MMAs

struct TrainCtl {
    uint64_t bar_mma[2];   // per tile slot: the MMA warp's commit of the slot's current step
    uint64_t opready[2];   // per tile slot: the epilogue threads have written the next step's operands
    uint64_t bar_w;
    uint32_t tmem_base;
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ uint32_t lane_addr(uint32_t tmem_base, uint32_t col) {
    return tmem_base + ((((uint32_t)threadIdx.x / 32u) % 4u) * 32u << 16) + col;
}

// Instruction descriptor of the weight-gradient product: FP16, both operands MN-major.
__host__ __device__ constexpr uint32_t idesc_f16_mn(uint32_t M, uint32_t N) {
    return idesc_f16(M, N, false) | (1u << 15) | (1u << 16);
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

// Epilogue of a 64-wide accumulator at column `col`: warpgroup g takes columns [16 g, 16 g + 16)
// of its row; ReLU (forward) or the mask of a kept ReLU output (backward), FP16 into the K = 64
// tile `dst`.
__device__ __forceinline__ void epi64(uint32_t tmem_base, uint32_t col, uint8_t* dst, bool relu, const uint8_t* mask) {
    const uint32_t r = threadIdx.x & 127u, c0 = (threadIdx.x >> 7) * 16u;
    {
        const uint32_t c = c0;
        float v[16];
        tmem_ld16(lane_addr(tmem_base, col + c), v);
        if (relu) {   // ReLU inside the packed conversion (cvt.rn.relu)
            uint32_t p[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) p[i] = pack2_relu(v[2 * i], v[2 * i + 1], false);
#pragma unroll
            for (int q = 0; q < 2; ++q)
                *reinterpret_cast<uint4*>(dst + tile_offset(r, c + 8 * q, 64)) = make_uint4(p[4 * q], p[4 * q + 1], p[4 * q + 2], p[4 * q + 3]);
            return;
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

// Shared-memory tiles of slot s, addressed through the plan (constant-bank offsets) so that no
// per-slot table of pointers goes to local memory.
struct Tiles {
    uint8_t* smem;
    const TrainMlpPlan& P;
    __device__ __forceinline__ uint8_t* x(uint32_t s) const { return smem + P.s_x[s]; }         // [128][kd] density input
    __device__ __forceinline__ uint8_t* rin(uint32_t s) const { return smem + P.s_rin[s]; }     // [128][32] density output | SH
    __device__ __forceinline__ uint8_t* kept(uint32_t s, int k) const { return smem + P.s_kept[s][k]; }   // [128][64]
    __device__ __forceinline__ uint8_t* dy(uint32_t s) const { return smem + P.s_dy[s]; }       // [128][<= 64] dL/d output
    // The input tile of layer l and its K (its width as a K-major operand).
    __device__ __forceinline__ const uint8_t* input(uint32_t s, int l, uint32_t& k) const {
        const int nd = (int)P.n_density;
        if (l == 0) { k = P.kd; return x(s); }
        if (l < nd) { k = 64; return kept(s, l - 1); }
        if (l == nd) { k = 32; return rin(s); }
        k = 64;
        return kept(s, l - 2);
    }
};

}  // namespace

__global__ void __launch_bounds__(kThreads, 1) train_mlp_kernel(const __grid_constant__ TrainMlpArgs A) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const TrainMlpPlan& P = A.plan;
    TrainCtl& ctl = *reinterpret_cast<TrainCtl*>(smem);
    uint8_t* img = smem + P.s_img;
    const uint32_t r = threadIdx.x & 127u, wg = threadIdx.x >> 7;
    const uint32_t n_tiles = (A.n + 127u) / 128u, n_pairs = (n_tiles + 1u) / 2u;
    const bool backward = A.dl_dout != nullptr;
    const int nd = (int)P.n_density, nl = (int)(P.n_density + P.n_rgb);
    const int n_steps = backward ? 2 * nl : nl;
    if (threadIdx.x == 0) {
        mbar_init(&ctl.bar_mma[0], 1);
        mbar_init(&ctl.bar_mma[1], 1);
        mbar_init(&ctl.opready[0], kEpiThreads);
        mbar_init(&ctl.opready[1], kEpiThreads);
        mbar_init(&ctl.bar_w, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x < 32) tmem_alloc(&ctl.tmem_base, 512);
    if (threadIdx.x == 0) bulk_load(img, A.images, P.img_bytes, &ctl.bar_w);
    bool ok = mbar_wait(&ctl.bar_w, 0);
    tc_fence_before();
    ok = __syncthreads_and(ok ? 1 : 0) != 0;   // uniform: the tile loop holds CTA barriers
    tc_fence_after();
    const uint32_t tmem = ctl.tmem_base;
    const Tiles T{smem, P};
    uint32_t phase = 0u, ready_phase = 0u;   // bit s: the parity to wait for on slot s's barrier
    uint32_t dw_started = 0;   // layers whose weight-gradient accumulator holds a value (the issuing thread's)
    const bool mma_warp = threadIdx.x >= kEpiThreads;

    // The MMAs of step k of slot s, then its commit (the MMA warp's first thread, once the slot's
    // operands are published).
    auto issue = [&](uint32_t s, int k) {
        if (threadIdx.x != kEpiThreads) return;
        const uint32_t d_col = tmem + s * 64u;
        if (k < nl) {
            const TrainMlpLayer& L = P.layer[k];
            uint32_t ka;
            const uint8_t* a = T.input(s, k, ka);
            const uint32_t idesc = idesc_f16(128, L.n_out, false);
            const uint32_t a0 = smem_addr(a), b0 = smem_addr(img + L.fwd_img);
            for (uint32_t ks = 0; ks < L.k_pad / 16u; ++ks)
                umma_f16(d_col, smem_desc(a0 + ks * 256u, 128, (ka / 8u) * 128u), smem_desc(b0 + ks * 256u, 128, (L.k_pad / 8u) * 128u),
                         idesc, ks ? 1u : 0u);
        } else {
            const int l = 2 * nl - 1 - k;
            const TrainMlpLayer& L = P.layer[l];
            // dX = dY W: A = dY (K-major, K = n_out), B = the W^T image (N = bwd_n, K = n_out)
            {
                const uint32_t idesc = idesc_f16(128, L.bwd_n, false);
                const uint32_t a0 = smem_addr(T.dy(s)), b0 = smem_addr(img + L.bwd_img), sbo = (L.n_out / 8u) * 128u;
                for (uint32_t ks = 0; ks < L.n_out / 16u; ++ks)
                    umma_f16(d_col, smem_desc(a0 + ks * 256u, 128, sbo), smem_desc(b0 + ks * 256u, 128, sbo), idesc, ks ? 1u : 0u);
            }
            // dW^T += X^T dY: A = the layer's input tile as an MN-major operand (features along M,
            // one core matrix of 8 features every 128 B; samples along K, one group of 8 rows every
            // (w / 8) * 128 B), B = dY the same way; K = 128 samples, 16 per instruction
            {
                uint32_t w;
                const uint8_t* x = T.input(s, l, w);
                const uint32_t idesc = idesc_f16_mn(128, L.n_out);
                const uint32_t a0 = smem_addr(x), b0 = smem_addr(T.dy(s));
                const uint32_t kgrp_a = (w / 8u) * 128u, kgrp_b = (L.n_out / 8u) * 128u;
                const bool acc0 = (dw_started >> l) & 1u;
                for (uint32_t ks = 0; ks < 8u; ++ks)
                    umma_f16(tmem + L.dw_col, smem_desc(a0 + ks * 2u * kgrp_a, kgrp_a, 128), smem_desc(b0 + ks * 2u * kgrp_b, kgrp_b, 128),
                             idesc, (acc0 || ks) ? 1u : 0u);
                dw_started |= 1u << l;
            }
        }
        umma_commit(&ctl.bar_mma[s]);
    };
    // Epilogue threads: each waits (bounded) for slot s's commit itself.  The commit orders the
    // MMAs' reads of the published tiles before any thread's next epilogue overwrites them, and no
    // thread can run a phase ahead: the next commit needs every epilogue thread's publish.  A wait
    // that gives up makes only that thread's flag false; the pair loop agrees on it at the next CTA
    // barrier, and the thread skips its later waits meanwhile (bounded work, results discarded).
    auto epi_wait = [&](uint32_t s) -> bool {
        const bool w = mbar_wait(&ctl.bar_mma[s], (phase >> s) & 1u);
        phase ^= 1u << s;
        __syncwarp();   // the epilogue's TMEM loads are warp-collective
        tc_fence_after();
        return w;
    };
    // Epilogue threads: publish slot s's operands for its next step to the MMA warp.
    auto publish = [&](uint32_t s) {
        fence_async_smem();
        tc_fence_before();
        mbar_arrive(&ctl.opready[s]);
    };
    // The MMA warp: wait (bounded) until slot s's operands are published.
    auto mma_wait = [&](uint32_t s) -> bool {
        const bool w = __all_sync(0xffffffffu, mbar_wait(&ctl.opready[s], (ready_phase >> s) & 1u));
        ready_phase ^= 1u << s;
        tc_fence_after();
        return w;
    };
    // The inputs of tile t into slot s: the encoding (FP32 -> FP16) in 8-column chunks dealt to
    // the four warpgroups, SH by warpgroups 0 and 1 into the colour input's columns 16..31.
    auto stage = [&](uint32_t s, uint32_t t) {
        const uint32_t row = t * 128u + r;
        const bool valid = row < A.n;
        for (uint32_t c = wg * 8u; c < P.kd; c += 32u) {
            float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (valid) {
                const float4* src = reinterpret_cast<const float4*>(A.xd + (size_t)row * P.kd + c);
                const float4 p0 = __ldg(src), p1 = __ldg(src + 1);
                v[0] = p0.x; v[1] = p0.y; v[2] = p0.z; v[3] = p0.w; v[4] = p1.x; v[5] = p1.y; v[6] = p1.z; v[7] = p1.w;
            }
            *reinterpret_cast<uint4*>(T.x(s) + tile_offset(r, c, P.kd)) =
                make_uint4(pack_h2(v[0], v[1]), pack_h2(v[2], v[3]), pack_h2(v[4], v[5]), pack_h2(v[6], v[7]));
        }
        if (wg < 2) {
            float v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = valid ? __ldg(A.xr + (size_t)row * 32 + 16 + 8 * wg + i) : 0.f;
            *reinterpret_cast<uint4*>(T.rin(s) + tile_offset(r, 16u + 8u * wg, 32)) =
                make_uint4(pack_h2(v[0], v[1]), pack_h2(v[2], v[3]), pack_h2(v[4], v[5]), pack_h2(v[6], v[7]));
        }
    };
    // The epilogue of step k of slot s (tile t).  Warp-uniform conditions only around the TMEM
    // loads (whole-warp instructions); `valid` guards stores alone.
    auto epilogue = [&](uint32_t s, uint32_t t, int k) {
        const uint32_t col = s * 64u;
        const uint32_t row = t * 128u + r;
        const bool valid = row < A.n;
        if (k < nl) {
            if (k < nd - 1) {
                epi64(tmem, col, T.kept(s, k), true, nullptr);
            } else if (k == nd - 1) {
                if (wg == 0) {   // density output: the colour input's columns 0..15, the raw density
                    float v[16];
                    tmem_ld16(lane_addr(tmem, col), v);
                    store16(T.rin(s), 32, r, 0, v);
                    if (A.out4 && valid) A.out4[(size_t)row * 4 + 3] = __half2float(__float2half_rn(v[0]));
                }
            } else if (k < nl - 1) {
                epi64(tmem, col, T.kept(s, k - 1), true, nullptr);
            } else if (wg == 0) {   // colour output; and the output gradient dL/d raw rgb (columns 3..15 zero)
                if (A.out4) {
                    float v[16];
                    tmem_ld16(lane_addr(tmem, col), v);
                    if (valid) {
                        float* o = A.out4 + (size_t)row * 4;
                        o[0] = __half2float(__float2half_rn(v[0]));
                        o[1] = __half2float(__float2half_rn(v[1]));
                        o[2] = __half2float(__float2half_rn(v[2]));
                    }
                }
                if (backward) {
                    float v[16];
#pragma unroll
                    for (int i = 0; i < 16; ++i) v[i] = (valid && i < 3) ? __ldg(A.dl_dout + (size_t)row * 4 + i) : 0.f;
                    store16(T.dy(s), 16, r, 0, v);
                }
            }
            return;
        }
        const int l = 2 * nl - 1 - k;
        if (l == 0) {
            // dL/d encoding, FP32, for the hash-table backward (8-column chunks dealt to the warpgroups)
            for (uint32_t c = wg * 8u; c < P.kd; c += 32u) {
                float v[16];
                tmem_ld16(lane_addr(tmem, col + (c & ~15u)), v);   // 16 columns; use the 8 of this chunk
                if (valid) {   // static register indices: the chunk's half of the 16 columns
                    float4* d = reinterpret_cast<float4*>(A.dxd + (size_t)row * P.kd + c);
                    const bool hi = (c & 8u) != 0u;
                    d[0] = hi ? make_float4(v[8], v[9], v[10], v[11]) : make_float4(v[0], v[1], v[2], v[3]);
                    d[1] = hi ? make_float4(v[12], v[13], v[14], v[15]) : make_float4(v[4], v[5], v[6], v[7]);
                }
            }
        } else if (l == nd) {
            // dL/d density output = the colour input's first 16 gradients + the raw density's own
            if (wg == 0) {
                float v[16];
                tmem_ld16(lane_addr(tmem, col), v);
                if (valid) v[0] += __ldg(A.dl_dout + (size_t)row * 4 + 3);
                store16(T.dy(s), 16, r, 0, v);
            }
        } else {
            // the layer's input is a kept ReLU output: mask
            uint32_t w;
            const uint8_t* mk = T.input(s, l, w);
            epi64(tmem, col, T.dy(s), false, mk);
        }
    };

    // Tile pairs (2p, 2p + 1); slot 1 idles for an odd last tile.  Per step the epilogue threads
    // take slot 0's epilogue, publish its operands, take slot 1's; the MMA warp issues each slot's
    // next step as soon as it is published.  Every pair starts at a CTA barrier (staging done, the
    // previous pair finished on both sides, the outcome so far agreed).
    for (uint32_t p = blockIdx.x; p < n_pairs; p += gridDim.x) {
        const uint32_t ta = 2u * p, tb = 2u * p + 1u;
        const bool has_b = tb < n_tiles;
        if (!mma_warp) {
            stage(0, ta);
            if (has_b) stage(1, tb);
        }
        fence_async_smem();
        tc_fence_before();
        ok = __syncthreads_and(ok ? 1 : 0) != 0;
        tc_fence_after();
        if (!ok) break;
        if (mma_warp) {
            issue(0, 0);
            if (has_b) issue(1, 0);
            for (int k = 0; k + 1 < n_steps && ok; ++k) {
                ok = mma_wait(0);
                if (!ok) break;
                issue(0, k + 1);
                if (has_b) {
                    ok = mma_wait(1);
                    if (!ok) break;
                    issue(1, k + 1);
                }
            }
        } else {
            for (int k = 0; k < n_steps; ++k) {
                ok = ok && epi_wait(0);
                epilogue(0, ta, k);
                if (k + 1 < n_steps) publish(0);
                if (has_b) {
                    ok = ok && epi_wait(1);
                    epilogue(1, tb, k);
                    if (k + 1 < n_steps) publish(1);
                }
            }
        }
    }
    tc_fence_before();
    ok = __syncthreads_and(ok ? 1 : 0) != 0;   // the flush below runs on all epilogue threads or none
    tc_fence_after();
    if (!ok && threadIdx.x == 0) atomicOr(A.err, INSTA_DEVERR_TIMEOUT);
    // ---- flush the weight gradients: accumulator row f = input feature f, column o = output o.
    // dw_started is thread 0's; the flush runs when the backward ran on at least one tile.
    if (backward && ok && !mma_warp && n_tiles > blockIdx.x * 2u) {
        for (int l = 0; l < nl; ++l) {
            const TrainMlpLayer& L = P.layer[l];
            const uint32_t cols = L.n_out, c0 = cols == 64u ? wg * 16u : 0u, c1 = cols == 64u ? c0 + 16u : (wg == 0 ? 16u : 0u);
            for (uint32_t c = c0; c < c1; c += 16) {
                float v[16];
                tmem_ld16(lane_addr(tmem, L.dw_col + c), v);
                if (r < L.n_in) {
                    float* g = A.grad + L.w_off;
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        if (c + i < L.n_out_real) atomicAdd(g + (size_t)(c + i) * L.n_in + r, v[i]);
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
    const uint32_t pairs = ((a.n + 127u) / 128u + 1u) / 2u;
    train_mlp_kernel<<<pairs < (uint32_t)sms ? pairs : (uint32_t)sms, kThreads, a.plan.smem_bytes, s>>>(a);
    return cudaGetLastError();
}

}  // namespace insta
