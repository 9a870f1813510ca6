// umma.cuh -- 5th-generation tensor-core (tcgen05) building blocks for the avatar MLPs.
//
// One CTA of 128 threads evaluates a 128-sample tile: thread t owns sample t, writes
// its activation row t into a shared-memory A tile, one elected thread issues
// tcgen05.mma (M = 128, accumulator in TMEM), and after the commit-mbarrier fires each
// warp reads its 32 TMEM lanes back with tcgen05.ld -- lane t of the accumulator is row
// t, i.e. the same thread's sample, so activations never cross threads.
//
// Operand tiles use the no-swizzle K-major canonical layout: 8-row x 16-byte core
// matrices; core matrices adjacent along K are LBO = 128 B apart and 8-row groups are
// SBO = (K / 8) * 128 B apart.  Element (r, k) of an R x K FP16 tile lives at byte
//   ((r / 8) * (K / 8) + k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2.
// Weights (B operands, [N][K] row-major = K-major) are pre-arranged in exactly this
// layout on the host and bulk-copied into shared memory once per CTA.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include "insta_types.h"

namespace insta {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__host__ __device__ constexpr uint32_t tile_offset(uint32_t r, uint32_t k, uint32_t K) {
    return ((r / 8) * (K / 8) + k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2;
}

// The same layout for 8-bit elements: a core matrix is 8 rows x 16 one-byte elements, so with K
// counted in bytes the byte geometry (and the descriptor strides) equal the 16-bit case.
__host__ __device__ constexpr uint32_t tile_offset8(uint32_t r, uint32_t k, uint32_t K) {
    return ((r / 8) * (K / 16) + k / 16) * 128 + (r % 8) * 16 + (k % 16);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;          // descriptor version for tcgen05
    return d;                        // base offset 0, relative LBO, no swizzle
}

// Instruction descriptor, kind::f16: FP32 accumulate, A/B FP16 (or BF16), both K-major.
__host__ __device__ constexpr uint32_t idesc_f16(uint32_t M, uint32_t N, bool bf16) {
    return (1u << 4) | ((bf16 ? 1u : 0u) << 7) | ((bf16 ? 1u : 0u) << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait for the mbarrier phase with the given parity: gives up after ~1 s.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    uint32_t a = smem_addr(bar);
    uint64_t t0 = 0;
    for (uint32_t it = 0;; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done) : "r"(a), "r"(parity) : "memory");
        if (done) return true;
        if ((it & 255u) == 0u) {
            uint64_t now = global_ns();
            if (t0 == 0) t0 = now;
            else if (now - t0 > 1000000000ull) return false;
        }
    }
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}
// kind::f8f6f4 with E4M3 A and B (instruction descriptor a/b formats 0, as idesc_f16(M, N, false));
// K = 32 per instruction.
__device__ __forceinline__ void umma_f8(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 32 consecutive FP32 accumulator columns of this thread's TMEM lane (one load, one wait).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// 8 packed 32-bit values into 8 consecutive TMEM columns of this thread's lane; tmem_st_wait
// makes the thread's stores complete (before a thread sync hands the columns to an MMA).
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t* v) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};\n"
                 ::"r"(taddr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]) : "memory");
}
__device__ __forceinline__ void tmem_st4(uint32_t taddr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};\n" ::"r"(taddr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}
__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// kind::f16 with the A operand in TMEM: row m of A in lane m, two 16-bit elements per 32-bit
// column (the even element in the low half), K = 16 per instruction = 8 columns from tmem_a.
__device__ __forceinline__ void umma_f16_ts(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n"
        ::"r"(tmem_d), "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}

// kind::f8f6f4 (E4M3) with the A operand in TMEM: four 8-bit elements per 32-bit column (element
// k in byte k % 4), K = 32 per instruction = 8 columns from tmem_a.
__device__ __forceinline__ void umma_f8_ts(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [%1], %2, %3, p;\n}\n"
        ::"r"(tmem_d), "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}

// Bulk (TMA 1D) copy global -> shared, completion tracked by an mbarrier transaction count.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

// Store one FP16 row (K values, K multiple of 8) into an A tile.
__device__ __forceinline__ void store_row(uint8_t* tile, uint32_t r, uint32_t K, const __half* v) {
    for (uint32_t c = 0; c < K / 8; ++c) {
        uint4 q;
        q.x = *reinterpret_cast<const uint32_t*>(&v[c * 8 + 0]);
        q.y = *reinterpret_cast<const uint32_t*>(&v[c * 8 + 2]);
        q.z = *reinterpret_cast<const uint32_t*>(&v[c * 8 + 4]);
        q.w = *reinterpret_cast<const uint32_t*>(&v[c * 8 + 6]);
        *reinterpret_cast<uint4*>(tile + tile_offset(r, c * 8, K)) = q;
    }
}


__device__ __forceinline__ __half to_act(float v, bool bf16) {
    if (bf16) {
        __nv_bfloat16 b = __float2bfloat16_rn(v);
        return __ushort_as_half(__bfloat16_as_ushort(b));
    }
    return __float2half_rn(v);
}
// Two FP32 values rounded to the activation type (round to nearest even, as to_act) and packed,
// a in the low half: one packed conversion instruction.
__device__ __forceinline__ uint32_t pack2_act(float a, float b, bool bf16) {
    if (bf16) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<const uint32_t*>(&h);
    }
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}
// ReLU and the rounding of pack2_act in one packed conversion (cvt.rn.relu: negative results
// become zero), a in the low half.  Same bits as pack2_act(fmaxf(a, 0), fmaxf(b, 0)) for every
// non-NaN input.
__device__ __forceinline__ uint32_t pack2_relu(float a, float b, bool bf16) {
    uint32_t r;
    if (bf16) asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
    else asm("cvt.rn.relu.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
    return r;
}
__device__ __forceinline__ float from_act(__half h, bool bf16) {
    if (bf16) return __bfloat162float(__ushort_as_bfloat16(__half_as_ushort(h)));
    return __half2float(h);
}


}  // namespace insta
