// train_kernels.cu -- the field's backward pass and the optimizer step, the tiny-cuda-nn side of
// train_nerf_step that NerfNetwork delegates to (NGP/nerf_network.h:296-383): gradients of every
// parameter (density MLP, colour MLP, hash table) for given output gradients, then Adam.
//
// Layout: per-sample activations are column-major matrices of the batch (one column per sample,
// `rows` floats each), so each MLP layer is one plain GEMM over the batch (cuBLAS, FP32):
//   forward    Y = W X            (W: [n_out][n_in] row-major, the snapshot's layer layout)
//   backward   dX = W^T dY, then the ReLU mask of the layer's input
//   weights    dW += dY X^T
// The hash encode and its backward (scatter-add of each corner's weighted gradient into the
// table, FP32 atomics) and the elementwise steps are kernels here.  The encode gathers the FP16
// copy of the training weights' table (as tiny-cuda-nn's mixed-precision training forward does);
// the layer products take the FP32 master weights (FP32 / TF32 products) or their FP16 images
// (the tcgen05 kernel); features and activations stay FP32 (no FP16 rounding between layers).
#include <cublas_v2.h>

#include "../../include/insta_gb300.h"
#include "device_common.cuh"
#include "kernels.h"

namespace insta {

// Table index of corner (cx, cy, cz) of level l: dense x + y res + z res^2 (wrapping on the far
// boundary), else the spatial hash.
__device__ __forceinline__ uint32_t corner_index(const FieldView& fv, uint32_t l, uint32_t cx, uint32_t cy, uint32_t cz) {
    const uint32_t res = fv.level_res[l], size = fv.level_size[l];
    if (fv.level_dense[l]) {
        uint32_t idx = cx + cy * res + cz * res * res;
        if (idx >= size) idx %= size;
        return idx;
    }
    return ((cx * 1u) ^ (cy * 2654435761u) ^ (cz * 805459861u)) & (size - 1u);
}

// Encode: X_d[:, 0:E] = hash encoding (E = levels x features), X_d[:, E:E+n_extra] = the record's
// expression dims, X_r[:, 16:32] = SH of the direction (X_r[:, 0:16] is filled by the density
// MLP's output).  The table entries come from fv.table: the FP16 copy of the training weights, as
// tiny-cuda-nn's mixed-precision training forward reads its half-precision grid (the FP32 master
// weights stay with the optimizer); the same gathers, weights and summation order as the render's
// encode (hash_level / hash_level_wide), the features kept in FP32.
template <int F>
__global__ void __launch_bounds__(256) train_encode_kernel(FieldView fv, const float* __restrict__ coords, uint32_t stride, uint32_t n,
                                                           float* __restrict__ xd, uint32_t kd, float* __restrict__ xr) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* c = coords + (size_t)i * stride;
    const V3 p = v3(c[0], c[1], c[2]);
    const __half2* t2 = reinterpret_cast<const __half2*>(fv.table);
    float* x = xd + (size_t)i * kd;
    for (uint32_t l = 0; l < fv.n_levels; ++l) {
        if constexpr (F == 2) {
            float a0, a1;
            hash_level(fv, t2, p, l, a0, a1);
            x[2 * l] = a0;
            x[2 * l + 1] = a1;
        } else {
            float a[F];
            hash_level_wide<F>(fv, t2, p, l, a);
#pragma unroll
            for (int f = 0; f < F; ++f) x[F * l + f] = a[f];
        }
    }
    for (uint32_t m = 0; m < fv.n_extra; ++m) x[F * fv.n_levels + m] = c[stride - fv.n_extra + m];
    float sh[16];
    sh4(c[8], c[9], c[10], sh);
    float* r = xr + (size_t)i * 32 + 16;
#pragma unroll
    for (int k = 0; k < 16; ++k) r[k] = sh[k];
}

static void launch_train_encode(const FieldView& fv, const float* coords, uint32_t stride, uint32_t n, float* xd, uint32_t kd, float* xr,
                                cudaStream_t s) {
    const unsigned blocks = (n + 255) / 256;
    if (fv.n_features == 8) train_encode_kernel<8><<<blocks, 256, 0, s>>>(fv, coords, stride, n, xd, kd, xr);
    else if (fv.n_features == 4) train_encode_kernel<4><<<blocks, 256, 0, s>>>(fv, coords, stride, n, xd, kd, xr);
    else train_encode_kernel<2><<<blocks, 256, 0, s>>>(fv, coords, stride, n, xd, kd, xr);
}

__global__ void __launch_bounds__(256) relu_kernel(float* __restrict__ h, size_t count) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) h[i] = fmaxf(h[i], 0.f);
}

// dX *= (H > 0): the ReLU derivative taken from the layer's (post-activation) input
__global__ void __launch_bounds__(256) relu_back_kernel(float* __restrict__ d, const float* __restrict__ h, size_t count) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        if (!(h[i] > 0.f)) d[i] = 0.f;
}

// The colour MLP's output gradient (rows 0..2 = dL/d raw rgb, padded rows 0) and the outputs.
__global__ void __launch_bounds__(256) train_out_kernel(uint32_t n, const float* __restrict__ yr, const float* __restrict__ xr,
                                                        const float* __restrict__ g, float* __restrict__ dyr, float* __restrict__ out4) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (out4) *reinterpret_cast<float4*>(out4 + (size_t)i * 4) = make_float4(yr[(size_t)i * 16], yr[(size_t)i * 16 + 1], yr[(size_t)i * 16 + 2], xr[(size_t)i * 32]);
    if (!g) return;
    float* d = dyr + (size_t)i * 16;
#pragma unroll
    for (int k = 0; k < 16; ++k) d[k] = k < 3 ? g[(size_t)i * 4 + k] : 0.f;
}

// dL/d(density output 0) += dL/d(raw density): the density MLP's first output is also the raw
// density the composite reads.
__global__ void __launch_bounds__(256) train_density_grad_kernel(uint32_t n, const float* __restrict__ g, float* __restrict__ dxr) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dxr[(size_t)i * 32] += g[(size_t)i * 4 + 3];
}

// Hash encode backward for F = 4 or 8 features per level: the corner weights of
// hash_backward_kernel times the F gradients, runs of equal entries within a warp summed first
// (the same segmented scan), one or two 16-byte reductions per entry and run.
template <int F>
__global__ void __launch_bounds__(256) hash_backward_wide_kernel(FieldView fv, const float* __restrict__ coords, uint32_t stride, uint32_t n,
                                                                 const float* __restrict__ dxd, uint32_t kd, float* __restrict__ gtable) {
    constexpr uint32_t FULL = 0xffffffffu;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x, lane = threadIdx.x & 31u;
    if ((i & ~31u) >= n) return;   // whole warps past the end leave; the rest stay for the shuffles
    const bool valid = i < n;
    const float* c = coords + (size_t)(valid ? i : 0) * stride;
    const V3 x = v3(c[0], c[1], c[2]);
    const float* dg = dxd + (size_t)(valid ? i : 0) * kd;
    for (uint32_t l = 0; l < fv.n_levels; ++l) {
        float g[F];
#pragma unroll
        for (int f = 0; f < F; ++f) g[f] = valid ? dg[F * l + f] : 0.f;
        const float s = fv.level_scale[l];
        const float px = fmaf(x.x, s, 0.5f), py = fmaf(x.y, s, 0.5f), pz = fmaf(x.z, s, 0.5f);
        const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
        const float rx = __fsub_rn(px, fx), ry = __fsub_rn(py, fy), rz = __fsub_rn(pz, fz);
        const uint32_t gx = (uint32_t)(int32_t)fx, gy = (uint32_t)(int32_t)fy, gz = (uint32_t)(int32_t)fz;
        float4* lt = reinterpret_cast<float4*>(gtable + (size_t)fv.level_off[l] * F);
#pragma unroll 1
        for (uint32_t cc = 0; cc < 8; ++cc) {
            const uint32_t bx = cc & 1u, by = (cc >> 1) & 1u, bz = (cc >> 2) & 1u;
            float w = bx ? rx : __fsub_rn(1.f, rx);
            w = __fmul_rn(w, by ? ry : __fsub_rn(1.f, ry));
            w = __fmul_rn(w, bz ? rz : __fsub_rn(1.f, rz));
            uint32_t idx = corner_index(fv, l, gx + bx, gy + by, gz + bz);
            if (!valid) idx = FULL;
            float v[F];
            bool any = false;
#pragma unroll
            for (int f = 0; f < F; ++f) v[f] = w * g[f];
            const uint32_t prev = __shfl_up_sync(FULL, idx, 1), next = __shfl_down_sync(FULL, idx, 1);
            const uint32_t heads = __ballot_sync(FULL, lane == 0 || prev != idx);
            if (heads != FULL) {
                const uint32_t start = 31u - __clz(heads & (FULL >> (31u - lane)));
#pragma unroll
                for (uint32_t d = 1; d < 32; d <<= 1) {
#pragma unroll
                    for (int f = 0; f < F; ++f) {
                        const float o = __shfl_up_sync(FULL, v[f], d);
                        if (lane >= start + d) v[f] += o;
                    }
                }
            }
#pragma unroll
            for (int f = 0; f < F; ++f) any |= v[f] != 0.f;
            if (valid && (lane == 31 || next != idx) && any) {
#pragma unroll
                for (int q = 0; q < F / 4; ++q)
                    atomicAdd(lt + (size_t)idx * (F / 4) + q, make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]));
            }
        }
    }
}

// Hash encode backward: every corner's trilinear weight times the encoding gradient, added into
// the table gradient (FP32, [entries][2] like the table, one 8-byte reduction per entry).
// Samples arrive in ray order, so neighbouring lanes of a warp often hit the same corner (every
// coarse level, and fine levels along short steps): lanes with equal entries in a row are summed
// first (a segmented scan over the warp) and only the last lane of each run adds to memory.
__global__ void __launch_bounds__(256) hash_backward_kernel(FieldView fv, const float* __restrict__ coords, uint32_t stride, uint32_t n,
                                                            const float* __restrict__ dxd, uint32_t kd, float* __restrict__ gtable) {
    constexpr uint32_t FULL = 0xffffffffu;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x, lane = threadIdx.x & 31u;
    if ((i & ~31u) >= n) return;   // whole warps past the end leave; the rest stay for the shuffles
    const bool valid = i < n;
    const float* c = coords + (size_t)(valid ? i : 0) * stride;
    const V3 x = v3(c[0], c[1], c[2]);
    const float* dg = dxd + (size_t)(valid ? i : 0) * kd;
    for (uint32_t l = 0; l < fv.n_levels; ++l) {
        const float g0 = valid ? dg[2 * l] : 0.f, g1 = valid ? dg[2 * l + 1] : 0.f;
        const float s = fv.level_scale[l];
        const float px = fmaf(x.x, s, 0.5f), py = fmaf(x.y, s, 0.5f), pz = fmaf(x.z, s, 0.5f);
        const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
        const float rx = __fsub_rn(px, fx), ry = __fsub_rn(py, fy), rz = __fsub_rn(pz, fz);
        const uint32_t gx = (uint32_t)(int32_t)fx, gy = (uint32_t)(int32_t)fy, gz = (uint32_t)(int32_t)fz;
        const uint32_t res = fv.level_res[l], size = fv.level_size[l];
        float2* lt = reinterpret_cast<float2*>(gtable + (size_t)fv.level_off[l] * 2);
#pragma unroll
        for (uint32_t cc = 0; cc < 8; ++cc) {
            const uint32_t bx = cc & 1u, by = (cc >> 1) & 1u, bz = (cc >> 2) & 1u;
            float w = bx ? rx : __fsub_rn(1.f, rx);
            w = __fmul_rn(w, by ? ry : __fsub_rn(1.f, ry));
            w = __fmul_rn(w, bz ? rz : __fsub_rn(1.f, rz));
            const uint32_t cx = gx + bx, cy = gy + by, cz = gz + bz;
            uint32_t idx;
            if (fv.level_dense[l]) {
                idx = cx + cy * res + cz * res * res;
                if (idx >= size) idx %= size;
            } else {
                idx = ((cx * 1u) ^ (cy * 2654435761u) ^ (cz * 805459861u)) & (size - 1u);
            }
            if (!valid) idx = FULL;
            float vx = w * g0, vy = w * g1;
            const uint32_t prev = __shfl_up_sync(FULL, idx, 1), next = __shfl_down_sync(FULL, idx, 1);
            const uint32_t heads = __ballot_sync(FULL, lane == 0 || prev != idx);
            if (heads != FULL) {
                // segmented inclusive scan: the run of this lane starts at the highest head at or below it
                const uint32_t start = 31u - __clz(heads & (FULL >> (31u - lane)));
#pragma unroll
                for (uint32_t d = 1; d < 32; d <<= 1) {
                    const float ox = __shfl_up_sync(FULL, vx, d), oy = __shfl_up_sync(FULL, vy, d);
                    if (lane >= start + d) { vx += ox; vy += oy; }
                }
            }
            if (valid && (lane == 31 || next != idx) && (vx != 0.f || vy != 0.f)) atomicAdd(lt + idx, make_float2(vx, vy));
        }
    }
}

void launch_hash_backward(const FieldView& fv, const float* coords, uint32_t stride, uint32_t n, const float* dxd, uint32_t kd,
                          float* gtable, cudaStream_t s) {
    const unsigned blocks = (n + 255) / 256;
    if (fv.n_features == 8) hash_backward_wide_kernel<8><<<blocks, 256, 0, s>>>(fv, coords, stride, n, dxd, kd, gtable);
    else if (fv.n_features == 4) hash_backward_wide_kernel<4><<<blocks, 256, 0, s>>>(fv, coords, stride, n, dxd, kd, gtable);
    else hash_backward_kernel<<<blocks, 256, 0, s>>>(fv, coords, stride, n, dxd, kd, gtable);
}

// Adam (the optimizer the INSTA configuration nests in its Ema, configs/nerf/main.json), in the
// form tiny-cuda-nn's Adam takes (absent here, restated from its published behaviour): the
// gradient is first divided by the loss scale the loss kernel multiplied in (LOSS_SCALE, 128 in
// train_nerf_step); the MLP weights (the first n_matrix parameters, "matrix" parameters) get the
// L2 term l2 * w and step every call; a hash-table entry whose gradient is exactly zero is left
// alone (weights, moments and its own step count unchanged: sparse updates of the table), and
// no L2 term is added to table entries.  The step uses the bias correction folded into the rate
// (Kingma & Ba, "Adam", sec. 2: lr_t = lr sqrt(1 - b2^t) / (1 - b1^t), w -= lr_t m / (sqrt(v) + eps))
// with t the parameter's own step count.  With an Ema (ema != nullptr) the bias-corrected running
// average of the weights (e_old scaled by decay * debias_old, plus (1 - decay) w, over debias_new)
// is kept in FP32 for every parameter and written as the FP16 parameters (the weights themselves
// to w16_train); without one the weights themselves are the FP16 parameters.
__global__ void __launch_bounds__(256) adam_kernel(size_t n, size_t n_matrix, float* __restrict__ w, float* __restrict__ m,
                                                   float* __restrict__ v, uint32_t* __restrict__ table_steps,
                                                   const float* __restrict__ g, float inv_loss_scale, float lr, float b1, float b2,
                                                   float eps, float l2, float lr_matrix, float* __restrict__ ema, float decay,
                                                   float debias_old, float debias_new, __half* __restrict__ w16,
                                                   __half* __restrict__ w16_train) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float gi = g[i] * inv_loss_scale;
        float wi = w[i];
        const bool matrix = i < n_matrix;
        if (matrix || gi != 0.f) {
            float lr_t = lr_matrix;
            if (matrix) {
                gi += l2 * wi;
            } else {
                const uint32_t t = ++table_steps[i - n_matrix];
                lr_t = lr * sqrtf(1.f - powf(b2, (float)t)) / (1.f - powf(b1, (float)t));
            }
            const float mi = b1 * m[i] + (1.f - b1) * gi;
            const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
            m[i] = mi;
            v[i] = vi;
            wi = wi - lr_t * mi / (sqrtf(vi) + eps);
            w[i] = wi;
        }
        float out = wi;
        if (ema) {
            // the first averaged step is the weights themselves (debias_old = 0)
            if (debias_old > 0.f) out = (ema[i] * (decay * debias_old) + (1.f - decay) * wi) / debias_new;
            ema[i] = out;
        }
        w16[i] = __float2half_rn(out);
        if (w16_train) w16_train[i] = __float2half_rn(wi);
    }
}

__global__ void __launch_bounds__(256) half_to_float_kernel(size_t n, const __half* __restrict__ a, float* __restrict__ b) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) b[i] = __half2float(a[i]);
}

// ---- training loss (compute_loss_kernel_train_nerf, testbed_nerf.cu:1305-1644) ----------------

__device__ __forceinline__ float tl_srgb_to_linear(float s) { return s <= 0.04045f ? s / 12.92f : powf((s + 0.055f) / 1.055f, 2.4f); }
__device__ __forceinline__ float tl_linear_to_srgb(float l) { return l < 0.0031308f ? 12.92f * l : 1.055f * powf(l, 0.41666f) - 0.055f; }
__device__ __forceinline__ float tl_logistic(float x) { return 1.f / (1.f + __expf(-x)); }

// loss_and_gradient (testbed_nerf.cu:116-180,1288-1303) of one channel
__device__ __forceinline__ void tl_loss(int type, float target, float pred, float& loss, float& grad) {
    const float d = pred - target;
    switch (type) {
        case 1: loss = fabsf(d); grad = copysignf(1.f, d); break;                                          // L1
        case 2: { const float f = 1.f / (fabsf(pred) + 1e-2f); loss = fabsf(d) * f; grad = copysignf(f, d); } break;   // MAPE
        case 3: { const float f = 1.f / (0.5f * (fabsf(pred) + fabsf(target)) + 1e-2f); loss = fabsf(d) * f; grad = copysignf(f, d); } break;
        case 4: {                                                                                           // Huber(0.1) / 5
            const float a = 0.1f, ad = fabsf(d);
            loss = ad > a ? ad - 0.5f * a : 0.5f / a * d * d;
            grad = ad > a ? (d > 0 ? 1.f : -1.f) : d / a;
            loss /= 5.f;
            grad /= 5.f;
        } break;
        case 5: { const float q = fabsf(d) + 1.f; loss = logf(q); grad = copysignf(1.f / q, d); } break;   // LogL1
        case 6: { const float f = 1.f / (pred * pred + 1e-2f); loss = d * d * f; grad = 2.f * d * f; } break;   // RelativeL2
        default: loss = d * d; grad = 2.f * d; break;                                                        // L2
    }
}

struct TrainLossArgs {
    uint32_t n_rays, max_rays, max_compacted, stride;
    float aabb_min[3], aabb_diag[3];
    int loss_type, depth_loss_type, srgb, linear_train, penalize;
    float loss_scale, depth_lambda, seg_lambda, near_distance, beta;
    const float *rays, *target, *background, *exposure, *depth, *mean_density;
    const int32_t* seg_mask;
    const uint32_t *rays_counter, *ray_indices;
    uint32_t* numsteps;
    const float *coords, *out;
    uint32_t* counter;
    float *coords_out, *dloss, *loss_out;
    uint32_t* base_in;   // each kept ray's block start before compaction (for the copy kernel)
    const float* pdf;    // per ray img_pdf * xy_pdf, or null (1)
    float* error_map;    // [images][res_y][res_x] or null
    uint32_t em_res[2], em_images;
    const float* image_xy;
    const uint32_t* image_index;
};

// The fields of one sample the loss reads: dt (warped), the deformed position, the raw outputs.
struct TlSample {
    float4 o;
    float c3, c5, c6, c7;
};
__device__ __forceinline__ TlSample tl_load(const float* c, const float* out) {
    TlSample t;
    t.o = *reinterpret_cast<const float4*>(out);
    t.c3 = c[3];
    t.c5 = c[5];
    t.c6 = c[6];
    t.c7 = c[7];
    return t;
}

// One thread per kept ray: the two passes over the ray's samples of the reference kernel.
__global__ void __launch_bounds__(32) train_loss_kernel(TrainLossArgs a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= min(*a.rays_counter, a.max_rays)) return;
    const uint32_t numsteps = a.numsteps[2 * i], base = a.numsteps[2 * i + 1];
    const uint32_t ray = a.ray_indices[i];
    const float* R = a.rays + (size_t)ray * 6;
    const float ox = R[0], oy = R[1], oz = R[2];
    const float* cin = a.coords + (size_t)base * a.stride;
    const float* nout = a.out + (size_t)base * 4;
    const float mx = MIN_CONE * 128.0f;
    float T = 1.f, rgb_ray[3] = {0.f, 0.f, 0.f}, depth_ray = 0.f;
    uint32_t cn = 0;
    bool stop = false;
    // four samples' fields are loaded before they are used (a few thousand rays give each SM about
    // one warp, so the loads' latency is hidden only by having several in flight); the arithmetic
    // and its order are those of the one-sample loop
    for (uint32_t j0 = 0; j0 < numsteps && !stop; j0 += 4u) {
        TlSample sm[4];
#pragma unroll
        for (uint32_t u = 0; u < 4u; ++u)
            if (j0 + u < numsteps) sm[u] = tl_load(cin + (size_t)(j0 + u) * a.stride, nout + (size_t)(j0 + u) * 4);
#pragma unroll
        for (uint32_t u = 0; u < 4u; ++u) {
            if (j0 + u >= numsteps) break;
            if (T < 1e-4f) { stop = true; break; }
            const float4 o = sm[u].o;
            const float px = a.aabb_min[0] + sm[u].c5 * a.aabb_diag[0], py = a.aabb_min[1] + sm[u].c6 * a.aabb_diag[1],
                        pz = a.aabb_min[2] + sm[u].c7 * a.aabb_diag[2];
            const float dt = sm[u].c3 * (mx - MIN_CONE) + MIN_CONE;
            const float dx = px - ox, dy = py - oy, dz = pz - oz;
            const float cur_depth = sqrtf(dx * dx + dy * dy + dz * dz);
            const float density = __expf(o.w);
            const float alpha = 1.f - __expf(-density * dt);
            const float w = alpha * T;
            rgb_ray[0] += w * tl_logistic(o.x);
            rgb_ray[1] += w * tl_logistic(o.y);
            rgb_ray[2] += w * tl_logistic(o.z);
            depth_ray += w * cur_depth;
            T *= (1.f - alpha);
            ++cn;
        }
    }
    const float T_ray = T;
    // target colour and background (random_bg_color draw in sRGB, linearised)
    float bg[3], tgt[3];
    const float* ts = a.target + (size_t)ray * 4;
    const float ta = ts[3];
    float ex[3] = {1.f, 1.f, 1.f};
    for (int k = 0; k < 3; ++k) {
        bg[k] = tl_srgb_to_linear(a.background ? a.background[(size_t)ray * 3 + k] : 0.f);
        if (a.exposure) ex[k] = expf(0.6931471805599453f * a.exposure[(size_t)ray * 3 + k]);
    }
    if (a.linear_train || !a.srgb) {
        for (int k = 0; k < 3; ++k) tgt[k] = ex[k] * ts[k] + (1.f - ta) * bg[k];
        if (!a.linear_train)
            for (int k = 0; k < 3; ++k) { tgt[k] = tl_linear_to_srgb(tgt[k]); bg[k] = tl_linear_to_srgb(bg[k]); }
    } else {
        for (int k = 0; k < 3; ++k) bg[k] = tl_linear_to_srgb(bg[k]);
        if (ta > 0.f)
            for (int k = 0; k < 3; ++k) tgt[k] = tl_linear_to_srgb(ex[k] * ts[k] / ta) * ta + (1.f - ta) * bg[k];
        else
            for (int k = 0; k < 3; ++k) tgt[k] = bg[k];
    }
    if (cn == numsteps)
        for (int k = 0; k < 3; ++k) rgb_ray[k] += T * bg[k];
    // compacted block
    const uint32_t cbase = atomicAdd(a.counter, cn);
    const uint32_t ccount = min(a.max_compacted - min(a.max_compacted, cbase), cn);
    a.numsteps[2 * i] = ccount;
    a.numsteps[2 * i + 1] = cbase;
    a.base_in[i] = base;
    if (ccount == 0) return;
    float seg_sup = 1.f, depth_lambda = a.depth_lambda;
    if (a.seg_mask) {
        const int m = a.seg_mask[ray];
        if (m == 120 || m == 130 || m == 140) seg_sup = a.seg_lambda;
        if (m <= 90 || m > 250) depth_lambda = 0.f;
        if (ta < 0.001f) depth_lambda = 0.f;
    }
    const float dn = sqrtf(R[3] * R[3] + R[4] * R[4] + R[5] * R[5]);
    const float target_depth = dn * ((depth_lambda > 0.f && a.depth) ? a.depth[ray] : -1.f);
    float dl, dg;
    tl_loss(a.depth_loss_type, target_depth, depth_ray, dl, dg);
    const float depth_grad = (target_depth > 0.f ? dg : 0.f) * depth_lambda;
    float lgrad[3], lsum = 0.f;
    const float pdf = a.pdf ? a.pdf[ray] : 1.f;
    for (int k = 0; k < 3; ++k) {
        float l, g;
        tl_loss(a.loss_type, tgt[k], rgb_ray[k], l, g);
        lgrad[k] = g * seg_sup;
        lsum += a.pdf ? __fdiv_rn(l, pdf) : l;   // lg.loss /= img_pdf * xy_pdf
    }
    const float mean_loss = lsum / 3.f;
    if (a.loss_out) a.loss_out[i] = mean_loss / (float)a.n_rays;
    if (a.error_map && a.image_index[ray] < a.em_images) {
        // the ray's mean loss splatted bilinearly at its image position (texel centres at +0.5);
        // the reference clamps the cell by the image resolution - 2, which equals the map's own
        // bound while the map is no larger than the image
        const float rx = (float)a.em_res[0], ry = (float)a.em_res[1];
        const float2 xy = *reinterpret_cast<const float2*>(a.image_xy + (size_t)ray * 2);
        const float px = fminf(fmaxf(fmaf(xy.x, rx, -0.5f), 0.f), __fsub_rn(rx, 1.0001f));
        const float py = fminf(fmaxf(fmaf(xy.y, ry, -0.5f), 0.f), __fsub_rn(ry, 1.0001f));
        const int ix0 = (int)px, iy0 = (int)py;
        const float wx = __fsub_rn(px, (float)ix0), wy = __fsub_rn(py, (float)iy0);
        const int ix = min(max(ix0, 0), (int)a.em_res[0] - 2), iy = min(max(iy0, 0), (int)a.em_res[1] - 2);
        float* em = a.error_map + (size_t)a.image_index[ray] * a.em_res[0] * a.em_res[1];
        const float ux = __fsub_rn(1.f, wx), uy = __fsub_rn(1.f, wy);
        atomicAdd(em + (size_t)iy * a.em_res[0] + ix, __fmul_rn(__fmul_rn(ux, uy), mean_loss));
        atomicAdd(em + (size_t)iy * a.em_res[0] + ix + 1, __fmul_rn(__fmul_rn(wx, uy), mean_loss));
        atomicAdd(em + (size_t)(iy + 1) * a.em_res[0] + ix, __fmul_rn(__fmul_rn(ux, wy), mean_loss));
        atomicAdd(em + (size_t)(iy + 1) * a.em_res[0] + ix + 1, __fmul_rn(__fmul_rn(wx, wy), mean_loss));
    }
    const float loss_scale = a.loss_scale / (float)a.n_rays;
    const float l1_density = (a.mean_density && *a.mean_density < 0.01f) ? 1e-4f : 0.f;
    // second pass: the per-sample gradients, and the records copied to their compacted block
    float rgb2[3] = {0.f, 0.f, 0.f}, depth2 = 0.f;
    T = 1.f;
    float* dout = a.dloss + (size_t)cbase * 4;
    for (uint32_t j0 = 0; j0 < ccount; j0 += 4u) {
        TlSample sm2[4];
#pragma unroll
        for (uint32_t u = 0; u < 4u; ++u)
            if (j0 + u < ccount) sm2[u] = tl_load(cin + (size_t)(j0 + u) * a.stride, nout + (size_t)(j0 + u) * 4);
#pragma unroll
        for (uint32_t u = 0; u < 4u; ++u) {
            const uint32_t j = j0 + u;
            if (j >= ccount) break;
            const TlSample& q = sm2[u];
            const float px = a.aabb_min[0] + q.c5 * a.aabb_diag[0], py = a.aabb_min[1] + q.c6 * a.aabb_diag[1],
                        pz = a.aabb_min[2] + q.c7 * a.aabb_diag[2];
            const float dx = px - ox, dy = py - oy, dz = pz - oz;
            const float depth = sqrtf(dx * dx + dy * dy + dz * dz);
            const float dt = q.c3 * (mx - MIN_CONE) + MIN_CONE;
            const float4 o = q.o;
            const float rgb[3] = {tl_logistic(o.x), tl_logistic(o.y), tl_logistic(o.z)};
            const float density = __expf(o.w);
            const float alpha = 1.f - __expf(-density * dt);
            const float w = alpha * T;
            for (int k = 0; k < 3; ++k) rgb2[k] += w * rgb[k];
            depth2 += w * depth;
            T *= (1.f - alpha);
            float d4[4], dot = 0.f;
            for (int k = 0; k < 3; ++k) {
                const float suffix = rgb_ray[k] - rgb2[k];
                d4[k] = loss_scale * ((w * lgrad[k]) * (rgb[k] * (1.f - rgb[k])));   // logistic: no output L2 term
                dot += lgrad[k] * (T * rgb[k] - suffix);
            }
            const float dd = __expf(fminf(fmaxf(o.w, -15.f), 15.f));
            const float depth_sup = depth_grad * (T * depth - (depth_ray - depth2));
            const float beta_sup = dt / (T_ray - 1.f + 1e-3f);
            float dmlp = dd * (dt * (dot + depth_sup) + a.beta * beta_sup);
            if (a.penalize) dmlp += (ta <= 0.01f) ? w : 0.f;
            d4[3] = loss_scale * dmlp + (o.w < 0.f ? -l1_density : 0.f) + (o.w > -10.f && depth < a.near_distance ? 1e-4f : 0.f);
            *reinterpret_cast<float4*>(dout + (size_t)j * 4) = make_float4(d4[0], d4[1], d4[2], d4[3]);
        }
    }
}

// The records of each kept ray's compacted block, copied after the loss kernel has placed the
// block: one warp per ray, the block's floats are contiguous on both sides (coalesced).
__global__ void __launch_bounds__(256) compact_copy_kernel(const uint32_t* __restrict__ rays_counter, uint32_t max_rays,
                                                           const uint32_t* __restrict__ numsteps_in, const uint32_t* __restrict__ numsteps,
                                                           uint32_t stride, const float* __restrict__ coords, float* __restrict__ coords_out) {
    const uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (k >= min(*rays_counter, max_rays)) return;
    const uint32_t count = numsteps[2 * k], cbase = numsteps[2 * k + 1], base = numsteps_in[k];
    const size_t nf = (size_t)count * stride;
    const float* src = coords + (size_t)base * stride;
    float* dst = coords_out + (size_t)cbase * stride;
    for (size_t f = lane; f < nf; f += 32) dst[f] = src[f];
}

// tiny-cuda-nn fill_rollover / fill_rollover_and_rescale: entries [count*width, total*width) repeat
// the first count*width entries; the repeated gradients are scaled by count / total.
__global__ void __launch_bounds__(256) rollover_kernel(size_t total, uint32_t width, const uint32_t* __restrict__ counter, uint32_t cap,
                                                       float* __restrict__ data, int rescale, uint32_t n_total) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t cnt = min(*counter, cap);
    const size_t have = (size_t)cnt * width;
    if (cnt == 0 || i < have || i >= total) return;
    float v = data[i % have];
    if (rescale) v = v * (float)cnt / (float)n_total;
    data[i] = v;
}

cudaError_t launch_train_loss(const ::insta_train_loss_desc& d, uint32_t* base_scratch, cudaStream_t s) {
    TrainLossArgs a{};
    a.n_rays = d.n_rays; a.max_rays = d.max_rays; a.max_compacted = d.max_samples_compacted; a.stride = d.stride;
    for (int k = 0; k < 3; ++k) { a.aabb_min[k] = d.aabb_min[k]; a.aabb_diag[k] = d.aabb_max[k] - d.aabb_min[k]; }
    a.loss_type = d.loss_type; a.depth_loss_type = d.depth_loss_type; a.srgb = d.srgb_targets; a.linear_train = d.train_in_linear_colors;
    a.penalize = d.penalize_density; a.loss_scale = d.loss_scale; a.depth_lambda = d.depth_supervision_lambda;
    a.seg_lambda = d.seg_mask_supervision_lambda; a.near_distance = d.near_distance; a.beta = d.beta;
    a.rays = d.rays; a.target = d.target; a.background = d.background; a.exposure = d.exposure; a.depth = d.depth;
    a.mean_density = d.mean_density; a.seg_mask = d.seg_mask; a.rays_counter = d.rays_counter; a.ray_indices = d.ray_indices;
    a.numsteps = d.numsteps; a.coords = d.coords; a.out = d.network_output; a.counter = d.numsteps_counter;
    a.coords_out = d.coords_out; a.dloss = d.dloss_doutput; a.loss_out = d.loss_output; a.base_in = base_scratch;
    a.pdf = d.pdf; a.error_map = d.error_map; a.em_res[0] = d.error_map_res[0]; a.em_res[1] = d.error_map_res[1];
    a.em_images = d.error_map_images;
    a.image_xy = d.image_xy; a.image_index = d.image_index;
    if (d.max_rays > 0) {
        // one ray per thread in 32-thread blocks: a batch of a few thousand rays spreads over every SM
        train_loss_kernel<<<(d.max_rays + 31) / 32, 32, 0, s>>>(a);
        compact_copy_kernel<<<(unsigned)(((size_t)d.max_rays * 32 + 255) / 256), 256, 0, s>>>(d.rays_counter, d.max_rays, base_scratch,
                                                                                               d.numsteps, d.stride, d.coords, d.coords_out);
    }
    if (d.target_batch_size > 0) {
        const size_t nd = (size_t)d.target_batch_size * 4, nc = (size_t)d.target_batch_size * d.stride;
        rollover_kernel<<<(unsigned)((nd + 255) / 256), 256, 0, s>>>(nd, 4, d.numsteps_counter, d.max_samples_compacted, d.dloss_doutput, 1,
                                                                       d.target_batch_size);
        rollover_kernel<<<(unsigned)((nc + 255) / 256), 256, 0, s>>>(nc, d.stride, d.numsteps_counter, d.max_samples_compacted, d.coords_out, 0,
                                                                       d.target_batch_size);
    }
    return cudaGetLastError();
}

// ------------------------------------------------------------ image / pixel draws, error map
constexpr float kMinPdf = 0.01f;                // construct_cdf_2d / _1d
constexpr float kMinPmf = 0.1f;                 // the image CDF of train_nerf_step
constexpr float kUniformFraction = 0.5f;        // sample_cdf_2d's uniform share

// binary_search (instant-ngp/include/neural-graphics-primitives/common.h:195-218): the first index
// whose value is not below val, clamped to length - 1.
__device__ __forceinline__ uint32_t cdf_search(float val, const float* __restrict__ data, uint32_t length) {
    uint32_t first = 0, count = length;
    while (count > 0) {
        const uint32_t step = count / 2, it = first + step;
        if (data[it] < val) { first = it + 1; count -= step + 1; }
        else count = step;
    }
    return min(first, length - 1);
}

// image_idx, nerf_random_image_pos_training (sample_cdf_2d) and the background draw per ray.
__global__ void __launch_bounds__(256) training_pixels_kernel(const ::insta_training_pixels_desc d) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n_rays) return;
    const uint32_t ni = d.n_images;
    uint32_t img;
    float img_pdf = 1.f;
    if (d.cdf_img) {
        const float u = ld_random_val(i + d.n_rays_total, 0xdeadbeefu, 0u);
        img = cdf_search(u, d.cdf_img, ni);
        const float prev = img > 0 ? d.cdf_img[img - 1] : 0.f;
        img_pdf = __fmul_rn(__fsub_rn(d.cdf_img[img], prev), (float)ni);
    } else {
        img = ((i + d.n_rays_total) * ni / d.n_rays) % ni;
    }
    Pcg32 rng{d.rng_state, d.rng_inc};
    rng.advance((int64_t)i * 8);   // N_MAX_RANDOM_SAMPLES_PER_RAY
    float sx = rng.next_float();
    float sy = rng.next_float();
    float xy_pdf = 1.f;
    if (d.cdf_x_cond_y) {
        if (sx < kUniformFraction) {
            sx = __fdiv_rn(sx, kUniformFraction);
        } else {
            sx = __fdiv_rn(__fsub_rn(sx, kUniformFraction), __fsub_rn(1.f, kUniformFraction));
            const uint32_t rx = d.cdf_res[0], ry = d.cdf_res[1];
            const float* cy = d.cdf_y + (size_t)img * ry;
            const uint32_t y = cdf_search(sy, cy, ry);
            float prev = y > 0 ? cy[y - 1] : 0.f;
            const float pmf_y = __fsub_rn(cy[y], prev);
            sy = __fdiv_rn(__fsub_rn(sy, prev), pmf_y);
            const float* cx = d.cdf_x_cond_y + ((size_t)img * ry + y) * rx;
            const uint32_t x = cdf_search(sx, cx, rx);
            prev = x > 0 ? cx[x - 1] : 0.f;
            const float pmf_x = __fsub_rn(cx[x], prev);
            sx = __fdiv_rn(__fsub_rn(sx, prev), pmf_x);
            xy_pdf = __fmul_rn(__fmul_rn(pmf_x, pmf_y), (float)(rx * ry));
            sx = __fdiv_rn(__fadd_rn((float)x, sx), (float)rx);
            sy = __fdiv_rn(__fadd_rn((float)y, sy), (float)ry);
        }
    }
    if (d.snap_to_pixel_centers) {
        const int w = d.resolution[2 * img], h = d.resolution[2 * img + 1];
        const int px = min(max((int)__fmul_rn(sx, (float)w), 0), w - 1), py = min(max((int)__fmul_rn(sy, (float)h), 0), h - 1);
        sx = __fdiv_rn(__fadd_rn((float)px, 0.5f), (float)w);
        sy = __fdiv_rn(__fadd_rn((float)py, 0.5f), (float)h);
    }
    d.out_image[i] = img;
    d.out_xy[2 * i] = sx;
    d.out_xy[2 * i + 1] = sy;
    if (d.out_pdf) d.out_pdf[i] = __fmul_rn(img_pdf, xy_pdf);
    if (d.out_background) {
        const float b0 = rng.next_float(), b1 = rng.next_float(), b2 = rng.next_float();
        d.out_background[3 * i] = b0;
        d.out_background[3 * i + 1] = b1;
        d.out_background[3 * i + 2] = b2;
    }
}

// construct_cdf_2d: a thread per (row, image).  The normalisation's multiply-add is one fused
// operation, as nvcc contracts it in the reference's kernel.
__global__ void __launch_bounds__(256) cdf_rows_kernel(uint32_t n_images, uint32_t h, uint32_t w, const float* __restrict__ data,
                                                      float* __restrict__ cdf_x, float* __restrict__ cdf_y) {
    const uint32_t y = blockIdx.x * blockDim.x + threadIdx.x, img = blockIdx.y;
    if (y >= h || img >= n_images) return;
    const size_t off = ((size_t)img * h + y) * w;
    float cum = 0.f;
    for (uint32_t x = 0; x < w; ++x) {
        cum = __fadd_rn(cum, __fadd_rn(data[off + x], 1e-10f));
        cdf_x[off + x] = cum;
    }
    cdf_y[(size_t)img * h + y] = cum;
    const float norm = __frcp_rn(cum);
    for (uint32_t x = 0; x < w; ++x)
        cdf_x[off + x] = fmaf(__fmul_rn(1.f - kMinPdf, cdf_x[off + x]), norm, __fdiv_rn(__fmul_rn(kMinPdf, (float)(x + 1)), (float)w));
}

// construct_cdf_1d (a thread per image), then one thread: the image CDF with its PMF.
__global__ void __launch_bounds__(256) cdf_cols_kernel(uint32_t n_images, uint32_t h, float* __restrict__ cdf_y, float* __restrict__ cdf_img) {
    const uint32_t img = blockIdx.x * blockDim.x + threadIdx.x;
    if (img >= n_images) return;
    float* cy = cdf_y + (size_t)img * h;
    float cum = 0.f;
    for (uint32_t y = 0; y < h; ++y) {
        cum = __fadd_rn(cum, cy[y]);
        cy[y] = cum;
    }
    cdf_img[img] = cum;
    const float norm = __frcp_rn(cum);
    for (uint32_t y = 0; y < h; ++y) cy[y] = fmaf(__fmul_rn(1.f - kMinPdf, cy[y]), norm, __fdiv_rn(__fmul_rn(kMinPdf, (float)(y + 1)), (float)h));
}

// The image CDF, which the reference computes on the host (separate multiply and add: the host
// build has no fused multiply-add), here in one device thread with the same operations.
__global__ void cdf_images_kernel(uint32_t n_images, float* __restrict__ cdf_img, float* __restrict__ pmf_img) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    float cum = 0.f;
    for (uint32_t i = 0; i < n_images; ++i) cum = __fadd_rn(cum, cdf_img[i]);
    const float norm = __fdiv_rn(1.f, cum);
    float run = 0.f;
    const float n = (float)n_images;
    for (uint32_t i = 0; i < n_images; ++i) {
        const float v = cdf_img[i];
        run = __fadd_rn(run, v);
        if (pmf_img) pmf_img[i] = __fadd_rn(__fmul_rn(__fmul_rn(1.f - kMinPmf, v), norm), __fdiv_rn(kMinPmf, n));
        cdf_img[i] = __fadd_rn(__fmul_rn(__fmul_rn(1.f - kMinPmf, run), norm), __fdiv_rn(__fmul_rn(kMinPmf, (float)(i + 1)), n));
    }
}

cudaError_t launch_training_pixels(const ::insta_training_pixels_desc& d, cudaStream_t s) {
    if (d.n_rays == 0) return cudaSuccess;
    training_pixels_kernel<<<(d.n_rays + 255) / 256, 256, 0, s>>>(d);
    return cudaGetLastError();
}

cudaError_t launch_error_map_cdf(const float* em, uint32_t n_images, uint32_t w, uint32_t h, float* cdf_x, float* cdf_y, float* cdf_img,
                                 float* pmf_img, cudaStream_t s) {
    cdf_rows_kernel<<<dim3((h + 255) / 256, n_images), 256, 0, s>>>(n_images, h, w, em, cdf_x, cdf_y);
    cdf_cols_kernel<<<(n_images + 255) / 256, 256, 0, s>>>(n_images, h, cdf_y, cdf_img);
    cdf_images_kernel<<<1, 32, 0, s>>>(n_images, cdf_img, pmf_img);
    return cudaGetLastError();
}

static unsigned grid_for(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, 152 * 32); }

size_t train_scratch_floats(const TrainShape& t, uint32_t n) {
    size_t per = t.kd + 32 + 16;   // X_d, X_r, Y_r
    for (int l = 0; l + 1 < t.n_density; ++l) per += 64;
    for (int l = 0; l + 1 < t.n_rgb; ++l) per += 64;
    return per * 2 * (size_t)n + 64;   // activations and their gradients
}

// Column-major GEMM helpers (all matrices are [rows x n] with leading dimension rows).
static cublasStatus_t fwd(cublasHandle_t h, const float* W, uint32_t n_out, uint32_t n_in, const float* X, uint32_t ldx, float* Y,
                          uint32_t ldy, uint32_t n) {
    const float one = 1.f, zero = 0.f;
    // Y (n_out x n) = W (n_out x n_in, stored row-major = col-major n_in x n_out, transposed) * X
    return cublasSgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, (int)n_out, (int)n, (int)n_in, &one, W, (int)n_in, X, (int)ldx, &zero, Y, (int)ldy);
}
static cublasStatus_t bwd(cublasHandle_t h, const float* W, uint32_t n_out, uint32_t n_in, const float* dY, uint32_t lddy, float* dX,
                          uint32_t lddx, uint32_t n) {
    const float one = 1.f, zero = 0.f;
    // dX (n_in x n) = W^T (n_in x n_out) * dY
    return cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)n_in, (int)n, (int)n_out, &one, W, (int)n_in, dY, (int)lddy, &zero, dX, (int)lddx);
}
static cublasStatus_t wgrad(cublasHandle_t h, const float* X, uint32_t ldx, uint32_t n_in, const float* dY, uint32_t lddy, uint32_t n_out,
                            float* dW, uint32_t n) {
    const float one = 1.f;
    // dW^T (n_in x n_out, = dW row-major) += X (n_in x n) * dY^T (n x n_out)
    return cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_T, (int)n_in, (int)n_out, (int)n, &one, X, (int)ldx, dY, (int)lddy, &one, dW, (int)n_in);
}

// The expression-dim columns of the density MLP's input gradient (after the 2 n_levels hash
// features), per sample.
__global__ void __launch_bounds__(256) extra_grad_kernel(uint32_t n, const float* __restrict__ dxd, uint32_t kd, uint32_t first,
                                                         uint32_t n_extra, float* __restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n * n_extra) return;
    const size_t s = i / n_extra, k = i % n_extra;
    out[i] = dxd[s * kd + first + k];
}

static cudaError_t launch_extra_grad(const FieldView& fv, const TrainShape& t, uint32_t n, const float* dxd, float* out, cudaStream_t s) {
    const uint32_t ne = fv.n_extra;
    if (!out || ne == 0) return cudaSuccess;
    extra_grad_kernel<<<(unsigned)(((size_t)n * ne + 255) / 256), 256, 0, s>>>(n, dxd, t.kd, fv.n_features * fv.n_levels, ne, out);
    return cudaGetLastError();
}

// compute_extra_dims_gradient_train_nerf: a thread per (kept ray, dim) sums the ray's samples,
// then one addition into the ray's image row.
__global__ void __launch_bounds__(256) extra_dims_gradient_kernel(const ::insta_extra_dims_gradient_desc d) {
    const uint32_t ne = d.n_extra_dims;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = (uint32_t)(t / ne), k = (uint32_t)(t % ne);
    if (i >= min(*d.rays_counter, d.max_rays)) return;
    const uint32_t count = d.numsteps[2 * i], base = d.numsteps[2 * i + 1];
    const uint32_t img = d.image_index[d.ray_indices[i]];
    if (count == 0 || img >= d.n_images) return;   // rays of images outside the gradient add nothing
    const float* g = d.dl_dextra + (size_t)base * ne + k;
    float sum = 0.f;
    for (uint32_t j = 0; j < count; ++j) sum += g[(size_t)j * ne];
    atomicAdd(d.extra_dims_gradient + (size_t)img * ne + k, sum);
}

cudaError_t launch_extra_dims_gradient(const ::insta_extra_dims_gradient_desc& d, cudaStream_t s) {
    const size_t threads = (size_t)d.max_rays * d.n_extra_dims;
    if (threads == 0) return cudaSuccess;
    extra_dims_gradient_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(d);
    return cudaGetLastError();
}

cudaError_t launch_field_train(cublasHandle_t h, const FieldView& fv, const TrainShape& t, const float* w32, const float* coords,
                               uint32_t stride, uint32_t n, const float* dl_dout, float* out4, float* grad, float* scratch,
                               cudaStream_t s, float* dl_dextra) {
    if (n == 0) return cudaSuccess;
    if (cublasSetStream(h, s) != CUBLAS_STATUS_SUCCESS) return cudaErrorUnknown;
    // activations: X_d [kd x n], H_d[l] [64 x n], X_r [32 x n] (rows 0..15 = density output), H_r[l] [64 x n], Y_r [16 x n]
    float* p = scratch;
    float* xd = p; p += (size_t)t.kd * n;
    float* hd[4];
    for (int l = 0; l + 1 < t.n_density; ++l) { hd[l] = p; p += (size_t)64 * n; }
    float* xr = p; p += (size_t)32 * n;
    float* hr[4];
    for (int l = 0; l + 1 < t.n_rgb; ++l) { hr[l] = p; p += (size_t)64 * n; }
    float* yr = p; p += (size_t)16 * n;
    // gradients of the same shapes
    float* dxd = p; p += (size_t)t.kd * n;
    float* dhd[4];
    for (int l = 0; l + 1 < t.n_density; ++l) { dhd[l] = p; p += (size_t)64 * n; }
    float* dxr = p; p += (size_t)32 * n;
    float* dhr[4];
    for (int l = 0; l + 1 < t.n_rgb; ++l) { dhr[l] = p; p += (size_t)64 * n; }
    float* dyr = p; p += (size_t)16 * n;

    launch_train_encode(fv, coords, stride, n, xd, t.kd, xr, s);
    bool okb = true;
    // density MLP: hidden layers then the 16 outputs into X_r rows 0..15
    const float* in = xd;
    uint32_t ldin = t.kd, kin = t.kd;
    for (int l = 0; l < t.n_density; ++l) {
        const bool last = l + 1 == t.n_density;
        float* out = last ? xr : hd[l];
        const uint32_t n_out = last ? 16u : 64u;
        okb &= fwd(h, w32 + t.layer_off[l], n_out, kin, in, ldin, out, last ? 32u : 64u, n) == CUBLAS_STATUS_SUCCESS;
        if (!last) relu_kernel<<<grid_for((size_t)64 * n), 256, 0, s>>>(out, (size_t)64 * n);
        in = out; ldin = 64; kin = 64;
    }
    // colour MLP
    in = xr; ldin = 32; kin = 32;
    for (int l = 0; l < t.n_rgb; ++l) {
        const int li = t.n_density + l;
        const bool last = l + 1 == t.n_rgb;
        float* out = last ? yr : hr[l];
        const uint32_t n_out = last ? 16u : 64u;
        okb &= fwd(h, w32 + t.layer_off[li], n_out, kin, in, ldin, out, n_out, n) == CUBLAS_STATUS_SUCCESS;
        if (!last) relu_kernel<<<grid_for((size_t)64 * n), 256, 0, s>>>(out, (size_t)64 * n);
        in = out; ldin = 64; kin = 64;
    }
    train_out_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, yr, xr, dl_dout, dyr, out4);
    if (!dl_dout || !grad) return okb ? cudaGetLastError() : cudaErrorUnknown;
    // colour MLP backward
    const float* dout = dyr;
    uint32_t lddout = 16, n_out = 16;
    for (int l = t.n_rgb - 1; l >= 0; --l) {
        const int li = t.n_density + l;
        const float* x = l == 0 ? xr : hr[l - 1];
        float* dx = l == 0 ? dxr : dhr[l - 1];
        const uint32_t k = l == 0 ? 32u : 64u;
        okb &= wgrad(h, x, k, k, dout, lddout, n_out, grad + t.layer_off[li], n) == CUBLAS_STATUS_SUCCESS;
        okb &= bwd(h, w32 + t.layer_off[li], n_out, k, dout, lddout, dx, k, n) == CUBLAS_STATUS_SUCCESS;
        if (l > 0) relu_back_kernel<<<grid_for((size_t)64 * n), 256, 0, s>>>(dx, hr[l - 1], (size_t)64 * n);
        dout = dx; lddout = k; n_out = k;
    }
    // dL/d density output: the colour input's rows 0..15, plus the raw density's own gradient
    train_density_grad_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, dl_dout, dxr);
    dout = dxr;
    lddout = 32;
    n_out = 16;
    for (int l = t.n_density - 1; l >= 0; --l) {
        const float* x = l == 0 ? xd : hd[l - 1];
        float* dx = l == 0 ? dxd : dhd[l - 1];
        const uint32_t k = l == 0 ? t.kd : 64u;
        okb &= wgrad(h, x, k, k, dout, lddout, n_out, grad + t.layer_off[l], n) == CUBLAS_STATUS_SUCCESS;
        okb &= bwd(h, w32 + t.layer_off[l], n_out, k, dout, lddout, dx, k, n) == CUBLAS_STATUS_SUCCESS;
        if (l > 0) relu_back_kernel<<<grid_for((size_t)64 * n), 256, 0, s>>>(dx, hd[l - 1], (size_t)64 * n);
        dout = dx; lddout = k; n_out = k;
    }
    launch_hash_backward(fv, coords, stride, n, dxd, t.kd, grad + t.table_off, s);
    if (!okb) return cudaErrorUnknown;
    return launch_extra_grad(fv, t, n, dxd, dl_dextra, s);
}

cudaError_t launch_field_train_tc(const FieldView& fv, const TrainShape& t, const TrainMlpPlan& plan, const TrainImageList& images,
                                  uint8_t* img_dev, const float* w32, const float* coords, uint32_t stride, uint32_t n,
                                  const float* dl_dout, float* out4, float* grad, float* scratch, uint32_t* err, cudaStream_t s,
                                  float* dl_dextra) {
    if (n == 0) return cudaSuccess;
    float* xd = scratch;
    float* xr = xd + (size_t)t.kd * n;
    float* dxd = xr + (size_t)32 * n;
    launch_train_encode(fv, coords, stride, n, xd, t.kd, xr, s);
    const bool bwd = dl_dout && grad;
    TrainMlpArgs a{};
    a.plan = plan;
    a.images = img_dev;
    a.xd = xd;
    a.xr = xr;
    a.dl_dout = bwd ? dl_dout : nullptr;
    a.out4 = out4;
    a.dxd = dxd;
    a.grad = grad;
    a.n = n;
    a.err = err;
    cudaError_t e = launch_train_mlp(a, images, w32, img_dev, s);
    if (e != cudaSuccess || !bwd) return e;
    launch_hash_backward(fv, coords, stride, n, dxd, t.kd, grad + t.table_off, s);
    return launch_extra_grad(fv, t, n, dxd, dl_dextra, s);
}

cudaError_t launch_adam(size_t n, size_t n_matrix, float* w, float* m, float* v, uint32_t* table_steps, const float* g, float loss_scale,
                        float lr, float b1, float b2, float eps, float l2, uint32_t step, float* ema, float decay, uint32_t ema_step,
                        __half* w16, __half* w16_train, cudaStream_t s) {
    const float lr_matrix = lr * sqrtf(1.f - powf(b2, (float)step)) / (1.f - powf(b1, (float)step));
    const float debias_old = 1.f - powf(decay, (float)(ema_step - 1u)), debias_new = 1.f - powf(decay, (float)ema_step);
    adam_kernel<<<grid_for(n), 256, 0, s>>>(n, n_matrix, w, m, v, table_steps, g, 1.f / loss_scale, lr, b1, b2, eps, l2, lr_matrix, ema,
                                            decay, debias_old, debias_new, w16, w16_train);
    return cudaGetLastError();
}

cudaError_t launch_half_to_float(size_t n, const void* a, float* b, cudaStream_t s) {
    half_to_float_kernel<<<grid_for(n), 256, 0, s>>>(n, static_cast<const __half*>(a), b);
    return cudaGetLastError();
}

}  // namespace insta
