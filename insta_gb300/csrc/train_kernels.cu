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
// table, FP32 atomics) and the elementwise steps are kernels here.  Values are FP32 from the
// FP16 parameters; the forward is that of the field evaluation in FP32 (no FP16 rounding between
// layers).
#include <cublas_v2.h>

#include "device_common.cuh"
#include "kernels.h"

namespace insta {

// Encode: X_d[:, 0:32] = hash encoding, X_d[:, 32:32+n_extra] = the record's expression dims,
// X_r[:, 16:32] = SH of the direction (X_r[:, 0:16] is filled by the density MLP's output).
__global__ void __launch_bounds__(256) train_encode_kernel(FieldView fv, const float* __restrict__ coords, uint32_t stride, uint32_t n,
                                                           float* __restrict__ xd, uint32_t kd, float* __restrict__ xr) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* c = coords + (size_t)i * stride;
    const __half2* table = reinterpret_cast<const __half2*>(fv.table);
    const V3 p = v3(c[0], c[1], c[2]);
    float* x = xd + (size_t)i * kd;
    for (uint32_t l = 0; l < fv.n_levels; ++l) {
        float a0, a1;
        hash_level(fv, table, p, l, a0, a1);
        x[2 * l] = a0;
        x[2 * l + 1] = a1;
    }
    for (uint32_t m = 0; m < fv.n_extra; ++m) x[2 * fv.n_levels + m] = c[stride - fv.n_extra + m];
    float sh[16];
    sh4(c[8], c[9], c[10], sh);
    float* r = xr + (size_t)i * 32 + 16;
#pragma unroll
    for (int k = 0; k < 16; ++k) r[k] = sh[k];
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

// Hash encode backward: every corner's trilinear weight times the encoding gradient, added into
// the table gradient (FP32, [entries][2] like the table).
__global__ void __launch_bounds__(256) hash_backward_kernel(FieldView fv, const float* __restrict__ coords, uint32_t stride, uint32_t n,
                                                            const float* __restrict__ dxd, uint32_t kd, float* __restrict__ gtable) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* c = coords + (size_t)i * stride;
    const V3 x = v3(c[0], c[1], c[2]);
    const float* dg = dxd + (size_t)i * kd;
    for (uint32_t l = 0; l < fv.n_levels; ++l) {
        const float g0 = dg[2 * l], g1 = dg[2 * l + 1];
        if (g0 == 0.f && g1 == 0.f) continue;
        const float s = fv.level_scale[l];
        const float px = fmaf(x.x, s, 0.5f), py = fmaf(x.y, s, 0.5f), pz = fmaf(x.z, s, 0.5f);
        const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
        const float rx = __fsub_rn(px, fx), ry = __fsub_rn(py, fy), rz = __fsub_rn(pz, fz);
        const uint32_t gx = (uint32_t)(int32_t)fx, gy = (uint32_t)(int32_t)fy, gz = (uint32_t)(int32_t)fz;
        const uint32_t res = fv.level_res[l], size = fv.level_size[l];
        float* lt = gtable + (size_t)fv.level_off[l] * 2;
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
            atomicAdd(lt + (size_t)idx * 2, w * g0);
            atomicAdd(lt + (size_t)idx * 2 + 1, w * g1);
        }
    }
}

// Adam (the optimizer the INSTA configuration nests in its Ema, configs/nerf/main.json): FP32
// master weights, first and second moments, L2 regularisation added to the gradient, bias
// correction; the FP16 parameters are written back.
__global__ void __launch_bounds__(256) adam_kernel(size_t n, float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                                                   const float* __restrict__ g, float lr, float b1, float b2, float eps, float l2,
                                                   float c1, float c2, __half* __restrict__ w16) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i] + l2 * w[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        w16[i] = __float2half_rn(wi);
    }
}

__global__ void __launch_bounds__(256) half_to_float_kernel(size_t n, const __half* __restrict__ a, float* __restrict__ b) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) b[i] = __half2float(a[i]);
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

cudaError_t launch_field_train(cublasHandle_t h, const FieldView& fv, const TrainShape& t, const float* w32, const float* coords,
                               uint32_t stride, uint32_t n, const float* dl_dout, float* out4, float* grad, float* scratch,
                               cudaStream_t s) {
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

    train_encode_kernel<<<(n + 255) / 256, 256, 0, s>>>(fv, coords, stride, n, xd, t.kd, xr);
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
    hash_backward_kernel<<<(n + 255) / 256, 256, 0, s>>>(fv, coords, stride, n, dxd, t.kd, grad + t.table_off);
    return okb ? cudaGetLastError() : cudaErrorUnknown;
}

cudaError_t launch_adam(size_t n, float* w, float* m, float* v, const float* g, float lr, float b1, float b2, float eps, float l2,
                        uint32_t step, __half* w16, cudaStream_t s) {
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    adam_kernel<<<grid_for(n), 256, 0, s>>>(n, w, m, v, g, lr, b1, b2, eps, l2, c1, c2, w16);
    return cudaGetLastError();
}

cudaError_t launch_half_to_float(size_t n, const void* a, float* b, cudaStream_t s) {
    half_to_float_kernel<<<grid_for(n), 256, 0, s>>>(n, static_cast<const __half*>(a), b);
    return cudaGetLastError();
}

}  // namespace insta
