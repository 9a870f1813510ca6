// render_kernels.cu -- the fused render path: one persistent launch marches rays through
// the occupancy bitfield, maps every sample to canonical space through the frame's BVH,
// encodes it on the hash grid, runs the density and colour MLPs on tcgen05 tiles and
// composites front to back.  Each CTA owns 128 ray slots (one per thread); the samples of
// one iteration form the M = 128 tile of the tensor-core MLP, so no sample stream ever
// leaves the SM.  Finished slots are refilled from a global ray counter.
#include "device_common.cuh"
#include "umma.cuh"
#include "kernels.h"

namespace insta {

__device__ __forceinline__ float srgb_to_linear(float s) { return s <= 0.04045f ? s / 12.92f : powf((s + 0.055f) / 1.055f, 2.4f); }

struct SampleIn {
    float pos[3];     // canonical position (network input rows 0..2)
    float dir[3];     // canonical warped direction (rows 8..10)
    float dpos[3];    // deformed world position (for depth)
    uint32_t mask;
};

// generate_next_nerf_network_inputs (:788) writes warp_position(pos) / warp_direction(dir);
// the warp hook (src/core.cu:470-519) maps it to canonical space in place.
__device__ __forceinline__ void deform_sample(const FrameView& fr, const DeformView& dv, const float* tmin, const float* tmax,
                                              V3 pos, V3 dir, SampleIn& s, uint32_t* err) {
    float cw[3], dw[3];
    const float pp[3] = {pos.x, pos.y, pos.z};
    const float dd[3] = {dir.x, dir.y, dir.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        cw[k] = __fdiv_rn(__fsub_rn(pp[k], tmin[k]), __fsub_rn(tmax[k], tmin[k]));
        dw[k] = __fmul_rn(__fadd_rn(dd[k], 1.0f), 0.5f);
        s.dpos[k] = __fadd_rn(tmin[k], __fmul_rn(cw[k], __fsub_rn(tmax[k], tmin[k])));
        s.pos[k] = cw[k];
        s.dir[k] = dw[k];
    }
    s.mask = 7u;   // untouched samples keep their expression dims
    V3 p = v3(cw[0], cw[1], cw[2]);
    if (!box_contains(dv.aabb_min, dv.aabb_max, p)) return;
    NearestResult r = nearest_triangle(fr, p, 0.f, err);
    if (r.id < 0) { atomicOr(err, INSTA_DEVERR_NO_TRI); return; }
    map_to_canonical(dv, fr.frames, (uint32_t)r.id, p, dw, s.pos, s.dir, &s.mask);
}

// Network inputs of one sample, rounded to the MLP activation type (FP16 or BF16).
__device__ __forceinline__ void build_inputs(const FieldView& fv, const float* extra_dims, const SampleIn& s, bool valid,
                                             __half* feat, __half* sh) {
    const bool bf16 = fv.precision == 1;
    float f[48], d[16];
#pragma unroll
    for (int i = 0; i < 48; ++i) f[i] = 0.f;
#pragma unroll
    for (int i = 0; i < 16; ++i) d[i] = 0.f;
    if (valid) {
        hash_encode(fv, v3(s.pos[0], s.pos[1], s.pos[2]), f);
        for (uint32_t m = 0; m < fv.n_extra; ++m)
            f[fv.n_levels * 2 + m] = s.mask != 7u ? 1.f : (extra_dims ? extra_dims[m] : 0.f);
        sh4(s.dir[0], s.dir[1], s.dir[2], d);
    }
#pragma unroll
    for (int i = 0; i < 48; ++i) feat[i] = to_act(f[i], bf16);
#pragma unroll
    for (int i = 0; i < 16; ++i) sh[i] = to_act(d[i], bf16);
}

// ------------------------------------------------------------------ render
struct RenderArgs {
    RenderView rv;
    FrameView fr;
    DeformView dv;
    FieldView fv;
    MlpPlan plan;
    const uint8_t* bitfield;
    const float* extra_dims;
    float* out_rgba;
    float* out_depth;
    uint32_t* ray_counter;
    unsigned long long* sample_counter;
    uint32_t* err;
};

__global__ void __launch_bounds__(128) render_kernel(const __grid_constant__ RenderArgs A) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    MlpSmem& sm = *reinterpret_cast<MlpSmem*>(smem_raw);
    uint8_t* w = smem_raw + ((sizeof(MlpSmem) + 1023) & ~size_t(1023));
    if (!mlp_setup(sm, w, A.fv.mlp_smem, A.plan.bytes)) {
        if (threadIdx.x == 0) atomicOr(A.err, INSTA_DEVERR_TIMEOUT);
        mlp_teardown(sm);
        return;
    }
    const RenderView& rv = A.rv;
    const uint32_t n_rays = (uint32_t)rv.width * (uint32_t)rv.height;
    const bool bf16 = A.fv.precision == 1;
    const V3 cam_fwd = v3(rv.cam[2], rv.cam[6], rv.cam[10]);
    const V3 cam_pos = v3(rv.cam[3], rv.cam[7], rv.cam[11]);

    int64_t pix = -1;
    bool active = true;
    RayState ray;
    float rgba[4] = {0.f, 0.f, 0.f, 0.f}, depth = 0.f, maxw = 0.f;
    uint32_t ns = 0;
    unsigned long long local_samples = 0;

    for (;;) {
        bool has = false;
        V3 pos = v3(0.f, 0.f, 0.f);
        float dt = 0.f;
        while (!has) {
            if (pix < 0) {
                if (!active) break;
                uint32_t idx = atomicAdd(A.ray_counter, 1u);
                if (idx >= n_rays) { active = false; break; }
                reinterpret_cast<float4*>(A.out_rgba)[idx] = make_float4(0.f, 0.f, 0.f, 0.f);
                A.out_depth[idx] = 1e10f;
                if (!ray_init(rv, idx % (uint32_t)rv.width, idx / (uint32_t)rv.width, A.bitfield, ray)) continue;
                pix = idx;
                rgba[0] = rgba[1] = rgba[2] = rgba[3] = 0.f;
                depth = 0.f; maxw = 0.f; ns = 0;
            }
            if (ns < rv.max_samples_per_ray && ray_next_sample(rv, A.bitfield, ray, pos, dt)) {
                has = true;
            } else {
                // shade_kernel_nerf (:1794-1827) into a zeroed frame buffer
                if (rgba[3] > 0.001f) {
                    float o[4] = {rgba[0], rgba[1], rgba[2], rgba[3]};
                    if (!rv.linear_colors) for (int k = 0; k < 3; ++k) o[k] = srgb_to_linear(o[k]);
                    reinterpret_cast<float4*>(A.out_rgba)[pix] = make_float4(o[0], o[1], o[2], o[3]);
                    if (o[3] > 0.2f) A.out_depth[pix] = depth;
                }
                pix = -1;
            }
        }
        if (!__syncthreads_or(has ? 1 : 0)) break;

        SampleIn s;
        if (has) deform_sample(A.fr, A.dv, rv.train_min, rv.train_max, pos, ray.d, s, A.err);
        __half feat[48], sh[16];
        build_inputs(A.fv, A.extra_dims, s, has, feat, sh);
        float rgb_raw[3], dens_raw = 0.f;
        bool ok = mlp_eval(sm, w, A.plan, bf16, feat, sh, rgb_raw, dens_raw);
        if (__syncthreads_or(ok ? 0 : 1)) {
            if (threadIdx.x == 0) atomicOr(A.err, INSTA_DEVERR_TIMEOUT);
            break;
        }
        if (has) {
            ++ns;
            ++local_samples;
            // composite_kernel_nerf (:840-999)
            float T = 1.f - rgba[3];
            float dtu = unwarp_dt(warp_dt(dt));
            float alpha = 1.f - expf(-expf(dens_raw) * dtu);
            float wgt = alpha * T;
#pragma unroll
            for (int k = 0; k < 3; ++k) rgba[k] += (1.0f / (1.0f + expf(-rgb_raw[k]))) * wgt;
            rgba[3] += wgt;
            if (wgt > maxw) {
                maxw = wgt;
                V3 dp = v3(s.dpos[0] - cam_pos.x, s.dpos[1] - cam_pos.y, s.dpos[2] - cam_pos.z);
                depth = dot_rn(cam_fwd, dp);
            }
            if (rgba[3] > 1.0f - rv.min_transmittance) {
                float a = rgba[3];
                for (int k = 0; k < 4; ++k) rgba[k] /= a;
                float o[4] = {rgba[0], rgba[1], rgba[2], rgba[3]};
                if (!rv.linear_colors) for (int k = 0; k < 3; ++k) o[k] = srgb_to_linear(o[k]);
                reinterpret_cast<float4*>(A.out_rgba)[pix] = make_float4(o[0], o[1], o[2], o[3]);
                if (o[3] > 0.2f) A.out_depth[pix] = depth;
                pix = -1;
            }
        }
    }
    // warp-aggregated sample count
    for (int o = 16; o > 0; o >>= 1) local_samples += __shfl_xor_sync(0xffffffffu, local_samples, o);
    if ((threadIdx.x & 31) == 0 && local_samples) atomicAdd(A.sample_counter, local_samples);
    mlp_teardown(sm);
}

// ------------------------------------------------------------------ field eval
struct FieldArgs {
    FieldView fv;
    MlpPlan plan;
    const float* coords;
    uint32_t stride;
    int64_t n;
    float* out4;
    uint32_t* err;
};

// NerfNetwork::inference_mixed_precision_impl (NGP/nerf_network.h:159-232) on NerfCoordinate
// records: out4[i] = (r, g, b, raw density) as stored by the network (FP16 values).
__global__ void __launch_bounds__(128) field_eval_kernel(const __grid_constant__ FieldArgs A) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    MlpSmem& sm = *reinterpret_cast<MlpSmem*>(smem_raw);
    uint8_t* w = smem_raw + ((sizeof(MlpSmem) + 1023) & ~size_t(1023));
    if (!mlp_setup(sm, w, A.fv.mlp_smem, A.plan.bytes)) {
        if (threadIdx.x == 0) atomicOr(A.err, INSTA_DEVERR_TIMEOUT);
        mlp_teardown(sm);
        return;
    }
    const bool bf16 = A.fv.precision == 1;
    const int64_t n_tiles = (A.n + 127) / 128;
    for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        int64_t i = tile * 128 + threadIdx.x;
        bool valid = i < A.n;
        SampleIn s;
        if (valid) {
            const float* c = A.coords + i * A.stride;
            for (int k = 0; k < 3; ++k) { s.pos[k] = c[k]; s.dir[k] = c[8 + k]; }
            s.mask = 7u;
        }
        __half feat[48], sh[16];
        build_inputs(A.fv, valid ? A.coords + i * A.stride + A.stride - A.fv.n_extra : nullptr, s, valid, feat, sh);
        float rgb_raw[3], dens_raw = 0.f;
        bool ok = mlp_eval(sm, w, A.plan, bf16, feat, sh, rgb_raw, dens_raw);
        if (__syncthreads_or(ok ? 0 : 1)) {
            if (threadIdx.x == 0) atomicOr(A.err, INSTA_DEVERR_TIMEOUT);
            break;
        }
        if (valid) reinterpret_cast<float4*>(A.out4)[i] = make_float4(rgb_raw[0], rgb_raw[1], rgb_raw[2], dens_raw);
    }
    mlp_teardown(sm);
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
static size_t mlp_smem_bytes(const MlpPlan& plan) {
    return ((sizeof(MlpSmem) + 1023) & ~size_t(1023)) + plan.bytes;
}

int render_ctas_per_sm(const MlpPlan& plan) {
    size_t smem = mlp_smem_bytes(plan);
    cudaFuncSetAttribute(render_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, render_kernel, 128, smem) != cudaSuccess) return 1;
    // 128 TMEM columns per CTA: at most 4 resident CTAs share an SM's 512 columns.
    return n < 1 ? 1 : (n > 4 ? 4 : n);
}

cudaError_t launch_render(const RenderLaunch& L, cudaStream_t s) {
    RenderArgs a;
    a.rv = L.rv; a.fr = L.fr; a.dv = L.dv; a.fv = L.fv; a.plan = *L.plan;
    a.bitfield = L.bitfield; a.extra_dims = L.extra_dims;
    a.out_rgba = L.out_rgba; a.out_depth = L.out_depth;
    a.ray_counter = L.ray_counter; a.sample_counter = L.sample_counter; a.err = L.err;
    size_t smem = mlp_smem_bytes(*L.plan);
    cudaError_t e = cudaFuncSetAttribute(render_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(L.ray_counter, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    render_kernel<<<L.grid, 128, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_field_eval(const FieldView& fv, const MlpPlan& plan, const float* coords, uint32_t stride, int64_t n,
                              float* out4, uint32_t* err, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    FieldArgs a;
    a.fv = fv; a.plan = plan; a.coords = coords; a.stride = stride; a.n = n; a.out4 = out4; a.err = err;
    size_t smem = mlp_smem_bytes(plan);
    cudaError_t e = cudaFuncSetAttribute(field_eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t tiles = (n + 127) / 128;
    int grid = (int)(tiles < (int64_t)sms * 4 ? tiles : (int64_t)sms * 4);
    field_eval_kernel<<<grid, 128, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_march_debug(const RenderView& rv, const uint8_t* bitfield, int max_out, float* out_t, float* out_dt,
                               int32_t* out_n, cudaStream_t s) {
    uint32_t n = (uint32_t)rv.width * (uint32_t)rv.height;
    march_debug_kernel<<<(n + 127) / 128, 128, 0, s>>>(rv, bitfield, max_out, out_t, out_dt, out_n);
    return cudaGetLastError();
}

}  // namespace insta
