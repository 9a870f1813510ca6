// kernels.h -- host-side launchers of the device kernels (internal to the library).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "insta_types.h"

namespace insta {

struct TriFrame;
struct MlpPlan;

cudaError_t launch_tri_frames(int F, const float* verts, const int32_t* faces, const uint32_t* mask, const float* canon_area,
                              float* area_out, TriFrame* out, int with_inverse, cudaStream_t s);
cudaError_t launch_bvh_build(const FrameView& fv, int n_leaves, const float* verts, const int32_t* faces, cudaStream_t s);
cudaError_t launch_occupancy(const FrameView& fv, double radius, uint8_t* bitfield, uint32_t* err, cudaStream_t s);
cudaError_t launch_canonical_map_soa(const FrameView& fv, const DeformView& dv, const float* pts, int64_t n, int32_t* out_idx,
                                     float* out_canon, uint32_t* err, cudaStream_t s);
cudaError_t launch_canonical_map_coords(const FrameView* frames_dev, uint32_t n_frames, const DeformView& dv, float* coords,
                                        uint32_t stride, uint32_t n_extra, int64_t n, int32_t frame_id, uint32_t* err, cudaStream_t s);

struct RenderLaunch {
    RenderView rv;
    FrameView fr;
    DeformView dv;
    FieldView fv;
    const MlpPlan* plan;        // host copy
    const uint8_t* bitfield;    // 8 mips
    const float* extra_dims;    // device, n_extra floats (may be null)
    float* out_rgba;            // device [H*W*4]
    float* out_depth;           // device [H*W]
    uint32_t* ray_counter;      // device, zeroed by the launcher
    unsigned long long* sample_counter;  // device, accumulated
    uint32_t* err;
    int grid;                   // persistent CTAs (0 = auto)
};

cudaError_t launch_render(const RenderLaunch& L, cudaStream_t s);
cudaError_t launch_field_eval(const FieldView& fv, const MlpPlan& plan, const float* coords, uint32_t stride, int64_t n,
                              float* out4, uint32_t* err, cudaStream_t s);
cudaError_t launch_march_debug(const RenderView& rv, const uint8_t* bitfield, int max_out, float* out_t, float* out_dt,
                               int32_t* out_n, cudaStream_t s);
int render_ctas_per_sm(const MlpPlan& plan);

}  // namespace insta
