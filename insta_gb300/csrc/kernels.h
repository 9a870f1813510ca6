// kernels.h -- host-side launchers of the device kernels (internal to the library).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "insta_types.h"

namespace insta {

struct TriFrame;

// Tile plan of the MLP weight image (see mlp_tiles.cuh); plain data shared with the host.
struct TilePlan;

// Alive-ray list, structure of arrays (float4 each):
//   a = (origin.xyz, t)   b = (dir.xyz, max_weight)   c = rgba   d = (depth, pixel, samples so far, previous slot)
struct RayBuf {
    float4* a;
    float4* b;
    float4* c;
    float4* d;
};

// Samples of a round are regrouped by spatial cell before the deform stage (a counting sort over
// a 64^3 grid spanning the frame's mesh box, Morton-ordered cells), so the 32 samples a warp
// queries together are neighbours in space whatever rays they came from.
constexpr uint32_t kSortBits = 18, kSortBins = 1u << kSortBits, kSortBlock = 1024;
constexpr uint32_t kStepShift = 27, kRayMask = (1u << kStepShift) - 1u;

struct WaveArgs {
    RenderView rv;
    FrameView fr;
    DeformView dv;
    FieldView fv;
    const uint8_t* bitfield;
    const float* extra_dims;
    float* out_rgba;
    float* out_depth;
    RayBuf rays_in, rays_out;
    const uint32_t* n_alive_in;
    uint32_t* n_alive_out;
    uint32_t* n_round;          // samples produced this round, per alive ray
    uint32_t* sample_index;     // [steps][n_alive]: stream position of sample k of ray r
    uint32_t* sample_ray;       // per sample (march order): ray slot | step k << kStepShift
    uint32_t* sample_key;       // per sample (march order): spatial cell of the position
    uint32_t* sample_order;     // sorted position -> march-order sample
    uint32_t* sort_bins;        // kSortBins cell counters, then cursors
    uint32_t* sort_block_sums;  // per 1024 cells
    uint32_t* n_samples_round;  // device count of this round's samples
    uint32_t steps;             // samples per ray per round
    uint8_t* tiles;             // encoded input tile records
    uint32_t tile_bytes, k_in;
    float4* samples;            // per sample: (pos.xyz, dt) from the march
    float2* aux;                // per sample: (dt, depth candidate)
    const uint2* out;           // per sample: FP16 (r, g, b, density)
    const float4* out_f32;      // per sample when the MLP runs in BF16
    unsigned long long* sample_counter;
    uint32_t* err;
};

cudaError_t launch_tri_frames(int F, const float* verts, const int32_t* faces, const uint32_t* mask, const float* canon_area,
                              float* area_out, TriFrame* out, int with_inverse, cudaStream_t s);
size_t bvh_scratch_bytes(int F);
cudaError_t launch_bvh_build(const FrameView& fv, const float* verts, const int32_t* faces, void* scratch, cudaStream_t s);
cudaError_t launch_occupancy(const FrameView& fv, double radius, uint8_t* bitfield, uint32_t* err, cudaStream_t s);
cudaError_t launch_canonical_map_soa(const FrameView& fv, const DeformView& dv, const float* pts, int64_t n, int32_t* out_idx,
                                     float* out_canon, uint32_t* err, cudaStream_t s);
cudaError_t launch_canonical_map_coords(const FrameView* frames_dev, uint32_t n_frames, const DeformView& dv, float* coords,
                                        uint32_t stride, uint32_t n_extra, int64_t n, int32_t frame_id, uint32_t* err, cudaStream_t s);

cudaError_t launch_ray_init(const WaveArgs& a, cudaStream_t s);
cudaError_t launch_march(const WaveArgs& a, cudaStream_t s);
cudaError_t launch_sort_samples(const WaveArgs& a, cudaStream_t s);
cudaError_t launch_deform_encode(const WaveArgs& a, cudaStream_t s);
cudaError_t launch_composite(const WaveArgs& a, cudaStream_t s);
cudaError_t launch_encode_coords(const FieldView& fv, const float* coords, uint32_t stride, int64_t n, uint8_t* tiles,
                                 uint32_t tile_bytes, uint32_t k_in, cudaStream_t s);
cudaError_t launch_unpack(const uint2* out, const float4* out_f32, int bf16, int64_t n, float4* dst, cudaStream_t s);
// Fixed device scratch of insta_field_eval_static (static_scratch.cu); first call per device looks it up.
int64_t static_max_samples();
cudaError_t static_scratch(int device, uint8_t** tiles, uint2** out, float4** out_f32);

cudaError_t launch_march_debug(const RenderView& rv, const uint8_t* bitfield, int max_out, float* out_t, float* out_dt,
                               int32_t* out_n, cudaStream_t s);

}  // namespace insta
