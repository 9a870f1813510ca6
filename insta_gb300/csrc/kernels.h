// kernels.h -- host-side launchers of the device kernels (internal to the library).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "insta_types.h"

struct insta_train_loss_desc;   // include/insta_gb300.h
struct insta_training_pixels_desc;
struct insta_extra_dims_gradient_desc;

namespace insta {

struct TriFrame;

// Tile plan of the MLP weight image and the MLP launch arguments (see mlp_tiles.cuh).
struct TilePlan;
struct MlpArgs;

// Alive-ray list, structure of arrays (float4 each):
//   a = (origin.xyz, t)   b = (dir.xyz, max_weight)   c = rgba   d = (depth, pixel, samples so far, request)
struct RayBuf {
    float4* a;
    float4* b;
    float4* c;
    float4* d;
};

// One render request of a batch: its camera, its frame's BVH and triangle frames, its avatar's
// deformation data, hash table and MLP weight image, its occupancy bits and its output buffers.
// All requests of a batch share one field layout (levels, widths), so the level tables and the
// MLP tile plan come from the batch, and only the parameter pointers differ per request.
struct ReqView {
    RenderView rv;
    FrameView fr;
    DeformView dv;
    const uint16_t* table;
    const uint8_t* mlp;
    const uint8_t* bitfield;
    const float* extra;         // n_extra floats on the device, or null (zeros)
    float* out_rgba;
    float* out_depth;
    uint32_t* out_samples;      // device: samples composited per pixel, or null
    uint32_t tiles_x;           // 8x4-pixel ray tiles per image row
    uint32_t tiles;             // ray tiles of the image
};

// Samples of a round are regrouped before the deform stage by a counting sort on
// (request, spatial cell): cells are a Morton-ordered grid over each frame's mesh box, so the
// 32 samples a warp queries together belong to one frame and are neighbours in space whatever
// rays they came from.  Each request's run of samples is padded to a multiple of 128 so every
// MLP tile belongs to one request (one avatar's weights).
constexpr uint32_t kSortBlock = 1024, kMaxSortBins = 1u << 24, kMaxRequests = 4096;
constexpr uint32_t kStepShift = 25, kRayMask = (1u << kStepShift) - 1u;
constexpr uint32_t kNoSample = 0xffffffffu;

// cell bits per request (multiple of 3, >= 12) so that n_reqs << bits stays within kMaxSortBins
inline uint32_t sort_cell_bits(uint32_t n_reqs, uint32_t start = 18) {
    uint32_t b = start;
    while (b > 12 && ((uint64_t)n_reqs << b) > kMaxSortBins) b -= 3;
    return b;
}
// record and point sets (canonical map, density-grid warp): 128^3 cells where the bins allow --
// their points are spread through each cell, unlike a render's neighbouring rays
inline uint32_t map_cell_bits(uint32_t n_frames) { return sort_cell_bits(n_frames, 21); }

struct WaveArgs {
    const ReqView* reqs;        // device table, n_reqs entries (request slots)
    uint32_t n_reqs;
    // ray_init: the requests whose rays start now -- slot init_slot[k] owns ray tiles
    // [init_tile[k], init_tile[k + 1]) of this launch
    const uint32_t* init_tile;  // [n_init + 1]
    const uint32_t* init_slot;  // [n_init]
    uint32_t n_init;
    uint32_t* req_alive;        // optional [n_reqs]: alive rays per request (ray_init adds, composite subtracts)
    uint32_t cell_bits;         // sort cells per request = 2^cell_bits
    FieldView fv;               // shared field layout (table / mlp pointers unused)
    RayBuf rays_in, rays_out;
    const uint32_t* n_alive_in;
    uint32_t* n_alive_out;
    uint32_t* n_round;          // samples produced this round, per alive ray
    uint32_t* sample_index;     // [steps][n_alive]: stream position of sample k of ray r
    uint32_t* sample_ray;       // per sample (march order): ray slot | step k << kStepShift
    uint32_t* sample_key;       // per sample: the sort key (march order), then the nearest triangle (sorted order)
    uint32_t* sample_order;     // sorted (padded) position -> march-order sample, kNoSample for padding
    uint32_t* sort_bins;        // n_reqs << cell_bits counters, then cursors
    uint32_t* sort_block_sums;  // per kSortBlock bins, then their exclusive offsets
    uint32_t* req_start;        // [n_reqs + 1] unpadded start of each request's samples
    uint32_t* req_seg;          // [n_reqs + 1] padded start of each request's samples
    uint32_t* n_samples_round;  // device count of this round's samples
    uint32_t* n_samples_padded; // the same after per-request padding to 128
    uint32_t steps;             // samples per ray per round
    const uint32_t* steps_dev;  // when set: the round's step count, written on the device (graph rounds)
    uint8_t* tiles;             // encoded input tile records
    uint32_t tile_bytes, k_in;
    float4* samples;            // per sample: (pos.xyz, dt) from the march
    float* march_t;             // [step][n_alive] the t of each ray's samples of the round (march scratch)
    float2* aux;                // per sample: (dt, depth candidate)
    const uint2* out;           // per sample: FP16 (r, g, b, density)
    const float4* out_f32;      // per sample when the MLP runs in BF16
    unsigned long long* sample_counter;
    uint32_t top_nodes;         // nearest stage: top tree nodes each warp stages in shared memory (0: none)
    unsigned long long* walk_stats;  // nearest stage: walk counters (see nearest_warp), or null
    uint32_t* nearest_work;     // nearest stage: [0] next 32-sample chunk, [1] warps finished (zero between launches)
    uint32_t* err;
};

cudaError_t launch_tri_frames(int F, const float* verts, const int32_t* faces, const uint32_t* mask, const float* canon_area,
                              float* area_out, TriFrame* out, int with_inverse, cudaStream_t s);
size_t bvh_scratch_bytes(int F);
// A batch of frames of one avatar: per-triangle frames, then one LBVH build per CTA (frame i
// uses scratch + i * bvh_scratch_bytes(F)); `table` holds frame_batch_table_bytes(n) device bytes.
struct FrameJob {
    const float* verts;
    TriFrame* frames;
};
size_t frame_batch_table_bytes(int n);
cudaError_t launch_frames_batch(int n, int F, const FrameView* views, const float* const* verts, const int32_t* faces,
                                const uint32_t* mask, const float* canon_area, void* scratch, void* table, cudaStream_t s);
cudaError_t launch_bvh_build(const FrameView& fv, const float* verts, const int32_t* faces, void* scratch, cudaStream_t s);
cudaError_t launch_occupancy(const FrameView& fv, double radius, uint8_t* bitfield, uint32_t* err, cudaStream_t s);
// Float (or FP16) density grid [n_cascades][128^3] (Morton order) -> bitfield with mips.
size_t density_scratch_bytes(uint32_t n_cascades);
// density-grid maintenance (update_density_grid_nerf): samples, the random-frame warp, and the
// max splat + decay of the float grid; coords are NerfCoordinate-strided (pos 0..2, dir 8..10)
cudaError_t launch_grid_samples(uint32_t n_uniform, uint32_t n_nonuniform, uint64_t rng_state, uint64_t rng_inc, uint32_t step,
                                const float* aabb_min, const float* aabb_max, const float* grid, uint32_t n_cascades, float* coords,
                                uint32_t stride, uint32_t* indices, cudaStream_t s);
cudaError_t launch_warp_random(const FrameView* frames_dev, uint32_t n_frames, const DeformView& dv, float* coords, uint32_t stride,
                               uint32_t n, uint64_t rng_state, uint64_t rng_inc, uint32_t* err, cudaStream_t s);
// the same warp with the samples sorted by (frame, 64^3 cell of the box dom_lo..dom_hi) and the
// warp-cooperative walk (n_frames <= kMaxRequests); scratch: warp_sorted_scratch_bytes
size_t warp_sorted_scratch_bytes(uint32_t n, uint32_t n_frames);
cudaError_t launch_warp_random_sorted(const FrameView* frames_dev, uint32_t n_frames, const DeformView& dv, float* coords, uint32_t stride,
                                      uint32_t n, uint64_t rng_state, uint64_t rng_inc, const float* dom_lo, const float* dom_hi,
                                      void* scratch, uint32_t* err, cudaStream_t s);
// insta_canonical_map on many records: (frame, cell)-sorted warp walk; fixed != 0: frames_dev is
// the one frame (n_frames 1) and holder only gates; scratch: warp_sorted_scratch_bytes(n, n_frames)
cudaError_t launch_canonical_map_coords_sorted(const FrameView* frames_dev, uint32_t n_frames, int fixed, const DeformView& dv, float* coords,
                                               uint32_t stride, uint32_t n_extra, uint32_t n, void* scratch, uint32_t* err, cudaStream_t s,
                                               const uint32_t* n_dev = nullptr);   // optional device count: records past it untouched
cudaError_t launch_splat_ema(uint32_t n, const uint32_t* indices, const uint2* out, const float4* out_f32, int f32_out, float* tmp,
                             float* grid, uint32_t n_cells, float decay, cudaStream_t s);
cudaError_t launch_density_grid(const void* grid, int fp16, uint32_t n_cascades, void* scratch, uint8_t* bitfield, cudaStream_t s);
cudaError_t launch_canonical_map_soa(const FrameView& fv, const DeformView& dv, const float* pts, int64_t n, int32_t* out_idx,
                                     float* out_canon, uint32_t* err, cudaStream_t s);
// The same map for large point sets: points are first sorted by a 64^3 cell of the frame's box
// (counting sort), so that the warp-cooperative nearest walk sees 32 neighbours at a time; the
// results go back to the callers' order.  scratch: map_sorted_scratch_bytes(n) bytes.
constexpr int64_t kMapSortedMin = 1 << 16;   // below this the per-point walk is as fast
size_t map_sorted_scratch_bytes(int64_t n);
cudaError_t launch_canonical_map_sorted(const FrameView& fv, const DeformView& dv, const float* pts, int64_t n, int32_t* out_idx,
                                        float* out_canon, void* scratch, uint32_t* err, cudaStream_t s);
// n_dev (optional): a device count; records [0, min(n, *n_dev)) are mapped
cudaError_t launch_canonical_map_coords(const FrameView* frames_dev, uint32_t n_frames, const DeformView& dv, float* coords,
                                        uint32_t stride, uint32_t n_extra, int64_t n, int32_t frame_id, uint32_t* err, cudaStream_t s,
                                        const uint32_t* n_dev = nullptr);

cudaError_t launch_ray_init(const WaveArgs& a, uint32_t total_tiles, cudaStream_t s);
cudaError_t launch_march(const WaveArgs& a, cudaStream_t s);
cudaError_t launch_sort_samples(const WaveArgs& a, cudaStream_t s);
cudaError_t launch_deform_encode(const WaveArgs& a, uint32_t blocks_per_sm, cudaStream_t s);
cudaError_t launch_nearest_stage(const WaveArgs& a, uint32_t blocks_per_sm, cudaStream_t s);
cudaError_t launch_map_encode(const WaveArgs& a, uint32_t blocks_per_sm, cudaStream_t s);
// deform + encode + MLP in one kernel after launch_nearest_stage (FP16 / BF16 fields)
cudaError_t launch_field_fused(const WaveArgs& a, const MlpArgs& m, uint32_t max_tiles, cudaStream_t s, uint32_t ctas_per_sm);
cudaError_t launch_composite(const WaveArgs& a, cudaStream_t s);
// generate_training_samples_nerf on caller-supplied rays (see insta_training_samples).
struct TrainArgs {
    const float* rays;          // [n][6] origin, unnormalised direction
    const uint32_t* image;      // [n] training image (= deformed frame id), written to `holder`
    const float* start_rand;    // [n] uniform draw of the start jitter
    const float* extra;         // [n_images][n_extra] or null
    uint32_t n_extra, n_images;
    int64_t n_rays;
    float aabb_min[3], aabb_max[3];
    float cone_angle;
    uint32_t max_samples;
    const uint8_t* bitfield;
    float* coords;              // [max_samples][stride]
    uint32_t stride;
    uint32_t* ray_indices;      // [n]
    uint32_t* numsteps;         // [n][2] (count, base)
    uint32_t* counters;         // [2] rays kept, samples requested
};
// tbuf (optional, [n_rays][1024] floats): the march runs once and a warp per kept ray writes the records
cudaError_t launch_training_samples(const TrainArgs& a, float* tbuf, cudaStream_t s);
constexpr int64_t kTrainMarchOnceMaxRays = 1 << 16;   // larger batches march twice (no per-ray buffer)

// extra_ones: every expression dim 1 instead of the records' last n_extra floats (the density-grid
// update's density evaluation)
cudaError_t launch_encode_coords(const FieldView& fv, const float* coords, uint32_t stride, int64_t n, uint8_t* tiles,
                                 uint32_t tile_bytes, uint32_t k_in, cudaStream_t s, bool extra_ones = false);
cudaError_t launch_unpack(const uint2* out, const float4* out_f32, int bf16, int64_t n, float4* dst, cudaStream_t s);
// Fixed device scratch of insta_field_eval_static (static_scratch.cu); first call per device looks it up.
int64_t static_max_samples();
cudaError_t static_scratch(int device, uint8_t** tiles, uint2** out, float4** out_f32);

// Device-driven rounds for the CUDA-graph render loop: round_begin sets a round's step count from
// its alive count and clears the counters it appends to; round_end (after the body's rounds) counts them
// and sets the loop's condition: rays alive and rounds left.
cudaError_t launch_round_begin(const uint32_t* n_alive_in, uint32_t* n_alive_out, uint32_t* n_samples_round, uint32_t* steps,
                               uint64_t round_cap, uint32_t max_steps, cudaStream_t s);
// Between the two rounds of the loop body: the second round's IF condition (rays left alive by
// the first), and b_ran for round_end's count; clears the second round's output count when it is
// skipped.
cudaError_t launch_round_mid(const uint32_t* a_alive_out, uint32_t* b_alive_out, uint32_t* b_ran, cudaGraphConditionalHandle c,
                             cudaStream_t s);
cudaError_t launch_round_end(const uint32_t* n_alive, uint32_t* rounds, const uint32_t* b_ran, unsigned long long* rounds_total,
                             uint32_t max_rounds, cudaGraphConditionalHandle cond, cudaStream_t s);
// The field's training side (train_kernels.cu): forward with saved activations, output
// gradients -> parameter gradients (FP32, snapshot order), Adam.
struct TrainShape {
    uint32_t kd;                 // density MLP input width (32 + expression dims)
    int n_density, n_rgb;        // layers of each MLP
    uint64_t layer_off[8];       // offsets of the layers' [n_out][n_in] weights in the parameters
    uint64_t table_off;          // offset of the hash table ([entries][2])
};
size_t train_scratch_floats(const TrainShape& t, uint32_t n);

// The layer products of training on tcgen05 (train_mlp.cu).  Layers in parameter order: the
// density MLP (hidden layers, then its 16 outputs), then the colour MLP (hidden layers, then its
// 16 padded outputs).
struct TrainMlpLayer {
    uint32_t n_out, n_in, k_pad;   // forward N, input width, forward K (n_in rounded to 16)
    uint64_t w_off;                // the layer's [n_out][n_in] weights in the parameters
    uint32_t fwd_img;              // image offset of the forward B tile (N = n_out, K = k_pad)
    uint32_t bwd_img, bwd_n;       // image offset of W^T (N = bwd_n, K = n_out) for dX
    uint32_t dw_col;               // TMEM column of the weight-gradient accumulator (n_out columns)
    uint32_t n_out_real;           // output rows that carry gradient (3 for the colour output)
};
// Shared memory: the weight images, then per tile slot (two) the density input [128][kd], the
// colour input [128][32], the kept hidden outputs [128][64] and dY [128][64], then a tail that
// the MN-major weight-gradient operands may read past the last tile without leaving the block's
// shared memory.
struct TrainMlpPlan {
    TrainMlpLayer layer[8];
    uint32_t n_density, n_rgb, kd;
    uint32_t img_bytes;
    uint32_t s_img, s_x[2], s_rin[2], s_kept[2][6], s_dy[2], smem_bytes;
};
struct TrainMlpArgs {
    TrainMlpPlan plan;
    const uint8_t* images;   // the weight images (device), img_bytes
    const float* xd;         // [n][kd] encoding
    const float* xr;         // [n][32]: columns 16..31 SH
    const float* dl_dout;    // [n][4] or null (forward only)
    float* out4;             // [n][4] or null
    float* dxd;              // [n][kd] dL/d encoding
    float* grad;             // parameter gradients (added to)
    uint32_t n;
    uint32_t* err;
};
struct TrainImageTile {
    uint32_t dst, n, k;                      // N x K FP16 tile at image byte offset dst
    uint64_t w_off;
    uint32_t rows, cols, row0, col0, transpose;
};
struct TrainImageList {
    TrainImageTile tile[17];
    uint32_t n_tiles;
};
cudaError_t launch_train_mlp(const TrainMlpArgs& a, const TrainImageList& images, const float* w32, uint8_t* img_dev, cudaStream_t s);
// insta_field_backward with INSTA_TRAIN_MATH_TCGEN05: encode (FP32 master table), the tcgen05 layer
// products, then the hash-table backward; scratch (2 kd + 32) n floats.
cudaError_t launch_field_train_tc(const FieldView& fv, const TrainShape& t, const TrainMlpPlan& plan, const TrainImageList& images,
                                  uint8_t* img_dev, const float* w32, const float* coords, uint32_t stride, uint32_t n,
                                  const float* dl_dout, float* out4, float* grad, float* scratch, uint32_t* err, cudaStream_t s,
                                  float* dl_dextra = nullptr);
cudaError_t launch_field_train(struct cublasContext* h, const FieldView& fv, const TrainShape& t, const float* w32, const float* coords,
                               uint32_t stride, uint32_t n, const float* dl_dout, float* out4, float* grad, float* scratch,
                               cudaStream_t s, float* dl_dextra = nullptr);
cudaError_t launch_extra_dims_gradient(const ::insta_extra_dims_gradient_desc& d, cudaStream_t s);
cudaError_t launch_adam(size_t n, size_t n_matrix, float* w, float* m, float* v, uint32_t* table_steps, const float* g, float loss_scale,
                        float lr, float b1, float b2, float eps, float l2, uint32_t step, float* ema, float decay, uint32_t ema_step,
                        __half* w16, __half* w16_train, cudaStream_t s);
cudaError_t launch_half_to_float(size_t n, const void* a, float* b, cudaStream_t s);
cudaError_t launch_train_loss(const ::insta_train_loss_desc& d, uint32_t* base_scratch, cudaStream_t s);
cudaError_t launch_training_pixels(const ::insta_training_pixels_desc& d, cudaStream_t s);
cudaError_t launch_error_map_cdf(const float* em, uint32_t n_images, uint32_t w, uint32_t h, float* cdf_x, float* cdf_y, float* cdf_img,
                                 float* pmf_img, cudaStream_t s);
cudaError_t launch_raycast(const RenderView& rv, const FrameView& fr, const float* center, int color_normal, float* out_rgba,
                           float* out_depth, int32_t* out_tri, uint32_t* err, cudaStream_t s);
cudaError_t launch_nearest_debug(const FrameView& fr, const float* pts, int64_t n, int32_t* out, uint32_t* err, cudaStream_t s);
cudaError_t launch_march_debug(const RenderView& rv, const uint8_t* bitfield, int max_out, float* out_t, float* out_dt,
                               int32_t* out_n, cudaStream_t s);

}  // namespace insta
