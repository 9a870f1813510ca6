/*
 * insta_gb300.h -- C ABI of the GB300-native INSTA deformation + render hot path.
 *
 * Plain C types only (no CUDA, Eigen or torch types).  Every function returns an
 * int status (INSTA_OK on success) and never throws; insta_last_error() gives the
 * message of the last failure on a context.  A context is bound to one CUDA
 * device and one stream; it is thread-compatible, not thread-safe (one host thread
 * per context at a time).
 *
 * Reference interfaces these entry points replace (INSTA repository paths;
 * "NGP/" = instant-ngp/include/neural-graphics-primitives/):
 *   insta_canonical_set         rta::TinyMesh ctor for the canonical mesh + rta::Core::load_meshes
 *                               adjacency and render box (src/tiny_mesh.cu:39-51,134-164,316-371;
 *                               src/core.cu:283-304)
 *   insta_frame_upload          rta::TinyMesh ctor for a tracked frame + BVH build and the GPU
 *                               pointer tables (src/tiny_mesh.cu:39-51,166-178;
 *                               instant-ngp/src/triangle_bvh.cu:548-631; src/core.cu:309-334)
 *   insta_occupancy_from_mesh   mark_flame_density_grid + update_density_grid_mean_and_bitfield
 *                               (instant-ngp/src/testbed_nerf.cu:364-389,2863-2878)
 *   insta_density_grid_update   update_density_grid_nerf + warp_random_samples (instant-ngp/src/
 *                               testbed_nerf.cu:487-583,2774-2861; src/core.cu:528-579)
 *   insta_density_grid_load     the snapshot's density grid -> bitfield (grid_to_bitfield +
 *                               bitfield_max_pool, instant-ngp/src/testbed_nerf.cu:585-632)
 *   insta_canonical_map         rta::Core::surface_closest_point / render_deformed -> `warp`
 *                               (src/core.cu:339-348,442-526,581-637)
 *   insta_canonical_map_soa     the same map on bare points (index + canonical xyz)
 *   insta_training_samples      generate_training_samples_nerf + warp (instant-ngp/src/
 *                               testbed_nerf.cu:1105-1285,3290)
 *   insta_params_load           Testbed::load_snapshot parameter blob, NerfNetwork::set_params
 *                               order (instant-ngp/src/testbed.cu:2952-3016; NGP/nerf_network.h:492-525)
 *   insta_field_eval            NerfNetwork::inference_mixed_precision_impl (NGP/nerf_network.h:159-232)
 *   insta_field_eval_training   the same with the training weights (use_inference_params = false)
 *   insta_field_backward        NerfNetwork's forward/backward for training (NGP/nerf_network.h:296-383)
 *   insta_field_backward_ex     the same, also returning the expression-dim input gradients
 *                               (instant-ngp/src/testbed_nerf.cu:3364-3380)
 *   insta_extra_dims_gradient   compute_extra_dims_gradient_train_nerf (instant-ngp/src/testbed_nerf.cu:1756-1791)
 *   insta_adam_step             the Adam optimizer of the trainer (configs/nerf/main.json)
 *   insta_train_set_math        FP32, TF32 or the library's tcgen05 layer products of the backward
 *   insta_train_loss            compute_loss_kernel_train_nerf (with the error map) + fill_rollover
 *                               (instant-ngp/src/testbed_nerf.cu:1305-1644,3298-3362)
 *   insta_training_pixels       image_idx + nerf_random_image_pos_training + the background draw of
 *                               generate_training_samples_nerf (instant-ngp/src/testbed_nerf.cu:1013-1105,1140-1144)
 *   insta_error_map_cdf         construct_cdf_2d / construct_cdf_1d + the image CDF of train_nerf_step
 *                               (instant-ngp/src/testbed_nerf.cu:1967-2020,3010-3041)
 *   insta_render                Testbed::render_nerf -> NerfTracer::init_rays_from_camera/trace +
 *                               shade_kernel_nerf (instant-ngp/src/testbed_nerf.cu:2030-2244,2320-2460)
 *   insta_march_debug           the sample positions advance_pos_nerf + generate_next_nerf_network_inputs
 *                               emit per ray (instant-ngp/src/testbed_nerf.cu:634-686,722-795)
 *   insta_raycast               rta::Core::raycast_flame -> SphereTracer::trace_bvh + shade_kernel_sdf
 *                               (src/core.cu:74-113,350-402; instant-ngp/src/testbed_sdf.cu:505-577,650-665)
 *   insta_nearest_debug         the render path's warp-cooperative closest_triangle on given points
 *                               (NGP/bvh.cuh:48-96 as called by the warp kernel, src/core.cu:470-478)
 */
#ifndef INSTA_GB300_H
#define INSTA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define INSTA_OK 0
#define INSTA_ERR_INVALID_ARG 1   /* bad pointer, size or index                           */
#define INSTA_ERR_CUDA 2          /* a CUDA runtime call failed                           */
#define INSTA_ERR_BUDGET 3        /* the context's device-memory budget would be exceeded */
#define INSTA_ERR_NOT_READY 4     /* canonical mesh, frame or parameters missing          */
#define INSTA_ERR_UNSUPPORTED 5   /* shape outside what the kernels implement             */
#define INSTA_ERR_DEVICE 6        /* a kernel reported an error (stack overflow, timeout) */

#define INSTA_PRECISION_FP16 0
#define INSTA_PRECISION_BF16 1
#define INSTA_PRECISION_FP8 2            /* MLPs in E4M3: per-layer weight scale, per-row activation scale, FP32 accumulate */

#define INSTA_FLAG_DISABLE_INTERP 0x1u   /* "disable_interp" (src/core.cu:201,495) */

typedef struct insta_ctx insta_ctx;

/* Hash grid + MLP shapes (configs/nerf/main.json keys).  per_level_scale <= 0 derives
 * it as exp(log(2048 * aabb_scale / base_resolution) / (n_levels - 1))
 * (instant-ngp/src/testbed.cu:2253-2258). */
typedef struct {
    uint32_t n_levels;              /* 16 */
    uint32_t n_features_per_level;  /* 2 (the benchmark field), 4 or 8 (INSTA's configs/nerf/main.json);
                                       n_levels x n_features_per_level a multiple of 8 in 16..128 */
    uint32_t log2_hashmap_size;     /* 19 */
    uint32_t base_resolution;       /* 16 */
    float per_level_scale;          /* 0 -> derived */
    uint32_t aabb_scale;            /* 2 */
    uint32_t n_extra_dims;          /* expression dims appended to the density input (0 or 16) */
    uint32_t density_neurons;       /* 64 */
    uint32_t density_hidden_layers; /* 1 */
    uint32_t density_output_dims;   /* 16 */
    uint32_t rgb_neurons;           /* 64 */
    uint32_t rgb_hidden_layers;     /* 2 */
    uint32_t precision;             /* INSTA_PRECISION_* */
} insta_field_desc;

/* One headless render request (Testbed::render_nerf arguments plus the avatar/frame). */
typedef struct {
    int32_t avatar;
    int32_t frame;                  /* deformed frame (m_target_deform_frame) */
    int32_t width, height;
    float focal_length[2];          /* pixels */
    float screen_center[2];         /* 0.5, 0.5 */
    float camera[12];               /* 3x4 row-major [R | origin]; columns right, down, forward */
    float cone_angle;               /* cone_angle_constant: 0 constant steps, 1/256 exponential */
    float min_transmittance;        /* rendering_min_transmittance (0.01) */
    uint32_t spp;                   /* sample index for the jitter sequence */
    uint32_t snap_to_pixel_centers; /* 1 (reference default) */
    uint32_t max_samples_per_ray;   /* 1024 */
    uint32_t linear_colors;         /* 0: shade converts sRGB -> linear */
    const float* extra_dims;        /* host, n_extra_dims floats, or NULL (zeros) */
    uint32_t* out_samples;          /* device u32[h*w] or NULL: samples composited into each pixel
                                       (the ray's NerfPayload::n_steps when it finished) */
} insta_render_desc;

/* Pipeline stages timed by insta_stats (CUDA events on the context's stream). */
#define INSTA_STAGE_FRAME 0          /* per-frame triangle frames + LBVH build   */
#define INSTA_STAGE_OCCUPANCY 1      /* occupancy bitfield from the mesh         */
#define INSTA_STAGE_RAY_INIT 2
#define INSTA_STAGE_MARCH 3
#define INSTA_STAGE_DEFORM_ENCODE 4  /* canonical map + hash encode + SH (after NEAREST) */
#define INSTA_STAGE_MLP 5            /* density + colour MLPs (tensor cores)     */
#define INSTA_STAGE_COMPOSITE 6
#define INSTA_STAGE_CANONICAL_MAP 7  /* insta_canonical_map / _soa               */
#define INSTA_STAGE_FIELD 8          /* insta_field_eval / _static               */
#define INSTA_STAGE_SORT 9           /* regrouping a round's samples by (request, cell) */
#define INSTA_STAGE_RAYCAST 10       /* insta_raycast                            */
#define INSTA_STAGE_TRAIN 11         /* insta_train_loss, field_backward, adam   */
#define INSTA_STAGE_NEAREST 12       /* the render's nearest-triangle walk, before DEFORM_ENCODE */
#define INSTA_STAGE_COUNT 13

typedef struct {
    uint64_t kernel_launches;        /* kernels the library launched */
    uint64_t last_render_samples;    /* network samples of the last insta_render */
    float stage_ms[INSTA_STAGE_COUNT];
    uint32_t stage_calls[INSTA_STAGE_COUNT];
    /* render nearest-triangle walk, counted while stage timing is on (per 32-sample warp walk):
       walks, inner nodes visited, leaves visited, bounding-disk tests, exact triangle tests */
    uint64_t walk_warps, walk_inner_nodes, walk_leaves, walk_bound_tests, walk_exact_tests;
} insta_stats;

/* -- context ---------------------------------------------------------------- */
int insta_ctx_create(int device, void* cuda_stream, uint64_t budget_bytes, insta_ctx** out);
int insta_ctx_destroy(insta_ctx* ctx);
const char* insta_last_error(const insta_ctx* ctx);
int insta_sync(insta_ctx* ctx);
int insta_memory_used(const insta_ctx* ctx, uint64_t* bytes);
/* Statistics: kernel launch count always; per-stage GPU time when stage timing is enabled. */
int insta_stats_enable(insta_ctx* ctx, int stage_timing);
int insta_stats_read(insta_ctx* ctx, insta_stats* out, int reset);

/* -- avatar geometry --------------------------------------------------------- */
/* verts f32[n_verts*3], faces i32[n_faces*3], mask u32[n_faces] (region ids, NULL = 15);
 * host or device pointers.  Builds adjacency, canonical frames and the render box
 * (mesh AABB inflated by 0.15 x its diagonal).  n_faces <= 16384. */
int insta_canonical_set(insta_ctx* ctx, int avatar, const float* verts, int n_verts, const int32_t* faces, int n_faces,
                        const uint32_t* mask);
/* Train box (Testbed::m_aabb, unit cube by default) and render box; NULL keeps a value. */
int insta_avatar_set_boxes(insta_ctx* ctx, int avatar, const float* train_min, const float* train_max,
                           const float* render_min, const float* render_max);
int insta_avatar_set_flags(insta_ctx* ctx, int avatar, uint32_t flags);
/* Per-frame tracked mesh (same topology): f32[n_verts*3], host or device pointer. */
int insta_frame_upload(insta_ctx* ctx, int avatar, int frame, const float* verts);
/* n frames of one avatar at once (frame ids unique, verts[i] host or device f32[n_verts*3]):
 * the per-triangle frames of all of them in one launch and one LBVH build per CTA, so a batch
 * of expressions builds in about the time of one.  Same result as n insta_frame_upload calls. */
int insta_frame_upload_batch(insta_ctx* ctx, int avatar, const int32_t* frames, int n, const float* const* verts);
/* The same upload (and, with occupancy_radius > 0, insta_occupancy_from_mesh) enqueued on a second
 * stream of the context and returned at once: it starts after the work already queued on the
 * context's stream and runs concurrently with later work; every later call that reads the frame
 * waits for it.  Double-buffered frames (upload frame k+1 while frame k renders) overlap the
 * LBVH build with rendering.  Host verts must stay unchanged until that later call when they
 * are in pinned memory (pageable memory is copied before the call returns).  Its kernels are
 * counted in insta_stats but not timed. */
int insta_frame_upload_async(insta_ctx* ctx, int avatar, int frame, const float* verts, double occupancy_radius);
/* Order the context's stream after the frame's pending asynchronous upload (no host wait). */
int insta_frame_wait(insta_ctx* ctx, int avatar, int frame);
int insta_frame_release(insta_ctx* ctx, int avatar, int frame);

/* -- occupancy ---------------------------------------------------------------- */
/* Cells (128^3, mip 0 over the unit cube) whose centre lies within `radius` of the frame's
 * surface (nearest triangle not in region 0) become occupied; mips 1..7 are max-pooled. */
int insta_occupancy_from_mesh(insta_ctx* ctx, int avatar, int frame, double radius);
/* 8 mips x 128^3 bits (2 MiB), Morton order per mip; host or device pointer. */
int insta_occupancy_set(insta_ctx* ctx, int avatar, int frame, const uint8_t* bits);
int insta_occupancy_get(insta_ctx* ctx, int avatar, int frame, uint8_t* bits);
/* A snapshot's density grid (density_grid_binary: n_cascades x 128^3 values, Morton order per
 * cascade; FP16 when fp16 != 0, else FP32; host or device) -> the frame's bitfield:
 * threshold min(0.01, mean of max(v, 0) over cascade 0), then the mip max-pool
 * (update_density_grid_mean_and_bitfield, instant-ngp/src/testbed_nerf.cu:585-632,2863-2878). */
int insta_density_grid_load(insta_ctx* ctx, int avatar, int frame, const void* grid, uint32_t n_cascades, int fp16);

/* -- density-grid maintenance ------------------------------------------------------ */
/* The PCG32 generator state (the pcg32 of tiny-cuda-nn, ngp's default_rng_t). */
typedef struct insta_pcg32 {
    uint64_t state, inc;
} insta_pcg32;

/* One update_density_grid_nerf step (instant-ngp/src/testbed_nerf.cu:2774-2861) with INSTA's
 * surface_closest_point hook on the sample positions (warp_random_samples, src/core.cu:528-579):
 * n_uniform samples over all cells and n_nonuniform over cells above the minimum optical
 * thickness, each warped to the canonical space through a random one of frames 0..n_frames-1
 * (the reference's m_meshes.size() - 1), density network at the canonical position (a field
 * with expression dims gets 1 in each of them, as NerfNetwork::density feeds them,
 * NGP/nerf_network.h:107-127,401-410), max splat into a fresh grid, then grid = max(grid * decay, new) (negative cells kept) and, for
 * bitfield_frame >= 0, that frame's bitfield (update_density_grid_mean_and_bitfield).
 * training_prep_nerf (:3427-3444) calls it with 128^3 * n_cascades uniform samples for the
 * first 256 steps, then 128^3 / 4 * n_cascades of each kind. */
typedef struct insta_density_update_desc {
    float decay;                      /* density_grid_decay (0.95)                            */
    uint32_t n_uniform, n_nonuniform;
    uint32_t n_cascades;              /* the grid's cascades (max_cascade + 1)                */
    float aabb_min[3], aabb_max[3];   /* Testbed::m_aabb: warp_position's box                 */
    insta_pcg32 grid_rng;             /* density_grid_rng; on return advanced by 2^32 as the
                                         reference's density_grid_rng.advance()              */
    insta_pcg32 warp_rng;             /* the warp's generator (m_random_generator), read only */
    uint32_t ema_step;                /* density_grid_ema_step; incremented on return         */
    int n_frames;                     /* frames 0 .. n_frames - 1 (all uploaded)              */
    int bitfield_frame;               /* frame receiving the new bitfield, or -1              */
    float* debug_pos;                 /* optional device [n][3]: the warped sample positions  */
    uint32_t* debug_idx;              /* optional device [n]: each sample's cell index        */
} insta_density_update_desc;

/* The avatar's float density grid (n_cascades x 128^3, Morton order; host or device pointer,
 * NULL = zeros; cells below zero are never updated, as mark_untrained_density_grid leaves them). */
int insta_density_grid_reset(insta_ctx* ctx, int avatar, const float* grid, uint32_t n_cascades);
int insta_density_grid_update(insta_ctx* ctx, int avatar, insta_density_update_desc* desc);
/* Copy the float grid out (host or device pointer, n_cascades x 128^3 floats; synchronises). */
int insta_density_grid_read(insta_ctx* ctx, int avatar, float* out);

/* -- deformation -------------------------------------------------------------- */
/* In place on NerfCoordinate records (device pointer, stride floats each: pos[3] dt holder
 * deformed_pos[3] dir[3] extra[n_extra]).  frame >= 0 maps every record with that frame
 * (render_deformed); frame < 0 takes the frame from `holder` (surface_closest_point). */
int insta_canonical_map(insta_ctx* ctx, int avatar, int frame, float* coords, uint32_t stride, uint32_t n_extra, int64_t n);
/* Bare points (device pointers): nearest triangle id (-1 when none) and canonical xyz. */
int insta_canonical_map_soa(insta_ctx* ctx, int avatar, int frame, const float* pts, int64_t n, int32_t* out_idx,
                            float* out_canon);

/* -- training samples ------------------------------------------------------------ */
/* The training-sample entry (generate_training_samples_nerf, instant-ngp/src/testbed_nerf.cu:
 * 1105-1285, then the warp with per-record frames, :3290 -> src/core.cu:339-348) for rays the
 * caller drew: rays f32[n][6] (origin, unnormalised direction), image u32[n] (training image =
 * uploaded frame id, written to `holder`), start_rand f32[n] (uniform [0,1) jitter draws),
 * extra f32[n_images][stride - 11] or NULL.  Marches the train box through grid_frame's
 * occupancy (<= 1024 steps per ray), reserves each ray's block of NerfCoordinate records
 * (stride floats) atomically, and maps them to canonical space in place.  ray_indices[k] and
 * numsteps[k] = (count, base) describe kept ray k; counters = (rays kept, samples requested);
 * blocks past max_samples are dropped as in the reference.  All pointers are device pointers;
 * asynchronous on the context's stream. */
int insta_training_samples(insta_ctx* ctx, int avatar, int grid_frame, const float* rays, const uint32_t* image,
                           const float* start_rand, const float* extra, uint32_t n_images, int64_t n_rays, float cone_angle,
                           uint32_t max_samples, float* coords, uint32_t stride, uint32_t* ray_indices, uint32_t* numsteps,
                           uint32_t* counters);

/* -- field -------------------------------------------------------------------- */
/* FP16 parameter blob in snapshot order (density MLP, rgb MLP, hash table); host or
 * device pointer.  n_params must equal insta_field_param_count(desc). */
int insta_field_param_count(const insta_field_desc* desc, uint64_t* n_params);
int insta_params_load(insta_ctx* ctx, int avatar, const insta_field_desc* desc, const uint16_t* params, uint64_t n_params);
/* out4[n][4] = (r, g, b, raw density) network outputs (device pointers). */
int insta_field_eval(insta_ctx* ctx, int avatar, const float* coords, uint32_t stride, int64_t n, float* out4);
/* The same evaluation with the training weights (inference_mixed_precision with
 * use_inference_params = false, ngp/src/testbed_nerf.cu:3295): differs from insta_field_eval only
 * while insta_adam_step runs with an Ema, whose average is then the field's parameters. */
int insta_field_eval_training(insta_ctx* ctx, int avatar, const float* coords, uint32_t stride, int64_t n, float* out4);

/* Same result as insta_field_eval, but the call allocates no device memory.  No counterpart
 * in the reference: it exists for callers that must not allocate on the hot path -- code that
 * records the work into a CUDA graph, real-time render callbacks with a fixed memory budget, or
 * hosts that own every device allocation through their own pool.  Its working memory is a
 * fixed array inside the library (about 2.5 MB on every GPU that loads the library, held until
 * the process exits), so at most 16384 samples per call; larger n returns
 * INSTA_ERR_INVALID_ARG.  The first call on a device looks the array up (make that call before
 * any stream capture).  All calls share the array: calls whose work overlaps on the GPU (other
 * streams, other contexts) race, so serialise them. */
int insta_field_eval_static(insta_ctx* ctx, int avatar, const float* coords, uint32_t stride, int64_t n, float* out4);

/* -- training side of the field ----------------------------------------------- */
/* NerfNetwork's backward (NGP/nerf_network.h:296-383, the tiny-cuda-nn side of train_nerf_step):
 * for n NerfCoordinate records (canonical position, direction, expression dims; device
 * pointers) and the loss gradient w.r.t. each record's outputs dl_dout f32[n][4] (raw r, g, b,
 * raw density), ADD the gradient of every parameter to grad f32[n_params] (snapshot order:
 * density MLP, colour MLP, hash table; 8-byte aligned).  On the FP32 master weights (the FP16
 * parameters widened at the first call after insta_params_load); the layer products in the
 * arithmetic insta_train_set_math selects (FP32 by default).
 * out4 (optional) gets the outputs of that FP32 forward; with dl_dout = grad = NULL only the
 * forward runs.  n < 2^24. */
int insta_field_backward(insta_ctx* ctx, int avatar, const float* coords, uint32_t stride, int64_t n, const float* dl_dout, float* grad,
                         float* out4);
/* insta_field_backward that also writes the gradient w.r.t. each record's expression dims,
 * dl_dextra f32[n][n_extra_dims] (NULL = none): the extra-dims part of the input gradient
 * NerfNetwork's backward returns when train_nerf_step prepares input gradients
 * (instant-ngp/src/testbed_nerf.cu:3364-3380).  Needs dl_dout and grad. */
int insta_field_backward_ex(insta_ctx* ctx, int avatar, const float* coords, uint32_t stride, int64_t n, const float* dl_dout,
                            float* grad, float* out4, float* dl_dextra);

/* compute_extra_dims_gradient_train_nerf (instant-ngp/src/testbed_nerf.cu:1756-1791): every kept
 * ray's compacted samples' expression-dim gradients summed into its training image's row of
 * extra_dims_gradient.  Each ray's samples are summed first, then added to the image's row
 * (the reference adds sample by sample; the sums differ by rounding only). */
typedef struct insta_extra_dims_gradient_desc {
    uint32_t max_rays;                /* size of the ray arrays                                     */
    uint32_t n_extra_dims;
    uint32_t n_images;
    const uint32_t* rays_counter;     /* rays kept (counters[0])                                    */
    const uint32_t* ray_indices;
    const uint32_t* numsteps;         /* [max_rays][2] compacted (count, base) as insta_train_loss leaves them */
    const uint32_t* image_index;      /* per original ray                                           */
    const float* dl_dextra;           /* f32[compacted samples][n_extra_dims] (insta_field_backward_ex) */
    float* extra_dims_gradient;       /* f32[n_images][n_extra_dims], added to                      */
} insta_extra_dims_gradient_desc;
int insta_extra_dims_gradient(insta_ctx* ctx, const insta_extra_dims_gradient_desc* desc);
/* Arithmetic of the backward's layer products: FP32 (default) or TF32 tensor-core GEMMs (inputs
 * rounded to TF32, FP32 accumulation; still finer than the reference's FP16 training arithmetic). */
#define INSTA_TRAIN_MATH_FP32 0
#define INSTA_TRAIN_MATH_TF32 1
/* The library's own tcgen05 kernel: per 128-sample tile the forward (activations kept in shared
 * memory) and the backward (input and weight gradients) as FP16 tensor-core products with FP32
 * accumulation -- the arithmetic class of tiny-cuda-nn's FP16 fully fused MLP training. */
#define INSTA_TRAIN_MATH_TCGEN05 2
int insta_train_set_math(insta_ctx* ctx, int math);
/* Adam (configs/nerf/main.json nests it in an Ema), as tiny-cuda-nn's Adam steps it: the gradient
 * is divided by loss_scale first (LOSS_SCALE, 128 in train_nerf_step); the MLP weights get
 * g + l2_reg * w and step every call; hash-table entries get no L2 term, and an entry whose
 * gradient is exactly zero is skipped (weights, moments and its own step count unchanged);
 * w -= lr sqrt(1 - beta2^t) / (1 - beta1^t) * m / (sqrt(v) + eps), t the parameter's step count.
 * The FP32 master weights, moments and table step counts stay on the device; the field's FP16
 * parameters and weight image are rewritten.  ema_decay > 0 adds the Ema wrapper: a
 * bias-corrected exponential average of the weights,
 * e_t = (decay (1 - decay^(t-1)) e_(t-1) + (1 - decay) w_t) / (1 - decay^t), becomes the field's
 * parameters (what rendering and insta_field_eval read), while the training forward of
 * insta_field_backward keeps reading the raw master weights. */
typedef struct insta_adam_config {
    float learning_rate, beta1, beta2, epsilon, l2_reg;
    float ema_decay;    /* 0: no Ema; configs/nerf/main.json: 0.95 */
    float loss_scale;   /* factor the gradients carry (128 from insta_train_loss's LOSS_SCALE); 0 reads as 1 */
} insta_adam_config;
int insta_adam_step(insta_ctx* ctx, int avatar, const float* grad, const insta_adam_config* cfg);

/* Training loss: compute_loss_kernel_train_nerf (instant-ngp/src/testbed_nerf.cu:1305-1644) for
 * the rays of insta_training_samples, then tiny-cuda-nn's fill_rollover(_and_rescale) as
 * train_nerf_step runs them (:3298-3362).  Per kept ray k: composite the raw network outputs of
 * its samples (logistic rgb, exponential density, stop below transmittance 1e-4), add the
 * background when the ray ran to its end, take the loss against the ray's target, reserve the
 * ray's compacted block (atomic on numsteps_counter, cut at max_samples_compacted), rewrite
 * numsteps[k] = (compacted count, compacted base), copy the block's records to coords_out and
 * write dL/d(raw output) f32[4] per compacted sample (colour, density, depth and beta terms, the
 * density regularisers).  With target_batch_size > 0 the compacted arrays are then filled to
 * target_batch_size by repeating them, the repeated gradients scaled by compacted / target.
 * Loss types use the reference's ELossType numbering. */
#define INSTA_LOSS_L2 0
#define INSTA_LOSS_L1 1
#define INSTA_LOSS_MAPE 2
#define INSTA_LOSS_SMAPE 3
#define INSTA_LOSS_HUBER 4
#define INSTA_LOSS_LOG_L1 5
#define INSTA_LOSS_RELATIVE_L2 6
typedef struct insta_train_loss_desc {
    uint32_t n_rays;                  /* rays per batch: losses and gradients are divided by it   */
    uint32_t max_rays;                /* size of the ray arrays below (the sample call's n)       */
    uint32_t max_samples_compacted;   /* capacity of coords_out / dloss_doutput                    */
    uint32_t target_batch_size;       /* 0 = no rollover, else <= max_samples_compacted           */
    float aabb_min[3], aabb_max[3];   /* the train box (unwarp_position)                          */
    int32_t loss_type, depth_loss_type;
    int32_t srgb_targets;             /* EColorSpace::SRGB (1) or Linear (0)                      */
    int32_t train_in_linear_colors;
    float loss_scale;                 /* LOSS_SCALE, 128 in the reference                          */
    float depth_supervision_lambda, seg_mask_supervision_lambda, near_distance, beta;
    int32_t penalize_density;
    uint32_t stride;                  /* floats per NerfCoordinate record                          */
    /* per original ray (indexed through ray_indices, like insta_training_samples' rays) */
    const float* rays;                /* f32[6]: origin, unnormalised direction                    */
    const float* target;              /* f32[4]: the image sample (linear rgb, alpha)              */
    const float* background;          /* f32[3] sRGB background (random_bg_color draw) or NULL = 0 */
    const float* exposure;            /* f32[3] exposure (log2 scale) or NULL = 0                  */
    const float* depth;               /* f32 depth image sample or NULL (no depth supervision)     */
    const int32_t* seg_mask;          /* i32 segmentation id or NULL (no segmentation rules)       */
    const float* mean_density;        /* the density grid's mean (1 float) or NULL (no L1 term)    */
    /* insta_training_samples' outputs and the network's */
    const uint32_t* rays_counter;     /* rays kept (counters[0])                                   */
    const uint32_t* ray_indices;
    uint32_t* numsteps;               /* [max_rays][2] in: (count, base); out: compacted           */
    const float* coords;              /* the sample records                                        */
    const float* network_output;      /* f32[samples][4] raw rgb + raw density                     */
    uint32_t* numsteps_counter;       /* compacted samples (zeroed by the caller)                  */
    float* coords_out;                /* [max_samples_compacted][stride]                            */
    float* dloss_doutput;             /* f32[max_samples_compacted][4]                              */
    float* loss_output;               /* f32[max_rays] per-ray loss / n_rays, or NULL               */
    /* importance sampling and the error map (compute_loss_kernel_train_nerf,
     * instant-ngp/src/testbed_nerf.cu:1411-1416,1494-1536; train_nerf_step runs it with
     * accumulate_error = true, :3248,3333).  Per original ray, as insta_training_pixels writes them. */
    const float* pdf;                 /* f32 img_pdf * xy_pdf the ray's loss is divided by, or NULL = 1 */
    float* error_map;                 /* f32[n_images][res_y][res_x]: each kept ray's mean loss added
                                         bilinearly at its image position, or NULL = off             */
    uint32_t error_map_res[2];        /* x, y (each >= 2, no larger than the images)                 */
    uint32_t error_map_images;        /* images of the error map; rays of other images deposit nothing */
    const float* image_xy;            /* f32[2] position in [0, 1]^2 of the ray's pixel              */
    const uint32_t* image_index;      /* the ray's training image                                     */
} insta_train_loss_desc;
/* All pointers are device pointers; asynchronous on the context's stream. */
int insta_train_loss(insta_ctx* ctx, const insta_train_loss_desc* desc);

/* The training batch's image and pixel draws of generate_training_samples_nerf and
 * compute_loss_kernel_train_nerf (instant-ngp/src/testbed_nerf.cu:1140-1144,1406-1420): per ray i
 * the image image_idx(i, ...) (evenly spread, or from cdf_img with ld_random_val(i + n_rays_total,
 * 0xdeadbeef) when the error-map CDFs are given), the step's pcg32 advanced by 8 i, the pixel
 * position nerf_random_image_pos_training (two draws, through sample_cdf_2d when the CDFs are
 * given, optionally snapped to pixel centres), then the random background colour draw
 * (random_val_3d, sRGB).  The caller turns (image, xy) into camera rays. */
typedef struct insta_training_pixels_desc {
    uint32_t n_rays;                  /* rays of the batch                                         */
    uint32_t n_rays_total;            /* rays drawn by the earlier steps                           */
    uint32_t n_images;
    const int32_t* resolution;        /* [n_images][2] image width, height (device)                 */
    int32_t snap_to_pixel_centers;
    uint64_t rng_state, rng_inc;      /* the step's pcg32 (m_rng)                                   */
    const float* cdf_x_cond_y;        /* insta_error_map_cdf's outputs, or all NULL = uniform       */
    const float* cdf_y;
    const float* cdf_img;
    uint32_t cdf_res[2];              /* x, y of the error map the CDFs were built from             */
    uint32_t* out_image;              /* [n_rays]                                                   */
    float* out_xy;                    /* [n_rays][2]                                                */
    float* out_pdf;                   /* [n_rays] img_pdf * xy_pdf, or NULL                          */
    float* out_background;            /* [n_rays][3] random_bg_color draw (sRGB), or NULL           */
} insta_training_pixels_desc;
int insta_training_pixels(insta_ctx* ctx, const insta_training_pixels_desc* desc);

/* The error map's sampling distributions (construct_cdf_2d, construct_cdf_1d and the image CDF of
 * train_nerf_step, instant-ngp/src/testbed_nerf.cu:1967-2020,3010-3041): per image and row the
 * conditional CDF over x (mixed with 1 % uniform), per image the CDF over rows (1 %), and over the
 * images the CDF with 10 % uniform.  error_map f32[n_images][res_y][res_x] in; cdf_x_cond_y
 * (same shape), cdf_y [n_images][res_y], cdf_img [n_images] and pmf_img [n_images] (or NULL) out.
 * Device pointers, asynchronous; the reference builds the image CDF on the host, here one device
 * thread runs the same loop. */
int insta_error_map_cdf(insta_ctx* ctx, const float* error_map, uint32_t n_images, uint32_t res_x, uint32_t res_y,
                        float* cdf_x_cond_y, float* cdf_y, float* cdf_img, float* pmf_img);

/* -- render ------------------------------------------------------------------- */
/* out_rgba f32[h*w*4] (linear RGBA, zero background), out_depth f32[h*w] (1e10 where no
 * hit).  Host pointers: the call returns after the copy back; device pointers: asynchronous. */
int insta_render(insta_ctx* ctx, const insta_render_desc* req, float* out_rgba, float* out_depth);
/* insta_render without waiting for host outputs: the copy back of a frame runs on the context's
 * copy stream (page-locked host buffers let it overlap the next render); the buffers hold the
 * frame after insta_sync or any later call that synchronises.  Device outputs: as insta_render.
 * No reference counterpart (render_nerf writes into its own render buffer). */
int insta_render_async(insta_ctx* ctx, const insta_render_desc* req, float* out_rgba, float* out_depth);
/* n requests rendered through one wavefront: each round marches, deforms, encodes, evaluates and
 * composites the alive rays of every request with one set of launches.  Requests may mix avatars,
 * frames, cameras and resolutions; their avatars must share one field layout (same
 * insta_field_desc).  out_rgba[i] / out_depth[i] as for insta_render (host or device, per
 * request).  Each request's pixels equal those of insta_render on that request alone.  At most
 * 4096 requests and 2^25 pixels per batch (one round's sample buffers hold a sample per pixel).  No reference counterpart: render_nerf renders one
 * view at a time (instant-ngp/src/testbed_nerf.cu:2320). */
int insta_render_batch(insta_ctx* ctx, const insta_render_desc* reqs, int n, float* const* out_rgba, float* const* out_depth);
/* Network samples evaluated by the last insta_render / insta_render_batch (synchronises). */
int insta_render_samples(insta_ctx* ctx, uint64_t* n_samples);

/* Launch shapes of the render wavefront, per context.  NerfTracer::trace fixes its own
 * (MIN/MAX_STEPS_INBETWEEN_COMPACTION 1/8 and n_steps_between_compaction = clamp(N0 / n_alive),
 * instant-ngp/src/testbed_nerf.cu:67-68,2172); here each round takes
 * clamp(round budget / n_alive, 1, max_steps_per_round) samples per alive ray.  A zero field keeps
 * the built-in choice.  Results do not depend on these (every sample's arithmetic is the same;
 * rays composite their samples in order): only speed does. */
typedef struct insta_tuning {
    uint32_t max_steps_per_round;   /* 1..128 (built-in 64) */
    uint32_t sort_cell_bits;        /* 12, 15, 18 or 21: Morton cells of a round's (request, cell) sort
                                       (built-in 18 = 64^3 per request, fewer when requests x cells > 4 Mi) */
    uint32_t mlp_ctas_per_sm;       /* 1..4 resident MLP CTAs per SM (built-in: as many as shared memory allows) */
    uint32_t deform_blocks_per_sm;  /* 1..64 blocks per SM of the deform + encode stage (built-in 16) */
    uint32_t bvh_top_nodes;         /* 0, 5 or 21: top levels of each frame's tree that every warp of the
                                       nearest-triangle stage copies into shared memory (built-in 0) */
    uint32_t fused_field_stage;     /* 1: deform + encode + MLP as one kernel (FP16 / BF16 fields);
                                       0 (built-in, faster on GB300): encode to global operand tiles, then the MLP */
    uint32_t mlp_slots;             /* MLP stage where every tile uses one weight image: 2..7 = one
                                       persistent CTA per SM with that many 128-sample tile slots sharing one
                                       copy of the weights (one sample row per thread); 1 = several CTAs per
                                       SM, each with its own copy (mlp_ctas_per_sm); 8 = FP16 / BF16 only:
                                       CTAs of two tiles each, an MMA-issuing warp and two epilogue warpgroups;
                                       0 = built-in: slots for FP8 fields, for batches of two or more
                                       requests on one weight image and for encodings wider than 64
                                       (measured faster there), else CTAs */
} insta_tuning;
int insta_tuning_set(insta_ctx* ctx, const insta_tuning* t);
int insta_tuning_get(insta_ctx* ctx, insta_tuning* t);
/* The autotuner: times insta_render_batch on the given requests (device outputs it allocates)
 * for candidate launch shapes -- coordinate descent over the fields above, each candidate the
 * median of `repeats` timed renders after one untimed one (CUDA events on the context's stream) --
 * then keeps the fastest with insta_tuning_set and returns it in *best (best_ms: its time per
 * batch).  No reference counterpart. */
int insta_autotune(insta_ctx* ctx, const insta_render_desc* reqs, int n, int repeats, insta_tuning* best, float* best_ms);
/* Per-ray sample t and dt (device pointers, [h*w][max_out]) and counts [h*w]. */
int insta_march_debug(insta_ctx* ctx, const insta_render_desc* req, int max_out, float* out_t, float* out_dt,
                      int32_t* out_n);
/* rta::Core::raycast_flame (src/core.cu:350-402): the tracked mesh of req->frame ray-traced
 * from req's camera -- init_rays_with_payload_kernel_sdf (instant-ngp/src/testbed_sdf.cu:505-577,
 * no slice plane, aperture or octree), the closest hit at t < 10 (TriangleBvh4::ray_intersect,
 * instant-ngp/src/triangle_bvh.cu:271-311; ties to the lowest triangle id) and INSTA's
 * shade_kernel_sdf (src/core.cu:74-113: three lights around the canonical centroid, or the normal
 * as colour when color_normal != 0).  Pixels whose hit lies inside the render box get RGBA
 * (alpha 1) and depth = the hit's z; the others keep their values.  out_tri (optional): the hit
 * triangle id or -1.  Host or device pointers. */
int insta_raycast(insta_ctx* ctx, const insta_render_desc* req, int color_normal, float* out_rgba, float* out_depth,
                  int32_t* out_tri);
/* Nearest triangle id of each point (device pointers: pts f32[n*3] in the frame's space, out
 * i32[n]) computed the way the render's deform stage computes it: the warp-cooperative walk over
 * 32 consecutive points. */
int insta_nearest_debug(insta_ctx* ctx, int avatar, int frame, const float* pts, int64_t n, int32_t* out_idx);

/* -- serving ------------------------------------------------------------------- */
/* A request loop on a worker thread that owns the context from insta_server_create to
 * insta_server_destroy (load avatars -- canonical mesh, parameters -- before creating it; make no
 * other call on the context meanwhile).  Each request renders one view of one avatar, with its
 * own tracked-mesh frame (frame_verts, host f32[n_verts*3], copied at submit; NULL renders the
 * already uploaded desc->frame).  Requests are admitted into request slots while slots, the
 * pixel budget and the context's memory budget allow; the rays of admitted requests join the
 * running wavefront at the next round, so requests that arrive while others are on the GPU run
 * together with them (continuous batching), and a slot frees as soon as its last ray has
 * composited.  Each request's pixels equal those of insta_render alone.  Frame ids >= 2^30 are
 * the server's.  No reference counterpart: the reference renders one view per render_nerf call. */
#define INSTA_REQ_QUEUED 0
#define INSTA_REQ_RUNNING 1
#define INSTA_REQ_DONE 2
#define INSTA_REQ_CANCELLED 3
#define INSTA_REQ_FAILED 4

typedef struct insta_server insta_server;
typedef struct {
    uint32_t max_inflight;          /* request slots (1..256) */
    uint64_t max_inflight_pixels;   /* pixels of admitted requests (<= 2^25) */
    double occupancy_radius;        /* request frames: occupancy from the mesh (0.015) */
    uint32_t rounds_per_launch;     /* rounds run as one CUDA-graph launch between admission points
                                       (even; 0 = 2); with per-stage timing on, rounds are host-driven */
    uint64_t round_samples;         /* samples marched per round at most (2^16..2^25; 0 = 2^25;
                                       raised to max_inflight_pixels): a smaller budget gives
                                       shorter rounds, so arriving requests join sooner, at more
                                       rounds per ray */
} insta_server_config;

int insta_server_create(insta_ctx* ctx, const insta_server_config* cfg, insta_server** out);
/* Cancels queued requests, lets running ones finish, joins the worker. */
int insta_server_destroy(insta_server* s);
/* out_rgba / out_depth as for insta_render (host: filled when the request is done). */
int insta_submit(insta_server* s, const insta_render_desc* req, const float* frame_verts, float* out_rgba, float* out_depth,
                 uint64_t* ticket);
/* state: INSTA_REQ_*; latency_ms (optional): submit -> done, -1 while not done. */
int insta_poll(insta_server* s, uint64_t ticket, int* state, double* latency_ms);
/* Blocks until the request is done, cancelled or failed (timeout_ms < 0: no limit). */
int insta_wait(insta_server* s, uint64_t ticket, int timeout_ms, int* state);
/* Queued: dropped before admission.  Running: finishes, its outputs are not delivered. */
int insta_cancel(insta_server* s, uint64_t ticket);
/* Forget a finished ticket. */
int insta_server_release(insta_server* s, uint64_t ticket);
const char* insta_server_error(insta_server* s, uint64_t ticket);

#ifdef __cplusplus
}
#endif
#endif
