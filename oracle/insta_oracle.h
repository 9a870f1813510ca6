/*
 * insta_oracle.h -- CPU restatement of INSTA's per-sample deformation and
 * render path.  TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke
 * check and by bench.py's CPU-baseline leg.  The product library never links
 * or calls anything declared here.
 *
 * Every function cites the reference file:line whose behaviour it restates.
 * Paths are relative to the INSTA repository; "ngp/" abbreviates
 * "instant-ngp/" and "NGP/" abbreviates
 * "instant-ngp/include/neural-graphics-primitives/".
 *
 * Floating-point contract: compiled with -ffp-contract=off so every a*b+c is
 * two roundings, and 3-term sums follow Eigen's halving reduction order
 * x0 + (x1 + x2) (4-term: (x0 + x1) + (x2 + x3)).  The CUDA kernels mirror
 * this order with __fmul_rn/__fadd_rn wherever a result must be bit-exact
 * (squared point-triangle and point-box distances, which decide the nearest
 * triangle index).
 */
#ifndef INSTA_ORACLE_H
#define INSTA_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same 48-byte record as ngp::Triangle (NGP/triangle.cuh:234-238). */
typedef struct {
    float a[3], b[3], c[3];
    float scaling;
    uint32_t id;
    uint32_t mask_id;
} orc_tri;

/* ngp::TriangleBvhNode (ngp/include/.../triangle_bvh.cuh:29-33): 32 bytes. */
typedef struct {
    float bb_min[3], bb_max[3];
    int32_t left_idx, right_idx;
} orc_bvh_node;

/* ---- mesh ------------------------------------------------------------ */
int orc_adjacency(const int32_t *faces, int n_faces, int n_verts, int32_t *out_adj);
void orc_build_triangles(const float *verts, const float *canon_verts, const int32_t *faces,
                         const uint32_t *mask, int n_faces, orc_tri *out);
float orc_tri_distance_sq(const orc_tri *t, const float *p);
float orc_box_distance_sq(const float *mn, const float *mx, const float *p);

/* ---- nearest triangle -------------------------------------------------- */
void orc_nearest_brute(const orc_tri *tris, int n_tris, const float *pts, int64_t n_pts,
                       int32_t *out_id, float *out_d2);
int orc_bvh4_build(const orc_tri *tris, int n_tris, int leaf_size, orc_bvh_node *out_nodes,
                   int max_nodes, orc_tri *out_sorted);
void orc_nearest_bvh(const orc_bvh_node *nodes, const orc_tri *sorted, const float *pts,
                     int64_t n_pts, int exact, int32_t *out_id, float *out_d2);

/* ---- deformation map --------------------------------------------------- */
typedef struct {
    const orc_tri *def_tris;      /* frame triangles, original order        */
    const orc_tri *can_tris;      /* canonical triangles, original order    */
    const int32_t *adjacency;     /* [F*3]                                  */
    const orc_bvh_node *nodes;    /* optional BVH over def_tris (NULL: brute) */
    const orc_tri *sorted;        /* BVH-ordered triangles                  */
    int n_tris;
    int disable_interp;
    int fp64;                     /* 1: FP64 twin of the whole map          */
    int bvh_exact;                /* 1: lowest-id ties; 0: reference `<=`   */
    float aabb_min[3], aabb_max[3];
} orc_deform;

void orc_canonical_map_soa(const orc_deform *d, const float *pts, int64_t n,
                           int32_t *out_idx, float *out_canon);
void orc_canonical_map_coords(const orc_deform *d, float *coords, uint32_t stride,
                              uint32_t n_extra, int64_t n, int32_t frame_id, uint32_t n_frames);

/* ---- occupancy --------------------------------------------------------- */
void orc_occupancy_from_mesh(const orc_tri *tris, int n_tris, double radius, uint8_t *bitfield);
float orc_density_grid_to_bitfield(const float *grid, uint32_t n_cascades, uint8_t *bitfield);

/* ---- density-grid maintenance -------------------------------------------- */
/* PCG32 (the pcg32 of tiny-cuda-nn, absent from the reference tree: restated from O'Neill's
 * published PCG XSH-RR 64/32 generator with its jump-ahead). */
typedef struct { uint64_t state, inc; } orc_pcg32;
uint32_t orc_pcg32_next_uint(orc_pcg32 *r);
float orc_pcg32_next_float(orc_pcg32 *r);
void orc_pcg32_advance(orc_pcg32 *r, int64_t delta);
void orc_pcg32_seed(orc_pcg32 *r, uint64_t initstate, uint64_t initseq);
/* generate_grid_samples_nerf_nonuniform (ngp/src/testbed_nerf.cu:487-516) for the uniform
 * (thresh -0.01) and the non-uniform (thresh 0.01) set, both from the same generator state:
 * out_pos [n][3] (warp_position'ed), out_idx [n]. */
void orc_grid_samples(uint32_t n_uniform, uint32_t n_nonuniform, orc_pcg32 rng, uint32_t step, const float *aabb_min,
                      const float *aabb_max, const float *grid, uint32_t n_cascades, float *out_pos, uint32_t *out_idx);
/* warp_random_samples (src/core.cu:528-579): a random frame of n_frames per point, its nearest
 * triangle, the canonical position; pos [n][3] in place; out_frame [n] (optional). */
void orc_warp_random_samples(const orc_deform *frames, uint32_t n_frames, orc_pcg32 rng, float *pos, int64_t n, uint32_t *out_frame);
uint32_t orc_morton3d(uint32_t x, uint32_t y, uint32_t z);

/* ---- field (hash grid + SH + MLPs) ------------------------------------ */
typedef struct {
    uint32_t n_levels, n_features, log2_table, base_res;
    float per_level_scale;
    uint32_t n_extra;             /* expression dims appended to the density input */
    uint32_t density_hidden;      /* neurons (64)                           */
    uint32_t density_layers;      /* hidden layers (1)                      */
    uint32_t density_out;         /* 16                                     */
    uint32_t rgb_hidden;          /* 64                                     */
    uint32_t rgb_layers;          /* hidden layers (2)                      */
    uint32_t rgb_out_padded;      /* 16                                     */
    int weight_format;            /* 0 fp16, 1 bf16, 2 fp8-e4m3 (per-layer scale) */
} orc_field_cfg;

uint64_t orc_field_layout(const orc_field_cfg *c, uint64_t *level_offsets, uint32_t *level_res,
                          uint32_t *level_size, uint64_t *mlp_params);
void orc_field_eval(const orc_field_cfg *c, const uint16_t *params, const float *layer_scales,
                    const float *coords, uint32_t stride, int64_t n, float *out4, int fp64);

/* ---- render ------------------------------------------------------------ */
typedef struct {
    int width, height;
    float focal[2];
    float screen_center[2];
    float cam[12];                /* 3x4 row-major: [R | origin]            */
    float render_aabb_min[3], render_aabb_max[3];
    float train_aabb_min[3], train_aabb_max[3];
    float cone_angle;
    float min_transmittance;
    uint32_t spp;
    uint32_t max_samples_per_ray;
    int snap_to_pixel_centers;
    int frame_id;
    const float *extra_dims;      /* [n_extra] inference expression vector or NULL */
    int linear_colors;            /* 0: shade converts sRGB -> linear       */
} orc_render_cfg;

int64_t orc_render(const orc_render_cfg *rc, const orc_deform *d, const uint8_t *bitfield,
                   const orc_field_cfg *fc, const uint16_t *params, const float *layer_scales,
                   int row_begin, int row_end, float *out_rgba, float *out_depth,
                   uint32_t *out_nsamples, int fp64);
typedef struct {
    uint32_t n_rays, max_samples_compacted, target_batch_size, stride;
    float aabb_min[3], aabb_max[3];
    int loss_type, depth_loss_type, srgb_targets, train_in_linear_colors, penalize_density;
    float loss_scale, depth_supervision_lambda, seg_mask_supervision_lambda, near_distance, beta;
    /* importance-sampling pdf and the error map (per original ray; NULL = off) */
    const float *pdf;
    float *error_map;
    uint32_t error_map_res[2];
    uint32_t error_map_images;
    const float *image_xy;
    const uint32_t *image_index;
} orc_train_loss_cfg;
/* image_idx + nerf_random_image_pos_training + the background draw (testbed_nerf.cu:1013-1105,
 * 1140-1144, 1406-1420) for rays [0, n_rays). */
void orc_training_pixels(uint32_t n_rays, uint32_t n_rays_total, uint32_t n_images, const int32_t *resolution, int snap,
                         orc_pcg32 rng, const float *cdf_x_cond_y, const float *cdf_y, const float *cdf_img, const uint32_t *cdf_res,
                         uint32_t *out_image, float *out_xy, float *out_pdf, float *out_background);
/* construct_cdf_2d, construct_cdf_1d and the image CDF of train_nerf_step (testbed_nerf.cu:1967-2020,
 * 3024-3041). */
void orc_error_map_cdf(const float *error_map, uint32_t n_images, uint32_t res_x, uint32_t res_y, float *cdf_x_cond_y,
                       float *cdf_y, float *cdf_img, float *pmf_img);
void orc_train_loss(const orc_train_loss_cfg *c, uint32_t n_kept, const float *rays, const float *target, const float *background,
                    const float *exposure, const float *depth_img, const int32_t *seg_mask, const float *mean_density,
                    const uint32_t *ray_indices, uint32_t *numsteps, const float *coords, const float *nout, uint32_t *counter,
                    float *coords_out, float *dloss, float *loss_out);
void orc_field_backward(const orc_field_cfg *c, const uint16_t *params, const float *coords, uint32_t stride, int64_t n,
                        const float *dl_dout, double *grad, float *out4);
/* ... and, when dl_dextra is given, the gradient w.r.t. each record's expression dims [n][n_extra]. */
void orc_field_backward_ex(const orc_field_cfg *c, const uint16_t *params, const float *coords, uint32_t stride, int64_t n,
                           const float *dl_dout, double *grad, float *out4, double *dl_dextra);
void orc_raycast(const orc_render_cfg *rc, const orc_tri *tris, int n_tris, const float *center, int color_normal, float *out_rgba,
                 float *out_depth, int32_t *out_tri);
int orc_march_ray(const orc_render_cfg *rc, const uint8_t *bitfield, int px, int py,
                  int max_out, float *out_t, float *out_dt, float *out_pos);
void orc_training_samples(const float *aabb_min, const float *aabb_max, float cone, const uint8_t *bf, const float *rays,
                          const uint32_t *image, const float *start_rand, const float *extra, uint32_t n_extra, int64_t n,
                          uint32_t max_samples, float *coords, uint32_t stride, uint32_t *ray_indices, uint32_t *numsteps,
                          uint32_t *counters);

/* ---- low-discrepancy helpers (NGP/random_val.cuh:159-322) -------------- */
float orc_ld_random_val(uint32_t index, uint32_t seed, uint32_t dim);
void orc_ld_random_pixel_offset(uint32_t spp, float out[2]);
uint32_t orc_sobol(uint32_t index, uint32_t dim);

/* ---- single reference functions (pin tests) ----------------------------- */
void orc_tbn(const orc_tri *t, float *m9);
void orc_tri2projection(const orc_tri *t, float *M16);
void orc_interpolate_transformation(const float *p, const int32_t *adj, const orc_tri *tris, uint32_t id, int invert, float *M16);
void orc_transform(const float *p, const float *dir, const float *Mw, const float *Mc, float *out_p, float *out_d);
/* march helpers (calc_dt, warp_dt / unwarp_dt, mip_from_dt, density_grid_occupied_at,
 * advance_to_next_voxel of ngp/src/testbed_nerf.cu) */
float orc_probe_calc_dt(float t, float cone);
float orc_probe_warp_dt(float dt);
float orc_probe_unwarp_dt(float dt);
int orc_probe_mip_from_dt(float dt, const float *pos);
int orc_probe_occupied_at(const float *pos, const uint8_t *bf, int mip);
float orc_probe_advance_to_next_voxel(float t, float cone, const float *pos, const float *dir, const float *idir, uint32_t res);

/* ---- half helpers ------------------------------------------------------ */
uint16_t orc_f2h(float x);
float orc_h2f(uint16_t h);
float orc_e4m3_round(float x);
int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
