/*
 * insta_oracle.c -- CPU restatement of INSTA's deformation + render hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, the smoke check and bench.py's
 * CPU-baseline leg load this library, and only as the checker (or as the
 * timed CPU baseline).  The CUDA product never links or calls it.
 *
 * Parity pin: the geometry primitives (distance_sq, box distance, tbn,
 * tri2projection, the BVH traversal, the Sobol/scrambling helpers) are pinned
 * against the reference's own headers compiled for the host (oracle/build_ref.py
 * builds oracle/_ref/libinsta_ref.so) and against the golden vectors that
 * script writes under tests/golden/.  The hash-grid encode, SH and MLPs have
 * no reference source in the repository (tiny-cuda-nn is an empty
 * submodule), so their restatement is the published method, unpinned.
 *
 * Build: gcc -O3 -fopenmp -ffp-contract=off -fPIC -shared (see oracle/build.py).
 */
#include "insta_oracle.h"

#include <math.h>
#include <float.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---------------------------------------------------------------- halves */
uint16_t orc_f2h(float x) { _Float16 h = (_Float16)x; uint16_t b; memcpy(&b, &h, 2); return b; }
float orc_h2f(uint16_t b) { _Float16 h; memcpy(&h, &b, 2); return (float)h; }
static uint16_t orc_f2bf16(float x) {
    uint32_t u; memcpy(&u, &x, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
static float orc_bf16_to_f(uint16_t b) { uint32_t u = (uint32_t)b << 16; float f; memcpy(&f, &u, 4); return f; }
/* FP8 E4M3 (1 sign, 4 exponent bits with bias 7, 3 mantissa bits; largest finite 448, no
 * infinities): x rounded to the nearest representable value, ties to even, saturating at +-448
 * (the SATFINITE conversion); NaN stays NaN. */
float orc_e4m3_round(float x) {
    if (x != x) return x;
    float a = fabsf(x);
    if (a >= 448.0f) return copysignf(448.0f, x);
    float q;
    if (a < 0.015625f) {                       /* below 2^-6: subnormals, quantum 2^-9 */
        q = nearbyintf(a * 512.0f) / 512.0f;
    } else {
        int e;
        frexpf(a, &e);                         /* a = m 2^e, m in [0.5, 1): leading bit 2^(e-1) */
        float quantum = ldexpf(1.0f, e - 4);   /* 3 mantissa bits below the leading one */
        q = nearbyintf(a / quantum) * quantum;
        if (q > 448.0f) q = 448.0f;
    }
    return copysignf(q, x);
}

/* ---------------------------------------------------------- field layout */
/* Per-level grid scale of the multiresolution hash encoding:
 * scale_l = b^l * N_min - 1 computed as exp2(l * log2 b) * N_min - 1 in float. */
static float orc_level_scale(const orc_field_cfg *c, uint32_t l) {
    return exp2f((float)l * log2f(c->per_level_scale)) * (float)c->base_res - 1.0f;
}
static uint32_t orc_grid_index(const uint32_t *cc, uint32_t res, uint32_t size) {
    uint64_t r3 = (uint64_t)res * res * res;
    uint32_t idx;
    if (r3 <= size) idx = cc[0] + cc[1] * res + cc[2] * res * res;
    else idx = (cc[0] * 1u) ^ (cc[1] * 2654435761u) ^ (cc[2] * 805459861u);
    return idx % size;
}

uint64_t orc_field_layout(const orc_field_cfg *c, uint64_t *lvl_off, uint32_t *lvl_res, uint32_t *lvl_size,
                          uint64_t *mlp_off) {
    uint64_t n_in = (uint64_t)c->n_levels * c->n_features + c->n_extra;
    uint64_t dens = c->density_hidden * n_in + (uint64_t)(c->density_layers - 1) * c->density_hidden * c->density_hidden
                    + (uint64_t)c->density_out * c->density_hidden;
    uint64_t rgb_in = c->density_out + 16;
    uint64_t rgb = c->rgb_hidden * rgb_in + (uint64_t)(c->rgb_layers - 1) * c->rgb_hidden * c->rgb_hidden
                   + (uint64_t)c->rgb_out_padded * c->rgb_hidden;
    mlp_off[0] = 0;
    mlp_off[1] = dens;
    mlp_off[2] = dens + rgb;
    uint64_t T = 1ull << c->log2_table, off = 0;
    for (uint32_t l = 0; l < c->n_levels; ++l) {
        float s = orc_level_scale(c, l);
        uint32_t res = (uint32_t)ceilf(s) + 1u;
        uint64_t r3 = (uint64_t)res * res * res;
        uint64_t sz = (r3 + 7) / 8 * 8;
        if (sz > T) sz = T;
        lvl_off[l] = off; lvl_res[l] = res; lvl_size[l] = (uint32_t)sz;
        off += sz;
    }
    return mlp_off[2] + off * c->n_features;
}

/* ------------------------------------------------- FP32 / FP64 instances */
static void tri2projection_raw_d(const orc_tri *t, double *M);
static int inverse4_d(const double *m, double *o);
#define R float
#define SFX(n) n##_f
#define R_SQRT sqrtf
#define R_EXP expf
#define R_FLOOR floorf
#define R_FABS fabsf
#define R_IS_FLOAT 1
#include "oracle_real.inc"
#undef R
#undef SFX
#undef R_SQRT
#undef R_EXP
#undef R_FLOOR
#undef R_FABS
#undef R_IS_FLOAT
#define R double
#define SFX(n) n##_d
#define R_SQRT sqrt
#define R_EXP exp
#define R_FLOOR floor
#define R_FABS fabs
#define R_IS_FLOAT 0
#include "oracle_real.inc"
#undef R
#undef SFX

/* ------------------------------------------------------------- geometry */
static inline float v3dot(const float *a, const float *b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }
static inline void v3cross(const float *a, const float *b, float *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
/* sign (NGP/common.h:191): copysignf(1, x). */
static inline float ngp_sign(float x) { return copysignf(1.0f, x); }
/* tcnn::clamp: val < lo ? lo : (hi < val ? hi : val). */
static inline float clampf_(float v, float lo, float hi) { return v < lo ? lo : (hi < v ? hi : v); }

/* Triangle::distance_sq (NGP/triangle.cuh:88-107). */
float orc_tri_distance_sq(const orc_tri *t, const float *pos) {
    float v21[3], p1[3], v32[3], p2[3], v13[3], p3[3], nor[3], tmp[3];
    for (int k = 0; k < 3; ++k) {
        v21[k] = t->b[k] - t->a[k]; p1[k] = pos[k] - t->a[k];
        v32[k] = t->c[k] - t->b[k]; p2[k] = pos[k] - t->b[k];
        v13[k] = t->a[k] - t->c[k]; p3[k] = pos[k] - t->c[k];
    }
    v3cross(v21, v13, nor);
    float s = 0.0f;
    v3cross(v21, nor, tmp); float s1 = ngp_sign(v3dot(tmp, p1));
    v3cross(v32, nor, tmp); float s2 = ngp_sign(v3dot(tmp, p2));
    v3cross(v13, nor, tmp); float s3 = ngp_sign(v3dot(tmp, p3));
    s = s1 + s2 + s3;
    if (s < 2.0f) {
        float e[3][3], d[3];
        const float *vv[3] = {v21, v32, v13}, *pp[3] = {p1, p2, p3};
        for (int i = 0; i < 3; ++i) {
            float f = clampf_(v3dot(vv[i], pp[i]) / v3dot(vv[i], vv[i]), 0.0f, 1.0f);
            for (int k = 0; k < 3; ++k) e[i][k] = vv[i][k] * f - pp[i][k];
            d[i] = v3dot(e[i], e[i]);
        }
        /* std::min({d0, d1, d2}): first smallest */
        float m = d[0];
        if (d[1] < m) m = d[1];
        if (d[2] < m) m = d[2];
        return m;
    }
    float nd = v3dot(nor, p1);
    return nd * nd / v3dot(nor, nor);
}

/* BoundingBox::distance_sq (NGP/bounding_box.cuh:228-230). */
float orc_box_distance_sq(const float *mn, const float *mx, const float *p) {
    float d[3];
    for (int k = 0; k < 3; ++k) {
        float a = mn[k] - p[k], b = p[k] - mx[k];
        float m = a < b ? b : a;   /* cwiseMax */
        d[k] = m < 0.0f ? 0.0f : m;
    }
    return v3dot(d, d);
}

static inline int box_contains(const float *mn, const float *mx, const float *p) {
    return p[0] >= mn[0] && p[0] <= mx[0] && p[1] >= mn[1] && p[1] <= mx[1] && p[2] >= mn[2] && p[2] <= mx[2];
}

/* ------------------------------------------------------------------ mesh */
static int cmp_int(const void *a, const void *b) { int x = *(const int *)a, y = *(const int *)b; return (x > y) - (x < y); }

/* TinyMesh::get_triangle_3_neighbours (src/tiny_mesh.cu:316-371): for each face, the sorted set
 * of faces sharing one of its edges, minus itself, padded with -1 to 3 entries.  (The reference
 * writes past slot 2 for non-manifold edges; here extra entries are dropped.)  Returns 0. */
int orc_adjacency(const int32_t *faces, int n_faces, int n_verts, int32_t *out_adj) {
    int *cnt = calloc((size_t)n_verts + 1, sizeof(int));
    for (int f = 0; f < n_faces; ++f) for (int k = 0; k < 3; ++k) cnt[faces[f * 3 + k] + 1]++;
    for (int v = 0; v < n_verts; ++v) cnt[v + 1] += cnt[v];
    int *vf = malloc(sizeof(int) * (size_t)n_faces * 3);
    int *fill = calloc((size_t)n_verts, sizeof(int));
    for (int f = 0; f < n_faces; ++f)
        for (int k = 0; k < 3; ++k) { int v = faces[f * 3 + k]; vf[cnt[v] + fill[v]++] = f; }
    for (int f = 0; f < n_faces; ++f) {
        int ids[256], n = 0;
        int e[3][2] = {{faces[f * 3], faces[f * 3 + 1]}, {faces[f * 3], faces[f * 3 + 2]}, {faces[f * 3 + 1], faces[f * 3 + 2]}};
        for (int ei = 0; ei < 3; ++ei) {
            int va = e[ei][0], vb = e[ei][1];
            for (int i = cnt[va]; i < cnt[va + 1]; ++i)
                for (int j = cnt[vb]; j < cnt[vb + 1]; ++j)
                    if (vf[i] == vf[j] && n < 256) ids[n++] = vf[i];
        }
        qsort(ids, (size_t)n, sizeof(int), cmp_int);
        int k = 0, prev = -2;
        for (int i = 0; i < 3; ++i) out_adj[f * 3 + i] = -1;
        for (int i = 0; i < n; ++i) {
            if (ids[i] == prev) continue;
            prev = ids[i];
            if (ids[i] != f && k < 3) out_adj[f * 3 + k++] = ids[i];
        }
    }
    free(cnt); free(vf); free(fill);
    return 0;
}

static float tri_area(const float *a, const float *b, const float *c) {
    float e1[3], e2[3], n[3];
    for (int k = 0; k < 3; ++k) { e1[k] = b[k] - a[k]; e2[k] = c[k] - a[k]; }
    v3cross(e1, e2, n);
    return 0.5f * sqrtf(v3dot(n, n));
}

/* TinyMesh::build_triangles (src/tiny_mesh.cu:134-164): id = face index, mask from the region map,
 * scaling = area(deformed) / area(canonical) (1 when canon_verts == NULL). */
void orc_build_triangles(const float *verts, const float *canon_verts, const int32_t *faces, const uint32_t *mask,
                         int n_faces, orc_tri *out) {
    for (int f = 0; f < n_faces; ++f) {
        orc_tri *t = &out[f];
        const int32_t *fc = &faces[f * 3];
        memcpy(t->a, &verts[fc[0] * 3], 12); memcpy(t->b, &verts[fc[1] * 3], 12); memcpy(t->c, &verts[fc[2] * 3], 12);
        t->id = (uint32_t)f;
        t->mask_id = mask ? mask[f] : 15u;
        float s = 1.0f;
        if (canon_verts) {
            float ca = tri_area(&canon_verts[fc[0] * 3], &canon_verts[fc[1] * 3], &canon_verts[fc[2] * 3]);
            s *= tri_area(t->a, t->b, t->c) / ca;
        }
        t->scaling = s;
    }
}

/* ------------------------------------------------------- nearest triangle */
void orc_nearest_brute(const orc_tri *tris, int n_tris, const float *pts, int64_t n_pts, int32_t *out_id, float *out_d2) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < n_pts; ++i) {
        float best = FLT_MAX; int32_t bid = -1;
        for (int t = 0; t < n_tris; ++t) {
            float d = orc_tri_distance_sq(&tris[t], &pts[i * 3]);
            if (d < best || (d == best && (int32_t)tris[t].id < bid)) { best = d; bid = (int32_t)tris[t].id; }
        }
        out_id[i] = bid;
        if (out_d2) out_d2[i] = best;
    }
}

/* TriangleBvhWithBranchingFactor<4>::build (ngp/src/triangle_bvh.cu:548-631): top-down, each node
 * splits its range twice (4 children) at the median of the max-variance centroid axis with
 * nth_element; leaves hold <= leaf_size triangles encoded as negative ranges.  Triangles are
 * reordered.  Returns the node count, or -1 when max_nodes is too small.  The median partition
 * here is a deterministic introselect (std::nth_element's element order is not reproduced; only
 * the multiset split at the median is). */
static float centroid_axis(const orc_tri *t, int axis) { return (t->a[axis] + t->b[axis] + t->c[axis]) / 3.0f; }

static void nth_split(orc_tri *v, int lo, int hi, int nth, int axis) {
    /* quickselect on [lo, hi) so that v[nth] is the nth order statistic */
    while (hi - lo > 1) {
        int mid = lo + (hi - lo) / 2;
        float pv = centroid_axis(&v[mid], axis);
        int i = lo, j = hi - 1;
        while (i <= j) {
            while (centroid_axis(&v[i], axis) < pv) ++i;
            while (pv < centroid_axis(&v[j], axis)) --j;
            if (i <= j) { orc_tri tmp = v[i]; v[i] = v[j]; v[j] = tmp; ++i; --j; }
        }
        if (nth <= j) hi = j + 1;
        else if (nth >= i) lo = i;
        else return;
    }
}

static void bbox_of(const orc_tri *v, int lo, int hi, float *mn, float *mx) {
    for (int k = 0; k < 3; ++k) { mn[k] = v[lo].a[k]; mx[k] = v[lo].a[k]; }
    for (int i = lo; i < hi; ++i) {
        const float *pts[3] = {v[i].a, v[i].b, v[i].c};
        for (int p = 0; p < 3; ++p)
            for (int k = 0; k < 3; ++k) { if (pts[p][k] < mn[k]) mn[k] = pts[p][k]; if (pts[p][k] > mx[k]) mx[k] = pts[p][k]; }
    }
}

int orc_bvh4_build(const orc_tri *tris, int n_tris, int leaf_size, orc_bvh_node *nodes, int max_nodes, orc_tri *v) {
    memcpy(v, tris, sizeof(orc_tri) * (size_t)n_tris);
    int n_nodes = 1;
    bbox_of(v, 0, n_tris, nodes[0].bb_min, nodes[0].bb_max);
    if (n_tris <= leaf_size) { nodes[0].left_idx = -1; nodes[0].right_idx = -n_tris - 1; return 1; }
    int *stack = malloc(sizeof(int) * 3 * (size_t)(n_tris + 8));
    int sp = 0;
    stack[sp++] = 0; stack[sp++] = 0; stack[sp++] = n_tris;
    while (sp > 0) {
        int end = stack[--sp], begin = stack[--sp], node = stack[--sp];
        int cb[4], ce[4];
        cb[0] = begin; ce[0] = end;
        int n_children = 1;
        while (n_children < 4) {
            for (int i = n_children - 1; i >= 0; --i) {
                int b = cb[i], e = ce[i];
                double mean[3] = {0, 0, 0}, var[3] = {0, 0, 0};
                float meanf[3] = {0, 0, 0}, varf[3] = {0, 0, 0};
                for (int t = b; t < e; ++t) for (int k = 0; k < 3; ++k) meanf[k] += centroid_axis(&v[t], k);
                for (int k = 0; k < 3; ++k) meanf[k] /= (float)(e - b);
                for (int t = b; t < e; ++t) for (int k = 0; k < 3; ++k) { float d = centroid_axis(&v[t], k) - meanf[k]; varf[k] += d * d; }
                for (int k = 0; k < 3; ++k) varf[k] /= (float)(e - b);
                (void)mean; (void)var;
                int axis = 0;
                if (varf[1] > varf[axis]) axis = 1;
                if (varf[2] > varf[axis]) axis = 2;
                int m = b + (e - b) / 2;
                nth_split(v, b, e, m, axis);
                cb[i * 2] = b; ce[i * 2 + 1] = e; ce[i * 2] = m; cb[i * 2 + 1] = m;
            }
            n_children *= 2;
        }
        nodes[node].left_idx = n_nodes;
        for (int i = 0; i < 4; ++i) {
            if (n_nodes >= max_nodes) { free(stack); return -1; }
            int ci = n_nodes++;
            bbox_of(v, cb[i], ce[i], nodes[ci].bb_min, nodes[ci].bb_max);
            if (ce[i] - cb[i] <= leaf_size) {
                nodes[ci].left_idx = -cb[i] - 1;
                nodes[ci].right_idx = -ce[i] - 1;
            } else {
                stack[sp++] = ci; stack[sp++] = cb[i]; stack[sp++] = ce[i];
            }
        }
        nodes[node].right_idx = n_nodes;
    }
    free(stack);
    return n_nodes;
}

/* closest_triangle (NGP/bvh.cuh:48-96): stack traversal, children sorted by box distance with the
 * 4-input sorting network (:28-46) so the nearest is popped first; children pushed when
 * dist <= best.  exact == 0 reproduces the reference's leaf rule (dist <= best: the last
 * triangle in BVH order wins ties).  exact == 1 keeps the lowest original id on ties and prunes
 * with a small relative slack so that the result equals the brute-force minimum. */
void orc_nearest_bvh(const orc_bvh_node *nodes, const orc_tri *sorted, const float *pts, int64_t n_pts, int exact,
                     int32_t *out_id, float *out_d2) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t q = 0; q < n_pts; ++q) {
        const float *p = &pts[q * 3];
        int stack[64]; int sp = 0;
        stack[sp++] = 0;
        float best = FLT_MAX; int bidx = -1; int32_t bid = -1;
        while (sp > 0) {
            int idx = stack[--sp];
            const orc_bvh_node *n = &nodes[idx];
            if (n->left_idx < 0) {
                int end = -n->right_idx - 1;
                for (int i = -n->left_idx - 1; i < end; ++i) {
                    float d = orc_tri_distance_sq(&sorted[i], p);
                    if (exact) {
                        if (d < best || (d == best && (int32_t)sorted[i].id < bid)) { best = d; bidx = i; bid = (int32_t)sorted[i].id; }
                    } else if (d <= best) { best = d; bidx = i; bid = (int32_t)sorted[i].id; }
                }
            } else {
                float cd[4]; int ci[4];
                for (int i = 0; i < 4; ++i) { ci[i] = n->left_idx + i; cd[i] = orc_box_distance_sq(nodes[ci[i]].bb_min, nodes[ci[i]].bb_max, p); }
                /* sorting network: compare_and_swap swaps when first < second (descending) */
#define CAS(x, y) if (cd[x] < cd[y]) { float td = cd[x]; cd[x] = cd[y]; cd[y] = td; int ti = ci[x]; ci[x] = ci[y]; ci[y] = ti; }
                CAS(0, 2) CAS(1, 3) CAS(0, 1) CAS(2, 3) CAS(1, 2)
#undef CAS
                for (int i = 0; i < 4; ++i) {
                    float lim = exact ? best * 1.0009765625f + 1e-12f : best;
                    if (cd[i] <= lim && sp < 64) stack[sp++] = ci[i];
                }
            }
        }
        (void)bidx;
        out_id[q] = bid;
        if (out_d2) out_d2[q] = best;
    }
}

/* -------------------------------------------------- canonical map (warp) */
static int32_t nearest_one(const orc_deform *d, const float *p) {
    int32_t id; float d2;
    if (d->nodes) orc_nearest_bvh(d->nodes, d->sorted, p, 1, d->bvh_exact, &id, &d2);
    else orc_nearest_brute(d->def_tris, d->n_tris, p, 1, &id, &d2);
    return id;
}

void orc_canonical_map_soa(const orc_deform *d, const float *pts, int64_t n, int32_t *out_idx, float *out_canon) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        int32_t id = nearest_one(d, &pts[i * 3]);
        out_idx[i] = id;
        if (id < 0) { memcpy(&out_canon[i * 3], &pts[i * 3], 12); continue; }
        if (d->fp64) map_with_triangle_d(d, id, &pts[i * 3], NULL, &out_canon[i * 3], NULL);
        else map_with_triangle_f(d, id, &pts[i * 3], NULL, &out_canon[i * 3], NULL);
    }
}

/* warp kernel (src/core.cu:442-526) over NerfCoordinate records (NGP/nerf.h:86-115):
 * pos[0..2], dt[3], holder[4], deformed_pos[5..7], dir[8..10], extra dims at the end.
 * frame_id < 0 takes the frame from `holder` (surface_closest_point); this oracle holds one
 * frame, so records naming another frame are left untouched. */
static void map_coord(const orc_deform *d, float *c, uint32_t stride, uint32_t n_extra, int32_t frame_id, uint32_t n_frames) {
    if (c[4] < 0.f) return;
    uint32_t fid = frame_id < 0 ? (uint32_t)c[4] : (uint32_t)frame_id;
    if (fid >= n_frames) return;
    if (!box_contains(d->aabb_min, d->aabb_max, c)) return;
    int32_t id = nearest_one(d, c);
    if (id < 0) return;
    float pos[3], dir[3];
    if (d->fp64) map_with_triangle_d(d, id, c, &c[8], pos, dir);
    else map_with_triangle_f(d, id, c, &c[8], pos, dir);
    memcpy(c, pos, 12);
    memcpy(&c[8], dir, 12);
    if (d->def_tris[id].mask_id != 7u)
        for (uint32_t m = 0; m < n_extra; ++m) c[stride - n_extra + m] = 1.f;
}

void orc_canonical_map_coords(const orc_deform *d, float *coords, uint32_t stride, uint32_t n_extra, int64_t n,
                              int32_t frame_id, uint32_t n_frames) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) map_coord(d, &coords[i * stride], stride, n_extra, frame_id, n_frames);
}

/* ------------------------------------------------------------- occupancy */
static uint32_t expand_bits(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
uint32_t orc_morton3d(uint32_t x, uint32_t y, uint32_t z) { return expand_bits(x) | (expand_bits(y) << 1) | (expand_bits(z) << 2); }
static uint32_t morton_invert(uint32_t x) {
    x = x & 0x49249249u;
    x = (x | (x >> 2)) & 0xc30c30c3u;
    x = (x | (x >> 4)) & 0x0f00f00fu;
    x = (x | (x >> 8)) & 0xff0000ffu;
    x = (x | (x >> 16)) & 0x0000ffffu;
    return x;
}

#define GRID 128u
#define GRID3 (GRID * GRID * GRID)

/* mark_flame_density_grid (ngp/src/testbed_nerf.cu:364-389) on the deformed mesh, then
 * grid_to_bitfield (:585-609, threshold min(0.01, mean) which keeps exactly the marked cells)
 * and bitfield_max_pool for mips 1..7 (:611-632).  bitfield: 8 * 128^3 / 8 bytes. */
void orc_occupancy_from_mesh(const orc_tri *tris, int n_tris, double radius, uint8_t *bitfield) {
    memset(bitfield, 0, GRID3 / 8 * 8);
    orc_tri *sorted = malloc(sizeof(orc_tri) * (size_t)n_tris);
    int max_nodes = 2 * n_tris + 16;
    orc_bvh_node *nodes = malloc(sizeof(orc_bvh_node) * (size_t)max_nodes);
    orc_bvh4_build(tris, n_tris, 2, nodes, max_nodes, sorted);
    uint8_t *mark = calloc(GRID3, 1);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < (int64_t)GRID3; ++i) {
        uint32_t x = morton_invert((uint32_t)i >> 0), y = morton_invert((uint32_t)i >> 1), z = morton_invert((uint32_t)i >> 2);
        float p[3] = {((float)x + 0.5f) / (float)GRID, ((float)y + 0.5f) / (float)GRID, ((float)z + 0.5f) / (float)GRID};
        for (int k = 0; k < 3; ++k) p[k] = (p[k] - 0.5f) * 1.0f + 0.5f;
        int32_t id; float d2;
        orc_nearest_bvh(nodes, sorted, p, 1, 1, &id, &d2);
        if (id >= 0 && (double)sqrtf(d2) < radius && tris[id].mask_id != 0u) mark[i] = 1;
    }
    for (uint32_t b = 0; b < GRID3 / 8; ++b) {
        uint8_t bits = 0;
        for (int j = 0; j < 8; ++j) bits |= mark[b * 8 + j] ? (uint8_t)(1u << j) : 0;
        bitfield[b] = bits;
    }
    for (uint32_t level = 1; level < 8; ++level) {
        const uint8_t *prev = bitfield + (size_t)(level - 1) * GRID3 / 8;
        uint8_t *next = bitfield + (size_t)level * GRID3 / 8;
        for (uint32_t i = 0; i < GRID3 / 64; ++i) {
            uint8_t bits = 0;
            for (int j = 0; j < 8; ++j) bits |= prev[i * 8 + j] > 0 ? (uint8_t)(1u << j) : 0;
            uint32_t x = morton_invert(i >> 0) + GRID / 8, y = morton_invert(i >> 1) + GRID / 8, z = morton_invert(i >> 2) + GRID / 8;
            next[orc_morton3d(x, y, z)] |= bits;
        }
    }
    free(mark); free(nodes); free(sorted);
}

/* update_density_grid_mean_and_bitfield (ngp/src/testbed_nerf.cu:2863-2878): the mean over
 * cascade 0 of max(v, 0) / 128^3 (terms in float, summed in double), grid_to_bitfield (:585-609)
 * with threshold min(0.01, mean) over the n_cascades given cascades (the bytes of the others are
 * 0), then bitfield_max_pool (:611-632), which ORs each pooled mip into the next mip's own bits.
 * grid: n_cascades * 128^3 floats, Morton order per cascade.  Returns the threshold. */
float orc_density_grid_to_bitfield(const float *grid, uint32_t n_cascades, uint8_t *bitfield) {
    double sum = 0.0;
    for (uint32_t i = 0; i < GRID3; ++i) sum += (double)(fmaxf(grid[i], 0.f) / (float)GRID3);
    const float mean = (float)sum;
    const float thresh = mean < 0.01f ? mean : 0.01f;
    for (uint32_t b = 0; b < GRID3 / 8 * 8; ++b) {
        uint8_t bits = 0;
        if (b < GRID3 / 8 * n_cascades)
            for (int j = 0; j < 8; ++j) bits |= grid[(size_t)b * 8 + j] > thresh ? (uint8_t)(1u << j) : 0;
        bitfield[b] = bits;
    }
    for (uint32_t level = 1; level < 8; ++level) {
        const uint8_t *prev = bitfield + (size_t)(level - 1) * GRID3 / 8;
        uint8_t *next = bitfield + (size_t)level * GRID3 / 8;
        for (uint32_t i = 0; i < GRID3 / 64; ++i) {
            uint8_t bits = 0;
            for (int j = 0; j < 8; ++j) bits |= prev[i * 8 + j] > 0 ? (uint8_t)(1u << j) : 0;
            uint32_t x = morton_invert(i >> 0) + GRID / 8, y = morton_invert(i >> 1) + GRID / 8, z = morton_invert(i >> 2) + GRID / 8;
            next[orc_morton3d(x, y, z)] |= bits;
        }
    }
    return thresh;
}

/* ------------------------------------------------ density-grid maintenance */
uint32_t orc_pcg32_next_uint(orc_pcg32 *r) {
    const uint64_t old = r->state;
    r->state = old * 0x5851f42d4c957f2dull + r->inc;
    const uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((~rot + 1u) & 31u));
}

float orc_pcg32_next_float(orc_pcg32 *r) {
    const uint32_t bits = (orc_pcg32_next_uint(r) >> 9) | 0x3f800000u;
    float f;
    memcpy(&f, &bits, 4);
    return f - 1.0f;
}

void orc_pcg32_advance(orc_pcg32 *r, int64_t delta_) {
    uint64_t cur_mult = 0x5851f42d4c957f2dull, cur_plus = r->inc, acc_mult = 1u, acc_plus = 0u;
    uint64_t delta = (uint64_t)delta_;
    while (delta > 0) {
        if (delta & 1) {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1) * cur_plus;
        cur_mult *= cur_mult;
        delta /= 2;
    }
    r->state = acc_mult * r->state + acc_plus;
}

void orc_pcg32_seed(orc_pcg32 *r, uint64_t initstate, uint64_t initseq) {
    r->state = 0u;
    r->inc = (initseq << 1u) | 1u;
    orc_pcg32_next_uint(r);
    r->state += initstate;
    orc_pcg32_next_uint(r);
}

void orc_grid_samples(uint32_t n_uniform, uint32_t n_nonuniform, orc_pcg32 rng, uint32_t step, const float *aabb_min,
                      const float *aabb_max, const float *grid, uint32_t n_cascades, float *out_pos, uint32_t *out_idx) {
    const uint32_t n = n_uniform + n_nonuniform;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
        const uint32_t i = (uint32_t)ii;
        const int uniform = i < n_uniform;
        const uint32_t li = uniform ? i : i - n_uniform, ne = uniform ? n_uniform : n_nonuniform;
        const float thresh = uniform ? -0.01f : 0.01f;
        orc_pcg32 r = rng;
        orc_pcg32_advance(&r, (int64_t)(uint32_t)(li * 4u));
        const uint32_t level = (uint32_t)(orc_pcg32_next_float(&r) * (float)n_cascades) % n_cascades;
        uint32_t idx = 0;
        for (uint32_t j = 0; j < 10; ++j) {
            idx = ((li + step * ne) * 56924617u + j * 19349663u + 96925573u) % GRID3;
            idx += level * GRID3;
            if (grid[idx] > thresh) break;
        }
        const uint32_t cell = idx % GRID3;
        const float cc[3] = {(float)morton_invert(cell), (float)morton_invert(cell >> 1), (float)morton_invert(cell >> 2)};
        float rr[3];
        for (int k = 0; k < 3; ++k) rr[k] = orc_pcg32_next_float(&r);
        const float scale = scalbnf(1.0f, (int)level);
        for (int k = 0; k < 3; ++k) {
            const float pos = ((cc[k] + rr[k]) / (float)GRID - 0.5f) * scale + 0.5f;
            out_pos[(size_t)i * 3 + k] = (pos - aabb_min[k]) / (aabb_max[k] - aabb_min[k]);
        }
        out_idx[i] = idx;
    }
}

void orc_warp_random_samples(const orc_deform *frames, uint32_t n_frames, orc_pcg32 rng, float *pos, int64_t n, uint32_t *out_frame) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        orc_pcg32 r = rng;
        orc_pcg32_advance(&r, (int64_t)(uint32_t)((uint32_t)i * n_frames));
        const uint32_t fid = (uint32_t)(orc_pcg32_next_float(&r) * (float)n_frames);
        if (out_frame) out_frame[i] = fid;
        if (fid >= n_frames) continue;
        const orc_deform *d = &frames[fid];
        float *p = &pos[i * 3];
        const int32_t id = nearest_one(d, p);
        if (id < 0) continue;
        float o[3];
        if (d->fp64) map_with_triangle_d(d, id, p, NULL, o, NULL);
        else map_with_triangle_f(d, id, p, NULL, o, NULL);
        memcpy(p, o, 12);
    }
}

/* ------------------------------------------------- low-discrepancy jitter */
/* Sobol direction numbers for dimensions 0 and 1 (van der Corput and the x+1 primitive
 * polynomial), generated by the standard recurrence (NGP/random_val.cuh:159-216 uses the
 * same sequence). */
uint32_t orc_sobol(uint32_t index, uint32_t dim) {
    uint32_t X = 0, v = 0x80000000u;
    for (uint32_t bit = 0; bit < 32; ++bit) {
        uint32_t dirn = (dim == 0) ? (0x80000000u >> bit) : v;
        if ((index >> bit) & 1u) X ^= dirn;
        v = v ^ (v >> 1);
    }
    return X;
}
static uint32_t hash_combine(uint32_t seed, uint32_t v) { return seed ^ (v + (seed << 6) + (seed >> 2)); }
static uint32_t reverse_bits(uint32_t x) {
    x = ((x & 0xaaaaaaaau) >> 1) | ((x & 0x55555555u) << 1);
    x = ((x & 0xccccccccu) >> 2) | ((x & 0x33333333u) << 2);
    x = ((x & 0xf0f0f0f0u) >> 4) | ((x & 0x0f0f0f0fu) << 4);
    x = ((x & 0xff00ff00u) >> 8) | ((x & 0x00ff00ffu) << 8);
    return (x >> 16) | (x << 16);
}
/* Laine-Karras style permutation (Burley 2020, "Practical Hash-based Owen Scrambling"). */
static uint32_t lk_permutation(uint32_t x, uint32_t seed) {
    x += seed;
    x ^= x * 0x6c50b47cu;
    x ^= x * 0xb82f1e52u;
    x ^= x * 0xc7afe638u;
    x ^= x * 0x8d22f6e6u;
    return x;
}
static uint32_t owen_scramble(uint32_t x, uint32_t seed) { return reverse_bits(lk_permutation(reverse_bits(x), seed)); }

/* ld_random_val (NGP/random_val.cuh:284-288). */
float orc_ld_random_val(uint32_t index, uint32_t seed, uint32_t dim) {
    const float S = (float)(1.0 / 4294967296.0);
    index = owen_scramble(index, seed);
    return (float)owen_scramble(orc_sobol(index, dim), hash_combine(seed, dim)) * S;
}
/* ld_random_pixel_offset (NGP/random_val.cuh:317-322). */
void orc_ld_random_pixel_offset(uint32_t spp, float out[2]) {
    const float S = (float)(1.0 / 4294967296.0);
    uint32_t i0 = owen_scramble(0, 0xdeadbeefu), i1 = owen_scramble(spp, 0xdeadbeefu);
    for (uint32_t d = 0; d < 2; ++d) {
        float v0 = (float)owen_scramble(orc_sobol(i0, d), hash_combine(0xdeadbeefu, d)) * S;
        float v1 = (float)owen_scramble(orc_sobol(i1, d), hash_combine(0xdeadbeefu, d)) * S;
        float o = (0.5f - v0) + v1;
        out[d] = o - floorf(o);
    }
}

/* ------------------------------------------------------------------ march */
#define SQRT3F 1.73205080757f
#define STEPSIZE (SQRT3F / 1024.0f)
#define MIN_CONE STEPSIZE
#define MAX_CONE (STEPSIZE * 128.0f * 1024.0f / 128.0f)

/* calc_dt (ngp/src/testbed_nerf.cu:91-93) */
static inline float calc_dt(float t, float cone) { return clampf_(t * cone, MIN_CONE, MAX_CONE); }
/* warp_dt / unwarp_dt (:303-311) */
static inline float warp_dt(float dt) { float mx = MIN_CONE * 128.0f; return (dt - MIN_CONE) / (mx - MIN_CONE); }
static inline float unwarp_dt(float dt) { float mx = MIN_CONE * 128.0f; return dt * (mx - MIN_CONE) + MIN_CONE; }

/* mip_from_pos / mip_from_dt (:471-485), max_cascade = 7 */
static inline int mip_from_pos(const float *p) {
    float m = fabsf(p[0] - 0.5f);
    float a1 = fabsf(p[1] - 0.5f), a2 = fabsf(p[2] - 0.5f);
    if (a1 > m) m = a1;
    if (a2 > m) m = a2;
    int e; frexpf(m, &e);
    int v = e + 1 > 0 ? e + 1 : 0;
    return v < 6 ? v : 6;
}
static inline int mip_from_dt(float dt, const float *p) {
    int mip = mip_from_pos(p);
    dt *= 2.0f * 128.0f;
    if (dt < 1.f) return mip;
    int e; frexpf(dt, &e);
    int v = e > mip ? e : mip;
    return v < 6 ? v : 6;
}
/* cascaded_grid_idx_at / density_grid_occupied_at (:313-337) */
static inline int occupied_at(const float *pos, const uint8_t *bf, int mip) {
    float s = scalbnf(1.0f, -mip);
    int ii[3];
    for (int k = 0; k < 3; ++k) {
        float q = pos[k] - 0.5f;
        q *= s;
        q += 0.5f;
        int v = (int)(q * 128.0f);
        ii[k] = v < 0 ? 0 : (v > 127 ? 127 : v);
    }
    uint32_t idx = orc_morton3d((uint32_t)ii[0], (uint32_t)ii[1], (uint32_t)ii[2]);
    return (bf[idx / 8 + (size_t)mip * GRID3 / 8] >> (idx % 8)) & 1;
}
/* distance_to_next_voxel / advance_to_next_voxel (:186-208) */
static inline float advance_to_next_voxel(float t, float cone, const float *pos, const float *dir, const float *idir, uint32_t res) {
    float fr = (float)res, tt[3];
    for (int k = 0; k < 3; ++k) {
        float p = fr * pos[k];
        tt[k] = (floorf(p + 0.5f + 0.5f * ngp_sign(dir[k])) - p) * idir[k];
    }
    float tm = tt[0] < tt[1] ? tt[0] : tt[1];
    tm = tm < tt[2] ? tm : tt[2];
    float dist = fmaxf(tm / fr, 0.0f);
    float target = t + dist;
    do { t += calc_dt(t, cone); } while (t < target);
    return t;
}

/* The march helpers above behind the C ABI, for the pin against the reference's own
 * (oracle/ref_march_probe.cpp). */
float orc_probe_calc_dt(float t, float cone) { return calc_dt(t, cone); }
float orc_probe_warp_dt(float dt) { return warp_dt(dt); }
float orc_probe_unwarp_dt(float dt) { return unwarp_dt(dt); }
int orc_probe_mip_from_dt(float dt, const float *pos) { return mip_from_dt(dt, pos); }
int orc_probe_occupied_at(const float *pos, const uint8_t *bf, int mip) { return occupied_at(pos, bf, mip); }
float orc_probe_advance_to_next_voxel(float t, float cone, const float *pos, const float *dir, const float *idir, uint32_t res) {
    return advance_to_next_voxel(t, cone, pos, dir, idir, res);
}

/* BoundingBox::ray_intersect (NGP/bounding_box.cuh:163-210), returns tmin or FLT_MAX */
static float aabb_ray_tmin(const float *mn, const float *mx, const float *o, const float *d) {
    float tmin = (mn[0] - o[0]) / d[0], tmax = (mx[0] - o[0]) / d[0];
    if (tmin > tmax) { float t = tmin; tmin = tmax; tmax = t; }
    float tymin = (mn[1] - o[1]) / d[1], tymax = (mx[1] - o[1]) / d[1];
    if (tymin > tymax) { float t = tymin; tymin = tymax; tymax = t; }
    if (tmin > tymax || tymin > tmax) return FLT_MAX;
    if (tymin > tmin) tmin = tymin;
    if (tymax < tmax) tmax = tymax;
    float tzmin = (mn[2] - o[2]) / d[2], tzmax = (mx[2] - o[2]) / d[2];
    if (tzmin > tzmax) { float t = tzmin; tzmin = tzmax; tzmax = t; }
    if (tmin > tzmax || tzmin > tmax) return FLT_MAX;
    if (tzmin > tmin) tmin = tzmin;
    return tmin;
}

typedef struct { float o[3], d[3], idir[3], t; int alive; } ray_state;

/* init_rays_with_payload_kernel_nerf (:1854-1963) + pixel_to_ray (NGP/common_device.cuh:260-315)
 * + advance_pos_nerf (:634-686) for one pixel. */
static void ray_init(const orc_render_cfg *rc, const uint8_t *bf, int x, int y, ray_state *r) {
    float off[2];
    orc_ld_random_pixel_offset(rc->snap_to_pixel_centers ? 0u : rc->spp, off);
    float u = ((float)x + off[0]) / (float)rc->width, v = ((float)y + off[1]) / (float)rc->height;
    float dc[3] = {(u - rc->screen_center[0]) * (float)rc->width / rc->focal[0],
                   (v - rc->screen_center[1]) * (float)rc->height / rc->focal[1], 1.0f};
    float d[3];
    for (int k = 0; k < 3; ++k) { const float *row = &rc->cam[k * 4]; float rr[3] = {row[0], row[1], row[2]}; d[k] = v3dot(rr, dc); }
    float z = v3dot(d, d);
    if (z > 0.f) { float s = sqrtf(z); d[0] /= s; d[1] /= s; d[2] /= s; }
    for (int k = 0; k < 3; ++k) { r->o[k] = rc->cam[k * 4 + 3]; r->d[k] = d[k]; r->idir[k] = 1.0f / d[k]; }
    float tm = aabb_ray_tmin(rc->render_aabb_min, rc->render_aabb_max, r->o, r->d);
    float t = fmaxf(tm, 0.05f) + 1e-6f;
    float p[3];
    for (int k = 0; k < 3; ++k) p[k] = r->o[k] + r->d[k] * t;
    r->alive = box_contains(rc->render_aabb_min, rc->render_aabb_max, p);
    if (!r->alive) return;
    uint32_t idx = (uint32_t)x + (uint32_t)rc->width * (uint32_t)y;
    float dt = calc_dt(t, rc->cone_angle);
    t += orc_ld_random_val(rc->spp, idx * 786433u, 0) * dt;
    for (;;) {
        for (int k = 0; k < 3; ++k) p[k] = r->o[k] + r->d[k] * t;
        if (!box_contains(rc->render_aabb_min, rc->render_aabb_max, p)) { r->alive = 0; break; }
        dt = calc_dt(t, rc->cone_angle);
        int mip = mip_from_dt(dt, p);
        if (!bf || occupied_at(p, bf, mip)) break;
        uint32_t res = GRID >> mip;
        t = advance_to_next_voxel(t, rc->cone_angle, p, r->d, r->idir, res);
    }
    r->t = t;
}

/* One step of generate_next_nerf_network_inputs (:760-791): march to the next occupied sample;
 * returns 0 when the ray leaves the render box. */
static int ray_next_sample(const orc_render_cfg *rc, const uint8_t *bf, ray_state *r, float *pos, float *dt_out, float *t_out) {
    float t = r->t, dt = 0.f;
    for (;;) {
        for (int k = 0; k < 3; ++k) pos[k] = r->o[k] + r->d[k] * t;
        if (!box_contains(rc->render_aabb_min, rc->render_aabb_max, pos)) { r->t = t; return 0; }
        dt = calc_dt(t, rc->cone_angle);
        int mip = mip_from_dt(dt, pos);
        if (!bf || occupied_at(pos, bf, mip)) break;
        uint32_t res = GRID >> mip;
        t = advance_to_next_voxel(t, rc->cone_angle, pos, r->d, r->idir, res);
    }
    *dt_out = dt;
    if (t_out) *t_out = t;
    r->t = t + dt;
    return 1;
}

/* ------------------------------------------------------------ raycast (visualisation) */
/* Triangle::ray_intersect (NGP/triangle.cuh:66-80), FLT_MAX for a miss. */
static float tri_ray_t(const orc_tri *tr, const float *ro, const float *rd) {
    float v1v0[3], v2v0[3], rov0[3];
    for (int k = 0; k < 3; ++k) { v1v0[k] = tr->b[k] - tr->a[k]; v2v0[k] = tr->c[k] - tr->a[k]; rov0[k] = ro[k] - tr->a[k]; }
    const float n[3] = {v1v0[1] * v2v0[2] - v1v0[2] * v2v0[1], v1v0[2] * v2v0[0] - v1v0[0] * v2v0[2], v1v0[0] * v2v0[1] - v1v0[1] * v2v0[0]};
    const float q[3] = {rov0[1] * rd[2] - rov0[2] * rd[1], rov0[2] * rd[0] - rov0[0] * rd[2], rov0[0] * rd[1] - rov0[1] * rd[0]};
    const float d = 1.0f / v3dot(rd, n);
    const float u = d * -v3dot(q, v2v0);
    const float v = d * v3dot(q, v1v0);
    float t = d * -v3dot(n, rov0);
    if (u < 0.0f || u > 1.0f || v < 0.0f || (u + v) > 1.0f || t < 0.0f) t = FLT_MAX;
    return t;
}

static float srgb_to_linear_f(float s) { return s <= 0.04045f ? s / 12.92f : powf((s + 0.055f) / 1.055f, 2.4f); }

/* rta::Core::raycast_flame (src/core.cu:350-402): init_rays_with_payload_kernel_sdf
 * (ngp/src/testbed_sdf.cu:505-577, no slice plane, no octree), the closest hit of
 * TriangleBvh4::ray_intersect (ngp/src/triangle_bvh.cu:271-311, hits at t < 10, ties to the lowest
 * triangle id) and INSTA's shade_kernel_sdf (src/core.cu:74-113).  Pixels whose hit point is
 * outside the render box (or without a hit) keep their values; out_tri gets -1 there. */
void orc_raycast(const orc_render_cfg *rc, const orc_tri *tris, int n_tris, const float *center, int color_normal, float *out_rgba,
                 float *out_depth, int32_t *out_tri) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t pix = 0; pix < (int64_t)rc->width * rc->height; ++pix) {
        const int x = (int)(pix % rc->width), y = (int)(pix / rc->width);
        float off[2];
        orc_ld_random_pixel_offset(rc->snap_to_pixel_centers ? 0u : rc->spp, off);
        const float u = ((float)x + off[0]) / (float)rc->width, v = ((float)y + off[1]) / (float)rc->height;
        const float dc[3] = {(u - rc->screen_center[0]) * (float)rc->width / rc->focal[0],
                             (v - rc->screen_center[1]) * (float)rc->height / rc->focal[1], 1.0f};
        float d[3], o[3];
        for (int k = 0; k < 3; ++k) { const float *row = &rc->cam[k * 4]; float rr[3] = {row[0], row[1], row[2]}; d[k] = v3dot(rr, dc); }
        const float z = v3dot(d, d);
        if (z > 0.f) { const float sz = sqrtf(z); d[0] /= sz; d[1] /= sz; d[2] /= sz; }
        for (int k = 0; k < 3; ++k) o[k] = rc->cam[k * 4 + 3];
        const float tm = aabb_ray_tmin(rc->render_aabb_min, rc->render_aabb_max, o, d);
        const float t0 = fmaxf(tm, 0.0f) + 1e-6f;
        for (int k = 0; k < 3; ++k) o[k] = o[k] + t0 * d[k];
        float best = 10.0f;   /* MAX_DIST */
        int32_t bid = -1;
        for (int t = 0; t < n_tris; ++t) {
            const float tt = tri_ray_t(&tris[t], o, d);
            if (tt < best || (tt == best && bid >= 0 && (uint32_t)tris[t].id < (uint32_t)bid)) { best = tt; bid = (int32_t)tris[t].id; }
        }
        float pos[3];
        for (int k = 0; k < 3; ++k) pos[k] = o[k] + best * d[k];
        if (bid < 0 || !box_contains(rc->render_aabb_min, rc->render_aabb_max, pos)) { if (out_tri) out_tri[pix] = -1; continue; }
        if (out_tri) out_tri[pix] = bid;
        const orc_tri *tr = NULL;
        for (int t = 0; t < n_tris; ++t) if ((int32_t)tris[t].id == bid) { tr = &tris[t]; break; }
        float e1[3], e2[3];
        for (int k = 0; k < 3; ++k) { e1[k] = tr->b[k] - tr->a[k]; e2[k] = tr->c[k] - tr->a[k]; }
        float nrm[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        for (int rep = 0; rep < 2; ++rep) {   /* Triangle::normal(), then the shader's normalized() */
            const float nz = v3dot(nrm, nrm);
            if (nz > 0.f) { const float s = sqrtf(nz); nrm[0] /= s; nrm[1] /= s; nrm[2] /= s; }
        }
        float col[3];
        if (color_normal) {
            for (int k = 0; k < 3; ++k) col[k] = srgb_to_linear_f(0.5f * nrm[k] + 0.5f);
        } else {
            const float lo[3][3] = {{0.f, 0.f, 1.f}, {1.5f, 0.25f, 0.5f}, {-1.5f, 0.25f, 0.5f}};
            float cs[3] = {0.f, 0.f, 0.f};
            for (int l = 0; l < 3; ++l) {
                const float light[3] = {center[0] + lo[l][0], center[1] + lo[l][1], center[2] + lo[l][2]};
                const float w = (1 / 3.f) * fminf(1.f, fmaxf(v3dot(nrm, light), 0.f));
                for (int k = 0; k < 3; ++k) cs[k] += w * 0.75f;
            }
            for (int k = 0; k < 3; ++k) col[k] = srgb_to_linear_f(cs[k]);
        }
        out_rgba[pix * 4 + 0] = col[0]; out_rgba[pix * 4 + 1] = col[1]; out_rgba[pix * 4 + 2] = col[2]; out_rgba[pix * 4 + 3] = 1.0f;
        out_depth[pix] = pos[2];
    }
}

int orc_march_ray(const orc_render_cfg *rc, const uint8_t *bf, int px, int py, int max_out, float *out_t, float *out_dt,
                  float *out_pos) {
    ray_state r;
    ray_init(rc, bf, px, py, &r);
    if (!r.alive) return 0;
    int n = 0;
    while (n < max_out && n < (int)rc->max_samples_per_ray) {
        float pos[3], dt, ts;
        if (!ray_next_sample(rc, bf, &r, pos, &dt, &ts)) break;
        out_t[n] = ts;
        out_dt[n] = dt;
        memcpy(&out_pos[n * 3], pos, 12);
        ++n;
    }
    return n;
}

/* generate_training_samples_nerf (ngp/src/testbed_nerf.cu:1105-1285) on caller-supplied rays:
 * rays [n][6] (origin, unnormalised direction), image[n] (written to `holder`), start_rand[n]
 * (the uniform draw of the start jitter), extra [n_images][n_extra] or NULL.  Rays are taken in
 * index order, so each ray's block of samples follows the previous one (the device reserves
 * blocks with atomics in arbitrary order; compare per ray).  counters: [0] rays kept,
 * [1] samples requested (as the reference's numsteps counter). */
void orc_training_samples(const float *aabb_min, const float *aabb_max, float cone, const uint8_t *bf, const float *rays,
                          const uint32_t *image, const float *start_rand, const float *extra, uint32_t n_extra, int64_t n,
                          uint32_t max_samples, float *coords, uint32_t stride, uint32_t *ray_indices, uint32_t *numsteps,
                          uint32_t *counters) {
    counters[0] = counters[1] = 0;
    for (int64_t i = 0; i < n; ++i) {
        const float *r = rays + i * 6;
        float o[3] = {r[0], r[1], r[2]}, d[3] = {r[3], r[4], r[5]};
        float z = v3dot(d, d);
        if (z > 0.f) { float sq = sqrtf(z); d[0] /= sq; d[1] /= sq; d[2] /= sq; }
        float idir[3] = {1.0f / d[0], 1.0f / d[1], 1.0f / d[2]};
        float startt = fmaxf(aabb_ray_tmin(aabb_min, aabb_max, o, d), 0.0f);
        startt += calc_dt(startt, cone) * start_rand[i];
        uint32_t j = 0;
        float t = startt, pos[3];
        for (int guard = 0; guard < (1 << 16) && j < 1024u; ++guard) {
            for (int k = 0; k < 3; ++k) pos[k] = o[k] + d[k] * t;
            if (!box_contains(aabb_min, aabb_max, pos)) break;
            float dt = calc_dt(t, cone);
            int mip = mip_from_dt(dt, pos);
            if (occupied_at(pos, bf, mip)) { ++j; t += dt; }
            else t = advance_to_next_voxel(t, cone, pos, d, idir, GRID >> mip);
        }
        if (j == 0) continue;
        uint32_t base = counters[1];
        counters[1] += j;
        if (base + j > max_samples) continue;
        uint32_t ri = counters[0]++;
        ray_indices[ri] = (uint32_t)i;
        numsteps[2 * ri] = j;
        numsteps[2 * ri + 1] = base;
        float wd[3];
        for (int k = 0; k < 3; ++k) wd[k] = (d[k] + 1.0f) * 0.5f;
        t = startt;
        uint32_t w = 0;
        for (int guard = 0; guard < (1 << 16) && w < j; ++guard) {
            for (int k = 0; k < 3; ++k) pos[k] = o[k] + d[k] * t;
            if (!box_contains(aabb_min, aabb_max, pos)) break;
            float dt = calc_dt(t, cone);
            int mip = mip_from_dt(dt, pos);
            if (occupied_at(pos, bf, mip)) {
                float *c = coords + (size_t)(base + w) * stride;
                for (int k = 0; k < 3; ++k) { c[k] = (pos[k] - aabb_min[k]) / (aabb_max[k] - aabb_min[k]); c[5 + k] = c[k]; c[8 + k] = wd[k]; }
                c[3] = warp_dt(dt);
                c[4] = (float)image[i];
                for (uint32_t m = 0; m < n_extra; ++m) c[stride - n_extra + m] = extra ? extra[(size_t)image[i] * n_extra + m] : 0.f;
                ++w;
                t += dt;
            } else {
                t = advance_to_next_voxel(t, cone, pos, d, idir, GRID >> mip);
            }
        }
    }
}

static float srgb_to_linear(float s) { return s <= 0.04045f ? s / 12.92f : powf((s + 0.055f) / 1.055f, 2.4f); }
static double logistic_d(double x) { return 1.0 / (1.0 + exp(-x)); }

/* Full headless render of rows [row_begin, row_end): NerfTracer::trace (:2112-2244) with
 * render_deformed (src/core.cu:610-637), NerfNetwork inference and composite_kernel_nerf
 * (:797-1009), then shade_kernel_nerf (:1794-1827) into a zeroed frame buffer.  The result is
 * independent of the tracer's compaction schedule, so each ray is processed to completion.
 * Returns the number of network samples evaluated. */
int64_t orc_render(const orc_render_cfg *rc, const orc_deform *d, const uint8_t *bf, const orc_field_cfg *fc,
                   const uint16_t *params, const float *layer_scales, int row_begin, int row_end, float *out_rgba,
                   float *out_depth, uint32_t *out_nsamples, int fp64) {
    uint64_t lvl_off[64], mlp_off[3];
    uint32_t lvl_res[64], lvl_size[64];
    orc_field_layout(fc, lvl_off, lvl_res, lvl_size, mlp_off);
    static const float ones[32] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
    if (!layer_scales) layer_scales = ones;
    const uint32_t stride = 11 + fc->n_extra;
    const float cam_fwd[3] = {rc->cam[2], rc->cam[6], rc->cam[10]};
    const float cam_pos[3] = {rc->cam[3], rc->cam[7], rc->cam[11]};
    int64_t total = 0;
    const int W = rc->width;
    int64_t n_px = (int64_t)(row_end - row_begin) * W;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
    for (int64_t q = 0; q < n_px; ++q) {
        int x = (int)(q % W), y = row_begin + (int)(q / W);
        size_t pix = (size_t)(y - row_begin) * W + x;
        float *fb = &out_rgba[pix * 4];
        fb[0] = fb[1] = fb[2] = fb[3] = 0.f;
        out_depth[pix] = 1e10f;
        uint32_t ns = 0;
        ray_state r;
        ray_init(rc, bf, x, y, &r);
        if (r.alive) {
            float rgba_f[4] = {0, 0, 0, 0}, depth_f = 0.f, maxw_f = 0.f;
            double rgba_d[4] = {0, 0, 0, 0}, depth_d = 0.0, maxw_d = 0.0;
            while (ns < rc->max_samples_per_ray) {
                float pos[3], dt;
                if (!ray_next_sample(rc, bf, &r, pos, &dt, NULL)) break;
                float coord[64];
                for (int k = 0; k < 3; ++k) {
                    coord[k] = (pos[k] - rc->train_aabb_min[k]) / (rc->train_aabb_max[k] - rc->train_aabb_min[k]);
                    coord[5 + k] = coord[k];
                    coord[8 + k] = (r.d[k] + 1.0f) * 0.5f;
                }
                coord[3] = warp_dt(dt);
                coord[4] = (float)rc->frame_id;
                for (uint32_t m = 0; m < fc->n_extra; ++m) coord[11 + m] = rc->extra_dims ? rc->extra_dims[m] : 0.f;
                map_coord(d, coord, stride, fc->n_extra, rc->frame_id, (uint32_t)rc->frame_id + 1u);
                ++ns;
                float dpos[3];
                for (int k = 0; k < 3; ++k) dpos[k] = rc->train_aabb_min[k] + coord[5 + k] * (rc->train_aabb_max[k] - rc->train_aabb_min[k]);
                float dtu = unwarp_dt(coord[3]);
                float dp[3] = {dpos[0] - cam_pos[0], dpos[1] - cam_pos[1], dpos[2] - cam_pos[2]};
                int done = 0;
                if (fp64) {
                    double o4[4];
                    field_one_d(fc, params, layer_scales, lvl_off, lvl_res, lvl_size, mlp_off, coord, stride, o4);
                    double T = 1.0 - rgba_d[3];
                    double alpha = 1.0 - exp(-exp(o4[3]) * (double)dtu);
                    double w = alpha * T;
                    for (int k = 0; k < 3; ++k) rgba_d[k] += logistic_d(o4[k]) * w;
                    rgba_d[3] += w;
                    if (w > maxw_d) { maxw_d = w; depth_d = (double)v3dot(cam_fwd, dp); }
                    if (rgba_d[3] > 1.0 - (double)rc->min_transmittance) {
                        double a = rgba_d[3];
                        for (int k = 0; k < 4; ++k) rgba_d[k] /= a;
                        done = 1;
                    }
                } else {
                    float o4[4];
                    field_one_f(fc, params, layer_scales, lvl_off, lvl_res, lvl_size, mlp_off, coord, stride, o4);
                    float T = 1.f - rgba_f[3];
                    float alpha = 1.f - expf(-expf(o4[3]) * dtu);
                    float w = alpha * T;
                    for (int k = 0; k < 3; ++k) rgba_f[k] += (1.0f / (1.0f + expf(-o4[k]))) * w;
                    rgba_f[3] += w;
                    if (w > maxw_f) { maxw_f = w; depth_f = v3dot(cam_fwd, dp); }
                    if (rgba_f[3] > 1.0f - rc->min_transmittance) {
                        float a = rgba_f[3];
                        for (int k = 0; k < 4; ++k) rgba_f[k] /= a;
                        done = 1;
                    }
                }
                if (done) break;
            }
            float out4[4], dep;
            if (fp64) { for (int k = 0; k < 4; ++k) out4[k] = (float)rgba_d[k]; dep = (float)depth_d; }
            else { memcpy(out4, rgba_f, 16); dep = depth_f; }
            if (out4[3] > 0.001f) {
                if (!rc->linear_colors) for (int k = 0; k < 3; ++k) out4[k] = srgb_to_linear(out4[k]);
                memcpy(fb, out4, 16);
                if (out4[3] > 0.2f) out_depth[pix] = dep;
            }
        }
        if (out_nsamples) out_nsamples[pix] = ns;
        total += ns;
    }
    return total;
}

/* Field evaluation over NerfCoordinate records; out4[i*4 + k] = (r, g, b, raw density). */
void orc_field_eval(const orc_field_cfg *c, const uint16_t *params, const float *layer_scales, const float *coords,
                    uint32_t stride, int64_t n, float *out4, int fp64) {
    uint64_t lvl_off[64], mlp_off[3];
    uint32_t lvl_res[64], lvl_size[64];
    orc_field_layout(c, lvl_off, lvl_res, lvl_size, mlp_off);
    static const float ones[32] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
    if (!layer_scales) layer_scales = ones;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        if (fp64) {
            double o[4];
            field_one_d(c, params, layer_scales, lvl_off, lvl_res, lvl_size, mlp_off, &coords[i * stride], stride, o);
            for (int k = 0; k < 4; ++k) out4[i * 4 + k] = (float)o[k];
        } else {
            float o[4];
            field_one_f(c, params, layer_scales, lvl_off, lvl_res, lvl_size, mlp_off, &coords[i * stride], stride, o);
            memcpy(&out4[i * 4], o, 16);
        }
    }
}

/* NerfNetwork's backward (NGP/nerf_network.h:296-383) in FP64 from the FP16 parameters: for each
 * record the forward with its activations, then the gradient of sum_i dl_dout[i] . out4[i]
 * w.r.t. every parameter, ADDED to grad[n_params] (snapshot order).  Single-threaded. */
static void layer_fwd_d(const uint16_t *W, const double *x, int n_in, int n_out, double *y, int relu) {
    for (int o = 0; o < n_out; ++o) {
        double acc = 0;
        for (int i = 0; i < n_in; ++i) acc += (double)orc_h2f(W[(size_t)o * n_in + i]) * x[i];
        y[o] = (relu && acc < 0) ? 0 : acc;
    }
}
/* dy -> dx = W^T dy, dW += dy x^T; relu mask of x applied by the caller */
static void layer_bwd_d(const uint16_t *W, const double *x, int n_in, int n_out, const double *dy, double *dx, double *dW) {
    for (int i = 0; i < n_in; ++i) dx[i] = 0;
    for (int o = 0; o < n_out; ++o) {
        if (dy[o] == 0) continue;
        for (int i = 0; i < n_in; ++i) {
            dx[i] += (double)orc_h2f(W[(size_t)o * n_in + i]) * dy[o];
            dW[(size_t)o * n_in + i] += dy[o] * x[i];
        }
    }
}

void orc_field_backward(const orc_field_cfg *c, const uint16_t *params, const float *coords, uint32_t stride, int64_t n,
                        const float *dl_dout, double *grad, float *out4) {
    orc_field_backward_ex(c, params, coords, stride, n, dl_dout, grad, out4, NULL);
}

void orc_field_backward_ex(const orc_field_cfg *c, const uint16_t *params, const float *coords, uint32_t stride, int64_t n,
                           const float *dl_dout, double *grad, float *out4, double *dl_dextra) {
    uint64_t lvl_off[64], mlp_off[3];
    uint32_t lvl_res[64], lvl_size[64];
    orc_field_layout(c, lvl_off, lvl_res, lvl_size, mlp_off);
    const uint16_t *table = params + mlp_off[2];
    const uint32_t F = c->n_features, n_enc = c->n_levels * F, n_in = n_enc + c->n_extra;
    const uint32_t H = c->density_hidden, HR = c->rgb_hidden, DO = c->density_out, RI = c->density_out + 16;
    for (int64_t s = 0; s < n; ++s) {
        const float *coord = &coords[s * stride];
        double feat[256], hd[4][128], dens[64], rin[128], hr[5][128], rgb[64];
        uint32_t cidx[64][8];
        double cw[64][8];
        for (uint32_t l = 0; l < c->n_levels; ++l) {
            const float scale = orc_level_scale(c, l);
            float pos[3], fr[3];
            uint32_t g[3];
            for (int k = 0; k < 3; ++k) {
                pos[k] = fmaf(coord[k], scale, 0.5f);
                float fl = floorf(pos[k]);
                fr[k] = pos[k] - fl;
                g[k] = (uint32_t)(int32_t)fl;
            }
            double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            for (uint32_t corner = 0; corner < 8; ++corner) {
                double w = 1;
                uint32_t cc[3];
                for (int k = 0; k < 3; ++k) {
                    uint32_t bit = (corner >> k) & 1u;
                    cc[k] = g[k] + bit;
                    w = w * (bit ? (double)fr[k] : 1.0 - (double)fr[k]);
                }
                uint32_t idx = orc_grid_index(cc, lvl_res[l], lvl_size[l]);
                cidx[l][corner] = idx;
                cw[l][corner] = w;
                const uint16_t *e = table + (lvl_off[l] + (uint64_t)idx) * F;
                for (uint32_t f = 0; f < F; ++f) acc[f] += w * (double)orc_h2f(e[f]);
            }
            for (uint32_t f = 0; f < F; ++f) feat[l * F + f] = acc[f];
        }
        const float *extra = coord + stride - c->n_extra;
        for (uint32_t k = 0; k < c->n_extra; ++k) feat[n_enc + k] = extra[k];
        /* density MLP */
        const uint16_t *Wd[8];
        const uint16_t *W = params + mlp_off[0];
        const double *x = feat;
        uint32_t k_in = n_in;
        for (uint32_t h = 0; h < c->density_layers; ++h) {
            Wd[h] = W;
            layer_fwd_d(W, x, (int)k_in, (int)H, hd[h], 1);
            W += (size_t)H * k_in;
            x = hd[h];
            k_in = H;
        }
        Wd[c->density_layers] = W;
        layer_fwd_d(W, x, (int)H, (int)DO, dens, 0);
        /* SH */
        double X = (double)coord[8] * 2 - 1, Y = (double)coord[9] * 2 - 1, Z = (double)coord[10] * 2 - 1;
        double xx = X * X, yy = Y * Y, zz = Z * Z, sh[16];
        sh[0] = 0.28209479177387814; sh[1] = -0.48860251190291987 * Y; sh[2] = 0.48860251190291987 * Z;
        sh[3] = -0.48860251190291987 * X; sh[4] = 1.0925484305920792 * X * Y; sh[5] = -1.0925484305920792 * Y * Z;
        sh[6] = 0.94617469575755997 * zz - 0.31539156525251999; sh[7] = -1.0925484305920792 * X * Z;
        sh[8] = 0.54627421529603959 * (xx - yy); sh[9] = 0.59004358992664352 * Y * (-3 * xx + yy);
        sh[10] = 2.8906114426405538 * X * Y * Z; sh[11] = 0.45704579946446572 * Y * (1 - 5 * zz);
        sh[12] = 0.3731763325901154 * Z * (5 * zz - 3); sh[13] = 0.45704579946446572 * X * (1 - 5 * zz);
        sh[14] = 1.4453057213202769 * Z * (xx - yy); sh[15] = 0.59004358992664352 * X * (-xx + 3 * yy);
        for (uint32_t k = 0; k < DO; ++k) rin[k] = dens[k];
        for (uint32_t k = 0; k < 16; ++k) rin[DO + k] = sh[k];
        /* colour MLP */
        const uint16_t *Wr[8];
        W = params + mlp_off[1];
        x = rin;
        k_in = RI;
        for (uint32_t h = 0; h < c->rgb_layers; ++h) {
            Wr[h] = W;
            layer_fwd_d(W, x, (int)k_in, (int)HR, hr[h], 1);
            W += (size_t)HR * k_in;
            x = hr[h];
            k_in = HR;
        }
        Wr[c->rgb_layers] = W;
        layer_fwd_d(W, x, (int)HR, (int)c->rgb_out_padded, rgb, 0);
        if (out4) { out4[s * 4] = (float)rgb[0]; out4[s * 4 + 1] = (float)rgb[1]; out4[s * 4 + 2] = (float)rgb[2]; out4[s * 4 + 3] = (float)dens[0]; }
        if (!dl_dout || !grad) continue;
        /* backward */
        double dy[128], dx[256];
        for (uint32_t k = 0; k < c->rgb_out_padded; ++k) dy[k] = k < 3 ? (double)dl_dout[s * 4 + k] : 0.0;
        uint32_t n_out = c->rgb_out_padded;
        for (int h = (int)c->rgb_layers; h >= 0; --h) {
            const double *xin = h == 0 ? rin : hr[h - 1];
            const uint32_t kk = h == 0 ? RI : HR;
            layer_bwd_d(Wr[h], xin, (int)kk, (int)n_out, dy, dx, grad + (Wr[h] - params));
            if (h > 0) for (uint32_t i = 0; i < kk; ++i) dy[i] = hr[h - 1][i] > 0 ? dx[i] : 0.0;
            else for (uint32_t i = 0; i < kk; ++i) dy[i] = dx[i];
            n_out = kk;
        }
        /* dy = dL/d rin; density output gradient = rows 0..DO-1, plus the raw density's own */
        dy[0] += (double)dl_dout[s * 4 + 3];
        n_out = DO;
        for (int h = (int)c->density_layers; h >= 0; --h) {
            const double *xin = h == 0 ? feat : hd[h - 1];
            const uint32_t kk = h == 0 ? n_in : H;
            layer_bwd_d(Wd[h], xin, (int)kk, (int)n_out, dy, dx, grad + (Wd[h] - params));
            if (h > 0) for (uint32_t i = 0; i < kk; ++i) dy[i] = hd[h - 1][i] > 0 ? dx[i] : 0.0;
            else for (uint32_t i = 0; i < kk; ++i) dy[i] = dx[i];
            n_out = kk;
        }
        /* dy = dL/d density input: the hash features, then the expression dims */
        if (dl_dextra)
            for (uint32_t k = 0; k < c->n_extra; ++k) dl_dextra[(size_t)s * c->n_extra + k] = dy[n_enc + k];
        /* hash table */
        double *gt = grad + mlp_off[2];
        for (uint32_t l = 0; l < c->n_levels; ++l)
            for (uint32_t corner = 0; corner < 8; ++corner)
                for (uint32_t f = 0; f < F; ++f) gt[(lvl_off[l] + (uint64_t)cidx[l][corner]) * F + f] += cw[l][corner] * dy[l * F + f];
    }
}

/* compute_loss_kernel_train_nerf (instant-ngp/src/testbed_nerf.cu:1305-1644) for rays in order
 * 0..n_kept-1, logistic rgb / exponential density, with the optional importance-sampling pdf and
 * error map (no envmap, sharpness grid or exposure gradient); then tiny-cuda-nn's fill_rollover(_and_rescale) restated from
 * its published source (train_nerf_step, :3349-3357): entries past the compacted count repeat the
 * compacted ones, the repeated gradients scaled by count / target.  Loss functions :116-180,
 * :1288-1303.  Single-threaded; the compacted bases follow ray order. */
static void loss_1(int type, float target, float pred, float *loss, float *grad) {
    const float d = pred - target;
    switch (type) {
    case 1: *loss = fabsf(d); *grad = copysignf(1.f, d); break;
    case 2: { float f = 1.f / (fabsf(pred) + 1e-2f); *loss = fabsf(d) * f; *grad = copysignf(f, d); } break;
    case 3: { float f = 1.f / (0.5f * (fabsf(pred) + fabsf(target)) + 1e-2f); *loss = fabsf(d) * f; *grad = copysignf(f, d); } break;
    case 4: { float a = 0.1f, ad = fabsf(d);
              *loss = (ad > a ? ad - 0.5f * a : 0.5f / a * d * d) / 5.f;
              *grad = (ad > a ? (d > 0 ? 1.f : -1.f) : d / a) / 5.f; } break;
    case 5: { float q = fabsf(d) + 1.f; *loss = logf(q); *grad = copysignf(1.f / q, d); } break;
    case 6: { float f = 1.f / (pred * pred + 1e-2f); *loss = d * d * f; *grad = 2.f * d * f; } break;
    default: *loss = d * d; *grad = 2.f * d; break;
    }
}
static float lin_to_srgb_f(float l) { return l < 0.0031308f ? 12.92f * l : 1.055f * powf(l, 0.41666f) - 0.055f; }
static float logistic_f(float x) { return 1.f / (1.f + expf(-x)); }

void orc_train_loss(const orc_train_loss_cfg *c, uint32_t n_kept, const float *rays, const float *target, const float *background,
                    const float *exposure, const float *depth_img, const int32_t *seg_mask, const float *mean_density,
                    const uint32_t *ray_indices, uint32_t *numsteps, const float *coords, const float *nout, uint32_t *counter,
                    float *coords_out, float *dloss, float *loss_out) {
    const float mx = MIN_CONE * 128.0f;
    float diag[3];
    for (int k = 0; k < 3; ++k) diag[k] = c->aabb_max[k] - c->aabb_min[k];
    for (uint32_t i = 0; i < n_kept; ++i) {
        const uint32_t ns = numsteps[2 * i], base = numsteps[2 * i + 1], ray = ray_indices[i];
        const float *R = rays + (size_t)ray * 6;
        const float *cin = coords + (size_t)base * c->stride, *o4 = nout + (size_t)base * 4;
        float T = 1.f, rgb_ray[3] = {0, 0, 0}, depth_ray = 0.f;
        uint32_t cn = 0;
        for (; cn < ns; ++cn) {
            if (T < 1e-4f) break;
            const float *cc = cin + (size_t)cn * c->stride, *o = o4 + (size_t)cn * 4;
            float p[3], dd = 0.f;
            for (int k = 0; k < 3; ++k) { p[k] = c->aabb_min[k] + cc[5 + k] * diag[k]; float t = p[k] - R[k]; dd += t * t; }
            const float dt = cc[3] * (mx - MIN_CONE) + MIN_CONE, cur = sqrtf(dd);
            const float alpha = 1.f - expf(-expf(o[3]) * dt), w = alpha * T;
            for (int k = 0; k < 3; ++k) rgb_ray[k] += w * logistic_f(o[k]);
            depth_ray += w * cur;
            T *= 1.f - alpha;
        }
        const float T_ray = T;
        const float *ts = target + (size_t)ray * 4, ta = ts[3];
        float bg[3], tgt[3], ex[3] = {1.f, 1.f, 1.f};
        for (int k = 0; k < 3; ++k) {
            bg[k] = srgb_to_linear_f(background ? background[(size_t)ray * 3 + k] : 0.f);
            if (exposure) ex[k] = expf(0.6931471805599453f * exposure[(size_t)ray * 3 + k]);
        }
        if (c->train_in_linear_colors || !c->srgb_targets) {
            for (int k = 0; k < 3; ++k) tgt[k] = ex[k] * ts[k] + (1.f - ta) * bg[k];
            if (!c->train_in_linear_colors) for (int k = 0; k < 3; ++k) { tgt[k] = lin_to_srgb_f(tgt[k]); bg[k] = lin_to_srgb_f(bg[k]); }
        } else {
            for (int k = 0; k < 3; ++k) bg[k] = lin_to_srgb_f(bg[k]);
            for (int k = 0; k < 3; ++k) tgt[k] = ta > 0.f ? lin_to_srgb_f(ex[k] * ts[k] / ta) * ta + (1.f - ta) * bg[k] : bg[k];
        }
        if (cn == ns) for (int k = 0; k < 3; ++k) rgb_ray[k] += T * bg[k];
        const uint32_t cbase = *counter;
        *counter += cn;
        const uint32_t mc = c->max_samples_compacted;
        const uint32_t ccount = (mc - (cbase < mc ? cbase : mc)) < cn ? (mc - (cbase < mc ? cbase : mc)) : cn;
        numsteps[2 * i] = ccount;
        numsteps[2 * i + 1] = cbase;
        if (ccount == 0) continue;
        float seg_sup = 1.f, dl = c->depth_supervision_lambda;
        if (seg_mask) {
            const int m = seg_mask[ray];
            if (m == 120 || m == 130 || m == 140) seg_sup = c->seg_mask_supervision_lambda;
            if (m <= 90 || m > 250) dl = 0.f;
            if (ta < 0.001f) dl = 0.f;
        }
        const float dn = sqrtf(R[3] * R[3] + R[4] * R[4] + R[5] * R[5]);
        const float td = dn * ((dl > 0.f && depth_img) ? depth_img[ray] : -1.f);
        float l_, g_;
        loss_1(c->depth_loss_type, td, depth_ray, &l_, &g_);
        const float depth_grad = (td > 0.f ? g_ : 0.f) * dl;
        float lg[3], ls = 0.f;
        /* lg.loss /= img_pdf * xy_pdf (testbed_nerf.cu:1494) */
        for (int k = 0; k < 3; ++k) {
            loss_1(c->loss_type, tgt[k], rgb_ray[k], &l_, &g_);
            lg[k] = g_ * seg_sup;
            ls += c->pdf ? l_ / c->pdf[ray] : l_;
        }
        const float mean_loss = ls / 3.f;
        if (loss_out) loss_out[i] = mean_loss / (float)c->n_rays;
        if (c->error_map && c->image_index[ray] < c->error_map_images) {
            /* testbed_nerf.cu:1510-1536: bilinear deposit at the ray's image position (xy * res - 0.5
             * is one fused multiply-add in the reference's nvcc build) */
            const float rx = (float)c->error_map_res[0], ry = (float)c->error_map_res[1];
            const float *xy = c->image_xy + (size_t)ray * 2;
            float px = fmaf(xy[0], rx, -0.5f), py = fmaf(xy[1], ry, -0.5f);
            px = px > 0.f ? px : 0.f; px = px < rx - 1.0001f ? px : rx - 1.0001f;
            py = py > 0.f ? py : 0.f; py = py < ry - 1.0001f ? py : ry - 1.0001f;
            int ix = (int)px, iy = (int)py;
            const float wx = px - (float)ix, wy = py - (float)iy;
            const int mxx = (int)c->error_map_res[0] - 2, mxy = (int)c->error_map_res[1] - 2;
            ix = ix < mxx ? ix : mxx; ix = ix > 0 ? ix : 0;
            iy = iy < mxy ? iy : mxy; iy = iy > 0 ? iy : 0;
            float *em = c->error_map + (size_t)c->image_index[ray] * c->error_map_res[0] * c->error_map_res[1];
            const size_t w = c->error_map_res[0];
            em[(size_t)iy * w + ix] += (1.f - wx) * (1.f - wy) * mean_loss;
            em[(size_t)iy * w + ix + 1] += wx * (1.f - wy) * mean_loss;
            em[(size_t)(iy + 1) * w + ix] += (1.f - wx) * wy * mean_loss;
            em[(size_t)(iy + 1) * w + ix + 1] += wx * wy * mean_loss;
        }
        const float scale = c->loss_scale / (float)c->n_rays;
        const float l1d = (mean_density && *mean_density < 0.01f) ? 1e-4f : 0.f;
        float rgb2[3] = {0, 0, 0}, depth2 = 0.f;
        T = 1.f;
        for (uint32_t j = 0; j < ccount; ++j) {
            const float *cc = cin + (size_t)j * c->stride, *o = o4 + (size_t)j * 4;
            memcpy(coords_out + (size_t)(cbase + j) * c->stride, cc, sizeof(float) * c->stride);
            float p[3], dd = 0.f;
            for (int k = 0; k < 3; ++k) { p[k] = c->aabb_min[k] + cc[5 + k] * diag[k]; float t = p[k] - R[k]; dd += t * t; }
            const float depth = sqrtf(dd), dt = cc[3] * (mx - MIN_CONE) + MIN_CONE;
            float rgb[3];
            for (int k = 0; k < 3; ++k) rgb[k] = logistic_f(o[k]);
            const float alpha = 1.f - expf(-expf(o[3]) * dt), w = alpha * T;
            for (int k = 0; k < 3; ++k) rgb2[k] += w * rgb[k];
            depth2 += w * depth;
            T *= 1.f - alpha;
            float *d4 = dloss + (size_t)(cbase + j) * 4, dot = 0.f;
            for (int k = 0; k < 3; ++k) {
                d4[k] = scale * ((w * lg[k]) * (rgb[k] * (1.f - rgb[k])));
                dot += lg[k] * (T * rgb[k] - (rgb_ray[k] - rgb2[k]));
            }
            const float ddens = expf(o[3] < -15.f ? -15.f : (o[3] > 15.f ? 15.f : o[3]));
            const float dsup = depth_grad * (T * depth - (depth_ray - depth2));
            const float bsup = dt / (T_ray - 1.f + 1e-3f);
            float dm = ddens * (dt * (dot + dsup) + c->beta * bsup);
            if (c->penalize_density) dm += ta <= 0.01f ? w : 0.f;
            d4[3] = scale * dm + (o[3] < 0.f ? -l1d : 0.f) + (o[3] > -10.f && depth < c->near_distance ? 1e-4f : 0.f);
        }
    }
    if (c->target_batch_size > 0) {
        const uint32_t cnt = *counter < c->max_samples_compacted ? *counter : c->max_samples_compacted;
        if (cnt > 0)
            for (uint32_t s = cnt; s < c->target_batch_size; ++s) {
                const uint32_t from = s % cnt;
                for (int k = 0; k < 4; ++k) dloss[(size_t)s * 4 + k] = dloss[(size_t)from * 4 + k] * (float)cnt / (float)c->target_batch_size;
                memcpy(coords_out + (size_t)s * c->stride, coords_out + (size_t)from * c->stride, sizeof(float) * c->stride);
            }
    }
}

/* ---------------------------------------------- single-function exports (pin tests) */
void orc_tbn(const orc_tri *t, float *m9) { tbn_f(t, m9); }
void orc_tri2projection(const orc_tri *t, float *M16) { tri2projection_f(t, M16); }
/* interpolate_transformation on the float path; invert applies the 4x4 inverse. */
void orc_interpolate_transformation(const float *p, const int32_t *adj, const orc_tri *tris, uint32_t id, int invert, float *M16) {
    float M[16];
    blend_projection_f(p, adj, tris, &tris[id], M);
    if (invert) { if (!inverse4_f(M, M16)) for (int k = 0; k < 16; ++k) M16[k] = (k % 5 == 0) ? 1.f : 0.f; }
    else memcpy(M16, M, sizeof(M));
}
/* transform_point / transform_direction (include/rta/affine.cuh:102-116). */
void orc_transform(const float *p, const float *dir, const float *Mw, const float *Mc, float *out_p, float *out_d) {
    float x4[4] = {p[0], p[1], p[2], 1.f}, l4[4], o4[4];
    for (int r = 0; r < 4; ++r) l4[r] = row4_f(&Mw[r * 4], x4);
    for (int r = 0; r < 4; ++r) o4[r] = row4_f(&Mc[r * 4], l4);
    for (int k = 0; k < 3; ++k) out_p[k] = o4[k];
    float ld[3], cd[3];
    for (int r = 0; r < 3; ++r) { float row[3] = {Mw[r * 4], Mw[r * 4 + 1], Mw[r * 4 + 2]}; ld[r] = dot3_f(row, dir); }
    for (int r = 0; r < 3; ++r) { float row[3] = {Mc[r * 4], Mc[r * 4 + 1], Mc[r * 4 + 2]}; cd[r] = dot3_f(row, ld); }
    normalize3_f(cd);
    memcpy(out_d, cd, 12);
}

/* ---- image / pixel draws and the error map's CDFs --------------------------------------- */
/* binary_search (NGP/common.h:195-218) */
static uint32_t cdf_search(float val, const float *data, uint32_t length) {
    uint32_t first = 0, count = length;
    while (count > 0) {
        const uint32_t step = count / 2, it = first + step;
        if (data[it] < val) { first = it + 1; count -= step + 1; }
        else count = step;
    }
    return first < length - 1 ? first : length - 1;
}

void orc_training_pixels(uint32_t n_rays, uint32_t n_rays_total, uint32_t n_images, const int32_t *resolution, int snap,
                         orc_pcg32 rng0, const float *cdf_x_cond_y, const float *cdf_y, const float *cdf_img, const uint32_t *cdf_res,
                         uint32_t *out_image, float *out_xy, float *out_pdf, float *out_background) {
    for (uint32_t i = 0; i < n_rays; ++i) {
        uint32_t img;
        float img_pdf = 1.f;
        if (cdf_img) { /* image_idx with the CDF (testbed_nerf.cu:1082-1094) */
            const float u = orc_ld_random_val(i + n_rays_total, 0xdeadbeefu, 0);
            img = cdf_search(u, cdf_img, n_images);
            const float prev = img > 0 ? cdf_img[img - 1] : 0.f;
            img_pdf = (cdf_img[img] - prev) * (float)n_images;
        } else {
            img = ((i + n_rays_total) * n_images / n_rays) % n_images;
        }
        orc_pcg32 rng = rng0;
        orc_pcg32_advance(&rng, (int64_t)i * 8);
        float sx = orc_pcg32_next_float(&rng);
        float sy = orc_pcg32_next_float(&rng);
        float xy_pdf = 1.f;
        if (cdf_x_cond_y) { /* sample_cdf_2d (testbed_nerf.cu:1013-1043) */
            if (sx < 0.5f) {
                sx /= 0.5f;
            } else {
                sx = (sx - 0.5f) / (1.0f - 0.5f);
                const uint32_t rx = cdf_res[0], ry = cdf_res[1];
                const float *cy = cdf_y + (size_t)img * ry;
                const uint32_t y = cdf_search(sy, cy, ry);
                float prev = y > 0 ? cy[y - 1] : 0.f;
                const float pmf_y = cy[y] - prev;
                sy = (sy - prev) / pmf_y;
                const float *cx = cdf_x_cond_y + ((size_t)img * ry + y) * rx;
                const uint32_t x = cdf_search(sx, cx, rx);
                prev = x > 0 ? cx[x - 1] : 0.f;
                const float pmf_x = cx[x] - prev;
                sx = (sx - prev) / pmf_x;
                xy_pdf = pmf_x * pmf_y * (float)(rx * ry);
                sx = ((float)x + sx) / (float)rx;
                sy = ((float)y + sy) / (float)ry;
            }
        }
        if (snap) { /* nerf_random_image_pos_training's pixel-centre snap (testbed_nerf.cu:1076-1078) */
            const int w = resolution[2 * img], h = resolution[2 * img + 1];
            int px = (int)(sx * (float)w), py = (int)(sy * (float)h);
            px = px > 0 ? px : 0; px = px < w - 1 ? px : w - 1;
            py = py > 0 ? py : 0; py = py < h - 1 ? py : h - 1;
            sx = ((float)px + 0.5f) / (float)w;
            sy = ((float)py + 0.5f) / (float)h;
        }
        out_image[i] = img;
        out_xy[2 * i] = sx;
        out_xy[2 * i + 1] = sy;
        if (out_pdf) out_pdf[i] = img_pdf * xy_pdf;
        if (out_background) /* train_with_random_bg_color: random_val_3d after the position */
            for (int k = 0; k < 3; ++k) out_background[3 * i + k] = orc_pcg32_next_float(&rng);
    }
}

void orc_error_map_cdf(const float *em, uint32_t n_images, uint32_t w, uint32_t h, float *cdf_x, float *cdf_y, float *cdf_img,
                       float *pmf_img) {
    const float a = 1.0f - 0.01f, b = 1.0f - 0.1f;
    for (uint32_t img = 0; img < n_images; ++img) {
        for (uint32_t y = 0; y < h; ++y) { /* construct_cdf_2d */
            const size_t off = ((size_t)img * h + y) * w;
            float cum = 0.f;
            for (uint32_t x = 0; x < w; ++x) { cum += em[off + x] + 1e-10f; cdf_x[off + x] = cum; }
            cdf_y[(size_t)img * h + y] = cum;
            const float norm = 1.0f / cum;
            for (uint32_t x = 0; x < w; ++x) cdf_x[off + x] = fmaf(a * cdf_x[off + x], norm, 0.01f * (float)(x + 1) / (float)w);
        }
        float *cy = cdf_y + (size_t)img * h; /* construct_cdf_1d */
        float cum = 0.f;
        for (uint32_t y = 0; y < h; ++y) { cum += cy[y]; cy[y] = cum; }
        cdf_img[img] = cum;
        const float norm = 1.0f / cum;
        for (uint32_t y = 0; y < h; ++y) cy[y] = fmaf(a * cy[y], norm, 0.01f * (float)(y + 1) / (float)h);
    }
    float cum = 0.f; /* the image CDF (host code of train_nerf_step) */
    for (uint32_t i = 0; i < n_images; ++i) cum += cdf_img[i];
    const float norm = 1.0f / cum;
    float run = 0.f;
    for (uint32_t i = 0; i < n_images; ++i) {
        const float v = cdf_img[i];
        run += v;
        if (pmf_img) pmf_img[i] = b * v * norm + 0.1f / (float)n_images;
        cdf_img[i] = b * run * norm + 0.1f * (float)(i + 1) / (float)n_images;
    }
}
