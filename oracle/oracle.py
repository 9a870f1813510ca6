"""ctypes front end of the CPU oracle (oracle/insta_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by
bench.py's CPU-baseline leg.  It is the checker (and the timed CPU baseline),
never the product: the library under insta_gb300/ does not import it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "insta_oracle.c"
INC = HERE / "oracle_real.inc"
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"


def build(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    deps = [SRC, INC, HERE / "insta_oracle.h"]
    if force or not LIB.exists() or any(d.stat().st_mtime > LIB.stat().st_mtime for d in deps):
        tmp = BUILD / f"liboracle.{os.getpid()}.so"
        cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=gnu11",
               "-Wall", "-Wno-unused-function", str(SRC), "-o", str(tmp), "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


class Tri(C.Structure):
    _fields_ = [("a", C.c_float * 3), ("b", C.c_float * 3), ("c", C.c_float * 3), ("scaling", C.c_float),
                ("id", C.c_uint32), ("mask_id", C.c_uint32)]


class Node(C.Structure):
    _fields_ = [("bb_min", C.c_float * 3), ("bb_max", C.c_float * 3), ("left_idx", C.c_int32), ("right_idx", C.c_int32)]


class Deform(C.Structure):
    _fields_ = [("def_tris", C.c_void_p), ("can_tris", C.c_void_p), ("adjacency", C.c_void_p), ("nodes", C.c_void_p),
                ("sorted", C.c_void_p), ("n_tris", C.c_int), ("disable_interp", C.c_int), ("fp64", C.c_int),
                ("bvh_exact", C.c_int), ("aabb_min", C.c_float * 3), ("aabb_max", C.c_float * 3)]


class FieldCfg(C.Structure):
    _fields_ = [("n_levels", C.c_uint32), ("n_features", C.c_uint32), ("log2_table", C.c_uint32), ("base_res", C.c_uint32),
                ("per_level_scale", C.c_float), ("n_extra", C.c_uint32), ("density_hidden", C.c_uint32),
                ("density_layers", C.c_uint32), ("density_out", C.c_uint32), ("rgb_hidden", C.c_uint32),
                ("rgb_layers", C.c_uint32), ("rgb_out_padded", C.c_uint32), ("weight_format", C.c_int)]


class RenderCfg(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("focal", C.c_float * 2), ("screen_center", C.c_float * 2),
                ("cam", C.c_float * 12), ("render_aabb_min", C.c_float * 3), ("render_aabb_max", C.c_float * 3),
                ("train_aabb_min", C.c_float * 3), ("train_aabb_max", C.c_float * 3), ("cone_angle", C.c_float),
                ("min_transmittance", C.c_float), ("spp", C.c_uint32), ("max_samples_per_ray", C.c_uint32),
                ("snap_to_pixel_centers", C.c_int), ("frame_id", C.c_int), ("extra_dims", C.c_void_p),
                ("linear_colors", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _lib.orc_tri_distance_sq.restype = C.c_float
        _lib.orc_box_distance_sq.restype = C.c_float
        _lib.orc_field_layout.restype = C.c_uint64
        _lib.orc_render.restype = C.c_int64
        _lib.orc_ld_random_val.restype = C.c_float
        _lib.orc_ld_random_val.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
        _lib.orc_sobol.restype = C.c_uint32
        _lib.orc_sobol.argtypes = [C.c_uint32, C.c_uint32]
        _lib.orc_morton3d.restype = C.c_uint32
        _lib.orc_num_threads.restype = C.c_int
        _lib.orc_occupancy_from_mesh.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_void_p]
        for n in ("orc_probe_calc_dt", "orc_probe_warp_dt", "orc_probe_unwarp_dt", "orc_probe_advance_to_next_voxel"):
            getattr(_lib, n).restype = C.c_float
        _lib.orc_probe_calc_dt.argtypes = [C.c_float, C.c_float]
        _lib.orc_probe_warp_dt.argtypes = [C.c_float]
        _lib.orc_probe_unwarp_dt.argtypes = [C.c_float]
        _lib.orc_probe_mip_from_dt.argtypes = [C.c_float, C.c_void_p]
        _lib.orc_probe_occupied_at.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        _lib.orc_probe_advance_to_next_voxel.argtypes = [C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32]
    return _lib


def ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def build_triangles(verts, canon_verts, faces, mask) -> np.ndarray:
    F = len(faces)
    out = np.zeros(F, dtype=np.dtype([("a", "<f4", 3), ("b", "<f4", 3), ("c", "<f4", 3), ("scaling", "<f4"), ("id", "<u4"), ("mask_id", "<u4")]))
    v = np.ascontiguousarray(verts, dtype=np.float32)
    cv = None if canon_verts is None else np.ascontiguousarray(canon_verts, dtype=np.float32)
    f = np.ascontiguousarray(faces, dtype=np.int32)
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint32)
    lib().orc_build_triangles(ptr(v), ptr(cv), ptr(f), ptr(m), C.c_int(F), ptr(out))
    return out


def adjacency(faces, n_verts) -> np.ndarray:
    f = np.ascontiguousarray(faces, dtype=np.int32)
    out = np.empty((len(f), 3), dtype=np.int32)
    lib().orc_adjacency(ptr(f), C.c_int(len(f)), C.c_int(n_verts), ptr(out))
    return out


def nearest_brute(tris, pts):
    p = np.ascontiguousarray(pts, dtype=np.float32)
    ids = np.empty(len(p), dtype=np.int32)
    d2 = np.empty(len(p), dtype=np.float32)
    lib().orc_nearest_brute(ptr(tris), C.c_int(len(tris)), ptr(p), C.c_int64(len(p)), ptr(ids), ptr(d2))
    return ids, d2


class Bvh:
    """TriangleBvh4 restated (instant-ngp/src/triangle_bvh.cu:548-631)."""

    def __init__(self, tris, leaf_size: int = 2):
        self.tris = tris
        max_nodes = 2 * len(tris) + 16
        self.nodes = np.zeros(max_nodes, dtype=np.dtype([("bb_min", "<f4", 3), ("bb_max", "<f4", 3), ("l", "<i4"), ("r", "<i4")]))
        self.sorted = np.zeros_like(tris)
        n = lib().orc_bvh4_build(ptr(tris), C.c_int(len(tris)), C.c_int(leaf_size), ptr(self.nodes), C.c_int(max_nodes), ptr(self.sorted))
        assert n > 0
        self.nodes = self.nodes[:n].copy()

    def nearest(self, pts, exact: bool = True):
        p = np.ascontiguousarray(pts, dtype=np.float32)
        ids = np.empty(len(p), dtype=np.int32)
        d2 = np.empty(len(p), dtype=np.float32)
        lib().orc_nearest_bvh(ptr(self.nodes), ptr(self.sorted), ptr(p), C.c_int64(len(p)), C.c_int(1 if exact else 0), ptr(ids), ptr(d2))
        return ids, d2


class Deformation:
    """The deformed->canonical map of the `warp` kernel on one frame."""

    def __init__(self, def_tris, can_tris, adj, bvh: Bvh | None = None, disable_interp=False, fp64=False, exact=True,
                 aabb=((0, 0, 0), (1, 1, 1))):
        self.keep = (def_tris, can_tris, adj, bvh)
        d = Deform()
        d.def_tris = def_tris.ctypes.data
        d.can_tris = can_tris.ctypes.data
        d.adjacency = adj.ctypes.data
        d.nodes = bvh.nodes.ctypes.data if bvh is not None else None
        d.sorted = bvh.sorted.ctypes.data if bvh is not None else None
        d.n_tris = len(def_tris)
        d.disable_interp = int(disable_interp)
        d.fp64 = int(fp64)
        d.bvh_exact = int(exact)
        d.aabb_min[:] = [float(x) for x in aabb[0]]
        d.aabb_max[:] = [float(x) for x in aabb[1]]
        self.d = d

    def map_soa(self, pts):
        p = np.ascontiguousarray(pts, dtype=np.float32)
        ids = np.empty(len(p), dtype=np.int32)
        out = np.empty_like(p)
        lib().orc_canonical_map_soa(C.byref(self.d), ptr(p), C.c_int64(len(p)), ptr(ids), ptr(out))
        return ids, out

    def map_coords(self, coords, n_extra=0, frame_id=-1, n_frames=1):
        c = np.ascontiguousarray(coords, dtype=np.float32).copy()
        stride = c.shape[1]
        lib().orc_canonical_map_coords(C.byref(self.d), ptr(c), C.c_uint32(stride), C.c_uint32(n_extra), C.c_int64(len(c)),
                                       C.c_int32(frame_id), C.c_uint32(n_frames))
        return c


def field_cfg(fc, weight_format: int = 0) -> FieldCfg:
    c = FieldCfg()
    c.n_levels, c.n_features, c.log2_table, c.base_res = fc.n_levels, fc.n_features, fc.log2_table, fc.base_res
    c.per_level_scale = fc.per_level_scale
    c.n_extra = fc.n_extra
    c.density_hidden, c.density_layers, c.density_out = fc.density_hidden, fc.density_layers, fc.density_out
    c.rgb_hidden, c.rgb_layers, c.rgb_out_padded = fc.rgb_hidden, fc.rgb_layers, fc.rgb_out_padded
    c.weight_format = weight_format
    return c


def fp8_layer_scales(fc, params) -> np.ndarray:
    """Per-layer FP8 weight scales max|W| / 448 (float32), in layer order (density, then colour)."""
    from insta_gb300 import layout as _layout
    lay = _layout.field_layout(fc)
    w = np.ascontiguousarray(params).view(np.float16).astype(np.float32)
    out = np.ones(8, np.float32)
    for i, (off, n, k, _last) in enumerate(lay.layers):
        mx = np.float32(np.abs(w[off:off + n * k]).max())
        out[i] = mx / np.float32(448.0) if mx > 0 else np.float32(1.0)
    return out


def field_eval(fc, params, coords, fp64=False, weight_format=0, layer_scales=None):
    """weight_format 2 (FP8) takes the per-layer scales (default: fp8_layer_scales)."""
    c = np.ascontiguousarray(coords, dtype=np.float32)
    out = np.empty((len(c), 4), dtype=np.float32)
    cfg = field_cfg(fc, weight_format)
    p = np.ascontiguousarray(params).view(np.uint16)
    if weight_format == 2 and layer_scales is None:
        layer_scales = fp8_layer_scales(fc, params)
    ls = None if layer_scales is None else np.ascontiguousarray(layer_scales, np.float32)
    lib().orc_field_eval(C.byref(cfg), ptr(p), ptr(ls) if ls is not None else None, ptr(c), C.c_uint32(c.shape[1]),
                         C.c_int64(len(c)), ptr(out), C.c_int(int(fp64)))
    return out


def field_backward(fc, params, coords, dl_dout=None, extra_grad=False):
    """NerfNetwork backward in FP64: (gradient of sum(dl_dout * out) w.r.t. every parameter
    [float64, snapshot order], the FP64 forward's outputs [n, 4]); with extra_grad also the
    gradient w.r.t. each record's expression dims [n, n_extra] (float64)."""
    c = np.ascontiguousarray(coords, dtype=np.float32)
    cfg = field_cfg(fc, 0)
    p = np.ascontiguousarray(params).view(np.uint16)
    grad = np.zeros(p.size, np.float64)
    out = np.zeros((len(c), 4), np.float32)
    g = None if dl_dout is None else np.ascontiguousarray(dl_dout, np.float32)
    dx = np.zeros((len(c), max(1, int(cfg.n_extra))), np.float64) if extra_grad else None
    lib().orc_field_backward_ex(C.byref(cfg), ptr(p), ptr(c), C.c_uint32(c.shape[1]), C.c_int64(len(c)),
                                ptr(g) if g is not None else None, ptr(grad) if g is not None else None, ptr(out),
                                ptr(dx) if dx is not None else None)
    return (grad, out, dx[:, :int(cfg.n_extra)]) if extra_grad else (grad, out)


class TrainLossCfg(C.Structure):
    _fields_ = [("n_rays", C.c_uint32), ("max_samples_compacted", C.c_uint32), ("target_batch_size", C.c_uint32),
                ("stride", C.c_uint32), ("aabb_min", C.c_float * 3), ("aabb_max", C.c_float * 3), ("loss_type", C.c_int),
                ("depth_loss_type", C.c_int), ("srgb_targets", C.c_int), ("train_in_linear_colors", C.c_int),
                ("penalize_density", C.c_int), ("loss_scale", C.c_float), ("depth_supervision_lambda", C.c_float),
                ("seg_mask_supervision_lambda", C.c_float), ("near_distance", C.c_float), ("beta", C.c_float),
                ("pdf", C.c_void_p), ("error_map", C.c_void_p), ("error_map_res", C.c_uint32 * 2),
                ("error_map_images", C.c_uint32), ("image_xy", C.c_void_p), ("image_index", C.c_void_p)]


def train_loss(cfg: dict, rays, target, ray_indices, numsteps, coords, network_output, background=None, exposure=None,
               depth=None, seg_mask=None, mean_density=None, pdf=None, error_map=None, image_xy=None, image_index=None):
    """compute_loss_kernel_train_nerf + fill_rollover over the kept rays in order.  cfg keys are
    TrainLossCfg's fields.  Returns (numsteps out, compacted counter, coords_out, dloss, loss); with
    error_map (f32[n_images][res_y][res_x], added to in place) the kept rays' mean losses are
    deposited into it."""
    c = TrainLossCfg()
    for k, v in cfg.items():
        if k in ("aabb_min", "aabb_max"):
            getattr(c, k)[:] = [float(x) for x in v]
        else:
            setattr(c, k, v)
    keep = []
    if pdf is not None:
        keep.append(np.ascontiguousarray(pdf, np.float32))
        c.pdf = keep[-1].ctypes.data
    if error_map is not None:
        assert error_map.dtype == np.float32 and error_map.flags.c_contiguous and error_map.ndim == 3
        c.error_map = error_map.ctypes.data
        c.error_map_res[0], c.error_map_res[1] = error_map.shape[2], error_map.shape[1]
        c.error_map_images = error_map.shape[0]
        keep += [np.ascontiguousarray(image_xy, np.float32), np.ascontiguousarray(image_index, np.uint32)]
        c.image_xy, c.image_index = keep[-2].ctypes.data, keep[-1].ctypes.data
    f32 = lambda a: None if a is None else np.ascontiguousarray(a, np.float32)
    rays, target, coords, network_output = f32(rays), f32(target), f32(coords), f32(network_output)
    background, exposure, depth = f32(background), f32(exposure), f32(depth)
    seg = None if seg_mask is None else np.ascontiguousarray(seg_mask, np.int32)
    md = None if mean_density is None else np.array([mean_density], np.float32)
    idx = np.ascontiguousarray(ray_indices, np.uint32)
    ns = np.ascontiguousarray(numsteps, np.uint32).copy()
    counter = np.zeros(1, np.uint32)
    cap = int(c.max_samples_compacted)
    coords_out = np.zeros((cap, int(c.stride)), np.float32)
    dloss = np.zeros((cap, 4), np.float32)
    loss = np.zeros(len(idx), np.float32)
    p = lambda a: None if a is None else ptr(a)
    lib().orc_train_loss(C.byref(c), C.c_uint32(len(idx)), ptr(rays), ptr(target), p(background), p(exposure), p(depth), p(seg), p(md),
                         ptr(idx), ptr(ns), ptr(coords), ptr(network_output), ptr(counter), ptr(coords_out), ptr(dloss), ptr(loss))
    return ns, int(counter[0]), coords_out, dloss, loss


def training_pixels(n_rays, n_rays_total, n_images, rng, resolution=None, snap=False, cdfs=None, cdf_res=(0, 0)):
    """image_idx + nerf_random_image_pos_training + the background draw per ray: (image u32[n],
    xy f32[n][2], pdf f32[n], background f32[n][3]).  cdfs = (cdf_x_cond_y, cdf_y, cdf_img) or None."""
    img = np.zeros(n_rays, np.uint32)
    xy = np.zeros((n_rays, 2), np.float32)
    pdf = np.zeros(n_rays, np.float32)
    bg = np.zeros((n_rays, 3), np.float32)
    res = None if resolution is None else np.ascontiguousarray(resolution, np.int32)
    cx = cy = ci = None
    if cdfs is not None:
        cx, cy, ci = (np.ascontiguousarray(a, np.float32) for a in cdfs)
    cr = np.array(cdf_res, np.uint32)
    p = lambda a: None if a is None else ptr(a)
    lib().orc_training_pixels(C.c_uint32(n_rays), C.c_uint32(n_rays_total), C.c_uint32(n_images), p(res), C.c_int(int(snap)), rng,
                              p(cx), p(cy), p(ci), ptr(cr), ptr(img), ptr(xy), ptr(pdf), ptr(bg))
    return img, xy, pdf, bg


def error_map_cdf(error_map):
    """construct_cdf_2d / _1d and the image CDF of an error map f32[n_images][res_y][res_x]:
    (cdf_x_cond_y, cdf_y, cdf_img, pmf_img)."""
    em = np.ascontiguousarray(error_map, np.float32)
    n, h, w = em.shape
    cx = np.zeros_like(em)
    cy = np.zeros((n, h), np.float32)
    ci = np.zeros(n, np.float32)
    pm = np.zeros(n, np.float32)
    lib().orc_error_map_cdf(ptr(em), C.c_uint32(n), C.c_uint32(w), C.c_uint32(h), ptr(cx), ptr(cy), ptr(ci), ptr(pm))
    return cx, cy, ci, pm


def occupancy(tris, radius=0.015) -> np.ndarray:
    bits = np.zeros(8 * 128 ** 3 // 8, dtype=np.uint8)
    lib().orc_occupancy_from_mesh(ptr(tris), C.c_int(len(tris)), C.c_double(radius), ptr(bits))
    return bits


def density_grid_to_bitfield(grid, n_cascades):
    """Bitfield (8 mips x 128^3 bits) and threshold from a float density grid [n_cascades, 128^3]."""
    g = np.ascontiguousarray(grid, dtype=np.float32).reshape(-1)
    bits = np.zeros(8 * 128 ** 3 // 8, np.uint8)
    f = lib().orc_density_grid_to_bitfield
    f.restype = C.c_float
    t = f(ptr(g), C.c_uint32(n_cascades), ptr(bits))
    return bits, float(t)


class Pcg32(C.Structure):
    """pcg32 state (tiny-cuda-nn's default_rng_t), restated in insta_oracle.c."""
    _fields_ = [("state", C.c_uint64), ("inc", C.c_uint64)]

    @staticmethod
    def seeded(initstate: int, initseq: int = 1) -> "Pcg32":
        r = Pcg32()
        lib().orc_pcg32_seed(C.byref(r), C.c_uint64(initstate), C.c_uint64(initseq))
        return r

    def copy(self) -> "Pcg32":
        return Pcg32(self.state, self.inc)

    def next_uint(self) -> int:
        f = lib().orc_pcg32_next_uint
        f.restype = C.c_uint32
        return int(f(C.byref(self)))

    def next_float(self) -> float:
        f = lib().orc_pcg32_next_float
        f.restype = C.c_float
        return float(f(C.byref(self)))

    def advance(self, delta: int = 1 << 32):
        lib().orc_pcg32_advance(C.byref(self), C.c_int64(delta))


def grid_samples(n_uniform, n_nonuniform, rng: Pcg32, step, aabb, grid, n_cascades):
    """generate_grid_samples_nerf_nonuniform for both sets: positions [n, 3] and cell indices [n]."""
    n = n_uniform + n_nonuniform
    pos = np.zeros((n, 3), np.float32)
    idx = np.zeros(n, np.uint32)
    mn = np.asarray(aabb[0], np.float32)
    mx = np.asarray(aabb[1], np.float32)
    g = np.ascontiguousarray(grid, dtype=np.float32)
    lib().orc_grid_samples(C.c_uint32(n_uniform), C.c_uint32(n_nonuniform), rng, C.c_uint32(step), ptr(mn), ptr(mx), ptr(g),
                           C.c_uint32(n_cascades), ptr(pos), ptr(idx))
    return pos, idx


def warp_random_samples(deforms, rng: Pcg32, pos):
    """warp_random_samples over the frames' Deformation objects: canonical positions and the frame each point took."""
    arr = (Deform * len(deforms))(*[d.d for d in deforms])
    p = np.ascontiguousarray(pos, dtype=np.float32).copy()
    fr = np.zeros(len(p), np.uint32)
    lib().orc_warp_random_samples(arr, C.c_uint32(len(deforms)), rng, ptr(p), C.c_int64(len(p)), ptr(fr))
    return p, fr


def render_cfg(width, height, focal, cam, render_box, train_box=((0, 0, 0), (1, 1, 1)), cone_angle=1 / 256, spp=0,
               min_transmittance=0.01, max_samples=1024, frame_id=0, snap=True, linear_colors=False) -> RenderCfg:
    r = RenderCfg()
    r.width, r.height = int(width), int(height)
    r.focal[:] = [float(focal[0]), float(focal[1])]
    r.screen_center[:] = [0.5, 0.5]
    r.cam[:] = [float(x) for x in np.asarray(cam, dtype=np.float32).reshape(-1)]
    r.render_aabb_min[:] = [float(x) for x in render_box[0]]
    r.render_aabb_max[:] = [float(x) for x in render_box[1]]
    r.train_aabb_min[:] = [float(x) for x in train_box[0]]
    r.train_aabb_max[:] = [float(x) for x in train_box[1]]
    r.cone_angle = float(np.float32(cone_angle))
    r.min_transmittance = float(min_transmittance)
    r.spp = spp
    r.max_samples_per_ray = max_samples
    r.snap_to_pixel_centers = int(snap)
    r.frame_id = frame_id
    r.extra_dims = None
    r.linear_colors = int(linear_colors)
    return r


def render(rc: RenderCfg, deform: Deformation, bits, fc, params, rows=None, fp64=False, weight_format=0, extra_dims=None,
           layer_scales=None):
    r0, r1 = (0, rc.height) if rows is None else rows
    n = (r1 - r0) * rc.width
    rgba = np.zeros((n, 4), dtype=np.float32)
    depth = np.zeros(n, dtype=np.float32)
    ns = np.zeros(n, dtype=np.uint32)
    cfg = field_cfg(fc, weight_format)
    p = np.ascontiguousarray(params).view(np.uint16)
    ed = None
    if extra_dims is not None:
        ed = np.ascontiguousarray(extra_dims, dtype=np.float32)
        rc.extra_dims = ed.ctypes.data
    if weight_format == 2 and layer_scales is None:
        layer_scales = fp8_layer_scales(fc, params)
    ls = None if layer_scales is None else np.ascontiguousarray(layer_scales, np.float32)
    total = lib().orc_render(C.byref(rc), C.byref(deform.d), ptr(bits), C.byref(cfg), ptr(p), ptr(ls) if ls is not None else None,
                             C.c_int(r0), C.c_int(r1),
                             ptr(rgba), ptr(depth), ptr(ns), C.c_int(int(fp64)))
    rc.extra_dims = None
    return rgba, depth, ns, int(total)


def raycast(rc: RenderCfg, tris, center, color_normal=False, rgba=None, depth=None):
    """raycast_flame: (rgba [h*w, 4], depth [h*w], hit triangle id or -1 [h*w]); rgba/depth keep
    their given values where nothing inside the render box is hit."""
    n = rc.width * rc.height
    rgba = np.zeros((n, 4), np.float32) if rgba is None else np.ascontiguousarray(rgba, np.float32).copy()
    depth = np.zeros(n, np.float32) if depth is None else np.ascontiguousarray(depth, np.float32).copy()
    tri = np.zeros(n, np.int32)
    c = np.ascontiguousarray(center, np.float32)
    lib().orc_raycast(C.byref(rc), ptr(tris), C.c_int(len(tris)), ptr(c), C.c_int(int(color_normal)), ptr(rgba), ptr(depth), ptr(tri))
    return rgba, depth, tri


def mesh_centroid(verts) -> np.ndarray:
    """TinyMesh::m_centorid: float32 running sum of the vertices in order, divided by their count."""
    c = np.zeros(3, np.float32)
    for v in np.asarray(verts, np.float32):
        c = (c + v).astype(np.float32)
    return (c / np.float32(len(verts))).astype(np.float32)


def march_ray(rc: RenderCfg, bits, px, py, max_out=1024):
    t = np.zeros(max_out, dtype=np.float32)
    dt = np.zeros(max_out, dtype=np.float32)
    pos = np.zeros((max_out, 3), dtype=np.float32)
    n = lib().orc_march_ray(C.byref(rc), ptr(bits), C.c_int(px), C.c_int(py), C.c_int(max_out), ptr(t), ptr(dt), ptr(pos))
    return t[:n], dt[:n], pos[:n]


def training_samples(bits, rays, image, start_rand, max_samples, train_box=((0, 0, 0), (1, 1, 1)), cone_angle=1 / 256,
                     extra=None, n_extra=0):
    """generate_training_samples_nerf on given rays: (coords [max_samples, 11 + n_extra], ray_indices,
    numsteps [n, 2], counters [2])."""
    rays = np.ascontiguousarray(rays, np.float32)
    n = len(rays)
    image = np.ascontiguousarray(image, np.uint32)
    rnd = np.ascontiguousarray(start_rand, np.float32)
    stride = 11 + n_extra
    coords = np.zeros((max_samples, stride), np.float32)
    ri = np.zeros(n, np.uint32)
    ns = np.zeros((n, 2), np.uint32)
    cnt = np.zeros(2, np.uint32)
    mn = np.asarray(train_box[0], np.float32)
    mx = np.asarray(train_box[1], np.float32)
    ex = None if extra is None else np.ascontiguousarray(extra, np.float32)
    lib().orc_training_samples(ptr(mn), ptr(mx), C.c_float(cone_angle), ptr(bits), ptr(rays), ptr(image), ptr(rnd),
                               ptr(ex) if ex is not None else None, C.c_uint32(n_extra), C.c_int64(n),
                               C.c_uint32(max_samples), ptr(coords), C.c_uint32(stride), ptr(ri), ptr(ns), ptr(cnt))
    return coords, ri, ns, cnt


def ld_random_val(index, seed, dim=0) -> float:
    return lib().orc_ld_random_val(index, seed, dim)


def pixel_offset(spp) -> np.ndarray:
    out = (C.c_float * 2)()
    lib().orc_ld_random_pixel_offset(C.c_uint32(spp), out)
    return np.array([out[0], out[1]], dtype=np.float32)


def num_threads() -> int:
    return lib().orc_num_threads()


# ------------------------------------------------------------------ march helpers (pin tests)
def march_bitfield() -> np.ndarray:
    """A fixed, seed-free 8-mip occupancy bitfield for the march-helper pins: byte i is a
    multiplicative hash of i (about half the bits set)."""
    i = np.arange(8 * 128 ** 3 // 8, dtype=np.uint64)
    return ((i * np.uint64(2654435761)) >> np.uint64(13)).astype(np.uint8)


def march_helpers(lib_, cases: dict, bitfield: np.ndarray) -> dict:
    """Run the march helpers of one library (the oracle's orc_probe_* or the reference's ref_*)
    over the input arrays in `cases`; returns their outputs."""
    pre = "orc_probe_" if hasattr(lib_, "orc_probe_calc_dt") else "ref_"
    f = lambda n: getattr(lib_, pre + ("density_grid_occupied_at" if n == "occupied_at" and pre == "ref_" else n))
    out = {}
    out["calc_dt"] = np.array([f("calc_dt")(C.c_float(t), C.c_float(c)) for t, c in zip(cases["dt_t"], cases["dt_cone"])], np.float32)
    out["warp_dt"] = np.array([f("warp_dt")(C.c_float(x)) for x in cases["warp_in"]], np.float32)
    out["unwarp_dt"] = np.array([f("unwarp_dt")(C.c_float(x)) for x in cases["unwarp_in"]], np.float32)
    mp = np.ascontiguousarray(cases["mip_pos"], np.float32)
    out["mip_from_dt"] = np.array([f("mip_from_dt")(C.c_float(d), ptr(mp[i])) for i, d in enumerate(cases["mip_dt"])], np.int32)
    op = np.ascontiguousarray(cases["occ_pos"], np.float32)
    out["occupied_at"] = np.array([f("occupied_at")(ptr(op[i]), ptr(bitfield), int(m)) for i, m in enumerate(cases["occ_mip"])], np.int32)
    ap, ad, ai = (np.ascontiguousarray(cases[k], np.float32) for k in ("adv_pos", "adv_dir", "adv_idir"))
    out["advance"] = np.array([f("advance_to_next_voxel")(C.c_float(t), C.c_float(c), ptr(ap[i]), ptr(ad[i]), ptr(ai[i]), C.c_uint32(int(r)))
                               for i, (t, c, r) in enumerate(zip(cases["adv_t"], cases["adv_cone"], cases["adv_res"]))], np.float32)
    return out


def march_cases(rng) -> dict:
    """Seeded inputs for the march-helper pins: step sizes around both clamps, positions over all
    cascades, rays in every direction octant (including axis-parallel ones) at every grid level."""
    n = 2000
    min_cone, max_cone = np.float32(1.73205080757 / 1024), np.float32(1.73205080757 / 1024 * 128)
    t = np.concatenate([rng.uniform(0, 4, n // 2), np.exp(rng.uniform(np.log(1e-3), np.log(150.0), n // 2))]).astype(np.float32)
    cone = rng.choice(np.array([0.0, 1 / 256, 1 / 128, 0.02], np.float32), n)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[np.arange(n // 10), rng.integers(0, 3, n // 10)] = 0.0   # a zero component: axis-parallel slabs
    d /= np.maximum(np.linalg.norm(d, axis=1, keepdims=True), 1e-12)
    with np.errstate(divide="ignore"):
        idir = (np.float32(1) / d).astype(np.float32)
    # occupancy lookups inside each mip's box [0.5 - 2^(m-1), 0.5 + 2^(m-1)] (the march never
    # leaves it), a few just outside where the index is clamped
    occ_mip = rng.integers(0, 8, n).astype(np.int32)
    half = np.ldexp(0.5, occ_mip).astype(np.float64)[:, None]
    occ_pos = (0.5 + rng.uniform(-1.0, 1.0, (n, 3)) * half * np.where(rng.random((n, 1)) < 0.02, 1.004, 0.999)).astype(np.float32)
    return {
        "dt_t": t, "dt_cone": cone,
        "warp_in": rng.uniform(min_cone, max_cone, n).astype(np.float32),
        "unwarp_in": rng.uniform(0, 1, n).astype(np.float32),
        "mip_pos": rng.uniform(-1.5, 2.5, (n, 3)).astype(np.float32),
        "mip_dt": np.exp(rng.uniform(np.log(1e-4), np.log(2.0), n)).astype(np.float32),
        "occ_pos": occ_pos, "occ_mip": occ_mip,
        "adv_t": rng.uniform(0.05, 2.0, n).astype(np.float32), "adv_cone": rng.choice(np.array([0.0, 1 / 256], np.float32), n),
        "adv_pos": rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32), "adv_dir": d, "adv_idir": idir,
        "adv_res": rng.choice(np.array([128, 64, 32, 16, 8, 4, 2, 1], np.uint32), n),
    }
