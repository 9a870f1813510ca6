"""ctypes binding of the C ABI (include/insta_gb300.h) exported by libinsta_gb300.so.

There is no CPU fallback: if the library is missing or no sm_10x GPU is
present, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

# the in-tree build; INSTA_GB300_LIB selects another build of the same library
LIB_PATH = Path(os.environ.get("INSTA_GB300_LIB", Path(__file__).resolve().parent / "_lib" / "libinsta_gb300.so"))

OK, ERR_INVALID_ARG, ERR_CUDA, ERR_BUDGET, ERR_NOT_READY, ERR_UNSUPPORTED, ERR_DEVICE = range(7)
PRECISION_FP16, PRECISION_BF16, PRECISION_FP8 = 0, 1, 2
FLAG_DISABLE_INTERP = 1

EXPORTS = [
    "insta_ctx_create", "insta_ctx_destroy", "insta_last_error", "insta_sync", "insta_memory_used",
    "insta_stats_enable", "insta_stats_read",
    "insta_canonical_set", "insta_avatar_set_boxes", "insta_avatar_set_flags", "insta_frame_upload",
    "insta_frame_upload_batch", "insta_frame_upload_async", "insta_frame_wait",
    "insta_frame_release", "insta_occupancy_from_mesh", "insta_occupancy_set", "insta_occupancy_get",
    "insta_density_grid_load", "insta_density_grid_reset", "insta_density_grid_update", "insta_density_grid_read",
    "insta_canonical_map", "insta_canonical_map_soa", "insta_training_samples", "insta_field_param_count", "insta_params_load",
    "insta_field_eval", "insta_field_eval_training", "insta_field_eval_static", "insta_field_backward", "insta_field_backward_ex", "insta_extra_dims_gradient", "insta_adam_step", "insta_train_loss", "insta_training_pixels", "insta_error_map_cdf", "insta_train_set_math", "insta_render", "insta_render_async", "insta_render_batch",
    "insta_render_samples", "insta_tuning_set", "insta_tuning_get", "insta_autotune", "insta_march_debug", "insta_nearest_debug",
    "insta_raycast",
    "insta_server_create", "insta_server_destroy", "insta_submit", "insta_poll", "insta_wait", "insta_cancel",
    "insta_server_release", "insta_server_error",
]

REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_CANCELLED, REQ_FAILED = range(5)


class ServerConfig(C.Structure):
    _fields_ = [("max_inflight", C.c_uint32), ("max_inflight_pixels", C.c_uint64), ("occupancy_radius", C.c_double),
                ("rounds_per_launch", C.c_uint32), ("round_samples", C.c_uint64)]


class Pcg32State(C.Structure):
    _fields_ = [("state", C.c_uint64), ("inc", C.c_uint64)]


class DensityUpdateDesc(C.Structure):
    _fields_ = [("decay", C.c_float), ("n_uniform", C.c_uint32), ("n_nonuniform", C.c_uint32), ("n_cascades", C.c_uint32),
                ("aabb_min", C.c_float * 3), ("aabb_max", C.c_float * 3), ("grid_rng", Pcg32State), ("warp_rng", Pcg32State),
                ("ema_step", C.c_uint32), ("n_frames", C.c_int32), ("bitfield_frame", C.c_int32),
                ("debug_pos", C.c_void_p), ("debug_idx", C.c_void_p)]


class AdamConfig(C.Structure):
    _fields_ = [("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("epsilon", C.c_float),
                ("l2_reg", C.c_float), ("ema_decay", C.c_float), ("loss_scale", C.c_float)]


LOSS_TYPES = {"l2": 0, "l1": 1, "mape": 2, "smape": 3, "huber": 4, "logl1": 5, "relativel2": 6}


class TrainLossDesc(C.Structure):
    _fields_ = [("n_rays", C.c_uint32), ("max_rays", C.c_uint32), ("max_samples_compacted", C.c_uint32),
                ("target_batch_size", C.c_uint32), ("aabb_min", C.c_float * 3), ("aabb_max", C.c_float * 3),
                ("loss_type", C.c_int32), ("depth_loss_type", C.c_int32), ("srgb_targets", C.c_int32),
                ("train_in_linear_colors", C.c_int32), ("loss_scale", C.c_float), ("depth_supervision_lambda", C.c_float),
                ("seg_mask_supervision_lambda", C.c_float), ("near_distance", C.c_float), ("beta", C.c_float),
                ("penalize_density", C.c_int32), ("stride", C.c_uint32),
                ("rays", C.c_void_p), ("target", C.c_void_p), ("background", C.c_void_p), ("exposure", C.c_void_p),
                ("depth", C.c_void_p), ("seg_mask", C.c_void_p), ("mean_density", C.c_void_p), ("rays_counter", C.c_void_p),
                ("ray_indices", C.c_void_p), ("numsteps", C.c_void_p), ("coords", C.c_void_p), ("network_output", C.c_void_p),
                ("numsteps_counter", C.c_void_p), ("coords_out", C.c_void_p), ("dloss_doutput", C.c_void_p),
                ("loss_output", C.c_void_p), ("pdf", C.c_void_p), ("error_map", C.c_void_p), ("error_map_res", C.c_uint32 * 2),
                ("error_map_images", C.c_uint32), ("image_xy", C.c_void_p), ("image_index", C.c_void_p)]


class ExtraDimsGradientDesc(C.Structure):
    _fields_ = [("max_rays", C.c_uint32), ("n_extra_dims", C.c_uint32), ("n_images", C.c_uint32), ("rays_counter", C.c_void_p),
                ("ray_indices", C.c_void_p), ("numsteps", C.c_void_p), ("image_index", C.c_void_p), ("dl_dextra", C.c_void_p),
                ("extra_dims_gradient", C.c_void_p)]


class TrainingPixelsDesc(C.Structure):
    _fields_ = [("n_rays", C.c_uint32), ("n_rays_total", C.c_uint32), ("n_images", C.c_uint32), ("resolution", C.c_void_p),
                ("snap_to_pixel_centers", C.c_int32), ("rng_state", C.c_uint64), ("rng_inc", C.c_uint64),
                ("cdf_x_cond_y", C.c_void_p), ("cdf_y", C.c_void_p), ("cdf_img", C.c_void_p), ("cdf_res", C.c_uint32 * 2),
                ("out_image", C.c_void_p), ("out_xy", C.c_void_p), ("out_pdf", C.c_void_p), ("out_background", C.c_void_p)]


class InstaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[insta error {code}] {msg}")
        self.code = code


class FieldDesc(C.Structure):
    _fields_ = [("n_levels", C.c_uint32), ("n_features_per_level", C.c_uint32), ("log2_hashmap_size", C.c_uint32),
                ("base_resolution", C.c_uint32), ("per_level_scale", C.c_float), ("aabb_scale", C.c_uint32),
                ("n_extra_dims", C.c_uint32), ("density_neurons", C.c_uint32), ("density_hidden_layers", C.c_uint32),
                ("density_output_dims", C.c_uint32), ("rgb_neurons", C.c_uint32), ("rgb_hidden_layers", C.c_uint32),
                ("precision", C.c_uint32)]


STAGES = ["frame", "occupancy", "ray_init", "march", "deform_encode", "mlp", "composite", "canonical_map", "field", "sort",
          "raycast", "train", "nearest"]


class Stats(C.Structure):
    _fields_ = [("kernel_launches", C.c_uint64), ("last_render_samples", C.c_uint64),
                ("stage_ms", C.c_float * len(STAGES)), ("stage_calls", C.c_uint32 * len(STAGES)),
                ("walk_warps", C.c_uint64), ("walk_inner_nodes", C.c_uint64), ("walk_leaves", C.c_uint64),
                ("walk_bound_tests", C.c_uint64), ("walk_exact_tests", C.c_uint64)]


class RenderDesc(C.Structure):
    _fields_ = [("avatar", C.c_int32), ("frame", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("focal_length", C.c_float * 2), ("screen_center", C.c_float * 2), ("camera", C.c_float * 12),
                ("cone_angle", C.c_float), ("min_transmittance", C.c_float), ("spp", C.c_uint32),
                ("snap_to_pixel_centers", C.c_uint32), ("max_samples_per_ray", C.c_uint32), ("linear_colors", C.c_uint32),
                ("extra_dims", C.c_void_p), ("out_samples", C.c_void_p)]


class Tuning(C.Structure):
    _fields_ = [("max_steps_per_round", C.c_uint32), ("sort_cell_bits", C.c_uint32), ("mlp_ctas_per_sm", C.c_uint32),
                ("deform_blocks_per_sm", C.c_uint32), ("bvh_top_nodes", C.c_uint32), ("fused_field_stage", C.c_uint32),
                ("mlp_slots", C.c_uint32)]


_lib = None


def load(path: Path | None = None):
    """Load the library (raises when it has not been built)."""
    global _lib
    if _lib is None:
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise RuntimeError(f"{p} missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        lib = C.CDLL(str(p))
        vp, i32, i64, u32, u64 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint32, C.c_uint64
        sig = {
            "insta_ctx_create": [C.c_int, vp, u64, C.POINTER(vp)],
            "insta_ctx_destroy": [vp],
            "insta_sync": [vp],
            "insta_memory_used": [vp, C.POINTER(u64)],
            "insta_stats_enable": [vp, C.c_int],
            "insta_stats_read": [vp, C.POINTER(Stats), C.c_int],
            "insta_canonical_set": [vp, C.c_int, vp, C.c_int, vp, C.c_int, vp],
            "insta_avatar_set_boxes": [vp, C.c_int, vp, vp, vp, vp],
            "insta_avatar_set_flags": [vp, C.c_int, u32],
            "insta_frame_upload": [vp, C.c_int, C.c_int, vp],
            "insta_frame_upload_batch": [vp, C.c_int, vp, C.c_int, C.POINTER(vp)],
            "insta_frame_upload_async": [vp, C.c_int, C.c_int, vp, C.c_double],
            "insta_frame_wait": [vp, C.c_int, C.c_int],
            "insta_frame_release": [vp, C.c_int, C.c_int],
            "insta_occupancy_from_mesh": [vp, C.c_int, C.c_int, C.c_double],
            "insta_occupancy_set": [vp, C.c_int, C.c_int, vp],
            "insta_occupancy_get": [vp, C.c_int, C.c_int, vp],
            "insta_density_grid_load": [vp, C.c_int, C.c_int, vp, u32, C.c_int],
            "insta_density_grid_reset": [vp, C.c_int, vp, u32],
            "insta_density_grid_update": [vp, C.c_int, C.POINTER(DensityUpdateDesc)],
            "insta_density_grid_read": [vp, C.c_int, vp],
            "insta_canonical_map": [vp, C.c_int, C.c_int, vp, u32, u32, i64],
            "insta_canonical_map_soa": [vp, C.c_int, C.c_int, vp, i64, vp, vp],
            "insta_training_samples": [vp, C.c_int, C.c_int, vp, vp, vp, vp, u32, i64, C.c_float, u32, vp, u32, vp, vp, vp],
            "insta_field_param_count": [C.POINTER(FieldDesc), C.POINTER(u64)],
            "insta_params_load": [vp, C.c_int, C.POINTER(FieldDesc), vp, u64],
            "insta_field_eval": [vp, C.c_int, vp, u32, i64, vp],
            "insta_field_eval_static": [vp, C.c_int, vp, u32, i64, vp],
            "insta_field_eval_training": [vp, C.c_int, vp, u32, i64, vp],
            "insta_field_backward": [vp, C.c_int, vp, u32, i64, vp, vp, vp],
            "insta_field_backward_ex": [vp, C.c_int, vp, u32, i64, vp, vp, vp, vp],
            "insta_extra_dims_gradient": [vp, C.POINTER(ExtraDimsGradientDesc)],
            "insta_adam_step": [vp, C.c_int, vp, C.POINTER(AdamConfig)],
            "insta_train_loss": [vp, C.POINTER(TrainLossDesc)],
            "insta_training_pixels": [vp, C.POINTER(TrainingPixelsDesc)],
            "insta_error_map_cdf": [vp, vp, u32, u32, u32, vp, vp, vp, vp],
            "insta_train_set_math": [vp, C.c_int],
            "insta_render": [vp, C.POINTER(RenderDesc), vp, vp],
            "insta_render_async": [vp, C.POINTER(RenderDesc), vp, vp],
            "insta_render_batch": [vp, C.POINTER(RenderDesc), C.c_int, C.POINTER(vp), C.POINTER(vp)],
            "insta_render_samples": [vp, C.POINTER(u64)],
            "insta_tuning_set": [vp, C.POINTER(Tuning)],
            "insta_tuning_get": [vp, C.POINTER(Tuning)],
            "insta_autotune": [vp, C.POINTER(RenderDesc), C.c_int, C.c_int, C.POINTER(Tuning), C.POINTER(C.c_float)],
            "insta_march_debug": [vp, C.POINTER(RenderDesc), C.c_int, vp, vp, vp],
            "insta_nearest_debug": [vp, C.c_int, C.c_int, vp, i64, vp],
            "insta_raycast": [vp, C.POINTER(RenderDesc), C.c_int, vp, vp, vp],
            "insta_server_create": [vp, C.POINTER(ServerConfig), C.POINTER(vp)],
            "insta_server_destroy": [vp],
            "insta_submit": [vp, C.POINTER(RenderDesc), vp, vp, vp, C.POINTER(u64)],
            "insta_poll": [vp, u64, C.POINTER(C.c_int), C.POINTER(C.c_double)],
            "insta_wait": [vp, u64, C.c_int, C.POINTER(C.c_int)],
            "insta_cancel": [vp, u64],
            "insta_server_release": [vp, u64],
            "insta_server_error": [vp, u64],
        }
        for name, args in sig.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = C.c_int
        lib.insta_last_error.argtypes = [vp]
        lib.insta_last_error.restype = C.c_char_p
        lib.insta_server_error.restype = C.c_char_p
        _lib = lib
    return _lib


def field_desc(fc, precision: int = PRECISION_FP16) -> FieldDesc:
    d = FieldDesc()
    d.n_levels, d.n_features_per_level, d.log2_hashmap_size = fc.n_levels, fc.n_features, fc.log2_table
    d.base_resolution, d.per_level_scale, d.aabb_scale = fc.base_res, fc.per_level_scale, fc.aabb_scale
    d.n_extra_dims = fc.n_extra
    d.density_neurons, d.density_hidden_layers, d.density_output_dims = fc.density_hidden, fc.density_layers, fc.density_out
    d.rgb_neurons, d.rgb_hidden_layers = fc.rgb_hidden, fc.rgb_layers
    d.precision = precision
    return d


def param_count(fc) -> int:
    n = C.c_uint64(0)
    rc = load().insta_field_param_count(C.byref(field_desc(fc)), C.byref(n))
    if rc:
        raise InstaError(rc, "invalid field description")
    return int(n.value)


def _addr(x):
    """Address of a numpy array (host) or a torch tensor (device or host)."""
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        assert x.flags["C_CONTIGUOUS"], "arrays must be C-contiguous"
        return C.c_void_p(x.ctypes.data)
    if hasattr(x, "data_ptr"):
        assert x.is_contiguous(), "tensors must be contiguous"
        return C.c_void_p(x.data_ptr())
    if isinstance(x, int):
        return C.c_void_p(x)
    raise TypeError(f"unsupported buffer type {type(x)}")


class Context:
    """One device, one stream, a device-memory budget; owns avatar residency."""

    def __init__(self, device: int = 0, stream: int | None = None, budget_bytes: int = 0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.insta_ctx_create(device, C.c_void_p(stream) if stream else None, budget_bytes, C.byref(h))
        if rc:
            raise InstaError(rc, "insta_ctx_create failed (no sm_10x GPU or CUDA error)")
        self.h = h

    def _check(self, rc):
        if rc:
            raise InstaError(rc, self.lib.insta_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.insta_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        self._check(self.lib.insta_sync(self.h))

    def memory_used(self) -> int:
        v = C.c_uint64(0)
        self._check(self.lib.insta_memory_used(self.h, C.byref(v)))
        return int(v.value)

    def stats_enable(self, stage_timing: bool = True):
        self._check(self.lib.insta_stats_enable(self.h, int(stage_timing)))

    def stats(self, reset: bool = False) -> dict:
        s = Stats()
        self._check(self.lib.insta_stats_read(self.h, C.byref(s), int(reset)))
        return {"kernel_launches": int(s.kernel_launches), "last_render_samples": int(s.last_render_samples),
                "stage_ms": {n: float(s.stage_ms[i]) for i, n in enumerate(STAGES)},
                "stage_calls": {n: int(s.stage_calls[i]) for i, n in enumerate(STAGES)},
                "walk": {k: int(getattr(s, "walk_" + k)) for k in ("warps", "inner_nodes", "leaves", "bound_tests", "exact_tests")}}

    def canonical_set(self, avatar, verts, faces, mask=None):
        v = np.ascontiguousarray(verts, dtype=np.float32)
        f = np.ascontiguousarray(faces, dtype=np.int32)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint32)
        self._check(self.lib.insta_canonical_set(self.h, avatar, _addr(v), len(v), _addr(f), len(f), _addr(m)))

    def set_boxes(self, avatar, train=None, render=None):
        def arr(x):
            return None if x is None else np.ascontiguousarray(x, dtype=np.float32)
        tmin, tmax = (None, None) if train is None else (arr(train[0]), arr(train[1]))
        rmin, rmax = (None, None) if render is None else (arr(render[0]), arr(render[1]))
        self._check(self.lib.insta_avatar_set_boxes(self.h, avatar, _addr(tmin), _addr(tmax), _addr(rmin), _addr(rmax)))

    def set_flags(self, avatar, flags):
        self._check(self.lib.insta_avatar_set_flags(self.h, avatar, flags))

    def frame_upload(self, avatar, frame, verts):
        v = verts if hasattr(verts, "data_ptr") else np.ascontiguousarray(verts, dtype=np.float32)
        self._check(self.lib.insta_frame_upload(self.h, avatar, frame, _addr(v)))

    def frame_upload_batch(self, avatar, frames, verts_list):
        vs = [v if hasattr(v, "data_ptr") else np.ascontiguousarray(v, dtype=np.float32) for v in verts_list]
        ids = np.ascontiguousarray(frames, dtype=np.int32)
        ptrs = (C.c_void_p * len(vs))(*[_addr(v).value for v in vs])
        self._check(self.lib.insta_frame_upload_batch(self.h, avatar, _addr(ids), len(vs), ptrs))

    def frame_upload_async(self, avatar, frame, verts, occupancy_radius=0.0):
        v = verts if hasattr(verts, "data_ptr") else np.ascontiguousarray(verts, dtype=np.float32)
        self._keep_async = v   # the buffer must outlive the copy when it is pinned or on the device
        self._check(self.lib.insta_frame_upload_async(self.h, avatar, frame, _addr(v), float(occupancy_radius)))

    def frame_wait(self, avatar, frame):
        self._check(self.lib.insta_frame_wait(self.h, avatar, frame))

    def frame_release(self, avatar, frame):
        self._check(self.lib.insta_frame_release(self.h, avatar, frame))

    def occupancy_from_mesh(self, avatar, frame, radius=0.015):
        self._check(self.lib.insta_occupancy_from_mesh(self.h, avatar, frame, float(radius)))

    def occupancy_set(self, avatar, frame, bits):
        b = np.ascontiguousarray(bits, dtype=np.uint8)
        self._check(self.lib.insta_occupancy_set(self.h, avatar, frame, _addr(b)))

    def occupancy_get(self, avatar, frame) -> np.ndarray:
        b = np.zeros(8 * 128 ** 3 // 8, dtype=np.uint8)
        self._check(self.lib.insta_occupancy_get(self.h, avatar, frame, _addr(b)))
        return b

    def density_grid_load(self, avatar, frame, grid, n_cascades):
        """grid: float32 or float16 array/tensor [n_cascades * 128^3] (Morton order per cascade)."""
        g = grid if hasattr(grid, "data_ptr") else np.ascontiguousarray(grid)
        fp16 = int(str(g.dtype).endswith("float16"))
        self._check(self.lib.insta_density_grid_load(self.h, avatar, frame, _addr(g), n_cascades, fp16))

    def density_grid_reset(self, avatar, n_cascades, grid=None):
        g = None if grid is None else (grid if hasattr(grid, "data_ptr") else np.ascontiguousarray(grid, dtype=np.float32))
        self._check(self.lib.insta_density_grid_reset(self.h, avatar, _addr(g) if g is not None else None, n_cascades))

    def density_grid_update(self, avatar, desc: DensityUpdateDesc):
        self._check(self.lib.insta_density_grid_update(self.h, avatar, C.byref(desc)))

    def density_grid_read(self, avatar, n_cascades) -> np.ndarray:
        g = np.zeros(n_cascades * 128 ** 3, dtype=np.float32)
        self._check(self.lib.insta_density_grid_read(self.h, avatar, _addr(g)))
        return g

    def training_samples(self, avatar, grid_frame, rays, image, start_rand, max_samples, coords, stride, ray_indices,
                         numsteps, counters, cone_angle=1 / 256, extra=None, n_images=0):
        self._check(self.lib.insta_training_samples(self.h, avatar, grid_frame, _addr(rays), _addr(image), _addr(start_rand),
                                                    _addr(extra), n_images, len(rays), float(cone_angle), max_samples,
                                                    _addr(coords), stride, _addr(ray_indices), _addr(numsteps), _addr(counters)))

    def canonical_map(self, avatar, frame, coords, stride, n_extra, n):
        self._check(self.lib.insta_canonical_map(self.h, avatar, frame, _addr(coords), stride, n_extra, n))

    def canonical_map_soa(self, avatar, frame, pts, n, out_idx, out_canon):
        self._check(self.lib.insta_canonical_map_soa(self.h, avatar, frame, _addr(pts), n, _addr(out_idx), _addr(out_canon)))

    def params_load(self, avatar, fc, params, precision=PRECISION_FP16):
        p = params if hasattr(params, "data_ptr") else np.ascontiguousarray(params).view(np.uint16)
        n = p.numel() if hasattr(p, "numel") else p.size
        self._check(self.lib.insta_params_load(self.h, avatar, C.byref(field_desc(fc, precision)), _addr(p), n))

    def field_eval(self, avatar, coords, stride, n, out4):
        self._check(self.lib.insta_field_eval(self.h, avatar, _addr(coords), stride, n, _addr(out4)))

    def field_eval_training(self, avatar, coords, stride, n, out4):
        """insta_field_eval_training: the training weights (differ from field_eval under an Ema)."""
        self._check(self.lib.insta_field_eval_training(self.h, avatar, _addr(coords), stride, n, _addr(out4)))

    def field_eval_static(self, avatar, coords, stride, n, out4):
        """insta_field_eval without device allocations (n <= 16384, shared fixed scratch)."""
        self._check(self.lib.insta_field_eval_static(self.h, avatar, _addr(coords), stride, n, _addr(out4)))

    def field_backward(self, avatar, coords, stride, n, dl_dout=None, grad=None, out4=None, dl_dextra=None):
        """insta_field_backward: ADDS d(sum dl_dout . out)/d(params) into grad (f32, snapshot order);
        with dl_dextra (f32[n][n_extra]) insta_field_backward_ex also writes the expression-dim
        gradients."""
        if dl_dextra is None:
            self._check(self.lib.insta_field_backward(self.h, avatar, _addr(coords), stride, n, _addr(dl_dout), _addr(grad), _addr(out4)))
        else:
            self._check(self.lib.insta_field_backward_ex(self.h, avatar, _addr(coords), stride, n, _addr(dl_dout), _addr(grad), _addr(out4),
                                                         _addr(dl_dextra)))

    def train_set_math(self, tf32, tcgen05=False):
        """insta_train_set_math: TF32 tensor-core layer products in the backward (else FP32), or with
        tcgen05=True the library's own tcgen05 kernel (FP16 operands, FP32 accumulation)."""
        self._check(self.lib.insta_train_set_math(self.h, 2 if tcgen05 else (1 if tf32 else 0)))

    def adam_step(self, avatar, grad, learning_rate=1.75e-3, beta1=0.9, beta2=0.99, epsilon=1e-15, l2_reg=1e-6, ema_decay=0.0,
                  loss_scale=1.0):
        """insta_adam_step; ema_decay > 0 adds the Ema wrapper (its average becomes the field's parameters);
        loss_scale is the factor the gradient carries (128 for gradients from insta_train_loss)."""
        cfg = AdamConfig(learning_rate, beta1, beta2, epsilon, l2_reg, ema_decay, loss_scale)
        self._check(self.lib.insta_adam_step(self.h, avatar, _addr(grad), C.byref(cfg)))

    _LOSS_PTRS = ("rays", "target", "background", "exposure", "depth", "seg_mask", "mean_density", "rays_counter", "ray_indices",
                  "numsteps", "coords", "network_output", "numsteps_counter", "coords_out", "dloss_doutput", "loss_output", "pdf",
                  "error_map", "image_xy", "image_index")

    def train_loss(self, **kw):
        """insta_train_loss: keyword arguments are insta_train_loss_desc's fields (buffers as
        device tensors); loss_type / depth_loss_type also accept names ("huber", "l2", ...)."""
        d = TrainLossDesc()
        d.loss_scale, d.seg_mask_supervision_lambda = 128.0, 1.0
        d.aabb_max[:] = [1.0, 1.0, 1.0]
        for k, v in kw.items():
            if k in self._LOSS_PTRS:
                a = _addr(v)
                setattr(d, k, a.value if a is not None else None)
            elif k in ("aabb_min", "aabb_max"):
                getattr(d, k)[:] = [float(x) for x in v]
            elif k == "error_map_res":
                d.error_map_res[:] = [int(x) for x in v]
            elif k in ("loss_type", "depth_loss_type") and isinstance(v, str):
                setattr(d, k, LOSS_TYPES[v.lower()])
            else:
                setattr(d, k, v)
        self._check(self.lib.insta_train_loss(self.h, C.byref(d)))

    def training_pixels(self, n_rays, n_images, rng_state, rng_inc, out_image, out_xy, out_pdf=None, out_background=None,
                        n_rays_total=0, resolution=None, snap=False, cdfs=None, cdf_res=(0, 0)):
        """insta_training_pixels: the batch's image and pixel draws (device buffers); cdfs =
        (cdf_x_cond_y, cdf_y, cdf_img) from error_map_cdf, or None for uniform draws."""
        d = TrainingPixelsDesc()
        d.n_rays, d.n_rays_total, d.n_images = n_rays, n_rays_total, n_images
        d.resolution = None if resolution is None else _addr(resolution).value
        d.snap_to_pixel_centers = int(snap)
        d.rng_state, d.rng_inc = rng_state, rng_inc
        if cdfs is not None:
            d.cdf_x_cond_y, d.cdf_y, d.cdf_img = (_addr(a).value for a in cdfs)
        d.cdf_res[:] = [int(x) for x in cdf_res]
        d.out_image, d.out_xy = _addr(out_image).value, _addr(out_xy).value
        d.out_pdf = None if out_pdf is None else _addr(out_pdf).value
        d.out_background = None if out_background is None else _addr(out_background).value
        self._check(self.lib.insta_training_pixels(self.h, C.byref(d)))

    def extra_dims_gradient(self, max_rays, n_extra_dims, n_images, rays_counter, ray_indices, numsteps, image_index, dl_dextra,
                            extra_dims_gradient):
        """insta_extra_dims_gradient on device buffers (per kept ray its samples' expression-dim
        gradients summed into its image's row, added to)."""
        d = ExtraDimsGradientDesc()
        d.max_rays, d.n_extra_dims, d.n_images = max_rays, n_extra_dims, n_images
        for k, v in (("rays_counter", rays_counter), ("ray_indices", ray_indices), ("numsteps", numsteps), ("image_index", image_index),
                     ("dl_dextra", dl_dextra), ("extra_dims_gradient", extra_dims_gradient)):
            setattr(d, k, _addr(v).value)
        self._check(self.lib.insta_extra_dims_gradient(self.h, C.byref(d)))

    def error_map_cdf(self, error_map, n_images, res_x, res_y, cdf_x_cond_y, cdf_y, cdf_img, pmf_img=None):
        """insta_error_map_cdf on device buffers."""
        self._check(self.lib.insta_error_map_cdf(self.h, _addr(error_map), n_images, res_x, res_y, _addr(cdf_x_cond_y), _addr(cdf_y),
                                                 _addr(cdf_img), _addr(pmf_img)))

    @staticmethod
    def render_desc(avatar, frame, width, height, focal, cam, cone_angle=1 / 256, spp=0, min_transmittance=0.01,
                    max_samples=1024, snap=True, linear_colors=False, extra_dims=None, out_samples=None) -> RenderDesc:
        r = RenderDesc()
        r.avatar, r.frame, r.width, r.height = avatar, frame, width, height
        r.focal_length[:] = [float(focal[0]), float(focal[1])]
        r.screen_center[:] = [0.5, 0.5]
        r.camera[:] = [float(x) for x in np.asarray(cam, dtype=np.float32).reshape(-1)]
        r.cone_angle = float(np.float32(cone_angle))
        r.min_transmittance = float(min_transmittance)
        r.spp, r.snap_to_pixel_centers, r.max_samples_per_ray = spp, int(snap), max_samples
        r.linear_colors = int(linear_colors)
        r.extra_dims = None if extra_dims is None else extra_dims.ctypes.data
        r.out_samples = None if out_samples is None else _addr(out_samples).value
        return r

    def render(self, req: RenderDesc, out_rgba, out_depth):
        self._check(self.lib.insta_render(self.h, C.byref(req), _addr(out_rgba), _addr(out_depth)))

    def render_async(self, req: RenderDesc, out_rgba, out_depth):
        """insta_render_async: host outputs are complete after sync()."""
        self._check(self.lib.insta_render_async(self.h, C.byref(req), _addr(out_rgba), _addr(out_depth)))

    def render_batch(self, reqs, out_rgba, out_depth):
        """reqs: list of RenderDesc; out_rgba / out_depth: lists of buffers (one pair per request)."""
        n = len(reqs)
        arr = (RenderDesc * n)(*reqs)
        pr = (C.c_void_p * n)(*[_addr(b).value for b in out_rgba])
        pd = (C.c_void_p * n)(*[_addr(b).value for b in out_depth])
        self._check(self.lib.insta_render_batch(self.h, arr, n, pr, pd))

    def tuning_set(self, max_steps_per_round=0, sort_cell_bits=0, mlp_ctas_per_sm=0, deform_blocks_per_sm=0, bvh_top_nodes=0,
                   fused_field_stage=0, mlp_slots=0):
        """insta_tuning_set: the wavefront's launch shapes (0 keeps a field's built-in choice)."""
        t = Tuning(max_steps_per_round, sort_cell_bits, mlp_ctas_per_sm, deform_blocks_per_sm, bvh_top_nodes, fused_field_stage, mlp_slots)
        self._check(self.lib.insta_tuning_set(self.h, C.byref(t)))

    def tuning_get(self) -> dict:
        t = Tuning()
        self._check(self.lib.insta_tuning_get(self.h, C.byref(t)))
        return {f: int(getattr(t, f)) for f, _ in Tuning._fields_}

    def autotune(self, reqs, repeats=3):
        """insta_autotune over a list of RenderDesc; returns (tuning dict, ms per batch)."""
        n = len(reqs)
        arr = (RenderDesc * n)(*reqs)
        t, ms = Tuning(), C.c_float(0)
        self._check(self.lib.insta_autotune(self.h, arr, n, repeats, C.byref(t), C.byref(ms)))
        return {f: int(getattr(t, f)) for f, _ in Tuning._fields_}, float(ms.value)

    def render_samples(self) -> int:
        v = C.c_uint64(0)
        self._check(self.lib.insta_render_samples(self.h, C.byref(v)))
        return int(v.value)

    def raycast(self, req: RenderDesc, out_rgba, out_depth, out_tri=None, color_normal=False):
        self._check(self.lib.insta_raycast(self.h, C.byref(req), int(color_normal), _addr(out_rgba), _addr(out_depth), _addr(out_tri)))

    def nearest_debug(self, avatar, frame, pts, n, out_idx):
        self._check(self.lib.insta_nearest_debug(self.h, avatar, frame, _addr(pts), n, _addr(out_idx)))

    def march_debug(self, req: RenderDesc, max_out, out_t, out_dt, out_n):
        self._check(self.lib.insta_march_debug(self.h, C.byref(req), max_out, _addr(out_t), _addr(out_dt), _addr(out_n)))


class Server:
    """The request loop (insta_server_*): owns `ctx` from creation to close()."""

    def __init__(self, ctx: Context, max_inflight=16, max_inflight_pixels=1 << 22, occupancy_radius=0.015, rounds_per_launch=0,
                 round_samples=0):
        self.ctx = ctx
        self.lib = ctx.lib
        cfg = ServerConfig(max_inflight, max_inflight_pixels, occupancy_radius, rounds_per_launch, round_samples)
        h = C.c_void_p()
        ctx._check(self.lib.insta_server_create(ctx.h, C.byref(cfg), C.byref(h)))
        self.h = h
        self._keep = {}

    def submit(self, req: RenderDesc, frame_verts, out_rgba, out_depth) -> int:
        v = None if frame_verts is None else np.ascontiguousarray(frame_verts, dtype=np.float32)
        t = C.c_uint64(0)
        rc = self.lib.insta_submit(self.h, C.byref(req), _addr(v), _addr(out_rgba), _addr(out_depth), C.byref(t))
        if rc:
            raise InstaError(rc, "insta_submit failed")
        self._keep[t.value] = (out_rgba, out_depth)   # outputs stay alive until the ticket is released
        return t.value

    def poll(self, ticket):
        st, lat = C.c_int(0), C.c_double(0)
        rc = self.lib.insta_poll(self.h, ticket, C.byref(st), C.byref(lat))
        if rc:
            raise InstaError(rc, "insta_poll failed")
        return st.value, lat.value

    def wait(self, ticket, timeout_ms=-1) -> int:
        st = C.c_int(0)
        rc = self.lib.insta_wait(self.h, ticket, timeout_ms, C.byref(st))
        if rc:
            raise InstaError(rc, "insta_wait failed")
        return st.value

    def cancel(self, ticket):
        self.lib.insta_cancel(self.h, ticket)

    def error(self, ticket) -> str:
        return self.lib.insta_server_error(self.h, ticket).decode()

    def release(self, ticket):
        self.lib.insta_server_release(self.h, ticket)
        self._keep.pop(ticket, None)

    def close(self):
        if getattr(self, "h", None):
            self.lib.insta_server_destroy(self.h)
            self.h = None
