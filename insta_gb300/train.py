"""One training step of the avatar's field over the C ABI: Testbed::train_nerf_step
(instant-ngp/src/testbed_nerf.cu:3170-3380) as INSTA runs it.

    insta_training_samples   generate_training_samples_nerf + surface_closest_point (:3252-3293)
    insta_field_eval_training  inference_mixed_precision on the uncompacted records with the
                             training weights (not the Ema's average)                 (:3295)
    insta_train_loss         compute_loss_kernel_train_nerf + fill_rollover          (:3298-3357)
    insta_field_backward     forward + backward on the compacted batch, gradients
                             overwritten (EGradientMode::Overwrite)                  (:3364-3368)
    insta_adam_step          the optimizer step                                      (train_nerf)

The caller draws the batch's rays, training-image ids, jitter, target samples and backgrounds
the way the reference's sampler does (device tensors, complete on torch's current stream when
step() is called; the context runs on its own stream and step() orders torch's work before
it).  Each step reads the two sample counters back to the host (the reference reads its
counters back too, one step later), so that the field evaluation covers exactly the records
the march wrote.  The optimizer is Adam in the configuration's Ema wrapper (decay 0.95): the
field renders with the averaged weights.  Not built: error-map importance sampling, camera /
exposure / extra-dims optimisation.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import abi
from . import layout as _layout


@dataclass
class TrainConfig:
    """configs/nerf/main.json-style settings (loss Huber, Ema(0.95) of Adam 1.75e-3, beta 0.9/0.99)."""
    n_rays_per_batch: int = 4096
    target_batch_size: int = 1 << 18
    max_samples: int = 1 << 20
    cone_angle: float = 0.0
    loss_type: str = "huber"
    depth_loss_type: str = "l1"
    srgb_targets: bool = True
    train_in_linear_colors: bool = False
    loss_scale: float = 128.0
    depth_supervision_lambda: float = 1.25   # "depth_weight"; no depth term without depth samples
    seg_mask_supervision_lambda: float = 40.0   # "seg_weight"
    near_distance: float = 0.2
    beta: float = 0.0
    penalize_density: bool = False
    aabb_min: tuple = (0.0, 0.0, 0.0)
    aabb_max: tuple = (1.0, 1.0, 1.0)
    tcgen05: bool = True               # the library's tcgen05 training kernel (FP16 operands, FP32 accumulation)
    tf32: bool = True                  # without it: TF32 tensor-core (else FP32) cuBLAS layer products
    adam: dict = field(default_factory=lambda: dict(learning_rate=1.75e-3, beta1=0.9, beta2=0.99, epsilon=1e-15, l2_reg=1e-6,
                                                    ema_decay=0.95))


class TrainStep:
    """Device buffers of one training batch and the step that runs the five entry points."""

    def __init__(self, ctx: abi.Context, avatar: int, fc, cfg: TrainConfig | None = None):
        import torch
        self.torch = torch
        self.ctx, self.avatar, self.fc = ctx, avatar, fc
        self.cfg = cfg = cfg or TrainConfig()
        if cfg.target_batch_size > cfg.max_samples:
            raise ValueError("target_batch_size must not exceed max_samples")
        self.stride = 11 + fc.n_extra
        n, m = cfg.n_rays_per_batch, cfg.max_samples
        dev = dict(device="cuda")
        self.coords = torch.zeros((m, self.stride), dtype=torch.float32, **dev)
        self.out = torch.zeros((m, 4), dtype=torch.float32, **dev)
        self.ray_indices = torch.zeros(n, dtype=torch.int32, **dev)
        self.numsteps = torch.zeros((n, 2), dtype=torch.int32, **dev)
        self.counters = torch.zeros(2, dtype=torch.int32, **dev)
        self.compacted = torch.zeros(1, dtype=torch.int32, **dev)
        self.coords_out = torch.zeros((cfg.target_batch_size, self.stride), dtype=torch.float32, **dev)
        self.dloss = torch.zeros((cfg.target_batch_size, 4), dtype=torch.float32, **dev)
        self.loss = torch.zeros(n, dtype=torch.float32, **dev)
        self.grad = torch.zeros(_layout.field_layout(fc).total, dtype=torch.float32, **dev)
        self.counters_host = torch.zeros(2, dtype=torch.int32, pin_memory=True)
        self.n_steps = 0
        self._last_kept = 0
        # the tcgen05 training kernel holds a field of at most 64 density inputs and 8 layers in one
        # CTA (wider fields, e.g. INSTA's 16 x 8 features + 16 expression dims, take the TF32 products)
        n_in = fc.n_levels * fc.n_features + fc.n_extra
        self.tcgen05 = cfg.tcgen05 and n_in <= 64 and fc.density_layers + fc.rgb_layers + 2 <= 8
        ctx.train_set_math(cfg.tf32, tcgen05=self.tcgen05)

    def step(self, grid_frame: int, rays, image, start_rand, target, background=None, extra=None, n_images: int = 0,
             depth=None, seg_mask=None, mean_density=None, exposure=None) -> dict:
        """One step.  rays f32[n][6], image i32[n], start_rand f32[n], target f32[n][4] (linear
        rgb + alpha), background f32[n][3] (sRGB), extra f32[n_images][n_extra]; device tensors
        with n = n_rays_per_batch.  Returns the step's counters and (lazily) its loss."""
        ctx, cfg = self.ctx, self.cfg
        n = cfg.n_rays_per_batch
        if len(rays) != n:
            raise ValueError(f"expected {n} rays, got {len(rays)}")
        self.counters.zero_()
        self.compacted.zero_()
        self.loss.zero_()
        self.grad.zero_()
        self.torch.cuda.current_stream().synchronize()   # torch's stream -> the context's stream
        ctx.training_samples(self.avatar, grid_frame, rays, image, start_rand, cfg.max_samples, self.coords, self.stride,
                             self.ray_indices, self.numsteps, self.counters, cone_angle=cfg.cone_angle, extra=extra,
                             n_images=n_images)
        ctx.sync()
        self.counters_host.copy_(self.counters)
        n_kept, n_samples = (int(x) for x in self.counters_host.numpy().view(np.uint32))
        n_samples = min(n_samples, cfg.max_samples)
        if n_samples > 0:
            # the loss reads the training weights (inference_mixed_precision with
            # use_inference_params = false), not the Ema's average
            ctx.field_eval_training(self.avatar, self.coords, self.stride, n_samples, self.out)
        ctx.train_loss(n_rays=n, max_rays=n, max_samples_compacted=cfg.target_batch_size,
                       target_batch_size=cfg.target_batch_size, aabb_min=cfg.aabb_min, aabb_max=cfg.aabb_max,
                       loss_type=cfg.loss_type, depth_loss_type=cfg.depth_loss_type, srgb_targets=int(cfg.srgb_targets),
                       train_in_linear_colors=int(cfg.train_in_linear_colors), loss_scale=cfg.loss_scale,
                       depth_supervision_lambda=cfg.depth_supervision_lambda,
                       seg_mask_supervision_lambda=cfg.seg_mask_supervision_lambda, near_distance=cfg.near_distance,
                       beta=cfg.beta, penalize_density=int(cfg.penalize_density), stride=self.stride, rays=rays,
                       target=target, background=background, exposure=exposure, depth=depth, seg_mask=seg_mask,
                       mean_density=mean_density, rays_counter=self.counters, ray_indices=self.ray_indices,
                       numsteps=self.numsteps, coords=self.coords, network_output=self.out,
                       numsteps_counter=self.compacted, coords_out=self.coords_out, dloss_doutput=self.dloss,
                       loss_output=self.loss)
        if n_samples > 0:
            ctx.field_backward(self.avatar, self.coords_out, self.stride, cfg.target_batch_size, self.dloss, self.grad)
            ctx.adam_step(self.avatar, self.grad, loss_scale=cfg.loss_scale, **cfg.adam)
        self.n_steps += 1
        self._last_kept = n_kept
        return {"rays_kept": n_kept, "samples": n_samples}

    def loss_value(self) -> float:
        """The last step's loss: sum of the kept rays' losses (each already divided by n_rays)."""
        self.ctx.sync()
        return float(self.loss[: self._last_kept].sum().item())
