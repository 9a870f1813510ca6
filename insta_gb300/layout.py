"""Parameter layout of the avatar field, in snapshot order.

NerfNetwork::set_params (NGP/nerf_network.h:492-525) lays the flat FP16
parameter vector out as: density MLP, rgb MLP, position (hash-grid)
encoding, direction encoding (spherical harmonics, no parameters).  The
tiny-cuda-nn internals of each block are not in the reference repository, so
this library fixes its own block layout and the C++ side
(``field_layout`` in ``insta_gb300/csrc/insta_abi.cu``) computes the same offsets:

* MLP layer ``k``: row-major ``[n_out][n_in]`` FP16 matrix, no bias;
* hash level ``l``: ``scale_l = exp2(l * log2(b)) * N_min - 1`` (float),
  ``res_l = ceil(scale_l) + 1``, ``size_l = min(roundup8(res_l^3), 2^log2T)``
  entries of ``n_features`` FP16 values, levels stored back to back.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class Layout:
    density_offset: int
    rgb_offset: int
    table_offset: int
    total: int
    level_offsets: list
    level_res: list
    level_size: list
    level_scale: list
    layers: list            # (offset, n_out, n_in, is_output)

    def mlp_layers(self, density_gain: float = 1.0):
        for i, (off, n_out, n_in, is_out) in enumerate(self.layers):
            gain = density_gain if (is_out and off < self.rgb_offset) else 1.0
            yield off, n_out, n_in, gain


def level_scale(per_level_scale: float, base_res: int, level: int) -> float:
    f = np.float32
    return float(f(f(np.exp2(f(f(level) * f(np.log2(f(per_level_scale)))))) * f(base_res)) - f(1.0))


def field_layout(cfg) -> Layout:
    n_enc = cfg.n_levels * cfg.n_features
    n_in = n_enc + cfg.n_extra
    layers = []
    off = 0
    widths = [n_in] + [cfg.density_hidden] * cfg.density_layers + [cfg.density_out]
    for k in range(len(widths) - 1):
        layers.append((off, widths[k + 1], widths[k], k == len(widths) - 2))
        off += widths[k + 1] * widths[k]
    rgb_off = off
    widths = [cfg.density_out + 16] + [cfg.rgb_hidden] * cfg.rgb_layers + [cfg.rgb_out_padded]
    for k in range(len(widths) - 1):
        layers.append((off, widths[k + 1], widths[k], k == len(widths) - 2))
        off += widths[k + 1] * widths[k]
    table_off = off
    T = 1 << cfg.log2_table
    lo, lr, ls, lsc = [], [], [], []
    eoff = 0
    for l in range(cfg.n_levels):
        s = level_scale(cfg.per_level_scale, cfg.base_res, l)
        res = int(math.ceil(np.float32(s))) + 1
        size = min((res ** 3 + 7) // 8 * 8, T)
        lo.append(eoff); lr.append(res); ls.append(size); lsc.append(s)
        eoff += size
    return Layout(0, rgb_off, table_off, table_off + eoff * cfg.n_features, lo, lr, ls, lsc, layers)
