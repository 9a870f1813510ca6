"""Seeded synthetic workloads standing in for INSTA's tracked-head datasets.

The reference's benchmarks run on captured actors (FLAME-topology meshes
per frame, src/tiny_mesh.cu:39-51) that are not distributed with it.  These
generators produce inputs with the same shapes, sizes and value ranges:

* a closed genus-0 head proxy with 5,122 vertices and 10,240 triangles
  (Fibonacci-sphere points triangulated by their convex hull), radius 0.1 m,
  centred at (0.5, 0.5, 0.5) -- the offset TinyMesh::load applies
  (src/tiny_mesh.cu:63-71);
* canonical shape = sphere + 8 seeded real spherical harmonics (l <= 4)
  of radial displacement with amplitude N(0, 0.01 m);
* deformed frame = canonical + sum of 50 seeded smooth per-vertex vector
  fields (low-order SH, 1.5 mm RMS each) times coefficients N(0, 0.3);
* per-triangle region ids (Face 2, EyeRegion 1, Lips 7, Torso 15 and
  optionally Boundary 0 -- include/rta/masking.h:30-48) from spherical caps;
* query points uniform in a 1 cm shell around the deformed surface;
* a pinhole camera 1 m from the head with a 20 degree vertical field of view;
* hash-grid parameters ~U(-0.1, 0.1) and Kaiming-uniform MLP weights (FP16).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

CENTER = np.array([0.5, 0.5, 0.5], dtype=np.float64)
RADIUS = 0.1
N_VERTS = 5122

MASK_BOUNDARY, MASK_EYE, MASK_FACE, MASK_LIPS, MASK_TORSO = 0, 1, 2, 7, 15


def _real_sh(lmax: int, dirs: np.ndarray) -> np.ndarray:
    """Real spherical harmonics up to degree lmax (orthonormal), columns ordered (l, m)."""
    x, y, z = dirs[:, 0], dirs[:, 1], dirs[:, 2]
    theta = np.arccos(np.clip(z, -1.0, 1.0))
    phi = np.arctan2(y, x)
    ct = np.cos(theta)
    cols = []
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            am = abs(m)
            # associated Legendre P_l^m(ct) by the standard recurrence
            pmm = np.ones_like(ct)
            somx2 = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
            fact = 1.0
            for _ in range(am):
                pmm = -pmm * fact * somx2
                fact += 2.0
            if l == am:
                plm = pmm
            else:
                pmmp1 = ct * (2 * am + 1) * pmm
                if l == am + 1:
                    plm = pmmp1
                else:
                    pll = None
                    for ll in range(am + 2, l + 1):
                        pll = ((2 * ll - 1) * ct * pmmp1 - (ll + am - 1) * pmm) / (ll - am)
                        pmm, pmmp1 = pmmp1, pll
                    plm = pll
            k = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
            if m == 0:
                cols.append(k * plm)
            elif m > 0:
                cols.append(math.sqrt(2.0) * k * np.cos(m * phi) * plm)
            else:
                cols.append(math.sqrt(2.0) * k * np.sin(am * phi) * plm)
    return np.stack(cols, axis=1)


def sphere_topology(n_verts: int = N_VERTS):
    """Unit directions (n_verts, 3) and outward-oriented faces (2 n_verts - 4, 3), int32.

    Fibonacci-lattice points triangulated by their convex hull; faces are put in
    a canonical order (rotated so the smallest vertex index leads, then sorted)
    so the topology does not depend on the hull library's output order.
    """
    from scipy.spatial import ConvexHull

    i = np.arange(n_verts, dtype=np.float64) + 0.5
    z = 1.0 - 2.0 * i / n_verts
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    golden = math.pi * (3.0 - math.sqrt(5.0))
    phi = golden * np.arange(n_verts)
    dirs = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    faces = ConvexHull(dirs).simplices.astype(np.int64)
    a, b, c = dirs[faces[:, 0]], dirs[faces[:, 1]], dirs[faces[:, 2]]
    flip = np.einsum("ij,ij->i", np.cross(b - a, c - a), a + b + c) < 0
    faces[flip] = faces[flip][:, [0, 2, 1]]
    # canonical rotation: smallest index first, orientation preserved
    k = np.argmin(faces, axis=1)
    faces = np.stack([faces[np.arange(len(faces)), (k + s) % 3] for s in range(3)], axis=1)
    order = np.lexsort((faces[:, 2], faces[:, 1], faces[:, 0]))
    return dirs, faces[order].astype(np.int32)


@dataclass
class Avatar:
    """One synthetic actor: canonical mesh, region masks and basis fields."""
    dirs: np.ndarray
    faces: np.ndarray
    canonical: np.ndarray          # (V, 3) float32
    mask: np.ndarray               # (F,) uint32
    basis: np.ndarray              # (50, V, 3) float64
    seed: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def n_verts(self) -> int:
        return int(self.canonical.shape[0])

    @property
    def n_faces(self) -> int:
        return int(self.faces.shape[0])

    def frame(self, coeffs: np.ndarray) -> np.ndarray:
        """Deformed vertices (V, 3) float32 for a coefficient vector over the basis fields."""
        disp = np.tensordot(np.asarray(coeffs, dtype=np.float64), self.basis, axes=(0, 0))
        return (self.canonical.astype(np.float64) + disp).astype(np.float32)

    def frame_coeffs(self, frame_seed: int) -> np.ndarray:
        return np.random.default_rng([self.seed, 1000 + frame_seed]).normal(0.0, 0.3, size=self.basis.shape[0])

    def render_aabb(self):
        """Canonical mesh AABB inflated by 0.15 x its diagonal (src/tiny_mesh.cu:157-162)."""
        v = self.canonical.astype(np.float32)
        mn, mx = v.min(axis=0), v.max(axis=0)
        infl = np.float32(np.linalg.norm((mx - mn).astype(np.float32)) * np.float32(0.15))
        return (mn - infl).astype(np.float32), (mx + infl).astype(np.float32)


def _cap_masks(dirs: np.ndarray, faces: np.ndarray, with_boundary: bool) -> np.ndarray:
    cen = dirs[faces].mean(axis=1)
    cen /= np.linalg.norm(cen, axis=1, keepdims=True)
    mask = np.full(len(faces), MASK_TORSO, dtype=np.uint32)

    def cap(axis, deg):
        a = np.asarray(axis, dtype=np.float64)
        a /= np.linalg.norm(a)
        return cen @ a > math.cos(math.radians(deg))

    mask[cap([0, 0.1, 1], 55)] = MASK_FACE
    mask[cap([0.35, 0.3, 0.89], 12)] = MASK_EYE
    mask[cap([-0.35, 0.3, 0.89], 12)] = MASK_EYE
    mask[cap([0.0, -0.4, 0.9], 14)] = MASK_LIPS
    if with_boundary:
        mask[cap([0, -1, 0.2], 18)] = MASK_BOUNDARY
    return mask


def make_avatar(seed: int = 0, n_verts: int = N_VERTS, with_boundary: bool = False,
                n_basis: int = 50, basis_rms: float = 1.5e-3) -> Avatar:
    dirs, faces = sphere_topology(n_verts)
    rng = np.random.default_rng([seed, 7])
    sh = _real_sh(4, dirs)                               # (V, 25)
    pick = rng.choice(sh.shape[1], size=8, replace=False)
    amp = rng.normal(0.0, 0.01, size=8)
    radius = RADIUS + sh[:, pick] @ amp
    canonical = (CENTER + dirs * radius[:, None]).astype(np.float32)
    low = sh[:, :9]                                      # l <= 2
    basis = np.empty((n_basis, n_verts, 3))
    for k in range(n_basis):
        w = rng.normal(size=(9, 3))
        f = low @ w
        f *= basis_rms / math.sqrt(np.mean(np.sum(f * f, axis=1)))
        basis[k] = f
    mask = _cap_masks(dirs, faces, with_boundary)
    return Avatar(dirs=dirs, faces=faces, canonical=canonical, mask=mask, basis=basis, seed=seed)


def shell_points(verts: np.ndarray, faces: np.ndarray, n: int, seed: int = 0,
                 half_width: float = 5e-3) -> np.ndarray:
    """n points: area-weighted surface samples offset along the face normal by U(-w, w)."""
    rng = np.random.default_rng([seed, 11])
    v = verts.astype(np.float64)
    a, b, c = v[faces[:, 0]], v[faces[:, 1]], v[faces[:, 2]]
    nrm = np.cross(b - a, c - a)
    area = 0.5 * np.linalg.norm(nrm, axis=1)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    f = rng.choice(len(faces), size=n, p=area / area.sum())
    r1, r2 = rng.random(n), rng.random(n)
    s = np.sqrt(r1)
    p = (1 - s)[:, None] * a[f] + (s * (1 - r2))[:, None] * b[f] + (s * r2)[:, None] * c[f]
    p += nrm[f] * rng.uniform(-half_width, half_width, size=n)[:, None]
    return p.astype(np.float32)


def camera(yaw_deg: float = 0.0, distance: float = 1.0, fov_y_deg: float = 20.0,
           width: int = 512, height: int = 512):
    """Pinhole camera looking at the head centre: (3x4 [R | origin] float32, focal (2,))."""
    yaw = math.radians(yaw_deg)
    origin = CENTER + distance * np.array([math.sin(yaw), 0.0, math.cos(yaw)])
    fwd = CENTER - origin
    fwd /= np.linalg.norm(fwd)
    down = np.array([0.0, -1.0, 0.0])
    down -= fwd * (down @ fwd)
    down /= np.linalg.norm(down)
    right = np.cross(down, fwd)
    cam = np.zeros((3, 4), dtype=np.float32)
    cam[:, 0], cam[:, 1], cam[:, 2], cam[:, 3] = right, down, fwd, origin
    fy = 0.5 * height / math.tan(math.radians(fov_y_deg) / 2.0)
    return cam, np.array([fy, fy], dtype=np.float32)


@dataclass
class FieldConfig:
    """Hash grid + MLP shapes (configs/nerf/main.json-style keys)."""
    n_levels: int = 16
    n_features: int = 2
    log2_table: int = 19
    base_res: int = 16
    aabb_scale: int = 2
    n_extra: int = 0
    density_hidden: int = 64
    density_layers: int = 1
    density_out: int = 16
    rgb_hidden: int = 64
    rgb_layers: int = 2
    rgb_out_padded: int = 16

    @property
    def per_level_scale(self) -> float:
        """Testbed::reset_network (ngp/src/testbed.cu:2246-2258), evaluated in float."""
        f = np.float32
        return float(f(np.exp(f(np.log(f(2048.0) * f(self.aabb_scale) / f(self.base_res))) / f(self.n_levels - 1))))


def insta_field_config() -> FieldConfig:
    """The field INSTA trains with its shipped configuration (configs/nerf/main.json: 16 levels of
    8 features, 2^18 entries per level, base resolution 16; 16 expression dims appended to the
    density input ("exp_params"); density MLP 2 hidden layers of 64, 16 outputs; colour MLP 3
    hidden layers of 64)."""
    return FieldConfig(n_levels=16, n_features=8, log2_table=18, base_res=16, n_extra=16, density_layers=2, rgb_layers=3)


def field_params(cfg: FieldConfig, seed: int = 0, density_gain: float = 1.0) -> np.ndarray:
    """FP16 parameter blob in snapshot order: density MLP, rgb MLP, hash table
    (NerfNetwork::set_params, NGP/nerf_network.h:492-525).  Each MLP layer is a
    row-major [n_out][n_in] matrix; the hash table is [entries][n_features]."""
    from . import layout as _layout
    lay = _layout.field_layout(cfg)
    rng = np.random.default_rng([seed, 23])
    out = np.empty(lay.total, dtype=np.float16)
    for (off, n_out, n_in, gain) in lay.mlp_layers(density_gain):
        bound = math.sqrt(6.0 / n_in) * gain
        out[off:off + n_out * n_in] = rng.uniform(-bound, bound, size=n_out * n_in).astype(np.float16)
    out[lay.table_offset:] = rng.uniform(-0.1, 0.1, size=lay.total - lay.table_offset).astype(np.float16)
    return out
