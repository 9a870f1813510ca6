import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103a GPU and the built CUDA library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def avatar():
    from insta_gb300 import synthetic as S
    return S.make_avatar(0)


@pytest.fixture(scope="session")
def frame0(avatar):
    return avatar.frame(avatar.frame_coeffs(0))


@pytest.fixture(scope="session")
def oracle_frame(oracle, avatar, frame0):
    """Oracle triangles, adjacency and BVH for frame 0."""
    can = oracle.build_triangles(avatar.canonical, None, avatar.faces, avatar.mask)
    dtr = oracle.build_triangles(frame0, avatar.canonical, avatar.faces, avatar.mask)
    adj = oracle.adjacency(avatar.faces, avatar.n_verts)
    bvh = oracle.Bvh(dtr)
    return {"can": can, "def": dtr, "adj": adj, "bvh": bvh}


@pytest.fixture(scope="session")
def ctx():
    from insta_gb300 import abi
    c = abi.Context(0)
    yield c
    c.close()


def psnr(a, b, peak=1.0):
    mse = float(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2))
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)


def train_loss_batch(n_rays, seed, stride=11, max_steps=20):
    """Synthetic kept rays: per-ray sample blocks (contiguous, shuffled kept order), records inside
    the unit train box along each ray, raw network outputs, targets and backgrounds."""
    rng = np.random.default_rng(seed)
    counts = rng.integers(1, max_steps + 1, n_rays).astype(np.uint32)
    bases = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint32)
    n_s = int(counts.sum())
    rays = np.zeros((n_rays, 6), np.float32)
    rays[:, :3] = rng.uniform(-0.5, 0.0, (n_rays, 3))
    rays[:, 3:] = rng.normal(size=(n_rays, 3))
    coords = np.zeros((n_s, stride), np.float32)
    coords[:, 3] = rng.uniform(0, 0.02, n_s)
    coords[:, 5:8] = rng.uniform(0.2, 0.8, (n_s, 3))
    coords[:, 8:11] = 0.5
    if stride > 11:
        coords[:, 11:] = rng.uniform(-1, 1, (n_s, stride - 11))
    out = np.zeros((n_s, 4), np.float32)
    out[:, :3] = rng.normal(size=(n_s, 3))
    out[:, 3] = rng.uniform(-2, 3, n_s)
    target = rng.uniform(0, 1, (n_rays, 4)).astype(np.float32)
    target[::3, 3] = 1.0
    bg = rng.uniform(0, 1, (n_rays, 3)).astype(np.float32)
    perm = rng.permutation(n_rays).astype(np.uint32)        # kept ray k -> original ray perm[k]
    numsteps = np.stack([counts, bases], 1)                  # blocks in kept order
    return dict(rays=rays, target=target, background=bg, ray_indices=perm, numsteps=numsteps, coords=coords,
                network_output=out)


def loss_cfg(**kw):
    cfg = dict(n_rays=64, max_samples_compacted=1 << 16, target_batch_size=0, stride=11, aabb_min=(0, 0, 0),
               aabb_max=(1, 1, 1), loss_type=0, depth_loss_type=0, srgb_targets=1, train_in_linear_colors=0,
               penalize_density=0, loss_scale=1.0, depth_supervision_lambda=0.0, seg_mask_supervision_lambda=1.0,
               near_distance=0.0, beta=0.0)
    cfg.update(kw)
    return cfg
