"""Density-grid maintenance (update_density_grid_nerf with INSTA's random-frame warp) through the C
ABI against the oracle, on a small sample count.

Tolerances:
* sample cell indices and the frame each sample is warped through: bit-exact (integer PCG32
  stream, same float operations);
* warped (canonical) sample positions: |err| <= 1e-5 x the mesh bounding-box diagonal, as for
  the canonical map;
* grid cells a sample landed in: the field bound (4e-3 + 1e-2 |raw density|, FP16 outputs)
  carried through exp, relative; every other cell: bit-exact (decay product);
* the bitfield: the oracle's grid_to_bitfield of the device grid, bit-exact away from +-1e-5 of
  the threshold.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

AVATAR = 3
N_CASCADES = 2
MIN_CONE = np.float32(1.73205080757) / np.float32(1024)


@pytest.fixture(scope="module", params=["benchmark", "insta"])
def grid_avatar(ctx, avatar, request):
    """The benchmark field and INSTA's shipped one (16 levels x 8 features, expression dims)."""
    from insta_gb300 import synthetic as S
    ctx.canonical_set(AVATAR, avatar.canonical, avatar.faces, avatar.mask)
    frames = [avatar.frame(avatar.frame_coeffs(20 + k)) for k in range(3)]
    for k, f in enumerate(frames):
        ctx.frame_upload(AVATAR, k, f)
    fc = S.FieldConfig() if request.param == "benchmark" else S.insta_field_config()
    params = S.field_params(fc, seed=4)
    ctx.params_load(AVATAR, fc, params)
    ctx.sync()
    return frames, fc, params


def test_density_grid_update(ctx, oracle, avatar, grid_avatar):
    from insta_gb300 import abi
    frames, fc, params = grid_avatar
    rng = np.random.default_rng(5)
    grid0 = rng.uniform(0.0, 0.03, N_CASCADES * 128 ** 3).astype(np.float32)
    grid0[rng.random(grid0.size) < 0.01] = -1.0          # cells never updated
    ctx.density_grid_reset(AVATAR, N_CASCADES, grid0)
    grid_rng = oracle.Pcg32.seeded(1234)
    warp_rng = oracle.Pcg32.seeded(42)
    nu, nn = 40000, 24000
    n = nu + nn
    d_pos = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    d_idx = torch.zeros(n, dtype=torch.int32, device="cuda")
    desc = abi.DensityUpdateDesc()
    desc.decay = 0.95
    desc.n_uniform, desc.n_nonuniform, desc.n_cascades = nu, nn, N_CASCADES
    desc.aabb_min[:] = [0.0, 0.0, 0.0]
    desc.aabb_max[:] = [1.0, 1.0, 1.0]
    desc.grid_rng = abi.Pcg32State(grid_rng.state, grid_rng.inc)
    desc.warp_rng = abi.Pcg32State(warp_rng.state, warp_rng.inc)
    desc.ema_step = 7
    desc.n_frames = 3
    desc.bitfield_frame = 0
    desc.debug_pos = d_pos.data_ptr()
    desc.debug_idx = d_idx.data_ptr()
    ctx.density_grid_update(AVATAR, desc)
    g = ctx.density_grid_read(AVATAR, N_CASCADES)
    bits = ctx.occupancy_get(AVATAR, 0)
    pos = d_pos.cpu().numpy()
    idx = d_idx.cpu().numpy().view(np.uint32)

    # host bookkeeping: ema step and the density-grid generator's 2^32 jump
    after = grid_rng.copy()
    after.advance(1 << 32)
    assert desc.ema_step == 8
    assert (desc.grid_rng.state, desc.grid_rng.inc) == (after.state, after.inc)

    # samples: cells bit-exact, positions through the same random frames within the map tolerance
    opos, oidx = oracle.grid_samples(nu, nn, grid_rng.copy(), 7, ((0, 0, 0), (1, 1, 1)), grid0, N_CASCADES)
    assert (idx == oidx).all()
    can = oracle.build_triangles(avatar.canonical, None, avatar.faces, avatar.mask)
    adj = oracle.adjacency(avatar.faces, avatar.n_verts)
    deforms = []
    for f in frames:
        dt = oracle.build_triangles(f, avatar.canonical, avatar.faces, avatar.mask)
        deforms.append(oracle.Deformation(dt, can, adj, oracle.Bvh(dt)))
    wpos, wframe = oracle.warp_random_samples(deforms, warp_rng.copy(), opos)
    assert set(np.unique(wframe)) == {0, 1, 2}
    v = avatar.canonical.astype(np.float64)
    diag = float(np.linalg.norm(v.max(0) - v.min(0)))
    assert np.abs(pos - wpos).max() <= 1e-5 * diag

    # splat + decay
    # (a field with expression dims gets 1 in each, NerfNetwork::density's fill)
    coords = np.zeros((n, 11 + fc.n_extra), np.float32)
    coords[:, :3] = wpos
    coords[:, 8:11] = 0.5
    coords[:, 11:] = 1.0
    raw = oracle.field_eval(fc, params, coords)[:, 3]
    thick = (np.exp(raw.astype(np.float64)) * np.float64(MIN_CONE)).astype(np.float32)
    tmp = np.zeros_like(grid0)
    np.maximum.at(tmp, oidx, thick)
    ref = np.where(grid0 < 0, grid0, np.maximum(grid0 * np.float32(0.95), tmp))
    hit = np.zeros(grid0.size, bool)
    hit[oidx] = True
    assert (g[~hit] == ref[~hit]).all()
    # the field bound (4e-3 + 1e-2 |raw|, FP16 outputs) through exp, plus the fast exponential
    raw_max = np.zeros_like(grid0)
    np.maximum.at(raw_max, oidx, np.abs(raw))
    tol = np.expm1(5e-3 + 1.2e-2 * raw_max[hit]) + 1e-5
    rel = np.abs(g[hit] - ref[hit]) / np.maximum(np.abs(ref[hit]), 1e-12)
    assert (rel <= tol).all(), float((rel - tol).max())

    # bitfield of the device grid
    obits, thresh = oracle.density_grid_to_bitfield(g, N_CASCADES)
    near = np.abs(g[: 128 ** 3 * N_CASCADES] - thresh) <= 1e-5 * max(thresh, 1e-12)
    mip0_dev = np.unpackbits(bits[: 128 ** 3 * N_CASCADES // 8], bitorder="little")
    mip0_ref = np.unpackbits(obits[: 128 ** 3 * N_CASCADES // 8], bitorder="little")
    assert (mip0_dev[~near] == mip0_ref[~near]).all()
    if not near.any():
        assert (bits == obits).all()


def test_density_grid_update_rejects_missing_frames(ctx, grid_avatar):
    from insta_gb300 import abi
    ctx.density_grid_reset(AVATAR, N_CASCADES, None)
    desc = abi.DensityUpdateDesc()
    desc.decay, desc.n_uniform, desc.n_cascades, desc.n_frames, desc.bitfield_frame = 0.95, 1024, N_CASCADES, 5, -1
    desc.aabb_max[:] = [1.0, 1.0, 1.0]
    with pytest.raises(abi.InstaError) as e:
        ctx.density_grid_update(AVATAR, desc)
    assert e.value.code == 4
    desc.n_frames, desc.n_cascades = 3, 3
    with pytest.raises(abi.InstaError) as e:
        ctx.density_grid_update(AVATAR, desc)
    assert e.value.code == 1
