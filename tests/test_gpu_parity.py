"""Parity of the CUDA path against the CPU oracle, through the C ABI (cuda:0).

Tolerances (from the task's parity bar):
* nearest-triangle indices: bit-exact, ties to the lowest triangle id;
* canonical coordinates: |err| <= 1e-5 x the mesh bounding-box diagonal;
* occupancy bits and march samples (t, dt): bit-exact;
* field outputs (FP16 network values): |err| <= 4e-3 + 1e-2 |x| (FP32 accumulation order);
* rendered pixels: PSNR >= 45 dB against the oracle render.
"""
import numpy as np
import pytest

from conftest import psnr

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def gpu_avatar(ctx, avatar, frame0):
    ctx.canonical_set(0, avatar.canonical, avatar.faces, avatar.mask)
    ctx.frame_upload(0, 0, frame0)
    ctx.frame_upload(0, 1, avatar.frame(avatar.frame_coeffs(1)))
    ctx.sync()
    return ctx


def diag(avatar):
    v = avatar.canonical.astype(np.float64)
    return float(np.linalg.norm(v.max(0) - v.min(0)))


@pytest.mark.parametrize("n_pts", [65536, 20000])
def test_nearest_bit_exact_and_canonical(gpu_avatar, oracle, oracle_frame, avatar, frame0, n_pts):
    """insta_canonical_map_soa: 65536 points take the sorted path (cell sort + warp walk), 20000
    the per-point walk."""
    from insta_gb300 import synthetic as S
    pts = S.shell_points(frame0, avatar.faces, n_pts, seed=3)
    n = len(pts)
    idx = torch.empty(n, dtype=torch.int32, device="cuda")
    out = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    gpu_avatar.canonical_map_soa(0, 0, dev(pts), n, idx, out)
    gpu_avatar.sync()
    idx, out = idx.cpu().numpy(), out.cpu().numpy()
    brute_ids, _ = oracle.nearest_brute(oracle_frame["def"], pts[:4096])
    assert (idx[:4096] == brute_ids).all()
    d = oracle.Deformation(oracle_frame["def"], oracle_frame["can"], oracle_frame["adj"], oracle_frame["bvh"])
    ref_ids, ref = d.map_soa(pts)
    assert (idx == ref_ids).all()
    assert np.abs(out - ref).max() <= 1e-5 * diag(avatar)
    d64 = oracle.Deformation(oracle_frame["def"], oracle_frame["can"], oracle_frame["adj"], oracle_frame["bvh"], fp64=True)
    _, ref64 = d64.map_soa(pts)
    assert np.abs(out - ref64).max() <= 1e-5 * diag(avatar)


def _morton_order(pts):
    lo, hi = pts.min(0), pts.max(0)
    q = np.clip(((pts - lo) / (hi - lo).max() * 1023).astype(np.int64), 0, 1023)
    key = np.zeros(len(pts), np.int64)
    for b in range(10):
        for k in range(3):
            key |= ((q[:, k] >> b) & 1) << (3 * b + k)
    return np.argsort(key, kind="stable")


def test_render_nearest_bit_exact(gpu_avatar, oracle, oracle_frame, avatar, frame0):
    """The render's warp-cooperative nearest-triangle walk on points up to 2 cm off the surface,
    as the render's samples are: a Morton-ordered block (coherent warps, as in the sorted sample
    stream), a block in random order (wide warps: a large union of nodes) and points off the
    vertices along their normal (vertex-nearest: several triangles at almost the same distance)."""
    from insta_gb300 import synthetic as S
    rng = np.random.default_rng(11)
    shell = S.shell_points(frame0, avatar.faces, 49152, seed=5, half_width=0.02)
    v = frame0.astype(np.float64)
    nrm = v - v.mean(0)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    off = (v + nrm * rng.uniform(0.0, 0.02, (len(v), 1))).astype(np.float32)
    pts = np.concatenate([shell[_morton_order(shell)][:32768], shell[32768:], off[_morton_order(off)]]).astype(np.float32)
    n = len(pts)
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    gpu_avatar.nearest_debug(0, 0, dev(pts), n, out)
    gpu_avatar.sync()
    ids = out.cpu().numpy()
    ref_ids, _ = oracle_frame["bvh"].nearest(pts)
    assert (ids == ref_ids).all(), int((ids != ref_ids).sum())
    pick = rng.choice(n, 4096, replace=False)
    brute_ids, _ = oracle.nearest_brute(oracle_frame["def"], pts[pick])
    assert (ids[pick] == brute_ids).all()


@pytest.mark.parametrize("yaw,color_normal", [(0.0, False), (35.0, True), (-60.0, False)])
def test_raycast_matches_oracle(gpu_avatar, oracle, oracle_frame, avatar, yaw, color_normal):
    """raycast_flame on the tracked frame: hit triangle ids and depths bit-exact (ties to the
    lowest id), shaded colours within 1e-5 (powf in srgb_to_linear), untouched pixels kept."""
    from insta_gb300 import synthetic as S
    W = H = 128
    cam, focal = S.camera(yaw, width=W, height=H)
    req = gpu_avatar.render_desc(0, 0, W, H, focal, cam)
    rgba = torch.full((W * H, 4), -1.0, dtype=torch.float32, device="cuda")
    depth = torch.full((W * H,), -1.0, dtype=torch.float32, device="cuda")
    tri = torch.empty(W * H, dtype=torch.int32, device="cuda")
    gpu_avatar.raycast(req, rgba, depth, tri, color_normal=color_normal)
    gpu_avatar.sync()
    rc = oracle.render_cfg(W, H, focal, cam, avatar.render_aabb())
    center = oracle.mesh_centroid(avatar.canonical)
    o_rgba, o_depth, o_tri = oracle.raycast(rc, oracle_frame["def"], center, color_normal,
                                            np.full((W * H, 4), -1.0, np.float32), np.full(W * H, -1.0, np.float32))
    got_tri = tri.cpu().numpy()
    assert (got_tri == o_tri).all(), int((got_tri != o_tri).sum())
    hit = o_tri >= 0
    assert hit.sum() > W * H // 10
    assert (depth.cpu().numpy() == o_depth).all()
    assert np.abs(rgba.cpu().numpy() - o_rgba).max() <= 1e-5
    assert (rgba.cpu().numpy()[~hit] == -1.0).all()


def test_raycast_host_buffers(gpu_avatar):
    from insta_gb300 import synthetic as S
    cam, focal = S.camera(10.0, width=64, height=48)
    req = gpu_avatar.render_desc(0, 0, 64, 48, focal, cam)
    rgba = np.full((64 * 48, 4), 7.0, np.float32)
    depth = np.full(64 * 48, 7.0, np.float32)
    d_rgba = torch.full((64 * 48, 4), 7.0, dtype=torch.float32, device="cuda")
    d_depth = torch.full((64 * 48,), 7.0, dtype=torch.float32, device="cuda")
    gpu_avatar.raycast(req, rgba, depth)
    gpu_avatar.raycast(req, d_rgba, d_depth)
    gpu_avatar.sync()
    assert (rgba == d_rgba.cpu().numpy()).all() and (depth == d_depth.cpu().numpy()).all()
    assert (rgba[:, 3] == 1.0).any() and (rgba[:, 3] == 7.0).any()


def make_coords(pts, dirs, holder, n_extra=0, extra_val=0.25):
    n = len(pts)
    c = np.zeros((n, 11 + n_extra), np.float32)
    c[:, 0:3] = pts
    c[:, 3] = 0.1
    c[:, 4] = holder
    c[:, 5:8] = pts
    c[:, 8:11] = (dirs + 1) * 0.5
    c[:, 11:] = extra_val
    return c


def test_canonical_map_coords_in_place(gpu_avatar, oracle, oracle_frame, avatar, frame0):
    """surface_closest_point / render_deformed semantics: holder-selected frame, skip rules, mask-7 expression dims."""
    from insta_gb300 import synthetic as S
    rng = np.random.default_rng(5)
    pts = S.shell_points(frame0, avatar.faces, 8192, seed=4)
    dirs = rng.normal(size=pts.shape).astype(np.float32)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    holder = np.zeros(len(pts), np.float32)
    holder[::7] = -1.0                     # not generated -> untouched
    pts[::11] += 5.0                       # outside the train box -> untouched
    c = make_coords(pts, dirs, holder, n_extra=16)
    cd = dev(c)
    gpu_avatar.canonical_map(0, 0, cd, c.shape[1], 16, len(c))
    gpu_avatar.sync()
    got = cd.cpu().numpy()
    d = oracle.Deformation(oracle_frame["def"], oracle_frame["can"], oracle_frame["adj"], oracle_frame["bvh"])
    ref = d.map_coords(c, n_extra=16, frame_id=0, n_frames=1)
    tol = 1e-5 * diag(avatar)
    assert np.abs(got[:, 0:3] - ref[:, 0:3]).max() <= tol
    assert np.abs(got[:, 8:11] - ref[:, 8:11]).max() <= 1e-5
    assert (got[:, 3:8] == c[:, 3:8]).all()
    assert (got[:, 11:] == ref[:, 11:]).all()
    untouched = (holder < 0) | (np.arange(len(c)) % 11 == 0)
    assert (got[untouched] == c[untouched]).all()
    # at least one lips sample keeps its expression dims, others get 1.0
    assert (got[~untouched, 11] == 1.0).any() and (got[~untouched, 11] == 0.25).any()


@pytest.mark.parametrize("variant", ["all_torso", "disable_interp", "boundary"])
def test_canonical_map_mask_variants(ctx, oracle, variant):
    """The warp's branches on other meshes: every triangle region 15 (rigid frames, expression
    dims reset everywhere), the disable-interp flag (rigid frames for face triangles too), and a
    mesh with a boundary region (mask 0)."""
    from insta_gb300 import abi, synthetic as S
    av = S.make_avatar(3, with_boundary=variant == "boundary")
    mask = np.full(av.n_faces, S.MASK_TORSO, np.uint32) if variant == "all_torso" else av.mask
    aid = {"all_torso": 10, "disable_interp": 11, "boundary": 12}[variant]
    fr = av.frame(av.frame_coeffs(2))
    ctx.canonical_set(aid, av.canonical, av.faces, mask)
    if variant == "disable_interp":
        ctx.set_flags(aid, abi.FLAG_DISABLE_INTERP)
    ctx.frame_upload(aid, 0, fr)
    rng = np.random.default_rng(9)
    pts = S.shell_points(fr, av.faces, 20000, seed=8)
    dirs = rng.normal(size=pts.shape).astype(np.float32)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    c = make_coords(pts, dirs, np.zeros(len(pts), np.float32), n_extra=16)
    cd = dev(c)
    ctx.canonical_map(aid, 0, cd, c.shape[1], 16, len(c))
    ctx.sync()
    got = cd.cpu().numpy()
    can = oracle.build_triangles(av.canonical, None, av.faces, mask)
    dtr = oracle.build_triangles(fr, av.canonical, av.faces, mask)
    d = oracle.Deformation(dtr, can, oracle.adjacency(av.faces, av.n_verts), oracle.Bvh(dtr), disable_interp=variant == "disable_interp")
    ref = d.map_coords(c, n_extra=16, frame_id=0, n_frames=1)
    assert np.abs(got[:, 0:3] - ref[:, 0:3]).max() <= 1e-5 * diag(av)
    assert np.abs(got[:, 8:11] - ref[:, 8:11]).max() <= 1e-5
    assert (got[:, 11:] == ref[:, 11:]).all()
    if variant == "all_torso":
        assert (got[:, 11:] == 1.0).all()


def test_canonical_map_holder_selects_frame(gpu_avatar, oracle, avatar, frame0):
    from insta_gb300 import synthetic as S
    f1 = avatar.frame(avatar.frame_coeffs(1))
    pts = S.shell_points(f1, avatar.faces, 2048, seed=8)
    dirs = np.tile(np.array([[0, 0, 1]], np.float32), (len(pts), 1))
    c = make_coords(pts, dirs, np.ones(len(pts), np.float32))
    cd = dev(c)
    gpu_avatar.canonical_map(0, -1, cd, 11, 0, len(c))
    gpu_avatar.sync()
    can = oracle.build_triangles(avatar.canonical, None, avatar.faces, avatar.mask)
    d1 = oracle.build_triangles(f1, avatar.canonical, avatar.faces, avatar.mask)
    adj = oracle.adjacency(avatar.faces, avatar.n_verts)
    ref = oracle.Deformation(d1, can, adj, oracle.Bvh(d1)).map_coords(c, frame_id=-1, n_frames=2)
    assert np.abs(cd.cpu().numpy()[:, :3] - ref[:, :3]).max() <= 1e-5 * diag(avatar)


@pytest.mark.parametrize("fixed", [True, False])
def test_canonical_map_sorted_paths(gpu_avatar, oracle, oracle_frame, avatar, frame0, fixed):
    """insta_canonical_map on 70,000 records takes the (frame, cell)-sorted walk: render_deformed
    (fixed frame 0) and surface_closest_point (holder frames 0 and 1), with skipped records
    (holder -1, outside the train box) left untouched."""
    from insta_gb300 import synthetic as S
    rng = np.random.default_rng(12)
    f1 = avatar.frame(avatar.frame_coeffs(1))
    n = 70000
    holder = rng.integers(0, 2, n).astype(np.float32)
    holder[rng.random(n) < 0.05] = -1.0
    pts = np.where((holder == 1)[:, None], S.shell_points(f1, avatar.faces, n, seed=13), S.shell_points(frame0, avatar.faces, n, seed=14))
    pts[rng.random(n) < 0.03] += 3.0
    dirs = rng.normal(size=(n, 3)).astype(np.float32)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    c = make_coords(pts.astype(np.float32), dirs, holder, n_extra=4)
    cd = dev(c)
    gpu_avatar.canonical_map(0, 0 if fixed else -1, cd, c.shape[1], 4, n)
    gpu_avatar.sync()
    got = cd.cpu().numpy()
    can, adj = oracle_frame["can"], oracle_frame["adj"]
    d0 = oracle.Deformation(oracle_frame["def"], can, adj, oracle_frame["bvh"])
    if fixed:
        ref = d0.map_coords(c, n_extra=4, frame_id=0, n_frames=1)
    else:
        dt1 = oracle.build_triangles(f1, avatar.canonical, avatar.faces, avatar.mask)
        d1 = oracle.Deformation(dt1, can, adj, oracle.Bvh(dt1))
        ref = c.copy()
        for h, d in ((0, d0), (1, d1)):
            sel = holder == h
            ref[sel] = d.map_coords(c[sel], n_extra=4, frame_id=-1, n_frames=2)
    assert np.abs(got[:, 0:3] - ref[:, 0:3]).max() <= 1e-5 * diag(avatar)
    assert np.abs(got[:, 8:11] - ref[:, 8:11]).max() <= 1e-5
    assert (got[:, 11:] == ref[:, 11:]).all() and (got[:, 3:8] == c[:, 3:8]).all()
    skipped = (holder < 0) | (np.abs(pts - 0.5).max(1) > 0.5)
    assert skipped.any() and (got[skipped] == c[skipped]).all()


def test_canonical_map_empty_is_noop(gpu_avatar):
    c = torch.zeros((0, 11), dtype=torch.float32, device="cuda")
    gpu_avatar.canonical_map(0, 0, c, 11, 0, 0)
    gpu_avatar.sync()


def test_training_samples(gpu_avatar, oracle, oracle_frame, avatar):
    """generate_training_samples_nerf + warp with per-record frames: per kept ray, the same number
    of samples, bit-exact march outputs (dt, holder, deformed position), canonical positions within
    1e-5 x the bbox diagonal of the oracle's map of the record's frame."""
    gpu_avatar.occupancy_from_mesh(0, 0, 0.015)
    bits = oracle.occupancy(oracle_frame["def"], 0.015)
    rng = np.random.default_rng(21)
    n = 3000
    c0 = np.array([0.5, 0.5, 0.5], np.float32)
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    org = c0 + u * 0.9
    tgt = c0 + rng.normal(0, 0.06, (n, 3))
    du = (tgt - org) * rng.uniform(0.5, 2.0, (n, 1))
    rays = np.concatenate([org, du], 1).astype(np.float32)
    image = rng.integers(0, 2, n).astype(np.uint32)
    rnd = rng.random(n).astype(np.float32)
    max_samples = 1 << 19
    coords = torch.zeros((max_samples, 11), device="cuda")
    ri = torch.zeros(n, dtype=torch.int32, device="cuda")
    ns = torch.zeros((n, 2), dtype=torch.int32, device="cuda")
    cnt = torch.zeros(2, dtype=torch.int32, device="cuda")
    gpu_avatar.training_samples(0, 0, dev(rays), dev(image.view(np.int32)), dev(rnd), max_samples, coords, 11, ri, ns, cnt)
    gpu_avatar.sync()
    c_ref, ri_ref, ns_ref, cnt_ref = oracle.training_samples(bits, rays, image, rnd, max_samples)
    cnt = cnt.cpu().numpy().view(np.uint32)
    assert (cnt == cnt_ref).all() and cnt[0] > 1000 and cnt[1] < max_samples
    # the oracle's records mapped with the frame each one names
    frames = {0: oracle_frame}
    f1 = avatar.frame(avatar.frame_coeffs(1))
    d1 = oracle.build_triangles(f1, avatar.canonical, avatar.faces, avatar.mask)
    frames[1] = {"def": d1, "can": oracle_frame["can"], "adj": oracle_frame["adj"], "bvh": oracle.Bvh(d1)}
    n_ref = int(cnt_ref[1])
    mapped = c_ref[:n_ref].copy()
    for h, fr in frames.items():
        rows = mapped[:, 4] == h
        d = oracle.Deformation(fr["def"], fr["can"], fr["adj"], fr["bvh"])
        mapped[rows] = d.map_coords(mapped[rows], frame_id=-1, n_frames=2)
    got = coords.cpu().numpy()
    ri, ns = ri.cpu().numpy(), ns.cpu().numpy()
    where = {int(i): k for k, i in enumerate(ri_ref[:cnt_ref[0]])}
    tol = 1e-5 * diag(avatar)
    err = 0.0
    for k in range(int(cnt[0])):
        i, m, b = int(ri[k]), int(ns[k, 0]), int(ns[k, 1])
        kr = where[i]
        assert m == int(ns_ref[kr, 0])
        br = int(ns_ref[kr, 1])
        g, r = got[b:b + m], mapped[br:br + m]
        assert (g[:, 3:8] == c_ref[br:br + m, 3:8]).all()
        err = max(err, float(np.abs(g[:, 0:3] - r[:, 0:3]).max()), float(np.abs(g[:, 8:11] - r[:, 8:11]).max()))
    assert err <= tol


def test_occupancy_bit_exact(gpu_avatar, oracle, oracle_frame):
    gpu_avatar.occupancy_from_mesh(0, 0, 0.015)
    got = gpu_avatar.occupancy_get(0, 0)
    ref = oracle.occupancy(oracle_frame["def"], 0.015)
    assert got.sum() > 0
    assert (got == ref).all()


def test_occupancy_bit_exact_with_boundary_region(ctx, oracle):
    """mark_flame_density_grid skips cells whose nearest triangle lies in region 0 (boundary)."""
    from insta_gb300 import synthetic as S
    av = S.make_avatar(4, with_boundary=True)
    assert (av.mask == S.MASK_BOUNDARY).any()
    fr = av.frame(av.frame_coeffs(3))
    ctx.canonical_set(13, av.canonical, av.faces, av.mask)
    ctx.frame_upload(13, 0, fr)
    ctx.occupancy_from_mesh(13, 0, 0.015)
    got = ctx.occupancy_get(13, 0)
    ref = oracle.occupancy(oracle.build_triangles(fr, av.canonical, av.faces, av.mask), 0.015)
    assert got.sum() > 0
    assert (got == ref).all()


@pytest.mark.parametrize("scale,fp16", [(0.05, False), (0.05, True), (0.004, False)])
def test_density_grid_bitfield(gpu_avatar, oracle, scale, fp16):
    """Snapshot density grid -> bitfield (grid_to_bitfield + max-pool), two cascades.  With the
    mean above 0.01 the threshold is exactly 0.01 and the bits are exact; below it the threshold
    is the mean, whose last bits depend on the summation order: cells within 1e-5 of it are
    excluded."""
    rng = np.random.default_rng(11)
    grid = rng.exponential(scale, size=2 * 128 ** 3).astype(np.float32)
    grid[rng.random(grid.size) < 0.3] *= -1.0   # negative densities count as 0 in the mean
    if fp16:
        grid = grid.astype(np.float16)
    gpu_avatar.density_grid_load(0, 1, grid, 2)
    got = gpu_avatar.occupancy_get(0, 1)
    ref, thresh = oracle.density_grid_to_bitfield(grid.astype(np.float32), 2)
    if scale > 0.02:
        assert thresh == np.float32(0.01)
        assert (got == ref).all()
    else:
        assert thresh < 0.01
        g32 = grid.astype(np.float32)
        near = np.abs(g32[:128 ** 3] - thresh) <= 1e-5 * thresh
        mip0_got = np.unpackbits(got[:128 ** 3 // 8], bitorder="little").astype(bool)
        mip0_ref = np.unpackbits(ref[:128 ** 3 // 8], bitorder="little").astype(bool)
        assert (mip0_got[~near] == mip0_ref[~near]).all()
        assert mip0_ref.sum() > 1000
    gpu_avatar.occupancy_from_mesh(0, 1, 0.015)


def test_march_samples_bit_exact(gpu_avatar, oracle, oracle_frame, avatar):
    from insta_gb300 import synthetic as S
    gpu_avatar.occupancy_from_mesh(0, 0, 0.015)
    W = H = 48
    cam, focal = S.camera(10.0, width=W, height=H)
    req = gpu_avatar.render_desc(0, 0, W, H, focal, cam)
    M = 256
    t = torch.zeros((W * H, M), dtype=torch.float32, device="cuda")
    dt = torch.zeros_like(t)
    n = torch.zeros(W * H, dtype=torch.int32, device="cuda")
    gpu_avatar.march_debug(req, M, t, dt, n)
    gpu_avatar.sync()
    t, dt, n = t.cpu().numpy(), dt.cpu().numpy(), n.cpu().numpy()
    bits = oracle.occupancy(oracle_frame["def"], 0.015)
    rc = oracle.render_cfg(W, H, focal, cam, avatar.render_aabb())
    total = 0
    for i in range(W * H):
        rt, rdt, _ = oracle.march_ray(rc, bits, i % W, i // W, M)
        assert n[i] == len(rt), i
        assert (t[i, :n[i]] == rt).all() and (dt[i, :n[i]] == rdt).all(), i
        total += n[i]
    assert total > 0


@pytest.fixture(scope="module")
def field_setup(gpu_avatar):
    from insta_gb300 import synthetic as S
    fc = S.FieldConfig()
    params = S.field_params(fc, seed=0)
    gpu_avatar.params_load(0, fc, params)
    return fc, params


def random_coords(n, seed=0, n_extra=0):
    rng = np.random.default_rng(seed)
    pts = rng.uniform(0.35, 0.65, size=(n, 3)).astype(np.float32)
    dirs = rng.normal(size=(n, 3)).astype(np.float32)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    c = make_coords(pts, dirs, np.zeros(n, np.float32), n_extra=n_extra)
    if n_extra:
        c[:, 11:] = rng.uniform(-1, 1, size=(n, n_extra))
    return c


def test_field_eval_matches_oracle(gpu_avatar, field_setup, oracle):
    fc, params = field_setup
    c = random_coords(5000, seed=1)       # not a multiple of the 128-sample tile
    out = torch.zeros((len(c), 4), dtype=torch.float32, device="cuda")
    gpu_avatar.field_eval(0, dev(c), 11, len(c), out)
    gpu_avatar.sync()
    got = out.cpu().numpy()
    ref = oracle.field_eval(fc, params, c)
    err = np.abs(got - ref)
    assert (err <= 4e-3 + 1e-2 * np.abs(ref)).all(), float(err.max())
    ref64 = oracle.field_eval(fc, params, c, fp64=True)
    assert np.abs(got - ref64).max() < 5e-2


def test_field_eval_bf16(gpu_avatar, oracle):
    from insta_gb300 import abi, synthetic as S
    fc = S.FieldConfig()
    params = S.field_params(fc, seed=2)
    gpu_avatar.params_load(3, fc, params, precision=abi.PRECISION_BF16)
    c = random_coords(1024, seed=9)
    out = torch.zeros((len(c), 4), dtype=torch.float32, device="cuda")
    gpu_avatar.field_eval(3, dev(c), 11, len(c), out)
    gpu_avatar.sync()
    ref = oracle.field_eval(fc, params, c, weight_format=1)
    err = np.abs(out.cpu().numpy() - ref)
    assert (err <= 3e-2 + 4e-2 * np.abs(ref)).all(), float(err.max())


def test_field_eval_fp8(gpu_avatar, oracle):
    """FP8 E4M3 MLPs (per-layer weight scale, per-row activation scale, FP32 accumulation) against
    the oracle's FP8 restatement.  Tensor-core accumulation order can move a re-quantised
    activation by one E4M3 step, so the bound is statistical; the error against FP64 is reported
    by the precision workload of bench.py."""
    from insta_gb300 import abi, synthetic as S
    fc = S.FieldConfig()
    params = S.field_params(fc, seed=2)
    gpu_avatar.params_load(5, fc, params, precision=abi.PRECISION_FP8)
    c = random_coords(4096, seed=12)
    out = torch.zeros((len(c), 4), dtype=torch.float32, device="cuda")
    gpu_avatar.field_eval(5, dev(c), 11, len(c), out)
    gpu_avatar.sync()
    got = out.cpu().numpy()
    ref = oracle.field_eval(fc, params, c, weight_format=2)
    err = np.abs(got - ref)
    assert np.isfinite(got).all()
    assert float(err.mean()) < 5e-3, float(err.mean())
    assert (err <= 5e-2 + 5e-2 * np.abs(ref)).mean() > 0.999, float(err.max())
    ref16 = oracle.field_eval(fc, params, c)
    assert np.abs(got - ref16).mean() < 5e-2


def render_pair(ctx, oracle, oracle_frame, avatar, fc, params, W, H, yaw=0.0, avatar_id=0):
    from insta_gb300 import synthetic as S
    cam, focal = S.camera(yaw, width=W, height=H)
    req = ctx.render_desc(avatar_id, 0, W, H, focal, cam)
    rgba = np.zeros((W * H, 4), np.float32)
    depth = np.zeros(W * H, np.float32)
    ctx.render(req, rgba, depth)
    n = ctx.render_samples()
    bits = oracle.occupancy(oracle_frame["def"], 0.015)
    d = oracle.Deformation(oracle_frame["def"], oracle_frame["can"], oracle_frame["adj"], oracle_frame["bvh"])
    rc = oracle.render_cfg(W, H, focal, cam, avatar.render_aabb())
    r_rgba, r_depth, ns, total = oracle.render(rc, d, bits, fc, params)
    return rgba, depth, n, r_rgba, r_depth, total


def test_render_psnr(gpu_avatar, field_setup, oracle, oracle_frame, avatar):
    fc, params = field_setup
    gpu_avatar.occupancy_from_mesh(0, 0, 0.015)
    rgba, depth, n, r_rgba, r_depth, total = render_pair(gpu_avatar, oracle, oracle_frame, avatar, fc, params, 96, 96, yaw=-12.0)
    assert total > 1000
    assert abs(n - total) <= max(2, total // 1000)
    assert psnr(rgba, r_rgba) >= 45.0
    hit = (r_rgba[:, 3] > 0.2) & (rgba[:, 3] > 0.2)
    if hit.any():
        assert np.abs(depth[hit] - r_depth[hit]).max() < 1e-3
    assert ((r_rgba[:, 3] > 0.2) == (rgba[:, 3] > 0.2)).mean() > 0.999


@pytest.mark.parametrize("variant", ["uniform_steps", "jitter", "max_samples", "odd_size", "linear_colors"])
def test_render_variants(gpu_avatar, field_setup, oracle, oracle_frame, avatar, variant):
    """Render options against the oracle: cone angle 0 (uniform steps, aabb_scale 1), sub-pixel
    jitter (spp 3, no snapping), a per-ray sample cap of 8, a ragged 37x23 frame, linear colours."""
    from insta_gb300 import synthetic as S
    fc, params = field_setup
    gpu_avatar.occupancy_from_mesh(0, 0, 0.015)
    W, H = (37, 23) if variant == "odd_size" else (64, 48)
    opts = {"uniform_steps": dict(cone_angle=0.0), "jitter": dict(spp=3, snap=False), "max_samples": dict(max_samples=8),
            "odd_size": {}, "linear_colors": dict(linear_colors=True)}[variant]
    cam, focal = S.camera(7.0, width=W, height=H)
    req = gpu_avatar.render_desc(0, 0, W, H, focal, cam, **opts)
    rgba = np.zeros((W * H, 4), np.float32)
    depth = np.zeros(W * H, np.float32)
    gpu_avatar.render(req, rgba, depth)
    n = gpu_avatar.render_samples()
    bits = oracle.occupancy(oracle_frame["def"], 0.015)
    d = oracle.Deformation(oracle_frame["def"], oracle_frame["can"], oracle_frame["adj"], oracle_frame["bvh"])
    ro = dict(opts)
    if "max_samples" in ro:
        ro["max_samples"] = ro.pop("max_samples")
    rc = oracle.render_cfg(W, H, focal, cam, avatar.render_aabb(), **ro)
    r_rgba, r_depth, ns, total = oracle.render(rc, d, bits, fc, params)
    assert total > 100
    assert abs(n - total) <= max(2, total // 1000)
    assert psnr(rgba, r_rgba) >= 45.0
    if variant == "max_samples":
        assert ns.max() <= 8


def test_render_opaque_early_termination(gpu_avatar, oracle, oracle_frame, avatar):
    """A dense field terminates rays early (composite_kernel_nerf :996-999)."""
    from insta_gb300 import synthetic as S
    fc = S.FieldConfig()
    params = S.field_params(fc, seed=4, density_gain=60.0)
    gpu_avatar.params_load(0, fc, params)
    gpu_avatar.occupancy_from_mesh(0, 0, 0.015)
    rgba, depth, n, r_rgba, r_depth, total = render_pair(gpu_avatar, oracle, oracle_frame, avatar, fc, params, 64, 64)
    assert (r_rgba[:, 3] > 0.99).sum() > 100
    assert psnr(rgba, r_rgba) >= 45.0
    gpu_avatar.params_load(0, fc, S.field_params(fc, seed=0))


def test_render_fp8(gpu_avatar, oracle, oracle_frame, avatar):
    """The render with FP8 MLPs against the oracle's FP8 render."""
    from insta_gb300 import abi, synthetic as S
    fc = S.FieldConfig()
    params = S.field_params(fc, seed=0)
    gpu_avatar.params_load(0, fc, params, precision=abi.PRECISION_FP8)
    gpu_avatar.occupancy_from_mesh(0, 0, 0.015)
    try:
        W = H = 64
        cam, focal = S.camera(5.0, width=W, height=H)
        req = gpu_avatar.render_desc(0, 0, W, H, focal, cam)
        rgba = np.zeros((W * H, 4), np.float32)
        depth = np.zeros(W * H, np.float32)
        gpu_avatar.render(req, rgba, depth)
        bits = oracle.occupancy(oracle_frame["def"], 0.015)
        d = oracle.Deformation(oracle_frame["def"], oracle_frame["can"], oracle_frame["adj"], oracle_frame["bvh"])
        rc = oracle.render_cfg(W, H, focal, cam, avatar.render_aabb())
        r_rgba, _, _, total = oracle.render(rc, d, bits, fc, params, weight_format=2)
        assert total > 1000
        assert psnr(rgba, r_rgba) >= 35.0
    finally:
        gpu_avatar.params_load(0, fc, params)


def test_render_device_outputs(gpu_avatar, field_setup, oracle, avatar):
    from insta_gb300 import synthetic as S
    gpu_avatar.occupancy_from_mesh(0, 0, 0.015)
    cam, focal = S.camera(0.0, width=32, height=32)
    req = gpu_avatar.render_desc(0, 0, 32, 32, focal, cam)
    rgba_h = np.zeros((32 * 32, 4), np.float32)
    depth_h = np.zeros(32 * 32, np.float32)
    gpu_avatar.render(req, rgba_h, depth_h)
    rgba_d = torch.zeros((32 * 32, 4), device="cuda")
    depth_d = torch.zeros(32 * 32, device="cuda")
    gpu_avatar.render(req, rgba_d, depth_d)
    gpu_avatar.sync()
    assert (rgba_d.cpu().numpy() == rgba_h).all() and (depth_d.cpu().numpy() == depth_h).all()
