"""Batched rendering (insta_render_batch) through the C ABI (cuda:0).

A batch renders every request's rays through one wavefront.  Per-ray work does not depend on
what else is in the batch, so each request's pixels must equal -- bit for bit -- those of
insta_render on that request alone, whatever the mix of frames, avatars, cameras and sizes.
One request of a mixed batch is also checked against the CPU oracle (PSNR >= 45 dB).
"""
import numpy as np
import pytest

from conftest import psnr

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def two_avatars(ctx):
    """Avatar 10 (seed 0, frames 0..2) and avatar 11 (seed 1, frames 0..1), same field layout."""
    from insta_gb300 import synthetic as S
    fc = S.FieldConfig()
    out = {}
    for aid, seed, n_frames in ((10, 0, 3), (11, 1, 2)):
        av = S.make_avatar(seed)
        ctx.canonical_set(aid, av.canonical, av.faces, av.mask)
        for f in range(n_frames):
            ctx.frame_upload(aid, f, av.frame(av.frame_coeffs(f)))
            ctx.occupancy_from_mesh(aid, f, 0.015)
        params = S.field_params(fc, seed=seed)
        ctx.params_load(aid, fc, params)
        out[aid] = (av, params)
    ctx.sync()
    return fc, out


def requests(ctx, specs):
    from insta_gb300 import synthetic as S
    reqs = []
    for aid, frame, w, h, yaw, spp in specs:
        cam, focal = S.camera(yaw, width=w, height=h)
        reqs.append(ctx.render_desc(aid, frame, w, h, focal, cam, spp=spp))
    return reqs


SPECS = [(10, 0, 64, 48, -10.0, 0), (10, 2, 40, 40, 15.0, 1), (11, 1, 72, 56, 0.0, 0), (10, 1, 33, 29, 25.0, 3),
         (11, 0, 48, 64, -25.0, 2)]


def single(ctx, req):
    rgba = np.zeros((req.width * req.height, 4), np.float32)
    depth = np.zeros(req.width * req.height, np.float32)
    ctx.render(req, rgba, depth)
    return rgba, depth


def test_batch_equals_single_renders(ctx, two_avatars):
    reqs = requests(ctx, SPECS)
    ref = [single(ctx, r) for r in reqs]
    rgba = [np.full((r.width * r.height, 4), -1, np.float32) for r in reqs]
    depth = [np.full(r.width * r.height, -1, np.float32) for r in reqs]
    ctx.render_batch(reqs, rgba, depth)
    for i, (a, b) in enumerate(zip(rgba, ref)):
        assert (a == b[0]).all(), f"request {i}: rgba differs"
        assert (depth[i] == b[1]).all(), f"request {i}: depth differs"
    # the mix is not trivial: every request hit the avatar
    assert all((b[0][:, 3] > 0.05).sum() > 20 for b in ref), [int((b[0][:, 3] > 0.05).sum()) for b in ref]


@pytest.mark.parametrize("slots", [0, 3, 7])
def test_one_avatar_batch_equals_single_renders(ctx, two_avatars, slots):
    """A batch whose requests all use one avatar's weights runs the MLP stage with the weights
    resident once per SM (the tile-slot kernel: by default for such batches, or forced with 3 or 7
    slots): each request's pixels still equal insta_render alone, bit for bit."""
    reqs = requests(ctx, [s for s in SPECS if s[0] == 10] + [(10, 0, 96, 80, 5.0, 0)])
    ref = [single(ctx, r) for r in reqs]
    rgba = [np.full((r.width * r.height, 4), -1, np.float32) for r in reqs]
    depth = [np.full(r.width * r.height, -1, np.float32) for r in reqs]
    before = ctx.tuning_get()
    ctx.tuning_set(mlp_slots=slots)
    try:
        ctx.render_batch(reqs, rgba, depth)
    finally:
        ctx.tuning_set(**before)
    for i, (a, b) in enumerate(zip(rgba, ref)):
        assert (a == b[0]).all(), f"request {i}: rgba differs"
        assert (depth[i] == b[1]).all(), f"request {i}: depth differs"


def test_batch_device_outputs_and_order(ctx, two_avatars):
    """Device outputs, and the same requests in reverse order, give the same pixels."""
    reqs = requests(ctx, SPECS)
    ref = [single(ctx, r) for r in reqs]
    rgba = [torch.zeros((r.width * r.height, 4), device="cuda") for r in reqs]
    depth = [torch.zeros(r.width * r.height, device="cuda") for r in reqs]
    rev = list(range(len(reqs)))[::-1]
    ctx.render_batch([reqs[i] for i in rev], [rgba[i] for i in rev], [depth[i] for i in rev])
    ctx.sync()
    for i in range(len(reqs)):
        assert (rgba[i].cpu().numpy() == ref[i][0]).all()
        assert (depth[i].cpu().numpy() == ref[i][1]).all()


def test_batch_request_matches_oracle(ctx, two_avatars, oracle):
    fc, avs = two_avatars
    av, params = avs[11]
    reqs = requests(ctx, SPECS)
    rgba = [np.zeros((r.width * r.height, 4), np.float32) for r in reqs]
    depth = [np.zeros(r.width * r.height, np.float32) for r in reqs]
    ctx.render_batch(reqs, rgba, depth)
    i = 2   # avatar 11, frame 1
    aid, frame, w, h, yaw, spp = SPECS[i]
    from insta_gb300 import synthetic as S
    fr = av.frame(av.frame_coeffs(frame))
    can = oracle.build_triangles(av.canonical, None, av.faces, av.mask)
    dtr = oracle.build_triangles(fr, av.canonical, av.faces, av.mask)
    adj = oracle.adjacency(av.faces, av.n_verts)
    bvh = oracle.Bvh(dtr)
    bits = oracle.occupancy(dtr, 0.015)
    d = oracle.Deformation(dtr, can, adj, bvh)
    cam, focal = S.camera(yaw, width=w, height=h)
    rc = oracle.render_cfg(w, h, focal, cam, av.render_aabb(), spp=spp)
    r_rgba, r_depth, ns, total = oracle.render(rc, d, bits, fc, params)
    assert total > 500
    assert psnr(rgba[i], r_rgba) >= 45.0


def test_batch_rejects_mixed_layouts(ctx, two_avatars):
    from insta_gb300 import abi, synthetic as S
    fc2 = S.FieldConfig(n_extra=16)
    av = S.make_avatar(2)
    ctx.canonical_set(12, av.canonical, av.faces, av.mask)
    ctx.frame_upload(12, 0, av.frame(av.frame_coeffs(0)))
    ctx.occupancy_from_mesh(12, 0, 0.015)
    ctx.params_load(12, fc2, S.field_params(fc2, seed=2))
    reqs = requests(ctx, [(10, 0, 16, 16, 0.0, 0), (12, 0, 16, 16, 0.0, 0)])
    rgba = [np.zeros((256, 4), np.float32) for _ in reqs]
    depth = [np.zeros(256, np.float32) for _ in reqs]
    with pytest.raises(abi.InstaError):
        ctx.render_batch(reqs, rgba, depth)


def test_frame_upload_batch_equals_single(ctx):
    """A batch upload builds the same BVHs and frames: identical occupancy and canonical maps."""
    from insta_gb300 import synthetic as S
    av = S.make_avatar(4)
    frames = [av.frame(av.frame_coeffs(k)) for k in range(5)]
    for aid in (20, 21):
        ctx.canonical_set(aid, av.canonical, av.faces, av.mask)
    for k, v in enumerate(frames):
        ctx.frame_upload(20, k, v)
    ctx.frame_upload_batch(21, list(range(5)), frames)
    pts = S.shell_points(frames[3], av.faces, 20000, seed=9)
    outs = {}
    for aid in (20, 21):
        got = []
        for k in range(5):
            ctx.occupancy_from_mesh(aid, k, 0.015)
            bits = ctx.occupancy_get(aid, k)
            idx = torch.empty(len(pts), dtype=torch.int32, device="cuda")
            can = torch.empty((len(pts), 3), device="cuda")
            ctx.canonical_map_soa(aid, k, torch.from_numpy(pts).cuda(), len(pts), idx, can)
            ctx.sync()
            got.append((bits, idx.cpu().numpy(), can.cpu().numpy()))
        outs[aid] = got
    for k in range(5):
        a, b = outs[20][k], outs[21][k]
        assert (a[0] == b[0]).all() and (a[1] == b[1]).all() and (a[2] == b[2]).all(), k
    assert outs[20][0][0].any()


def test_frame_upload_async_double_buffered(ctx):
    """Frames uploaded on the side stream while the previous frame renders give the same pixels as
    synchronous uploads."""
    from insta_gb300 import synthetic as S
    av = S.make_avatar(6)
    fc = S.FieldConfig()
    params = S.field_params(fc, seed=6)
    for aid in (30, 31):
        ctx.canonical_set(aid, av.canonical, av.faces, av.mask)
        ctx.params_load(aid, fc, params)
    frames = [av.frame(av.frame_coeffs(k)) for k in range(5)]
    W = H = 48
    reqs = []
    for k in range(5):
        cam, focal = S.camera(-20.0 + 10 * k, width=W, height=H)
        reqs.append((cam, focal))
    ref = []
    for k in range(5):
        ctx.frame_upload(30, 0, frames[k])
        ctx.occupancy_from_mesh(30, 0, 0.015)
        r = ctx.render_desc(30, 0, W, H, reqs[k][1], reqs[k][0])
        rgba = np.zeros((W * H, 4), np.float32)
        depth = np.zeros(W * H, np.float32)
        ctx.render(r, rgba, depth)
        ref.append((rgba, depth))
    got = []
    ctx.frame_upload_async(31, 0, frames[0], 0.015)
    outs = [(torch.zeros((W * H, 4), device="cuda"), torch.zeros(W * H, device="cuda")) for _ in range(5)]
    for k in range(5):
        if k + 1 < 5:
            ctx.frame_upload_async(31, (k + 1) % 2, frames[k + 1], 0.015)
        r = ctx.render_desc(31, k % 2, W, H, reqs[k][1], reqs[k][0])
        ctx.render(r, outs[k][0], outs[k][1])
    ctx.sync()
    for k in range(5):
        assert (outs[k][0].cpu().numpy() == ref[k][0]).all() and (outs[k][1].cpu().numpy() == ref[k][1]).all(), k
    assert (ref[0][0][:, 3] > 0.05).sum() > 20


def test_render_async_host_outputs_match_render(ctx, avatar):
    """insta_render_async: three frames in a row into page-locked host buffers (the two device
    staging pairs alternate) equal the synchronous renders once the context is synchronised."""
    from insta_gb300 import synthetic as S
    fc = S.FieldConfig()
    ctx.canonical_set(14, avatar.canonical, avatar.faces, avatar.mask)
    ctx.params_load(14, fc, S.field_params(fc, seed=6))
    for k in range(3):
        ctx.frame_upload(14, k, avatar.frame(avatar.frame_coeffs(30 + k)))
        ctx.occupancy_from_mesh(14, k, 0.015)
    reqs = []
    for k in range(3):
        cam, focal = S.camera(-10.0 + 10.0 * k, width=80, height=64)
        reqs.append(ctx.render_desc(14, k, 80, 64, focal, cam))
    sync_out = []
    for r in reqs:
        rgba, depth = np.zeros((80 * 64, 4), np.float32), np.zeros(80 * 64, np.float32)
        ctx.render(r, rgba, depth)
        sync_out.append((rgba, depth))
    pinned = [(torch.zeros((80 * 64, 4), dtype=torch.float32).pin_memory(), torch.zeros(80 * 64, dtype=torch.float32).pin_memory())
              for _ in range(3)]
    for r, (a, b) in zip(reqs, pinned):
        ctx.render_async(r, a.numpy(), b.numpy())
    ctx.sync()
    for (a, b), (ra, rb) in zip(pinned, sync_out):
        assert (a.numpy() == ra).all() and (b.numpy() == rb).all()
    assert sync_out[0][0][:, 3].max() > 0.05
