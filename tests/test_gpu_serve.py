"""The request loop (insta_server_*) through the C ABI (cuda:0).

Requests carry their own tracked-mesh frames and are admitted into a few slots while others are
on the GPU (continuous batching).  Each result must equal -- bit for bit -- insta_render of the
same request alone on the same context, whatever else was in flight.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def serve_ctx():
    from insta_gb300 import abi, synthetic as S
    ctx = abi.Context(0)
    fc = S.FieldConfig()
    avatars = {}
    for aid, seed in ((0, 5), (1, 6)):
        av = S.make_avatar(seed)
        ctx.canonical_set(aid, av.canonical, av.faces, av.mask)
        ctx.params_load(aid, fc, S.field_params(fc, seed=seed))
        avatars[aid] = av
    ctx.sync()
    yield ctx, avatars
    ctx.close()


def make_requests(ctx, avatars, n, seed):
    from insta_gb300 import synthetic as S
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        aid = int(rng.integers(0, 2))
        av = avatars[aid]
        w, h = [(32, 32), (48, 40), (64, 64), (40, 56)][int(rng.integers(0, 4))]
        yaw = float(rng.uniform(-30, 30))
        cam, focal = S.camera(yaw, width=w, height=h)
        verts = av.frame(av.frame_coeffs(100 + 7 * seed + k))
        out.append((ctx.render_desc(aid, -1, w, h, focal, cam), verts))
    return out


def single_render(ctx, req, verts):
    ctx.frame_upload(req.avatar, 7, verts)
    ctx.occupancy_from_mesh(req.avatar, 7, 0.015)
    req.frame = 7
    rgba = np.zeros((req.width * req.height, 4), np.float32)
    depth = np.zeros(req.width * req.height, np.float32)
    ctx.render(req, rgba, depth)
    return rgba, depth


def test_server_results_equal_single_renders(serve_ctx):
    from insta_gb300 import abi
    ctx, avatars = serve_ctx
    reqs = make_requests(ctx, avatars, 14, seed=1)
    outs = [(np.full((r.width * r.height, 4), -1, np.float32), np.full(r.width * r.height, -1, np.float32)) for r, _ in reqs]
    srv = abi.Server(ctx, max_inflight=4, max_inflight_pixels=3 * 64 * 64)
    tickets = [srv.submit(r, v, o[0], o[1]) for (r, v), o in zip(reqs, outs)]
    states = [srv.wait(t, 60000) for t in tickets]
    lat = [srv.poll(t)[1] for t in tickets]
    srv.close()
    assert states == [abi.REQ_DONE] * len(tickets), states
    assert all(x > 0 for x in lat)
    for (r, v), (rgba, depth) in zip(reqs, outs):
        ref_rgba, ref_depth = single_render(ctx, r, v)
        assert (rgba == ref_rgba).all() and (depth == ref_depth).all()
        assert (ref_rgba[:, 3] > 0.05).sum() > 10


def test_server_alone_equals_in_the_mix(serve_ctx):
    """The same request alone and among others gives the same pixels (device outputs)."""
    from insta_gb300 import abi
    ctx, avatars = serve_ctx
    reqs = make_requests(ctx, avatars, 9, seed=2)
    r0, v0 = reqs[0]
    srv = abi.Server(ctx, max_inflight=8, max_inflight_pixels=1 << 16)
    alone = (torch.zeros((r0.width * r0.height, 4), device="cuda"), torch.zeros(r0.width * r0.height, device="cuda"))
    t = srv.submit(r0, v0, *alone)
    assert srv.wait(t, 60000) == abi.REQ_DONE
    mix = [(torch.zeros((r.width * r.height, 4), device="cuda"), torch.zeros(r.width * r.height, device="cuda")) for r, _ in reqs]
    ts = [srv.submit(r, v, *o) for (r, v), o in zip(reqs, mix)]
    assert [srv.wait(x, 60000) for x in ts] == [abi.REQ_DONE] * len(ts)
    srv.close()
    torch.cuda.synchronize()
    assert torch.equal(alone[0], mix[0][0]) and torch.equal(alone[1], mix[0][1])


def test_server_short_rounds_equal_single_renders(serve_ctx):
    """A round budget of 2^16 samples (many short rounds, a few steps per ray each): the same
    pixels as insta_render alone; budgets outside 2^16..2^25 are refused."""
    from insta_gb300 import abi
    ctx, avatars = serve_ctx
    reqs = make_requests(ctx, avatars, 6, seed=3)
    outs = [(np.full((r.width * r.height, 4), -1, np.float32), np.full(r.width * r.height, -1, np.float32)) for r, _ in reqs]
    srv = abi.Server(ctx, max_inflight=4, max_inflight_pixels=2 * 64 * 64, round_samples=1 << 16)
    tickets = [srv.submit(r, v, o[0], o[1]) for (r, v), o in zip(reqs, outs)]
    states = [srv.wait(t, 60000) for t in tickets]
    srv.close()
    assert states == [abi.REQ_DONE] * len(tickets), states
    for (r, v), (rgba, depth) in zip(reqs, outs):
        ref_rgba, ref_depth = single_render(ctx, r, v)
        assert (rgba == ref_rgba).all() and (depth == ref_depth).all()
    for bad in (1000, (1 << 25) + 1):
        with pytest.raises(abi.InstaError) as e:
            abi.Server(ctx, max_inflight=2, max_inflight_pixels=1 << 16, round_samples=bad)
        assert e.value.code == abi.ERR_INVALID_ARG


def test_server_cancel_queued(serve_ctx):
    from insta_gb300 import abi, synthetic as S
    ctx, avatars = serve_ctx
    av = avatars[0]
    srv = abi.Server(ctx, max_inflight=1, max_inflight_pixels=256 * 256)
    cam, focal = S.camera(0.0, width=256, height=256)
    big = ctx.render_desc(0, -1, 256, 256, focal, cam)
    bufs = []
    tickets = []
    for k in range(6):
        o = (np.zeros((256 * 256, 4), np.float32), np.zeros(256 * 256, np.float32))
        bufs.append(o)
        tickets.append(srv.submit(big, av.frame(av.frame_coeffs(k)), o[0], o[1]))
    for t in tickets[3:]:
        srv.cancel(t)
    states = [srv.wait(t, 60000) for t in tickets]
    srv.close()
    assert states[0] == abi.REQ_DONE
    assert all(s in (abi.REQ_DONE, abi.REQ_CANCELLED) for s in states)
    assert states[-1] == abi.REQ_CANCELLED
