"""Fields wider than the benchmark's: INSTA's shipped layout (configs/nerf/main.json: 16 levels x 8
features, 16 expression dims, density MLP 2 hidden layers, colour MLP 3) and 4 features per level,
through the C ABI (cuda:0) against the oracle, which is written for any number of features per
level.  Tolerances as the benchmark field's tests: field outputs |err| <= 4e-3 + 1e-2 |x| (FP16),
rendered pixels PSNR >= 45 dB, FP32 backward within 1e-4 (outputs) / 1e-3 (per-block gradient
norms) of the FP64 oracle."""
import numpy as np
import pytest

from conftest import psnr

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

AV_INSTA, AV_F4 = 40, 41


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def coords(n, seed, n_extra=16):
    rng = np.random.default_rng(seed)
    c = np.zeros((n, 11 + n_extra), np.float32)
    c[:, :3] = rng.uniform(0.35, 0.65, size=(n, 3))
    d = rng.normal(size=(n, 3))
    c[:, 8:11] = (d / np.linalg.norm(d, axis=1, keepdims=True) + 1) * 0.5
    c[:, 11:] = rng.uniform(-1, 1, size=(n, n_extra))
    return c


def configs():
    from insta_gb300 import synthetic as S
    return {"insta": (AV_INSTA, S.insta_field_config()), "f4": (AV_F4, S.FieldConfig(n_levels=12, n_features=4, n_extra=16))}


@pytest.fixture(scope="module")
def wide(ctx, avatar, frame0):
    from insta_gb300 import synthetic as S
    out = {}
    for k, (aid, fc) in configs().items():
        params = S.field_params(fc, seed=7)
        ctx.canonical_set(aid, avatar.canonical, avatar.faces, avatar.mask)
        ctx.frame_upload(aid, 0, frame0)
        ctx.occupancy_from_mesh(aid, 0, 0.015)
        ctx.params_load(aid, fc, params)
        out[k] = (aid, fc, params)
    ctx.sync()
    return out


@pytest.mark.parametrize("kind", ["insta", "f4"])
def test_wide_field_eval_matches_oracle(ctx, wide, oracle, kind):
    aid, fc, params = wide[kind]
    c = coords(5000, seed=3)          # not a multiple of the 128-sample tile
    out = torch.zeros((len(c), 4), dtype=torch.float32, device="cuda")
    ctx.field_eval(aid, dev(c), c.shape[1], len(c), out)
    ctx.sync()
    got = out.cpu().numpy()
    ref = oracle.field_eval(fc, params, c)
    err = np.abs(got - ref)
    assert (err <= 4e-3 + 1e-2 * np.abs(ref)).all(), float(err.max())
    assert np.abs(got - oracle.field_eval(fc, params, c, fp64=True)).max() < 5e-2
    # the no-allocation entry runs the same kernels: same bits
    st = torch.zeros_like(out)
    ctx.field_eval_static(aid, dev(c[:4000]), c.shape[1], 4000, st)
    ctx.sync()
    assert np.array_equal(st.cpu().numpy()[:4000], got[:4000])


def test_wide_field_bf16(ctx, wide, oracle):
    from insta_gb300 import abi, synthetic as S
    fc = S.insta_field_config()
    params = S.field_params(fc, seed=8)
    ctx.params_load(AV_INSTA + 10, fc, params, precision=abi.PRECISION_BF16)
    c = coords(2048, seed=4)
    out = torch.zeros((len(c), 4), dtype=torch.float32, device="cuda")
    ctx.field_eval(AV_INSTA + 10, dev(c), c.shape[1], len(c), out)
    ctx.sync()
    ref = oracle.field_eval(fc, params, c, weight_format=1)
    err = np.abs(out.cpu().numpy() - ref)
    assert (err <= 3e-2 + 4e-2 * np.abs(ref)).all(), float(err.max())


def test_wide_field_render_psnr(ctx, wide, oracle, oracle_frame, avatar):
    from insta_gb300 import synthetic as S
    aid, fc, params = wide["insta"]
    W = H = 64
    extra = np.random.default_rng(5).uniform(-1, 1, 16).astype(np.float32)
    cam, focal = S.camera(-10.0, width=W, height=H)
    req = ctx.render_desc(aid, 0, W, H, focal, cam, extra_dims=extra)
    rgba = np.zeros((W * H, 4), np.float32)
    depth = np.zeros(W * H, np.float32)
    ctx.render(req, rgba, depth)
    n = ctx.render_samples()
    bits = oracle.occupancy(oracle_frame["def"], 0.015)
    d = oracle.Deformation(oracle_frame["def"], oracle_frame["can"], oracle_frame["adj"], oracle_frame["bvh"])
    rc = oracle.render_cfg(W, H, focal, cam, avatar.render_aabb())
    r_rgba, r_depth, ns, total = oracle.render(rc, d, bits, fc, params, extra_dims=extra)
    assert total > 500
    assert abs(n - total) <= max(2, total // 1000)
    assert psnr(rgba, r_rgba) >= 45.0


def test_wide_field_mlp_kernels_equal(ctx, wide):
    """INSTA's field through the tile-slot MLP kernel (slots sized for the 144-wide encoding) and
    the per-CTA kernel: the same bits."""
    from insta_gb300 import synthetic as S
    aid, fc, params = wide["insta"]
    W = H = 96
    extra = np.linspace(-1, 1, 16).astype(np.float32)
    cam, focal = S.camera(8.0, width=W, height=H)
    req = ctx.render_desc(aid, 0, W, H, focal, cam, extra_dims=extra)
    outs = []
    for slots in (1, 4):
        rgba = np.zeros((W * H, 4), np.float32)
        depth = np.zeros(W * H, np.float32)
        ctx.tuning_set(mlp_slots=slots)
        try:
            ctx.render(req, rgba, depth)
        finally:
            ctx.tuning_set()
        outs.append((rgba, depth))
    assert (outs[0][0][:, 3] > 0.01).sum() > 100
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("kind", ["insta", "f4"])
def test_wide_field_backward_matches_oracle(ctx, wide, oracle, kind):
    """FP32 layer products (cuBLAS) and the 4- / 8-feature table backward (16-byte reductions)
    against the FP64 oracle; the expression-dim input gradients too."""
    from insta_gb300 import layout as L
    aid, fc, params = wide[kind]
    lay = L.field_layout(fc)
    n = 3000
    c = coords(n, seed=6)
    g_out = np.random.default_rng(7).normal(size=(n, 4)).astype(np.float32)
    grad = torch.zeros(lay.total, dtype=torch.float32, device="cuda")
    out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    dx = torch.zeros((n, 16), dtype=torch.float32, device="cuda")
    ctx.field_backward(aid, dev(c), c.shape[1], n, dev(g_out), grad, out, dl_dextra=dx)
    ctx.sync()
    ref_g, ref_out, ref_dx = oracle.field_backward(fc, params, c, g_out, extra_grad=True)
    got_out = out.cpu().numpy()
    assert np.abs(got_out - ref_out).max() <= 1e-4 + 1e-4 * np.abs(ref_out).max()
    g = grad.cpu().numpy().astype(np.float64)
    blocks = [(off, off + n_out * n_in) for (off, n_out, n_in, _) in lay.mlp_layers(1.0)] + [(lay.table_offset, lay.total)]
    for lo, hi in blocks:
        a, b = g[lo:hi], ref_g[lo:hi]
        assert np.linalg.norm(b) > 0, (lo, hi)
        assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(b), (lo, hi, np.linalg.norm(a - b) / np.linalg.norm(b))
    touched_ref = ref_g[lay.table_offset:] != 0
    assert ((g[lay.table_offset:] != 0) <= touched_ref).all()
    gx = dx.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(gx - ref_dx) <= 1e-3 * np.linalg.norm(ref_dx)


def test_wide_field_limits(ctx, wide):
    """What the wide layout does not take: the tcgen05 training kernel (its tiles hold at most 64
    density inputs; TrainStep picks the TF32 products for such fields) and FP8 MLPs (at most 128
    density inputs)."""
    from insta_gb300 import abi, layout as L, synthetic as S, train as T
    aid, fc, params = wide["insta"]
    lay = L.field_layout(fc)
    c = coords(256, seed=9)
    g_out = np.ones((256, 4), np.float32)
    grad = torch.zeros(lay.total, dtype=torch.float32, device="cuda")
    ctx.train_set_math(False, tcgen05=True)
    try:
        with pytest.raises(abi.InstaError) as e:
            ctx.field_backward(aid, dev(c), c.shape[1], 256, dev(g_out), grad, None)
        assert e.value.code == 5
    finally:
        ctx.train_set_math(False)
    with pytest.raises(abi.InstaError) as e:
        ctx.params_load(AV_INSTA + 11, fc, params, precision=abi.PRECISION_FP8)
    assert e.value.code == 5
    step = T.TrainStep(ctx, aid, fc, T.TrainConfig(n_rays_per_batch=256, target_batch_size=1 << 12, max_samples=1 << 14))
    assert not step.tcgen05
    ctx.train_set_math(False)
