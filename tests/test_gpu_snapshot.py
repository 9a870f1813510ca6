"""A snapshot document applied through insta_gb300.snapshot renders exactly like the same
parameters and density grid loaded directly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("layout", ["benchmark", "insta"])
def test_snapshot_apply_renders_like_direct_load(ctx, avatar, frame0, layout):
    """The benchmark field and INSTA's shipped one (16 levels x 8 features, expression dims)."""
    from insta_gb300 import snapshot as SN, synthetic as S
    fc = S.FieldConfig() if layout == "benchmark" else S.insta_field_config()
    params = S.field_params(fc, seed=2)
    rng = np.random.default_rng(1)
    grid = np.where(rng.random(2 * 128 ** 3) < 0.2, 0.05, 0.0).astype(np.float16)
    s = SN.Snapshot(params=params, density_grid=grid,
                    aabb=(np.zeros(3, np.float32), np.ones(3, np.float32)), render_aabb=tuple(np.asarray(b, np.float32) for b in avatar.render_aabb()),
                    aabb_scale=fc.aabb_scale,
                    config={"encoding": {"n_levels": fc.n_levels, "n_features_per_level": fc.n_features, "log2_hashmap_size": fc.log2_table,
                                         "base_resolution": fc.base_res},
                            "network": {"n_neurons": fc.density_hidden, "n_hidden_layers": fc.density_layers, "n_output_dims": fc.density_out},
                            "rgb_network": {"n_neurons": fc.rgb_hidden, "n_hidden_layers": fc.rgb_layers}, "exp_params": fc.n_extra})
    doc = SN.write_snapshot(None, s)
    outs = []
    extra = np.linspace(-1, 1, fc.n_extra).astype(np.float32) if fc.n_extra else None
    for avatar_id, via_snapshot in ((5, True), (6, False)):
        ctx.canonical_set(avatar_id, avatar.canonical, avatar.faces, avatar.mask)
        ctx.frame_upload(avatar_id, 0, frame0)
        if via_snapshot:
            SN.apply_snapshot(ctx, avatar_id, SN.read_snapshot(doc), frame=0)
        else:
            ctx.params_load(avatar_id, fc, params)
            ctx.set_boxes(avatar_id, train=((0, 0, 0), (1, 1, 1)), render=avatar.render_aabb())
            ctx.density_grid_load(avatar_id, 0, grid, 2)
        cam, focal = S.camera(5.0, width=96, height=96)
        req = ctx.render_desc(avatar_id, 0, 96, 96, focal, cam, extra_dims=extra)
        rgba = torch.zeros((96 * 96, 4), device="cuda")
        depth = torch.zeros(96 * 96, device="cuda")
        ctx.render(req, rgba, depth)
        ctx.sync()
        outs.append((rgba.cpu().numpy(), depth.cpu().numpy(), ctx.occupancy_get(avatar_id, 0)))
    assert (outs[0][2] == outs[1][2]).all()
    assert (outs[0][0] == outs[1][0]).all() and (outs[0][1] == outs[1][1]).all()
    assert outs[0][0][:, 3].max() > 0.05
