"""CPU checks: the oracle against itself and against properties of the reference algorithm,
the synthetic workload, the parameter layout, and the C-ABI library's exports."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_synthetic_mesh_shape(avatar):
    assert avatar.canonical.shape == (5122, 3)
    assert avatar.faces.shape == (10240, 3)
    # closed genus-0: every edge shared by exactly two faces
    f = avatar.faces
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    _, cnt = np.unique(e, axis=0, return_counts=True)
    assert (cnt == 2).all()
    assert set(np.unique(avatar.mask)) == {1, 2, 7, 15}


def test_adjacency_matches_edge_sharing(oracle, avatar):
    adj = oracle.adjacency(avatar.faces, avatar.n_verts)
    assert adj.shape == (10240, 3)
    assert (adj >= 0).all()   # closed mesh: three edge neighbours each
    f = avatar.faces
    for i in range(0, len(f), 997):
        for j in adj[i]:
            assert len(set(f[i]) & set(f[j])) == 2


def test_bvh_exact_equals_brute_force(oracle, avatar, frame0, oracle_frame):
    from insta_gb300 import synthetic as S
    pts = S.shell_points(frame0, avatar.faces, 3000, seed=2)
    bid, bd = oracle.nearest_brute(oracle_frame["def"], pts)
    eid, ed = oracle_frame["bvh"].nearest(pts, exact=True)
    assert (bid == eid).all() and (bd == ed).all()
    # the reference rule (last in BVH order wins ties) gives the same distance
    rid, rd = oracle_frame["bvh"].nearest(pts, exact=False)
    assert (rd == bd).all()


def test_ties_go_to_lowest_id(oracle):
    """Duplicate and degenerate triangles: equal distances resolve to the lowest id."""
    tri = np.array([[0.4, 0.4, 0.5], [0.6, 0.4, 0.5], [0.5, 0.6, 0.5]], np.float32)
    verts = np.concatenate([tri, tri, [[0.5, 0.5, 0.5], [0.5, 0.5, 0.5], [0.5, 0.5, 0.5]]]).astype(np.float32)
    faces = np.array([[3, 4, 5], [0, 1, 2], [6, 7, 8]], np.int32)   # face 0 and 1 coincide
    tris = oracle.build_triangles(verts, None, faces, None)
    pts = np.array([[0.5, 0.45, 0.52], [0.5, 0.45, 0.48]], np.float32)
    ids, _ = oracle.nearest_brute(tris, pts)
    assert (ids == 0).all()


def test_fp64_twin_close(oracle, avatar, frame0, oracle_frame):
    from insta_gb300 import synthetic as S
    pts = S.shell_points(frame0, avatar.faces, 4000, seed=6)
    d32 = oracle.Deformation(oracle_frame["def"], oracle_frame["can"], oracle_frame["adj"], oracle_frame["bvh"])
    d64 = oracle.Deformation(oracle_frame["def"], oracle_frame["can"], oracle_frame["adj"], oracle_frame["bvh"], fp64=True)
    _, a = d32.map_soa(pts)
    _, b = d64.map_soa(pts)
    assert np.abs(a - b).max() < 1e-6


def test_identity_frame_maps_to_itself(oracle, avatar):
    """A frame equal to the canonical mesh maps every point to itself (up to rounding)."""
    from insta_gb300 import synthetic as S
    can = oracle.build_triangles(avatar.canonical, None, avatar.faces, avatar.mask)
    dtr = oracle.build_triangles(avatar.canonical, avatar.canonical, avatar.faces, avatar.mask)
    adj = oracle.adjacency(avatar.faces, avatar.n_verts)
    d = oracle.Deformation(dtr, can, adj, oracle.Bvh(dtr), disable_interp=True)
    pts = S.shell_points(avatar.canonical, avatar.faces, 2000, seed=1)
    _, out = d.map_soa(pts)
    assert np.abs(out - pts).max() < 1e-6


def test_layout_python_matches_oracle(oracle):
    import ctypes as C
    from insta_gb300 import layout, synthetic as S
    for n_extra in (0, 16):
        fc = S.FieldConfig(n_extra=n_extra)
        lay = layout.field_layout(fc)
        cfg = oracle.field_cfg(fc)
        lo = (C.c_uint64 * 64)(); lr = (C.c_uint32 * 64)(); ls = (C.c_uint32 * 64)(); mo = (C.c_uint64 * 3)()
        total = oracle.lib().orc_field_layout(C.byref(cfg), lo, lr, ls, mo)
        assert total == lay.total
        assert list(lr[:16]) == lay.level_res and list(ls[:16]) == lay.level_size


def test_field_oracle_fp16_vs_fp64(oracle):
    from insta_gb300 import synthetic as S
    fc = S.FieldConfig()
    params = S.field_params(fc, seed=0)
    rng = np.random.default_rng(0)
    c = np.zeros((256, 11), np.float32)
    c[:, :3] = rng.uniform(0.35, 0.65, (256, 3))
    c[:, 8:11] = 0.5
    a = oracle.field_eval(fc, params, c)
    b = oracle.field_eval(fc, params, c, fp64=True)
    assert np.isfinite(a).all() and np.abs(a - b).max() < 5e-2


def test_sobol_dimension_zero_is_bit_reversal(oracle):
    lib = oracle.lib()
    for i in (0, 1, 2, 3, 12345, 0xdeadbeef):
        rev = int(f"{i:032b}"[::-1], 2)
        assert lib.orc_sobol(i, 0) == rev
    # dimension 1 direction numbers follow v_k = v_{k-1} ^ (v_{k-1} >> 1)
    assert [lib.orc_sobol(1 << b, 1) for b in range(4)] == [0x80000000, 0xc0000000, 0xa0000000, 0xf0000000]


def test_pixel_offset_spp0_is_centre(oracle):
    off = oracle.pixel_offset(0)
    assert np.abs(off - 0.5).max() < 1e-6


def header_functions():
    txt = (ROOT / "include" / "insta_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(insta_\w+)\s*\(", txt, re.M)))


def test_library_exports_every_declared_symbol():
    from insta_gb300 import abi, build as B
    lib_path = B.build()
    lib = ctypes.CDLL(str(lib_path))
    names = header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(abi.EXPORTS) == names


def test_param_count_without_gpu():
    """insta_field_param_count is pure host code and agrees with the Python layout: the benchmark
    field, INSTA's shipped layout (16 levels x 8 features, 16 expression dims, 2 + 3 hidden layers)
    and 4 features per level; layouts the kernels do not take are rejected."""
    from insta_gb300 import abi, layout, synthetic as S
    for fc in (S.FieldConfig(), S.insta_field_config(), S.FieldConfig(n_levels=12, n_features=4, n_extra=16)):
        assert abi.param_count(fc) == layout.field_layout(fc).total
    assert S.insta_field_config().n_levels * S.insta_field_config().n_features == 128
    for bad in (S.FieldConfig(n_features=1), S.FieldConfig(n_features=16, n_levels=16), S.FieldConfig(n_levels=6, n_features=2),
                S.FieldConfig(n_levels=18, n_features=8)):
        with pytest.raises(abi.InstaError):
            abi.param_count(bad)


def test_pcg32_published_sequence(oracle):
    """The pcg32 restatement (tiny-cuda-nn's default_rng_t) reproduces the PCG demo's first outputs
    for seed 42, sequence 54, and its jump-ahead equals stepping."""
    r = oracle.Pcg32.seeded(42, 54)
    assert [r.next_uint() for _ in range(6)] == [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293, 0xbfa4784b, 0xcbed606e]
    a = oracle.Pcg32.seeded(7)
    b = a.copy()
    for _ in range(1000):
        a.next_uint()
    b.advance(1000)
    assert (a.state, a.inc) == (b.state, b.inc)
    c, e = oracle.Pcg32.seeded(9), oracle.Pcg32.seeded(9)
    c.advance(1 << 32)
    e.advance(1 << 31)
    e.advance(1 << 31)
    assert c.state == e.state
    f = oracle.Pcg32.seeded(3).next_float()
    assert 0.0 <= f < 1.0


def test_grid_samples_land_in_their_cells(oracle):
    """generate_grid_samples_nerf_nonuniform: every sample lies in the cell its index names (at the
    cell's cascade scale), and non-uniform samples prefer cells above the threshold."""
    rng = np.random.default_rng(0)
    grid = np.where(rng.random(2 * 128 ** 3) < 0.3, 0.5, 0.0).astype(np.float32)
    pos, idx = oracle.grid_samples(5000, 5000, oracle.Pcg32.seeded(11), 3, ((0, 0, 0), (1, 1, 1)), grid, 2)
    level = idx // 128 ** 3
    cell = idx % 128 ** 3

    def compact(x):
        x = x & 0x49249249
        x = (x | (x >> 2)) & 0xc30c30c3
        x = (x | (x >> 4)) & 0x0f00f00f
        x = (x | (x >> 8)) & 0xff0000ff
        return (x | (x >> 16)) & 0x0000ffff

    c = np.stack([compact(cell.astype(np.int64) >> k) for k in range(3)], 1)
    local = ((pos - 0.5) / np.exp2(level)[:, None] + 0.5) * 128
    assert (np.floor(local + 1e-4) >= c - 1e-3).all() and (local <= c + 1 + 1e-4).all()
    occupied = grid[idx] > 0
    assert occupied[5000:].mean() > 0.9 and occupied[:5000].mean() < 0.45


def test_field_backward_oracle_matches_finite_differences(oracle):
    """The FP64 backward of the field (the oracle for insta_field_backward) against central
    differences of its own forward: the field is piecewise linear in every single parameter
    (trilinear hash weights, ReLU MLPs), so a difference over a step that flips no ReLU is exact
    up to the FP32 rounding of the outputs."""
    from insta_gb300 import synthetic as S
    fc = S.FieldConfig(n_extra=16)
    params = S.field_params(fc, seed=3)
    rng = np.random.default_rng(4)
    n = 6
    c = np.zeros((n, 11 + 16), np.float32)
    c[:, :3] = rng.uniform(0.35, 0.65, (n, 3))
    d = rng.normal(size=(n, 3))
    c[:, 8:11] = (d / np.linalg.norm(d, axis=1, keepdims=True) + 1) * 0.5
    c[:, 11:] = rng.uniform(-1, 1, (n, 16))
    g_out = rng.normal(size=(n, 4)).astype(np.float32)
    grad, out = oracle.field_backward(fc, params, c, g_out)
    np.testing.assert_allclose(out, oracle.field_eval(fc, params, c, fp64=True), rtol=1e-6, atol=1e-6)
    from insta_gb300 import layout as L
    table_off = L.field_layout(fc).table_offset
    w16 = np.ascontiguousarray(params).view(np.uint16).view(np.float16)
    nz_table = table_off + np.flatnonzero(grad[table_off:])
    picks = np.concatenate([rng.choice(table_off, 40, replace=False), rng.choice(nz_table, 40, replace=False)])

    def loss(p):
        return float((oracle.field_backward(fc, p.view(np.uint16), c)[1].astype(np.float64) * g_out).sum())

    checked = 0
    for i in picks:
        hi, lo = w16.copy(), w16.copy()
        hi[i] = np.float16(float(w16[i]) + 0.002)
        lo[i] = np.float16(float(w16[i]) - 0.002)
        step = float(hi[i]) - float(lo[i])
        fd = (loss(hi) - loss(lo)) / step
        assert abs(fd - grad[i]) <= 2e-3 + 2e-2 * abs(grad[i]), (int(i), fd, grad[i])
        checked += 1
    assert checked == 80 and np.abs(grad[nz_table]).max() > 0


def test_extra_dims_gradient_oracle_matches_finite_differences(oracle):
    """The oracle's gradient w.r.t. the expression dims (the input gradient train_nerf_step asks
    for when it optimises them) against central differences of the FP64 forward: the field is
    piecewise linear in each input dim, so a step that flips no ReLU gives the slope up to the
    FP32 rounding of the outputs."""
    from insta_gb300 import synthetic as S
    fc = S.FieldConfig(n_extra=16)
    params = S.field_params(fc, seed=3)
    rng = np.random.default_rng(9)
    n = 5
    c = np.zeros((n, 11 + 16), np.float32)
    c[:, :3] = rng.uniform(0.35, 0.65, (n, 3))
    d = rng.normal(size=(n, 3))
    c[:, 8:11] = (d / np.linalg.norm(d, axis=1, keepdims=True) + 1) * 0.5
    c[:, 11:] = rng.uniform(-1, 1, (n, 16))
    g_out = rng.normal(size=(n, 4)).astype(np.float32)
    _, _, dx = oracle.field_backward(fc, params, c, g_out, extra_grad=True)
    assert dx.shape == (n, 16) and np.abs(dx).max() > 0
    def f(s_, k, h):
        c2 = c[s_:s_ + 1].copy()
        c2[0, 11 + k] = np.float32(c2[0, 11 + k] + np.float32(h))
        return float((oracle.field_eval(fc, params, c2, fp64=True).astype(np.float64) * g_out[s_]).sum()), float(c2[0, 11 + k])

    for s_ in range(n):
        for k in range(0, 16, 3):
            (fp, xp), (f0, x0), (fm, xm) = f(s_, k, 5e-4), f(s_, k, 0.0), f(s_, k, -5e-4)
            # central, right and left slopes: a ReLU kink inside one side leaves the other exact
            slopes = [(fp - fm) / (xp - xm), (fp - f0) / (xp - x0), (f0 - fm) / (x0 - xm)]
            assert min(abs(v - dx[s_, k]) for v in slopes) <= 2e-3 + 2e-2 * abs(dx[s_, k]), (s_, k, slopes, dx[s_, k])


@pytest.mark.parametrize("loss_type,srgb", [(0, 1), (4, 0), (0, 0)])
def test_train_loss_oracle_gradients_match_finite_differences(oracle, loss_type, srgb):
    from conftest import loss_cfg, train_loss_batch
    """dL/d(raw output) of the loss kernel is the derivative of its own per-ray losses: with
    loss_scale 1 and the regularisers off, dloss = 3 d(sum of loss_output)/d(output) (the loss is
    the channel mean divided by n_rays, the gradient the channel sum divided by n_rays)."""
    b = train_loss_batch(16, seed=loss_type + 10 * srgb)
    cfg = loss_cfg(n_rays=16, loss_type=loss_type, srgb_targets=srgb)
    ns, cnt, _, dloss, loss = oracle.train_loss(cfg, **b)
    assert cnt == int(b["numsteps"][:, 0].sum())
    out = b["network_output"].astype(np.float64)
    rng = np.random.default_rng(1)
    picks = rng.choice(len(out), 30, replace=False)
    for s in picks:
        for ch in range(4):
            vals = []
            for h in (+1e-2, -1e-2):
                o2 = out.copy()
                o2[s, ch] += h
                vals.append(float(oracle.train_loss(cfg, **{**b, "network_output": o2})[4].astype(np.float64).sum()))
            fd = 3 * (vals[0] - vals[1]) / 2e-2
            # the kernel writes each ray's block at its compacted base; rays are compacted in kept order
            k = int(np.searchsorted(b["numsteps"][:, 1], s, side="right") - 1)
            j = s - int(b["numsteps"][k, 1])
            an = float(dloss[int(ns[k, 1]) + j, ch])
            assert abs(fd - an) <= 2e-4 + 2e-2 * abs(an), (s, ch, fd, an)


def test_train_loss_oracle_compaction_and_rollover(oracle):
    """Blocks past max_samples_compacted are cut (the ray that crosses it keeps its prefix), the
    compacted arrays are filled to target_batch_size by repetition, the repeated gradients scaled
    by count / target."""
    from conftest import loss_cfg, train_loss_batch
    b = train_loss_batch(40, seed=5)
    total = int(b["numsteps"][:, 0].sum())
    cap = total * 2 // 3
    ns, cnt, cout, dloss, _ = oracle.train_loss(loss_cfg(n_rays=40, max_samples_compacted=cap, target_batch_size=cap), **b)
    assert cnt == total and int(ns[:, 0].sum()) == cap
    ref_ns, _, ref_cout, ref_dloss, _ = oracle.train_loss(loss_cfg(n_rays=40), **b)
    for k in range(40):
        c, base = int(ns[k, 0]), int(ns[k, 1])
        assert base == int(ref_ns[k, 1])
        if c:
            np.testing.assert_array_equal(dloss[base:base + c], ref_dloss[base:base + c])
            np.testing.assert_array_equal(cout[base:base + c], ref_cout[base:base + c])
    ns2, _, cout2, dloss2, _ = oracle.train_loss(loss_cfg(n_rays=40, max_samples_compacted=2 * total, target_batch_size=2 * total - 5),
                                                 **b)
    n = 2 * total - 5
    src = np.arange(total, n) % total
    np.testing.assert_array_equal(cout2[total:n], cout2[src])
    np.testing.assert_allclose(dloss2[total:n], dloss2[src] * np.float32(total / n), rtol=1e-6)


def _np_loss_forward(cfg, b, k):
    """Per-ray loss of compute_loss_kernel_train_nerf (instant-ngp/src/testbed_nerf.cu:1305-1460),
    restated independently in NumPy float64 for kept ray k: composite with the transmittance stop,
    background added when the ray ran out, target from the image sample, loss mean / n_rays."""
    mn, mx = np.array(cfg["aabb_min"], np.float64), np.array(cfg["aabb_max"], np.float64)
    min_cone = np.sqrt(3.0) / 1024.0
    count, base = (int(x) for x in b["numsteps"][k])
    ray = int(b["ray_indices"][k])
    T, rgb = 1.0, np.zeros(3)
    n = 0
    for j in range(count):
        if T < 1e-4:
            break
        c = b["coords"][base + j].astype(np.float64)
        o = b["network_output"][base + j].astype(np.float64)
        dt = c[3] * (min_cone * 128 - min_cone) + min_cone
        alpha = 1.0 - np.exp(-np.exp(o[3]) * dt)
        rgb += alpha * T / (1.0 + np.exp(-o[:3]))
        T *= 1.0 - alpha
        n += 1
    s2l = lambda s: np.where(s <= 0.04045, s / 12.92, ((s + 0.055) / 1.055) ** 2.4)
    l2s = lambda l: np.where(l < 0.0031308, 12.92 * l, 1.055 * np.power(np.maximum(l, 0), 0.41666) - 0.055)
    bg = s2l(b["background"][ray].astype(np.float64))
    tex = b["target"][ray].astype(np.float64)
    if cfg["train_in_linear_colors"] or not cfg["srgb_targets"]:
        tgt = tex[:3] + (1 - tex[3]) * bg
        if not cfg["train_in_linear_colors"]:
            tgt, bg = l2s(tgt), l2s(bg)
    else:
        bg = l2s(bg)
        tgt = l2s(tex[:3] / tex[3]) * tex[3] + (1 - tex[3]) * bg if tex[3] > 0 else bg
    if n == count:
        rgb = rgb + T * bg
    d = rgb - tgt
    if cfg["loss_type"] == 4:   # Huber(0.1) / 5
        ad = np.abs(d)
        loss = np.where(ad > 0.1, ad - 0.05, 0.5 / 0.1 * d * d) / 5
    else:                       # L2
        loss = d * d
    return loss.mean() / cfg["n_rays"]


@pytest.mark.parametrize("loss_type,srgb,linear", [(0, 1, 0), (4, 1, 0), (0, 0, 0), (4, 1, 1)])
def test_train_loss_oracle_matches_numpy_restatement(oracle, loss_type, srgb, linear):
    from conftest import loss_cfg, train_loss_batch
    b = train_loss_batch(24, seed=30 + loss_type + srgb, max_steps=40)
    b["network_output"][::3, 3] += 4.0          # some rays reach the transmittance stop
    b["target"][1::4, 3] = 0.0                  # transparent samples: the target is the background
    cfg = loss_cfg(n_rays=24, loss_type=loss_type, srgb_targets=srgb, train_in_linear_colors=linear)
    _, _, _, _, loss = oracle.train_loss(cfg, **b)
    ref = np.array([_np_loss_forward(cfg, b, k) for k in range(24)])
    np.testing.assert_allclose(loss, ref, rtol=2e-4, atol=1e-9)


def _np_loss_gradients(cfg, b, k, extra, mean_density):
    """dL/d(raw output) of compute_loss_kernel_train_nerf's second pass (instant-ngp/src/
    testbed_nerf.cu:1465-1560) for kept ray k, restated in NumPy float64 with every term on:
    colour (L2), depth supervision (L1) with the segmentation rules, beta, density penalty,
    near-distance and mean-density regularisers."""
    mn, mx = np.array(cfg["aabb_min"], np.float64), np.array(cfg["aabb_max"], np.float64)
    min_cone = np.sqrt(3.0) / 1024.0
    count, base = (int(x) for x in b["numsteps"][k])
    ray = int(b["ray_indices"][k])
    R = b["rays"][ray].astype(np.float64)
    samples = []
    T, rgb_ray, depth_ray = 1.0, np.zeros(3), 0.0
    for j in range(count):
        if T < 1e-4:
            break
        c = b["coords"][base + j].astype(np.float64)
        o = b["network_output"][base + j].astype(np.float64)
        pos = mn + c[5:8] * (mx - mn)
        depth = np.linalg.norm(pos - R[:3])
        dt = c[3] * (min_cone * 128 - min_cone) + min_cone
        alpha = 1.0 - np.exp(-np.exp(o[3]) * dt)
        rgb = 1.0 / (1.0 + np.exp(-o[:3]))
        w = alpha * T
        rgb_ray += w * rgb
        depth_ray += w * depth
        T *= 1.0 - alpha
        samples.append((o, rgb, depth, dt, alpha))
    T_ray = T
    tex = b["target"][ray].astype(np.float64)
    bg = np.zeros(3)
    tgt = tex[:3] + (1 - tex[3]) * bg          # trained in linear colours, black background
    if len(samples) == count:
        rgb_ray = rgb_ray + T * bg
    seg, lam = 1.0, cfg["depth_supervision_lambda"]
    m = int(extra["seg_mask"][ray])
    if m in (120, 130, 140):
        seg = cfg["seg_mask_supervision_lambda"]
    if m <= 90 or m > 250 or tex[3] < 0.001:
        lam = 0.0
    target_depth = np.linalg.norm(R[3:]) * (extra["depth"][ray] if lam > 0 else -1.0)
    depth_grad = (np.sign(depth_ray - target_depth) if target_depth > 0 else 0.0) * lam
    lg = 2.0 * (rgb_ray - tgt) * seg
    scale = cfg["loss_scale"] / cfg["n_rays"]
    l1 = 1e-4 if mean_density < 0.01 else 0.0
    out, T, rgb2, depth2 = [], 1.0, np.zeros(3), 0.0
    for o, rgb, depth, dt, alpha in samples:
        w = alpha * T
        rgb2 += w * rgb
        depth2 += w * depth
        T *= 1.0 - alpha
        suffix = rgb_ray - rgb2
        d = np.zeros(4)
        d[:3] = scale * (w * lg) * rgb * (1 - rgb)
        dmlp = np.exp(np.clip(o[3], -15, 15)) * (dt * (lg @ (T * rgb - suffix) + depth_grad * (T * depth - (depth_ray - depth2)))
                                                 + cfg["beta"] * dt / (T_ray - 1 + 1e-3))
        if cfg["penalize_density"] and tex[3] <= 0.01:
            dmlp += w
        d[3] = scale * dmlp + (-l1 if o[3] < 0 else 0.0) + (1e-4 if (o[3] > -10 and depth < cfg["near_distance"]) else 0.0)
        out.append(d)
    return np.array(out).reshape(-1, 4)


def test_train_loss_oracle_gradients_match_numpy_all_terms(oracle):
    from conftest import loss_cfg, train_loss_batch
    n = 20
    b = train_loss_batch(n, seed=41, max_steps=30)
    b["background"] = np.zeros((n, 3), np.float32)
    b["target"][::5, 3] = 0.0
    rng = np.random.default_rng(42)
    extra = dict(depth=rng.uniform(0.2, 2.0, n).astype(np.float32),
                 seg_mask=np.array([0, 100, 120, 130, 140, 255, 91, 250] * 3, np.int32)[:n])
    cfg = loss_cfg(n_rays=n, loss_type=0, depth_loss_type=1, srgb_targets=0, train_in_linear_colors=1, loss_scale=128.0,
                   depth_supervision_lambda=1.25,
                   seg_mask_supervision_lambda=40.0, near_distance=0.6, beta=0.05, penalize_density=1)
    ns, _, _, dloss, _ = oracle.train_loss(cfg, **b, **extra, mean_density=0.005)
    for k in range(n):
        ref = _np_loss_gradients(cfg, b, k, extra, 0.005)
        c, base = int(ns[k, 0]), int(ns[k, 1])
        assert c == len(ref)
        got = dloss[base:base + c].astype(np.float64)
        np.testing.assert_allclose(got, ref, rtol=2e-3, atol=1e-6 * max(1.0, np.abs(ref).max()))
