"""Parity at the benchmark's own sizes, through the C ABI (cuda:0).

The small-case tests in test_gpu_parity.py exercise every branch; these run the same checks on the
full workloads, where the sorted paths, the round budget, several rounds per frame and the
multi-round alive lists are exercised the way the benchmark exercises them:

* canonical map of 1,048,576 points in a 1 cm shell (the point workload): nearest-triangle ids
  bit-exact against the oracle (ties to the lowest id) and against brute force on a subset,
  canonical coordinates within 1e-5 x the mesh bounding-box diagonal of the FP32 and FP64
  oracles;
* the whole 512x512 frame (the single-frame render workload): PSNR >= 45 dB against the oracle
  render, per-pixel composited sample counts equal to the oracle's march (rays whose early
  termination flips on rounding aside, < 0.1 %), depths within 1e-3 where both are opaque;
* the same frame with at most 3 samples per ray per round (so the rays span up to tens of rounds
  and the alive lists are compacted every round), other launch shapes, staged tree tops, and the
  split deform + encode / MLP kernels: bit-identical to the default schedule and to the
  host-driven rounds -- a sample's arithmetic never depends on how rays are grouped;
* the whole 1024x1024 frame with FP16, BF16 and FP8 E4M3 MLPs (the precision workload) against
  the oracle's restatement of each format, and a 32-row band against the FP64 oracle.
"""
import numpy as np
import pytest

from conftest import psnr

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

AV = 0


def diag(avatar):
    v = avatar.canonical.astype(np.float64)
    return float(np.linalg.norm(v.max(0) - v.min(0)))


@pytest.fixture(scope="module")
def full(avatar, frame0):
    from insta_gb300 import abi, synthetic as S
    c = abi.Context(0)
    c.canonical_set(AV, avatar.canonical, avatar.faces, avatar.mask)
    c.frame_upload(AV, 0, frame0)
    c.occupancy_from_mesh(AV, 0, 0.015)
    fc = S.FieldConfig()
    params = S.field_params(fc, seed=0)
    c.params_load(AV, fc, params)
    c.sync()
    yield c, fc, params
    c.close()


@pytest.fixture(scope="module")
def deform(oracle, oracle_frame):
    return oracle.Deformation(oracle_frame["def"], oracle_frame["can"], oracle_frame["adj"], oracle_frame["bvh"])


@pytest.fixture(scope="module")
def bits(oracle, oracle_frame):
    return oracle.occupancy(oracle_frame["def"], 0.015)


def test_canonical_map_1m_points(full, oracle, oracle_frame, avatar, frame0, deform):
    from insta_gb300 import synthetic as S
    ctx = full[0]
    n = 1 << 20
    pts = S.shell_points(frame0, avatar.faces, n, seed=0, half_width=5e-3)
    idx = torch.empty(n, dtype=torch.int32, device="cuda")
    out = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    ctx.canonical_map_soa(AV, 0, torch.from_numpy(pts).cuda(), n, idx, out)
    ctx.sync()
    idx, out = idx.cpu().numpy(), out.cpu().numpy()
    ref_ids, ref = deform.map_soa(pts)
    assert (idx == ref_ids).all(), int((idx != ref_ids).sum())
    pick = np.random.default_rng(1).choice(n, 8192, replace=False)
    brute_ids, _ = oracle.nearest_brute(oracle_frame["def"], pts[pick])
    assert (idx[pick] == brute_ids).all()
    assert np.abs(out - ref).max() <= 1e-5 * diag(avatar)
    d64 = oracle.Deformation(oracle_frame["def"], oracle_frame["can"], oracle_frame["adj"], oracle_frame["bvh"], fp64=True)
    _, ref64 = d64.map_soa(pts)
    assert np.abs(out - ref64).max() <= 1e-5 * diag(avatar)


def render_gpu(ctx, W, H, yaw=0.0, tuning=None, host_rounds=False):
    from insta_gb300 import synthetic as S
    cam, focal = S.camera(yaw, width=W, height=H)
    counts = torch.zeros(W * H, dtype=torch.int32, device="cuda")
    req = ctx.render_desc(AV, 0, W, H, focal, cam, out_samples=counts)
    rgba = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda")
    depth = torch.zeros(W * H, dtype=torch.float32, device="cuda")
    if tuning:
        ctx.tuning_set(**tuning)
    if host_rounds:
        ctx.stats_enable(True)
    try:
        torch.cuda.synchronize()
        ctx.render(req, rgba, depth)
        n = ctx.render_samples()
    finally:
        if tuning:
            ctx.tuning_set()
        if host_rounds:
            ctx.stats_enable(False)
    return rgba.cpu().numpy(), depth.cpu().numpy(), counts.cpu().numpy().astype(np.uint32), n


@pytest.fixture(scope="module")
def frame512(full, oracle, avatar, deform, bits):
    from insta_gb300 import synthetic as S
    ctx, fc, params = full
    W = H = 512
    got = render_gpu(ctx, W, H)
    cam, focal = S.camera(0.0, width=W, height=H)
    rc = oracle.render_cfg(W, H, focal, cam, avatar.render_aabb())
    ref = oracle.render(rc, deform, bits, fc, params)
    return got, ref


def test_render_512_full_frame(frame512):
    (rgba, depth, counts, n), (r_rgba, r_depth, ns, total) = frame512
    assert total > 1_000_000
    assert psnr(rgba, r_rgba) >= 45.0
    # the GPU evaluates a round's samples before compositing them, so a ray that terminates early
    # was evaluated up to the end of its round: n >= the composited total
    assert counts.sum() <= n
    assert abs(int(counts.sum()) - total) <= total // 1000
    assert (counts == ns).mean() > 0.999, float((counts == ns).mean())
    assert (rgba[:, 3] > 0.001).sum() > 10000          # the avatar covers a good part of the frame
    hit = (r_rgba[:, 3] > 0.2) & (rgba[:, 3] > 0.2)    # depth is written where a pixel is opaque enough
    if hit.any():
        assert np.abs(depth[hit] - r_depth[hit]).max() < 1e-3
    assert ((r_rgba[:, 3] > 0.2) == (rgba[:, 3] > 0.2)).mean() > 0.999


def test_render_512_multi_round_bit_identical(full, frame512):
    (rgba, depth, counts, _), (_, _, ns, _) = frame512
    ctx = full[0]
    assert ns.max() > 3 * 3          # some rays span at least four rounds of 3 steps
    m_rgba, m_depth, m_counts, m_n = render_gpu(ctx, 512, 512, tuning=dict(max_steps_per_round=3))
    assert np.array_equal(m_rgba, rgba) and np.array_equal(m_depth, depth) and np.array_equal(m_counts, counts)
    h_rgba, h_depth, h_counts, _ = render_gpu(ctx, 512, 512, tuning=dict(max_steps_per_round=5), host_rounds=True)
    assert np.array_equal(h_rgba, rgba) and np.array_equal(h_depth, depth) and np.array_equal(h_counts, counts)
    w_rgba, w_depth, w_counts, _ = render_gpu(ctx, 512, 512, tuning=dict(max_steps_per_round=64))   # the longest rounds
    assert np.array_equal(w_rgba, rgba) and np.array_equal(w_depth, depth) and np.array_equal(w_counts, counts)
    s_rgba, s_depth, s_counts, _ = render_gpu(ctx, 512, 512, tuning=dict(sort_cell_bits=15, mlp_ctas_per_sm=1,
                                                                          deform_blocks_per_sm=8, bvh_top_nodes=21))
    assert np.array_equal(s_rgba, rgba) and np.array_equal(s_depth, depth) and np.array_equal(s_counts, counts)
    # the MLP stage with the weights resident once per SM (tile slots), and as CTAs of two tiles
    # with an MMA-issuing warp (8), against one copy per CTA
    for n_slots in (7, 2, 8):
        k_rgba, k_depth, k_counts, _ = render_gpu(ctx, 512, 512, tuning=dict(mlp_slots=n_slots))
        assert np.array_equal(k_rgba, rgba) and np.array_equal(k_depth, depth) and np.array_equal(k_counts, counts)
    # the deform + encode + MLP stage as one kernel, against encode to global tiles + MLP (default)
    f_rgba, f_depth, f_counts, _ = render_gpu(ctx, 512, 512, tuning=dict(fused_field_stage=1, bvh_top_nodes=5))
    assert np.array_equal(f_rgba, rgba) and np.array_equal(f_depth, depth) and np.array_equal(f_counts, counts)


@pytest.mark.parametrize("precision", [1, 2])
def test_mlp_slots_equal_ctas_bf16_fp8(full, precision):
    """BF16 and FP8 E4M3 MLPs: the tile-slot kernel (weights resident once per SM, one row per
    thread, the FP8 row scale without an exchange) gives the same bits as the per-CTA kernel."""
    ctx, fc, params = full
    ctx.params_load(AV, fc, params, precision=precision)
    try:
        a = render_gpu(ctx, 256, 256, yaw=-8.0, tuning=dict(mlp_slots=1))
        b = render_gpu(ctx, 256, 256, yaw=-8.0, tuning=dict(mlp_slots=6))
        c = render_gpu(ctx, 256, 256, yaw=-8.0, tuning=dict(mlp_slots=8))   # two-tile CTAs (FP8: per-CTA kernel)
    finally:
        ctx.params_load(AV, fc, params)
    assert (a[0][:, 3] > 0.05).sum() > 1000
    for x, y, z in zip(a[:3], b[:3], c[:3]):
        assert np.array_equal(x, y) and np.array_equal(x, z)


@pytest.mark.parametrize("precision,min_psnr", [(0, 45.0), (1, 45.0), (2, 35.0)])
def test_render_1024_precision(full, oracle, avatar, deform, bits, precision, min_psnr):
    """1024x1024: FP16 (the plain path), BF16, FP8 E4M3 MLPs against the oracle's restatement of
    the same format (the FP8 bound is looser: tensor-core accumulation order can move a
    re-quantised activation by one E4M3 step); a 32-row band against the FP64 oracle."""
    from insta_gb300 import synthetic as S
    ctx, fc, params = full
    W = H = 1024
    ctx.params_load(AV, fc, params, precision=precision)
    try:
        rgba, depth, counts, n = render_gpu(ctx, W, H, yaw=4.0)
    finally:
        ctx.params_load(AV, fc, params)
    cam, focal = S.camera(4.0, width=W, height=H)
    rc = oracle.render_cfg(W, H, focal, cam, avatar.render_aabb())
    r_rgba, _, ns, total = oracle.render(rc, deform, bits, fc, params, weight_format=precision)
    assert total > 4_000_000
    assert psnr(rgba, r_rgba) >= min_psnr
    assert abs(int(counts.sum()) - total) <= total // 500
    rows = (496, 528)
    r64, _, _, _ = oracle.render(rc, deform, bits, fc, params, rows=rows, fp64=True)
    band = rgba[rows[0] * W:rows[1] * W]
    assert psnr(band, r64) >= {0: 60.0, 1: 50.0, 2: 40.0}[precision]
