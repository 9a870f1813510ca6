"""Training side of the field (insta_field_backward, insta_adam_step, insta_train_loss) through the
C ABI (cuda:0).

Oracle: the FP64 forward/backward of the same network (oracle.field_backward), itself checked
against finite differences on the CPU.  Tolerances:
* FP32 forward outputs: |err| <= 1e-4 + 1e-4 |x| against the FP64 forward;
* parameter gradients: per layer and for the hash table, ||g - ref|| <= 1e-3 ||ref|| (FP32
  GEMMs and atomics against FP64; a ReLU that flips on a pre-activation within rounding of 0
  moves one sample's share, which the norm absorbs), and every entry within 1e-2 of the
  block's largest gradient;
* Adam: the FP16 parameters it writes give field outputs within the field parity tolerance
  (4e-3 + 1e-2 |x|) of the oracle run on a NumPy FP32 Adam of the same gradient;
* loss: per kept ray the same compacted count and records (bit-exact), gradients within
  1e-5 of the batch's largest + 1e-4 relative, per-ray losses 1e-5 relative (the kernel's
  __expf against the oracle's expf).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

AVATAR = 21


def coords(n, seed, n_extra=16):
    rng = np.random.default_rng(seed)
    c = np.zeros((n, 11 + n_extra), np.float32)
    c[:, :3] = rng.uniform(0.3, 0.7, size=(n, 3))
    d = rng.normal(size=(n, 3))
    c[:, 8:11] = (d / np.linalg.norm(d, axis=1, keepdims=True) + 1) * 0.5
    c[:, 11:] = rng.uniform(-1, 1, size=(n, n_extra))
    return c


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture()
def field(ctx):
    from insta_gb300 import layout as L, synthetic as S
    fc = S.FieldConfig(n_extra=16)
    params = S.field_params(fc, seed=5)
    ctx.params_load(AVATAR, fc, params)
    return fc, params, L.field_layout(fc)


def blocks(lay):
    out = [(off, off + n_out * n_in) for (off, n_out, n_in, _) in lay.mlp_layers(1.0)]
    return out + [(lay.table_offset, lay.total)]


def test_backward_matches_oracle(ctx, field, oracle):
    fc, params, lay = field
    n = 3000                                   # not a multiple of any tile or block
    c = coords(n, seed=1)
    g_out = np.random.default_rng(2).normal(size=(n, 4)).astype(np.float32)
    grad = torch.zeros(lay.total, dtype=torch.float32, device="cuda")
    out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    ctx.field_backward(AVATAR, dev(c), c.shape[1], n, dev(g_out), grad, out)
    ctx.sync()
    ref_g, ref_out = oracle.field_backward(fc, params, c, g_out)
    got_out = out.cpu().numpy()
    assert np.abs(got_out - ref_out).max() <= 1e-4 + 1e-4 * np.abs(ref_out).max()
    g = grad.cpu().numpy().astype(np.float64)
    for lo, hi in blocks(lay):
        a, b = g[lo:hi], ref_g[lo:hi]
        assert np.linalg.norm(b) > 0, (lo, hi)
        assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(b), (lo, hi, np.linalg.norm(a - b) / np.linalg.norm(b))
        assert np.abs(a - b).max() <= 1e-2 * np.abs(b).max(), (lo, hi)
    # the table gradient touches exactly the entries the samples' corners reach
    touched_ref = ref_g[lay.table_offset:] != 0
    assert ((g[lay.table_offset:] != 0) <= touched_ref).all()


def test_backward_tf32(ctx, field, oracle):
    """insta_train_set_math(TF32): layer products on tensor cores with TF32 inputs (10-bit
    mantissa, the reference trains in FP16) and FP32 accumulation: outputs within 5e-3 of the
    largest, per-block gradient norms within 5e-2 of the FP64 oracle (a weight gradient sums
    thousands of products of both signs, so TF32 input rounding shows at the percent level there:
    2 % measured on the first layer)."""
    fc, params, lay = field
    n = 3000
    c = coords(n, seed=11)
    g_out = np.random.default_rng(12).normal(size=(n, 4)).astype(np.float32)
    grad = torch.zeros(lay.total, dtype=torch.float32, device="cuda")
    out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    ctx.train_set_math(True)
    try:
        ctx.field_backward(AVATAR, dev(c), c.shape[1], n, dev(g_out), grad, out)
        ctx.sync()
    finally:
        ctx.train_set_math(False)
    ref_g, ref_out = oracle.field_backward(fc, params, c, g_out)
    assert np.abs(out.cpu().numpy() - ref_out).max() <= 5e-3 * np.abs(ref_out).max()
    g = grad.cpu().numpy().astype(np.float64)
    for lo, hi in blocks(lay):
        a, b = g[lo:hi], ref_g[lo:hi]
        assert np.linalg.norm(a - b) <= 5e-2 * np.linalg.norm(b), (lo, hi, np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n", [3000, 77, 128 * 152 * 2 + 5])
def test_backward_tcgen05(ctx, field, oracle, n):
    """insta_train_set_math(TCGEN05): the library's tcgen05 kernel, FP16 operands (encoding, kept
    activations, output gradients, weights) with FP32 accumulation, the arithmetic class of the
    reference's FP16 fused MLP training: outputs within 5e-3 of the largest, per-block gradient
    norms within 5e-2 of the FP64 oracle.  Sizes: ragged, one partial tile, and more tiles than
    CTAs (each CTA keeps its weight-gradient accumulators in TMEM over several tiles)."""
    fc, params, lay = field
    c = coords(n, seed=21 + n)
    g_out = np.random.default_rng(22 + n).normal(size=(n, 4)).astype(np.float32)
    grad = torch.zeros(lay.total, dtype=torch.float32, device="cuda")
    out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    ctx.train_set_math(False, tcgen05=True)
    try:
        ctx.field_backward(AVATAR, dev(c), c.shape[1], n, dev(g_out), grad, out)
        ctx.sync()
        out_fwd = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        ctx.field_backward(AVATAR, dev(c), c.shape[1], n, None, None, out_fwd)   # forward only
        ctx.sync()
    finally:
        ctx.train_set_math(False)
    ref_g, ref_out = oracle.field_backward(fc, params, c, g_out)
    got = out.cpu().numpy()
    assert np.abs(got - ref_out).max() <= 5e-3 * np.abs(ref_out).max()
    assert np.array_equal(out_fwd.cpu().numpy(), got)
    g = grad.cpu().numpy().astype(np.float64)
    for lo, hi in blocks(lay):
        a, b = g[lo:hi], ref_g[lo:hi]
        assert np.linalg.norm(a - b) <= 5e-2 * np.linalg.norm(b), (lo, hi, np.linalg.norm(a - b) / np.linalg.norm(b))
    touched_ref = ref_g[lay.table_offset:] != 0
    assert ((g[lay.table_offset:] != 0) <= touched_ref).all()


@pytest.mark.parametrize("tcgen05", [False, True])
def test_extra_dims_gradient(ctx, field, oracle, tcgen05):
    """insta_field_backward_ex's expression-dim gradients against the FP64 oracle (FP32 products:
    within 1e-4 of the largest; tcgen05's FP16 operands: norm within 5e-2), then
    insta_extra_dims_gradient: each kept ray's samples summed into its image's row, against a
    float64 sum of the same per-sample gradients (1e-5 of the largest row)."""
    fc, params, lay = field
    n = 3000
    c = coords(n, seed=31)
    g_out = np.random.default_rng(32).normal(size=(n, 4)).astype(np.float32)
    grad = torch.zeros(lay.total, dtype=torch.float32, device="cuda")
    dx = torch.zeros((n, 16), dtype=torch.float32, device="cuda")
    ctx.train_set_math(False, tcgen05=tcgen05)
    try:
        ctx.field_backward(AVATAR, dev(c), c.shape[1], n, dev(g_out), grad, None, dl_dextra=dx)
        ctx.sync()
    finally:
        ctx.train_set_math(False)
    _, _, ref_dx = oracle.field_backward(fc, params, c, g_out, extra_grad=True)
    got = dx.cpu().numpy().astype(np.float64)
    if tcgen05:
        assert np.linalg.norm(got - ref_dx) <= 5e-2 * np.linalg.norm(ref_dx)
    else:
        assert np.abs(got - ref_dx).max() <= 1e-4 * np.abs(ref_dx).max()
    # per image sums over kept rays' compacted blocks (rays in a shuffled order, some empty)
    rng = np.random.default_rng(33)
    n_rays, n_img = 400, 5
    counts = rng.integers(0, 15, n_rays).astype(np.uint32)
    counts[0] = 0
    total = int(counts.sum())
    assert total <= n
    bases = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint32)
    perm = rng.permutation(n_rays).astype(np.uint32)
    img = rng.integers(0, n_img, n_rays).astype(np.uint32)
    img[perm[3]] = n_img + 2                                   # a ray of an image outside the gradient adds nothing
    kept = n_rays - 7                                          # the last rays were not kept
    out = torch.zeros((n_img, 16), dtype=torch.float32, device="cuda")
    i32 = lambda a: dev(a.view(np.int32))
    ctx.extra_dims_gradient(n_rays, 16, n_img, i32(np.array([kept], np.uint32)), i32(perm), i32(np.stack([counts, bases], 1)), i32(img),
                            dx, out)
    ctx.sync()
    ref = np.zeros((n_img, 16), np.float64)
    for i in range(kept):
        if img[perm[i]] < n_img:
            ref[img[perm[i]]] += got[bases[i]:bases[i] + counts[i]].sum(0)
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-5 * np.abs(ref).max()


def test_backward_accumulates_and_forward_only(ctx, field, oracle):
    fc, params, lay = field
    n = 700
    c = dev(coords(n, seed=3))
    g_out = dev(np.random.default_rng(4).normal(size=(n, 4)).astype(np.float32))
    g1 = torch.zeros(lay.total, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()                             # torch's stream -> the context's stream
    ctx.field_backward(AVATAR, c, 27, n, g_out, g1)
    ctx.sync()
    g2 = g1.clone()
    out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ctx.field_backward(AVATAR, c, 27, n, g_out, g2)      # adds a second copy
    ctx.field_backward(AVATAR, c, 27, n, None, None, out)  # forward only
    ctx.sync()
    a, b = g1.cpu().numpy(), g2.cpu().numpy()
    assert np.allclose(b, 2 * a, rtol=1e-5, atol=1e-7 * np.abs(a).max())
    ref_out = oracle.field_backward(fc, params, c.cpu().numpy())[1]
    assert np.abs(out.cpu().numpy() - ref_out).max() <= 1e-4 + 1e-4 * np.abs(ref_out).max()


def numpy_adam(w, g, steps, lr, b1, b2, eps, l2, n_matrix, loss_scale=1.0, decay=None):
    """FP32 NumPy restatement of insta_adam_step: gradient / loss_scale; L2 and a step every call
    for the first n_matrix (MLP) parameters; table entries with a zero gradient skipped, the others
    counting their own steps; lr sqrt(1 - b2^t) / (1 - b1^t) * m / (sqrt(v) + eps).  With decay the
    Ema's bias-corrected average is returned beside the weights."""
    w = w.astype(np.float32).copy()
    m = np.zeros_like(w)
    v = np.zeros_like(w)
    t_tab = np.zeros(w.size - n_matrix, np.int64)
    e = None
    for t in range(1, steps + 1):
        gi = (g / np.float32(loss_scale)).astype(np.float32)
        upd = np.ones(w.size, bool)
        upd[n_matrix:] = gi[n_matrix:] != 0
        gi[:n_matrix] += np.float32(l2) * w[:n_matrix]
        t_tab[upd[n_matrix:]] += 1
        tt = np.concatenate([np.full(n_matrix, t), np.maximum(t_tab, 1)]).astype(np.float64)
        lr_t = (lr * np.sqrt(1 - b2 ** tt) / (1 - b1 ** tt)).astype(np.float32)
        m_new = np.float32(b1) * m + np.float32(1 - b1) * gi
        v_new = np.float32(b2) * v + np.float32(1 - b2) * gi * gi
        w_new = w - lr_t * m_new / (np.sqrt(v_new) + np.float32(eps))
        m, v, w = np.where(upd, m_new, m), np.where(upd, v_new, v), np.where(upd, w_new, w)
        if decay is not None:
            e = w.copy() if e is None else (e * np.float32(decay * (1 - decay ** (t - 1))) + np.float32(1 - decay) * w) / np.float32(1 - decay ** t)
    return w if decay is None else (w, e)


@pytest.mark.parametrize("loss_scale", [1.0, 128.0])
def test_adam_matches_numpy(ctx, field, oracle, loss_scale):
    """Two Adam steps on a gradient that touches only part of the hash table (2000 points): the
    field outputs match the oracle on a NumPy FP32 restatement; with loss_scale 128 the gradient
    carries the factor, so the step equals the unscaled one; untouched table entries (zero
    gradient) keep their values, the MLP weights all move."""
    fc, params, lay = field
    n = 2000
    c = coords(n, seed=6)
    g_out = np.random.default_rng(7).normal(size=(n, 4)).astype(np.float32)
    grad = torch.zeros(lay.total, dtype=torch.float32, device="cuda")
    ctx.field_backward(AVATAR, dev(c), 27, n, dev(g_out * np.float32(loss_scale)), grad)
    cfg = dict(learning_rate=1e-2, beta1=0.9, beta2=0.99, epsilon=1e-15, l2_reg=1e-6)
    ctx.adam_step(AVATAR, grad, loss_scale=loss_scale, **cfg)
    ctx.adam_step(AVATAR, grad, loss_scale=loss_scale, **cfg)          # second step: the moments carry over
    cq = coords(1500, seed=8)
    out = torch.zeros((len(cq), 4), dtype=torch.float32, device="cuda")
    ctx.field_eval(AVATAR, dev(cq), 27, len(cq), out)
    ctx.sync()
    g = grad.cpu().numpy()
    n_matrix = lay.table_offset
    tab_zero = g[n_matrix:] == 0
    assert tab_zero.any() and not tab_zero.all()
    w32 = numpy_adam(params.astype(np.float32), g, 2, cfg["learning_rate"], cfg["beta1"], cfg["beta2"], cfg["epsilon"],
                     cfg["l2_reg"], n_matrix, loss_scale)
    assert np.array_equal(w32[n_matrix:][tab_zero], params.astype(np.float32)[n_matrix:][tab_zero])
    w_new = w32.astype(np.float16)
    ref = oracle.field_eval(fc, w_new, cq)
    before = oracle.field_eval(fc, params, cq)
    got = out.cpu().numpy()
    assert np.abs(ref - before).max() > 0.05          # the step moved the field
    err = np.abs(got - ref)
    assert (err <= 4e-3 + 1e-2 * np.abs(ref)).all(), float(err.max())


def test_adam_ema_matches_numpy(ctx, field, oracle):
    """Adam inside the Ema wrapper (decay 0.95, 3 steps): the field's parameters -- what
    insta_field_eval and rendering read -- are the bias-corrected average of the weights, within the
    field parity tolerance of the oracle on a NumPy FP32 Adam + Ema; the training forward keeps
    the raw weights (FP16-rounded for the oracle, hence the same tolerance)."""
    fc, params, lay = field
    n = 2000
    c = coords(n, seed=13)
    g_out = np.random.default_rng(14).normal(size=(n, 4)).astype(np.float32)
    grad = torch.zeros(lay.total, dtype=torch.float32, device="cuda")
    ctx.field_backward(AVATAR, dev(c), 27, n, dev(g_out), grad)
    cfg = dict(learning_rate=1e-2, beta1=0.9, beta2=0.99, epsilon=1e-15, l2_reg=1e-6)
    decay = 0.95
    for _ in range(3):
        ctx.adam_step(AVATAR, grad, ema_decay=decay, **cfg)
    cq = coords(1500, seed=15)
    inf_out = torch.zeros((len(cq), 4), dtype=torch.float32, device="cuda")
    train_out = torch.zeros((len(cq), 4), dtype=torch.float32, device="cuda")
    dq = dev(cq)
    tc_out = torch.zeros((len(cq), 4), dtype=torch.float32, device="cuda")
    ctx.field_eval(AVATAR, dq, 27, len(cq), inf_out)
    ctx.field_backward(AVATAR, dq, 27, len(cq), None, None, train_out)
    ctx.field_eval_training(AVATAR, dq, 27, len(cq), tc_out)
    ctx.sync()
    g = grad.cpu().numpy()
    w, e = numpy_adam(params.astype(np.float32), g, 3, cfg["learning_rate"], cfg["beta1"], cfg["beta2"], cfg["epsilon"],
                      cfg["l2_reg"], lay.table_offset, decay=decay)
    ref_inf = oracle.field_eval(fc, e.astype(np.float16), cq)
    ref_train = oracle.field_eval(fc, w.astype(np.float16), cq)
    got_inf, got_train = inf_out.cpu().numpy(), train_out.cpu().numpy()
    assert np.abs(ref_inf - ref_train).max() > 0.02                     # the average differs from the weights
    assert (np.abs(got_inf - ref_inf) <= 4e-3 + 1e-2 * np.abs(ref_inf)).all(), float(np.abs(got_inf - ref_inf).max())
    assert (np.abs(got_train - ref_train) <= 4e-3 + 1e-2 * np.abs(ref_train)).all(), float(np.abs(got_train - ref_train).max())
    got_tc = tc_out.cpu().numpy()   # the tensor-core evaluation of the training weights' FP16 copy
    assert (np.abs(got_tc - ref_train) <= 4e-3 + 1e-2 * np.abs(ref_train)).all(), float(np.abs(got_tc - ref_train).max())


def test_regression_loss_decreases(ctx, field):
    """A few hundred Adam steps fitting fixed targets with an L2 loss: the backward's sign and
    scale, and the optimizer state across steps, together reduce the loss by 10x."""
    fc, params, lay = field
    n = 4096
    c = dev(coords(n, seed=9))
    target = dev(np.random.default_rng(10).uniform(-1, 1, size=(n, 4)).astype(np.float32))
    out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    grad = torch.zeros(lay.total, dtype=torch.float32, device="cuda")
    losses = []
    for step in range(200):
        torch.cuda.synchronize()                         # the context's stream is not torch's
        ctx.field_backward(AVATAR, c, 27, n, None, None, out)
        ctx.sync()
        diff = out - target
        losses.append(float((diff * diff).mean()))
        grad.zero_()
        dl = (2.0 / diff.numel()) * diff
        torch.cuda.synchronize()
        ctx.field_backward(AVATAR, c, 27, n, dl, grad)
        ctx.adam_step(AVATAR, grad, learning_rate=1e-2)
        ctx.sync()
    assert np.isfinite(losses).all() and losses[-1] < 0.1 * losses[0], (losses[0], losses[-1])


def test_argument_errors(ctx, field):
    from insta_gb300 import abi
    fc, params, lay = field
    c = dev(coords(16, seed=0))
    g = torch.zeros(lay.total, dtype=torch.float32, device="cuda")
    with pytest.raises(abi.InstaError):
        ctx.field_backward(AVATAR, c, 27, 16, dev(np.zeros((16, 4), np.float32)), None)   # gradients without a target
    with pytest.raises(abi.InstaError):
        ctx.field_backward(AVATAR, c, 11, 16, None, None, torch.zeros((16, 4), device="cuda"))   # stride < 11 + 16
    with pytest.raises(abi.InstaError):
        ctx.field_backward(55, c, 27, 16, None, None, torch.zeros((16, 4), device="cuda"))   # no field on avatar 55
    with pytest.raises(abi.InstaError):
        ctx.adam_step(55, g)


def run_loss(ctx, b, cfg, mean_density=None, extra=None, **more):
    """insta_train_loss on device copies of a synthetic batch; returns host arrays.  `more` goes
    to the description as given (device tensors, error_map_res)."""
    n = len(b["ray_indices"])
    cap = cfg["max_samples_compacted"]
    as_dev = lambda v: dev(v.view(np.int32) if v.dtype == np.uint32 else v)   # torch has no general uint32
    d = {k: as_dev(v) for k, v in b.items()}
    d.update({k: as_dev(v) for k, v in (extra or {}).items()})
    ns = d["numsteps"].clone()
    counter = torch.zeros(1, dtype=torch.int32, device="cuda")
    rays_counter = torch.tensor([n], dtype=torch.int32, device="cuda")
    cout = torch.zeros((cap, cfg["stride"]), dtype=torch.float32, device="cuda")
    dloss = torch.zeros((cap, 4), dtype=torch.float32, device="cuda")
    loss = torch.zeros(n, dtype=torch.float32, device="cuda")
    md = None if mean_density is None else torch.tensor([mean_density], dtype=torch.float32, device="cuda")
    kw = {k: v for k, v in cfg.items()}
    kw.update(d)
    kw.update(numsteps=ns, numsteps_counter=counter, rays_counter=rays_counter, coords_out=cout, dloss_doutput=dloss,
              loss_output=loss, mean_density=md, max_rays=n)
    kw.update(more)
    torch.cuda.synchronize()                             # buffers filled on torch's stream
    ctx.train_loss(**kw)
    ctx.sync()
    return ns.cpu().numpy().view(np.uint32), int(counter.item()), cout.cpu().numpy(), dloss.cpu().numpy(), loss.cpu().numpy()


def check_blocks(got, ref, n_kept):
    """Per kept ray: same compacted count, same records, gradients within 1e-5 of the batch's
    largest plus 1e-4 relative (__expf against the oracle's expf), losses to 1e-5 relative."""
    ns, cnt, cout, dloss, loss = got
    rns, rcnt, rcout, rdloss, rloss = ref
    assert cnt == rcnt
    scale = np.abs(rdloss).max()
    for k in range(n_kept):
        c, base, rbase = int(ns[k, 0]), int(ns[k, 1]), int(rns[k, 1])
        assert c == int(rns[k, 0]), k
        np.testing.assert_array_equal(cout[base:base + c], rcout[rbase:rbase + c])
        err = np.abs(dloss[base:base + c] - rdloss[rbase:rbase + c])
        assert (err <= 1e-5 * scale + 1e-4 * np.abs(rdloss[rbase:rbase + c])).all(), (k, float(err.max()))
    np.testing.assert_allclose(loss, rloss, rtol=1e-5, atol=1e-9)


@pytest.mark.parametrize("loss_type,srgb,linear", [(4, 1, 0), (0, 0, 0), (1, 1, 1), (6, 1, 0)])
def test_train_loss_matches_oracle(ctx, oracle, loss_type, srgb, linear):
    from conftest import loss_cfg, train_loss_batch
    b = train_loss_batch(3000, seed=loss_type, stride=27)
    cfg = loss_cfg(n_rays=4096, stride=27, loss_type=loss_type, srgb_targets=srgb, train_in_linear_colors=linear, loss_scale=128.0)
    got = run_loss(ctx, b, cfg)
    ref = oracle.train_loss(cfg, **b)
    check_blocks(got, ref, 3000)


def test_train_loss_all_terms(ctx, oracle):
    """Depth supervision, segmentation rules, beta, density penalty, near-distance and mean-density
    regularisers, exposure; dense rays that stop early on transmittance."""
    from conftest import loss_cfg, train_loss_batch
    n = 2000
    b = train_loss_batch(n, seed=7, stride=27, max_steps=60)
    rng = np.random.default_rng(8)
    b["network_output"][::2, 3] += 5.0                      # opaque stretches: early termination
    extra = dict(depth=rng.uniform(0.2, 2.0, n).astype(np.float32),
                 seg_mask=rng.choice([0, 100, 120, 130, 140, 255], n).astype(np.int32),
                 exposure=rng.uniform(-0.5, 0.5, (n, 3)).astype(np.float32))
    b["target"][::5, 3] = 0.0                                # transparent targets (density penalty)
    cfg = loss_cfg(n_rays=n, stride=27, loss_type=4, depth_loss_type=1, loss_scale=128.0, depth_supervision_lambda=1.25,
                   seg_mask_supervision_lambda=40.0, near_distance=0.4, beta=0.05, penalize_density=1)
    got = run_loss(ctx, {**b, **extra}, cfg, mean_density=0.005)
    ref = oracle.train_loss(cfg, **b, **extra, mean_density=0.005)
    check_blocks(got, ref, n)
    assert int(got[0][:, 0].sum()) < int(b["numsteps"][:, 0].sum())     # some rays stopped early


def test_train_loss_cap_and_rollover(ctx, oracle):
    """max_samples_compacted cuts the batch (which ray is cut depends on the atomic order), the
    rest is filled to target_batch_size by repetition with the repeated gradients rescaled."""
    from conftest import loss_cfg, train_loss_batch
    b = train_loss_batch(1000, seed=11, stride=27)
    total = int(b["numsteps"][:, 0].sum())
    cap = total // 2
    cfg_cut = loss_cfg(n_rays=1000, stride=27, max_samples_compacted=cap, target_batch_size=cap)
    ns, cnt, cout, dloss, _ = run_loss(ctx, b, cfg_cut)
    assert cnt == total and int(ns[:, 0].sum()) == cap
    rns, _, rcout, rdloss, _ = oracle.train_loss(loss_cfg(n_rays=1000, stride=27), **b)
    scale = np.abs(rdloss).max()
    for k in range(1000):
        c, base, rbase = int(ns[k, 0]), int(ns[k, 1]), int(rns[k, 1])
        assert c <= int(rns[k, 0])
        if c:
            np.testing.assert_array_equal(cout[base:base + c], rcout[rbase:rbase + c])
            assert np.abs(dloss[base:base + c] - rdloss[rbase:rbase + c]).max() <= 1e-5 * scale + 1e-4 * np.abs(rdloss).max()
    # rollover past a count below the target: the tail repeats the head
    b2 = train_loss_batch(200, seed=12, stride=27)
    t2 = int(b2["numsteps"][:, 0].sum())
    tgt = t2 + 777
    ns2, cnt2, cout2, dloss2, _ = run_loss(ctx, b2, loss_cfg(n_rays=200, stride=27, max_samples_compacted=tgt, target_batch_size=tgt))
    assert cnt2 == t2
    src = np.arange(t2, tgt) % t2
    np.testing.assert_array_equal(cout2[t2:tgt], cout2[src])
    np.testing.assert_allclose(dloss2[t2:tgt], dloss2[src] * np.float32(t2 / tgt), rtol=1e-6, atol=0)


def test_train_loss_error_map_and_pdf(ctx, oracle):
    """The error map of compute_loss_kernel_train_nerf: each kept ray's mean loss (divided by its
    importance-sampling pdf) splatted bilinearly at its image position, rays at the corners of
    the image included.  Deposits are atomic additions in any order: the map agrees with the
    oracle's to 1e-5 of its largest cell; blocks, gradients and losses as in the other tests."""
    from conftest import loss_cfg, train_loss_batch
    n, n_img, rx, ry = 2500, 3, 37, 23
    b = train_loss_batch(n, seed=21, stride=27)
    rng = np.random.default_rng(22)
    xy = rng.uniform(0, 1, (n, 2)).astype(np.float32)
    xy[:5] = [[0, 0], [1, 1], [0, 1], [1, 0], [0.5, 0.5]]
    img = rng.integers(0, n_img, n).astype(np.uint32)
    pdf = rng.uniform(0.5, 2.0, n).astype(np.float32)
    cfg = loss_cfg(n_rays=n, stride=27, loss_type=4, loss_scale=128.0)
    em_dev = torch.zeros((n_img, ry, rx), dtype=torch.float32, device="cuda")
    img[7] = n_img + 4                                   # an image outside the map deposits nothing
    got = run_loss(ctx, b, cfg, extra=dict(image_xy=xy, image_index=img, pdf=pdf), error_map=em_dev, error_map_res=(rx, ry),
                   error_map_images=n_img)
    em_ref = np.zeros((n_img, ry, rx), np.float32)
    ref = oracle.train_loss(cfg, **b, pdf=pdf, error_map=em_ref, image_xy=xy, image_index=img)
    check_blocks(got, ref, n)
    em = em_dev.cpu().numpy()
    assert np.abs(em - em_ref).max() <= 1e-5 * np.abs(em_ref).max()
    assert ((em != 0) == (em_ref != 0)).all()


@pytest.mark.parametrize("mode", ["uniform", "cdf", "cdf_snap"])
def test_training_pixels_and_cdf_match_oracle(ctx, oracle, mode):
    """insta_error_map_cdf and insta_training_pixels against the oracle bit for bit: the CDFs,
    then per ray the image (evenly spread or from cdf_img with the low-discrepancy draw), the
    position (pcg32 sub-stream, sample_cdf_2d, pixel-centre snap), the pdf and the background
    draw."""
    n, n_img, total, w, h = 5000, 7, 12345, 37, 23
    res = np.array([[640, 480], [512, 512], [37, 23], [1, 1], [1024, 768], [3, 2], [256, 256]], np.int32)
    rng = oracle.Pcg32.seeded(1337, 11)
    cdfs = None
    if mode != "uniform":
        em = np.random.default_rng(4).gamma(0.5, 1.0, (n_img, h, w)).astype(np.float32)
        em[3] = 0.0
        rcx, rcy, rci, rpm = oracle.error_map_cdf(em)
        cx = torch.zeros((n_img, h, w), dtype=torch.float32, device="cuda")
        cy = torch.zeros((n_img, h), dtype=torch.float32, device="cuda")
        ci = torch.zeros(n_img, dtype=torch.float32, device="cuda")
        pm = torch.zeros(n_img, dtype=torch.float32, device="cuda")
        ctx.error_map_cdf(dev(em), n_img, w, h, cx, cy, ci, pm)
        ctx.sync()
        for g, r in ((cx, rcx), (cy, rcy), (ci, rci), (pm, rpm)):
            np.testing.assert_array_equal(g.cpu().numpy(), r)
        cdfs = (cx, cy, ci)
    snap = mode == "cdf_snap"
    out_img = torch.zeros(n, dtype=torch.int32, device="cuda")
    out_xy = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    out_pdf = torch.zeros(n, dtype=torch.float32, device="cuda")
    out_bg = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    ctx.training_pixels(n, n_img, rng.state, rng.inc, out_img, out_xy, out_pdf, out_bg, n_rays_total=total, resolution=dev(res),
                        snap=snap, cdfs=cdfs, cdf_res=(w, h))
    ctx.sync()
    ri, rxy, rpdf, rbg = oracle.training_pixels(n, total, n_img, rng, resolution=res, snap=snap,
                                                cdfs=None if cdfs is None else (rcx, rcy, rci), cdf_res=(w, h))
    np.testing.assert_array_equal(out_img.cpu().numpy().view(np.uint32), ri)
    np.testing.assert_array_equal(out_xy.cpu().numpy(), rxy)
    np.testing.assert_array_equal(out_pdf.cpu().numpy(), rpdf)
    np.testing.assert_array_equal(out_bg.cpu().numpy(), rbg)


@pytest.mark.parametrize("layout", ["benchmark", "insta"])
def test_train_step_fits_a_constant_colour(ctx, avatar, frame0, layout):
    """insta_gb300.train.TrainStep: training samples -> field evaluation -> loss -> backward ->
    Adam, 80 steps towards an opaque constant-colour target, lowers the batch loss 4x (INSTA's wider
    field gets there within its first steps, so against the first step's loss); for the
    benchmark field (tcgen05 layer products) and INSTA's shipped one (16 levels x 8 features, 16
    expression dims, 2 + 3 hidden layers: TF32 layer products, 16-byte table reductions)."""
    from insta_gb300 import synthetic as S
    from insta_gb300.train import TrainConfig, TrainStep
    aid = 22 if layout == "benchmark" else 23
    ctx.canonical_set(aid, avatar.canonical, avatar.faces, avatar.mask)
    ctx.frame_upload(aid, 0, frame0)
    ctx.occupancy_from_mesh(aid, 0, 0.015)
    fc = S.FieldConfig() if layout == "benchmark" else S.insta_field_config()
    ctx.params_load(aid, fc, S.field_params(fc, seed=2))
    cfg = TrainConfig(n_rays_per_batch=4096, target_batch_size=1 << 16, max_samples=1 << 19)
    cfg.adam["learning_rate"] = 1e-2
    ts = TrainStep(ctx, aid, fc, cfg)
    assert ts.tcgen05 == (layout == "benchmark")
    extra = dev(np.linspace(-0.5, 0.5, fc.n_extra, dtype=np.float32).reshape(1, -1)) if fc.n_extra else None
    rng = np.random.default_rng(3)
    n = cfg.n_rays_per_batch
    target = dev(np.tile(np.array([[0.8, 0.3, 0.2, 1.0]], np.float32), (n, 1)))
    image = dev(np.zeros(n, np.int32))
    losses, kept = [], []
    for step in range(80):
        c0 = np.array([0.5, 0.5, 0.5], np.float32)
        u = rng.normal(size=(n, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        org = c0 + u * 0.9
        tgt = c0 + rng.normal(0, 0.05, (n, 3))
        rays = dev(np.concatenate([org, tgt - org], 1).astype(np.float32))
        info = ts.step(0, rays, image, dev(rng.random(n).astype(np.float32)), target, extra=extra, n_images=1 if extra is not None else 0)
        kept.append(info["rays_kept"])
        losses.append(ts.loss_value())
    ctx.train_set_math(False)
    assert min(kept) > n // 2
    assert np.isfinite(losses).all() and np.mean(losses[-5:]) < 0.25 * losses[0], (losses[:5], losses[-5:])
    if layout == "benchmark":
        assert np.mean(losses[-5:]) < 0.25 * np.mean(losses[:5]), (losses[:5], losses[-5:])


def test_empty_and_invalid_training_calls(ctx, field):
    """Edge cases: no kept rays (nothing written, the rollover leaves the buffers alone), zero
    samples to the backward, and the arguments the entry points reject."""
    from insta_gb300 import abi
    fc, params, lay = field
    cap = 64
    zero = torch.zeros(1, dtype=torch.int32, device="cuda")
    counter = torch.zeros(1, dtype=torch.int32, device="cuda")
    cout = torch.full((cap, 27), 7.0, device="cuda")
    dloss = torch.full((cap, 4), 7.0, device="cuda")
    one = torch.zeros((1, 27), device="cuda")
    torch.cuda.synchronize()
    ctx.train_loss(n_rays=16, max_rays=16, max_samples_compacted=cap, target_batch_size=cap, stride=27, rays=torch.zeros((16, 6), device="cuda"),
                   target=torch.zeros((16, 4), device="cuda"), rays_counter=zero, ray_indices=torch.zeros(16, dtype=torch.int32, device="cuda"),
                   numsteps=torch.zeros((16, 2), dtype=torch.int32, device="cuda"), coords=one, network_output=torch.zeros((1, 4), device="cuda"),
                   numsteps_counter=counter, coords_out=cout, dloss_doutput=dloss)
    g = torch.zeros(lay.total, dtype=torch.float32, device="cuda")
    ctx.field_backward(AVATAR, one, 27, 0, torch.zeros((1, 4), device="cuda"), g)   # n = 0: nothing to do
    ctx.sync()
    assert int(counter.item()) == 0 and bool((cout == 7.0).all()) and bool((dloss == 7.0).all()) and float(g.abs().sum()) == 0.0
    with pytest.raises(abi.InstaError):
        ctx.train_loss(n_rays=0, max_rays=0, max_samples_compacted=cap, stride=27, rays_counter=zero, numsteps_counter=counter)
    with pytest.raises(abi.InstaError):
        ctx.train_loss(n_rays=1, max_rays=0, max_samples_compacted=cap, target_batch_size=cap + 1, stride=27, rays_counter=zero,
                       numsteps_counter=counter, coords_out=cout, dloss_doutput=dloss)
    with pytest.raises(abi.InstaError):
        ctx.train_loss(n_rays=1, max_rays=0, max_samples_compacted=cap, loss_type=9, stride=27, rays_counter=zero, numsteps_counter=counter)
    with pytest.raises(abi.InstaError):
        ctx.adam_step(AVATAR, g, ema_decay=1.0)
    with pytest.raises(abi.InstaError):
        ctx._check(ctx.lib.insta_train_set_math(ctx.h, 7))
