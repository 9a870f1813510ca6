"""The oracle's restatement of the error map (compute_loss_kernel_train_nerf's deposit, the CDF
builders of train_nerf_step) and of the training batch's image / pixel draws (image_idx,
nerf_random_image_pos_training), against float64 NumPy and statistical properties, without a GPU.
The draws rest on the oracle's pcg32 and ld_random_val, both pinned elsewhere (the PCG demo's
published outputs, the reference's own Sobol code)."""
import numpy as np
import pytest


def np_cdf(em):
    """float64 restatement of construct_cdf_2d / _1d and the image CDF."""
    em = em.astype(np.float64)
    n, h, w = em.shape
    row = np.cumsum(em + 1e-10, axis=2)
    tot = row[:, :, -1]
    cx = 0.99 * row / tot[:, :, None] + 0.01 * np.arange(1, w + 1) / w
    cy_raw = np.cumsum(tot, axis=1)
    ci_raw = cy_raw[:, -1]
    cy = 0.99 * cy_raw / ci_raw[:, None] + 0.01 * np.arange(1, h + 1) / h
    s = ci_raw.sum()
    pm = 0.9 * ci_raw / s + 0.1 / n
    ci = 0.9 * np.cumsum(ci_raw) / s + 0.1 * np.arange(1, n + 1) / n
    return cx, cy, ci, pm


def test_error_map_cdf_matches_float64(oracle):
    em = np.random.default_rng(0).gamma(0.5, 1.0, (4, 23, 37)).astype(np.float32)
    em[2] = 0.0                                                # an image without error: uniform CDFs
    got = oracle.error_map_cdf(em)
    for g, r in zip(got, np_cdf(em)):
        np.testing.assert_allclose(g, r, rtol=2e-6, atol=2e-7)
    cx, cy, ci, pm = got
    assert (np.diff(cx, axis=2) >= 0).all() and (np.diff(cy, axis=1) >= 0).all() and (np.diff(ci) >= 0).all()
    assert abs(float(pm.sum()) - 1.0) < 1e-5 and abs(float(ci[-1]) - 1.0) < 1e-5


def test_training_pixels_uniform_draws(oracle):
    """No CDFs: image (i + n_rays_total) n_images / n_rays mod n_images, then the ray's pcg32
    sub-stream (advanced by 8 i): two draws for the position, three for the background."""
    n, n_img, total = 300, 7, 12345
    rng = oracle.Pcg32.seeded(42, 54)
    img, xy, pdf, bg = oracle.training_pixels(n, total, n_img, rng)
    i = np.arange(n, dtype=np.uint64)
    np.testing.assert_array_equal(img, (((i + total) * n_img) // n) % n_img)
    assert (pdf == 1.0).all()
    for k in (0, 1, 150, 299):
        r = rng.copy()
        r.advance(8 * k)
        draws = [r.next_float() for _ in range(5)]
        assert list(xy[k]) == draws[:2] and list(bg[k]) == draws[2:]


def test_training_pixels_snap_to_pixel_centres(oracle):
    n, n_img = 500, 3
    res = np.array([[640, 480], [37, 23], [1, 1]], np.int32)
    img, xy, _, _ = oracle.training_pixels(n, 0, n_img, oracle.Pcg32.seeded(7, 3), resolution=res, snap=True)
    wh = res[img].astype(np.float64)
    frac = xy * wh - 0.5
    assert np.allclose(frac, np.round(frac), atol=1e-4)        # pixel centres
    assert ((xy > 0) & (xy < 1)).all()


def test_training_pixels_follow_the_error_map(oracle):
    """With the CDFs half the position draws are uniform and half follow the map: a map with one
    hot cell per image receives about half of that image's samples there, and the pdf the draw
    reports is that cell's mass x cells (1 for the uniform half); images follow cdf_img."""
    n_img, h, w = 2, 8, 16
    em = np.full((n_img, h, w), 1e-3, np.float32)
    em[0, 3, 5] = 10.0
    em[1, 6, 2] = 30.0
    cx, cy, ci, pm = oracle.error_map_cdf(em)
    n = 40000
    img, xy, pdf, _ = oracle.training_pixels(n, 0, n_img, oracle.Pcg32.seeded(3, 9), cdfs=(cx, cy, ci), cdf_res=(w, h))
    frac_img = np.bincount(img, minlength=n_img) / n
    np.testing.assert_allclose(frac_img, pm, atol=0.01)
    for k, (hy, hx) in enumerate([(3, 5), (6, 2)]):
        sel = img == k
        cell = (np.floor(xy[sel, 1] * h) == hy) & (np.floor(xy[sel, 0] * w) == hx)
        assert 0.45 < cell.mean() < 0.56, (k, cell.mean())
    assert (pdf > 0).all() and np.isfinite(pdf).all()


def test_loss_deposits_each_kept_rays_mean_loss(oracle):
    """The error map gains exactly the kept rays' mean losses (bilinear weights sum to one), in
    each ray's own image slab; with a pdf the losses are divided by it."""
    from conftest import loss_cfg, train_loss_batch
    n = 400
    b = train_loss_batch(n, seed=5, stride=11)
    rng = np.random.default_rng(6)
    xy = rng.uniform(0, 1, (n, 2)).astype(np.float32)
    xy[:4] = [[0, 0], [1, 1], [0, 1], [1, 0]]
    img = rng.integers(0, 3, n).astype(np.uint32)
    pdf = rng.uniform(0.5, 2.0, n).astype(np.float32)
    cfg = loss_cfg(n_rays=n, stride=11, loss_type=0)
    em = np.zeros((3, 9, 13), np.float32)
    _, _, _, _, loss = oracle.train_loss(cfg, **b, pdf=pdf, error_map=em, image_xy=xy, image_index=img)
    _, _, _, _, loss1 = oracle.train_loss(cfg, **b)
    per_ray = loss * n                                          # mean loss of kept ray k
    np.testing.assert_allclose(em.sum(), per_ray.sum(), rtol=1e-5)
    for s in range(3):
        np.testing.assert_allclose(em[s].sum(), per_ray[img[b["ray_indices"]] == s].sum(), rtol=1e-5)
    np.testing.assert_allclose(loss, loss1 / pdf[b["ray_indices"]], rtol=1e-6)
