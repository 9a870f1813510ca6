"""The oracle pinned against the reference's own code.

* golden: tests/golden/reference_geometry.npz holds outputs of the INSTA headers compiled for
  the host (tests/golden/make_golden.py via oracle/build_ref.py); the oracle must reproduce them
  -- bit-exact for squared distances, the traversal result and the jitter sequences, within
  float rounding for frames and transforms.
* live: where the INSTA sources are present (this build container) the same comparisons run on
  fresh random inputs against oracle/_ref/libinsta_ref.so.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_geometry.npz"


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLDEN))


def p(a):
    return C.c_void_p(a.ctypes.data)


def test_golden_distance_sq_bit_exact(oracle, g):
    lib = oracle.lib()
    tris, pts = g["dist_tris"], g["dist_pts"]
    ours = np.array([lib.orc_tri_distance_sq(p(tris[i:i + 1]), p(pts[i])) for i in range(len(tris))], np.float32)
    assert (ours.view(np.uint32) == g["dist_ref"].view(np.uint32)).all()


def test_golden_box_distance_bit_exact(oracle, g):
    lib = oracle.lib()
    ours = np.array([lib.orc_box_distance_sq(p(g["box_min"][i]), p(g["box_max"][i]), p(g["box_pts"][i]))
                     for i in range(len(g["box_pts"]))], np.float32)
    assert (ours.view(np.uint32) == g["box_ref"].view(np.uint32)).all()


def test_golden_frames(oracle, g):
    lib = oracle.lib()
    ft = g["frame_tris"]
    tbn = np.zeros((len(ft), 9), np.float32)
    proj = np.zeros((len(ft), 16), np.float32)
    for i in range(len(ft)):
        lib.orc_tbn(p(ft[i:i + 1]), p(tbn[i]))
        lib.orc_tri2projection(p(ft[i:i + 1]), p(proj[i]))
    # regular triangles: identical operation order, identical bits
    e1 = ft["b"] - ft["a"]
    e2 = ft["c"] - ft["a"]
    s2 = np.sum(np.cross(e1, e2) ** 2, 1) / (np.sum(e1 ** 2, 1) * np.sum(e2 ** 2, 1))
    regular = s2 > 1e-10
    assert (tbn[regular] == g["tbn_ref"][regular]).all()
    assert (proj[regular] == g["proj_ref"][regular]).all()
    # Near-degenerate triangles: the oracle (like the device) builds these frames in FP64, a
    # deliberate deviation -- the reference's FP32 frame is ill-conditioned there.  They must
    # match an FP64 evaluation of the same formula (or the reference bit for bit, when the
    # triangle is regular enough to take the FP32 path).
    for i in np.flatnonzero(~regular):
        if (proj[i] == g["proj_ref"][i]).all():
            continue
        a, b, c = (ft[k][i].astype(np.float64) for k in ("a", "b", "c"))
        n = np.cross(b - a, c - a); n /= np.linalg.norm(n)
        bt = np.cross(b - a, n); bt /= np.linalg.norm(bt)
        tg = np.cross(bt, n); tg /= np.linalg.norm(tg)
        m = np.stack([tg, bt, n], axis=1) * (ft["scaling"][i] if ft["mask_id"][i] == 1 else 1.0)
        assert np.abs(proj[i].reshape(4, 4)[:3, :3] - m).max() < 1e-6, i


def test_golden_blended_frames_and_transforms(oracle, g):
    lib = oracle.lib()
    q, ids, adj = g["blend_pts"], g["blend_ids"], g["mesh_adj"]
    got = np.zeros_like(g["blend_ref"])
    for i in range(len(q)):
        lib.orc_interpolate_transformation(p(q[i]), p(adj), p(g["mesh_def"]), C.c_uint32(int(ids[i])), C.c_int(1), p(got[i, 0]))
        lib.orc_interpolate_transformation(p(q[i]), p(adj), p(g["mesh_can"]), C.c_uint32(int(ids[i])), C.c_int(0), p(got[i, 1]))
    ref = g["blend_ref"]
    assert np.abs(got[:, 1] - ref[:, 1]).max() <= 1e-6
    assert np.abs(got[:, 0] - ref[:, 0]).max() <= 1e-3 * max(1.0, np.abs(ref[:, 0]).max())
    tp = np.zeros((len(q), 3), np.float32)
    td = np.zeros((len(q), 3), np.float32)
    for i in range(len(q)):
        lib.orc_transform(p(q[i]), p(g["transform_dirs"][i]), p(ref[i, 0]), p(ref[i, 1]), p(tp[i]), p(td[i]))
    assert np.abs(tp - g["transform_p_ref"]).max() <= 1e-6
    assert np.abs(td - g["transform_d_ref"]).max() <= 1e-6


def test_golden_closest_triangle(oracle, g):
    """closest_triangle (NGP/bvh.cuh:48-96) on the same BVH: the oracle's reference-rule traversal
    returns the same triangle and distance; the exact (lowest-id) rule returns the same distance."""
    lib = oracle.lib()
    nodes, srt, qq = g["bvh_nodes"], g["bvh_sorted"], g["closest_pts"]
    ids = np.zeros(len(qq), np.int32)
    d2 = np.zeros(len(qq), np.float32)
    lib.orc_nearest_bvh(p(nodes), p(srt), p(qq), C.c_int64(len(qq)), C.c_int(0), p(ids), p(d2))
    ref_ids = srt["id"][g["closest_slot_ref"]].astype(np.int32)
    assert (ids == ref_ids).all()
    assert (np.sqrt(d2).astype(np.float32) == g["closest_dist_ref"]).all()
    lib.orc_nearest_bvh(p(nodes), p(srt), p(qq), C.c_int64(len(qq)), C.c_int(1), p(ids), p(d2))
    assert (np.sqrt(d2).astype(np.float32) == g["closest_dist_ref"]).all()


def test_golden_low_discrepancy(oracle, g):
    lib = oracle.lib()
    sob = np.array([[lib.orc_sobol(int(i), d) for d in (0, 1)] for i in g["sobol_idx"]], np.uint32)
    assert (sob == g["sobol_ref"]).all()
    ld = np.array([oracle.ld_random_val(int(i), int(s), 0) for i, s in zip(g["sobol_idx"], g["ld_seeds"])], np.float32)
    assert (ld.view(np.uint32) == g["ld_ref"].view(np.uint32)).all()
    off = np.array([oracle.pixel_offset(s) for s in range(64)], np.float32)
    assert (off.view(np.uint32) == g["pixel_offset_ref"].view(np.uint32)).all()


@pytest.fixture(scope="module")
def ref():
    from oracle import build_ref
    if not build_ref.available():
        pytest.skip("INSTA sources not present on this machine; the golden vectors carry the pin")
    lib = C.CDLL(str(build_ref.build(quiet=True)))
    lib.ref_tri_distance_sq.restype = C.c_float
    lib.ref_closest_triangle.restype = C.c_int
    return lib


def _random_triangles(rng, n):
    import importlib.util
    spec = importlib.util.spec_from_file_location("mk", Path(__file__).resolve().parent / "golden" / "make_golden.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    return mk.random_triangles(rng, n)


def test_live_reference_distance_and_traversal(oracle, ref):
    rng = np.random.default_rng(99)
    tris = _random_triangles(rng, 4000)
    pts = (tris["a"] + rng.normal(0, 1e-2, (len(tris), 3))).astype(np.float32)
    lib = oracle.lib()
    a = np.array([lib.orc_tri_distance_sq(p(tris[i:i + 1]), p(pts[i])) for i in range(len(tris))], np.float32)
    b = np.array([ref.ref_tri_distance_sq(p(tris[i:i + 1]), p(pts[i])) for i in range(len(tris))], np.float32)
    assert (a.view(np.uint32) == b.view(np.uint32)).all()
    from insta_gb300 import synthetic as S
    av = S.make_avatar(5, n_verts=1002)
    fr = av.frame(av.frame_coeffs(9))
    dtr = oracle.build_triangles(fr, av.canonical, av.faces, av.mask)
    bvh = oracle.Bvh(dtr, leaf_size=2)
    q = S.shell_points(fr, av.faces, 3000, seed=8)
    ids, d2 = bvh.nearest(q, exact=False)
    for i in range(len(q)):
        d = C.c_float(0)
        slot = ref.ref_closest_triangle(p(bvh.nodes), p(bvh.sorted), p(q[i]), C.byref(d))
        assert bvh.sorted["id"][slot] == ids[i]
        assert np.float32(np.sqrt(d2[i])) == np.float32(d.value)


# ---------------------------------------------------------------- march helpers
# calc_dt, warp_dt / unwarp_dt, mip_from_dt, density_grid_occupied_at and advance_to_next_voxel
# (instant-ngp/src/testbed_nerf.cu:91-93,186-208,300-337,471-485) compiled from the reference
# file's own text (oracle/ref_march_probe.cpp): the oracle's restatement, which the GPU march is
# tested against bit for bit, must reproduce them bit for bit.
GOLDEN_MARCH = Path(__file__).resolve().parent / "golden" / "reference_march.npz"
MARCH_KEYS = ("calc_dt", "warp_dt", "unwarp_dt", "mip_from_dt", "occupied_at", "advance")


def _bits(a):
    a = np.asarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else a


def test_golden_march_helpers_bit_exact(oracle):
    g = dict(np.load(GOLDEN_MARCH))
    ours = oracle.march_helpers(oracle.lib(), g, oracle.march_bitfield())
    for k in MARCH_KEYS:
        assert (_bits(ours[k]) == _bits(g["ref_" + k])).all(), k
    # the cases reach both clamps of calc_dt, every mip and every grid level of the DDA
    dt = g["ref_calc_dt"]
    assert (dt == dt.min()).sum() > 50 and (dt == dt.max()).sum() >= 10 and abs(dt.max() / dt.min() - 1024) < 1e-2
    assert set(np.unique(g["ref_mip_from_dt"])) == set(range(7))
    assert 0.2 < g["ref_occupied_at"].mean() < 0.8
    # calc_cone_angle is the constant (the pixel-size variant is commented out in the reference)
    assert (g["cone_ref"] == g["dt_cone"]).all()


def test_live_reference_march_helpers(oracle, ref):
    from oracle import oracle as O
    for n in ("ref_calc_dt", "ref_warp_dt", "ref_unwarp_dt", "ref_advance_to_next_voxel"):
        getattr(ref, n).restype = C.c_float
    ref.ref_calc_dt.argtypes = [C.c_float, C.c_float]
    ref.ref_warp_dt.argtypes = [C.c_float]
    ref.ref_unwarp_dt.argtypes = [C.c_float]
    ref.ref_mip_from_dt.argtypes = [C.c_float, C.c_void_p]
    ref.ref_density_grid_occupied_at.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32]
    ref.ref_advance_to_next_voxel.argtypes = [C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32]
    cases = O.march_cases(np.random.default_rng(123))
    bf = O.march_bitfield()
    a = O.march_helpers(oracle.lib(), cases, bf)
    b = O.march_helpers(ref, cases, bf)
    for k in MARCH_KEYS:
        assert (_bits(a[k]) == _bits(b[k])).all(), k
