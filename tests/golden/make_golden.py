"""Generate tests/golden/reference_geometry.npz and tests/golden/reference_march.npz from the
reference's own code.

Runs oracle/_ref/libinsta_ref.so -- Triangle::distance_sq, BoundingBox::distance_sq,
Triangle::tbn, tri2projection, interpolate_transformation, transform_point/direction,
closest_triangle, sobol, ld_random_val and ld_random_pixel_offset compiled for the host from
the INSTA headers, and the march helpers of instant-ngp/src/testbed_nerf.cu (calc_dt,
warp_dt / unwarp_dt, mip_from_dt, density_grid_occupied_at, advance_to_next_voxel) compiled from
the text of that file (oracle/build_ref.py) -- on seeded inputs and stores inputs and outputs.
The oracle is then checked against these vectors on machines without the INSTA sources.

    python tests/golden/make_golden.py            # both files
    python tests/golden/make_golden.py --march    # reference_march.npz only
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import build_ref, oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_geometry.npz"
OUT_MARCH = Path(__file__).resolve().parent / "reference_march.npz"
F32P = C.POINTER(C.c_float)


def ref_lib():
    lib = C.CDLL(str(build_ref.build(quiet=True)))
    for n in ("ref_tri_distance_sq", "ref_box_distance_sq", "ref_ld_random_val"):
        getattr(lib, n).restype = C.c_float
    lib.ref_ld_random_val.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
    lib.ref_sobol.restype = C.c_uint32
    lib.ref_sobol.argtypes = [C.c_uint32, C.c_uint32]
    lib.ref_closest_triangle.restype = C.c_int
    for n in ("ref_calc_dt", "ref_warp_dt", "ref_unwarp_dt", "ref_advance_to_next_voxel", "ref_distance_to_next_voxel",
              "ref_calc_cone_angle"):
        getattr(lib, n).restype = C.c_float
    lib.ref_calc_dt.argtypes = [C.c_float, C.c_float]
    lib.ref_warp_dt.argtypes = [C.c_float]
    lib.ref_unwarp_dt.argtypes = [C.c_float]
    lib.ref_calc_cone_angle.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float]
    lib.ref_mip_from_dt.argtypes = [C.c_float, C.c_void_p]
    lib.ref_density_grid_occupied_at.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32]
    lib.ref_advance_to_next_voxel.argtypes = [C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32]
    return lib


def p(a):
    return C.c_void_p(a.ctypes.data)


def random_triangles(rng, n):
    """Triangles of mixed shapes: regular, slivers, near-degenerate, plus scaling and masks."""
    tri = np.zeros(n, dtype=np.dtype([("a", "<f4", 3), ("b", "<f4", 3), ("c", "<f4", 3), ("scaling", "<f4"), ("id", "<u4"), ("mask_id", "<u4")]))
    a = rng.uniform(0.4, 0.6, (n, 3))
    e1 = rng.normal(0, 4e-3, (n, 3))
    e2 = rng.normal(0, 4e-3, (n, 3))
    sl = rng.random(n) < 0.15            # slivers: second edge almost parallel to the first
    e2[sl] = e1[sl] * rng.uniform(0.3, 2.0, (sl.sum(), 1)) + rng.normal(0, 1e-7, (sl.sum(), 3))
    tri["a"] = a
    tri["b"] = a + e1
    tri["c"] = a + e2
    tri["scaling"] = rng.uniform(0.8, 1.25, n)
    tri["id"] = np.arange(n)
    tri["mask_id"] = rng.choice([1, 2, 7, 15], n)
    return tri


def main():
    lib = ref_lib()
    rng = np.random.default_rng(2024)
    g = {}
    # point-triangle and point-box squared distances
    tris = random_triangles(rng, 1500)
    pts = (tris["a"] + rng.normal(0, 6e-3, (len(tris), 3))).astype(np.float32)
    g["dist_tris"], g["dist_pts"] = tris, pts
    g["dist_ref"] = np.array([lib.ref_tri_distance_sq(p(tris[i:i + 1]), p(pts[i])) for i in range(len(tris))], np.float32)
    mn = rng.uniform(0.3, 0.6, (1000, 3)).astype(np.float32)
    mx = (mn + rng.uniform(0, 0.05, (1000, 3))).astype(np.float32)
    bp = rng.uniform(0.25, 0.7, (1000, 3)).astype(np.float32)
    g["box_min"], g["box_max"], g["box_pts"] = mn, mx, bp
    g["box_ref"] = np.array([lib.ref_box_distance_sq(p(mn[i]), p(mx[i]), p(bp[i])) for i in range(1000)], np.float32)
    # frames
    ft = tris[:400]
    tbn = np.zeros((len(ft), 9), np.float32)
    proj = np.zeros((len(ft), 16), np.float32)
    for i in range(len(ft)):
        lib.ref_tbn(p(ft[i:i + 1]), p(tbn[i]))
        lib.ref_tri2projection(p(ft[i:i + 1]), p(pts[i]), p(proj[i]))
    g["frame_tris"], g["tbn_ref"], g["proj_ref"] = ft, tbn, proj
    # a small closed mesh: blended frames, transforms and the nearest-triangle traversal
    from insta_gb300 import synthetic as S
    av = S.make_avatar(3, n_verts=402)
    frame = av.frame(av.frame_coeffs(3))
    can = O.build_triangles(av.canonical, None, av.faces, av.mask)
    dtr = O.build_triangles(frame, av.canonical, av.faces, av.mask)
    adj = O.adjacency(av.faces, av.n_verts)
    g["mesh_can"], g["mesh_def"], g["mesh_adj"] = can, dtr, adj
    q = S.shell_points(frame, av.faces, 600, seed=5)
    ids = rng.integers(0, len(dtr), len(q)).astype(np.uint32)
    blend = np.zeros((len(q), 2, 16), np.float32)
    for i in range(len(q)):
        lib.ref_interpolate_transformation(p(q[i]), p(adj), p(dtr), C.c_uint32(int(ids[i])), C.c_int(1), p(blend[i, 0]))
        lib.ref_interpolate_transformation(p(q[i]), p(adj), p(can), C.c_uint32(int(ids[i])), C.c_int(0), p(blend[i, 1]))
    g["blend_pts"], g["blend_ids"], g["blend_ref"] = q, ids, blend
    dirs = rng.normal(size=(len(q), 3)).astype(np.float32)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    tp = np.zeros((len(q), 3), np.float32)
    td = np.zeros((len(q), 3), np.float32)
    for i in range(len(q)):
        lib.ref_transform(p(q[i]), p(dirs[i]), p(blend[i, 0]), p(blend[i, 1]), p(tp[i]), p(td[i]))
    g["transform_dirs"], g["transform_p_ref"], g["transform_d_ref"] = dirs, tp, td
    bvh = O.Bvh(dtr, leaf_size=2)
    g["bvh_nodes"], g["bvh_sorted"] = bvh.nodes, bvh.sorted
    qq = S.shell_points(frame, av.faces, 2000, seed=6)
    slot = np.zeros(len(qq), np.int32)
    dist = np.zeros(len(qq), np.float32)
    for i in range(len(qq)):
        d = C.c_float(0)
        slot[i] = lib.ref_closest_triangle(p(bvh.nodes), p(bvh.sorted), p(qq[i]), C.byref(d))
        dist[i] = d.value
    g["closest_pts"], g["closest_slot_ref"], g["closest_dist_ref"] = qq, slot, dist
    # low-discrepancy sequences
    idx = np.concatenate([np.arange(64), rng.integers(0, 2 ** 32, 136, dtype=np.uint64)]).astype(np.uint32)
    g["sobol_idx"] = idx
    g["sobol_ref"] = np.array([[lib.ref_sobol(int(i), d) for d in (0, 1)] for i in idx], np.uint32)
    seeds = (np.arange(200, dtype=np.uint64) * 786433 % (2 ** 32)).astype(np.uint32)
    g["ld_seeds"] = seeds
    g["ld_ref"] = np.array([lib.ref_ld_random_val(int(i), int(s), 0) for i, s in zip(idx, seeds)], np.float32)
    off = np.zeros((64, 2), np.float32)
    for s in range(64):
        lib.ref_ld_random_pixel_offset(C.c_uint32(s), p(off[s]))
    g["pixel_offset_ref"] = off
    np.savez_compressed(OUT, **g)
    print(OUT, OUT.stat().st_size, "bytes")


def march_main(lib=None):
    """The march helpers on seeded inputs (oracle.march_cases) over oracle.march_bitfield()."""
    lib = lib or ref_lib()
    cases = O.march_cases(np.random.default_rng(77))
    out = O.march_helpers(lib, cases, O.march_bitfield())
    g = dict(cases)
    g.update({"ref_" + k: v for k, v in out.items()})
    # calc_cone_angle returns the constant whatever the cosine and focal length (:82-89)
    g["cone_ref"] = np.array([lib.ref_calc_cone_angle(c, 1000.0, 1000.0, k) for c, k in zip(cases["warp_in"], cases["dt_cone"])],
                             np.float32)
    np.savez_compressed(OUT_MARCH, **g)
    print(OUT_MARCH, OUT_MARCH.stat().st_size, "bytes")


if __name__ == "__main__":
    if "--march" not in sys.argv:
        main()
    march_main()
