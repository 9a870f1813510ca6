"""Snapshot documents (Testbed::save_snapshot / load_snapshot layout) and the msgpack codec."""
import numpy as np
import pytest

from insta_gb300 import snapshot as SN


def sample_doc():
    return {
        "small": [0, 1, 127, 128, 255, 256, 65535, 65536, 2 ** 32 - 1, 2 ** 32, 2 ** 63],
        "neg": [-1, -32, -33, -128, -129, -32768, -32769, -2 ** 31, -2 ** 31 - 1, -2 ** 63],
        "floats": [0.5, -1.25e-7, 3.0e38],
        "f32": np.float32(0.1),
        "strs": ["", "a" * 31, "b" * 32, "c" * 300, "d" * 70000],
        "bins": [b"", b"x" * 255, b"y" * 256, b"z" * 70000],
        "nest": {"t": True, "f": False, "n": None, "l": list(range(20)), "m": {str(i): i for i in range(20)}},
    }


def test_msgpack_round_trip():
    d = sample_doc()
    back = SN.unpackb(SN.packb(d))
    want = dict(d)
    want["f32"] = float(np.float32(0.1))
    assert back == want


def test_msgpack_matches_reference_codec():
    msgpack = pytest.importorskip("msgpack")
    d = sample_doc()
    d.pop("f32")
    assert msgpack.unpackb(SN.packb(d), raw=False, strict_map_key=False) == d
    assert SN.unpackb(msgpack.packb(d, use_bin_type=True)) == d
    with pytest.raises(ValueError):
        SN.unpackb(SN.packb(d)[:-3])


def test_snapshot_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    config = {"encoding": {"otype": "HashGrid", "n_levels": 16, "n_features_per_level": 8, "log2_hashmap_size": 18, "base_resolution": 16},
              "network": {"n_neurons": 64, "n_hidden_layers": 2, "n_output_dims": 16},
              "rgb_network": {"n_neurons": 64, "n_hidden_layers": 3}, "exp_params": 16}
    s = SN.Snapshot(params=rng.normal(size=1000).astype(np.float16), density_grid=rng.random(2 * 128 ** 3).astype(np.float16),
                    aabb=(np.zeros(3, np.float32), np.ones(3, np.float32)),
                    render_aabb=(np.full(3, 0.2, np.float32), np.full(3, 0.8, np.float32)), aabb_scale=2, training_step=1234,
                    loss=0.125, config=config)
    path = tmp_path / "avatar.msgpack"
    SN.write_snapshot(path, s)
    r = SN.read_snapshot(path)
    assert (r.params.view(np.uint16) == s.params.view(np.uint16)).all()
    assert (r.density_grid.view(np.uint16) == s.density_grid.view(np.uint16)).all() and r.n_cascades == 2
    assert all((a == b).all() for a, b in zip(r.aabb, s.aabb)) and all((a == b).all() for a, b in zip(r.render_aabb, s.render_aabb))
    assert (r.aabb_scale, r.training_step, r.loss) == (2, 1234, 0.125)
    fc = r.field_config()
    assert (fc.n_levels, fc.n_features, fc.log2_table, fc.base_res, fc.n_extra) == (16, 8, 18, 16, 16)
    assert (fc.density_hidden, fc.density_layers, fc.density_out, fc.rgb_hidden, fc.rgb_layers, fc.aabb_scale) == (64, 2, 16, 64, 3, 2)
    # that is INSTA's shipped field, and the library takes it
    from insta_gb300 import abi, layout, synthetic as S
    want = S.insta_field_config()
    assert (fc.n_levels, fc.n_features, fc.log2_table, fc.n_extra, fc.density_layers, fc.rgb_layers) == \
        (want.n_levels, want.n_features, want.log2_table, want.n_extra, want.density_layers, want.rgb_layers)
    assert abi.param_count(fc) == layout.field_layout(fc).total


def test_snapshot_fp32_params_and_errors():
    p = np.linspace(-1, 1, 64, dtype=np.float32)
    doc = {"snapshot": {"version": 1, "params_type": "float", "params_binary": p.tobytes(), "density_grid_size": 128,
                        "density_grid_binary": b""}}
    r = SN.read_snapshot(SN.packb(doc))
    assert (r.params == p.astype(np.float16)).all() and r.density_grid is None
    doc["snapshot"]["version"] = 0
    with pytest.raises(ValueError):
        SN.read_snapshot(SN.packb(doc))
    doc["snapshot"]["version"] = 1
    doc["snapshot"]["density_grid_size"] = 64
    doc["snapshot"]["density_grid_binary"] = b"\0\0" * 64 ** 3
    with pytest.raises(ValueError):
        SN.read_snapshot(SN.packb(doc))
    with pytest.raises(ValueError):
        SN.read_snapshot(SN.packb({"encoding": {}}))


# Every key Testbed::load_snapshot (instant-ngp/src/testbed.cu:2952-3016) reads from the snapshot
# block, the ones without a default (operator[]) and the ones with (value()); the trainer's
# deserialize reads params_binary.
LOAD_SNAPSHOT_KEYS = [("version",), ("aabb",), ("render_aabb",), ("bounding_radius",), ("density_grid_size",),
                      ("nerf", "rgb", "rays_per_batch"), ("nerf", "rgb", "measured_batch_size"),
                      ("nerf", "rgb", "measured_batch_size_before_compaction"), ("nerf", "aabb_scale"),
                      ("density_grid_binary",), ("training_step",), ("loss",), ("params_binary",)]


@pytest.mark.parametrize("with_grid", [False, True])
def test_written_snapshot_has_every_key_load_snapshot_reads(with_grid):
    rng = np.random.default_rng(1)
    s = SN.Snapshot(params=rng.normal(size=64).astype(np.float16),
                    density_grid=rng.random(128 ** 3).astype(np.float16) if with_grid else None,
                    aabb=(np.zeros(3, np.float32), np.ones(3, np.float32)), render_aabb=(np.zeros(3, np.float32), np.ones(3, np.float32)),
                    aabb_scale=2, bounding_radius=0.75, rays_per_batch=4096, measured_batch_size=200000,
                    measured_batch_size_before_compaction=250000)
    doc = SN.unpackb(SN.write_snapshot(None, s))
    for key in LOAD_SNAPSHOT_KEYS:
        node = doc["snapshot"]
        for k in key:
            assert k in node, key
            node = node[k]
    r = SN.read_snapshot(SN.write_snapshot(None, s))
    assert (r.bounding_radius, r.rays_per_batch, r.measured_batch_size, r.measured_batch_size_before_compaction) == \
        (0.75, 4096, 200000, 250000)
    assert (r.density_grid is not None) == with_grid
