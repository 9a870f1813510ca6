"""Error behaviour of the C ABI (statuses, never a crash): invalid arguments, missing state,
unsupported shapes and the device-memory budget."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def code_of(fn):
    from insta_gb300 import abi
    with pytest.raises(abi.InstaError) as e:
        fn()
    return int(str(e.value).split("]")[0].split()[-1])


def test_missing_state_and_bad_arguments():
    from insta_gb300 import abi, synthetic as S
    ctx = abi.Context(0)
    av = S.make_avatar(0, n_verts=402)
    cam, focal = S.camera(0.0, width=16, height=16)
    req = ctx.render_desc(0, 0, 16, 16, focal, cam)
    out = (np.zeros((256, 4), np.float32), np.zeros(256, np.float32))
    assert code_of(lambda: ctx.render(req, *out)) == 4                     # no avatar
    ctx.canonical_set(0, av.canonical, av.faces, av.mask)
    assert code_of(lambda: ctx.render(req, *out)) == 4                     # no parameters
    fc = S.FieldConfig()
    ctx.params_load(0, fc, S.field_params(fc))
    assert code_of(lambda: ctx.render(req, *out)) == 4                     # no frame
    ctx.frame_upload(0, 0, av.frame(av.frame_coeffs(0)))
    assert code_of(lambda: ctx.render(req, *out)) == 4                     # no occupancy
    ctx.occupancy_from_mesh(0, 0, 0.015)
    ctx.render(req, *out)                                                  # now it renders
    bad = ctx.render_desc(0, 0, 0, 16, focal, cam)
    assert code_of(lambda: ctx.render(bad, *out)) == 1                     # bad resolution
    huge = ctx.render_desc(0, 0, 8192, 4097, focal, cam)                   # > 2^25 pixels: more than a round holds
    assert code_of(lambda: ctx.render(huge, *out)) == 1
    big = [ctx.render_desc(0, 0, 1024, 1024, focal, cam) for _ in range(33)]   # 33 Mpx in one batch
    assert code_of(lambda: ctx.render_batch(big, [out[0]] * 33, [out[1]] * 33)) == 1
    assert code_of(lambda: ctx.occupancy_from_mesh(0, 0, -1.0)) == 1       # bad radius
    assert code_of(lambda: ctx.occupancy_get(0, 5)) == 4                   # unknown frame
    fc12 = S.FieldConfig(n_levels=6)     # 12 hash features: not whole 8-feature groups
    assert code_of(lambda: ctx.params_load(1, fc12, np.zeros(10, np.float16))) == 5   # unsupported shape
    ctx.close()


def test_device_memory_budget():
    from insta_gb300 import abi, synthetic as S
    ctx = abi.Context(0, budget_bytes=8 << 20)
    av = S.make_avatar(0, n_verts=402)
    ctx.canonical_set(0, av.canonical, av.faces, av.mask)
    fc = S.FieldConfig()
    # the hash table alone (~32 MiB) does not fit an 8 MiB budget
    assert code_of(lambda: ctx.params_load(0, fc, S.field_params(fc))) == 3
    assert ctx.memory_used() <= 8 << 20
    ctx.close()
