"""Host-side logic of the training entry points, without a GPU: the loss description the Python
binding builds (names of loss types, buffers, defaults) and the step loop's argument checks."""
import ctypes as C

import numpy as np
import pytest


class FakeLib:
    """Stands in for the C library: records the descriptions it is handed."""

    def __init__(self):
        self.calls = []

    def insta_train_loss(self, h, desc_ref):
        d = C.cast(desc_ref, C.POINTER(self.desc_type)).contents
        # copy now: array fields are views into the caller's struct, gone after the call
        self.calls.append({name: (list(v) if isinstance(v, C.Array) else v) for name, v in ((n, getattr(d, n)) for n, *_ in d._fields_)})
        return 0

    def insta_train_set_math(self, h, math):
        self.calls.append({"math": math})
        return 0 if math in (0, 1, 2) else 1

    def insta_last_error(self, h):
        return b"unknown training math"

    def insta_ctx_destroy(self, h):
        return 0


def fake_context():
    from insta_gb300 import abi
    ctx = abi.Context.__new__(abi.Context)
    ctx.lib = FakeLib()
    ctx.lib.desc_type = abi.TrainLossDesc
    ctx.h = C.c_void_p(1)
    return ctx


def test_train_loss_description_fields():
    from insta_gb300 import abi
    ctx = fake_context()
    rays = np.zeros((8, 6), np.float32)
    counter = np.zeros(1, np.uint32)
    ctx.train_loss(n_rays=8, max_rays=8, max_samples_compacted=64, stride=27, loss_type="huber", depth_loss_type="l1",
                   aabb_min=(0.1, 0.2, 0.3), rays=rays, numsteps_counter=counter, background=None)
    d = ctx.lib.calls[-1]
    assert d["loss_type"] == abi.LOSS_TYPES["huber"] == 4 and d["depth_loss_type"] == 1
    assert d["n_rays"] == 8 and d["max_samples_compacted"] == 64 and d["stride"] == 27
    assert d["loss_scale"] == 128.0 and d["seg_mask_supervision_lambda"] == 1.0      # reference defaults
    assert d["aabb_min"] == pytest.approx([0.1, 0.2, 0.3]) and d["aabb_max"] == [1.0, 1.0, 1.0]
    assert d["rays"] == rays.ctypes.data and d["numsteps_counter"] == counter.ctypes.data
    assert d["background"] is None and d["target"] is None


def test_train_set_math_passes_and_rejects():
    from insta_gb300 import abi
    ctx = fake_context()
    ctx.train_set_math(True)
    ctx.train_set_math(False)
    ctx.train_set_math(False, tcgen05=True)
    assert [c["math"] for c in ctx.lib.calls] == [1, 0, 2]
    with pytest.raises(abi.InstaError):
        ctx._check(ctx.lib.insta_train_set_math(ctx.h, 7))


def test_train_step_rejects_a_batch_larger_than_its_buffer():
    pytest.importorskip("torch")
    from insta_gb300 import synthetic as S
    from insta_gb300.train import TrainConfig, TrainStep
    with pytest.raises(ValueError):
        TrainStep(fake_context(), 0, S.FieldConfig(), TrainConfig(target_batch_size=1 << 20, max_samples=1 << 18))
