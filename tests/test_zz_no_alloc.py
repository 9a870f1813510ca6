"""insta_field_eval_static: the entry point that allocates no device memory.

Callers that must not allocate while they run (code recorded into a CUDA graph, real-time
callbacks with a fixed memory budget, hosts that hand out all device memory from their own
pool) use it instead of insta_field_eval.  Its working memory is a fixed array inside the
library, so it must return the same values as the allocating path, call after call, and
reject batches larger than that array holds.  This file is collected last so a failure here
never hides the other GPU tests.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

# the tolerance of the field parity tests: FP16 outputs, FP32 accumulation order
ATOL, RTOL = 4e-3, 1e-2


def coords(n, seed):
    rng = np.random.default_rng(seed)
    c = np.zeros((n, 11), np.float32)
    c[:, :3] = rng.uniform(0.35, 0.65, size=(n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    c[:, 8:11] = (d + 1) * 0.5
    return c


def test_static_matches_allocating_path_twice():
    from insta_gb300 import abi, synthetic as S
    ctx = abi.Context(0)
    try:
        fc = S.FieldConfig()
        ctx.params_load(7, fc, S.field_params(fc, seed=11))
        for call, n in enumerate((3000, 16384)):
            c = torch.from_numpy(coords(n, seed=20 + call)).cuda()
            ref = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
            got = torch.full((n, 4), float("nan"), dtype=torch.float32, device="cuda")
            ctx.field_eval(7, c, 11, n, ref)
            ctx.field_eval_static(7, c, 11, n, got)
            ctx.sync()
            r, g = ref.cpu().numpy(), got.cpu().numpy()
            assert np.isfinite(g).all()
            assert (np.abs(g - r) <= ATOL + RTOL * np.abs(r)).all(), float(np.abs(g - r).max())
        with pytest.raises(abi.InstaError) as e:
            c = torch.zeros((16385, 11), dtype=torch.float32, device="cuda")
            ctx.field_eval_static(7, c, 11, 16385, torch.zeros((16385, 4), device="cuda"))
        assert e.value.code == abi.ERR_INVALID_ARG
    finally:
        ctx.close()
