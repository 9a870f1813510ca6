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
    """Two static calls in a row (3000 and 16384 samples) equal the allocating path bit for bit:
    the static path runs the same encode, MLP and unpack kernels, and rows of a tile do not mix,
    so whatever an earlier call left in the shared array (padding rows of a partial tile) cannot
    reach a valid sample.  Another avatar's call with a different size runs in between.  Neither
    the context's allocation counter nor the device's free memory moves across the static calls
    (after the first one, which looks up the array's device address), and a batch larger than
    the array is rejected."""
    from insta_gb300 import abi, synthetic as S
    ctx = abi.Context(0)
    try:
        fc = S.FieldConfig()
        ctx.params_load(7, fc, S.field_params(fc, seed=11))
        ctx.params_load(8, fc, S.field_params(fc, seed=12))
        sizes = (3000, 16384)
        cs = [torch.from_numpy(coords(n, seed=20 + call)).cuda() for call, n in enumerate(sizes)]
        refs = [torch.zeros((n, 4), dtype=torch.float32, device="cuda") for n in sizes]
        gots = [torch.full((n, 4), float("nan"), dtype=torch.float32, device="cuda") for n in sizes]
        other_c = torch.from_numpy(coords(777, seed=30)).cuda()
        other = torch.zeros((777, 4), dtype=torch.float32, device="cuda")
        warm = torch.zeros((5, 4), dtype=torch.float32, device="cuda")
        for c, r in zip(cs, refs):
            ctx.field_eval(7, c, 11, c.shape[0], r)
        ctx.field_eval_static(8, other_c[:5], 11, 5, warm)     # first call on this device: address lookup
        ctx.sync()
        used0, free0 = ctx.memory_used(), torch.cuda.mem_get_info()[0]
        for call, (c, g) in enumerate(zip(cs, gots)):
            ctx.field_eval_static(7, c, 11, c.shape[0], g)
            if call == 0:
                ctx.field_eval_static(8, other_c, 11, 777, other)   # a different avatar and size in between
        ctx.sync()
        assert ctx.memory_used() == used0
        assert torch.cuda.mem_get_info()[0] == free0
        for r, g in zip(refs, gots):
            r, g = r.cpu().numpy(), g.cpu().numpy()
            assert np.isfinite(g).all()
            assert np.array_equal(g, r), float(np.abs(g - r).max())
            assert (np.abs(g - r) <= ATOL + RTOL * np.abs(r)).all()
        ref_other = torch.zeros((777, 4), dtype=torch.float32, device="cuda")
        ctx.field_eval(8, other_c, 11, 777, ref_other)
        ctx.sync()
        assert np.array_equal(other.cpu().numpy(), ref_other.cpu().numpy())
        with pytest.raises(abi.InstaError) as e:
            c = torch.zeros((16385, 11), dtype=torch.float32, device="cuda")
            ctx.field_eval_static(7, c, 11, 16385, torch.zeros((16385, 4), device="cuda"))
        assert e.value.code == abi.ERR_INVALID_ARG
    finally:
        ctx.close()
