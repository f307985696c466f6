"""vxl_voxelize_noalloc, the voxelizer entry point for callers that cannot
allocate device memory (it uses the library's fixed static device table as
its only scratch), checked through the C ABI against vxl_voxelize on two
calls in a row. This file is collected last on purpose."""
import numpy as np
import pytest

from tests import vox_cases
from tests.gpu_util import dev, export_r8

pytestmark = pytest.mark.gpu


def _instances(rng, nmodels, count, n, clear_every):
    out = []
    for i in range(count):
        op = 0 if (clear_every and i % clear_every == clear_every - 1) else 1
        out.append((vox_cases.world_matrix(rng, -0.5, n / 10.0), int(rng.integers(0, nmodels)), op))
    return out


def test_voxelize_noalloc_matches_voxelize(vxl, ctx):
    import torch

    rng = np.random.default_rng(20261203)
    models = [vox_cases.random_model(rng, *rng.integers(3, 40, 3)) for _ in range(6)]
    d_models = [dev(m) for m in models]
    mdesc = [(d.data_ptr(),) + m.shape[::-1] for m, d in zip(models, d_models)]
    n = 160
    ref = vxl.Grid(ctx, n, n, n)          # updated by vxl_voxelize
    tgt = vxl.Grid(ctx, n, n, n)          # updated by vxl_voxelize_noalloc
    desc = tgt.describe()
    S = n // 2
    for call, (count, clear_every) in enumerate([(90, 0), (70, 3)]):
        insts = _instances(rng, len(models), count, n, clear_every)
        a0 = np.tile(np.array([S - 1, S - 1, S - 1, 0, 0, 0], np.int32), (count, 1))
        aabb_ref, aabb_na = dev(a0), dev(a0)
        vxl.voxelize(ctx, ref, mdesc, insts, aabb_ref)
        vxl.voxelize_noalloc(desc, mdesc, insts, aabb_na)
        torch.cuda.synchronize()
        g_ref, g_na = export_r8(ref), export_r8(tgt)
        assert g_ref.any(), call
        assert np.array_equal(g_na, g_ref), "call %d: grids differ in %d bytes" % (call, int((g_na != g_ref).sum()))
        assert torch.equal(aabb_na, aabb_ref), call
        assert tgt.count() == ref.count()


def test_voxelize_noalloc_rejects_oversize(vxl, ctx):
    n = 16
    g = vxl.Grid(ctx, n, n, n)
    m = dev(np.full((2, 2, 2), 20, np.uint8))
    too_many = [(np.eye(4, dtype=np.float32).reshape(16), 0, 1)] * (16384 + 1)
    with pytest.raises(vxl.VxlError) as e:
        vxl.voxelize_noalloc(g.describe(), [(m.data_ptr(), 2, 2, 2)], too_many)
    assert e.value.status == 5 and "exceed" in str(e.value)
